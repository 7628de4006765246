"""Benchmark of the radiance pass on GB300: probe-rays/s on the demo-scale plain workload.

Workload (one "step"): the 64x64x16-block terrain world plus 2000 random blocks of 32 types,
8 successive passes (multi-bounce, each reading the previous pass's volume), each over a seeded
10% subset of the probes, 256 rays per probe, max_dist 256, blend 0.1, FP32 radiance.

  value      probe-rays/s with every input resident in HBM (request lists uploaded once), the
             step's 8 passes in one lumrad_radiance_passes_resident call (one march launch for
             all 8, then each pass's finalize in order; bit-identical to 8 single passes);
             CUDA events on the pass stream around each step; L2 flushed (256 MiB write)
             between steps, outside the timed region.
  single_pass  the same step as 8 lumrad_radiance_pass_resident calls (one frame's update each).
  e2e        the same metric through the C ABI with host buffers: each step copies its 8 request
             lists host->device (lumrad_radiance_passes, the lists back to back in one page-locked
             array) and reads the radiance volume back.
  roofline   the bound that limits the step's kernels (march + 8 finalize launches): instruction
             issue.  achieved = warp instructions per step (ncu's smsp__inst_executed.sum over the
             same 9 launches, NCU_WARP_INST_PER_STEP) / the kernels' own duration (the span of
             the %globaltimer stamps they write, lumrad_get_kernel_times);
             peak = one warp instruction per cycle on each of the 4 schedulers of every SM at the SM
             clock sampled during the timed region.  Beside it, the memory rooflines: algorithmic
             bytes of one step (3 B per grid+palette lookup, 16+8*12 B per hit, 8+2*12 B per probe;
             counts exact from the kernels' counters) over the same duration, against the
             measured HBM copy peak and an L2-resident read rate measured in the run.
  cpu_baseline  the CPU oracle (port, OpenMP over all host cores) on whole steps, ~12 s.

--impl reference times the reference's implementation of the same workload on the host cores:
Lum's radiance.comp compiled as C++ from its source (oracle/build_ref.py), one process per core.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from lum_gb300 import worldgen  # noqa: E402

WORKLOAD = {
    "workload": "plain radiance update, demo scale: 64x64x16 blocks + 2000 random blocks, "
                "32 block types, 8 passes x 10% probes, 256 rays/probe, max_dist 256, FP32",
    "world_blocks": [64, 64, 16], "extra_blocks": 2000, "block_types": 32, "passes_per_step": 8,
    "probe_fraction": 0.1, "rays_per_probe": 256, "max_dist": 256.0, "blend": 0.1, "seed": 1234,
}
PASSES = 8
RAYS = 256
MAX_DIST = 256.0
BLEND = 0.1
SEED = 1234
S_R = 12            # bytes of FP32 RGB radiance per probe
BATCH_ROUND_TASKS = 1 << 20   # 32-ray tasks per march/finalize round of a batch
# DRAM bytes (read + write) of one step's kernels (the march launch over 8 passes and the 8
# finalize launches, whose extra CTAs copy each pass's unlisted probes) in ncu captures of this
# workload (the march's launch, and 3 of the 8 finalize launches scaled to 8); ncu replays with cold
# caches (march 1.09 + 376.37 MB: most of the step's 430 MB of 32-byte ray results leave the L2
# before their finalize launches; finalizes 442.51 + 0.77 MB)
NCU_DRAM_BYTES_PER_STEP = 820.74e6
# L2 bytes (lts__t_bytes.sum) of the same launches in the same captures (march 825.5 MB: its world
# lookups are shared-memory loads, finalizes 1255.3 MB)
NCU_L2_BYTES_PER_STEP = 2080.8e6
# Warp instructions (smsp__inst_executed.sum) of the same launches: the march over the 8 passes
# (464.5 M) and the 8 finalize launches (302.8 M); deterministic up to the march queue's task order
NCU_WARP_INST_PER_STEP = 464.5e6 + 302.8e6
SCHEDULERS_PER_SM = 4


def pass_lists(dims):
    return [worldgen.probe_subset(dims, 0.1, seed=SEED, stream=p) for p in range(PASSES)]


def algorithmic_bytes(steps: int, hits: int, probes: int) -> int:
    return 3 * steps + hits * (16 + 8 * S_R) + probes * (8 + 2 * S_R)


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def l2_read_gbs(device: int) -> float:
    """L2-resident read rate of this GPU, the reference for the path's L2 roofline: one kernel
    summing 64 rows that are all the same 24 MiB float array (a stride-0 view: 1.5 GiB read from
    a buffer well inside the 129 MB L2), best of 5 launches, CUDA events."""
    import torch
    n = 24 * 1024 * 1024 // 4
    rows = 64
    a = torch.rand(n, device=f"cuda:{device}")
    v = a.expand(rows, n)
    out = torch.empty(rows, device=a.device)
    for _ in range(3):
        torch.sum(v, dim=1, out=out)
    best = 0.0
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.sum(v, dim=1, out=out)
        e1.record()
        e1.synchronize()
        best = max(best, 4.0 * n * rows / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(world, lists, budget_s: float = 12.0):
    """The CPU oracle (the port: OpenMP over workgroups, all host cores) on whole steps of the
    workload, repeated until about `budget_s` seconds of CPU work."""
    import oracle
    cores = oracle.max_threads()
    prev = np.zeros(world.grid.shape + (3,), dtype=np.float32)
    steps = 0
    t0 = time.perf_counter()
    while True:
        cur = prev
        for p in range(PASSES):
            cur, _, _ = oracle.radiance_pass(world, lists[p], rays=RAYS, max_dist=MAX_DIST, blend=BLEND,
                                             time_seed=p, prev=cur)
        steps += 1
        dt = time.perf_counter() - t0
        if dt >= budget_s:
            break
    rays = steps * sum(l.shape[0] for l in lists) * RAYS
    return {"value": rays / dt, "unit": "probe-rays/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full steps (8 passes x 6554 probes x 256 rays), {dt:.1f} s"}


def reference_runner(world):
    """Runs a pass of the reference's own shader code (radiance.comp compiled as C++) on all host
    cores, or, where it cannot be built, the port.  Returns (run(req, prev, seed) -> next, kind, cores)."""
    from oracle import build_ref
    try:
        if not build_ref.available():
            raise RuntimeError("no reference shader source")
        build_ref.build(rays=(RAYS,))
        from oracle import ref_pool
        pool = ref_pool.RefPool(world, RAYS)

        def run(req, prev, seed):
            return pool.run_pass(req.astype(np.int8), prev, max_dist=MAX_DIST, blend=BLEND, time_seed=seed)
        run.close = pool.close
        return run, "reference", pool.processes
    except Exception:
        import oracle

        def run(req, prev, seed):
            return oracle.radiance_pass(world, req, rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=seed,
                                        prev=prev)[0]
        run.close = lambda: None
        return run, "port", oracle.max_threads()


BATCH_WORKLOAD = {
    "workload": "batched radiance update: 256 independent terrain worlds, dims uniform per axis in "
                "4x4x4..32x32x16 blocks, update lists U(1%,100%) of each world's probes, rays/probe "
                "one of {32,64,128,256}, max_dist 128, blend 0.1, FP32",
    "worlds": 256, "min_blocks": [4, 4, 4], "max_blocks": [32, 32, 16], "seed": SEED,
}


def batched_leg(local: int, steps: int, warmup: int, flush, tuning=None):
    """Mixed-size workload: one autotuned batch (one graph replay per step, all 256 worlds in the
    same persistent launches) against the plain path (one pass per world, each world alone)."""
    import torch
    import lum_gb300
    mix = worldgen.mixed_worlds(n=BATCH_WORKLOAD["worlds"], seed=SEED)
    rws = []
    for w, req, r in mix:
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], device=local)
        rw.load(w)
        rws.append(rw)
    rays_per_step = sum(req.shape[0] * r for _, req, r in mix)
    tasks = sum((req.shape[0] * r // 32 + 7) // 8 * 8 for _, req, r in mix)   # 32-ray subgroups, 8-aligned
    out = {"config": dict(BATCH_WORKLOAD, rays_per_step=rays_per_step,
                          probes_per_step=int(sum(req.shape[0] for _, req, _ in mix)),
                          l2="flushed between steps (256 MiB write)")}
    with lum_gb300.RadianceBatch(rws) as b:
        for i, (w, req, r) in enumerate(mix):
            b.set_requests(i, req, lum_gb300.pass_params(rays=r, max_dist=128.0, blend=0.1))
        t0 = time.perf_counter()
        if tuning is None:
            tuning = b.autotune(repeats=3)
        else:   # fixed settings (profiling captures): guided divisor, chunk cap, march CTAs per SM
            b.set_tuning(*tuning)
            tuning = {"guided_div": tuning[0], "max_chunk": tuning[1], "march_ctas": tuning[2], "fixed": True}
        out["tuning"] = dict(tuning, seconds=round(time.perf_counter() - t0, 2))
        for k in range(warmup):
            b.run(k)
        b.synchronize()
        ms = []
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            b.run(k)
            b.synchronize()
            ms.append(b.last_ms())
        st = b.stats()
        batched = rays_per_step / (np.mean(ms) / 1000.0)
        for k in range(warmup):
            b.run_per_world(k)
        b.synchronize()
        pms = []
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            b.run_per_world(k)
            b.synchronize()
            pms.append(b.last_ms())
        plain = rays_per_step / (np.mean(pms) / 1000.0)
    for rw in rws:
        rw.close()
    out.update({"value": batched, "unit": "probe-rays/s", "ms_per_step": float(np.mean(ms)),
                "plain_value": plain, "plain_ms_per_step": float(np.mean(pms)),
                "speedup_vs_plain": batched / plain, "steps": steps,
                "ray_steps_per_s": st["steps"] / (ms[-1] / 1000.0),
                "gpu_launches_per_step": 1 + 2 * -(-tasks // BATCH_ROUND_TASKS)})
    return out


SERVE_WORKLOAD = {
    "workload": "relight serving: 64 resident terrain worlds, block counts lognormal in 8^3..64x64x32, "
                "Poisson stream of relight requests, each editing U(1%,5%) of its world's blocks "
                "(seeded block-type changes) and relighting the probes within 2 blocks of the edits, "
                "64 rays/probe, max_dist 128, blend 0.1, FP32, HBM budget 120 GB",
    "worlds": 64, "requests_per_rate": 10000, "radius": 2, "rays_per_probe": 64, "hbm_budget_gb": 120,
    "seed": SEED,
}


def _serve_trace(srv, reqs, arrivals, params_of, allow_shed=False):
    """Submits every request with its arrival time (offset into the future), serves them all and
    returns (latencies s, rays, span s) of the requests that ran (allow_shed: requests shed by a
    queueing bound are left out)."""
    import lum_gb300
    base = srv.now() + 0.5 + 2e-5 * len(reqs)
    for k, (w, e) in enumerate(reqs):
        srv.submit(w, e, params_of(k), base + float(arrivals[k]))
    late = srv.now() > base
    srv.run(timeout_s=600)
    d = srv.poll(len(reqs) + 16)
    ok = d["status"] == 0
    if allow_shed:
        ok_or_shed = ok | (d["status"] == lum_gb300._native.LUMRAD_ETIMEOUT)
        assert len(d) == len(reqs) and ok_or_shed.all(), "serving trace failed"
        d = d[ok]
    else:
        assert len(d) == len(reqs) and ok.all(), "serving trace failed"
    lat = d["done_s"] - d["arrival_s"]
    rays = int((d["probes"].astype(np.int64) * d["rays_per_probe"]).sum())
    span = float(d["done_s"].max() - d["arrival_s"].min())
    return lat, rays, span, late


def aux_leg(local: int, reps: int, with_cpu: bool):
    """The steps either side of the pass, each through the library's API on the GPU and, beside
    it, on the host cores through the oracle's restatement of the reference's own algorithm (the
    dirty-probe derivation, which the reference lacks, against this library's host path):
      update_list  the 27-neighbour update list of the demo world (65,536 blocks), list returned
                   to the host (the reference builds it on the CPU every frame)
      dirty_list   the probes within 2 blocks of a 1% edit of a 64x64x32 world, list returned
      shift        radiance scroll by (1, 1, 0): the demo world and a 512x512x64 one (16.8M blocks)
      gather       diffuse.frag's 8-probe gather at 1M points of the demo world, device buffers
      blockify     one frame of blockify + map of 8 rotated 32^3 models into the demo world
      frame        lumrad_update_radiance: one frame of the drop-in (device update list of the demo
                   world, then the pass over it) at the reference's 64 rays, max_dist 128
      precision    the demo step (8 passes in one call) with FP32, FP16, BF16 and RGB10A2 storage,
                   steps back to back (L2 not flushed)
    Device times are CUDA events on the context's stream around enqueued calls (shift, gather);
    calls that return a host result (lists, blockify) are timed wall-clock, synchronising."""
    import torch
    import lum_gb300
    hbm_peak, _ = load_peaks()
    dev = torch.device("cuda", local)
    world = worldgen.demo_world(SEED)
    rw = lum_gb300.RadianceWorld(world.dims, max_block_types=2048, device=local)   # room for the models' blocks
    rw.load(world)
    stream = torch.cuda.ExternalStream(rw.stream(), device=dev)
    lists = pass_lists(world.dims)
    rw.radiance_passes(lists, [lum_gb300.pass_params(rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=p)
                               for p in range(PASSES)])
    vol = rw.get_radiance()
    W = world.n_blocks

    def wall(fn, n):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n

    def device(fn, n):
        fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1000.0 / n

    def cpu_time(fn, n=3):
        fn()
        t0 = time.perf_counter()
        for _ in range(n):
            fn()
        return (time.perf_counter() - t0) / n

    oracle = None
    if with_cpu:
        import oracle as _oracle   # the CPU side only
        oracle = _oracle
    out = {"config": {"world": list(world.dims), "seed": SEED}}

    # f1: update list
    t = wall(rw.build_update_list, reps)
    n_list = int(rw.build_update_list().shape[0])
    e = {"us_per_call": t * 1e6, "blocks_per_s": W / t, "listed": n_list}
    if oracle:
        tc = cpu_time(lambda: oracle.update_list(world))
        e["cpu"] = {"us_per_call": tc * 1e6, "kind": "port", "cores": 1}
    out["update_list"] = e

    # f1: dirty probes of an edit request
    wd = worldgen.terrain_world((64, 64, 32), seed=SEED)
    edits = worldgen.edit_request(wd.dims, 0.01, seed=SEED, stream=0)
    with lum_gb300.RadianceWorld(wd.dims, max_block_types=wd.palette.shape[0], device=local) as rd:
        rd.load(wd)
        t = wall(lambda: rd.build_dirty_list(edits, 2), reps)
        n_dirty = int(rd.build_dirty_list(edits, 2).shape[0])
    e = {"us_per_call": t * 1e6, "edits": int(edits.shape[0]), "dirty_probes": n_dirty}
    tc = cpu_time(lambda: lum_gb300.dirty_probes(wd.dims, edits, 2), 5)
    e["cpu"] = {"us_per_call": tc * 1e6, "kind": "host path of this library (no reference counterpart)", "cores": 1}
    out["dirty_list"] = e

    # f2: radiance scroll, HBM-bound: 16 B read + 16 B written per block
    t = device(lambda: rw.shift_radiance(1, 1, 0), reps)
    e = {"us_per_call": t * 1e6, "gbs": 32.0 * W / t / 1e9}
    with lum_gb300.RadianceWorld((512, 512, 64), max_block_types=1, device=local) as rb:
        sb = torch.cuda.ExternalStream(rb.stream(), device=dev)

        def dev_big(n):
            rb.shift_radiance(1, 1, 0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(sb)
            for _ in range(n):
                rb.shift_radiance(1, 1, 0)
            e1.record(sb)
            e1.synchronize()
            return e0.elapsed_time(e1) / 1000.0 / n
        tb = dev_big(reps)
    wb = 512 * 512 * 64
    e["large"] = {"blocks": wb, "us_per_call": tb * 1e6, "gbs": 32.0 * wb / tb / 1e9,
                  "hbm_frac": 32.0 * wb / tb / 1e9 / hbm_peak}
    if oracle:
        tc = cpu_time(lambda: oracle.shift_radiance(vol, (1, 1, 0)))
        e["cpu"] = {"us_per_call": tc * 1e6, "kind": "port", "cores": 1}
    out["shift"] = e

    # f4: gather at 1M points inside the world
    n_pts = 1 << 20
    rng = np.random.default_rng(SEED)
    pos = rng.random((n_pts, 3)) * np.array(world.dims) * 16
    nrm = rng.normal(size=(n_pts, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    pts = np.concatenate([pos, nrm], axis=1).astype(np.float32)
    d_pts = torch.from_numpy(pts).to(dev)
    d_rgb = torch.empty((n_pts, 3), dtype=torch.float32, device=dev)
    t = device(lambda: rw.gather_device(d_pts.data_ptr(), n_pts, d_rgb.data_ptr()), reps)
    alg = (24 + 12 + 8 * 16) * n_pts
    e = {"points": n_pts, "us_per_call": t * 1e6, "points_per_s": n_pts / t, "gbs": alg / t / 1e9,
         "hbm_frac": alg / t / 1e9 / hbm_peak}
    if oracle:
        tc = cpu_time(lambda: oracle.gather(vol, pts), 1)
        e["cpu"] = {"us_per_call": tc * 1e6, "kind": "port", "cores": 1}
    out["gather"] = e

    # f3: blockify + map of 8 rotated 32^3 models
    mrng = np.random.default_rng(SEED + 1)
    model = ((mrng.random((32, 32, 32)) < 0.5) * mrng.integers(1, 256, (32, 32, 32))).astype(np.uint8)
    mid = rw.load_model(model)
    meshes = []
    for i in range(8):
        q = mrng.normal(size=4)
        q = tuple(float(x) for x in (q / np.linalg.norm(q)))
        meshes.append((mid, q, tuple(float(x) for x in mrng.random(3) * np.array(world.dims) * 16 * 0.8 + 40)))
    static = world.palette.shape[0]
    t = wall(lambda: rw.blockify(static, meshes), reps)
    e = {"meshes": len(meshes), "model_voxels": int(model.size), "us_per_call": t * 1e6}
    if oracle:
        pal = np.zeros((2048, 16, 16, 16), np.uint8)
        pal[:static] = world.palette
        tc = cpu_time(lambda: oracle.blockify(world.grid, pal, static, [model], meshes), 1)
        e["cpu"] = {"us_per_call": tc * 1e6, "kind": "port", "cores": 1}
    out["blockify"] = e

    # the drop-in frame: update list on the device, then the pass over all 51,992 listed probes
    rw.blockify(static, [])   # the origin world again
    fp = lum_gb300.pass_params(rays=64, max_dist=128.0, blend=0.1, time_seed=0)
    t = wall(lambda: rw.update_radiance(fp), reps)
    out["frame"] = {"us_per_call": t * 1e6, "probes": n_list, "rays_per_probe": 64,
                    "probe_rays_per_s": n_list * 64 / t}
    rw.close()

    # the demo step at each radiance storage precision (C4: FP16/BF16 storage, FP32 arithmetic)
    plist = [lum_gb300.pass_params(rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=p) for p in range(PASSES)]
    rays_step = sum(l.shape[0] for l in lists) * RAYS
    prec = {}
    for name in ("fp32", "fp16", "bf16", "rgb10a2"):
        with lum_gb300.RadianceWorld(world.dims, max_block_types=world.palette.shape[0], precision=name,
                                     device=local) as rp:
            rp.load(world)
            for p, l in enumerate(lists):
                rp.upload_requests(p, l)
            sp = torch.cuda.ExternalStream(rp.stream(), device=dev)
            rp.radiance_passes_resident(list(range(PASSES)), plist)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(sp)
            for _ in range(reps):
                rp.radiance_passes_resident(list(range(PASSES)), plist)
            e1.record(sp)
            e1.synchronize()
            t = e0.elapsed_time(e1) / 1000.0 / reps
            prec[name] = {"ms_per_step": t * 1e3, "probe_rays_per_s": rays_step / t}
    out["precision"] = prec
    return out


def serving_leg(local: int, n_requests: int = 10000, rates=(2000.0, 5000.0, 10000.0, 20000.0), inflight: int = 4):
    """Continuous batching of relight requests over 64 resident worlds, at each arrival rate and
    saturated (every request due at once); the plain form (one request per launch, one launch
    at a time) saturated, for comparison."""
    import lum_gb300
    worlds = worldgen.serving_worlds(SERVE_WORKLOAD["worlds"], seed=SEED)
    rws = []
    for w in worlds:
        rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], device=local)
        rw.load(w)
        rws.append(rw)
    # requests: uniform world, U(1%,5%) edits
    u = worldgen.uniform(SEED, 9301, 2 * n_requests).reshape(n_requests, 2)
    reqs = []
    for k in range(n_requests):
        wi = int(u[k, 0] * len(worlds))
        reqs.append((wi, worldgen.edit_request(worlds[wi].dims, 0.01 + 0.04 * u[k, 1], seed=SEED, stream=k)))

    def params_of(k):
        return lum_gb300.pass_params(rays=SERVE_WORKLOAD["rays_per_probe"], max_dist=128.0, blend=0.1, time_seed=k)

    def summary(lat, rays, span, late):
        return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "probe_rays_per_s": rays / span, "requests_per_s": len(lat) / span, "span_s": span,
                "submitted_late": bool(late)}

    out = {"config": dict(SERVE_WORKLOAD, requests_per_rate=n_requests,
                          world_blocks_total=int(sum(w.n_blocks for w in worlds)),
                          l2="inputs resident; no flush (a serving loop runs warm)")}
    budget = SERVE_WORKLOAD["hbm_budget_gb"] * 1e9
    srv = lum_gb300.RadianceServer(device=local, hbm_budget_bytes=budget, max_inflight=inflight)
    for rw in rws:
        srv.add_world(rw)
    # warm-up: a short saturated trace
    _serve_trace(srv, reqs[:200], np.zeros(200), params_of)
    sweep = []
    for rate in rates:
        arr = worldgen.poisson_arrivals(n_requests, rate, seed=SEED + int(rate))
        sweep.append(dict(summary(*_serve_trace(srv, reqs, arr, params_of)), rate_per_s=rate))
    sat = summary(*_serve_trace(srv, reqs, np.zeros(n_requests), params_of))
    st = srv.stats()
    srv.close()
    # overload with a queueing bound: requests that waited past max_queue_ms are shed, the rest
    # keep a bounded latency
    bounded = None
    if rates:
        bound_ms = 2.0
        bsrv = lum_gb300.RadianceServer(device=local, hbm_budget_bytes=budget, max_inflight=inflight,
                                        max_queue_ms=bound_ms)
        for rw in rws:
            bsrv.add_world(rw)
        _serve_trace(bsrv, reqs[:200], np.zeros(200), params_of, allow_shed=True)
        shed0 = bsrv.stats()["shed"]
        rate = max(rates)
        arr = worldgen.poisson_arrivals(n_requests, rate, seed=SEED + int(rate))
        lat, rays, span, late = _serve_trace(bsrv, reqs, arr, params_of, allow_shed=True)
        shed = bsrv.stats()["shed"] - shed0
        bounded = dict(summary(lat, rays, span, late), rate_per_s=rate, max_queue_ms=bound_ms,
                       shed=int(shed), shed_fraction=shed / n_requests)
        bsrv.close()
    plain = lum_gb300.RadianceServer(device=local, hbm_budget_bytes=budget, max_inflight=1,
                                     max_requests_per_launch=1)
    for rw in rws:
        plain.add_world(rw)
    _serve_trace(plain, reqs[:200], np.zeros(200), params_of)
    psat = summary(*_serve_trace(plain, reqs, np.zeros(n_requests), params_of))
    plain.close()
    # the same trace through the device-resident request loop (one CUDA graph polling a ring)
    dev = lum_gb300.RadianceServer(device=local, hbm_budget_bytes=budget, device_loop=True)
    for rw in rws:
        dev.add_world(rw)
    _serve_trace(dev, reqs[:200], np.zeros(200), params_of)
    dsweep = []
    for rate in rates:
        arr = worldgen.poisson_arrivals(n_requests, rate, seed=SEED + int(rate))
        dsweep.append(dict(summary(*_serve_trace(dev, reqs, arr, params_of)), rate_per_s=rate))
    dsat = summary(*_serve_trace(dev, reqs, np.zeros(n_requests), params_of))
    dst = dev.stats()
    dev.close()
    for rw in rws:
        rw.close()
    out.update({"value": sat["probe_rays_per_s"], "unit": "probe-rays/s", "sweep": sweep, "saturated": sat,
                "plain_saturated": psat, "speedup_vs_plain": sat["probe_rays_per_s"] / psat["probe_rays_per_s"],
                "launches": st["launches"], "max_requests_in_launch": st["max_requests_in_launch"],
                "resident_gb": st["resident_bytes"] / 1e9, "peak_inflight_mb": st["peak_inflight_bytes"] / 1e6,
                "max_inflight": inflight, "overload_bounded": bounded,
                "device_loop": {"sweep": dsweep, "saturated": dsat, "graph_launches": dst["launches"],
                                "how": "one CUDA graph (WHILE node) per busy period: admit -> edits -> dirty "
                                       "lists -> pass -> completions, polling a page-locked request ring"}})
    return out


def max_over_ranks(v: float, pg, device) -> float:
    """The largest of every rank's v: the slowest replica sets the job's time."""
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: float, world_size: int, seconds: float) -> float:
    """Whole-job throughput of replicas: every rank processes units_per_rank in `seconds` (the max)."""
    return world_size * units_per_rank / seconds


def dist_setup(args):
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world_size > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        pg = dist
    return rank, local, world_size, pg


def run_reference(args, rank, world_size, pg):
    """The reference's implementation of the same workload on the host cores: Lum's
    radiance.comp compiled as C++ (its Vulkan path is unavailable on this machine), one process per
    core; the port (OpenMP) where that cannot be built."""
    if rank != 0:
        return
    world = worldgen.demo_world(SEED)
    lists = pass_lists(world.dims)
    run, kind, cores = reference_runner(world)
    prev = np.zeros(world.grid.shape + (3,), dtype=np.float32)
    t_total = 0.0
    rays_total = 0
    for step in range(args.warmup + args.steps):
        cur = prev
        t0 = time.perf_counter()
        for p in range(PASSES):
            cur = run(lists[p], cur, p)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            t_total += dt
            rays_total += sum(l.shape[0] for l in lists) * RAYS
    run.close()
    value = rays_total / t_total
    sample = "full steps: 8 passes x 6554 probes x 256 rays"
    line = {"metric": "probe-rays/s", "value": value, "unit": "probe-rays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded value-noise terrain, splitmix64)", "impl": "reference",
            "config": dict(WORKLOAD, l2="flushed between steps (256 MiB write)",
                           parallelism="replicas" if world_size > 1 else "single GPU"),
            "cpu_baseline": {"value": value, "unit": "probe-rays/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "probe-rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": ("Lum's shaders/radiance.comp compiled as C++ from its source, one process per host core; "
                     "its Vulkan path is unavailable on this box") if kind == "reference" else
                    "the CPU restatement (port) of radiance.comp, OpenMP over all host cores"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--legs", default="demo,batched,serving,aux",
                    help="comma list of legs: demo (the headline line), batched (the mixed-size batch), "
                         "serving (relight requests), aux (the steps either side of the pass)")
    ap.add_argument("--serve-requests", type=int, default=10000, help="requests per arrival rate (serving leg)")
    ap.add_argument("--batch-tuning", default=None, type=lambda s: tuple(int(x) for x in s.split(",")),
                    help="fixed batch settings G,C,M (guided divisor, chunk cap, march CTAs per SM) instead of "
                         "the autotuner (for profiling captures)")
    args = ap.parse_args()
    legs = set(args.legs.split(","))
    rank, local, world_size, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world_size, pg)
        return

    import torch
    import lum_gb300

    torch.cuda.set_device(local)
    if "demo" not in legs:   # a diagnostics run of other legs only (profiling); not the headline line
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
        out = {"diagnostics": True}
        if "batched" in legs:
            out["batched"] = batched_leg(local, max(3, args.steps // 2), args.warmup, flush, args.batch_tuning)
        if "serving" in legs:
            out["serving"] = serving_leg(local, n_requests=args.serve_requests)
        if "aux" in legs:
            out["aux"] = aux_leg(local, 20, not args.no_cpu and rank == 0)
        if rank == 0:
            print(json.dumps(out))
        return
    world = worldgen.demo_world(SEED)
    lists = pass_lists(world.dims)
    probes_per_step = sum(l.shape[0] for l in lists)
    rays_per_step = probes_per_step * RAYS

    # ---------------------------------------------------------------- resident (value)
    rw = lum_gb300.RadianceWorld(world.dims, max_block_types=world.palette.shape[0], device=local)
    rw.load(world)
    for p, l in enumerate(lists):
        rw.upload_requests(p, l)
    stream = torch.cuda.ExternalStream(rw.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    def params(p):
        return lum_gb300.pass_params(rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=p)

    # exact per-pass counters (identical on every run: the traversal is deterministic)
    pass_bytes = []
    pass_steps = []
    for p in range(PASSES):
        rw.radiance_pass_resident(p, params(p))
        st = rw.pass_stats()
        pass_steps.append(st["steps"])
        pass_bytes.append(algorithmic_bytes(st["steps"], st["hits"], st["probes"]))
    slots = list(range(PASSES))
    plist = [params(p) for p in range(PASSES)]

    def step_resident():
        # the step's 8 passes in one call: one march launch for all of them, then each pass's
        # finalize in order (bit-identical to 8 single passes); one kernel-time entry
        rw.radiance_passes_resident(slots, plist)
        return 1

    for _ in range(args.warmup):
        step_resident()
    rw.synchronize()

    def timed_steps(run, n):
        st, kt_all = [], []
        for _ in range(n):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            k = run()
            e1.record(stream)
            kt_all.append(float(rw.kernel_times(k).sum()))   # synchronises after the step
            st.append(e0.elapsed_time(e1))
        return st, kt_all

    def single_step():
        for p in range(PASSES):
            rw.radiance_pass_resident(p, params(p))
        return PASSES

    with ClockSampler(local) as clocks:
        # ~1.5 s of the same passes first, so the clock samples see the GPU under this load
        soak_end = time.perf_counter() + 1.5
        while time.perf_counter() < soak_end:
            step_resident()
            rw.synchronize()
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        step_ms, kernel_ms = timed_steps(step_resident, args.steps)
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
        # the drop-in's one-pass-per-call path (a frame's update_radiance) on the same passes
        single_ms, single_kernel_ms = timed_steps(single_step, args.steps)
    dev = f"cuda:{local}"
    total_ms = max_over_ranks(float(sum(step_ms)), pg, dev)
    value = job_value(args.steps * rays_per_step, world_size, total_ms / 1000.0)
    single_total_ms = max_over_ranks(float(sum(single_ms)), pg, dev)

    hbm_peak, peak_kind = load_peaks()
    l2_peak = l2_read_gbs(local)
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count
    bytes_per_launch = float(np.sum(pass_bytes))       # the step's 8 passes: one march launch
    kern_avg_s = float(np.mean(kernel_ms)) / 1000.0    # march + 8 finalize launches of a step
    achieved = bytes_per_launch / kern_avg_s / 1e9

    # ---------------------------------------------------------------- end to end (e2e)
    rw2 = lum_gb300.RadianceWorld(world.dims, max_block_types=world.palette.shape[0], device=local)
    rw2.load(world)
    # the caller's request lists (back to back in one array) and result buffer in page-locked
    # host memory
    pinned = torch.from_numpy(np.concatenate(lists)).pin_memory()
    host_lists = pinned.numpy()                       # the 8 lists back to back
    counts = [l.shape[0] for l in lists]
    pparams = (lum_gb300.PassParams * PASSES)(*plist)
    out_t = torch.empty(world.grid.shape + (3,), dtype=torch.float32).pin_memory()
    host_out = out_t.numpy()
    for _ in range(max(1, args.warmup)):
        rw2.radiance_passes_packed(host_lists, counts, pparams)
        rw2.get_radiance(out=host_out)
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rw2.radiance_passes_packed(host_lists, counts, pparams)
        rw2.get_radiance(out=host_out)
        e2e_s += time.perf_counter() - t0
    e2e_value = job_value(args.steps * rays_per_step, world_size, max_over_ranks(e2e_s, pg, dev))
    h2d = int(sum(l.shape[0] * 8 for l in lists))
    d2h = int(world.n_blocks * 12)   # the volume as packed RGB floats

    batched = None
    if "batched" in legs:
        batched = batched_leg(local, max(3, args.steps // 2), args.warmup, flush, args.batch_tuning)
    serving = None
    if "serving" in legs:
        serving = serving_leg(local, n_requests=args.serve_requests)
    aux = None
    if "aux" in legs:
        aux = aux_leg(local, 20, not args.no_cpu and rank == 0)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(world, lists)

    clk = clocks.summary()
    sm_hz = (clk["sm_mhz"] or clk["sm_max_mhz"] or 2070.0) * 1e6
    issue_peak = SCHEDULERS_PER_SM * num_sms * sm_hz              # warp instructions per second
    issue_achieved = NCU_WARP_INST_PER_STEP / kern_avg_s
    if rank == 0:
        line = {
            "metric": "probe-rays/s", "value": value, "unit": "probe-rays/s", "n_gpus": world_size,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded value-noise terrain, splitmix64)",
            "config": dict(WORKLOAD, l2="flushed between steps (256 MiB write)",
                           parallelism="replicas" if world_size > 1 else "single GPU"),
            "e2e": {"value": e2e_value, "unit": "probe-rays/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "issue", "achieved": issue_achieved, "peak": issue_peak, "unit": "warp-inst/s",
                         "frac": issue_achieved / issue_peak, "traffic": NCU_DRAM_BYTES_PER_STEP,
                         "peak_kind": f"4 schedulers x {num_sms} SMs x the sampled SM clock",
                         "warp_inst_per_step": NCU_WARP_INST_PER_STEP, "kernel_ms_avg": kern_avg_s * 1e3,
                         "launch": "one step: a march launch over its 8 passes + 8 finalize launches",
                         "ray_steps_per_s": float(np.sum(pass_steps)) / kern_avg_s,
                         "hbm": {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                                 "peak_kind": peak_kind, "bytes_per_launch": bytes_per_launch,
                                 "traffic": NCU_DRAM_BYTES_PER_STEP},
                         "l2": {"achieved": achieved, "peak": l2_peak, "unit": "GB/s", "frac": achieved / l2_peak,
                                "peak_kind": "measured in this run: L2-resident read (64 row sums over one 24 MiB "
                                             "array, one launch, best of 5)",
                                "traffic": NCU_L2_BYTES_PER_STEP}},
            "single_pass": {"value": job_value(args.steps * rays_per_step, world_size, single_total_ms / 1000.0),
                            "unit": "probe-rays/s", "ms_per_step": single_total_ms / args.steps,
                            "kernel_ms_per_pass": float(np.mean(single_kernel_ms)) / PASSES,
                            "path": "lumrad_radiance_pass_resident once per pass (one frame's update)"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": (1 + PASSES) * args.steps,   # one march + a finalize per pass, per step
            "batched": batched,
            "serving": serving,
            "aux": aux,
        }
        print(json.dumps(line))
    rw.close()
    rw2.close()
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
