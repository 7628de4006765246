"""Radiance storage precision at full size: FP32, FP16, BF16 and the reference's own 10-bit UNORM
(A2B10G10R10) storage, all with FP32 arithmetic, against the FP64 oracle (FP32 traversal, FP64
shading, no storage rounding), per pass.

Workload: the 64x64x32-block terrain world (32 block types), every probe updated each pass,
256 rays per probe, max_dist 256, blend 0.1, 16 successive passes from a zero volume.  Hit records
of every precision are compared bit for bit with the FP64 oracle's on a 2% probe subset.

Error of a channel: |gpu - oracle| / max(|oracle|, 1e-3) (radiance is clamped to [0, 1]; the
floor keeps near-black probes from dominating).  Prints a markdown table.

Run on a GPU machine:  python -m tests.precision_report
"""
from __future__ import annotations

import sys
import time

import numpy as np

from lum_gb300 import worldgen

DIMS = (64, 64, 32)
PASSES = 16
RAYS = 256
MAX_DIST = 256.0
BLEND = 0.1
FLOOR = 1e-3


def measure(dims=DIMS, passes=PASSES, precisions=("fp32", "fp16", "bf16", "rgb10a2")):
    """Runs the workload; returns {"rows": {prec: [(max rel, RMS rel, max abs) per pass]},
    "hits_ok": {prec: bool}, "probes", "subset", "oracle_s", "threads"}."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world(dims, seed=1234, n_types=32)
    req = worldgen.all_probes(w.dims)
    sub = worldgen.probe_subset(w.dims, 0.02, seed=1234, stream=5)
    zero = np.zeros(w.grid.shape + (3,), dtype=np.float32)

    t0 = time.perf_counter()
    ref = []
    cur = zero.astype(np.float64)
    for p in range(passes):
        cur, _, _ = oracle.radiance_pass(w, req, rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=p, prev=cur,
                                         precision="f64")
        ref.append(cur)
    _, ref_hits, _ = oracle.radiance_pass(w, sub, rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=0,
                                          prev=zero.astype(np.float64), precision="f64", record_hits=True)
    t_oracle = time.perf_counter() - t0

    rows = {}
    hits_ok = {}
    for prec in precisions:
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=prec) as rw:
            rw.load(w)
            rw.radiance_pass(sub, lum_gb300.pass_params(rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=0,
                                                        record_hits=True))
            hits_ok[prec] = rw.get_hits().tobytes() == ref_hits.tobytes()
            rw.set_radiance(zero)
            out = []
            for p in range(passes):
                rw.radiance_pass(req, lum_gb300.pass_params(rays=RAYS, max_dist=MAX_DIST, blend=BLEND, time_seed=p))
                g = rw.get_radiance().astype(np.float64)
                d = np.abs(g - ref[p])
                rel = d / np.maximum(np.abs(ref[p]), FLOOR)
                out.append((float(rel.max()), float(np.sqrt(np.mean(rel ** 2))), float(d.max())))
            rows[prec] = out
    return {"rows": rows, "hits_ok": hits_ok, "probes": int(req.shape[0]), "subset": int(sub.shape[0]),
            "oracle_s": t_oracle, "threads": oracle.max_threads()}


def main(dims=DIMS, passes=PASSES) -> int:
    m = measure(dims, passes)
    rows, hits_ok, t_oracle = m["rows"], m["hits_ok"], m["oracle_s"]
    print(f"World {dims[0]}x{dims[1]}x{dims[2]} blocks, {m['probes']} probes x {RAYS} rays, max_dist {MAX_DIST:g}, "
          f"blend {BLEND}, {passes} passes from zero; FP64 oracle {t_oracle:.1f} s on {m['threads']} threads.")
    print(f"Hit records bit-exact vs the FP64 oracle on {m['subset']} probes: "
          + ", ".join(f"{k} {'yes' if v else 'NO'}" for k, v in hits_ok.items()))
    print()
    precs = list(rows)
    print("| pass | " + " | ".join(f"{k.upper()} max rel | {k.upper()} RMS rel" for k in precs) + " |")
    print("|---:|" + "---:|---:|" * len(precs))
    for p in range(passes):
        cells = []
        for prec in precs:
            mx, rms, _ = rows[prec][p]
            cells += [f"{mx:.2e}", f"{rms:.2e}"]
        print(f"| {p + 1} | " + " | ".join(cells) + " |")
    print()
    print("Max absolute error, worst pass: " + ", ".join(f"{k} {max(r[2] for r in rows[k]):.2e}" for k in precs))
    worst = {k: max(r[0] for r in v) for k, v in rows.items()}
    print()
    print("Worst over all passes (max rel): " + ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
    return 0 if all(hits_ok.values()) else 1


if __name__ == "__main__":
    sys.exit(main())
