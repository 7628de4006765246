"""Several passes in one call (lumrad_radiance_passes[_resident]): the marches of consecutive
passes share one launch and the finalize steps run in order.  Each case equals the same passes
run one call at a time, bit for bit, and the oracle's chained passes within 1e-5."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _passes(w):
    """Eight passes with different lists, ray counts (one subgroup, subgroups combined in one CTA,
    3 subgroups combined through global scratch, 16 subgroups), bounds, blends and slicing, and
    an empty list."""
    lists = [worldgen.probe_subset(w.dims, f, seed=40, stream=i) for i, f in
             enumerate((0.3, 1.0, 0.5, 0.2, 0.7, 0.4, 0.6, 0.9))]
    lists[5] = lists[5][:0]
    spec = [dict(rays=64, max_dist=96.0, blend=0.1), dict(rays=256, max_dist=96.0, blend=0.2),
            dict(rays=96, max_dist=96.0, blend=0.1), dict(rays=512, max_dist=64.0, blend=0.3),
            dict(rays=32, max_dist=64.0, blend=0.1), dict(rays=64, max_dist=64.0, blend=0.1),
            dict(rays=128, max_dist=128.0, blend=0.05, size=2, shift=1), dict(rays=64, max_dist=128.0, blend=0.1)]
    for i, s in enumerate(spec):
        s["time_seed"] = 11 + 3 * i
    return lists, spec


def _run(w, lists, spec, prev, mode, precision="fp32"):
    import lum_gb300
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        params = [lum_gb300.pass_params(**s) for s in spec]
        steps = hits = probes = 0
        if mode == "single":
            for l, p in zip(lists, params):
                rw.radiance_pass(l, p)
                st = rw.pass_stats()
                steps += st["steps"]; hits += st["hits"]; probes += st["probes"]
        elif mode == "multi":
            rw.radiance_passes(lists, params)
            st = rw.pass_stats()
            steps, hits, probes = st["steps"], st["hits"], st["probes"]
            assert rw.kernel_times(64).shape[0] == 1   # one entry for the call
        else:
            for i, l in enumerate(lists):
                rw.upload_requests(10 + i, l)
            rw.radiance_passes_resident([10 + i for i in range(len(lists))], params)
            st = rw.pass_stats()
            steps, hits, probes = st["steps"], st["hits"], st["probes"]
        return rw.get_radiance(), (steps, hits, probes)


@pytest.mark.parametrize("mode", ["multi", "resident"])
def test_passes_equal_single_passes_and_oracle(mode):
    import oracle
    w = worldgen.terrain_world((11, 9, 6), seed=41, n_types=12)
    lists, spec = _passes(w)
    prev = random_prev(w, seed=42)
    single, st_single = _run(w, lists, spec, prev, "single")
    got, st = _run(w, lists, spec, prev, mode)
    assert got.tobytes() == single.tobytes()
    assert st == st_single
    cur = prev
    for l, s in zip(lists, spec):
        cur, _, _ = oracle.radiance_pass(w, l, prev=cur, **s)
    assert rel_err(got, cur).max() <= RTOL


@pytest.mark.parametrize("precision", ["fp16", "bf16", "rgb10a2"])
def test_passes_low_precision(precision):
    w = worldgen.terrain_world((9, 8, 5), seed=43, n_types=10)
    lists, spec = _passes(w)
    prev = random_prev(w, seed=44)
    single, st_single = _run(w, lists, spec, prev, "single", precision)
    got, st = _run(w, lists, spec, prev, "multi", precision)
    assert got.tobytes() == single.tobytes()
    assert st == st_single


def test_passes_split_into_launches_and_rounds():
    """Passes larger than one shared march launch: 2^19 tasks each (one launch apiece) and 2^20
    tasks (rounds, as a single pass runs), between smaller ones."""
    w = worldgen.terrain_world((64, 64, 32), seed=45, n_types=24)
    allp = worldgen.all_probes(w.dims)
    small = worldgen.probe_subset(w.dims, 0.05, seed=46)
    lists = [small, allp, allp, small, allp, small]
    spec = [dict(rays=64), dict(rays=128), dict(rays=128), dict(rays=32), dict(rays=256), dict(rays=64)]
    for i, s in enumerate(spec):
        s.update(max_dist=48.0, blend=0.1, time_seed=i)
    prev = random_prev(w, seed=47)
    single, st_single = _run(w, lists, spec, prev, "single")
    got, st = _run(w, lists, spec, prev, "multi")
    assert got.tobytes() == single.tobytes()
    assert st == st_single


def test_passes_bad_arguments():
    import lum_gb300
    w = worldgen.terrain_world((4, 4, 4), seed=48)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        req = worldgen.all_probes(w.dims)
        with pytest.raises(lum_gb300.LumRadError):
            rw.radiance_passes([req], [lum_gb300.pass_params(rays=64, size=0)])
        with pytest.raises(lum_gb300.LumRadError):
            rw.radiance_passes([req], [lum_gb300.pass_params(rays=64, record_hits=True)])
        with pytest.raises(lum_gb300.LumRadError):
            rw.radiance_passes_resident([3], [lum_gb300.pass_params(rays=64)])
        rw.radiance_passes([], [])   # nothing to do
        rw.radiance_passes([req], [lum_gb300.pass_params(rays=64)])   # the context is still usable
        assert rw.get_radiance().max() > 0.0


def test_read_back_into_pinned_buffer():
    """get_radiance into a page-locked array (copied to directly) equals the staged read-back."""
    import torch
    import lum_gb300
    w = worldgen.terrain_world((7, 6, 5), seed=49)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.radiance_passes([worldgen.all_probes(w.dims)] * 2,
                           [lum_gb300.pass_params(rays=64, blend=0.2, time_seed=s) for s in (1, 2)])
        staged = rw.get_radiance()
        t = torch.zeros(w.grid.shape + (3,), dtype=torch.float32).pin_memory()
        got = rw.get_radiance(out=t.numpy())
        assert got.tobytes() == staged.tobytes()
        assert t.numpy().tobytes() == staged.tobytes()
        with pytest.raises(ValueError):
            rw.get_radiance(out=np.zeros(3, np.float32))


def test_page_locked_lists():
    """Lists in page-locked memory (adjacent in one array, apart, or mixed with pageable ones) are
    copied straight from the caller's arrays; the volume equals the staged copies' one."""
    import torch
    import lum_gb300
    w = worldgen.terrain_world((9, 7, 5), seed=50)
    lists = [worldgen.probe_subset(w.dims, f, seed=51, stream=i) for i, f in enumerate((0.4, 0.0, 0.8, 0.5))]
    params = [lum_gb300.pass_params(rays=64, blend=0.1, time_seed=20 + i) for i in range(4)]
    flat = torch.from_numpy(np.concatenate(lists)).pin_memory()
    cuts = np.cumsum([0] + [l.shape[0] for l in lists])
    adjacent = [flat.numpy()[cuts[i]:cuts[i + 1]] for i in range(4)]
    apart_t = [torch.from_numpy(l.copy()).pin_memory() for l in lists]
    apart = [t.numpy() for t in apart_t]
    mixed = [apart[0], lists[1], apart[2], lists[3]]
    out = []
    for ls in (lists, adjacent, apart, mixed):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            rw.radiance_passes(ls, params)
            rw.radiance_passes(ls, params)   # the stream busy or idle: either copy path
            out.append(rw.get_radiance())
    for o in out[1:]:
        assert o.tobytes() == out[0].tobytes()


def test_more_passes_than_one_launch_marks():
    """40 passes in one call: the marches share launches of at most 32 passes (one mark bit per
    pass and probe), so the call spans two; lists hold entries outside the world (skipped, as the
    single pass skips them) and repeat probes across passes.  Equal to single passes, bit for bit,
    and a second call (the marks cleared by the first) equal again."""
    w = worldgen.terrain_world((8, 7, 5), seed=52, n_types=10)
    rng = np.random.default_rng(53)
    lists = []
    for i in range(40):
        l = worldgen.probe_subset(w.dims, 0.05 + 0.02 * (i % 7), seed=54, stream=i)
        bad = np.array([[-1, 0, 0, 0], [w.dims[0], 1, 1, 0], [2, w.dims[1], 0, 0], [0, 0, -3, 0]], np.int16)
        l = np.concatenate([l, bad[rng.permutation(4)[: i % 3]]])
        lists.append(np.ascontiguousarray(l[rng.permutation(l.shape[0])]))
    spec = [dict(rays=(32, 64, 128)[i % 3], max_dist=64.0, blend=0.15, time_seed=100 + i) for i in range(40)]
    prev = random_prev(w, seed=55)
    single, st_single = _run(w, lists, spec, prev, "single")
    got, st = _run(w, lists, spec, prev, "resident")
    assert got.tobytes() == single.tobytes()
    assert st == st_single
    import lum_gb300
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        params = [lum_gb300.pass_params(**s) for s in spec]
        rw.radiance_passes(lists, params)
        rw.radiance_passes(lists[:5], params[:5])
        twice = rw.get_radiance()
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        for l, s in zip(lists + lists[:5], spec + spec[:5]):
            rw.radiance_pass(l, lum_gb300.pass_params(**s))
        assert twice.tobytes() == rw.get_radiance().tobytes()


def test_back_to_back_calls_equal_synchronised_calls():
    """Pass calls right after one another start their march in the previous pass's finalize tail
    (the rays in the other buffer, the pass start after a wait): one-pass and several-pass calls
    back to back, with an empty pass, an edit, an upload and a read-back between some of them,
    equal the same calls each followed by a synchronisation, bit for bit, and the oracle's chain
    within 1e-5."""
    import dataclasses

    import lum_gb300
    import oracle
    w = worldgen.terrain_world((12, 10, 6), seed=56, n_types=12)
    lists = [worldgen.probe_subset(w.dims, f, seed=57, stream=i) for i, f in enumerate((0.3, 0.6, 0.2, 0.5, 0.4, 0.7))]
    spec = [dict(rays=(64, 128, 256, 32, 64, 128)[i], max_dist=80.0, blend=0.1 + 0.02 * i, time_seed=30 + i)
            for i in range(6)]
    edit = (3, 4, 2, 7)
    prev = random_prev(w, seed=58)

    def run(sync):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            rw.set_radiance(prev)
            for i, l in enumerate(lists):
                rw.upload_requests(i, l)
            rw.upload_requests(6, lists[0][:0])   # an empty list: a pass of copies only
            params = [lum_gb300.pass_params(**s) for s in spec]
            steps = [lambda: rw.radiance_pass_resident(0, params[0]),
                     lambda: rw.radiance_pass_resident(6, params[1]),
                     lambda: rw.radiance_pass_resident(1, params[1]),
                     lambda: rw.radiance_passes_resident([2, 3], params[2:4]),
                     lambda: rw.radiance_pass_resident(4, params[4]),
                     lambda: rw.set_world_block(*edit),
                     lambda: rw.radiance_pass_resident(5, params[5]),
                     lambda: rw.radiance_passes_resident([0, 1], params[:2]),
                     lambda: rw.get_radiance(),
                     lambda: rw.radiance_pass_resident(2, params[2]),
                     lambda: rw.radiance_passes_resident([3, 4, 5], params[3:6])]
            for f in steps:
                f()
                if sync:
                    rw.synchronize()
            return rw.get_radiance()

    fast, slow = run(False), run(True)
    assert fast.tobytes() == slow.tobytes()
    cur = prev
    grid = w.grid
    order = [0, 1, 2, 3, 4, "edit", 5, 0, 1, 2, 3, 4, 5]
    for k in order:
        if k == "edit":
            grid = grid.copy()
            grid[edit[2], edit[1], edit[0]] = edit[3]
            continue
        cur, _, _ = oracle.radiance_pass(dataclasses.replace(w, grid=grid), lists[k], prev=cur, **spec[k])
    assert rel_err(fast, cur).max() <= RTOL


def test_kernel_times_from_device_timestamps():
    """Each pass's kernel time comes from timestamps its own kernels write (no events between the
    launches): positive for passes with tasks, zero for an empty pass, one entry per call."""
    import lum_gb300
    w = worldgen.terrain_world((16, 16, 8), seed=59, n_types=12)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        allp = worldgen.all_probes(w.dims)
        rw.upload_requests(0, allp)
        rw.upload_requests(1, allp[:0])
        p = lum_gb300.pass_params(rays=128, max_dist=64.0, blend=0.1)
        for _ in range(3):
            rw.radiance_pass_resident(0, p)
        rw.radiance_pass_resident(1, p)
        rw.radiance_passes_resident([0, 0], [p, p])
        kt = rw.kernel_times(64)
        assert kt.shape[0] == 5
        assert (kt[:3] > 0.0).all() and kt[3] == 0.0 and kt[4] > 0.0
        assert (kt < 1000.0).all()
        assert rw.pass_stats()["gpu_ms"] > 0.0


def test_packed_lists_equal_separate_lists():
    """radiance_passes_packed (lists back to back in one array, a zero-length one among them, in
    page-locked memory or not) equals radiance_passes over the separate lists, bit for bit."""
    import torch
    import lum_gb300
    w = worldgen.terrain_world((9, 8, 6), seed=60, n_types=10)
    lists = [worldgen.probe_subset(w.dims, f, seed=61, stream=i) for i, f in enumerate((0.4, 0.0, 0.7, 0.3))]
    lists[1] = lists[1][:0]
    params = [lum_gb300.pass_params(rays=(64, 32, 128, 64)[i], blend=0.1, time_seed=70 + i) for i in range(4)]
    packed = np.ascontiguousarray(np.concatenate(lists))
    counts = [l.shape[0] for l in lists]
    out = []
    for mode in ("lists", "packed", "packed-pinned"):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            if mode == "lists":
                rw.radiance_passes(lists, params)
            elif mode == "packed":
                rw.radiance_passes_packed(packed, counts, params)
            else:
                pinned = torch.from_numpy(packed.copy()).pin_memory()
                rw.radiance_passes_packed(pinned.numpy(), counts, (lum_gb300.PassParams * 4)(*params))
            out.append(rw.get_radiance())
    assert out[1].tobytes() == out[0].tobytes()
    assert out[2].tobytes() == out[0].tobytes()


def test_update_radiance_between_dependent_passes():
    """Frames of lumrad_update_radiance (the list built on the device) between one-pass calls over
    resident lists, back to back, equal the same calls each followed by a synchronisation."""
    import lum_gb300
    w = worldgen.terrain_world((14, 12, 6), seed=62, n_types=12)
    lists = [worldgen.probe_subset(w.dims, f, seed=63, stream=i) for i, f in enumerate((0.3, 0.5, 0.2))]
    prev = random_prev(w, seed=64)

    def run(sync):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            rw.set_radiance(prev)
            for i, l in enumerate(lists):
                rw.upload_requests(i, l)
            steps = []
            for k in range(3):
                steps.append(lambda k=k: rw.radiance_pass_resident(k, lum_gb300.pass_params(rays=64, blend=0.2,
                                                                                              time_seed=10 + k)))
                steps.append(lambda k=k: rw.update_radiance(lum_gb300.pass_params(rays=32, blend=0.1,
                                                                                  time_seed=20 + k)))
            steps.append(lambda: rw.radiance_pass_resident(0, lum_gb300.pass_params(rays=128, time_seed=30)))
            for f in steps:
                f()
                if sync:
                    rw.synchronize()
            return rw.get_radiance()

    assert run(False).tobytes() == run(True).tobytes()
