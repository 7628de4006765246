"""The workloads at their full sizes, through properties that do not need the oracle to redo the
whole job: a full demo-scale pass against the oracle (1.68M rays), determinism of a full step,
the 256-world batch equal to its worlds run one by one, a full 64x64x32 pass against the oracle,
a radiance scroll round trip, and the 64-world server equal to each world served alone."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, rel_err

pytestmark = pytest.mark.gpu

SEED = 1234


def _demo_lists(dims):
    return [worldgen.probe_subset(dims, 0.1, seed=SEED, stream=p) for p in range(8)]


def test_demo_scale_pass_matches_oracle():
    """One pass of the demo-scale workload (6,554 probes x 256 rays, max_dist 256) bit for bit in
    hit counts and within 1e-5 in radiance."""
    import lum_gb300
    import oracle
    w = worldgen.demo_world(SEED)
    lst = _demo_lists(w.dims)[3]
    prev = (worldgen.uniform(SEED, 5, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.5).astype(np.float32)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        rw.radiance_pass(lst, lum_gb300.pass_params(rays=256, max_dist=256.0, blend=0.1, time_seed=3))
        got = rw.get_radiance()
        st = rw.pass_stats()
    ref, _, ref_st = oracle.radiance_pass(w, lst, rays=256, max_dist=256.0, blend=0.1, time_seed=3, prev=prev)
    assert (st["steps"], st["hits"]) == (ref_st["steps"], ref_st["hits"])
    assert rel_err(got, ref).max() <= RTOL


def test_demo_step_is_deterministic():
    """Two runs of a full 8-pass step give the same volume bit for bit."""
    import lum_gb300
    w = worldgen.demo_world(SEED)
    lists = _demo_lists(w.dims)
    out = []
    for _ in range(2):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            for p, l in enumerate(lists):
                rw.radiance_pass(l, lum_gb300.pass_params(rays=256, max_dist=256.0, blend=0.1, time_seed=p))
            out.append(rw.get_radiance())
    assert out[0].tobytes() == out[1].tobytes()
    assert out[0].max() > 0.0


def test_full_batch_equals_worlds_one_by_one():
    """The 256-world mixed batch (58.6M rays, 2 rounds) equals each world's own pass."""
    import lum_gb300
    mix = worldgen.mixed_worlds(n=256, seed=SEED)

    def make():
        rws = []
        for w, req, r in mix:
            rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0])
            rw.load(w)
            rws.append(rw)
        return rws

    a, b = make(), make()
    with lum_gb300.RadianceBatch(a) as ba, lum_gb300.RadianceBatch(b) as bb:
        for i, (w, req, r) in enumerate(mix):
            p = lum_gb300.pass_params(rays=r, max_dist=128.0, blend=0.1)
            ba.set_requests(i, req, p)
            bb.set_requests(i, req, p)
        for seed in (0, 1):
            ba.run(seed)
            bb.run_per_world(seed)
        ba.synchronize()
        bb.synchronize()
        for x, y in zip(a, b):
            assert x.get_radiance().tobytes() == y.get_radiance().tobytes()
    for rw in a + b:
        rw.close()


def test_precision_world_pass_and_scroll_round_trip():
    """A full pass of the 64x64x32 world (all 131,072 probes x 96 rays: 393,216 tasks in two
    rounds) against the oracle; then a scroll by s and back by -s restores every cell the two
    shifts keep inside the world."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world((64, 64, 32), seed=SEED, n_types=32)
    req = worldgen.all_probes(w.dims)
    prev = (worldgen.uniform(SEED, 6, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.5).astype(np.float32)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        rw.radiance_pass(req, lum_gb300.pass_params(rays=96, max_dist=128.0, blend=0.1, time_seed=1))
        got = rw.get_radiance()
        ref, _, _ = oracle.radiance_pass(w, req, rays=96, max_dist=128.0, blend=0.1, time_seed=1, prev=prev)
        assert rel_err(got, ref).max() <= RTOL
        s = (5, -3, 2)
        rw.shift_radiance(*s)
        rw.shift_radiance(-s[0], -s[1], -s[2])
        back = rw.get_radiance()
        X, Y, Z = w.dims
        # restored exactly: the cells p with p - s inside the world, [max(s,0), n + min(s,0)) per axis
        keep = (slice(max(s[2], 0), Z + min(s[2], 0)), slice(max(s[1], 0), Y + min(s[1], 0)),
                slice(max(s[0], 0), X + min(s[0], 0)))
        inner = oracle.shift_radiance(oracle.shift_radiance(got, s), (-s[0], -s[1], -s[2]))
        assert back.tobytes() == inner.tobytes()
        assert np.array_equal(back[keep], got[keep])


def test_full_server_world_alone_equals_mix():
    """The 64 serving worlds with 4 relight requests each, all in one server: each world ends
    as it does when its requests are served alone."""
    import lum_gb300
    worlds = worldgen.serving_worlds(64, seed=SEED)
    reqs = [(k % 64, worldgen.edit_request(worlds[k % 64].dims, 0.01 + 0.04 * ((k * 7) % 5) / 4, seed=SEED,
                                           stream=k)) for k in range(256)]

    def serve(which):
        with lum_gb300.RadianceServer(max_inflight=3) as srv:
            rws = []
            for i in which:
                rw = lum_gb300.RadianceWorld(worlds[i].dims, max_block_types=worlds[i].palette.shape[0])
                rw.load(worlds[i])
                srv.add_world(rw)
                rws.append(rw)
            idx = {i: k for k, i in enumerate(which)}
            for k, (i, e) in enumerate(reqs):
                if i in idx:
                    srv.submit(idx[i], e, lum_gb300.pass_params(rays=64, blend=0.1, time_seed=k))
            srv.run(timeout_s=300)
            out = {i: srv.get_radiance(idx[i]) for i in which}
        for rw in rws:
            rw.close()
        return out

    mixed = serve(list(range(64)))
    for i in (0, 17, 42, 63):
        assert serve([i])[i].tobytes() == mixed[i].tobytes()


def test_demo_step_in_one_call_equals_single_passes():
    """The headline step: the demo world's 8 passes (6,554 probes x 256 rays each) through one
    several-pass call, bit for bit the 8 single passes, counters included."""
    import lum_gb300
    w = worldgen.demo_world(SEED)
    lists = _demo_lists(w.dims)
    params = [lum_gb300.pass_params(rays=256, max_dist=256.0, blend=0.1, time_seed=p) for p in range(8)]
    out, stats = [], []
    for multi in (False, True):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            if multi:
                rw.radiance_passes(lists, params)
                st = rw.pass_stats()
                stats.append((st["steps"], st["hits"], st["probes"]))
            else:
                s = [0, 0, 0]
                for l, p in zip(lists, params):
                    rw.radiance_pass(l, p)
                    st = rw.pass_stats()
                    s = [s[0] + st["steps"], s[1] + st["hits"], s[2] + st["probes"]]
                stats.append(tuple(s))
            out.append(rw.get_radiance())
    assert out[0].tobytes() == out[1].tobytes()
    assert stats[0] == stats[1]
