"""Edge cases of the pass against the oracle: the largest ray counts (a probe's subgroups combined
across CTAs), the longest world axis, passes of several rounds (with probes whose subgroups
straddle a round boundary), all-air and all-solid worlds, and FP16/BF16 batches and servers."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, assert_hits_equal, gpu_pass, oracle_pass, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _check(w, req, prev, **p):
    got, hits, st = gpu_pass(w, req, prev, **p)
    ref, ref_hits, ref_st = oracle_pass(w, req, prev, **p)
    assert_hits_equal(hits, ref_hits)
    assert rel_err(got, ref).max() <= RTOL
    assert (st["steps"], st["hits"]) == (ref_st["steps"], ref_st["hits"])


@pytest.mark.parametrize("rays", [512, 1024])
def test_largest_ray_counts(rays):
    """R/32 = 16 or 32 subgroups: a probe spans several CTAs and combines through global scratch."""
    w = worldgen.terrain_world((6, 5, 4), seed=31)
    req = worldgen.probe_subset(w.dims, 0.5, seed=2)
    _check(w, req, random_prev(w), rays=rays, max_dist=96.0, blend=0.2, time_seed=5)


def test_longest_axis():
    """A 2047-block axis (the largest world_size accepts) and a single-block axis."""
    w = worldgen.terrain_world((2047, 2, 1), seed=32, n_types=8)
    req = worldgen.probe_subset(w.dims, 0.3, seed=3)
    _check(w, req, random_prev(w), rays=32, max_dist=200.0, blend=0.1, time_seed=1)


def test_several_rounds_with_straddling_probes():
    """131,072 probes x 96 rays = 393,216 tasks: two rounds of the kernels, and probes whose three
    subgroups fall on both sides of the round boundary."""
    w = worldgen.terrain_world((64, 64, 32), seed=33)
    req = worldgen.all_probes(w.dims)
    prev = random_prev(w)
    got, _, st = gpu_pass(w, req, prev, rays=96, max_dist=64.0, blend=0.1, time_seed=2)
    ref, _, ref_st = oracle_pass(w, req, prev, rays=96, max_dist=64.0, blend=0.1, time_seed=2)
    assert rel_err(got, ref).max() <= RTOL
    assert (st["steps"], st["hits"]) == (ref_st["steps"], ref_st["hits"])


@pytest.mark.parametrize("fill", ["air", "solid"])
def test_uniform_worlds(fill):
    w = worldgen.terrain_world((7, 6, 5), seed=34)
    w.grid = np.zeros_like(w.grid) if fill == "air" else np.full_like(w.grid, 3)
    w.palette[3] = 9   # a fully solid block type
    req = worldgen.all_probes(w.dims)
    _check(w, req, random_prev(w), rays=64, max_dist=128.0, blend=0.1, time_seed=0)


@pytest.mark.parametrize("precision", ["fp16", "bf16", "rgb10a2"])
def test_low_precision_batch_and_server(precision):
    """FP16/BF16 contexts in a batch and in a server: identical to the same passes run one
    context at a time (the storage type rounds identically on every path)."""
    import lum_gb300
    mix = worldgen.mixed_worlds(n=4, seed=35, max_dims=(10, 9, 6))

    def make():
        out = []
        for i, (w, req, r) in enumerate(mix):
            rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision)
            rw.load(w)
            rw.set_radiance(random_prev(w, seed=300 + i))
            out.append(rw)
        return out

    solo, batched = make(), make()
    with lum_gb300.RadianceBatch(batched) as b:
        for i, (w, req, r) in enumerate(mix):
            b.set_requests(i, req, lum_gb300.pass_params(rays=r, blend=0.1))
        b.run(6)
        b.synchronize()
    for (w, req, r), rs, rb in zip(mix, solo, batched):
        rs.radiance_pass(req, lum_gb300.pass_params(rays=r, blend=0.1, time_seed=6))
        assert rs.get_radiance().tobytes() == rb.get_radiance().tobytes()
    # the server: one relight request per world equals radiance_pass over its dirty list
    served = make()
    with lum_gb300.RadianceServer(precision=precision) as srv:
        for rw in served:
            srv.add_world(rw)
        edits = [worldgen.edit_request(w.dims, 0.03, seed=36, stream=i) for i, (w, _, _) in enumerate(mix)]
        for i, e in enumerate(edits):
            srv.submit(i, e, lum_gb300.pass_params(rays=64, blend=0.1, time_seed=9))
        srv.run(timeout_s=60)
        for i, ((w, _, _), e) in enumerate(zip(mix, edits)):
            with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision) as one:
                we = worldgen.World(grid=worldgen.apply_edits(w.grid, e), palette=w.palette, materials=w.materials)
                one.load(we)
                one.set_radiance(random_prev(w, seed=300 + i))
                one.radiance_pass(worldgen.dirty_probes(w.dims, e, 2), lum_gb300.pass_params(rays=64, blend=0.1,
                                                                                              time_seed=9))
                assert one.get_radiance().tobytes() == srv.get_radiance(i).tobytes()
    for rw in solo + batched + served:
        rw.close()
