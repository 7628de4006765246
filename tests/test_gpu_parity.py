"""GPU pass vs CPU oracle through the C ABI: hit records bit-exact, radiance within 1e-5 relative.

Cases follow the pass's parameters and the edge cases of its inputs: rays per probe 32..256,
time slicing (size/shift), i8vec4 requests, multi-pass Jacobi chains, non-power-of-two worlds
(REPEAT wrap of the radiance fetch), out-of-world requests, negative / unloaded / special block
ids, a non-empty palette slot 0, empty lists.
"""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, assert_hits_equal, gpu_pass, oracle_pass, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _check(world, req, prev, **params):
    got, hits, stats = gpu_pass(world, req, prev, **params)
    ref, ref_hits, ref_stats = oracle_pass(world, req, prev, **params)
    assert_hits_equal(hits, ref_hits)
    assert rel_err(got, ref).max() <= RTOL
    assert stats["steps"] == ref_stats["steps"] and stats["hits"] == ref_stats["hits"]
    return got, ref


def test_small_world_reference_constants():
    """8x8x8 world, all 512 probes, 64 rays, max_dist 128, blend 0.1."""
    w = worldgen.small_world()
    got, ref = _check(w, worldgen.all_probes(w.dims), random_prev(w), rays=64, max_dist=128.0, blend=0.1,
                      time_seed=0)
    assert np.array_equal(got, ref), "FP32 radiance is expected bit-identical to the oracle"


@pytest.mark.parametrize("rays", [32, 96, 128, 256])
def test_rays_per_probe(rays):
    w = worldgen.small_world(seed=11)
    req = worldgen.probe_subset(w.dims, 0.25, seed=5)
    _check(w, req, random_prev(w), rays=rays, max_dist=128.0, blend=0.1, time_seed=17)


def test_time_slicing_size_shift():
    w = worldgen.small_world(seed=3)
    req = worldgen.all_probes(w.dims)
    _check(w, req, random_prev(w), rays=64, max_dist=128.0, blend=0.01, time_seed=5, size=3, shift=2)


def test_i8_requests_match_i16():
    import lum_gb300
    w = worldgen.small_world(seed=4)
    req = worldgen.probe_subset(w.dims, 0.5, seed=2)
    prev = random_prev(w)
    outs = []
    for r in (req, req.astype(np.int8)):
        with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
            rw.load(w)
            rw.set_radiance(prev)
            rw.radiance_pass(r, lum_gb300.pass_params(rays=64, blend=0.1, time_seed=9))
            outs.append(rw.get_radiance())
    assert np.array_equal(outs[0], outs[1])


def test_multi_pass_chain():
    w = worldgen.terrain_world((12, 10, 6), seed=21, extra_blocks=40)
    req = worldgen.all_probes(w.dims)
    _check(w, req, random_prev(w), passes=3, seeds=[0, 1, 2], rays=64, max_dist=256.0, blend=0.1)


def test_non_power_of_two_world():
    w = worldgen.terrain_world((5, 7, 3), seed=8, n_types=5)
    req = worldgen.all_probes(w.dims)
    _check(w, req, random_prev(w), rays=64, max_dist=200.0, blend=0.3, time_seed=2)


def test_odd_ids_and_slot0():
    """Negative ids (OpSMod palette aliasing), ids past the loaded slots, SPECIAL_BLOCK, and a
    non-empty palette slot 0 (air blocks are then not empty)."""
    w = worldgen.terrain_world((9, 9, 5), seed=30, n_types=8)
    g = w.grid.reshape(-1).copy()
    idx = worldgen.randint(31, 1, 60, 0, g.size)
    vals = np.array([-1, -5, -63, -64, -200, 9, 40, 4095, 32767, 12], dtype=np.int16)
    g[idx] = vals[np.arange(60) % vals.size]
    pal = w.palette.copy()
    pal[0, 3:5, :, 6:9] = 17
    w2 = worldgen.World(grid=g.reshape(w.grid.shape), palette=pal, materials=w.materials)
    _check(w2, worldgen.all_probes(w2.dims), random_prev(w2), rays=64, max_dist=160.0, blend=0.2, time_seed=4)


def test_out_of_world_requests_and_empty_list():
    w = worldgen.small_world(seed=12)
    req = worldgen.probe_subset(w.dims, 0.2, seed=1)
    req = np.concatenate([req, np.array([[-1, 2, 2, 0], [8, 0, 0, 0], [3, 3, 40, 0]], dtype=np.int16)])
    _check(w, req, random_prev(w), rays=32, max_dist=128.0, blend=0.5, time_seed=1)
    _check(w, np.zeros((0, 4), np.int16), random_prev(w), rays=64, max_dist=128.0, blend=0.1, time_seed=0)
    _check(w, req[:2], random_prev(w), rays=64, max_dist=128.0, blend=0.1, time_seed=0, size=3, shift=0)


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_low_precision_storage_vs_fp64(precision):
    """FP16/BF16 storage with FP32 math: hits stay bit-exact; radiance error vs the FP64 oracle
    is bounded by the storage rounding (2^-11 / 2^-8 relative per pass, compounded)."""
    w = worldgen.terrain_world((10, 10, 6), seed=5, extra_blocks=20)
    req = worldgen.all_probes(w.dims)
    prev = random_prev(w)
    got, hits, _ = gpu_pass(w, req, prev, precision=precision, passes=2, seeds=[0, 1], rays=64,
                            max_dist=128.0, blend=0.1)
    ref, ref_hits, _ = oracle_pass(w, req, prev, passes=2, seeds=[0, 1], precision="f64", rays=64,
                                   max_dist=128.0, blend=0.1)
    assert_hits_equal(hits, ref_hits)
    tol = 2e-3 if precision == "fp16" else 1.6e-2
    err = rel_err(got, ref, floor=1e-3)
    assert err.max() <= tol, (precision, err.max())


@pytest.mark.parametrize("rays,odd", [(64, False), (96, True), (256, False)])
def test_rgb10a2_storage_matches_oracle(rays, odd):
    """The reference's own volume format (A2B10G10R10_UNORM): three chained passes, hit records and
    volumes bit for bit against the oracle storing the same 10-bit codes; R = 96 combines a probe's
    subgroups across finalize CTAs; odd block ids and a non-empty slot 0."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world((9, 8, 6), seed=61, extra_blocks=20)
    if odd:
        g = w.grid.reshape(-1).copy()
        idx = worldgen.randint(62, 1, 40, 0, g.size)
        vals = np.array([-1, -5, -63, -64, 9, 40, 32767, 12], dtype=np.int16)
        g[idx] = vals[np.arange(40) % vals.size]
        pal = w.palette.copy()
        pal[0, 3:5, :, 6:9] = 17
        w = worldgen.World(grid=g.reshape(w.grid.shape), palette=pal, materials=w.materials)
    req = worldgen.probe_subset(w.dims, 0.7, seed=63)
    prev = random_prev(w, scale=0.9)
    p = dict(rays=rays, max_dist=128.0, blend=0.3)
    ref = oracle.quantize_unorm10(prev)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision="rgb10a2") as rw:
        rw.load(w)
        rw.set_radiance(prev)
        assert rw.get_radiance().tobytes() == ref.tobytes()   # the upload quantises like the oracle
        for s in range(3):
            rw.radiance_pass(req, lum_gb300.pass_params(time_seed=s, record_hits=True, **p))
            ref, ref_hits, _ = oracle.radiance_pass(w, req, prev=ref, time_seed=s, record_hits=True, unorm10=True, **p)
            assert_hits_equal(rw.get_hits(), ref_hits)
            got = rw.get_radiance()
            assert got.tobytes() == ref.tobytes(), (s, np.abs(got - ref).max())


def test_more_than_256_block_ids():
    """A world with ~280 distinct block ids: compact ids are 16-bit (the march's and the refine's
    wide forms; more than 256 masks never fit shared memory beside the rays' rings, so the world is
    read through L1).  Hit records bit-exact and radiance within 1e-5 against the oracle, over two
    chained passes."""
    w = worldgen.terrain_world((16, 16, 8), seed=33, n_types=300)
    assert len(np.unique(w.grid)) > 257
    prev = random_prev(w)
    req = worldgen.all_probes(w.dims)
    got, hits, _ = gpu_pass(w, req, prev, passes=2, seeds=[3, 4], rays=64, max_dist=160.0, blend=0.2)
    ref, ref_hits, _ = oracle_pass(w, req, prev, passes=2, seeds=[3, 4], rays=64, max_dist=160.0, blend=0.2)
    assert_hits_equal(hits, ref_hits)
    assert rel_err(got, ref).max() <= RTOL


def test_more_than_256_block_ids_in_several_passes_and_a_batch():
    """The same wide world through one several-pass call and inside a batch (the unstaged march):
    equal to single passes, bit for bit."""
    import lum_gb300
    w = worldgen.terrain_world((16, 16, 8), seed=34, n_types=300)
    other = worldgen.terrain_world((6, 5, 4), seed=35, n_types=8)
    lists = [worldgen.probe_subset(w.dims, f, seed=36, stream=i) for i, f in enumerate((0.5, 0.3))]
    params = [lum_gb300.pass_params(rays=64, max_dist=96.0, blend=0.1, time_seed=40 + i) for i in range(2)]
    prev = random_prev(w)

    def world(x):
        rw = lum_gb300.RadianceWorld(x.dims, max_block_types=x.palette.shape[0])
        rw.load(x)
        return rw

    with world(w) as a, world(w) as b:
        a.set_radiance(prev)
        b.set_radiance(prev)
        for l, p in zip(lists, params):
            a.radiance_pass(l, p)
        b.radiance_passes(lists, params)
        single = a.get_radiance()
        assert b.get_radiance().tobytes() == single.tobytes()
    with world(w) as c, world(other) as d:
        c.set_radiance(prev)
        with lum_gb300.RadianceBatch([c, d]) as bt:
            bt.set_requests(0, lists[0], params[0])
            bt.set_requests(1, worldgen.all_probes(other.dims), lum_gb300.pass_params(rays=32))
            bt.run(params[0].time_seed)
            bt.synchronize()
        with world(w) as e:
            e.set_radiance(prev)
            e.radiance_pass(lists[0], params[0])
            assert c.get_radiance().tobytes() == e.get_radiance().tobytes()


def test_more_than_256_block_ids_staged():
    """A world small enough that 16-bit compact ids for 258 ids (257 block ids and air) still fit
    shared memory beside the rays' rings (9x9x4 blocks): the staged wide march, without hit
    records, against the oracle within 1e-5, and equal to the recording (unstaged) pass."""
    import lum_gb300
    base = worldgen.terrain_world((9, 9, 4), seed=37, n_types=257)
    g = np.zeros(9 * 9 * 4, np.int16)
    g[:257] = np.arange(1, 258, dtype=np.int16)
    g = g[worldgen.randint(38, 1, g.size, 0, 1 << 30).argsort(kind="stable")]
    w = worldgen.World(grid=g.reshape(4, 9, 9), palette=base.palette, materials=base.materials)
    prev = random_prev(w)
    req = worldgen.all_probes(w.dims)
    params = dict(rays=64, max_dist=96.0, blend=0.2, time_seed=5)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0]) as rw:
        rw.load(w)
        rw.set_radiance(prev)
        rw.radiance_pass(req, lum_gb300.pass_params(**params))
        got = rw.get_radiance()
    ref, _, _ = oracle_pass(w, req, prev, **params)
    assert rel_err(got, ref).max() <= RTOL
    rec, _, _ = gpu_pass(w, req, prev, **params)
    assert rec.tobytes() == got.tobytes()
