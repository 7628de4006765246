"""The device work either side of the pass, bit for bit against the oracle: the update-list
builder (internal_render.cpp:1142-1168), update_radiance with it, the radiance scroll
(shift_radiance, :1218-1335) and the consumer's 8-probe gather (diffuse.frag:24-90)."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import RTOL, random_prev, rel_err

pytestmark = pytest.mark.gpu


def _world(dims=(12, 10, 7), seed=3, negative=True):
    w = worldgen.terrain_world(dims, seed=seed, n_types=32, extra_blocks=15)
    if negative:   # negative ids make some neighbourhood sums <= 0 despite solid blocks
        g = w.grid.copy()
        u = worldgen.randint(seed, 77, 40, 0, g.size)
        g.reshape(-1)[u] = -worldgen.randint(seed, 78, 40, 1, 60).astype(np.int16)
        w.grid = g
    return w


def _rw(w, precision="fp32"):
    import lum_gb300
    rw = lum_gb300.RadianceWorld(w.dims, max_block_types=w.palette.shape[0], precision=precision)
    rw.load(w)
    return rw


@pytest.mark.parametrize("dims", [(12, 10, 7), (33, 5, 9), (1, 1, 1), (64, 3, 2)])
def test_update_list_matches_oracle(dims):
    import oracle
    w = _world(dims)
    specials = np.array([[0, 0, 0, 0], [dims[0] - 1, 0, dims[2] - 1, 0], [0, 0, 0, 0],
                         [dims[0] // 2, dims[1] // 2, dims[2] // 2, 0]], dtype=np.int16)
    with _rw(w) as rw:
        for s in specials:
            rw.request_update(*[int(v) for v in s[:3]])
        got = rw.build_update_list()
        ref = oracle.update_list(w, specials)
        assert np.array_equal(got, ref)
        # building alone keeps the special queue; the next build sees the same list
        assert np.array_equal(rw.build_update_list(), ref)


def test_update_list_large_world():
    import oracle
    w = worldgen.demo_world(1234)
    with _rw(w) as rw:
        assert np.array_equal(rw.build_update_list(), oracle.update_list(w))


def test_update_radiance_uses_the_list():
    """update_radiance (device list, specials consumed) equals radiance_pass over the oracle's list."""
    import lum_gb300
    import oracle
    w = _world()
    prev = random_prev(w)
    p = lum_gb300.pass_params(rays=64, blend=0.1, time_seed=4)
    with _rw(w) as a, _rw(w) as b:
        a.set_radiance(prev)
        b.set_radiance(prev)
        a.request_update(1, 1, 1)
        a.update_radiance(p)
        b.radiance_pass(oracle.update_list(w, np.array([[1, 1, 1, 0]], np.int16)), p)
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()
        # the special was consumed
        assert np.array_equal(a.build_update_list(), oracle.update_list(w))


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16", "rgb10a2"])
def test_shift_matches_oracle(precision):
    import oracle
    w = _world((9, 8, 6), negative=False)
    prev = random_prev(w, seed=9)
    with _rw(w, precision) as rw:
        rw.set_radiance(prev)
        cur = rw.get_radiance()
        for s in [(1, 0, 0), (-2, 3, 1), (0, 0, -5), (8, 0, 0), (9, 0, 0), (0, -8, 0), (3, 3, 6), (0, 0, 0)]:
            rw.shift_radiance(*s)
            cur = oracle.shift_radiance(cur, s)
            assert rw.get_radiance().tobytes() == cur.tobytes(), s


def test_stored_shift_applies_before_each_update():
    import lum_gb300
    import oracle
    w = _world((10, 9, 6), negative=False)
    prev = random_prev(w, seed=11)
    p = lum_gb300.pass_params(rays=32, blend=0.2, time_seed=2)
    with _rw(w) as a, _rw(w) as b:
        a.set_radiance(prev)
        b.set_radiance(prev)
        a.set_radiance_shift(1, -1, 0)
        assert a.get_radiance_shift() == (1, -1, 0)
        for _ in range(2):
            a.update_radiance(p)
            b.shift_radiance(1, -1, 0)
            b.radiance_pass(oracle.update_list(w), p)
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16", "rgb10a2"])
def test_gather_matches_oracle(precision):
    import oracle
    w = _world((7, 6, 5), negative=False)
    rng = np.random.default_rng(8)
    vol = (rng.random(w.grid.shape + (3,)) * 0.999).astype(np.float32)
    n = 4000
    pos = (rng.random((n, 3)) * 1.2 - 0.1) * np.array([7, 6, 5]) * 16   # some points outside
    pos[:50] = np.floor(pos[:50] / 16) * 16 + 8                          # exactly at probe centres
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[50:60] = 0.0                                                     # degenerate normals
    pts = np.concatenate([pos, nrm], axis=1).astype(np.float32)
    with _rw(w, precision) as rw:
        rw.set_radiance(vol)
        got = rw.gather(pts)
        ref = oracle.gather(rw.get_radiance(), pts)
    assert got.tobytes() == ref.tobytes()


def _quat(seed):
    q = np.random.default_rng(seed).normal(size=4)
    return tuple((q / np.linalg.norm(q)).astype(np.float32))


def _models():
    rng = np.random.default_rng(21)
    a = (rng.random((12, 9, 14)) < 0.6) * rng.integers(1, 256, (12, 9, 14))
    b = (rng.random((5, 20, 7)) < 0.8) * rng.integers(1, 256, (5, 20, 7))
    return [a.astype(np.uint8), b.astype(np.uint8)]


def test_blockify_matches_oracle():
    """Blockified grid and palette bit for bit, then a pass over the blockified world equals the
    oracle's pass on the oracle's blockified world."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world((8, 7, 6), seed=12, n_types=20)
    models = _models()
    meshes = [(0, _quat(1), (20.3, 17.9, 30.2)),
              (1, _quat(2), (64.0, 40.5, 9.0)),
              (0, (0.0, 0.0, 0.0, 1.0), (-6.5, 3.0, -2.0)),   # partly below the world: aliasing into block 0
              (1, _quat(3), (25.0, 30.0, 20.0))]              # overlaps the first mesh
    static = w.palette.shape[0]
    with lum_gb300.RadianceWorld(w.dims, max_block_types=200) as rw:
        rw.load(w)
        ids = [rw.load_model(m) for m in models]
        assert ids == [0, 1]
        rw.blockify(static, meshes)
        got_g, got_p = rw.get_world(), rw.get_block_palette()
        pal = np.zeros((200, 16, 16, 16), np.uint8)
        pal[:static] = w.palette
        ref_g, ref_p = oracle.blockify(w.grid, pal, static, models, meshes)
        assert np.array_equal(got_g, ref_g)
        assert np.array_equal(got_p, ref_p)
        assert got_g.max() > static   # temporary blocks were made
        # a pass over the blockified world
        req = worldgen.all_probes(w.dims)
        prev = random_prev(w)
        rw.set_radiance(prev)
        p = lum_gb300.pass_params(rays=64, max_dist=128.0, blend=0.1, time_seed=3, record_hits=True)
        rw.radiance_pass(req, p)
        got = rw.get_radiance()
        hits = rw.get_hits()
        wb = worldgen.World(grid=ref_g, palette=ref_p, materials=w.materials)
        ref, ref_hits, _ = oracle.radiance_pass(wb, req, rays=64, max_dist=128.0, blend=0.1, time_seed=3, prev=prev,
                                                record_hits=True)
        assert hits.tobytes() == ref_hits.tobytes()
        assert rel_err(got, ref).max() <= RTOL
        # the next frame starts from the origin world again
        rw.blockify(static, [])
        assert np.array_equal(rw.get_world(), w.grid)
        pal2 = rw.get_block_palette()
        assert np.array_equal(pal2[:static], w.palette) and not pal2[static:].any()


def test_blockify_out_of_slots_leaves_the_world():
    import lum_gb300
    w = worldgen.terrain_world((6, 6, 4), seed=13, n_types=8)
    with lum_gb300.RadianceWorld(w.dims, max_block_types=12) as rw:
        rw.load(w)
        m = rw.load_model(np.ones((40, 40, 40), np.uint8))
        with pytest.raises(lum_gb300.LumRadError) as ei:
            rw.blockify(9, [(m, (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0))])
        assert ei.value.code == lum_gb300._native.LUMRAD_ENOMEM
        assert np.array_equal(rw.get_world(), w.grid)


@pytest.mark.parametrize("dims,frac,radius", [((8, 8, 8), 0.002, 2), ((16, 12, 9), 0.05, 2), ((33, 17, 5), 0.03, 1),
                                              ((64, 64, 32), 0.01, 2), ((7, 5, 3), 0.5, 3), ((20, 20, 20), 0.001, 0)])
def test_dirty_list_on_device_matches_host(dims, frac, radius):
    """The device derivation of a relight request's probes equals the host one and numpy's."""
    import lum_gb300
    w = worldgen.terrain_world(dims, seed=41, n_types=8)
    edits = worldgen.edit_request(dims, frac, seed=42, stream=radius)
    with _rw(w) as rw:
        got = rw.build_dirty_list(edits, radius)
        assert np.array_equal(got, lum_gb300.dirty_probes(dims, edits, radius))
        assert np.array_equal(got, worldgen.dirty_probes(dims, edits, radius))
        assert rw.build_dirty_list(np.zeros((0, 4), np.int16), radius).shape == (0, 4)


def test_blockify_frames_of_different_sizes():
    """Consecutive frames with more, then fewer, meshes (the smaller frame clears the slots the
    larger one used), and an origin world holding a dynamic id above the static blocks (its slot
    is mapped into like a temporary one): each frame's grid and palette equal the oracle's."""
    import lum_gb300
    import oracle
    w = worldgen.terrain_world((9, 8, 6), seed=14, n_types=20)
    static = w.palette.shape[0]
    w.grid[2, 3, 4] = static + 30          # a dynamic id set by the caller
    models = _models()
    frames = [[(0, _quat(5), (30.0, 20.0, 25.0)), (1, _quat(6), (70.0, 50.0, 40.0)), (0, _quat(7), (60.5, 66.0, 49.0)),
               (0, (0.0, 0.0, 0.0, 1.0), (64.0, 48.0, 32.0))],
              [(1, _quat(8), (20.0, 30.0, 20.0))],
              [],
              [(0, _quat(9), (50.0, 40.0, 30.0)), (1, _quat(10), (30.0, 60.0, 50.0))]]
    with lum_gb300.RadianceWorld(w.dims, max_block_types=240) as rw:
        rw.load(w)
        for m in models:
            rw.load_model(m)
        pal = np.zeros((240, 16, 16, 16), np.uint8)
        pal[:static] = w.palette
        for meshes in frames:
            rw.blockify(static, meshes)
            ref_g, ref_p = oracle.blockify(w.grid, pal, static, models, meshes)
            assert np.array_equal(rw.get_world(), ref_g)
            assert np.array_equal(rw.get_block_palette(), ref_p)


def test_update_radiance_frames_without_waiting():
    """update_radiance launches the pass for the longest list and reads the list's length on the
    device (no host wait): frames back to back, sliced (size 2), adaptive (size 0) and with
    specials, equal passes over the oracle's list; the frame's counters survive a later list build."""
    import lum_gb300
    import oracle
    w = _world((10, 9, 7), seed=5)
    prev = random_prev(w)
    full = oracle.update_list(w)
    with _rw(w) as a, _rw(w) as b:
        a.set_radiance(prev)
        b.set_radiance(prev)
        frames = [dict(rays=64, blend=0.1, time_seed=3), dict(rays=128, blend=0.2, time_seed=4, size=2, shift=1),
                  dict(rays=32, blend=0.1, time_seed=5)]
        for f in frames:
            a.update_radiance(lum_gb300.pass_params(**f))
        for f in frames:
            b.radiance_pass(full, lum_gb300.pass_params(**f))
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()
        # a special request; the counters of the frame, then another list build
        a.request_update(2, 3, 1)
        a.request_update(0, 0, 6)
        with_specials = oracle.update_list(w, np.array([[2, 3, 1, 0], [0, 0, 6, 0]], np.int16))
        a.update_radiance(lum_gb300.pass_params(rays=64, blend=0.1, time_seed=6))
        b.radiance_pass(with_specials, lum_gb300.pass_params(rays=64, blend=0.1, time_seed=6))
        sa = a.pass_stats()
        a.build_update_list()   # another list on the device after the frame
        assert a.pass_stats()["probes"] == sa["probes"] == with_specials.shape[0]
        sb = b.pass_stats()
        assert (sa["steps"], sa["hits"], sa["rays"]) == (sb["steps"], sb["hits"], sb["rays"])
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()
    # adaptive slicing (size 0): on a small world every frame stays at size 1, seeded by its index
    with _rw(w) as a, _rw(w) as b:
        for k in range(3):
            a.update_radiance(lum_gb300.pass_params(rays=64, blend=0.1, size=0))
            b.radiance_pass(full, lum_gb300.pass_params(rays=64, blend=0.1, time_seed=k))
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()


def test_adaptive_slicing_grows_and_shrinks():
    """magicSize adaptation of update_radiance (internal_render.cpp:1190-1203): a previous pass
    slower than 2.2 ms grows the slice by one, faster than 1.8 ms shrinks it, in between keeps it,
    clamped to [1, 10]; frame k then updates requests shift = k % size, shift + size, ... with
    time seed k.  The previous pass's time is set through the test hook (the reference reads its
    timestamp query), so the sequence of slices is known; every frame equals lumrad_radiance_pass
    with that size, shift and seed over the oracle's update list."""
    import lum_gb300
    import oracle
    from lum_gb300 import _native as N
    w = _world((10, 9, 7), seed=6)
    full = oracle.update_list(w)
    prev = random_prev(w)
    # (previous pass ms as the hook reports it, slice size the frame must use); frame 0 has no
    # previous pass (0 ms: size stays 1)
    plan = [(None, 1), (3.0, 2), (2.5, 3), (2.0, 3), (1.9, 3), (1.0, 2), (0.5, 1), (0.5, 1)]
    plan += [(9.0, s) for s in range(2, 11)] + [(9.0, 10), (2.2, 10), (1.8, 10), (1.79, 9)]
    with _rw(w) as a, _rw(w) as b:
        a.set_radiance(prev)
        b.set_radiance(prev)
        for k, (ms, size) in enumerate(plan):
            if ms is not None:
                N.check(a.lib.lumrad_test_hook(a.h, N.LUMRAD_TEST_PASS_MS, ms))
            a.update_radiance(lum_gb300.pass_params(rays=32, blend=0.2, size=0))
            b.radiance_pass(full, lum_gb300.pass_params(rays=32, blend=0.2, size=size, shift=k % size, time_seed=k))
            assert a.pass_stats()["probes"] == b.pass_stats()["probes"] == full.shape[0] // size, k
            assert a.get_radiance().tobytes() == b.get_radiance().tobytes(), (k, ms, size)
        N.check(a.lib.lumrad_test_hook(a.h, N.LUMRAD_TEST_PASS_MS, -1.0))   # measured again
        a.update_radiance(lum_gb300.pass_params(rays=32, blend=0.2, size=0))   # a small pass: < 1.8 ms
        b.radiance_pass(full, lum_gb300.pass_params(rays=32, blend=0.2, size=8, shift=len(plan) % 8,
                                                    time_seed=len(plan)))
        assert a.get_radiance().tobytes() == b.get_radiance().tobytes()
