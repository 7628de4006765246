"""The device work either side of the pass, bit for bit against the oracle: the update-list
builder (internal_render.cpp:1142-1168), update_radiance with it, the radiance scroll
(shift_radiance, :1218-1335) and the consumer's 8-probe gather (diffuse.frag:24-90)."""
import numpy as np
import pytest

from lum_gb300 import worldgen
from tests.helpers import random_prev

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


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
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


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
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
