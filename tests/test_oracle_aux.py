"""The oracle's restatements of the work either side of the pass, against independent numpy
restatements: shift_radiance (internal_render.cpp:1218-1335) and diffuse.frag's 8-probe gather
(:24-90)."""
import numpy as np
import pytest

import oracle


def _shift_numpy(v, s):
    """new(p) = old(p + s) where p + s is inside, old(p) elsewhere; no change if any |s| >= size."""
    Z, Y, X, _ = v.shape
    if abs(s[0]) >= X or abs(s[1]) >= Y or abs(s[2]) >= Z:
        return v.copy()
    out = v.copy()
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    qx, qy, qz = x + s[0], y + s[1], z + s[2]
    ok = (qx >= 0) & (qx < X) & (qy >= 0) & (qy < Y) & (qz >= 0) & (qz < Z)
    out[z[ok], y[ok], x[ok]] = v[qz[ok], qy[ok], qx[ok]]
    return out


@pytest.mark.parametrize("s", [(0, 0, 0), (1, 0, 0), (-1, 2, 0), (3, -4, 2), (-5, -6, -3), (6, 0, 0), (0, 7, 0),
                               (0, 0, -4), (-6, 1, 1), (2, 2, 9)])
def test_shift_matches_numpy(s):
    rng = np.random.default_rng(3)
    v = rng.random((4, 7, 6, 3), dtype=np.float32)
    assert np.array_equal(oracle.shift_radiance(v, s), _shift_numpy(v, s))


def _gather_numpy(vol, pts):
    """diffuse.frag:36-90 in float64 (an independent restatement; agrees to rounding)."""
    Z, Y, X, _ = vol.shape
    out = np.zeros((pts.shape[0], 3))
    for k, (px, py, pz, nx, ny, nz) in enumerate(pts.astype(np.float64)):
        p = np.array([px, py, pz])
        nrm = np.array([nx, ny, nz])
        zero = np.clip(np.trunc(np.floor(p - 8.0) / 16.0).astype(int), 0, [X, Y, Z])
        zp = zero * 16.0 + 8.0
        alpha = np.clip((p - zp) / 16.0, 0, 1)
        tw, tc = 0.0, np.zeros(3)
        for i in range(8):
            off = np.array([i & 1, (i >> 1) & 1, (i >> 2) & 1])
            d = zp + off * 16.0 - p
            dn = d / np.sqrt(d @ d)
            tri = np.where(off == 1, alpha, 1.0 - alpha)
            w = tri.prod() * np.clip(dn @ nrm, 0.1, 1.0)
            q = np.clip(zero + off, 0, [X, Y, Z])
            c = np.zeros(3) if (q[0] >= X or q[1] >= Y or q[2] >= Z) else vol[q[2], q[1], q[0]].astype(np.float64)
            c = np.clip(c, 0.0, 2.0)
            w = max(1e-7, w)
            tw += w
            tc += w * c
        out[k] = tc / tw
    return out


def test_gather_matches_numpy():
    rng = np.random.default_rng(5)
    vol = (rng.random((5, 6, 7, 3)) * 2.5).astype(np.float32)   # some probes above the clamp at 2
    n = 300
    pos = rng.random((n, 3)) * np.array([7, 6, 5]) * 16
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    pts = np.concatenate([pos, nrm], axis=1).astype(np.float32)
    got = oracle.gather(vol, pts)
    ref = _gather_numpy(vol, pts)
    assert np.allclose(got, ref, rtol=2e-6, atol=2e-7)


def test_gather_closed_forms():
    vol = np.full((4, 4, 4, 3), 0.5, dtype=np.float32)   # both points' 8 probes lie inside
    pts = np.array([[20, 21, 22, 0, 0, 1], [31.3, 9.1, 40.7, 0.6, 0.0, 0.8]], dtype=np.float32)
    assert np.array_equal(oracle.gather(vol, pts), np.full((2, 3), 0.5, np.float32))   # uniform volume, exactly
    vol[:] = 5.0
    assert np.array_equal(oracle.gather(vol, pts), np.full((2, 3), 2.0, np.float32))   # probes clamp at 2
    # below the volume the probe index clamps to 0 (the corner probes); past the far side
    # (index clamped to world_size) every probe reads 0
    far = np.array([[-500, -500, -500, 0, 1, 0], [5000, 5000, 5000, 1, 0, 0]], dtype=np.float32)
    assert np.array_equal(oracle.gather(vol, far), np.array([[2, 2, 2], [0, 0, 0]], np.float32))


def test_blockify_identity_places_the_model():
    """A solid 8^3 model at shift (16,16,16): the 2x2x2 blocks under its AABB get temporary slots
    2..9 in z-y-x order; block (1,1,1) (id 1) is copied from static slot 1; the model's voxels land
    in voxels 0..7 of block (1,1,1)'s slot."""
    grid = np.zeros((4, 4, 4), np.int16)
    grid[1, 1, 1] = 1
    pal = np.zeros((16, 16, 16, 16), np.uint8)
    pal[1] = 3
    model = np.full((8, 8, 8), 7, np.uint8)
    g, p = oracle.blockify(grid, pal, 2, [model], [(0, (0, 0, 0, 1), (16, 16, 16))])
    want = grid.copy()
    slot = 2
    for z in range(2):
        for y in range(2):
            for x in range(2):
                want[z, y, x] = slot
                slot += 1
    assert np.array_equal(g, want)
    expect = np.zeros_like(pal)
    expect[1] = 3
    expect[9] = 3
    expect[9, 0:8, 0:8, 0:8] = 7
    assert np.array_equal(p, expect)


def test_blockify_runs_out_of_slots():
    grid = np.zeros((4, 4, 4), np.int16)
    pal = np.zeros((5, 16, 16, 16), np.uint8)
    model = np.ones((20, 20, 20), np.uint8)
    assert oracle.blockify(grid, pal, 2, [model], [(0, (0, 0, 0, 1), (8, 8, 8))]) is None
