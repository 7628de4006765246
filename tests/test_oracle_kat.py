"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors for this path, so these pin the oracle's
building blocks against independent statements of the same definitions: hash33
(radiance.comp:51-59) re-implemented with Python integers, the spherical-Fibonacci table
(:293-306), closed forms for an empty world and for axis-aligned rays into a single block, and
the update-list rule (internal_render.cpp:1142-1168) restated with numpy.
"""
import math

import numpy as np
import pytest

import oracle
from lum_gb300 import worldgen

K = 1103515245


def py_hash33(x, y, z):
    m = 0xFFFFFFFF
    for _ in range(3):
        x, y, z = (((x >> 8) ^ y) * K) & m, (((y >> 8) ^ z) * K) & m, (((z >> 8) ^ x) * K) & m
    return np.array([x, y, z], dtype=np.float32) * np.float32(2.0 ** -32)


@pytest.mark.parametrize("seed", [(0, 0, 0), (1, 0, 0), (5, 5, 5), (64, 3, 3), (0xFFFFFFFF, 7, 9),
                                  (123456789, 987654321, 42), (2**31, 2**31 + 1, 17)])
def test_hash33_known_answers(seed):
    got = oracle.hash33(*seed)
    want = py_hash33(*seed)
    assert got.tobytes() == want.tobytes(), (got, want)


def test_hash33_range_and_spread():
    vals = np.array([oracle.hash33(i + 11, 11, 11) for i in range(2000)])
    assert vals.min() >= 0.0 and vals.max() <= 1.0
    assert abs(vals.mean() - 0.5) < 0.03


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_direction_table(n):
    t = oracle.direction_table(n)
    norms = np.linalg.norm(t.astype(np.float64), axis=1)
    assert np.all(np.abs(norms - 1.0) < 1e-6)
    # cos(theta) = 1 - (2i+1)/n exactly as the shader's float expression
    i = np.arange(n, dtype=np.float32)
    cos_t = np.float32(1.0) - (np.float32(2.0) * i + np.float32(1.0)) * (np.float32(1.0) / np.float32(n))
    assert np.array_equal(t[:, 2], cos_t)
    # phi = 2*pi*frac(i*(golden-1)) in float; x = cos(phi)*sin(theta) with cos in double
    golden = np.float32(np.sqrt(np.float32(5.0))) * np.float32(0.5) + np.float32(0.5)
    a = i * (golden - np.float32(1.0))
    phi = np.float32(2.0) * np.float32(math.pi) * (a - np.floor(a))
    sin_t = np.sqrt(np.clip(np.float32(1.0) - cos_t * cos_t, 0, 1)).astype(np.float32)
    x = np.cos(phi.astype(np.float64)).astype(np.float32) * sin_t
    assert np.array_equal(t[:, 0], x)


def test_library_direction_table_matches_oracle():
    import lum_gb300
    for n in (32, 64, 96, 256):
        assert lum_gb300.direction_table(n).tobytes() == oracle.direction_table(n).tobytes()


def _world(grid, n_types=2, fill=None, mats=None):
    grid = np.ascontiguousarray(grid, dtype=np.int16)
    pal = np.zeros((n_types + 1, 16, 16, 16), dtype=np.uint8)
    for t in range(1, n_types + 1):
        pal[t] = t if fill is None else fill[t]
    m = np.zeros((256, 6), dtype=np.float32) if mats is None else mats
    return worldgen.World(grid=grid, palette=pal, materials=m)


def _sky(d):
    g = np.float32(0.5), np.float32(0.5), np.float32(-0.9)
    v = np.array(g, dtype=np.float32)
    s = np.float32(1.0) / np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
    gl = v * s
    d = np.asarray(d, dtype=np.float32)
    gdot = -((d[0] * gl[0] + d[1] * gl[1]) + d[2] * gl[2])
    light = np.zeros(3, dtype=np.float32)
    if gdot > np.float32(0.95):
        light = light + gdot * (np.array([0.9, 0.9, 0.6], dtype=np.float32) * np.float32(3.0))
    return light + np.array([0.53, 0.81, 0.92], dtype=np.float32) * np.float32(0.1)


def test_empty_world_every_ray_sees_the_sky():
    """In an all-air world every ray misses; the probe is a closed-form blend of sky values."""
    w = _world(np.zeros((4, 4, 4)))
    req = worldgen.all_probes(w.dims)
    nxt, hits, st = oracle.radiance_pass(w, req, rays=64, blend=1.0, record_hits=True)
    assert st["hits"] == 0 and np.all((hits["flags"] & 1) == 0)
    dirs = oracle.direction_table(64)
    # with blend 1 the stored value is the mean over rays; every miss adds at least the sky term
    sky = np.array([0.53, 0.81, 0.92], dtype=np.float32) * np.float32(0.1)
    assert np.all(nxt >= sky - 1e-6)
    for (x, y, z, _) in req[:4]:
        assert np.all(nxt[z, y, x] <= 1.0)
    assert dirs.shape == (64, 3)


def test_axis_aligned_ray_hits_the_block_face():
    """A (nearly) +x ray at y,z inside a solid block hits its first voxel column: the refine DDA
    lands on x = 16*bx with an x-step, normal -x."""
    g = np.zeros((3, 3, 3), dtype=np.int16)
    g[1, 1, 2] = 1                   # block (x=2, y=1, z=1)
    mats = np.zeros((256, 6), dtype=np.float32)
    mats[1] = [0.5, 0.25, 1.0, 1.0, 2.0, 0.0]
    w = _world(g, n_types=1, mats=mats)
    d = np.array([0.99999, 0.003, 0.002], dtype=np.float32)
    light, hit = oracle.trace_ray(w, [5.25, 20.5, 24.5], d / np.linalg.norm(d))
    assert hit["flags"] & 1
    assert tuple(hit["voxel"]) == (32, 20, 24)
    assert hit["voxel_id"] == 1 and hit["flags"] & 0x02
    # radiance is zero, so light = albedo * emission
    assert np.allclose(light, [1.0, 0.5, 2.0])


def test_zero_direction_component_is_defined():
    """An exactly axis-aligned direction makes 1/d infinite: the march still ends (bounded),
    and the NaN that the refine produces is reported canonically."""
    g = np.zeros((3, 3, 3), dtype=np.int16)
    g[1, 1, 2] = 1
    w = _world(g, n_types=1)
    light, hit = oracle.trace_ray(w, [5.25, 20.5, 24.5], [1.0, 0.0, 0.0])
    assert hit["coarse_steps"] < 2 * 128 + 3
    f = np.array([hit["fraction"]], dtype=np.float32)
    assert not np.isnan(f[0]) or f.view(np.uint32)[0] == 0x7FC00000


def test_ray_leaving_the_world_misses():
    g = np.zeros((2, 2, 2), dtype=np.int16)
    g[0, 0, 0] = 1
    w = _world(g, n_types=1)
    d = np.array([0.05, 0.6, 0.8], dtype=np.float32)
    d = d / np.linalg.norm(d)
    light, hit = oracle.trace_ray(w, [20.0, 20.0, 20.0], d)
    assert not (hit["flags"] & 1)
    assert np.allclose(light, _sky(d))


def test_origin_inside_solid_gives_zero_normal():
    """Quirk (radiance.comp:249-285): when the voxel 1.5 back along the ray is already solid the
    refine loop never runs: no step flags, refine fraction 0, hit point = ray origin."""
    g = np.ones((2, 2, 2), dtype=np.int16)
    w = _world(g, n_types=1)
    d = np.array([0.6, 0.05, 0.8], dtype=np.float32)
    light, hit = oracle.trace_ray(w, [16.5, 16.5, 16.5], d / np.linalg.norm(d))
    assert hit["flags"] & 1
    assert hit["refine_steps"] == 0 and (hit["flags"] & 0x0E) == 0
    assert hit["fraction"] == 0.0


def test_update_list_rule_matches_numpy():
    w = worldgen.terrain_world((10, 9, 7), seed=3, extra_blocks=15)
    g = w.grid.astype(np.int64)
    Z, Y, X = g.shape
    pad = np.pad(g, 1, mode="edge")
    s = np.zeros_like(g)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                s += pad[dz:dz + Z, dy:dy + Y, dx:dx + X]
    zz, yy, xx = np.nonzero(s > 0)
    want = np.stack([xx, yy, zz, np.zeros_like(xx)], axis=1).astype(np.int16)
    specials = np.array([[0, 0, 6, 0], [1, 2, 3, 0], [0, 0, 6, 0]], dtype=np.int16)
    got = oracle.update_list(w, specials)
    base = got[: want.shape[0]]
    assert np.array_equal(base, want)
    extra = got[want.shape[0]:]
    listed = set(map(tuple, want[:, :3].tolist()))
    for sp in specials:
        if tuple(sp[:3].tolist()) not in listed:
            assert any(np.array_equal(sp, e) for e in extra)
    # specials are only de-duplicated against the rule, not against each other
    n_dup = sum(tuple(sp[:3].tolist()) not in listed for sp in specials)
    assert extra.shape[0] == n_dup


def test_oracle_deterministic_across_thread_counts():
    w = worldgen.terrain_world((8, 8, 6), seed=9, extra_blocks=10)
    req = worldgen.all_probes(w.dims)
    a, ha, _ = oracle.radiance_pass(w, req, rays=64, blend=0.1, record_hits=True, threads=1)
    b, hb, _ = oracle.radiance_pass(w, req, rays=64, blend=0.1, record_hits=True, threads=4)
    assert a.tobytes() == b.tobytes() and ha.tobytes() == hb.tobytes()


def test_f64_oracle_keeps_fp32_traversal():
    w = worldgen.terrain_world((8, 8, 6), seed=10)
    req = worldgen.all_probes(w.dims)
    a, ha, _ = oracle.radiance_pass(w, req, rays=64, blend=0.1, record_hits=True, precision="f32")
    b, hb, _ = oracle.radiance_pass(w, req, rays=64, blend=0.1, record_hits=True, precision="f64")
    assert ha.tobytes() == hb.tobytes()
    assert np.max(np.abs(a - b)) < 1e-5


def test_sky_constants_of_the_kernels():
    """The kernels' sky/sun constants (hex literals in radiance_device.cuh) are the FP32
    round-to-nearest values of the shader's expressions (radiance.comp:334-343):
    normalize(0.5, 0.5, -0.9) as v * (1 / sqrt(dot(v, v))), 0.9*3, 0.6*3 and 0.1*(0.53, 0.81, 0.92)."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "lum_gb300", "csrc", "radiance_device.cuh")).read()
    consts = {k: int(v, 16) for k, v in re.findall(r"(k[A-Za-z]+) = 0x([0-9a-f]+)u", src)}
    f = np.float32
    v = (f(0.5), f(0.5), f(-0.9))
    dd = f(f(f(v[0] * v[0]) + f(v[1] * v[1])) + f(v[2] * v[2]))
    s = f(f(1.0) / f(np.sqrt(dd)))
    want = {"kGl": f(v[0] * s), "kGlz": f(v[2] * s), "kSun": f(f(0.9) * f(3.0)), "kSunB": f(f(0.6) * f(3.0)),
            "kSkyR": f(f(0.53) * f(0.1)), "kSkyG": f(f(0.81) * f(0.1)), "kSkyB": f(f(0.92) * f(0.1))}
    for k, x in want.items():
        assert consts[k] == int(np.array(x, dtype=np.float32).view(np.uint32)), k
