"""The CPU oracle against the reference shader itself (no GPU).

oracle/build_ref.py compiles Lum's shaders/radiance.comp as C++ from the reference tree (GLSL shim,
verbatim function bodies).  Its dispatch harness reports, per ray, the value subgroupAdd received
(the ray's light) and the number of grid fetches CastRay_fast made.  The oracle must reproduce both
bit for bit, and the radiance volume the shader stores.  The shader fetches twice per coarse step
(GetVoxel(pos).x and GetVoxel(pos).y, radiance.comp:212-213) and twice at the origin (:195-196),
so its fetch count minus 2 is 2*coarse_steps + refine lookups.

Skipped where the reference sources are absent (the GPU machine).
"""
import numpy as np
import pytest

import oracle
from lum_gb300 import worldgen
from oracle import build_ref
from tests.helpers import random_prev

pytestmark = pytest.mark.skipif(not build_ref.reference_present(), reason="reference sources absent")


@pytest.fixture(scope="module", autouse=True)
def ref_libs():
    build_ref.build()


def compare(world, req, rays=64, max_dist=128.0, blend=0.1, seed=0, size=1, shift=0, prev=None, unorm10=False):
    if prev is None:
        prev = random_prev(world)
    rn, rl, ri, abandoned = build_ref.run_pass(world, req.astype(np.int8), rays=rays, max_dist=max_dist,
                                               blend=blend, time_seed=seed, size=size, shift=shift, prev=prev,
                                               unorm10=unorm10)
    assert abandoned == 0
    groups = req.shape[0] // size
    ol = np.zeros((groups * rays, 3), dtype=np.float32)
    on, oh, _ = oracle.radiance_pass(world, req, rays=rays, max_dist=max_dist, blend=blend, time_seed=seed,
                                     size=size, shift=shift, prev=prev, record_hits=True, ray_light=ol,
                                     unorm10=unorm10)
    assert on.tobytes() == rn.tobytes(), "radiance differs from the reference shader"
    bad = np.nonzero((ol.view(np.uint32) != rl.view(np.uint32)).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} rays' light differs, first {bad[:5]}"
    coarse = oh["coarse_steps"].astype(np.int64)
    refine = np.where(oh["flags"] & 1, 1 + oh["refine_steps"].astype(np.int64), 0)
    assert np.array_equal(ri[:, 0], 2 * coarse + refine), "lookup counts differ"
    # for hits, the shader's last palette fetch is the refine's final voxel
    hit = (oh["flags"] & 1).astype(bool)
    vox_ref = ri[:, 4:7].copy()
    vox_ref[:, 0] &= 15
    vox_ref[:, 1] &= 15
    vox_ref[:, :2] += 16 * ri[:, 1:3]
    vox_ref[:, 2] = ri[:, 6] + 16 * ri[:, 3]
    inside = hit & (oh["voxel"] >= 0).all(axis=1)
    assert np.array_equal(vox_ref[inside], oh["voxel"][inside])
    return on


def test_reference_constants_small_world():
    w = worldgen.small_world()
    compare(w, worldgen.all_probes(w.dims), rays=64, max_dist=128.0, blend=0.1)


@pytest.mark.parametrize("rays", [32, 128, 256])
def test_rays_per_probe_variants(rays):
    w = worldgen.small_world(seed=9)
    compare(w, worldgen.probe_subset(w.dims, 0.3, seed=1), rays=rays, max_dist=200.0, blend=0.3, seed=11)


def test_time_slicing():
    w = worldgen.terrain_world((9, 7, 5), seed=2, extra_blocks=10)
    compare(w, worldgen.all_probes(w.dims), rays=64, blend=0.01, seed=7, size=3, shift=2)


def test_reference_world_size_and_long_rays():
    """The reference's compiled-in world size (48x48x16) with max_dist 256."""
    w = worldgen.terrain_world((48, 48, 16), seed=77, extra_blocks=300)
    compare(w, worldgen.probe_subset(w.dims, 0.03, seed=3), rays=64, max_dist=256.0, seed=5)


def test_odd_ids_and_nonempty_slot0():
    w = worldgen.terrain_world((9, 9, 5), seed=30, n_types=8)
    g = w.grid.reshape(-1).copy()
    idx = worldgen.randint(31, 1, 60, 0, g.size)
    vals = np.array([-1, -5, -63, -64, -200, 9, 40, 4095, 32767, 12], dtype=np.int16)
    g[idx] = vals[np.arange(60) % vals.size]
    pal = w.palette.copy()
    pal[0, 3:5, :, 6:9] = 17
    w2 = worldgen.World(grid=g.reshape(w.grid.shape), palette=pal, materials=w.materials)
    compare(w2, worldgen.all_probes(w2.dims), rays=64, max_dist=160.0, blend=0.2, seed=4)


def test_non_power_of_two_world_and_chain():
    w = worldgen.terrain_world((5, 7, 3), seed=8, n_types=5)
    req = worldgen.all_probes(w.dims)
    cur = random_prev(w)
    for s in range(3):
        cur = compare(w, req, rays=64, max_dist=128.0, blend=0.3, seed=s, prev=cur)


def test_out_of_world_requests():
    w = worldgen.small_world(seed=12)
    req = worldgen.probe_subset(w.dims, 0.2, seed=1)
    req = np.concatenate([req, np.array([[-1, 2, 2, 0], [8, 0, 0, 0], [3, 3, 40, 0]], dtype=np.int16)])
    compare(w, req, rays=32, blend=0.5, seed=1)


def test_rgb10a2_storage_chain():
    """The volume stored in the rgb10_a2 image's own format: every written channel is a 10-bit
    code (code/1023), and three chained passes read the rounded volume back through the
    trilinear fetch; the oracle equals the reference shader bit for bit."""
    w = worldgen.terrain_world((7, 6, 5), seed=19, extra_blocks=12)
    req = worldgen.all_probes(w.dims)
    cur = oracle.quantize_unorm10(random_prev(w))
    for s in range(3):
        cur = compare(w, req, rays=64, max_dist=128.0, blend=0.3, seed=s, prev=cur, unorm10=True)
        codes = cur * np.float32(1023)
        assert np.array_equal(codes, np.rint(codes)), "stored values are not 10-bit codes"
    assert np.unique(cur).size > 50
