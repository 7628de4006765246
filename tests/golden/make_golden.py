"""Generates the golden fixtures of this directory from the reference itself.

Each fixture holds a pass's inputs and the radiance volumes Lum's own shaders/radiance.comp
produces from them, compiled as C++ by oracle/build_ref.py (this script therefore needs the
reference tree; the GPU machine only reads the committed .npz files).

  demo_scene.npz   the reference's demo world as examples/cdemo.c sets it up: assets/scene
                   (48x48x16), blocks 1-14 from the listed .vox files, the material palette of
                   tank_body.vox, the update list of update_radiance's 27-neighbour rule;
                   64 rays, max_dist 128, REACTIVNESS 0.01, two passes (frames 0 and 1)
  terrain_c1.npz   the 8x8x8 seeded terrain world, all probes, 64 rays, blend 0.1, one pass
  slicing_r256.npz a 12x10x6 terrain world, 256 rays, max_dist 256, size 2 / shift 1
  odd_ids.npz      negative, unloaded and special block ids and a non-empty slot 0, 32 rays
  demo_scene_rgb10a2.npz  the demo scene's first three frames with the volume stored in the
                   rgb10_a2 image's own 10-bit format (the reference's RADIANCE_FORMAT)
  terrain_rgb10a2.npz     a 10x8x6 terrain world, 128 rays, blend 0.3, three chained passes in
                   the 10-bit format

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from lum_gb300 import vox, worldgen  # noqa: E402
from oracle import build_ref  # noqa: E402

ASSETS = os.path.join(build_ref.REFERENCE, "assets")
DEMO_BLOCKS = ["dirt", "grass", "grassNdirt", "stone_dirt", "bush", "leaves", "iron", "lamp", "stone_brick",
               "stone_brick_cracked", "stone_pack", "bark", "wood", "planks"]


def demo_world():
    slots = 15   # LumSettings.static_block_palette_size default (crenderer.h:41)
    grid = vox.load_scene(os.path.join(ASSETS, "scene"), (48, 48, 16), slots)
    pal = np.zeros((slots, 16, 16, 16), dtype=np.uint8)
    for i, name in enumerate(DEMO_BLOCKS, start=1):
        pal[i] = vox.load_block(os.path.join(ASSETS, name + ".vox")).transpose(2, 1, 0)   # [x][y][z] -> [z][y][x]
    mats = vox.material_palette(os.path.join(ASSETS, "tank_body.vox"))
    return worldgen.World(grid=grid, palette=pal, materials=mats)


def run_reference(world, req, prev, passes, unorm10=False, **p):
    outs = []
    cur = prev
    for i in range(passes):
        q = dict(p)
        q["time_seed"] = p.get("time_seed", 0) + i
        cur, _, _, abandoned = build_ref.run_pass(world, req.astype(np.int8), prev=cur, unorm10=unorm10, **q)
        assert abandoned == 0
        outs.append(cur)
    return np.stack(outs)


def save(name, world, req, prev, passes, unorm10=False, **p):
    if unorm10:
        prev = oracle.quantize_unorm10(prev)   # the image holds 10-bit codes from the start
    out = run_reference(world, req, prev, passes, unorm10=unorm10, **p)
    extra = {"storage": np.array("rgb10a2")} if unorm10 else {}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), grid=world.grid, palette=world.palette,
                        materials=world.materials, requests=req, prev=prev, expected=out,
                        params=np.array([p["rays"], p["max_dist"], p["blend"], p.get("time_seed", 0),
                                         p.get("size", 1), p.get("shift", 0), passes], dtype=np.float64), **extra)
    print(f"{name}: {req.shape[0]} requests, {passes} pass(es), mean radiance {out[-1].mean():.5f}")


def main():
    build_ref.build()
    w = demo_world()
    req = oracle.update_list(w)
    save("demo_scene", w, req, np.zeros(w.grid.shape + (3,), np.float32), 2,
         rays=64, max_dist=128.0, blend=0.01, time_seed=0)

    w = worldgen.small_world()
    prev = (worldgen.uniform(7, 99, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.5).astype(np.float32)
    save("terrain_c1", w, worldgen.all_probes(w.dims), prev, 1, rays=64, max_dist=128.0, blend=0.1, time_seed=0)

    w = worldgen.terrain_world((12, 10, 6), seed=21, extra_blocks=40)
    prev = (worldgen.uniform(8, 99, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.5).astype(np.float32)
    save("slicing_r256", w, worldgen.all_probes(w.dims), prev, 2, rays=256, max_dist=256.0, blend=0.1,
         time_seed=3, size=2, shift=1)

    w = worldgen.terrain_world((9, 9, 5), seed=30, n_types=8)
    g = w.grid.reshape(-1).copy()
    idx = worldgen.randint(31, 1, 60, 0, g.size)
    vals = np.array([-1, -5, -63, -64, -200, 9, 40, 4095, 32767, 12], dtype=np.int16)
    g[idx] = vals[np.arange(60) % vals.size]
    pal = w.palette.copy()
    pal[0, 3:5, :, 6:9] = 17
    w = worldgen.World(grid=g.reshape(w.grid.shape), palette=pal, materials=w.materials)
    prev = (worldgen.uniform(9, 99, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.5).astype(np.float32)
    save("odd_ids", w, worldgen.all_probes(w.dims), prev, 1, rays=32, max_dist=160.0, blend=0.2, time_seed=4)

    # the reference's own volume format
    w = demo_world()
    req = oracle.update_list(w)
    save("demo_scene_rgb10a2", w, req, np.zeros(w.grid.shape + (3,), np.float32), 3, unorm10=True,
         rays=64, max_dist=128.0, blend=0.01, time_seed=0)
    w = worldgen.terrain_world((10, 8, 6), seed=23, extra_blocks=20)
    prev = (worldgen.uniform(10, 99, w.n_blocks * 3).reshape(w.grid.shape + (3,)) * 0.7).astype(np.float32)
    save("terrain_rgb10a2", w, worldgen.all_probes(w.dims), prev, 3, unorm10=True, rays=128, max_dist=128.0,
         blend=0.3, time_seed=2)


if __name__ == "__main__":
    main()
