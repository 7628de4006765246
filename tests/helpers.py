"""Shared test helpers: run one pass through the C ABI and through the CPU oracle."""
from __future__ import annotations

import numpy as np

from lum_gb300 import worldgen

RTOL = 1e-5      # FP32 radiance vs the FP32 oracle (relative, floor 1e-6)


def random_prev(world, seed: int = 7, scale: float = 0.5) -> np.ndarray:
    u = worldgen.uniform(seed, 99, world.n_blocks * 3)
    return (u.reshape(world.grid.shape + (3,)) * scale).astype(np.float32)


def gpu_pass(world, req, prev, precision="fp32", passes=1, seeds=None, **params):
    import lum_gb300
    with lum_gb300.RadianceWorld(world.dims, max_block_types=world.palette.shape[0], precision=precision) as rw:
        rw.load(world)
        rw.set_radiance(prev)
        hits = None
        for i in range(passes):
            p = dict(params)
            if seeds is not None:
                p["time_seed"] = seeds[i]
            rw.radiance_pass(req, lum_gb300.pass_params(record_hits=True, **p))
            hits = rw.get_hits()
        stats = rw.pass_stats()
        return rw.get_radiance(), hits, stats


def oracle_pass(world, req, prev, passes=1, seeds=None, precision="f32", **params):
    import oracle
    cur = prev.astype(np.float32 if precision == "f32" else np.float64)
    hits = stats = None
    for i in range(passes):
        p = dict(params)
        if seeds is not None:
            p["time_seed"] = seeds[i]
        cur, hits, stats = oracle.radiance_pass(world, req, prev=cur, record_hits=True, precision=precision, **p)
    return cur, hits, stats


def rel_err(got, ref, floor=1e-6):
    return np.abs(got.astype(np.float64) - ref.astype(np.float64)) / np.maximum(np.abs(ref.astype(np.float64)), floor)


def assert_hits_equal(got, ref):
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if got.tobytes() != ref.tobytes():
        diff = np.nonzero(got != ref)[0]
        raise AssertionError(f"{diff.size} of {got.size} hit records differ; first {diff[:5]}:\n"
                             f"gpu    {got[diff[:3]]}\noracle {ref[diff[:3]]}")
