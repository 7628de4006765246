"""The reference shader (compiled as C++ by build_ref) on all host cores — TEST INFRASTRUCTURE.

The shader's emulation keeps its state in globals, so parallelism is by processes: a spawn-started
pool whose workers each load the world once and run a slice of a dispatch's workgroups.  The
previous radiance volume is shared with the workers through shared memory.  Used by bench.py's
reference arm only.
"""
from __future__ import annotations

import multiprocessing as mp
import os
from multiprocessing import shared_memory

import numpy as np

_W = {}


def _init(grid, palette, materials, rays, shm_name):
    from oracle import build_ref
    shm = shared_memory.SharedMemory(name=shm_name)
    prev = np.ndarray(grid.shape + (3,), dtype=np.float32, buffer=shm.buf)
    _W.update(grid=grid, palette=palette, materials=materials, rays=rays, lib=build_ref.load(rays), shm=shm,
              prev=prev)


def _run(args):
    import ctypes as C

    from oracle import build_ref
    req, max_dist, blend, seed, size, shift, g0, g1 = args
    lib = _W["lib"]
    grid, pal, mats, prev = _W["grid"], _W["palette"], _W["materials"], _W["prev"]
    Z, Y, X = grid.shape
    w = build_ref.RefWorld(X, Y, Z, grid.ctypes.data, pal.ctypes.data, pal.shape[0], mats.ctypes.data)
    q = req[np.arange(g0, g1) * size + shift, :3].astype(np.int64)
    ok = (q >= 0).all(axis=1) & (q[:, 0] < X) & (q[:, 1] < Y) & (q[:, 2] < Z)
    q = q[ok]
    nxt = prev.copy()   # the harness writes only the probes of its workgroups
    lib.lumref_pass(C.byref(w), req.ctypes.data, req.shape[0], seed, size, shift, max_dist, blend, prev.ctypes.data,
                    nxt.ctypes.data, None, None, g0, g1)
    return q, nxt[q[:, 2], q[:, 1], q[:, 0]]


class RefPool:
    def __init__(self, world, rays: int, processes: int | None = None):
        from oracle import build_ref
        build_ref.load(rays)   # fail early if the library is missing
        self.processes = processes or os.cpu_count() or 1
        self.rays = rays
        self.shape = tuple(world.grid.shape) + (3,)
        self.shm = shared_memory.SharedMemory(create=True, size=int(np.prod(self.shape)) * 4)
        self.prev = np.ndarray(self.shape, dtype=np.float32, buffer=self.shm.buf)
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(self.processes, initializer=_init,
                             initargs=(np.ascontiguousarray(world.grid, dtype=np.int16),
                                       np.ascontiguousarray(world.palette, dtype=np.uint8),
                                       np.ascontiguousarray(world.materials, dtype=np.float32), rays, self.shm.name))

    def run_pass(self, requests_i8, prev, max_dist=128.0, blend=0.01, time_seed=0, size=1, shift=0):
        req = np.ascontiguousarray(requests_i8, dtype=np.int8)
        self.prev[...] = prev
        groups = req.shape[0] // size
        n = max(1, min(groups, 2 * self.processes))
        edges = np.linspace(0, groups, n + 1).astype(int)
        jobs = [(req, max_dist, blend, time_seed, size, shift, int(a), int(b))
                for a, b in zip(edges[:-1], edges[1:]) if b > a]
        nxt = np.array(prev, dtype=np.float32, copy=True)
        for q, v in self.pool.map(_run, jobs):
            nxt[q[:, 2], q[:, 1], q[:, 0]] = v
        return nxt

    def close(self):
        self.pool.close()
        self.pool.join()
        self.shm.close()
        self.shm.unlink()
