"""CPU oracle of the radiance pass — TEST INFRASTRUCTURE, not product code.

Builds oracle/radiance_oracle.cpp with g++ (OpenMP, -ffp-contract=off) into oracle/_build/ and
wraps it with ctypes.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker or the timed CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "radiance_oracle.cpp")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]

HIT_DTYPE = np.dtype([("voxel", "<i4", (3,)), ("block", "<i2"), ("voxel_id", "u1"), ("flags", "u1"),
                      ("coarse_steps", "<u2"), ("refine_steps", "u1"), ("coarse_voxel", "u1"),
                      ("fraction", "<f4")])


class OWorld(C.Structure):
    _fields_ = [("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int), ("grid", C.c_void_p),
                ("palette", C.c_void_p), ("n_slots", C.c_int), ("materials", C.c_void_p)]


class OParams(C.Structure):
    _fields_ = [("rays", C.c_int), ("max_dist", C.c_float), ("blend", C.c_float), ("time_seed", C.c_int),
                ("size", C.c_int), ("shift", C.c_int), ("unorm10", C.c_int)]


class OStats(C.Structure):
    _fields_ = [("probes", C.c_uint64), ("rays", C.c_uint64), ("steps", C.c_uint64), ("hits", C.c_uint64)]


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++", *CXXFLAGS, SRC, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        build()
    lib = C.CDLL(LIB)
    P = C.c_void_p
    lib.oracle_pass_f32.argtypes = [P, P, C.c_int, P, P, P, P, P, P, C.c_int]
    lib.oracle_pass_f64.argtypes = [P, P, C.c_int, P, P, P, P, P, P, C.c_int]
    lib.oracle_hash33.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, P]
    lib.oracle_hash33.restype = None
    lib.oracle_direction_table.argtypes = [C.c_int, P]
    lib.oracle_trace_ray.argtypes = [P, P, P, P, C.c_float, P, P]
    lib.oracle_update_list.argtypes = [P, P, C.c_int, P, C.c_int, P]
    lib.oracle_shift.argtypes = [C.c_int, C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_int]
    lib.oracle_gather.argtypes = [C.c_int, C.c_int, C.c_int, P, P, C.c_int, P]
    lib.oracle_blockify.argtypes = [C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P, C.c_int]
    lib.oracle_max_threads.restype = C.c_int
    _lib = lib
    return lib


class _Keep:
    """Holds the arrays an OWorld points into."""

    def __init__(self, grid, palette, materials):
        self.grid = np.ascontiguousarray(grid, dtype=np.int16)
        self.palette = np.ascontiguousarray(palette, dtype=np.uint8)
        self.materials = np.ascontiguousarray(materials, dtype=np.float32)
        Z, Y, X = self.grid.shape
        self.c = OWorld(X, Y, Z, self.grid.ctypes.data, self.palette.ctypes.data,
                        self.palette.shape[0], self.materials.ctypes.data)


def world_struct(world) -> _Keep:
    """world: an object with grid (Z,Y,X) int16, palette (slots,16,16,16) [slot,z,y,x], materials (256,6)."""
    return _Keep(world.grid, world.palette, world.materials)


def radiance_pass(world, requests: np.ndarray, rays: int = 64, max_dist: float = 128.0, blend: float = 0.01,
                  time_seed: int = 0, size: int = 1, shift: int = 0, prev: np.ndarray | None = None,
                  precision: str = "f32", record_hits: bool = False, threads: int = 0,
                  ray_light: np.ndarray | None = None, unorm10: bool = False):
    """One pass; returns (next radiance (Z,Y,X,3), hits or None, stats dict).
    ray_light, if given, receives each ray's light ((groups*rays, 3), the pass's precision).
    unorm10: the volume is stored as A2B10G10R10_UNORM (prev must hold such values already,
    e.g. quantize_unorm10's)."""
    lib = load()
    k = world_struct(world)
    Z, Y, X = k.grid.shape
    dt = np.float32 if precision == "f32" else np.float64
    if prev is None:
        prev = np.zeros((Z, Y, X, 3), dtype=dt)
    prev = np.ascontiguousarray(prev, dtype=dt)
    nxt = np.empty_like(prev)
    req = np.ascontiguousarray(requests, dtype=np.int16)
    p = OParams(rays, max_dist, blend, time_seed, size, shift, 1 if unorm10 else 0)
    groups = req.shape[0] // size
    hits = np.zeros(groups * rays, dtype=HIT_DTYPE) if record_hits else None
    st = OStats()
    fn = lib.oracle_pass_f32 if precision == "f32" else lib.oracle_pass_f64
    rc = fn(C.byref(k.c), req.ctypes.data if req.size else None, req.shape[0], C.byref(p),
            prev.ctypes.data, nxt.ctypes.data, hits.ctypes.data if hits is not None else None,
            C.byref(st), ray_light.ctypes.data if ray_light is not None else None, threads)
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return nxt, hits, {"probes": st.probes, "rays": st.rays, "steps": st.steps, "hits": st.hits}


def quantize_unorm10(rgb: np.ndarray) -> np.ndarray:
    """Float RGB as an A2B10G10R10_UNORM image holds it: clamped to [0, 1] (NaN -> 0), code = round
    to nearest even of v * 1023 in FP32, read back as code / 1023 in FP32."""
    v = np.nan_to_num(np.asarray(rgb, dtype=np.float32), nan=0.0)
    v = np.clip(v, np.float32(0), np.float32(1))
    return (np.rint(v * np.float32(1023)) / np.float32(1023)).astype(np.float32)


def hash33(x: int, y: int, z: int) -> np.ndarray:
    out = np.zeros(3, dtype=np.float32)
    load().oracle_hash33(x & 0xFFFFFFFF, y & 0xFFFFFFFF, z & 0xFFFFFFFF, out.ctypes.data)
    return out


def direction_table(n: int) -> np.ndarray:
    out = np.zeros((n, 3), dtype=np.float32)
    load().oracle_direction_table(n, out.ctypes.data)
    return out


def trace_ray(world, origin, direction, max_dist: float = 128.0, prev: np.ndarray | None = None):
    lib = load()
    k = world_struct(world)
    Z, Y, X = k.grid.shape
    if prev is None:
        prev = np.zeros((Z, Y, X, 3), dtype=np.float32)
    prev = np.ascontiguousarray(prev, dtype=np.float32)
    o = np.asarray(origin, dtype=np.float32)
    d = np.asarray(direction, dtype=np.float32)
    light = np.zeros(3, dtype=np.float32)
    hit = np.zeros(1, dtype=HIT_DTYPE)
    lib.oracle_trace_ray(C.byref(k.c), prev.ctypes.data, o.ctypes.data, d.ctypes.data, max_dist,
                         light.ctypes.data, hit.ctypes.data)
    return light, hit[0]


def update_list(world, specials: np.ndarray | None = None) -> np.ndarray:
    lib = load()
    k = world_struct(world)
    sp = np.zeros((0, 4), dtype=np.int16) if specials is None else np.ascontiguousarray(specials, dtype=np.int16)
    cap = k.grid.size + sp.shape[0]
    out = np.zeros((max(cap, 1), 4), dtype=np.int16)
    n = C.c_int()
    rc = lib.oracle_update_list(C.byref(k.c), sp.ctypes.data if sp.size else None, sp.shape[0],
                                out.ctypes.data, cap, C.byref(n))
    if rc != 0:
        raise ValueError("special request outside the world")
    return out[: n.value]


def shift_radiance(volume: np.ndarray, shift) -> np.ndarray:
    """shift_radiance (internal_render.cpp:1218-1335) of a (Z, Y, X, 3) float32 volume; returns a copy."""
    v = np.ascontiguousarray(volume, dtype=np.float32).copy()
    Z, Y, X, _ = v.shape
    load().oracle_shift(X, Y, Z, v.ctypes.data, int(shift[0]), int(shift[1]), int(shift[2]))
    return v


def gather(volume: np.ndarray, points: np.ndarray) -> np.ndarray:
    """diffuse.frag:24-90's 8-probe gather of a (Z, Y, X, 3) float32 volume at (n, 6) points."""
    v = np.ascontiguousarray(volume, dtype=np.float32)
    p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 6)
    out = np.zeros((p.shape[0], 3), dtype=np.float32)
    Z, Y, X, _ = v.shape
    load().oracle_gather(X, Y, Z, v.ctypes.data, p.ctypes.data, p.shape[0], out.ctypes.data)
    return out


def blockify(grid: np.ndarray, palette: np.ndarray, static_blocks: int, models, meshes):
    """One frame of blockify + exec_copies + map (internal_render.cpp:977-1070,1375-1520, map.comp).
    grid (Z,Y,X) int16, palette (n_slots,16,16,16) uint8 [slot,z,y,x], models: list of (sz,sy,sx)
    uint8 arrays, meshes: [(model, quat xyzw, shift xyz)].  Returns (grid, palette) or None when
    the temporary slots run out."""
    g = np.ascontiguousarray(grid, dtype=np.int16).copy()
    p = np.ascontiguousarray(palette, dtype=np.uint8).copy()
    Z, Y, X = g.shape
    n = len(meshes)
    arrs = [np.ascontiguousarray(models[m[0]], dtype=np.uint8) for m in meshes]
    ptrs = (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in arrs])
    msize = np.array([[a.shape[2], a.shape[1], a.shape[0]] for a in arrs] or [[1, 1, 1]], dtype=np.int32)
    rot = np.array([m[1] for m in meshes] or [[0, 0, 0, 1]], dtype=np.float32)
    sh = np.array([m[2] for m in meshes] or [[0, 0, 0]], dtype=np.float32)
    rc = load().oracle_blockify(X, Y, Z, g.ctypes.data, p.ctypes.data, p.shape[0], int(static_blocks), ptrs,
                                msize.ctypes.data, rot.ctypes.data, sh.ctypes.data, n)
    if rc == -2:
        return None
    return g, p


def max_threads() -> int:
    return load().oracle_max_threads()
