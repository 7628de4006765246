"""lum_gb300 — GB300-native per-block radiance-field update (Lum's radiance pass).

The product is the shared library liblumrad.so behind include/lumrad.h; this package builds it
(`lum_gb300.build`) and wraps it for Python callers (`RadianceWorld`), in the shape of Lum's C API
(src/renderer/api/crenderer.h): create a world, load blocks, materials and the block grid, run
radiance passes, read the radiance volume back.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import (HIT_DTYPE, PRECISION, LumRadError, Material, PassParams, PassStats, Settings,
                      check, load, ptr)

__all__ = ["RadianceWorld", "RadianceBatch", "RadianceServer", "PassParams", "LumRadError", "HIT_DTYPE", "load",
           "pass_params", "dirty_probes", "direction_table"]


def pass_params(rays: int = 64, max_dist: float = 128.0, blend: float = 0.01, time_seed: int = 0,
                size: int = 1, shift: int = 0, record_hits: bool = False) -> PassParams:
    """Pass parameters; the defaults are radiance.comp's own constants."""
    return PassParams(rays, max_dist, blend, time_seed, size, shift, 1 if record_hits else 0)


class RadianceWorld:
    """One world resident on one GPU (a LumRadContext)."""

    def __init__(self, world_size, max_block_types: int = 64, precision: str = "fp32", device: int = 0):
        self.lib = load()
        X, Y, Z = (int(v) for v in world_size)
        self.dims = (X, Y, Z)
        s = Settings((C.c_int * 3)(X, Y, Z), int(max_block_types), PRECISION[precision], int(device))
        h = C.c_void_p()
        check(self.lib.lumrad_create(C.byref(s), C.byref(h)))
        self.h = h
        self.precision = precision
        self.max_block_types = max_block_types

    # ---- lifetime
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lumrad_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_blocks(self) -> int:
        return self.dims[0] * self.dims[1] * self.dims[2]

    def synchronize(self) -> None:
        check(self.lib.lumrad_synchronize(self.h))

    # ---- inputs
    def load_world(self, grid: np.ndarray) -> None:
        g = np.ascontiguousarray(grid, dtype=np.int16)
        assert g.size == self.n_blocks
        check(self.lib.lumrad_load_world(self.h, ptr(g)))

    def set_world_block(self, x: int, y: int, z: int, block: int) -> None:
        check(self.lib.lumrad_set_world_block(self.h, x, y, z, block))

    def get_world_block(self, x: int, y: int, z: int) -> int:
        out = C.c_int16()
        check(self.lib.lumrad_get_world_block(self.h, x, y, z, C.byref(out)))
        return int(out.value)

    def load_block(self, block: int, voxels_xyz: np.ndarray) -> None:
        """voxels indexed [x][y][z] (Lum's BlockVoxels)."""
        v = np.ascontiguousarray(voxels_xyz, dtype=np.uint8)
        assert v.shape == (16, 16, 16)
        check(self.lib.lumrad_load_block(self.h, block, ptr(v)))

    def upload_block_palette(self) -> None:
        check(self.lib.lumrad_upload_block_palette(self.h))

    def load_materials(self, mats: np.ndarray) -> None:
        m = np.ascontiguousarray(mats, dtype=np.float32)
        assert m.shape == (256, 6)
        check(self.lib.lumrad_load_materials(self.h, ptr(m)))

    def upload_material_palette(self) -> None:
        check(self.lib.lumrad_upload_material_palette(self.h))

    def load(self, world) -> None:
        """Loads a worldgen.World: grid, every palette slot and the materials, then uploads."""
        self.load_world(world.grid)
        for slot in range(min(world.palette.shape[0], self.max_block_types)):
            self.load_block(slot, world.block_voxels(slot))
        self.upload_block_palette()
        self.load_materials(world.materials)
        self.upload_material_palette()

    # ---- radiance volume
    def get_radiance(self, out: np.ndarray | None = None) -> np.ndarray:
        """The volume as (Z, Y, X, 3) float32; into `out` if given (a page-locked `out`, e.g. a
        pinned torch tensor's numpy view, receives the device copy directly)."""
        X, Y, Z = self.dims
        if out is None:
            out = np.empty((Z, Y, X, 3), dtype=np.float32)
        elif out.dtype != np.float32 or out.size != 3 * self.n_blocks or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 array of (Z, Y, X, 3) values")
        check(self.lib.lumrad_get_radiance(self.h, ptr(out)))
        return out

    def set_radiance(self, rgb: np.ndarray) -> None:
        r = np.ascontiguousarray(rgb, dtype=np.float32)
        assert r.size == 3 * self.n_blocks
        check(self.lib.lumrad_set_radiance(self.h, ptr(r)))

    # ---- passes
    def build_update_list(self) -> np.ndarray:
        """The update list (27-neighbour rule, then the queued specials); one build when it fits
        every block plus 4,096 specials, else a second with the exact size."""
        n = C.c_int()
        cap = self.n_blocks + 4096
        out = np.empty((cap, 4), dtype=np.int16)
        check(self.lib.lumrad_build_update_list(self.h, ptr(out), cap, C.byref(n)))
        if n.value > cap:
            out = np.empty((n.value, 4), dtype=np.int16)
            check(self.lib.lumrad_build_update_list(self.h, ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def build_dirty_list(self, edits, radius: int = 2) -> np.ndarray:
        """Probes within `radius` blocks of the edits, derived on the device; (n, 4) int16."""
        e = _edits(edits)
        n = C.c_int()
        out = np.zeros((self.n_blocks, 4), dtype=np.int16)
        check(self.lib.lumrad_build_dirty_list(self.h, e.ctypes.data if e.size else None, e.size, radius, ptr(out),
                                               self.n_blocks, C.byref(n)))
        return out[: n.value]

    def request_update(self, x: int, y: int, z: int) -> None:
        check(self.lib.lumrad_request_update(self.h, x, y, z))

    def update_radiance(self, params: PassParams) -> None:
        check(self.lib.lumrad_update_radiance(self.h, C.byref(params)))

    def radiance_pass(self, requests: np.ndarray, params: PassParams) -> None:
        req = np.ascontiguousarray(requests)
        assert req.ndim == 2 and req.shape[1] == 4
        if req.dtype == np.int8:
            check(self.lib.lumrad_radiance_pass_i8(self.h, ptr(req), req.shape[0], C.byref(params)))
        else:
            req = req.astype(np.int16, copy=False)
            check(self.lib.lumrad_radiance_pass(self.h, ptr(req), req.shape[0], C.byref(params)))

    def load_model(self, voxels_zyx: np.ndarray) -> int:
        """A voxel model given as a (sz, sy, sx) uint8 array (x-fastest in memory); returns its index."""
        v = np.ascontiguousarray(voxels_zyx, dtype=np.uint8)
        sz, sy, sx = v.shape
        i = C.c_int()
        check(self.lib.lumrad_load_model(self.h, ptr(v), sx, sy, sz, C.byref(i)))
        return int(i.value)

    def blockify(self, static_blocks: int, meshes) -> None:
        """meshes: [(model index, (qx, qy, qz, qw), (sx, sy, sz))] in processing order."""
        from ._native import MeshTransform
        n = len(meshes)
        models = (C.c_int * max(n, 1))(*[int(m[0]) for m in meshes])
        tr = (MeshTransform * max(n, 1))()
        for k, (_, q, s) in enumerate(meshes):
            tr[k].rot[:] = [float(v) for v in q]
            tr[k].shift[:] = [float(v) for v in s]
        check(self.lib.lumrad_blockify(self.h, int(static_blocks), models, tr, n))

    def get_world(self) -> np.ndarray:
        X, Y, Z = self.dims
        out = np.empty((Z, Y, X), dtype=np.int16)
        check(self.lib.lumrad_get_world(self.h, ptr(out)))
        return out

    def get_block_palette(self) -> np.ndarray:
        """(max_block_types, 16, 16, 16) uint8 indexed [slot, z, y, x]."""
        out = np.empty((self.max_block_types, 16, 16, 16), dtype=np.uint8)
        check(self.lib.lumrad_get_block_palette(self.h, ptr(out)))
        return out

    def shift_radiance(self, dx: int, dy: int, dz: int) -> None:
        check(self.lib.lumrad_shift_radiance(self.h, int(dx), int(dy), int(dz)))

    def set_radiance_shift(self, dx: int, dy: int, dz: int) -> None:
        check(self.lib.lumrad_set_radiance_shift(self.h, int(dx), int(dy), int(dz)))

    def get_radiance_shift(self) -> tuple:
        out = (C.c_int * 3)()
        check(self.lib.lumrad_get_radiance_shift(self.h, out))
        return tuple(out)

    def gather(self, points: np.ndarray) -> np.ndarray:
        """diffuse.frag's 8-probe radiance gather at (n, 6) points (position, normal)."""
        p = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 6)
        out = np.zeros((p.shape[0], 3), dtype=np.float32)
        check(self.lib.lumrad_gather_radiance(self.h, ptr(p), p.shape[0], ptr(out)))
        return out

    def gather_device(self, d_points: int, n: int, d_rgb: int) -> None:
        """The gather on device pointers ((n, 6) and (n, 3) float32), enqueued on this context's
        stream (e.g. torch tensors' data_ptr())."""
        check(self.lib.lumrad_gather_radiance_device(self.h, C.c_void_p(d_points), int(n), C.c_void_p(d_rgb)))

    def radiance_passes(self, lists, params) -> None:
        """Passes over int16 (n, 4) lists in order, as radiance_pass over each would run them;
        their marches share launches.  Lists that already are C-contiguous int16 (n, 4) arrays are
        passed as they are (the call's own cost sits before the GPU's first launch)."""
        n = len(lists)
        ptrs = (C.c_void_p * max(n, 1))()
        counts = (C.c_int * max(n, 1))()
        keep = []
        for i, r in enumerate(lists):
            if not (type(r) is np.ndarray and r.dtype == np.int16 and r.ndim == 2 and r.shape[1] == 4
                    and r.flags.c_contiguous):
                r = np.ascontiguousarray(r, dtype=np.int16).reshape(-1, 4)
                keep.append(r)
            ptrs[i] = r.__array_interface__["data"][0]
            counts[i] = r.shape[0]
        ps = params if isinstance(params, C.Array) else (PassParams * max(n, 1))(*params)
        check(self.lib.lumrad_radiance_passes(self.h, ptrs, counts, ps, n))

    def radiance_passes_packed(self, requests: np.ndarray, counts, params) -> None:
        """radiance_passes over lists stored back to back in one C-contiguous int16 (total, 4)
        array: list i is the next counts[i] rows.  One pointer lookup instead of one per list
        (a page-locked array is copied straight from, as one run)."""
        if not (type(requests) is np.ndarray and requests.dtype == np.int16 and requests.ndim == 2
                and requests.shape[1] == 4 and requests.flags.c_contiguous):
            raise ValueError("requests must be a C-contiguous int16 (total, 4) array")
        n = len(counts)
        ptrs = (C.c_void_p * max(n, 1))()
        cts = (C.c_int * max(n, 1))()
        base, off = requests.ctypes.data, 0
        for i, c in enumerate(counts):
            c = int(c)
            if c < 0:
                raise ValueError("counts must be non-negative")
            ptrs[i] = base + 8 * off
            cts[i] = c
            off += c
        if off != requests.shape[0]:
            raise ValueError("counts must add up to the rows of requests")
        ps = params if isinstance(params, C.Array) else (PassParams * max(n, 1))(*params)
        check(self.lib.lumrad_radiance_passes(self.h, ptrs, cts, ps, n))

    def radiance_passes_resident(self, slots, params) -> None:
        n = len(slots)
        sl = (C.c_int * max(n, 1))(*[int(s) for s in slots])
        ps = (PassParams * max(n, 1))(*params)
        check(self.lib.lumrad_radiance_passes_resident(self.h, sl, ps, n))

    def upload_requests(self, slot: int, requests: np.ndarray) -> None:
        req = np.ascontiguousarray(requests, dtype=np.int16)
        check(self.lib.lumrad_upload_requests(self.h, slot, ptr(req), req.shape[0]))

    def radiance_pass_resident(self, slot: int, params: PassParams) -> None:
        check(self.lib.lumrad_radiance_pass_resident(self.h, slot, C.byref(params)))

    def get_hits(self) -> np.ndarray:
        n = C.c_size_t()
        rc = self.lib.lumrad_get_hits(self.h, None, 0, C.byref(n))
        check(rc)
        out = np.zeros(n.value, dtype=HIT_DTYPE)
        check(self.lib.lumrad_get_hits(self.h, out.ctypes.data, n.value, C.byref(n)))
        return out

    def stream(self) -> int:
        """cudaStream_t of this context as an integer handle."""
        out = C.c_void_p()
        check(self.lib.lumrad_get_stream(self.h, C.byref(out)))
        return int(out.value or 0)

    def kernel_times(self, cap: int = 64) -> np.ndarray:
        """Device ms of the pass kernels of the last min(cap, 64) passes, oldest first."""
        out = np.zeros(cap, dtype=np.float32)
        n = C.c_int()
        check(self.lib.lumrad_get_kernel_times(self.h, ptr(out), cap, C.byref(n)))
        return out[: n.value]

    def pass_stats(self) -> dict:
        s = PassStats()
        check(self.lib.lumrad_get_pass_stats(self.h, C.byref(s)))
        return {"probes": s.probes, "rays": s.rays, "steps": s.steps, "hits": s.hits, "gpu_ms": s.gpu_ms}


class RadianceBatch:
    """Many RadianceWorlds updated by one graph-replayed launch (lumrad_batch_*)."""

    def __init__(self, worlds):
        self.lib = load()
        self.worlds = list(worlds)
        arr = (C.c_void_p * len(self.worlds))(*[w.h.value for w in self.worlds])
        h = C.c_void_p()
        check(self.lib.lumrad_batch_create(arr, len(self.worlds), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.lumrad_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_requests(self, i: int, requests: np.ndarray, params: PassParams) -> None:
        req = np.ascontiguousarray(requests, dtype=np.int16)
        check(self.lib.lumrad_batch_set_requests(self.h, i, ptr(req), req.shape[0], C.byref(params)))

    def run(self, time_seed: int = 0) -> None:
        check(self.lib.lumrad_batch_run(self.h, time_seed))

    def run_per_world(self, time_seed: int = 0) -> None:
        check(self.lib.lumrad_batch_run_per_world(self.h, time_seed))

    def synchronize(self) -> None:
        check(self.lib.lumrad_batch_synchronize(self.h))

    def last_ms(self) -> float:
        ms = C.c_float()
        check(self.lib.lumrad_batch_last_ms(self.h, C.byref(ms)))
        return float(ms.value)

    def set_tuning(self, guided_div: int = 2, max_chunk: int = 16, march_ctas: int = 0) -> None:
        from ._native import Tuning
        t = Tuning(guided_div, max_chunk, march_ctas, 0.0)
        check(self.lib.lumrad_batch_set_tuning(self.h, C.byref(t)))

    def autotune(self, repeats: int = 3) -> dict:
        from ._native import Tuning
        t = Tuning()
        check(self.lib.lumrad_batch_autotune(self.h, repeats, C.byref(t)))
        return {"guided_div": t.guided_div, "max_chunk": t.max_chunk, "march_ctas": t.march_ctas,
                "pass_ms": t.pass_ms}

    def stats(self) -> dict:
        s = PassStats()
        check(self.lib.lumrad_batch_stats(self.h, C.byref(s)))
        return {"probes": s.probes, "rays": s.rays, "steps": s.steps, "hits": s.hits, "gpu_ms": s.gpu_ms}


def _edits(edits) -> np.ndarray:
    from ._native import EDIT_DTYPE
    e = np.asarray(edits)
    if e.dtype != EDIT_DTYPE:
        e = np.ascontiguousarray(e, dtype=np.int16).reshape(-1, 4)
        e = e.view(EDIT_DTYPE).reshape(-1)
    return np.ascontiguousarray(e)


class RadianceServer:
    """Relight requests over resident worlds, continuously batched (lumrad_server_*)."""

    def __init__(self, device: int = 0, precision: str = "fp32", hbm_budget_bytes: float = 0.0,
                 max_inflight: int = 4, max_requests_per_launch: int = 0, radius: int = 2,
                 device_loop: bool = False, poll_ms: float = 0.0, max_queue_ms: float = 0.0):
        from ._native import ServerSettings
        self.lib = load()
        s = ServerSettings(int(device), PRECISION[precision], float(hbm_budget_bytes), int(max_inflight),
                           int(max_requests_per_launch), int(radius), 1 if device_loop else 0, float(poll_ms),
                           float(max_queue_ms))
        h = C.c_void_p()
        check(self.lib.lumrad_server_create(C.byref(s), C.byref(h)))
        self.h = h
        self.worlds = []

    def close(self):
        if getattr(self, "h", None):
            self.lib.lumrad_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_world(self, world: RadianceWorld) -> int:
        i = C.c_int()
        check(self.lib.lumrad_server_add_world(self.h, world.h, C.byref(i)))
        self.worlds.append(world)
        return int(i.value)

    def submit(self, world: int, edits, params: PassParams, arrival_s: float = -1.0) -> int:
        e = _edits(edits)
        rid = C.c_longlong()
        check(self.lib.lumrad_server_submit(self.h, world, e.ctypes.data if e.size else None, e.size,
                                            C.byref(params), float(arrival_s), C.byref(rid)))
        return int(rid.value)

    def progress(self) -> None:
        check(self.lib.lumrad_server_progress(self.h))

    def run(self, timeout_s: float = 600.0) -> None:
        check(self.lib.lumrad_server_run(self.h, float(timeout_s)))

    def cancel(self, request: int) -> bool:
        """Cancels a request not launched yet; True if it was."""
        out = C.c_int()
        check(self.lib.lumrad_server_cancel(self.h, int(request), C.byref(out)))
        return bool(out.value)

    def poll(self, cap: int = 65536) -> np.ndarray:
        from ._native import COMPLETION_DTYPE
        out = np.zeros(cap, dtype=COMPLETION_DTYPE)
        n = C.c_int()
        check(self.lib.lumrad_server_poll(self.h, out.ctypes.data, cap, C.byref(n)))
        return out[: n.value]

    def now(self) -> float:
        return float(self.lib.lumrad_server_now(self.h))

    def get_radiance(self, world: int) -> np.ndarray:
        if not 0 <= world < len(self.worlds):
            from ._native import LUMRAD_EINVAL
            raise LumRadError(LUMRAD_EINVAL, "unknown world")
        X, Y, Z = self.worlds[world].dims
        out = np.empty((Z, Y, X, 3), dtype=np.float32)
        check(self.lib.lumrad_server_get_radiance(self.h, world, ptr(out)))
        return out

    def stats(self) -> dict:
        from ._native import ServerStats
        s = ServerStats()
        check(self.lib.lumrad_server_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}


def dirty_probes(world_size, edits, radius: int = 2) -> np.ndarray:
    """Probes within Chebyshev distance `radius` of the edits, (n, 4) int16 in scan order."""
    e = _edits(edits)
    ws = (C.c_int * 3)(*[int(v) for v in world_size])
    n = C.c_int()
    lib = load()
    check(lib.lumrad_dirty_probes(ws, e.ctypes.data if e.size else None, e.size, radius, None, 0, C.byref(n)))
    out = np.zeros((max(n.value, 1), 4), dtype=np.int16)
    check(lib.lumrad_dirty_probes(ws, e.ctypes.data if e.size else None, e.size, radius, ptr(out), n.value,
                                  C.byref(n)))
    return out[: n.value]


def direction_table(rays: int) -> np.ndarray:
    out = np.zeros((rays, 3), dtype=np.float32)
    check(load().lumrad_direction_table(rays, ptr(out)))
    return out
