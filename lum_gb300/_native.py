"""ctypes binding of liblumrad.so (include/lumrad.h).

This is the binding a Python caller of the C ABI writes; the tests and the benchmark use it.
It never falls back to anything: if the shared library is missing or does not load, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

LUMRAD_OK = 0
LUMRAD_EINVAL = -1
LUMRAD_ENOMEM = -2
LUMRAD_EDEVICE = -3
LUMRAD_ETIMEOUT = -4
LUMRAD_ESTATE = -5
LUMRAD_ECANCELED = -6
LUMRAD_TEST_LEAN_FINALIZE = 1
LUMRAD_TEST_PASS_MS = 2
LUMRAD_MAX_CHUNK = 4095   # include/lumrad.h: the largest LumRadTuning.max_chunk

PRECISION = {"fp32": 0, "fp16": 1, "bf16": 2, "rgb10a2": 3}


class Settings(C.Structure):
    _fields_ = [("world_size", C.c_int * 3), ("max_block_types", C.c_int),
                ("precision", C.c_int), ("device", C.c_int)]


class Material(C.Structure):
    _fields_ = [("color", C.c_float * 4), ("emmit", C.c_float), ("rough", C.c_float)]


class PassParams(C.Structure):
    _fields_ = [("rays_per_probe", C.c_int), ("max_dist", C.c_float), ("blend", C.c_float),
                ("time_seed", C.c_int), ("size", C.c_int), ("shift", C.c_int),
                ("record_hits", C.c_int)]


class MeshTransform(C.Structure):
    _fields_ = [("rot", C.c_float * 4), ("shift", C.c_float * 3)]


class PassStats(C.Structure):
    _fields_ = [("probes", C.c_uint64), ("rays", C.c_uint64), ("steps", C.c_uint64),
                ("hits", C.c_uint64), ("gpu_ms", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("guided_div", C.c_int), ("max_chunk", C.c_int), ("march_ctas", C.c_int), ("pass_ms", C.c_float)]


class ServerSettings(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("hbm_budget_bytes", C.c_double),
                ("max_inflight", C.c_int), ("max_requests_per_launch", C.c_int), ("radius", C.c_int),
                ("device_loop", C.c_int), ("poll_ms", C.c_float), ("max_queue_ms", C.c_float)]


class ServerStats(C.Structure):
    _fields_ = [("launches", C.c_longlong), ("requests", C.c_longlong), ("probes", C.c_uint64),
                ("rays", C.c_uint64), ("resident_bytes", C.c_double), ("launch_bytes", C.c_double),
                ("peak_inflight_bytes", C.c_double), ("max_requests_in_launch", C.c_int),
                ("evictions", C.c_longlong), ("readmissions", C.c_longlong), ("peak_device_bytes", C.c_double),
                ("shed", C.c_longlong)]


# LumRadEdit and LumRadCompletion as numpy records (same layout as the C structs)
EDIT_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2"), ("z", "<i2"), ("block", "<i2")])
COMPLETION_DTYPE = np.dtype([("request", "<i8"), ("world", "<i4"), ("status", "<i4"), ("probes", "<i4"),
                             ("rays_per_probe", "<i4"), ("arrival_s", "<f8"), ("start_s", "<f8"),
                             ("done_s", "<f8")])
assert EDIT_DTYPE.itemsize == 8 and COMPLETION_DTYPE.itemsize == 48

# LumRadHit as a numpy record (24 bytes, same layout as the C struct)
HIT_DTYPE = np.dtype([("voxel", "<i4", (3,)), ("block", "<i2"), ("voxel_id", "u1"), ("flags", "u1"),
                      ("coarse_steps", "<u2"), ("refine_steps", "u1"), ("coarse_voxel", "u1"),
                      ("fraction", "<f4")])
assert HIT_DTYPE.itemsize == 24

# every symbol include/lumrad.h declares, with (restype, argtypes)
_P = C.c_void_p
_SIGS = {
    "lumrad_create": (C.c_int, [C.POINTER(Settings), C.POINTER(_P)]),
    "lumrad_destroy": (None, [_P]),
    "lumrad_last_error": (C.c_char_p, []),
    "lumrad_synchronize": (C.c_int, [_P]),
    "lumrad_load_world": (C.c_int, [_P, _P]),
    "lumrad_set_world_block": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int16]),
    "lumrad_get_world_block": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int16)]),
    "lumrad_load_block": (C.c_int, [_P, C.c_int16, _P]),
    "lumrad_upload_block_palette": (C.c_int, [_P]),
    "lumrad_load_materials": (C.c_int, [_P, _P]),
    "lumrad_upload_material_palette": (C.c_int, [_P]),
    "lumrad_get_radiance": (C.c_int, [_P, _P]),
    "lumrad_set_radiance": (C.c_int, [_P, _P]),
    "lumrad_build_update_list": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_int)]),
    "lumrad_request_update": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "lumrad_update_radiance": (C.c_int, [_P, C.POINTER(PassParams)]),
    "lumrad_radiance_pass": (C.c_int, [_P, _P, C.c_int, C.POINTER(PassParams)]),
    "lumrad_radiance_pass_i8": (C.c_int, [_P, _P, C.c_int, C.POINTER(PassParams)]),
    "lumrad_upload_requests": (C.c_int, [_P, C.c_int, _P, C.c_int]),
    "lumrad_radiance_pass_resident": (C.c_int, [_P, C.c_int, C.POINTER(PassParams)]),
    "lumrad_radiance_passes": (C.c_int, [_P, _P, _P, C.POINTER(PassParams), C.c_int]),
    "lumrad_radiance_passes_resident": (C.c_int, [_P, _P, C.POINTER(PassParams), C.c_int]),
    "lumrad_get_hits": (C.c_int, [_P, _P, C.c_size_t, C.POINTER(C.c_size_t)]),
    "lumrad_get_pass_stats": (C.c_int, [_P, C.POINTER(PassStats)]),
    "lumrad_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "lumrad_get_kernel_times": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_int)]),
    "lumrad_direction_table": (C.c_int, [C.c_int, _P]),
    "lumrad_load_model": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "lumrad_blockify": (C.c_int, [_P, C.c_int, _P, _P, C.c_int]),
    "lumrad_get_world": (C.c_int, [_P, _P]),
    "lumrad_get_block_palette": (C.c_int, [_P, _P]),
    "lumrad_shift_radiance": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "lumrad_set_radiance_shift": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "lumrad_get_radiance_shift": (C.c_int, [_P, _P]),
    "lumrad_gather_radiance": (C.c_int, [_P, _P, C.c_int, _P]),
    "lumrad_gather_radiance_device": (C.c_int, [_P, _P, C.c_int, _P]),
    "lumrad_radiance_pass_noalloc": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, C.c_int, _P, _P, C.POINTER(PassParams),
                                               _P]),
    "lumrad_radiance_pass_noalloc_status": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "lumrad_test_hook": (C.c_int, [_P, C.c_int, C.c_double]),
    "lumrad_batch_create": (C.c_int, [_P, C.c_int, C.POINTER(_P)]),
    "lumrad_batch_destroy": (None, [_P]),
    "lumrad_batch_set_requests": (C.c_int, [_P, C.c_int, _P, C.c_int, C.POINTER(PassParams)]),
    "lumrad_batch_run": (C.c_int, [_P, C.c_int]),
    "lumrad_batch_run_per_world": (C.c_int, [_P, C.c_int]),
    "lumrad_batch_synchronize": (C.c_int, [_P]),
    "lumrad_batch_last_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "lumrad_batch_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
    "lumrad_batch_autotune": (C.c_int, [_P, C.c_int, C.POINTER(Tuning)]),
    "lumrad_batch_stats": (C.c_int, [_P, C.POINTER(PassStats)]),
    "lumrad_server_create": (C.c_int, [C.POINTER(ServerSettings), C.POINTER(_P)]),
    "lumrad_server_destroy": (None, [_P]),
    "lumrad_server_add_world": (C.c_int, [_P, _P, C.POINTER(C.c_int)]),
    "lumrad_server_submit": (C.c_int, [_P, C.c_int, _P, C.c_int, C.POINTER(PassParams), C.c_double,
                                       C.POINTER(C.c_longlong)]),
    "lumrad_server_progress": (C.c_int, [_P]),
    "lumrad_server_run": (C.c_int, [_P, C.c_double]),
    "lumrad_server_poll": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_int)]),
    "lumrad_server_cancel": (C.c_int, [_P, C.c_longlong, C.POINTER(C.c_int)]),
    "lumrad_server_now": (C.c_double, [_P]),
    "lumrad_server_get_radiance": (C.c_int, [_P, C.c_int, _P]),
    "lumrad_server_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "lumrad_dirty_probes": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, C.POINTER(C.c_int)]),
    "lumrad_build_dirty_list": (C.c_int, [_P, _P, C.c_int, C.c_int, _P, C.c_int, C.POINTER(C.c_int)]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads liblumrad.so (building it first if it is absent); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"liblumrad.so not built: {path}")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class LumRadError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lumrad error {code}: {msg}")
        self.code = code


def check(rc: int) -> None:
    if rc != LUMRAD_OK:
        raise LumRadError(rc, load().lumrad_last_error().decode(errors="replace"))


def ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data
