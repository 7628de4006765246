"""The C ABI library without a GPU: it loads, exports every symbol include/lumrad.h declares,
and rejects bad arguments before touching a device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import lum_gb300
from lum_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "lumrad.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lumrad_\w+)\s*\(", src)))


def test_library_loads_and_exports_every_declared_symbol():
    lib = lum_gb300.load()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_native._SIGS), "binding lacks a signature for a declared symbol"


def test_binding_constants_match_header():
    """Every LUMRAD_ status code, test hook and limit the binding copies equals the header's."""
    src = open(os.path.join(ROOT, "include", "lumrad.h")).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(LUMRAD_\w+)\s+\(?(-?\d+)\)?", src)}
    enums = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LUMRAD_\w+)\s*=\s*(-?\d+)", src)}
    header = {**enums, **defines}
    copied = {k: v for k, v in vars(_native).items() if k.startswith("LUMRAD_") and isinstance(v, int)}
    assert "LUMRAD_MAX_CHUNK" in copied and "LUMRAD_OK" in copied
    for k, v in copied.items():
        assert k in header, k
        assert header[k] == v, (k, header[k], v)


def test_struct_sizes_match_header():
    assert C.sizeof(_native.Settings) == 24
    assert C.sizeof(_native.Material) == 24
    assert C.sizeof(_native.PassParams) == 28
    assert _native.HIT_DTYPE.itemsize == 24


def test_create_rejects_bad_settings_without_gpu():
    lib = lum_gb300.load()
    h = C.c_void_p()
    for ws, slots, prec in [((0, 4, 4), 8, 0), ((4, 4, 4), 0, 0), ((4, 4, 4), 5000, 0), ((4, 4, 4), 8, 7),
                            ((2048, 4, 4), 8, 0)]:
        s = _native.Settings((C.c_int * 3)(*ws), slots, prec, 0)
        rc = lib.lumrad_create(C.byref(s), C.byref(h))
        assert rc == _native.LUMRAD_EINVAL, (ws, slots, prec, rc)
        assert lib.lumrad_last_error()


def test_null_arguments_are_errors_not_crashes():
    lib = lum_gb300.load()
    assert lib.lumrad_create(None, None) == _native.LUMRAD_EINVAL
    assert lib.lumrad_load_world(None, None) == _native.LUMRAD_EINVAL
    assert lib.lumrad_radiance_pass(None, None, 0, None) == _native.LUMRAD_EINVAL
    assert lib.lumrad_get_hits(None, None, 0, None) == _native.LUMRAD_EINVAL
    assert lib.lumrad_direction_table(0, None) == _native.LUMRAD_EINVAL
    lib.lumrad_destroy(None)


def test_create_without_gpu_reports_device_error():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    with pytest.raises(lum_gb300.LumRadError) as e:
        lum_gb300.RadianceWorld((4, 4, 4))
    assert e.value.code == _native.LUMRAD_EDEVICE


def test_ctypes_layouts_match_the_header(tmp_path):
    """Every struct the binding mirrors has the header's size and field offsets: a C program built
    against include/lumrad.h prints them (gcc), the ctypes classes must agree."""
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"LumRadSettings": _native.Settings, "LumRadMaterial": _native.Material,
             "LumRadPassParams": _native.PassParams, "LumRadMeshTransform": _native.MeshTransform,
             "LumRadPassStats": _native.PassStats, "LumRadTuning": _native.Tuning,
             "LumRadServerSettings": _native.ServerSettings, "LumRadServerStats": _native.ServerStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lumrad.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append(f'  printf("{cname} .sizeof %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            name, field, value = line.split()
            got[(name, field)] = int(value)
    for cname, cls in pairs.items():
        assert got[(cname, ".sizeof")] == C.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])


def test_packed_lists_are_checked_before_any_call():
    """radiance_passes_packed rejects a non-int16 or non-(n, 4) array and counts that do not add up
    to its rows, before it reaches the library (no GPU needed)."""
    rw = lum_gb300.RadianceWorld.__new__(lum_gb300.RadianceWorld)

    class NoCall:
        def lumrad_radiance_passes(self, *a):
            raise AssertionError("the library must not be called")

    rw.lib = NoCall()
    rw.h = None
    p = [lum_gb300.pass_params(rays=64)] * 2
    good = np.zeros((5, 4), np.int16)
    with pytest.raises(ValueError):
        rw.radiance_passes_packed(good.astype(np.int32), [2, 3], p)
    with pytest.raises(ValueError):
        rw.radiance_passes_packed(np.zeros((5, 3), np.int16), [2, 3], p)
    with pytest.raises(ValueError):
        rw.radiance_passes_packed(good, [2, 2], p)
    with pytest.raises(ValueError):
        rw.radiance_passes_packed(good, [6, -1], p)
