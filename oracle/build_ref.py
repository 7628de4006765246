"""Compiles the reference shader, shaders/radiance.comp, as C++ — TEST INFRASTRUCTURE.

The reference's GPU path is a Vulkan compute shader; no graphics stack exists here, so instead
its own GLSL source (read where it lies, in the reference tree) is compiled on the CPU with g++
against oracle/glsl_shim.hpp.  The function bodies are compiled verbatim.  Only GLSL syntax that
C++ cannot express is rewritten, each rewrite matched exactly and checked by count, so a change
in the shader fails the build instead of silently drifting:

  R1  drop `#version`, `#extension` and `precision` lines; inline the two `#include`s;
  R2  the descriptor bindings (radiance.comp:16-25) become shim resources the harness binds;
  R3  the specialization and push constants (:27-35) become mutable globals of the same names
      (the int constant typed so that `%` on it keeps GLSL's OpSMod semantics);
  R4  `in T x` / `out T x` parameters become `T x` / `T& x`;
  R5  `#define RAYS_PER_PROBE (64)` takes the compile-time value LUMREF_R (built for 32..256);
  R6  `float max_dist = 16.0*8.0;` (the shader's TODO quality setting) reads a global;
  R7  `const ivec3 world_size` (consts.glsl:1) becomes a mutable global set per world;
  R8  the workgroup-size declaration is dropped and `void main()` is renamed `shader_main()`.

Outputs go to oracle/_ref/ (git-ignored): the generated source and one shared library per R.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference tree: $LUM_REFERENCE, else a checkout named `reference` beside this repository
# (absent on machines that only build from the generated source, see available())
REFERENCE = os.environ.get("LUM_REFERENCE") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.realpath(HERE))), "reference")
SHADER = os.path.join(REFERENCE, "shaders", "radiance.comp")
CONSTS = os.path.join(REFERENCE, "shaders", "common", "consts.glsl")
RAYS = (32, 64, 128, 256)
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-fsingle-precision-constant", "-ffp-contract=off",
            "-fno-fast-math", "-w"]


def reference_present() -> bool:
    return os.path.exists(SHADER) and os.path.exists(CONSTS)


def _sub(pattern, repl, text, count, flags=0):
    new, n = re.subn(pattern, repl, text, flags=flags)
    if n != count:
        raise RuntimeError(f"shader adaptation: expected {count} match(es) of {pattern!r}, found {n}")
    return new


def _keep_lines(repl_fn):
    """Wraps a replacement so the replaced text keeps its line count (stable #line mapping)."""
    def f(m):
        out = repl_fn(m)
        return out + "\n" * (m.group(0).count("\n") - out.count("\n"))
    return f


def adapt(shader: str, consts: str) -> str:
    # R7
    consts = _sub(r"^const ivec3 world_size\s*=", "ivec3 world_size =", consts, 1, re.M)
    s = shader
    # R1
    s = _sub(r"^#version[^\n]*$", "", s, 1, re.M)
    s = _sub(r"^precision highp (int|float);$", "", s, 2, re.M)
    s = _sub(r"^#extension[^\n]*$", "", s, 1, re.M)
    s = _sub(r'^#include "common\\ext\.glsl"$', "", s, 1, re.M)
    s = _sub(r'^#include "common\\consts\.glsl"$', lambda m: consts.replace("\n", " "), s, 1, re.M)
    # R2: samplers and the storage image
    s = _sub(r"layout\(set = 0, binding = \d(?:, rgb10_a2)?\) uniform (?:writeonly )?(\w+) (\w+);",
             r"\1 \2;", s, 5)
    # R2: the request buffer (a runtime-sized array becomes a pointer)
    s = _sub(r"layout\(std430,set = 0, binding = 5\) restrict readonly buffer (\w+)\{\s*(\w+) (\w+)\[\];\s*\} (\w+);",
             _keep_lines(lambda m: f"struct {m.group(1)} {{ const {m.group(2)}* {m.group(3)}; }} {m.group(4)};"),
             s, 1)
    # R3 (an int constant gets the shim's glsl_int type: `%` on it is OpSMod, as in SPIR-V)
    s = _sub(r"layout\(constant_id = \d\) const int (\w+) = ([^;]+);", r"glsl_int \1 = \2;", s, 1)
    s = _sub(r"layout\(constant_id = \d\) const float (\w+) = ([^;]+);", r"float \1 = \2;", s, 1)
    s = _sub(r"layout\(push_constant\) uniform restrict readonly (\w+)\{([^}]*)\} (\w+);",
             _keep_lines(lambda m: f"struct {m.group(1)} {{{' '.join(m.group(2).split())}}} {m.group(3)};"), s, 1)
    # R4
    s = _sub(r"\bout (\w+) (\w+)(?=\s*[,)])", r"\1& \2", s, 7)
    s = _sub(r"\bin (\w+) (\w+)(?=\s*[,)])", r"\1 \2", s, 7)
    # R5, R6
    s = _sub(r"^#define RAYS_PER_PROBE \(64\)", "#define RAYS_PER_PROBE (LUMREF_R)", s, 1, re.M)
    s = _sub(r"float max_dist = 16\.0\*8\.0;", "float max_dist = lumref_max_dist;", s, 1)
    # R8
    s = _sub(r"^layout\(local_size_x = RAYS_PER_PROBE[^\n]*\) in;$", "", s, 1, re.M)
    s = _sub(r"^void main\(\)\{", "void shader_main(){", s, 1, re.M)
    return s


def generate() -> str:
    shader = open(SHADER).read()
    consts = open(CONSTS).read()
    body = adapt(shader, consts)
    shim = os.path.join(HERE, "glsl_shim.hpp")
    harness = os.path.join(HERE, "ref_harness.inc")
    src = (f'#include "{shim}"\n'
           "#define shared\n"
           "namespace lumref {\n"
           "float lumref_max_dist = 128.0;\n"
           f'#line 1 "{SHADER}"\n'
           f"{body}\n"
           f'#include "{harness}"\n'
           "}  // namespace lumref\n")
    os.makedirs(OUT, exist_ok=True)
    path = os.path.join(OUT, "radiance_ref.cpp")
    with open(path, "w") as f:
        f.write(src)
    return path


def lib_path(rays: int) -> str:
    return os.path.join(OUT, f"libradiance_ref_r{rays}.so")


def generated_source() -> str:
    return os.path.join(OUT, "radiance_ref.cpp")


def available() -> bool:
    """The reference shader can be built here: from its sources, or from the C++ generated from
    them (which travels with the repository's build outputs to machines without the sources)."""
    return reference_present() or os.path.exists(generated_source())


def build(rays=RAYS) -> list[str]:
    if reference_present():
        src = generate()
    elif os.path.exists(generated_source()):
        src = generated_source()
    else:
        raise RuntimeError(f"reference shader not found at {SHADER} and no generated source")

    def one(r):
        tmp = lib_path(r) + ".tmp"
        res = subprocess.run(["g++", *CXXFLAGS, f"-DLUMREF_R={r}", src, "-o", tmp], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"reference shader build failed (R={r}):\n{res.stderr[-4000:]}")
        os.replace(tmp, lib_path(r))
        return lib_path(r)

    with ThreadPoolExecutor(max_workers=len(rays)) as ex:
        return list(ex.map(one, rays))


class RefWorld(C.Structure):
    _fields_ = [("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int), ("grid", C.c_void_p),
                ("palette", C.c_void_p), ("n_slots", C.c_int), ("materials", C.c_void_p)]


_libs: dict[int, C.CDLL] = {}


def load(rays: int) -> C.CDLL:
    if rays not in _libs:
        path = lib_path(rays)
        if not os.path.exists(path):
            raise RuntimeError(f"reference shader library not built: {path}")
        lib = C.CDLL(path)
        P = C.c_void_p
        lib.lumref_pass.argtypes = [P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, P, P, P, P,
                                    C.c_int, C.c_int]
        lib.lumref_set_unorm10.argtypes = [C.c_int]
        lib.lumref_set_unorm10.restype = None
        _libs[rays] = lib
    return _libs[rays]


def run_pass(world, requests_i8: np.ndarray, rays: int = 64, max_dist: float = 128.0, blend: float = 0.01,
             time_seed: int = 0, size: int = 1, shift: int = 0, prev: np.ndarray | None = None,
             unorm10: bool = False):
    """One dispatch of the reference shader.  Returns (next, ray_light, ray_info, abandoned).
    unorm10: the written volume takes the rgb10_a2 image's 10-bit codes (prev must hold such
    values already)."""
    lib = load(rays)
    lib.lumref_set_unorm10(1 if unorm10 else 0)
    grid = np.ascontiguousarray(world.grid, dtype=np.int16)
    pal = np.ascontiguousarray(world.palette, dtype=np.uint8)
    mats = np.ascontiguousarray(world.materials, dtype=np.float32)
    Z, Y, X = grid.shape
    w = RefWorld(X, Y, Z, grid.ctypes.data, pal.ctypes.data, pal.shape[0], mats.ctypes.data)
    if prev is None:
        prev = np.zeros((Z, Y, X, 3), dtype=np.float32)
    prev = np.ascontiguousarray(prev, dtype=np.float32)
    nxt = prev.copy()
    req = np.ascontiguousarray(requests_i8, dtype=np.int8)
    groups = req.shape[0] // size
    light = np.zeros((groups * rays, 3), dtype=np.float32)
    info = np.zeros((groups * rays, 7), dtype=np.int32)
    abandoned = lib.lumref_pass(C.byref(w), req.ctypes.data if req.size else None, req.shape[0], time_seed, size,
                                shift, max_dist, blend, prev.ctypes.data, nxt.ctypes.data, light.ctypes.data,
                                info.ctypes.data, 0, groups)
    return nxt, light, info, abandoned


if __name__ == "__main__":
    print(build())
