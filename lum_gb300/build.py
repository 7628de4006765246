"""Builds liblumrad.so (the C ABI of include/lumrad.h) for sm_103a, in-tree.

nvcc compiles every translation unit in parallel into lum_gb300/_build/ and links one shared
library with the CUDA runtime linked statically, so the library loads without torch.
Device code is built with -fmad=false and host code with -ffp-contract=off: no FMA contraction
anywhere, which the bit-exact hit records depend on.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblumrad.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I", INCLUDE,
          "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math"]
DEVICE = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]

SOURCES = ["radiance_pass.cu", "radiance_aux.cu", "radiance_serve.cu", "lumrad_host.cpp", "lumrad_batch.cpp",
           "lumrad_serve.cpp", "lumrad_blockify.cpp"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc(), *ARCH, *COMMON, *DEVICE, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd))
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles and links liblumrad.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra if s.endswith(".cu") else [], verbose or ptxas_info),
                           SOURCES))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
