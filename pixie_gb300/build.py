"""Builds the in-tree CUDA library pixie_gb300/libpxg.so for sm_103a.

Each translation unit compiles in parallel with nvcc (or g++ for the host
geometry); float code uses -fmad=false / -ffp-contract=off so float32
expressions keep the reference's operation order.  Usage:
    python -m pixie_gb300.build
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpxg.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["raster.cu", "composite.cu", "filters.cu", "tcblur.cu", "ringblur.cu", "smallblur.cu", "smooth.cu", "paint.cu", "stroke.cu", "abi.cu", "noalloc.cu"]
HOST_UNITS = ["host_geom.cpp"]


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "pxg.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(src), _headers_mtime()):
        return obj
    if unit.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
               "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-I/usr/local/cuda/include", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = CUDA_UNITS + HOST_UNITS
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(_compile, units))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
