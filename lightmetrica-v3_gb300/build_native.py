"""Builds liblmgpu.so (CUDA kernels for sm_103a + host runtime) in-tree.

    python lightmetrica-v3_gb300/build_native.py

Translation units compile in parallel; the library lands in lightmetrica/_lib/ next to the Python
package that loads it. No CMake: nvcc for .cu, the host compiler for .cpp, nvcc to link.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lightmetrica", "_lib")
LIB = os.path.join(LIBDIR, "liblmgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    # --fmad=false: every product and sum rounds as written (explicit fmaf() stays fused), so the
    # same device function gives the same bits in every kernel that inlines it
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math",
    "-I", INCLUDE,
]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-I", INCLUDE]

CU_SOURCES = ["accel.cu", "render.cu", "bvh_gpu.cu"]
# render.cu: single-precision division and square root to about 2 ulp instead of correctly rounded
# (the shading math; 36.6 -> 34.7 ms of shade per headline frame). The triangle test and the
# normalization keep explicitly rounded intrinsics, so hits stay bit-exact; the slab test's
# reciprocals gain at most 2 ulp, inside its 2^-18 widening.
PER_SOURCE_FLAGS = {"render.cu": ["--prec-div=false", "--prec-sqrt=false"]}
CPP_SOURCES = ["bvh_build.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra_nvcc: list[str] | None = None, force: bool = False) -> str:
    """Compiles the stale sources (all of them with force=True, e.g. when extra_nvcc changes)
    and links lightmetrica/_lib/liblmgpu.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    cxx = os.environ.get("CXX", "g++")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "lmgpu.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + PER_SOURCE_FLAGS.get(src, []) + (extra_nvcc or []) + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([cxx] + CXX_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
