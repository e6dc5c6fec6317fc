"""Builds libartful_cuda.so in-tree: the C11 host set-up with gcc, the CUDA kernels and the C ABI with
nvcc for sm_103a only.  Each kernel translation unit carries the float flags that define its rounding.
With debug=True it builds libartful_cuda_debug.so instead: the same sources with ARTF_CUDA_DEBUG_BOUNDS,
every table read and frame write checked against its region (lensCore.cuh), the first index outside
reported by the C ABI as ARTF_CUDA_EBOUNDS.

    python -m artful_gb300.build [--verbose] [--debug]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libartful_cuda.so")
DEBUG_OBJ = os.path.join(HERE, "_build_debug")
DEBUG_LIB = os.path.join(HERE, "libartful_cuda_debug.so")
DEBUG = ["-DARTF_CUDA_DEBUG_BOUNDS"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I" + INCLUDE, "-I" + CSRC]
# How float rounds in each kernel unit.
EXACT = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
FAST = ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
UNITS = {
    "abi.cu": [],
    "lensExact.cu": EXACT,
    "lensFast.cu": FAST,
    "lensFp64.cu": [],
    "lensMixed.cu": FAST,
    "probe.cu": ["-fmad=true"],
    "noAlloc.cu": [],
    "post.cu": EXACT,
    "lensTangent.cu": [],
    "lensAdjoint.cu": FAST,
    "fluid.cu": EXACT,
    "disc.cu": EXACT,
}
C_UNITS = ["holeHost.c", "synthScene.c", "renderer.c"]
CFLAGS = ["-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wextra", "-I" + INCLUDE]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_info: bool = False, debug: bool = False) -> str:
    obj, lib = (DEBUG_OBJ, DEBUG_LIB) if debug else (OBJ, LIB)
    os.makedirs(obj, exist_ok=True)
    jobs = []
    for name, flags in UNITS.items():
        out = os.path.join(obj, name + ".o")
        extra = (["-Xptxas", "-v"] if ptxas_info else []) + (DEBUG if debug else [])
        jobs.append([nvcc()] + NVCC_COMMON + flags + extra + ["-c", os.path.join(CSRC, name), "-o", out])
    for name in C_UNITS:
        out = os.path.join(obj, name + ".o")
        jobs.append([os.environ.get("CC", "gcc")] + CFLAGS + ["-c", os.path.join(CSRC, name), "-o", out])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as pool:
        logs = list(pool.map(lambda c: _run(c, verbose), jobs))
    if ptxas_info:
        for log in logs:
            print(log)
    objs = [j[-1] for j in jobs]
    _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lpthread"], verbose)
    return lib


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas" in sys.argv, debug="--debug" in sys.argv))
