"""Every entry point that launches work opens a named NVTX range for its whole call and closes it on
every return, errors included.  Checked with NVTX's own injection interface on the CPU: a recorder
library (tests/nvtx/nvtxRecorder.c) loaded through NVTX_INJECTION64_PATH logs the pushes and pops of a
process that calls the entry points with no context (each returns an error status before any CUDA call,
after its range has opened)."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAMES = ["artfCudaHoleTrace", "artfCudaHoleRender", "artfCudaHoleDraw", "artfCudaHoleTraceRays",
         "artfCudaHoleTangents", "artfCudaHoleAdjoint", "artfCudaHoleBatch", "artfCudaBatchGraphCreate",
         "artfCudaBatchGraphLaunch", "artfCudaAutotune", "artfCudaPaintDisc", "artfCudaFluidNew",
         "artfCudaFluidAdvance", "artfCudaFluidStep", "artfCudaPostLaunch", "artfCudaHoleBatchNoAlloc"]

CALLS = """
import sys
sys.path.insert(0, {root!r})
from artful_gb300 import capi
lib = capi.load()
N = None
statuses = [
    lib.artfCudaHoleTrace(N, N, N, N, N, N, N, N, N),
    lib.artfCudaHoleRender(N, N, N, N, 0, N, 0, N, N, N),
    lib.artfCudaHoleDraw(N, N, N, N, 0, N, 0, N, N, N, N),
    lib.artfCudaHoleTraceRays(N, N, N, N, N, 0, 1.0, 0, N, N, N, N, N, N),
    lib.artfCudaHoleTangents(N, N, N, N, N, N, N, N),
    lib.artfCudaHoleAdjoint(N, N, 0, 0, 0, N, N, N, 0, N, N, N, N),
    lib.artfCudaHoleBatch(N, N, 0, N, N),
    lib.artfCudaBatchGraphCreate(N, N, 0, N, N),
    lib.artfCudaBatchGraphLaunch(N, N),
    lib.artfCudaAutotune(N, N, 0, N, N),
    lib.artfCudaPaintDisc(N, N, 0.0, 0.0, 0.0),
    lib.artfCudaFluidNew(N, 0.0, 0.0, 0.0, 0.0, N),
    lib.artfCudaFluidAdvance(N, 0.0, N),
    lib.artfCudaFluidStep(N, 0, 0.0),
    lib.artfCudaPostLaunch(N, N, N, N, N),
    lib.artfCudaHoleBatchNoAlloc(N, 0, N, N, N),
]
assert all(s != 0 for s in statuses), statuses
print("ok")
"""


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "nvtx3", "nvToolsExt.h")) else None


def test_entry_points_open_and_close_their_ranges(lib, tmp_path):
    inc = _cuda_include()
    if inc is None:
        pytest.skip("no NVTX headers")
    recorder = str(tmp_path / "libnvtxRecorder.so")
    subprocess.run(["gcc", "-shared", "-fPIC", "-I" + inc, os.path.join(ROOT, "tests", "nvtx", "nvtxRecorder.c"),
                    "-o", recorder], check=True)
    log = tmp_path / "ranges.log"
    env = dict(os.environ, NVTX_INJECTION64_PATH=recorder, ARTF_NVTX_LOG=str(log))
    run = subprocess.run([sys.executable, "-c", CALLS.format(root=ROOT)], env=env, capture_output=True, text=True,
                         timeout=120)
    assert run.returncode == 0 and "ok" in run.stdout, run.stderr[-2000:]
    lines = log.read_text().splitlines()
    pushed = [x.split(" ", 1)[1] for x in lines if x.startswith("push ")]
    assert pushed == NAMES, pushed
    assert lines == [y for name in NAMES for y in ("push " + name, "pop")]
