"""Shared fixtures.  `-m gpu` tests run the CUDA library on a GB300; the others need no GPU.

The product library and the oracle are built on first use when missing (the build is in-tree and
quick); a test that needs the reference itself (oracle/_ref) skips where it was not built.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and runs the CUDA library on it")


@pytest.fixture(scope="session")
def lib():
    from artful_gb300 import build, capi
    if not os.path.exists(capi.LIB_PATH):
        build.build()
    return capi.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import binding
    binding.build_oracle()
    return binding.oracle()


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden.npz")))
    return meta, arrays


@pytest.fixture(scope="session")
def ctx(lib):
    import ctypes as C
    from artful_gb300 import capi
    handle = C.c_void_p()
    status = lib.artfCudaCreate(0, C.byref(handle))
    if status != 0:
        pytest.fail(f"artfCudaCreate failed on this GPU: {lib.artfCudaLastError().decode()}")
    yield handle
    lib.artfCudaDestroy(handle)
