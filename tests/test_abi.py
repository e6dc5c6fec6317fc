"""The C ABI library loads and exports every entry point its headers declare; its argument checks work
without a GPU."""
import ctypes as C
import os
import re

import pytest

from artful_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for header in os.listdir(os.path.join(ROOT, "include")):
        if not header.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", header)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(artf\w+)\s*\([^;{]*\)\s*;", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_the_header(lib):
    assert set(capi.SIGNATURES) >= set(n for n in declared_functions() if n.startswith("artfCuda")), \
        set(declared_functions()) - set(capi.SIGNATURES)


def test_struct_sizes_match_the_reference_layouts():
    assert C.sizeof(capi.HoleFrame) == 368      # src/scene/sceneInternal.h:302-319
    assert C.sizeof(capi.BlackHoleDesc) == 92   # include/artful/scene.h:470-490
    assert C.sizeof(capi.Camera) == 44          # include/artful/scene.h:314-320
    assert capi.MAP_FLOATS == 2887424            # sceneInternal.h:329


def test_argument_errors_without_a_device(lib):
    assert lib.artfCudaCreate(0, None) == -1
    assert lib.artfCudaSetMap(None, None, 0) == -1
    assert lib.artfCudaHoleTrace(None, None, None, None, None, None, None, None, None) == -1
    assert b"context" in lib.artfCudaLastError()
    assert lib.artfCudaFrameRead(None, None, None) == -1
    assert b"context" in lib.artfCudaLastError()


def test_create_reports_no_device_here(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert lib.artfCudaCreate(0, C.byref(h)) == -2
    assert not h.value


def test_enumerations_match_the_headers():
    """The Python constants the harness passes are the values the headers give."""
    text = ""
    for header in ("artful_cuda.h", "artful_cuda_renderer.h"):
        text += open(os.path.join(ROOT, "include", header)).read()

    def value(name):
        m = re.search(r"\b" + name + r"\s*=\s*(\d+)", text)
        assert m, name
        return int(m.group(1))

    assert capi.BACKEND == value("ARTF_CUDA_BACKEND")
    assert (capi.EXACT, capi.FP32, capi.FP64, capi.MIXED) == tuple(
        value(n) for n in ("ARTF_CUDA_EXACT", "ARTF_CUDA_FP32", "ARTF_CUDA_FP64", "ARTF_CUDA_MIXED"))
    assert (capi.ORDER_HEAVY_FIRST, capi.ORDER_PIXELS) == (value("ARTF_CUDA_ORDER_HEAVY_FIRST"),
                                                           value("ARTF_CUDA_ORDER_PIXELS"))
