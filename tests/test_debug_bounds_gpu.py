"""The bounds-checked debug build (artful_gb300/libartful_cuda_debug.so, built with ARTF_CUDA_DEBUG_BOUNDS):
every table row or entry the shading reads is checked against its own region of the map or fluid, and
every frame, ray-plane and ray-end write against its buffer; the first index outside is reported by the
C ABI as ARTF_CUDA_EBOUNDS, with no fault: the read stays inside the buffer, as in the release build,
and the write is skipped.

A clean view reports nothing and keeps the release build's bits (the reference's odd sizes, 1 x 1, 3 x 2
and 101 x 67, in the exact and the mixed precision).  A host-made frame the clamps do not cover, a
Doppler factor of 6 (the reference does not clamp it), shifts a receding crossing's colour below zero:
its colour index then falls before the colour table, inside the map, where the release build reads the
ring table as the reference would, and the debug build says so."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from tests import gpu_helpers as g

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dlib():
    from artful_gb300 import build
    if not os.path.exists(capi.DEBUG_LIB_PATH):
        build.build(debug=True)
    return capi.load(capi.DEBUG_LIB_PATH)


@pytest.fixture(scope="module")
def dctx(dlib):
    handle = C.c_void_p()
    capi.check(dlib.artfCudaCreate(0, C.byref(handle)), dlib)
    yield handle
    dlib.artfCudaDestroy(handle)


def _inputs(lib, name):
    scene = scenes.golden_scenes()[name]
    frame, frame64, clamped = scenes.frame(scene)
    return frame, frame64, scenes.synth_map(lib, clamped, scene.seed, scene.emissivity), scenes.unit_fluid()


def _trace(lib, ctx, frame, frame64, precision):
    import torch
    w, h = frame.size[0], frame.size[1]
    hdr = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    opts = capi.TraceOptions(precision, 0, 0, 1.0, 0.0, 0, 0, 1)
    status = lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64) if frame64 is not None else None, None,
                                   None, C.byref(opts), hdr.data_ptr(), None, None)
    torch.cuda.synchronize()
    return status, hdr.cpu().numpy()


@pytest.mark.parametrize("precision", [capi.EXACT, capi.MIXED])
@pytest.mark.parametrize("name", ["odd_1x1", "odd_3x2", "odd_101x67"])
def test_clean_views_report_nothing_and_keep_their_bits(lib, ctx, dlib, dctx, name, precision):
    frame, frame64, m, fluid = _inputs(lib, name)
    g.set_inputs(lib, ctx, m, fluid)
    g.set_inputs(dlib, dctx, m, fluid)
    status, got = _trace(dlib, dctx, frame, frame64, precision)
    assert status == 0, dlib.artfCudaLastError()
    status, want = _trace(lib, ctx, frame, frame64, precision)
    assert status == 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_a_colour_outside_its_table_is_reported_not_faulted(lib, ctx, dlib, dctx):
    frame, frame64, m, fluid = _inputs(lib, "c1")
    frame.look[1] = 6.0
    frame64.look[1] = 6.0
    g.set_inputs(lib, ctx, m, fluid)
    g.set_inputs(dlib, dctx, m, fluid)
    status, _ = _trace(lib, ctx, frame, None, capi.EXACT)
    assert status == 0  # the release build reads inside the map, as the reference does
    status, _ = _trace(dlib, dctx, frame, None, capi.EXACT)
    assert status == capi.EBOUNDS
    assert b"colour index" in dlib.artfCudaLastError()
    status, _ = _trace(dlib, dctx, frame, frame64, capi.MIXED)
    assert status == capi.EBOUNDS
    # the word starts clear at every trace: the same context traces a clean frame with no report
    frame.look[1] = frame64.look[1] = 1.0
    status, _ = _trace(dlib, dctx, frame, frame64, capi.MIXED)
    assert status == 0, dlib.artfCudaLastError()
