"""Frames in bands (ArtfCudaTraceOptions.bandRays, after vulkan.c:1729-1756): a frame of more rays than
the band allows goes out as launches of whole tile rows, each waited for.  Every pixel's rays are traced
within one band, so the frame is the same bits as one launch, in every precision."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from artful_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _trace(lib, ctx, torch, frame, frame64, precision, jitter, band_rays, ends=False):
    w, h = frame.size[0], frame.size[1]
    hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    rays = jitter if jitter else frame.size[2] ** 2
    e = torch.empty((w * h * rays * 32,), dtype=torch.uint8, device="cuda") if ends else None
    opts = capi.TraceOptions(precision, jitter, 1, 1.0, 0.0, 0, 0, 1, 0, 0, 0, band_rays)
    stats = capi.TraceStats()
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, None, C.byref(opts),
                                     hdr.data_ptr(), e.data_ptr() if ends else None, C.byref(stats)))
    return hdr.cpu().numpy(), (e.cpu().numpy() if ends else None), stats


@pytest.fixture(scope="module")
def c2(lib, ctx):
    scene = scenes.config2(4)
    frame, frame64, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    fluid = scenes.unit_fluid()
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 0))
    return scene


@pytest.mark.parametrize("precision", [capi.EXACT, capi.FP32, capi.FP64, capi.MIXED])
def test_bands_give_the_same_frame(lib, ctx, c2, precision):
    """1080p, 4 rays a pixel (8.3e6 rays) in bands of at most 1e6 rays: 32 tile rows (30,720 rays each) a
    band, 9 bands."""
    import torch
    frame, frame64, _ = scenes.frame(c2)
    whole, ends_whole, s1 = _trace(lib, ctx, torch, frame, frame64, precision, 4, -1, ends=precision == capi.MIXED)
    banded, ends_banded, s2 = _trace(lib, ctx, torch, frame, frame64, precision, 4, 1_000_000,
                                     ends=precision == capi.MIXED)
    assert s1.bands == 1 and s2.bands == 9
    assert s1.rays == s2.rays == 1920 * 1080 * 4 and s1.steps == s2.steps
    np.testing.assert_array_equal(whole.view(np.uint32), banded.view(np.uint32))
    if ends_whole is not None:
        np.testing.assert_array_equal(ends_whole, ends_banded)


def test_the_reference_threshold(lib, ctx, c2):
    """By default a frame goes out in bands above 6.4e7 rays, 8e6 a band: 3840 x 2160 x 8 rays (6.6e7) in
    9 bands of 65 tile rows; 1080p x 4 in one."""
    import torch
    d = c2.desc
    big = scenes.Scene("big", d, c2.camera, 3840, 2160, seed=c2.seed, jitter=8)
    frame, frame64, _ = scenes.frame(big)
    default, _, s1 = _trace(lib, ctx, torch, frame, frame64, capi.FP32, 8, 0)
    whole, _, s2 = _trace(lib, ctx, torch, frame, frame64, capi.FP32, 8, -1)
    assert s1.bands == 9 and s2.bands == 1
    np.testing.assert_array_equal(default.view(np.uint32), whole.view(np.uint32))
    frame, frame64, _ = scenes.frame(c2)
    _, _, s3 = _trace(lib, ctx, torch, frame, frame64, capi.FP32, 4, 0)
    assert s3.bands == 1


def test_bands_of_an_odd_frame(lib, ctx, c2):
    """101 x 67 (17 tile rows, the last of 3 rows) in bands of one tile row, mixed precision with ray
    planes, against one launch."""
    import torch
    odd = scenes.Scene("odd", c2.desc, c2.camera, 101, 67, seed=c2.seed, jitter=4)
    frame, frame64, _ = scenes.frame(odd)
    whole, _, s1 = _trace(lib, ctx, torch, frame, frame64, capi.MIXED, 4, -1)
    banded, _, s2 = _trace(lib, ctx, torch, frame, frame64, capi.MIXED, 4, 101 * 4 * 4)
    assert s2.bands == 17
    np.testing.assert_array_equal(whole.view(np.uint32), banded.view(np.uint32))


def test_heavy_first_frames_are_the_same_bits(lib, ctx, c2):
    """1080p, 4 rays a pixel, mixed: heavy tiles first (the default) against pixel order, whole and in
    bands: the frame and every ray's end the same bytes."""
    import torch
    frame, frame64, _ = scenes.frame(c2)
    w, h = frame.size[0], frame.size[1]
    got = []
    for order, band in ((capi.ORDER_PIXELS, -1), (capi.ORDER_HEAVY_FIRST, -1), (capi.ORDER_HEAVY_FIRST, 2_000_000)):
        hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        e = torch.empty((w * h * 4 * 32,), dtype=torch.uint8, device="cuda")
        opts = capi.TraceOptions(capi.MIXED, 4, 1, 1.0, 0.0, 0, 0, 1, 0, 0, 0, band, order)
        stats = capi.TraceStats()  # (given: the call waits for its stream)
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, None, C.byref(opts),
                                         hdr.data_ptr(), e.data_ptr(), C.byref(stats)))
        got.append((hdr.cpu().numpy().view(np.uint32), e.cpu().numpy()))
    for hdr, e in got[1:]:
        np.testing.assert_array_equal(hdr, got[0][0])
        np.testing.assert_array_equal(e, got[0][1])
