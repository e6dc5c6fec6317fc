"""The allocation-free batch entry point (artfCudaHoleBatchNoAlloc), on a GB300 through the C ABI.

It exists for callers that cannot call cudaMalloc: an engine that owns all device memory through its own
allocator, or a render thread that must not stall on an allocation.  Its scratch (view table and queue
counters) is one fixed array per device, so it holds at most 64 views a call.  This file is collected
last, so that a run stopping at its first failure has already run every other test; it also passes alone
in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from artful_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _views(lib, count):
    import torch
    views, keep = [], []
    for scene in scenes.config3_views(count, seed=5):
        scene.width = max(8, scene.width // 4) | 1
        scene.height = max(4, scene.height // 4)
        frame, frame64, clamped = scenes.frame(scene)
        m = torch.from_numpy(scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)).cuda()
        fluid = torch.from_numpy(scenes.unit_fluid()).cuda()
        hdr = torch.zeros((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
        views.append(capi.View(frame, frame64, m.data_ptr(), fluid.data_ptr(), hdr.data_ptr(), None))
        keep.append((m, fluid, hdr))
    return (capi.View * count)(*views), keep


def _within_tolerance(got, want):
    """The tolerance of the parity tests: pixel classes agree and radiance within 1e-3 relative."""
    classes = np.mean(got[..., 3] == want[..., 3])
    lum, ref = got[..., :3].astype(np.float64).sum(-1), want[..., :3].astype(np.float64).sum(-1)
    rel = np.abs(lum - ref) / np.maximum(np.abs(ref), 1e-3)
    return classes >= 0.999 and np.mean(rel <= 1e-3) >= 0.999


def test_no_alloc_batch_matches_the_context_batch_twice_in_a_row(lib, ctx):
    import torch
    views, keep = _views(lib, 5)
    opts = capi.TraceOptions(capi.MIXED, 0, 0, 1.0, 0.0, 0, 0, 1)
    want_stats = capi.TraceStats()
    capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(opts), C.byref(want_stats)))
    torch.cuda.synchronize()
    want = [hdr.cpu().numpy().copy() for _, _, hdr in keep]
    for call in range(2):
        for _, _, hdr in keep:
            hdr.zero_()
        torch.cuda.synchronize()
        stats = capi.TraceStats()
        capi.check(lib.artfCudaHoleBatchNoAlloc(views, len(views), C.byref(opts), None, C.byref(stats)))
        torch.cuda.synchronize()
        for i, (_, _, hdr) in enumerate(keep):
            assert _within_tolerance(hdr.cpu().numpy(), want[i]), (call, i)
        # the counters start from zero on every call
        assert stats.rays == want_stats.rays and stats.steps == want_stats.steps, call


def test_no_alloc_batch_refuses_what_it_cannot_hold(lib):
    views, keep = _views(lib, 1)
    opts = capi.TraceOptions(capi.MIXED, 0, 0, 1.0, 0.0, 0, 0, 1)
    many = (capi.View * (capi.NOALLOC_MAX_VIEWS + 1))(*([views[0]] * (capi.NOALLOC_MAX_VIEWS + 1)))
    assert lib.artfCudaHoleBatchNoAlloc(many, len(many), C.byref(opts), None, None) == -1
    assert b"64 views" in lib.artfCudaLastError()
    no_map = (capi.View * 1)(capi.View(views[0].frame, views[0].frame64, None, views[0].fluid, views[0].hdr, None))
    assert lib.artfCudaHoleBatchNoAlloc(no_map, 1, C.byref(opts), None, None) == -1


def test_no_alloc_batch_on_a_caller_stream_and_refused_in_a_capture(lib, ctx):
    """On the caller's own stream the batch is the context batch's; on a stream being captured it is
    refused (its host staging would be replayed stale), and the capture ends cleanly."""
    import torch
    views, keep = _views(lib, 3)
    opts = capi.TraceOptions(capi.MIXED, 0, 0, 1.0, 0.0, 0, 0, 1)
    capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(opts), None))
    torch.cuda.synchronize()
    want = [hdr.cpu().numpy().copy() for _, _, hdr in keep]
    stream = torch.cuda.Stream()
    for _, _, hdr in keep:
        hdr.zero_()
    torch.cuda.synchronize()
    capi.check(lib.artfCudaHoleBatchNoAlloc(views, len(views), C.byref(opts), C.c_void_p(stream.cuda_stream), None))
    stream.synchronize()
    for i, (_, _, hdr) in enumerate(keep):
        assert _within_tolerance(hdr.cpu().numpy(), want[i]), i
    graph = torch.cuda.CUDAGraph()
    status = None
    with torch.cuda.graph(graph, stream=stream):
        keep[0][2].add_(0.0)  # (the capture holds one plain op)
        status = lib.artfCudaHoleBatchNoAlloc(views, len(views), C.byref(opts), C.c_void_p(stream.cuda_stream), None)
    assert status == -1
    assert b"captured" in lib.artfCudaLastError()
    torch.cuda.synchronize()
