"""Batches of uneven views in one persistent launch, their CUDA graphs, the autotuner, and device loss
injected on the host: on a GB300 through the C ABI."""
import ctypes as C

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from tests import gpu_helpers as g

pytestmark = pytest.mark.gpu


def _views(lib, count=6, scale=0.25, rays=1):
    """Views of configuration 3 (seed 2), shrunk so the test stays small, each with its own map, and room
    for the ends of `rays` rays a pixel (the views' own 1 x 1 samples, or a jitter of that many)."""
    import torch
    out, keep = [], []
    for scene in scenes.config3_views(count, seed=2):
        scene.width = max(8, int(scene.width * scale)) | 1  # (odd widths: ragged tiles)
        scene.height = max(4, int(scene.height * scale))
        frame, frame64, clamped = scenes.frame(scene)
        m = torch.from_numpy(scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)).cuda()
        fluid = torch.from_numpy(scenes.unit_fluid()).cuda()
        hdr = torch.zeros((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
        assert scene.desc.samples == 1
        ends = torch.zeros((scene.width * scene.height * rays * 32,), dtype=torch.uint8, device="cuda")
        out.append(capi.View(frame, frame64, m.data_ptr(), fluid.data_ptr(), hdr.data_ptr(), ends.data_ptr()))
        keep.append((scene, m, fluid, hdr, ends))
    return (capi.View * len(out))(*out), keep


def _opts(**kw):
    o = capi.TraceOptions(capi.MIXED, 0, 0, 1.0, 0.0, 0, 0, 1)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def test_batch_equals_each_view_alone(lib, ctx):
    import torch
    views, keep = _views(lib)
    stats = capi.TraceStats()
    capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(_opts()), C.byref(stats)))
    batch = [(hdr.cpu().numpy().copy(), ends.cpu().numpy().copy()) for _, _, _, hdr, ends in keep]
    assert stats.rays == sum(s.width * s.height for s, *_ in keep)
    for i, (scene, m, fluid, hdr, ends) in enumerate(keep):
        hdr.zero_()
        alone = capi.TraceStats()
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(views[i].frame), C.byref(views[i].frame64), m.data_ptr(),
                                         fluid.data_ptr(), C.byref(_opts()), hdr.data_ptr(), ends.data_ptr(),
                                         C.byref(alone)))
        torch.cuda.synchronize()
        assert np.array_equal(hdr.cpu().numpy().view(np.uint32), batch[i][0].view(np.uint32)), i
        assert np.array_equal(ends.cpu().numpy(), batch[i][1]), i


def test_graph_replays_and_updates(lib, ctx):
    import torch
    views, keep = _views(lib, count=4)
    graph = C.c_void_p()
    capi.check(lib.artfCudaBatchGraphCreate(ctx, views, len(views), C.byref(_opts()), C.byref(graph)))
    try:
        capi.check(lib.artfCudaBatchGraphLaunch(graph, None))
        torch.cuda.synchronize()
        first = [hdr.cpu().numpy().copy() for *_, hdr, _ in keep]
        for *_, hdr, _ in keep:
            hdr.zero_()
        stats = capi.TraceStats()
        capi.check(lib.artfCudaBatchGraphLaunch(graph, C.byref(stats)))
        assert all(np.array_equal(a, hdr.cpu().numpy()) for a, (*_, hdr, _) in zip(first, keep))
        assert stats.rays > 0 and stats.ms > 0
        # move every eye a little: the replayed graph traces the new frames
        moved = []
        for i, (scene, *_) in enumerate(keep):
            scene.camera = scenes.camera(60.0 + i, 25.0 + i)
            frame, frame64, _ = scenes.frame(scene)
            moved.append(capi.View(frame, frame64, views[i].map, views[i].fluid, views[i].hdr, views[i].ends))
        moved = (capi.View * len(moved))(*moved)
        capi.check(lib.artfCudaBatchGraphUpdate(graph, moved, len(moved)))
        capi.check(lib.artfCudaBatchGraphLaunch(graph, None))
        torch.cuda.synchronize()
        replayed = [hdr.cpu().numpy().copy() for *_, hdr, _ in keep]
        capi.check(lib.artfCudaHoleBatch(ctx, moved, len(moved), C.byref(_opts()), None))
        torch.cuda.synchronize()
        assert all(np.array_equal(a, hdr.cpu().numpy()) for a, (*_, hdr, _) in zip(replayed, keep))
        assert not all(np.array_equal(a, b) for a, b in zip(first, replayed))
        assert lib.artfCudaBatchGraphUpdate(graph, moved, len(moved) - 1) == -1
    finally:
        lib.artfCudaBatchGraphDestroy(graph)


def test_autotune_picks_a_shape_and_keeps_results(lib, ctx):
    import torch
    views, keep = _views(lib, count=5, scale=0.5)
    capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(_opts()), None))
    torch.cuda.synchronize()
    before = [hdr.cpu().numpy().copy() for *_, hdr, _ in keep]
    t = capi.Tuning()
    capi.check(lib.artfCudaAutotune(ctx, views, len(views), C.byref(_opts()), C.byref(t)))
    assert t.blockSize in (64, 128, 192, 256) and t.compactEvery >= 16 and 16 <= t.fp64Batch <= 32
    assert 0 < t.ms <= t.defaultMs * 1.05 and t.trials > 10
    # the tuned shape changes when the work runs, never the result
    capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(_opts()), None))
    torch.cuda.synchronize()
    assert all(np.array_equal(a, hdr.cpu().numpy()) for a, (*_, hdr, _) in zip(before, keep))


def test_batch_rejects_bad_requests(lib, ctx):
    views, keep = _views(lib, count=2)
    assert lib.artfCudaHoleBatch(ctx, views, 0, C.byref(_opts()), None) == -1
    assert lib.artfCudaHoleBatch(ctx, views, 2, C.byref(_opts(precision=capi.EXACT)), None) == -1
    bad = (capi.View * 1)(capi.View(views[0].frame, views[0].frame64, views[0].map, views[0].fluid, None, None))
    assert lib.artfCudaHoleBatch(ctx, bad, 1, C.byref(_opts()), None) == -1
    assert b"hdr" in lib.artfCudaLastError()


def test_device_loss_injected_on_the_host(lib):
    """The reference's contract (renderer.h:107-109): after a device loss every call fails and the
    context must be replaced; a new one works.  The loss is made on the host: no GPU fault."""
    import torch
    scene = scenes.golden_scenes()["odd_3x2"]
    frame, frame64, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    hdr = torch.empty((2, 3, 4), device="cuda")
    for attempt in range(2):
        handle = C.c_void_p()
        capi.check(lib.artfCudaCreate(0, C.byref(handle)))
        try:
            g.set_inputs(lib, handle, m, scenes.unit_fluid())
            opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 0)
            if attempt == 0:
                capi.check(lib.artfCudaFailAfter(handle, 1))
                assert lib.artfCudaHoleTrace(handle, C.byref(frame), None, None, None, C.byref(opts),
                                             hdr.data_ptr(), None, None) == 0
                assert lib.artfCudaHoleTrace(handle, C.byref(frame), None, None, None, C.byref(opts),
                                             hdr.data_ptr(), None, None) == -6
                assert lib.artfCudaSetMap(handle, m.ctypes.data, 0) == -6
            else:
                assert lib.artfCudaHoleTrace(handle, C.byref(frame), None, None, None, C.byref(opts),
                                             hdr.data_ptr(), None, None) == 0
        finally:
            lib.artfCudaDestroy(handle)


def test_allocation_failure_injected_on_the_host(lib):
    """With allocations made to fail on the host (artfCudaFailAllocAfter), each call that needs to grow a
    buffer reports ARTF_CUDA_ENOMEM and nothing else: a failure at any point of the mixed trace's host
    path (frame, view table, its staging, ray planes, order) or of the draw path leaves the context
    usable, and once allowed again the same calls give the same bits as a context that never failed."""
    scene = scenes.golden_scenes()["c1"]
    frame, frame64, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    fluid = scenes.unit_fluid()
    mixed = capi.TraceOptions(capi.MIXED, 4, 5, 1.0, 0.0, 0, 0, 1)
    exact = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 1)
    shape = (scene.height, scene.width)

    def render(handle):
        hdr = np.zeros(shape + (4,), np.float32)
        status = lib.artfCudaHoleRender(handle, C.byref(frame), None, m.ctypes.data, 0, fluid.ctypes.data, 0,
                                        C.byref(mixed), hdr.ctypes.data, None)
        return status, hdr

    def draw(handle):
        bgra = np.zeros(shape, np.uint32)
        status = lib.artfCudaHoleDraw(handle, C.byref(frame), C.byref(frame64), m.ctypes.data, 0,
                                      fluid.ctypes.data, 0, C.byref(exact), None, bgra.ctypes.data, None)
        return status, bgra

    clean = C.c_void_p()
    capi.check(lib.artfCudaCreate(0, C.byref(clean)))
    try:
        want_hdr, want_bgra = render(clean)[1], draw(clean)[1]
    finally:
        lib.artfCudaDestroy(clean)
    failures = 0
    for budget in range(8):
        handle = C.c_void_p()
        capi.check(lib.artfCudaCreate(0, C.byref(handle)))
        try:
            capi.check(lib.artfCudaFailAllocAfter(handle, budget))
            for call in (render, draw):
                status, _ = call(handle)
                assert status in (0, -3), status
                failures += status == -3
                if status == -3:
                    assert b"memory" in lib.artfCudaLastError() or b"allocation" in lib.artfCudaLastError()
            capi.check(lib.artfCudaFailAllocAfter(handle, -1))
            status, hdr = render(handle)
            assert status == 0 and np.array_equal(hdr.view(np.uint32), want_hdr.view(np.uint32))
            status, bgra = draw(handle)
            assert status == 0 and np.array_equal(bgra, want_bgra)
        finally:
            lib.artfCudaDestroy(handle)
    assert failures >= 4  # (the early budgets fail the first call that allocates)


@pytest.mark.parametrize("jitter", [0, 3])
def test_heavy_first_gives_the_same_bits(lib, ctx, jitter):
    """The queue's order (ArtfCudaTraceOptions.order) changes when a ray is traced, never what it computes:
    a batch of uneven views, one ray a pixel (a unit a pixel) and three (a unit a ray), heavy tiles first
    against pixel order, frames and ray ends the same bytes, and the same counts."""
    import torch
    views, keep = _views(lib, rays=max(jitter, 1))
    out = {}
    for order in (capi.ORDER_HEAVY_FIRST, capi.ORDER_PIXELS):
        stats = capi.TraceStats()
        for *_, hdr, ends in keep:
            hdr.zero_()
            ends.zero_()
        capi.check(lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(_opts(jitter=jitter, order=order)),
                                         C.byref(stats)))
        torch.cuda.synchronize()
        out[order] = ([(hdr.cpu().numpy().copy(), ends.cpu().numpy().copy()) for *_, hdr, ends in keep],
                      (stats.rays, stats.steps, stats.crossings, stats.escapes, stats.fp64Steps))
    (a, sa), (b, sb) = out[capi.ORDER_HEAVY_FIRST], out[capi.ORDER_PIXELS]
    assert sa == sb
    for i, ((ha, ea), (hb, eb)) in enumerate(zip(a, b)):
        assert np.array_equal(ha.view(np.uint32), hb.view(np.uint32)), i
        assert np.array_equal(ea, eb), i
    assert lib.artfCudaHoleBatch(ctx, views, len(views), C.byref(_opts(order=2)), None) == -1  # ARTF_CUDA_EINVAL


@pytest.mark.parametrize("guards", [0, capi.GUARD_MOTION | capi.GUARD_RADIAL | capi.GUARD_PSI])
def test_every_queue_kernel_gives_a_view_the_same_bits(lib, ctx, guards):
    """A frame runs the single-view queue kernel (its view a kernel parameter) and a graph of that one
    view the view table's; each has a form with the guards chosen at run time and one with all of them as
    constants.  Both pairs give the view the same bytes, four jittered rays a pixel (ray planes)."""
    import torch
    views, keep = _views(lib, count=1, scale=0.5, rays=4)
    scene, m, fluid, hdr, ends = keep[0]
    opts = _opts(jitter=4, seed=7, guards=guards)
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(views[0].frame), C.byref(views[0].frame64), m.data_ptr(),
                                     fluid.data_ptr(), C.byref(opts), hdr.data_ptr(), ends.data_ptr(),
                                     C.byref(capi.TraceStats())))
    torch.cuda.synchronize()
    alone, alone_ends = hdr.cpu().numpy().copy(), ends.cpu().numpy().copy()
    assert (alone[..., :3] > 0).any()
    hdr.zero_()
    ends.zero_()
    graph = C.c_void_p()
    capi.check(lib.artfCudaBatchGraphCreate(ctx, views, 1, C.byref(opts), C.byref(graph)))
    try:
        capi.check(lib.artfCudaBatchGraphLaunch(graph, C.byref(capi.TraceStats())))
        torch.cuda.synchronize()
        assert np.array_equal(hdr.cpu().numpy().view(np.uint32), alone.view(np.uint32))
        assert np.array_equal(ends.cpu().numpy(), alone_ends)
    finally:
        lib.artfCudaBatchGraphDestroy(graph)
