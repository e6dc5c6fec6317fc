"""The renderer backend (artful_cuda_renderer.h) through its eight-entry table, as Artful's public calls
would dispatch to it, and the draw path (trace, bloom, tone map) against the reference renderer's own
BGRA frames (tests/golden/): on a GB300 through the C ABI."""
import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from oracle import binding
from tests import gpu_helpers as g
from tests.test_oracle import DRAW_CASES, _draw_case

pytestmark = pytest.mark.gpu


class Backend:
    """A renderer made by artfCudaNew, called only through its table (rendererInternal.h:7-16)."""

    def __init__(self, lib, width, height):
        self.lib = lib
        opts = capi.RendererOptions(capi.BACKEND)
        opts.width, opts.height = width, height
        self.ptr = lib.artfCudaNew(C.byref(opts))
        assert self.ptr, lib.artfCudaLastError()
        self.head = C.cast(self.ptr, C.POINTER(capi.RendererHead)).contents
        self.vt = self.head.vt.contents
        self.width, self.height = width, height

    def draw(self, scene):
        return self.vt.draw(self.ptr, scene)

    def read(self):
        out = np.zeros((self.height, self.width), np.uint32)
        assert self.vt.readPixels(self.ptr, out.ctypes.data)
        return out

    def light(self):
        out = np.zeros((self.height, self.width, 4), np.float32)
        assert self.lib.artfCudaRendererReadLight(self.ptr, out.ctypes.data)
        return out

    def resize(self, w, h):
        self.vt.resize(self.ptr, w, h)
        self.width, self.height = w, h

    def free(self):
        self.vt.destroy(self.ptr)


def _scene(lib, view):
    s = lib.artfCudaSceneNew()
    lib.artfCudaSceneSetSeed(s, view.seed, view.emissivity)
    lib.artfCudaSceneSetCamera(s, C.byref(view.camera))
    lib.artfCudaSceneSetBlackHole(s, C.byref(view.desc))
    return s


@pytest.mark.parametrize("name", DRAW_CASES)
def test_draw_path_matches_reference_frames(lib, ctx, golden, name):
    meta, arrays = golden
    view = _draw_case(name)
    frame, frame64, clamped = scenes.frame(view)
    m = scenes.synth_map(lib, clamped, view.seed, view.emissivity)
    bgra = np.zeros((view.height, view.width), np.uint32)
    light = np.zeros((view.height, view.width, 4), np.float32)
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 1)
    stats = capi.TraceStats()
    fluid = scenes.unit_fluid()
    capi.check(lib.artfCudaHoleDraw(ctx, C.byref(frame), C.byref(frame64), m.ctypes.data, 0,
                                    fluid.ctypes.data, 0, C.byref(opts), light.ctypes.data,
                                    bgra.ctypes.data, C.byref(stats)))
    assert hashlib.sha256(bgra.tobytes()).hexdigest() == meta["draw"][name]["bgra_sha256"]
    assert stats.ms > 0


def test_backend_through_its_table(lib, golden):
    meta, arrays = golden
    view = _draw_case("c1_bloom")
    r = Backend(lib, view.width, view.height)
    s = _scene(lib, view)
    try:
        assert b"CUDA" in r.vt.description(r.ptr)
        assert r.vt.pixels(r.ptr) is None
        assert r.draw(s)
        assert hashlib.sha256(r.read().tobytes()).hexdigest() == meta["draw"]["c1_bloom"]["bgra_sha256"]
        light = np.ascontiguousarray(r.light()[..., :3])
        assert hashlib.sha256(light.tobytes()).hexdigest() == meta["views"]["c1"]["hdr_sha256"]
        stats = capi.FrameStats()
        r.vt.stats(r.ptr, C.cast(C.pointer(stats), C.c_void_p))
        assert stats.lensMs > 0 and stats.cpuMs >= stats.lensMs * 0.5
        # the odd sizes of the reference's own test (tests.c:4393-4400), and back
        for w, h in ((160, 90), (101, 67), (3, 2), (1, 1)):
            r.resize(w, h)
            assert r.draw(s)
        r.resize(101, 67)
        assert r.draw(s)
        # (the 101 x 67 view draws what the reference draws at that size)
        odd = _draw_case("odd_101x67_bloom")
        assert odd.camera.position.z == view.camera.position.z
        assert np.array_equal(r.read(), arrays["draw_odd_101x67_bloom"])
        # the hole removed: black; put back: the same picture
        lib.artfCudaSceneSetBlackHole(s, None)
        assert r.draw(s)
        assert np.all(r.read() == 0xFF000000)
        lib.artfCudaSceneSetBlackHole(s, C.byref(odd.desc))
        assert r.draw(s)
        assert np.array_equal(r.read(), arrays["draw_odd_101x67_bloom"])
    finally:
        r.free()
        lib.artfCudaSceneFree(s)


def test_backend_overlay_goes_over_the_frame(lib, golden):
    _, arrays = golden
    view = _draw_case("odd_101x67_bloom")
    r = Backend(lib, view.width, view.height)
    s = _scene(lib, view)
    try:
        overlay = np.zeros((20, 30), np.uint32)
        overlay[:, :15] = 0x80400000   # half-covering, premultiplied red
        overlay[:, 15:] = 0xFF00FF00   # opaque green
        o = capi.Overlay(overlay.ctypes.data, 30, 20, 0, False, None, 0)
        r.vt.setOverlay(r.ptr, C.cast(C.pointer(o), C.c_void_p))
        assert r.draw(s)
        got = r.read()
        base = arrays["draw_odd_101x67_bloom"]
        assert np.all(got[:20, 15:30] == 0xFF00FF00)
        assert np.array_equal(got[20:], base[20:])
        p, q = int(got[5, 5]), int(base[5, 5])
        red = (p >> 16) & 255
        assert abs(red - (0x40 + ((q >> 16) & 255) * 127 // 255)) <= 1
    finally:
        r.free()
        lib.artfCudaSceneFree(s)


def test_backend_device_loss_then_a_new_renderer(lib, golden):
    """The reference's lost-device contract (renderer.h:107-109, tests.c:2719-2749): draw returns false,
    the renderer is freed, the scene goes to a new one, which draws the same bytes.  The loss is injected
    on the host: the GPU is never faulted."""
    meta, _ = golden
    view = _draw_case("c1_bloom")
    s = _scene(lib, view)
    try:
        r = Backend(lib, view.width, view.height)
        capi.check(lib.artfCudaFailAfter(lib.artfCudaRendererContext(r.ptr), 1))
        assert r.draw(s)
        first = r.read()
        assert not r.draw(s)
        r.free()
        r = Backend(lib, view.width, view.height)
        assert r.draw(s)
        assert np.array_equal(r.read(), first)
        assert hashlib.sha256(first.tobytes()).hexdigest() == meta["draw"]["c1_bloom"]["bgra_sha256"]
        r.free()
    finally:
        lib.artfCudaSceneFree(s)


def test_backend_mixed_precision_stays_within_tolerance(lib, golden):
    _, arrays = golden
    view = _draw_case("odd_101x67_bloom")
    r = Backend(lib, view.width, view.height)
    s = _scene(lib, view)
    try:
        lib.artfCudaRendererSetPrecision(r.ptr, capi.MIXED)
        assert r.draw(s)
        got = r.read().view(np.uint8).reshape(view.height, view.width, 4).astype(int)
        want = arrays["draw_odd_101x67_bloom"].view(np.uint8).reshape(view.height, view.width, 4).astype(int)
        worst = np.abs(got - want)[..., :3].max(-1)
        # the reference's CPU-versus-GPU bar (tests.c:4402-4450): under 1 % of pixels off by more than 24/255
        assert np.mean(worst > 24) < 0.01 and np.mean(worst > 96) < 0.001
    finally:
        r.free()
        lib.artfCudaSceneFree(s)


def test_backend_draws_the_reference_scene_over_time(lib, golden):
    """Device inputs: the reference's own scene (its painted disc, its gas started and advanced by
    artfSceneSetBlackHole, hole.c:242-271) drawn by the reference's software renderer over a timeline,
    against this backend painting the disc and stepping the gas on the GPU from the same settings: every
    frame the same bytes.  A second renderer that joins halfway catches the gas up in one call and draws the
    same; switching device inputs off and on again redraws the same."""
    meta, arrays = golden
    want = meta["timeline"]["bgra_sha256"]
    width, height, steps = scenes.timeline()
    r = Backend(lib, width, height)
    lib.artfCudaRendererSetDeviceInputs(r.ptr, True)
    late = None
    s = lib.artfCudaSceneNew()
    try:
        drawn = 0
        for i, (cam, desc, draw) in enumerate(steps):
            lib.artfCudaSceneSetCamera(s, C.byref(cam))
            lib.artfCudaSceneSetBlackHole(s, C.byref(desc))
            if not draw:
                continue
            assert r.draw(s)
            assert hashlib.sha256(r.read().tobytes()).hexdigest() == want[drawn], (i, drawn)
            if drawn == 5:   # after the clock ran far back: a new renderer, a gas 23 steps on
                late = Backend(lib, width, height)
                lib.artfCudaRendererSetDeviceInputs(late.ptr, True)
            if late is not None:
                assert late.draw(s)
                assert hashlib.sha256(late.read().tobytes()).hexdigest() == want[drawn], ("late", i)
            drawn += 1
        assert drawn == len(want)
        assert np.array_equal(r.read(), arrays["timeline_last"])
        # host inputs (the scene's synthetic map) in between, then device inputs again: the same frame
        lib.artfCudaRendererSetDeviceInputs(r.ptr, False)
        assert r.draw(s)
        assert not np.array_equal(r.read(), arrays["timeline_last"])
        lib.artfCudaRendererSetDeviceInputs(r.ptr, True)
        assert r.draw(s)
        assert np.array_equal(r.read(), arrays["timeline_last"])
    finally:
        r.free()
        if late is not None:
            late.free()
        lib.artfCudaSceneFree(s)


def test_draw_with_what_the_context_holds(lib, ctx, golden):
    """artfCudaHoleDraw with no host map or fluid draws the context's: uploaded once, then drawn again."""
    meta, _ = golden
    view = _draw_case("c1_bloom")
    frame, frame64, clamped = scenes.frame(view)
    m = scenes.synth_map(lib, clamped, view.seed, view.emissivity)
    fluid = scenes.unit_fluid()
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 0))
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 1)
    bgra = np.zeros((view.height, view.width), np.uint32)
    capi.check(lib.artfCudaHoleDraw(ctx, C.byref(frame), C.byref(frame64), None, 0, None, 0, C.byref(opts), None,
                                    bgra.ctypes.data, None))
    assert hashlib.sha256(bgra.tobytes()).hexdigest() == meta["draw"]["c1_bloom"]["bgra_sha256"]


def test_frame_read_after_a_draw(lib, ctx, golden):
    """A draw that copies nothing back leaves its frame on the device; artfCudaFrameRead returns the same
    light and BGRA a draw into host buffers gives, and refuses once the light buffer has been reused."""
    meta, _ = golden
    view = _draw_case("c1_bloom")
    frame, frame64, clamped = scenes.frame(view)
    m = scenes.synth_map(lib, clamped, view.seed, view.emissivity)
    fluid = scenes.unit_fluid()
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 1)
    shape = (view.height, view.width)
    light, bgra = np.zeros(shape + (4,), np.float32), np.zeros(shape, np.uint32)
    capi.check(lib.artfCudaHoleDraw(ctx, C.byref(frame), C.byref(frame64), m.ctypes.data, 0, fluid.ctypes.data, 0,
                                    C.byref(opts), light.ctypes.data, bgra.ctypes.data, None))
    capi.check(lib.artfCudaHoleDraw(ctx, C.byref(frame), C.byref(frame64), m.ctypes.data, 0, fluid.ctypes.data, 0,
                                    C.byref(opts), None, None, None))
    light2, bgra2 = np.zeros_like(light), np.zeros_like(bgra)
    capi.check(lib.artfCudaFrameRead(ctx, light2.ctypes.data, bgra2.ctypes.data))
    assert np.array_equal(bgra2, bgra) and np.array_equal(light2.view(np.uint32), light.view(np.uint32))
    assert hashlib.sha256(bgra2.tobytes()).hexdigest() == meta["draw"]["c1_bloom"]["bgra_sha256"]
    only = np.zeros_like(bgra)
    capi.check(lib.artfCudaFrameRead(ctx, None, only.ctypes.data))
    assert np.array_equal(only, bgra)
    # the host path's render reuses the light buffer: nothing drawn to read any more
    capi.check(lib.artfCudaHoleRender(ctx, C.byref(frame), C.byref(frame64), m.ctypes.data, 0, fluid.ctypes.data, 0,
                                      C.byref(opts), light2.ctypes.data, None))
    assert lib.artfCudaFrameRead(ctx, None, only.ctypes.data) == -1
    assert b"no frame drawn" in lib.artfCudaLastError()
