"""The disc fluid stepped on the GPU (artful_gb300/csrc/fluid.cu): its field's bytes against the
reference's (golden hashes recorded from fluid.c) and against the oracle run here; the reference's own
determinism test; the trace reading the field where it lies on the device."""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from oracle import binding

pytestmark = pytest.mark.gpu


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


class GpuFluid:
    def __init__(self, lib, ctx, inner, outer, spin, time):
        self.lib = lib
        self.handle = C.c_void_p()
        capi.check(lib.artfCudaFluidNew(ctx, inner, outer, spin, time, C.byref(self.handle)))

    def advance(self, time):
        stepped = C.c_int()
        capi.check(self.lib.artfCudaFluidAdvance(self.handle, time, C.byref(stepped)))
        return bool(stepped.value)

    def read(self):
        out = np.empty(capi.FLUID_FLOATS, np.float32)
        capi.check(self.lib.artfCudaFluidRead(self.handle, out.ctypes.data))
        return out, self.lib.artfCudaFluidTime(self.handle)

    def free(self):
        self.lib.artfCudaFluidFree(self.handle)


@pytest.mark.parametrize("name", ["a0.9", "a0.998", "a-0.5"])
def test_gpu_fluid_is_the_reference_byte_for_byte(lib, ctx, golden, name):
    meta, _ = golden
    case = meta["fluid"][name]
    fl = GpuFluid(lib, ctx, case["inner"], case["outer"], case["spin"], case["time"])
    field, t = fl.read()
    assert _sha(field) == case["states"][0]["field_sha256"] and t == case["states"][0]["time"]
    for want in case["states"][1:]:
        stepped = fl.advance(want["advance_to"])
        field, t = fl.read()
        assert stepped == want["stepped"], want["advance_to"]
        assert t == want["time"]
        assert _sha(field) == want["field_sha256"], want["advance_to"]
    fl.free()


def test_gpu_fluid_equals_the_oracle(lib, ctx, oracle_lib):
    """A disc the fixtures do not hold, against the oracle run on this machine."""
    inner, outer, spin = 1.7, 20.0, 0.6
    a = GpuFluid(lib, ctx, inner, outer, spin, 3.3)
    b = binding.Fluid(oracle_lib, "oracle", inner, outer, spin, 3.3)
    for target in (None, 4.1, 9.7):
        if target is not None:
            assert a.advance(target) == b.advance(target)
        fa, ta = a.read()
        fb, tb = b.read()
        assert ta == tb
        np.testing.assert_array_equal(fa.view(np.uint32), fb.view(np.uint32))
    a.free()
    b.free()


def test_gpu_fluid_is_deterministic(lib, ctx):
    """The reference's own check (tests.c:4180-4194): one hop or two to the same moment give the same
    bytes, the gas moved, and less than a step does nothing."""
    inner, outer, spin = float(lib.artfCudaIsco(0.9)), 12.0, 0.9
    a = GpuFluid(lib, ctx, inner, outer, spin, 0.0)
    b = GpuFluid(lib, ctx, inner, outer, spin, 0.0)
    before, _ = a.read()
    assert a.advance(2.0)
    assert b.advance(1.0) and b.advance(2.0)
    fa, _ = a.read()
    fb, _ = b.read()
    assert not np.array_equal(before, fa)
    np.testing.assert_array_equal(fa.view(np.uint32), fb.view(np.uint32))
    assert not a.advance(lib.artfCudaFluidTime(a.handle) + 0.1)
    a.free()
    b.free()


def test_gpu_fluid_rejects_bad_discs(lib, ctx):
    h = C.c_void_p()
    assert lib.artfCudaFluidNew(ctx, 0.0, 12.0, 0.5, 0.0, C.byref(h)) == -1
    assert lib.artfCudaFluidNew(ctx, 5.0, 4.0, 0.5, 0.0, C.byref(h)) == -1
    assert lib.artfCudaFluidNew(ctx, 2.0, 12.0, 1.5, 0.0, C.byref(h)) == -1
    assert lib.artfCudaFluidNew(ctx, 2.0, 12.0, 0.5, 0.0, None) == -1
    assert lib.artfCudaFluidAdvance(None, 1.0, None) == -1


def test_trace_reads_the_field_on_the_device(lib, ctx):
    """A frame traced with the GPU fluid's field where it lies equals the frame traced from a host copy
    of that field uploaded to the context: the field needs no trip through the host."""
    import torch
    scene = scenes.config1()
    frame, frame64, clamped = scenes.frame(scene)
    map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    fl = GpuFluid(lib, ctx, float(clamped.discInner), float(clamped.discOuter), float(clamped.spin), 0.0)
    field, _ = fl.read()
    capi.check(lib.artfCudaSetMap(ctx, map_.ctypes.data, 0))
    capi.check(lib.artfCudaSetFluid(ctx, field.ctypes.data, 0))
    h, w = scene.height, scene.width
    out = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for _ in range(2)]
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 0)
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, None, C.byref(opts),
                                     out[0].data_ptr(), None, None))
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, lib.artfCudaFluidField(fl.handle),
                                     C.byref(opts), out[1].data_ptr(), None, None))
    torch.cuda.ExternalStream(lib.artfCudaStream(ctx)).synchronize()
    a, b = out[0].cpu().numpy(), out[1].cpu().numpy()
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (field != 1.0).any()  # (a real field, not the unit one)
    fl.free()


def test_counted_steps_equal_the_advances(lib, ctx):
    """The field depends only on the steps taken since the start: a gas advanced call by call and one
    stepped once by the count artfCudaFluidClock gives (more than four calls' 48) hold the same bytes and
    the same time.  (That the trace reads a gas handed to the context is the renderer's timeline test.)"""
    inner, outer, spin = float(lib.artfCudaIsco(0.9)), 12.0, 0.9
    a = GpuFluid(lib, ctx, inner, outer, spin, 2.0)
    b = GpuFluid(lib, ctx, inner, outer, spin, 2.0)
    clock, total = C.c_double(2.0), 0
    try:
        for target in (2.7, 3.1, 12.0, 11.0, 16.05, 26.0, 36.0, 46.0, 56.0):
            a.advance(target)
            total += lib.artfCudaFluidClock(C.byref(clock), target)
        assert total > 4 * 48  # (more than one run of artfCudaFluidStep's staging)
        capi.check(lib.artfCudaFluidStep(b.handle, total, clock.value))
        fa, ta = a.read()
        fb, tb = b.read()
        assert ta == tb == clock.value
        assert _sha(fa) == _sha(fb)
        capi.check(lib.artfCudaUseFluid(ctx, b.handle))
        capi.check(lib.artfCudaSetFluid(ctx, scenes.unit_fluid().ctypes.data, 0))  # (as other tests left it)
        assert lib.artfCudaUseFluid(ctx, None) != 0
        assert lib.artfCudaFluidStep(b.handle, -1, 1.0) != 0
    finally:
        a.free()
        b.free()
