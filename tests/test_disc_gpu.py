"""The reference's painted disc map made on the GPU (artful_gb300/csrc/disc.cu): byte for byte the
reference's (golden hashes recorded from hole.c) and the oracle's; into the context's map, where the trace
reads it."""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _paint(lib, ctx, torch, inner, outer, spin):
    dev = torch.empty(capi.MAP_FLOATS, dtype=torch.float32, device="cuda")
    capi.check(lib.artfCudaPaintDisc(ctx, dev.data_ptr(), inner, outer, spin))
    return dev.cpu().numpy()


@pytest.mark.parametrize("name", ["c1", "retro_edge", "spinless_3x3"])
def test_gpu_painted_map_is_the_reference(lib, ctx, golden, name):
    import torch
    case = golden[0]["painted"][name]
    m = _paint(lib, ctx, torch, case["inner"], case["outer"], case["spin"])
    assert _sha(m) == case["map_sha256"]


def test_gpu_painted_map_equals_the_oracle(lib, ctx, oracle_lib):
    import torch
    inner, outer, spin = 4.0, 17.0, 0.3
    got = _paint(lib, ctx, torch, inner, outer, spin)
    want = np.zeros(capi.MAP_FLOATS, np.float32)
    oracle_lib.oraclePaintDisc(want.ctypes.data)
    oracle_lib.oracleSetRings(want.ctypes.data, inner, outer, spin)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_painted_into_the_context_map_is_what_the_trace_reads(lib, ctx):
    """Painted straight into the context's map, a frame equals the frame traced from the same map
    uploaded from the host."""
    import torch
    scene = scenes.golden_scenes()["c1"]
    frame, frame64, clamped = scenes.frame(scene)
    capi.check(lib.artfCudaPaintDisc(ctx, None, clamped.discInner, clamped.discOuter, clamped.spin))
    fluid = scenes.unit_fluid()
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 0))
    h, w = scene.height, scene.width
    out = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for _ in range(2)]
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 0)
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, None, C.byref(opts),
                                     out[0].data_ptr(), None, None))
    torch.cuda.ExternalStream(lib.artfCudaStream(ctx)).synchronize()
    painted = _paint(lib, ctx, torch, clamped.discInner, clamped.discOuter, clamped.spin)
    capi.check(lib.artfCudaSetMap(ctx, painted.ctypes.data, 0))
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64), None, None, C.byref(opts),
                                     out[1].data_ptr(), None, None))
    torch.cuda.ExternalStream(lib.artfCudaStream(ctx)).synchronize()
    a, b = out[0].cpu().numpy(), out[1].cpu().numpy()
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a[..., :3] > 0).any()


def test_paint_rejects_bad_discs(lib, ctx):
    assert lib.artfCudaPaintDisc(ctx, None, 0.0, 12.0, 0.5) == -1
    assert lib.artfCudaPaintDisc(ctx, None, 5.0, 4.0, 0.5) == -1
    assert lib.artfCudaPaintDisc(None, None, 2.0, 12.0, 0.5) == -1


def test_gpu_painted_maps_of_seeded_discs_equal_the_oracle(lib, ctx, oracle_lib):
    """Fifty seeded discs (spin in [-0.998, 0.998], inner edge 1 to 1.5 times the ISCO, outer edge 1 to 20
    M beyond it): every painted map the reference's byte for byte.  The gas, dust, colours and sky are
    the same for every disc (hole.c paints them once); the ring tables follow the disc."""
    import torch
    painted = np.zeros(capi.MAP_FLOATS, np.float32)
    oracle_lib.oraclePaintDisc(painted.ctypes.data)
    rng = np.random.default_rng(50)
    for _ in range(50):
        spin = float(rng.uniform(-0.998, 0.998))
        inner = float(np.float32(lib.artfCudaIsco(spin) * rng.uniform(1.0, 1.5)))
        outer = float(np.float32(inner + rng.uniform(1.0, 20.0)))
        got = _paint(lib, ctx, torch, inner, outer, spin)
        want = painted.copy()
        oracle_lib.oracleSetRings(want.ctypes.data, inner, outer, spin)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"{inner} {outer} {spin}")
