"""Parity of the CUDA traces through the C ABI, on a GB300.

  exact  the reference's bits: against the golden fixtures (the reference's own outputs) and the oracle
  fp32   FMA and fast reciprocals: pixel classes and radiance within the stated tolerances
  fp64   plain double: against the oracle's double instantiation
  mixed  FP32 with FP64 guards: endpoint error against the FP64 trace
"""
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from oracle import binding
from tests import gpu_helpers as g

pytestmark = pytest.mark.gpu

WHOLE = [n for n, s in scenes.golden_scenes().items() if s.whole]


def _scene_inputs(lib, name):
    scene = scenes.golden_scenes()[name]
    frame, frame64, clamped = scenes.frame(scene)
    return scene, frame, frame64, scenes.synth_map(lib, clamped, scene.seed, scene.emissivity), scenes.unit_fluid()


@pytest.mark.parametrize("name", list(scenes.golden_scenes()))
def test_exact_rays_match_reference_bits(lib, ctx, golden, name):
    _, arrays = golden
    scene, frame, frame64, m, fluid = _scene_inputs(lib, name)
    g.set_inputs(lib, ctx, m, fluid)
    rays = arrays[f"{name}_rays"]
    rgb, _ = g.trace_rays(lib, ctx, frame, None, capi.EXACT, rays[:, 0], rays[:, 1], rays[:, 2])
    want = arrays[f"{name}_rgb"]
    assert np.array_equal(rgb.view(np.uint32), want.view(np.uint32)), np.argwhere(rgb != want)[:5]


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("name", WHOLE)
def test_exact_frames_match_reference_bits(lib, ctx, golden, name, persistent):
    meta, _ = golden
    scene, frame, frame64, m, fluid = _scene_inputs(lib, name)
    g.set_inputs(lib, ctx, m, fluid)
    hdr, stats = g.trace(lib, ctx, frame, None, capi.EXACT, persistent=persistent)
    rgb = np.ascontiguousarray(hdr[..., :3])
    assert hashlib.sha256(rgb.tobytes()).hexdigest() == meta["views"][name]["hdr_sha256"]
    assert stats.rays == scene.width * scene.height * frame.size[2] ** 2


def test_exact_jittered_1080p_rows_match_reference_bits(lib, ctx, golden):
    meta, arrays = golden
    scene = scenes.config2(4)
    frame, frame64, clamped = scenes.frame(scene)
    g.set_inputs(lib, ctx, scenes.synth_map(lib, clamped, scene.seed, scene.emissivity), scenes.unit_fluid())
    hdr, stats = g.trace(lib, ctx, frame, None, capi.EXACT, jitter=4, seed=scene.jitter_seed)
    assert stats.rays == 1920 * 1080 * 4
    for i, y in enumerate(meta["c2_rows"]["rows"]):
        assert np.array_equal(hdr[y, :, :3], arrays["c2_rows"][i])


def test_exact_classes_and_ends_match_oracle(lib, ctx, golden):
    _, arrays = golden
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    g.set_inputs(lib, ctx, m, fluid)
    hdr, ends, stats = g.trace(lib, ctx, frame, None, capi.EXACT, ends=True)
    ohdr, oends = binding.render32(frame, m, fluid, ends=True)
    assert np.array_equal(hdr.view(np.uint32), ohdr.view(np.uint32))
    for field in ("hitR", "hitPhi", "dir", "mino", "steps", "crossings", "kind"):
        a, b = ends[field], oends[field]
        same = (a == b) | (np.isnan(a) & np.isnan(b)) if a.dtype.kind == "f" else a == b
        assert np.all(same), field
    assert stats.steps == int(ends["steps"].astype(np.int64).sum())
    assert stats.crossings == int(ends["crossings"].astype(np.int64).sum())
    assert np.mean(g.classes_of(hdr[..., 3]) == arrays["c1_classes"]) == 1.0


def _tolerance_report(hdr, want, bits_want):
    ring = g.ring_mask(bits_want)
    keep = ~ring
    agree = np.mean(g.classes_of(hdr[..., 3])[keep] == g.classes_of(bits_want)[keep])
    a = hdr[..., :3].astype(np.float64)
    b = want[..., :3].astype(np.float64)
    lum_a, lum_b = a.sum(-1), b.sum(-1)
    rel = np.abs(lum_a - lum_b) / np.maximum(np.abs(lum_b), 1e-3)
    return agree, rel[keep], ring.mean()


def test_fast_fp32_within_tolerance(lib, ctx):
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    g.set_inputs(lib, ctx, m, fluid)
    hdr, _ = g.trace(lib, ctx, frame, None, capi.FP32)
    want = binding.render32(frame, m, fluid)
    agree, rel, _ = _tolerance_report(hdr, want, want[..., 3])
    assert agree >= 0.999
    assert np.quantile(rel, 0.99) <= 1e-3
    assert abs(hdr[..., :3].astype(np.float64).sum() / want[..., :3].astype(np.float64).sum() - 1) < 1e-3


def test_fp64_matches_double_oracle(lib, ctx):
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "odd_101x67")
    g.set_inputs(lib, ctx, m, fluid)
    hdr, ends, _ = g.trace(lib, ctx, frame, frame64, capi.FP64, ends=True)
    want, oends = binding.render64(frame, frame64, m, fluid, ends=True)
    agree, rel, _ = _tolerance_report(hdr, want.astype(np.float32), want[..., 3])
    qs = {q: float(np.quantile(rel, q)) for q in (0.5, 0.9, 0.99, 0.999)}
    # The GPU's FP64 trace fuses multiply-adds and the CPU's does not: one rounding apart per operation,
    # amplified along the orbit; the median pixel is at FP32's resolution of the stored radiance.
    assert agree >= 0.999, qs
    assert qs[0.5] <= 1e-6 and qs[0.99] <= 1e-4, qs
    same_steps = np.mean(ends["steps"] == oends["steps"])
    assert same_steps >= 0.99


def test_mixed_endpoints_against_fp64(lib, ctx):
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    g.set_inputs(lib, ctx, m, fluid)
    hdr, ends, stats = g.trace(lib, ctx, frame, frame64, capi.MIXED, ends=True)
    ref, rends, _ = g.trace(lib, ctx, frame, frame64, capi.FP64, ends=True)
    agree, rel, _ = _tolerance_report(hdr, ref, ref[..., 3])
    assert agree >= 0.999
    assert np.quantile(rel, 0.99) <= 1e-3
    assert 0 < stats.fp64Steps < stats.steps


def test_pixel_centres_match_the_reference_positions(lib, ctx, golden):
    """The exact per-ray entry at the helper's pixel centres reproduces the reference's frame."""
    meta, arrays = golden
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "odd_101x67")
    g.set_inputs(lib, ctx, m, fluid)
    nx, ny = g.pixel_centres(frame)
    rgb, _ = g.trace_rays(lib, ctx, frame, None, capi.EXACT, nx, ny, 0.0)
    assert np.array_equal(rgb.reshape(arrays["odd_101x67_hdr"].shape), arrays["odd_101x67_hdr"])


def test_mixed_scheduler_is_independent_of_batching(lib, ctx):
    """The warp-batched scheduler changes when FP64 work runs, never what it computes: the frame is the
    same bits whatever the batch sizes and waits, and agrees with the per-ray path (a separate kernel,
    whose multiply-adds the compiler may fuse otherwise) to FP32 rounding."""
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    g.set_inputs(lib, ctx, m, fluid)
    base, base_ends, s_base = g.trace(lib, ctx, frame, frame64, capi.MIXED, ends=True)
    for batch, refill, wait in ((1, 1, 0), (16, 32, 0), (32, 8, 8), (7, 3, 200)):
        hdr, ends, s = g.trace(lib, ctx, frame, frame64, capi.MIXED, ends=True, batch=batch, wait=wait,
                               refill=refill)
        assert np.array_equal(hdr.view(np.uint32), base.view(np.uint32)), (batch, refill, wait)
        assert np.array_equal(ends.view(np.uint8), base_ends.view(np.uint8))
        assert s.fp64Steps == s_base.fp64Steps and s.steps == s_base.steps
        assert s.fp64Rounds <= s.fp64Horizon + s.fp64Radial + s.fp64Polar
    nx, ny = g.pixel_centres(frame)
    per_ray, ends_list, s_list = g.trace_rays(lib, ctx, frame, frame64, capi.MIXED, nx, ny, 0.0, ends=True)
    lum = base[..., :3].reshape(-1, 3).astype(np.float64).sum(1)
    lum_ray = per_ray.astype(np.float64).sum(1)
    rel = np.abs(lum - lum_ray) / np.maximum(lum_ray, 1e-3)
    assert np.mean(rel <= 1e-3) >= 0.999
    assert abs(int(s_list.steps) - int(s_base.steps)) <= 1e-3 * s_base.steps


def test_mixed_guards_select_their_fp64_work(lib, ctx):
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    g.set_inputs(lib, ctx, m, fluid)
    _, s_all = g.trace(lib, ctx, frame, frame64, capi.MIXED)
    assert s_all.fp64Horizon > 0 and s_all.fp64Radial > 0 and s_all.fp64Polar > 0
    _, s = g.trace(lib, ctx, frame, frame64, capi.MIXED, guards=capi.GUARD_MOTION | capi.GUARD_PSI)
    assert s.fp64Steps == 0 and s.fp64Rounds == 0
    _, s = g.trace(lib, ctx, frame, frame64, capi.MIXED, guards=capi.GUARD_HORIZON)
    assert s.fp64Radial == 0 and s.fp64Polar == 0 and s.fp64Horizon > 0
    _, s = g.trace(lib, ctx, frame, frame64, capi.MIXED, guards=capi.GUARD_POLAR | capi.GUARD_MOTION)
    assert s.fp64Radial == 0 and s.fp64Horizon == 0 and s.fp64Polar > 0
    _, s = g.trace(lib, ctx, frame, frame64, capi.MIXED, band=0.99)
    assert s.fp64Horizon < s_all.fp64Horizon


def test_host_path_equals_device_path(lib, ctx):
    import ctypes as C
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "odd_101x67")
    out = np.zeros((scene.height, scene.width, 4), np.float32)
    opts = capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 0)
    capi.check(lib.artfCudaHoleRender(ctx, C.byref(frame), None, m.ctypes.data, 1, fluid.ctypes.data, 1,
                                      C.byref(opts), out.ctypes.data, None))
    g.set_inputs(lib, ctx, m, fluid)
    hdr, _ = g.trace(lib, ctx, frame, None, capi.EXACT)
    assert np.array_equal(out.view(np.uint32), hdr.view(np.uint32))


def test_host_path_into_page_locked_memory(lib, ctx):
    """Into a page-locked buffer the trace's kernels write the frame directly: the same bits as the copy
    into a plain array, for the exact trace and for the mixed one with its ray planes."""
    import ctypes as C
    import torch
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "c1")
    for opts in (capi.TraceOptions(capi.EXACT, 0, 0, 1.0, 0.0, 0, 0, 1),
                 capi.TraceOptions(capi.MIXED, 4, 5, 1.0, 0.0, 0, 0, 1)):
        plain = np.zeros((scene.height, scene.width, 4), np.float32)
        locked = torch.zeros((scene.height, scene.width, 4), dtype=torch.float32).pin_memory()
        for buf in (plain.ctypes.data, locked.data_ptr()):
            capi.check(lib.artfCudaHoleRender(ctx, C.byref(frame), None, m.ctypes.data, 0, fluid.ctypes.data, 0,
                                              C.byref(opts), buf, None))
        assert np.array_equal(plain.view(np.uint32), locked.numpy().view(np.uint32))
        assert plain[..., :3].sum() > 0


def test_bad_options_are_refused(lib, ctx):
    import ctypes as C
    scene, frame, frame64, m, fluid = _scene_inputs(lib, "odd_3x2")
    g.set_inputs(lib, ctx, m, fluid)
    import torch
    hdr = torch.empty((2, 3, 4), device="cuda")
    for opts in (capi.TraceOptions(7, 0, 0, 1.0, 0, 0, 0, 0), capi.TraceOptions(0, -1, 0, 1.0, 0, 0, 0, 0),
                 capi.TraceOptions(0, 0, 0, 2.0, 0, 0, 0, 0)):
        assert lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(opts), hdr.data_ptr(), None,
                                     None) == capi_einval()


def capi_einval():
    return -1


def test_double_float_pairs_hold_their_bits(lib):
    """The wide sub-steps' double-float arithmetic (hi + lo) on the device against exact rational
    arithmetic, on 4000 seeded normalised pairs of either sign from 2^-8 to 2^8: a sum within 2^-45 of
    |a| + |b|, a product within 2^-44 of |a b|, the Newton-refined reciprocal within 2^-41 and reciprocal
    square root within 2^-40 relative (theory: about 2^-48, 2^-46, 2^-44 and 2^-43), and every result a
    normalised pair (hi is the pair's value rounded to float)."""
    import ctypes as C
    from fractions import Fraction
    rng = np.random.default_rng(17)
    n = 4000
    x = rng.uniform(-8.0, 8.0, (n, 2))
    x = np.sign(rng.uniform(-1, 1, (n, 2))) * np.exp2(x) * (1.0 + rng.uniform(0.0, 1.0, (n, 2)))
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    records = np.ascontiguousarray(np.stack([hi[:, 0], lo[:, 0], hi[:, 1], lo[:, 1]], 1), np.float32)
    out = np.zeros((n, 8), np.float32)
    capi.check(lib.artfCudaCheckPairs(None, records.ctypes.data, n, out.ctypes.data))

    def value(h, l):
        return Fraction(float(h)) + Fraction(float(l))

    worst = {"sum": 0.0, "product": 0.0, "recip": 0.0, "root": 0.0}
    for i in range(n):
        a, b = value(records[i, 0], records[i, 1]), value(records[i, 2], records[i, 3])
        got = [value(out[i, 2 * k], out[i, 2 * k + 1]) for k in range(4)]
        for k in range(4):
            pair_hi, pair_lo = out[i, 2 * k], out[i, 2 * k + 1]
            assert np.float32(np.float64(pair_hi) + np.float64(pair_lo)) == pair_hi, (i, k, pair_hi, pair_lo)
        worst["sum"] = max(worst["sum"], float(abs(got[0] - (a + b)) / (abs(a) + abs(b))))
        worst["product"] = max(worst["product"], float(abs(got[1] - a * b) / abs(a * b)))
        worst["recip"] = max(worst["recip"], float(abs(got[2] * a - 1)))
        worst["root"] = max(worst["root"], float(abs(got[3] * got[3] * abs(a) - 1) / 2))
    bounds = {"sum": 2.0 ** -45, "product": 2.0 ** -44, "recip": 2.0 ** -41, "root": 2.0 ** -40}
    for k, bound in bounds.items():
        assert worst[k] <= bound, (k, worst[k], bound)


def test_integer_conversions_match_the_hardware(lib):
    """The mixed trace's float <-> double conversions on the integer pipe give the hardware's bits: float
    to double on every float, double to float on 2^28 doubles around float's range and its rounding ties."""
    import ctypes as C
    bad = (C.c_uint64 * 4)()
    capi.check(lib.artfCudaCheckConversions(None, 1 << 28, bad))
    assert bad[0] == 0, f"float to double: {bad[0]} differ, first {bad[2]:#010x}"
    assert bad[1] == 0, f"double to float: {bad[1]} differ, first {bad[3]:#018x}"
