"""The gradients on the GPU: the FP64 forward-mode reference against central finite differences of FP64
renders, and the FP32 adjoint against the forward-mode reference; the adjoint's invariances (checkpoint
interval, batching, repetition), its argument checks, and the torch.autograd.Function of the harness.

Scenes: the adjoint workload's perturbed start (a = 0.6, i = 55 deg, r_in = 1.1 r_ISCO, q = 2.7,
r_obs = 32) at reduced sizes, one ray at each pixel's centre."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from artful_gb300 import capi, fit

pytestmark = pytest.mark.gpu

W, H = 64, 36


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module")
def scene(lib, ctx, torch):
    target, start = fit.config4_params()
    m = fit.param_map(start)
    fluid = np.ones(capi.FLUID_FLOATS, np.float32)
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 0))
    return target, start


def _tangents(lib, ctx, torch, p, w, h):
    """(h, w, 3, 6): radiance and its five derivatives, FP64 forward mode."""
    f, f64, jac = fit.frames(p, w, h)
    out = torch.empty((h, w, 3, 6), dtype=torch.float64, device="cuda")
    capi.check(lib.artfCudaHoleTangents(ctx, C.byref(p), C.byref(f), C.byref(f64), jac.ctypes.data, None, None,
                                        out.data_ptr()))
    return out.cpu().numpy()


def _fp64_render(lib, ctx, torch, p, w, h, own_map=True):
    """The FP64 trace of a parameter scene with its own map (the parameter-dependent ring tables)."""
    f, f64, _ = fit.frames(p, w, h)
    m = torch.from_numpy(fit.param_map(p)).cuda() if own_map else None
    hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    opts = capi.TraceOptions(capi.FP64, 0, 0, 1.0, 0.0, 0, 0, 0, 0, 0, 0)
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(f), C.byref(f64), m.data_ptr() if own_map else None, None,
                                     C.byref(opts), hdr.data_ptr(), None, None))
    torch.cuda.ExternalStream(lib.artfCudaStream(ctx)).synchronize()
    return hdr.cpu().numpy()[..., :3].astype(np.float64)


def test_tangent_values_are_the_fp64_trace(lib, ctx, torch, scene):
    """The forward-mode reference's values: the FP64 trace (whose ring tables it evaluates from their
    formulas, not the float tables: within float rounding of the tables)."""
    _, start = scene
    t = _tangents(lib, ctx, torch, start, W, H)[..., 0]
    r = _fp64_render(lib, ctx, torch, start, W, H)
    scale = np.abs(r).max()
    assert scale > 0
    close = np.abs(t - r) <= 1e-5 * np.abs(r) + 1e-7 * scale
    assert close.mean() >= 0.999, close.mean()


def _differences(lib, ctx, torch, p, q, h, render):
    theta = fit.theta_of(p)
    up, down = theta.copy(), theta.copy()
    up[q] += h
    down[q] -= h
    if render:
        return (_fp64_render(lib, ctx, torch, fit.with_theta(p, up), W, H)
                - _fp64_render(lib, ctx, torch, fit.with_theta(p, down), W, H)) / (2 * h)
    return (_tangents(lib, ctx, torch, fit.with_theta(p, up), W, H)[..., 0]
            - _tangents(lib, ctx, torch, fit.with_theta(p, down), W, H)[..., 0]) / (2 * h)


def test_tangents_match_differences_of_their_values(lib, ctx, torch, scene):
    """The dual numbers against central differences (h = 1e-6) of the same FP64 trace's values: the
    derivative of exactly what is computed.  Entries that carry a derivative (above 1% of the image's
    largest) agree within 1e-4 for at least 96% (the rest straddle a texel's kink or a discrete choice)."""
    _, start = scene
    tan = _tangents(lib, ctx, torch, start, W, H)
    for q in range(5):
        fd = _differences(lib, ctx, torch, start, q, 1e-6, render=False)
        t = tan[..., 1 + q]
        floor = 1e-2 * np.abs(t).max()
        carry = np.maximum(np.abs(t), np.abs(fd)) > floor
        assert carry.sum() > 30, (fit.PARAM_NAMES[q], carry.sum())
        agree = np.abs(fd - t) <= 1e-4 * np.abs(t) + 1e-4 * floor
        assert agree[carry].mean() >= 0.96, (fit.PARAM_NAMES[q], agree[carry].mean())


def test_tangents_match_central_differences_of_fp64_renders(lib, ctx, torch, scene):
    """Central differences of h = 1e-4 of the FP64 trace's renders (each scene with its own map).  The
    image is continuous but only piecewise smooth in theta (bilinear texels: the sky's point stars are
    one-texel tents), so a step of 1e-4 straddles kinks on many pixels; where the differences of h = 1e-4
    and h = 1e-6 agree (the image smooth at this scale), the forward-mode derivative agrees with them
    within 0.2% for at least 99% of the entries."""
    _, start = scene
    tan = _tangents(lib, ctx, torch, start, W, H)
    for q in range(5):
        wide = _differences(lib, ctx, torch, start, q, 1e-4, render=True)
        narrow = _differences(lib, ctx, torch, start, q, 1e-6, render=False)
        t = tan[..., 1 + q]
        floor = 1e-2 * np.abs(t).max()
        carry = np.maximum(np.abs(t), np.abs(wide)) > floor
        smooth = carry & (np.abs(wide - narrow) <= 1e-3 * np.maximum(np.abs(wide), np.abs(narrow)) + 1e-4 * floor)
        assert smooth.sum() >= 0.3 * carry.sum() and smooth.sum() > 10, (fit.PARAM_NAMES[q], smooth.sum(), carry.sum())
        agree = np.abs(wide - t) <= 2e-3 * np.abs(t) + 1e-4 * floor
        assert agree[smooth].mean() >= 0.99, (fit.PARAM_NAMES[q], agree[smooth].mean())


def _loss_and_grad_from_tangents(tan, target):
    """The loss and its gradient from the FP64 forward-mode reference, for a target (h, w, 3)."""
    value = tan[..., 0]
    d = value - target
    n = d.size
    loss = float((d * d).sum() / n)
    grad = np.array([float((2.0 * d * tan[..., 1 + q]).sum() / n) for q in range(5)])
    return loss, grad


def _adjoint(lib, ctx, torch, params, targets, w, h, k=32, hdr=None):
    adj = fit.Adjoint(lib, ctx, w, h, checkpoint=k)
    t = torch.from_numpy(np.ascontiguousarray(targets, np.float32)).cuda()
    return adj(params, t, hdr)


def _rgba(rgb):
    out = np.zeros(rgb.shape[:-1] + (4,), np.float32)
    out[..., :3] = rgb
    return out


@pytest.mark.parametrize("w,h", [(W, H), (128, 72)])
def test_adjoint_matches_forward_mode(lib, ctx, torch, scene, w, h):
    """The FP32 adjoint's loss and gradient against the FP64 forward-mode reference's, for a target that
    weights every pixel differently (the start's own image, each channel scaled by a seeded factor in
    [0.7, 1.3])."""
    _, start = scene
    tan = _tangents(lib, ctx, torch, start, w, h)
    rng = np.random.default_rng(11)
    target = tan[..., 0] * rng.uniform(0.7, 1.3, size=tan[..., 0].shape)
    loss64, grad64 = _loss_and_grad_from_tangents(tan, target)
    loss, grad, stats = _adjoint(lib, ctx, torch, [start], _rgba(target)[None], w, h)
    assert stats.rays == w * h and stats.steps > 0
    assert loss[0] == pytest.approx(loss64, rel=2e-3)
    err = np.abs(grad[0] - grad64)
    assert np.all(err <= 2e-2 * np.abs(grad64) + 5e-3 * np.abs(grad64).max()), (grad[0], grad64)


@pytest.mark.parametrize("k", [1, 32])
def test_adjoint_workload_per_pixel(lib, ctx, torch, scene, k):
    """The adjoint workload (512 x 288; every state kept, or checkpoints every 32 steps): loss between
    the start and the target's image.  Each pixel's share of the gradient against the forward-mode reference's: where the
    FP32 ray and the FP64 ray make the same choices (their radiance agrees within 1e-3), at least 99% of the
    shares that carry weight agree within 2%, and those pixels' sums within 0.5% of the gradient's largest
    component.  The few pixels where FP32 and FP64 choose differently (another star cell, a crossing
    found or missed) carry the rest of the difference of the totals."""
    target_p, start = scene
    w, h = 512, 288
    target = _tangents(lib, ctx, torch, target_p, w, h)[..., 0]
    tan = _tangents(lib, ctx, torch, start, w, h)
    loss64, grad64 = _loss_and_grad_from_tangents(tan, target)
    hdr = torch.zeros((1, h, w, 4), dtype=torch.float32, device="cuda")
    shares = torch.zeros((1, h, w, 5), dtype=torch.float32, device="cuda")
    adj = fit.Adjoint(lib, ctx, w, h, checkpoint=k)
    loss, grad, _ = adj([start], torch.from_numpy(_rgba(target)[None]).cuda(), hdr, pixel_grads=shares)
    assert loss[0] == pytest.approx(loss64, rel=2e-3)
    value = tan[..., 0]
    same = (np.abs(hdr.cpu().numpy()[0, ..., :3] - value) <= 1e-3 * np.abs(value) + 1e-6).all(-1)
    assert same.mean() >= 0.995
    ref = np.stack([(2.0 * (value - target) * tan[..., 1 + q]).sum(-1) / value.size for q in range(5)], -1)
    got = shares.cpu().numpy()[0]
    # the shares add up to the gradient, to the rounding of the float sums that formed it (a warp adds its
    # pixels' float shares before the tiles are added in double): bounded by the shares' magnitudes, since
    # a component's total may be far smaller than its parts
    flat = got.reshape(-1, 5).astype(np.float64)
    assert np.all(np.abs(flat.sum(0) - grad[0]) <= 1e-5 * np.abs(flat).sum(0) + 1e-12), (flat.sum(0), grad[0])
    for q in range(5):
        floor = 1e-2 * np.abs(ref[..., q]).max()
        carry = same & (np.maximum(np.abs(ref[..., q]), np.abs(got[..., q])) > floor)
        agree = np.abs(got[..., q] - ref[..., q]) <= 2e-2 * np.abs(ref[..., q]) + 1e-3 * floor
        assert agree[carry].mean() >= 0.99, (fit.PARAM_NAMES[q], agree[carry].mean())
    part = np.abs(got[same].sum(0) - ref[same].sum(0))
    assert np.all(part <= 5e-3 * np.abs(grad64).max()), (got[same].sum(0), ref[same].sum(0))


def test_adjoint_invariances(lib, ctx, torch, scene):
    """The checkpoint interval changes what is recomputed, not the result (1: every state kept, nothing
    recomputed); a view's result does not depend on the views batched with it; the same call gives the
    same bits."""
    target_p, start = scene
    target = _rgba(_tangents(lib, ctx, torch, target_p, W, H)[..., 0])
    base = _adjoint(lib, ctx, torch, [start], target[None], W, H, k=32)
    for k in (1, 8, 16, 64):
        other = _adjoint(lib, ctx, torch, [start], target[None], W, H, k=k)
        assert other[0][0] == base[0][0]
        np.testing.assert_allclose(other[1], base[1], rtol=1e-5, atol=1e-7 * np.abs(base[1]).max())
    again = _adjoint(lib, ctx, torch, [start], target[None], W, H, k=32)
    np.testing.assert_array_equal(again[1], base[1])
    second = fit.with_theta(start, fit.theta_of(start) * np.array([1.2, 0.9, 1.0, 1.1, 0.95]))
    batch = _adjoint(lib, ctx, torch, [second, start, second], np.stack([target] * 3), W, H, k=32)
    np.testing.assert_array_equal(batch[1][1], base[1][0])
    np.testing.assert_array_equal(batch[1][0], batch[1][2])
    assert batch[0][1] == base[0][0]


def test_adjoint_hdr_is_its_forward_radiance(lib, ctx, torch, scene):
    """The radiance the adjoint's forward pass writes: the FP64 trace's within FP32 accuracy."""
    _, start = scene
    adj = fit.Adjoint(lib, ctx, W, H)
    hdr = adj.render([start]).cpu().numpy()[0, ..., :3]
    r = _fp64_render(lib, ctx, torch, start, W, H)
    scale = np.abs(r).max()
    close = np.abs(hdr - r) <= 1e-3 * np.abs(r) + 1e-5 * scale
    assert close.mean() >= 0.995, close.mean()


def test_adjoint_rejects_bad_arguments(lib, ctx, torch, scene):
    _, start = scene
    t = torch.zeros((2, H, W, 4), dtype=torch.float32, device="cuda")
    res = (capi.AdjointResult * 2)()
    arr = (capi.HoleParams * 2)(start, start)
    # (a count above the limit is refused before params is read)
    for n, k in ((1, 0), (1, 65), (0, 32), (capi.ADJOINT_MAX_VIEWS + 1, 32)):
        assert lib.artfCudaHoleAdjoint(ctx, arr, n, W, H, None, None, t.data_ptr(), k, None, None, res, None) == -1
    assert lib.artfCudaHoleAdjoint(ctx, arr, 1, W, H, None, None, None, 32, None, None, res, None) == -1
    assert lib.artfCudaHoleAdjoint(ctx, arr, 1, 0, H, None, None, t.data_ptr(), 32, None, None, res, None) == -1
    bad = fit.with_theta(start, [1.5, 1.0, 1.0, 3.0, 30.0])  # |a| > 1
    arr2 = (capi.HoleParams * 1)(bad)
    assert lib.artfCudaHoleAdjoint(ctx, arr2, 1, W, H, None, None, t.data_ptr(), 32, None, None, res, None) != 0


def test_adjoint_trail_beyond_the_device_is_refused_cleanly(lib, ctx, torch, scene):
    """Every state of four 4096 x 4096 views kept would need 620 GB of trail, more than the device holds:
    the device refuses the allocation, the call returns ARTF_CUDA_ENOMEM before any launch, and the next
    call on the same context gives the bits it gave before (the refused allocation does not surface as a
    later launch's error)."""
    target_p, start = scene
    target = _rgba(_tangents(lib, ctx, torch, target_p, W, H)[..., 0])
    before = _adjoint(lib, ctx, torch, [start], target[None], W, H, k=1)
    n, side = 4, 4096
    assert n * side * side * 192 * 48 > 2 * torch.cuda.get_device_properties(0).total_memory
    big = torch.zeros((n, side, side, 4), dtype=torch.float32, device="cuda")  # a full-size target all the same
    arr = (capi.HoleParams * n)(*([start] * n))
    res = (capi.AdjointResult * n)()
    status = lib.artfCudaHoleAdjoint(ctx, arr, n, side, side, None, None, big.data_ptr(), 1, None, None, res, None)
    assert status == capi.ENOMEM, status
    del big
    after = _adjoint(lib, ctx, torch, [start], target[None], W, H, k=1)
    assert after[0][0] == before[0][0]
    np.testing.assert_array_equal(after[1], before[1])


def test_autograd_function_and_a_short_fit(lib, ctx, torch, scene):
    """The harness's torch.autograd.Function hands back the adjoint's gradient, and Adam on it brings a
    small fit's loss down (to under 60 % of the start's; with a constant rate it may then wander, the
    loss having the image's edges in it, and where it wanders to moves with the gradient's last bits)."""
    target_p, start = scene
    w, h = 96, 54
    adj = fit.Adjoint(lib, ctx, w, h)
    targets = adj.render([target_p])
    HoleLoss = fit.hole_loss()
    theta = torch.from_numpy(fit.theta_of(start)[None]).requires_grad_(True)
    loss = HoleLoss.apply(theta, adj, [start], targets)
    loss.sum().backward()
    _, grad, _ = adj([start], targets)
    np.testing.assert_array_equal(theta.grad.numpy(), grad)
    fitted, history, _ = fit.fit_batch(adj, [(target_p, start)], steps=40, free=range(5))
    assert history[1:].min() < 0.6 * history[0], history
