"""The Python check harness around the adjoint.

- `HoleLoss`, a torch.autograd.Function: its forward runs the C ABI's artfCudaHoleAdjoint over a batch
  of views (one launch: each view's loss and its gradient in the five scene parameters) and its
  backward hands back the gradient that launch computed.  The derivatives are the CUDA kernel's; torch
  supplies device buffers and the optimiser, nothing else.
- The scene parameters of the adjoint's workloads: 512 x 288 with a perturbed start, and 32 independent
  fits of 256 x 144 from seed 3.
- `fit_batch`: Adam over all fits at once, every step one adjoint launch for every view.
- `fd_gradients`: the plain alternative, central finite differences of FP64 renders (the FP64 trace
  of the same library, each perturbed scene with its own map tables), for comparison.

Parameters are theta = (spin, inclination [rad], inner radius / ISCO, emissivity index q, distance [M]).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import capi

PARAM_NAMES = ("spin", "inclination", "innerScale", "emissivity", "distance")
SPIN_LIMIT = 0.997  # below the scenes' 0.998, leaving room for a difference step


def _torch():
    import torch
    return torch


def hole_params(spin: float, inclination: float, inner_scale: float, emissivity: float, distance: float,
                seed: int = 4, fov: float = 0.6, outer: float = 12.0, height: float = 1e-3, doppler: float = 1.0,
                stars: float = 1.0, time_: float = 0.0) -> capi.HoleParams:
    """A scene by its five parameters (inclination in radians); the rest as the reference's defaults and
    the benchmark scenes (thin disc to 12 M, pinhole of 0.6 rad)."""
    d = capi.load().artfCudaBlackHoleDefaults()
    return capi.HoleParams(spin, inclination, inner_scale, emissivity, distance, fov, outer, height,
                           d.discThickness, d.discGain, doppler, stars, time_, seed)


def theta_of(p: capi.HoleParams) -> np.ndarray:
    return np.array([getattr(p, n) for n in PARAM_NAMES], np.float64)


def with_theta(p: capi.HoleParams, theta) -> capi.HoleParams:
    q = capi.HoleParams()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(capi.HoleParams))
    for n, v in zip(PARAM_NAMES, theta):
        setattr(q, n, float(v))
    return q


def frames(p: capi.HoleParams, width: int, height: int):
    """The FP32 and FP64 frames of a parameter scene and the Jacobian (28 x 5) of its frame fields."""
    lib = capi.load()
    f, f64 = capi.HoleFrame(), capi.HoleFrame64()
    jac = np.zeros((capi.GRAD_FIELDS, 5), np.float64)
    capi.check(lib.artfCudaHoleParamsFrames(C.byref(p), width, height, C.byref(f), C.byref(f64), jac.ctypes.data))
    return f, f64, jac


def param_map(p: capi.HoleParams) -> np.ndarray:
    m = np.zeros(capi.MAP_FLOATS, np.float32)
    capi.check(capi.load().artfCudaHoleParamsMap(C.byref(p), m.ctypes.data))
    return m


# ---- the workloads ------------------------------------------------------------------------------------

def config4_params():
    """The target (a = 0.7, i = 60 deg, r_in = r_ISCO, q = 3, r_obs = 30) and the perturbed start
    (a = 0.6, i = 55 deg, r_in = 1.1 r_ISCO, q = 2.7, r_obs = 32), 512 x 288."""
    target = hole_params(0.7, math.radians(60.0), 1.0, 3.0, 30.0, seed=4)
    start = hole_params(0.6, math.radians(55.0), 1.1, 2.7, 32.0, seed=4)
    return target, start


DRAWN = (0, 1, 2)  # the parameters configuration 5 draws: spin, inclination, inner radius


def config5_fits(count: int = 32, seed: int = 3, stars: float = 1.0, offset=DRAWN):
    """Independent fits: targets a in [0.1, 0.99], i in [20, 85] deg, r_in in [1, 1.5] r_ISCO (q = 3 and
    r_obs = 30 held), each start off by 15% up or down in the parameters `offset` (by default the three
    drawn ones; the spin at most 0.997), the rest at the target's values."""
    rng = np.random.default_rng(seed)
    fits = []
    for _ in range(count):
        a = float(rng.uniform(0.1, 0.99))
        incl = math.radians(float(rng.uniform(20.0, 85.0)))
        scale = float(rng.uniform(1.0, 1.5))
        target = hole_params(a, incl, scale, 3.0, 30.0, seed=seed, stars=stars)
        signs = rng.choice([-1.0, 1.0], size=5)
        start = theta_of(target)
        for q in offset:
            start[q] *= 1.0 + 0.15 * signs[q]
        start[0] = min(start[0], SPIN_LIMIT)
        fits.append((target, with_theta(target, start)))
    return fits


# ---- the adjoint through the C ABI -----------------------------------------------------------------------

class Adjoint:
    """artfCudaHoleAdjoint for views of one size: losses (n,), gradients (n, 5), the launch's stats.
    checkpoint: the interval of the rays' kept states; 1 keeps every state (48 bytes a step, up to 192
    steps a ray) and recomputes nothing, the fastest; 8 .. 64 keep less and recompute in between."""

    def __init__(self, lib, ctx, width: int, height: int, map_ptr=None, fluid_ptr=None, checkpoint: int = 1):
        self.lib, self.ctx = lib, ctx
        self.width, self.height = width, height
        self.map_ptr, self.fluid_ptr = map_ptr, fluid_ptr
        self.checkpoint = checkpoint
        self.last_stats = None

    def __call__(self, params, targets, hdr=None, checkpoint: int | None = None, pixel_grads=None):
        n = len(params)
        arr = (capi.HoleParams * n)(*params)
        res = (capi.AdjointResult * n)()
        stats = capi.TraceStats()
        capi.check(self.lib.artfCudaHoleAdjoint(
            self.ctx, arr, n, self.width, self.height, self.map_ptr, self.fluid_ptr, targets.data_ptr(),
            checkpoint or self.checkpoint, hdr.data_ptr() if hdr is not None else None,
            pixel_grads.data_ptr() if pixel_grads is not None else None, res, C.byref(stats)))
        self.last_stats = stats
        loss = np.array([r.loss for r in res], np.float64)
        grad = np.array([list(r.grad) for r in res], np.float64)
        return loss, grad, stats

    def render(self, params):
        """The adjoint's own forward radiance for each view (its loss against a zero target)."""
        torch = _torch()
        n = len(params)
        zero = torch.zeros((n, self.height, self.width, 4), dtype=torch.float32, device="cuda")
        hdr = torch.empty_like(zero)
        self(params, zero, hdr)
        return hdr


def hole_loss():
    """The torch.autograd.Function: theta (n, 5, float64, host) -> per-view losses (n,)."""
    torch = _torch()

    class HoleLoss(torch.autograd.Function):
        @staticmethod
        def forward(fctx, theta, adjoint, base, targets):
            params = [with_theta(b, t) for b, t in zip(base, theta.detach().cpu().numpy())]
            loss, grad, _ = adjoint(params, targets)
            fctx.save_for_backward(torch.from_numpy(grad))
            return torch.from_numpy(loss)

        @staticmethod
        def backward(fctx, grad_out):
            (grad,) = fctx.saved_tensors
            return grad_out[:, None] * grad, None, None, None

    return HoleLoss


def project(theta: np.ndarray) -> np.ndarray:
    """Keeps a fit inside the scenes the frame accepts, with room for a difference step: |a| <= 0.997,
    i in (0, pi), r_in >= 0.5 r_ISCO, r_obs >= 4."""
    t = theta.copy()
    t[..., 0] = np.clip(t[..., 0], -SPIN_LIMIT, SPIN_LIMIT)
    t[..., 1] = np.clip(t[..., 1], 1e-3, math.pi - 1e-3)
    t[..., 2] = np.maximum(t[..., 2], 0.5)
    t[..., 4] = np.maximum(t[..., 4], 4.0)
    return t


def _free_mask(free):
    torch = _torch()
    mask = torch.zeros(5, dtype=torch.float64)
    mask[list(free)] = 1.0
    return mask


def fit_batch(adjoint: Adjoint, fits, steps: int = 200, lr: float = 1e-2, free=DRAWN):
    """Adam on every fit at once (lr on theta relative to its starting guess, so one rate suits every
    parameter's scale); each step one adjoint launch over all views.  Only the parameters `free` move
    (by default the three configuration 5 draws); the others stay at their starting values.  Returns the
    fitted theta (n, 5), the per-step mean loss, and the wall time in seconds (targets excluded)."""
    torch = _torch()
    HoleLoss = hole_loss()
    targets_p = [t for t, _ in fits]
    base = [s for _, s in fits]
    targets = adjoint.render(targets_p)
    scale = torch.from_numpy(np.stack([theta_of(s) for s in base]))
    z = torch.zeros_like(scale, requires_grad=True)
    mask = _free_mask(free)
    opt = torch.optim.Adam([z], lr=lr)
    history = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        theta = scale * (1.0 + z)
        loss = HoleLoss.apply(theta, adjoint, base, targets)
        total = loss.sum()
        opt.zero_grad()
        total.backward()
        z.grad *= mask
        opt.step()
        with torch.no_grad():
            kept = torch.from_numpy(project((scale * (1.0 + z)).numpy()))
            z.copy_(kept / scale - 1.0)
        history.append(float(loss.detach().mean()))
    wall = time.perf_counter() - t0
    theta = (scale * (1.0 + z)).detach().numpy()
    return theta, np.array(history), wall


def recovery_error(theta: np.ndarray, fits) -> np.ndarray:
    """|fitted - true| / |true| per fit and parameter."""
    truth = np.stack([theta_of(t) for t, _ in fits])
    return np.abs(theta - truth) / np.abs(truth)


# ---- the plain alternative: FP64 forward renders and central differences ----------------------------------

class Fp64Loss:
    """The loss of views rendered by the FP64 trace (artfCudaHoleBatch), each scene with its own map
    (the parameter-dependent ring tables rebuilt on the host and copied up; the rest of the map shared)."""

    def __init__(self, lib, ctx, width: int, height: int, base_map: np.ndarray, fluid_ptr: int, capacity: int):
        torch = _torch()
        self.lib, self.ctx = lib, ctx
        self.width, self.height = width, height
        self.fluid_ptr = fluid_ptr
        self.host_map = base_map.copy()
        dev = torch.from_numpy(base_map).cuda()
        self.maps = dev.repeat(capacity, 1)  # (capacity, MAP_FLOATS)
        self.hdr = torch.empty((capacity, height, width, 4), dtype=torch.float32, device="cuda")
        self.capacity = capacity

    def render(self, params):
        """One FP64 trace launch a scene (artfCudaHoleTrace), on the context's stream."""
        torch = _torch()
        n = len(params)
        assert n <= self.capacity
        rings = np.empty((n, capi.MAP_HEIGHT * 2), np.float32)
        glow = np.empty((n, capi.MAP_HEIGHT), np.float32)
        framed = []
        for k, p in enumerate(params):
            f, f64, _ = frames(p, self.width, self.height)
            cam, desc = capi.Camera(), capi.BlackHoleDesc()
            capi.check(self.lib.artfCudaHoleParamsScene(C.byref(p), C.byref(cam), C.byref(desc)))
            sd = capi.SynthDesc(p.seed, desc.discInner, desc.discOuter, desc.spin, p.emissivity, 2000)
            self.lib.artfCudaSynthRings(C.byref(sd), self.host_map.ctypes.data)
            rings[k] = self.host_map[capi.ROWS_AT:capi.ROWS_AT + capi.MAP_HEIGHT * 2]
            glow[k] = self.host_map[capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT]
            framed.append((f, f64))
        self.maps[:n, capi.ROWS_AT:capi.ROWS_AT + capi.MAP_HEIGHT * 2] = torch.from_numpy(rings).cuda()
        self.maps[:n, capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT] = torch.from_numpy(glow).cuda()
        torch.cuda.synchronize()
        opts = capi.TraceOptions(capi.FP64, 0, 0, 1.0, 0.0, 0, 0, 0, 0, 0, 0)
        for k, (f, f64) in enumerate(framed):
            capi.check(self.lib.artfCudaHoleTrace(self.ctx, C.byref(f), C.byref(f64), self.maps[k].data_ptr(),
                                                  self.fluid_ptr, C.byref(opts), self.hdr[k].data_ptr(), None,
                                                  None))
        torch.cuda.ExternalStream(self.lib.artfCudaStream(self.ctx)).synchronize()
        return self.hdr[:n]

    def losses(self, params, targets):
        """Per-view mean squared error of linear RGB against targets (n, h, w, 4)."""
        hdr = self.render(params)
        d = (hdr[..., :3].double() - targets[..., :3].double())
        return (d * d).mean(dim=(1, 2, 3)).cpu().numpy()


def fd_gradients(fp64: Fp64Loss, params, targets, h: float = 1e-4):
    """Losses and central-difference gradients (step h on each parameter) of the FP64 renders: one batch
    of 11 scenes a view."""
    torch = _torch()
    n = len(params)
    scenes, tiles = [], []
    for k, p in enumerate(params):
        theta = theta_of(p)
        scenes.append(p)
        tiles.append(k)
        for q in range(5):
            for sign in (1.0, -1.0):
                t = theta.copy()
                t[q] += sign * h
                scenes.append(with_theta(p, t))
                tiles.append(k)
    out = np.empty(len(scenes))
    for lo in range(0, len(scenes), fp64.capacity):
        chunk = scenes[lo:lo + fp64.capacity]
        idx = torch.tensor(tiles[lo:lo + fp64.capacity], device="cuda")
        out[lo:lo + len(chunk)] = fp64.losses(chunk, targets.index_select(0, idx))
    out = out.reshape(n, 11)
    grads = (out[:, 1::2] - out[:, 2::2]) / (2 * h)
    return out[:, 0], grads


def fit_batch_fd(fp64: Fp64Loss, fits, targets, steps: int = 200, lr: float = 1e-2, h: float = 1e-4,
                 free=DRAWN):
    """The same fit as fit_batch with gradients from fd_gradients (FP64 renders, central differences):
    the fitted theta (n, 5), the per-step mean loss, and the wall time in seconds."""
    torch = _torch()
    base = [s for _, s in fits]
    scale = torch.from_numpy(np.stack([theta_of(s) for s in base]))
    z = torch.zeros_like(scale, requires_grad=True)
    mask = _free_mask(free)
    opt = torch.optim.Adam([z], lr=lr)
    history = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        theta = (scale * (1.0 + z)).detach().numpy()
        loss, grad = fd_gradients(fp64, [with_theta(b, t) for b, t in zip(base, theta)], targets, h)
        opt.zero_grad()
        z.grad = torch.from_numpy(grad) * scale * mask  # d loss / d z = d loss / d theta * scale
        opt.step()
        with torch.no_grad():
            kept = torch.from_numpy(project((scale * (1.0 + z)).numpy()))
            z.copy_(kept / scale - 1.0)
        history.append(float(loss.mean()))
    wall = time.perf_counter() - t0
    return (scale * (1.0 + z)).detach().numpy(), np.array(history), wall
