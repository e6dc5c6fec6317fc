"""Device-side helpers for the `-m gpu` tests: every trace goes through the C ABI (ctypes), with device
buffers from torch (plumbing only)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from artful_gb300 import capi
from oracle import binding

END_DTYPE = binding.END_DTYPE


def _torch():
    import torch
    return torch


def set_inputs(lib, ctx, map_, fluid):
    capi.check(lib.artfCudaSetMap(ctx, map_.ctypes.data, 0))
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 0))


def trace(lib, ctx, frame, frame64, precision, jitter=0, seed=0, step_scale=1.0, persistent=0, ends=False,
          band=0.0, guards=0, batch=0, wait=0, refill=0, block=0):
    """One frame on the device from the context's map and fluid: (H, W, 4) HDR, the ray ends, the stats."""
    torch = _torch()
    w, h = frame.size[0], frame.size[1]
    rays = jitter if jitter else frame.size[2] ** 2
    hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    e = torch.empty((w * h * rays * 32,), dtype=torch.uint8, device="cuda") if ends else None
    opts = capi.TraceOptions(precision, jitter, seed, step_scale, band, block, wait, persistent, guards, batch,
                             refill)
    stats = capi.TraceStats()
    capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), C.byref(frame64) if frame64 is not None else None, None,
                                     None, C.byref(opts), hdr.data_ptr(), e.data_ptr() if ends else None,
                                     C.byref(stats)))
    out = hdr.cpu().numpy()
    if ends:
        return out, np.frombuffer(e.cpu().numpy().tobytes(), END_DTYPE), stats
    return out, stats


def trace_rays(lib, ctx, frame, frame64, precision, nx, ny, t, step_scale=1.0, ends=False):
    torch = _torch()
    n = len(nx)
    dx = torch.from_numpy(np.ascontiguousarray(nx, np.float32)).cuda()
    dy = torch.from_numpy(np.ascontiguousarray(ny, np.float32)).cuda()
    dt = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(t, (n,)), np.float32)).cuda()
    rgb = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    e = torch.empty((n * 32,), dtype=torch.uint8, device="cuda") if ends else None
    stats = capi.TraceStats()
    capi.check(lib.artfCudaHoleTraceRays(ctx, C.byref(frame), C.byref(frame64) if frame64 is not None else None,
                                         None, None, precision, step_scale, n, dx.data_ptr(), dy.data_ptr(),
                                         dt.data_ptr(), rgb.data_ptr(), e.data_ptr() if ends else None,
                                         C.byref(stats)))
    out = rgb.cpu().numpy()
    if ends:
        return out, np.frombuffer(e.cpu().numpy().tobytes(), END_DTYPE), stats
    return out, stats


def pixel_centres(frame):
    """The image positions of one ray at each pixel's centre, in the reference's float arithmetic
    (lens.inc:367-369: the eight-pixel group's base column, then the lane)."""
    w, h = frame.size[0], frame.size[1]
    x = np.arange(w, dtype=np.int64)
    y = np.arange(h, dtype=np.int64)
    half = np.float32(0.5)
    nx = (np.float32(x & 7).astype(np.float32) + ((x & ~7).astype(np.float32) + half)) * np.float32(frame.image[1]) \
        - np.float32(1)
    ny = np.float32(1) - (y.astype(np.float32) + half) * np.float32(frame.image[2])
    nx = np.broadcast_to(nx.astype(np.float32)[None, :], (h, w))
    ny = np.broadcast_to(ny.astype(np.float32)[:, None], (h, w))
    return np.ascontiguousarray(nx).ravel(), np.ascontiguousarray(ny).ravel()


def ring_mask(bits: np.ndarray) -> np.ndarray:
    """Pixels within one pixel of the shadow's edge (the photon ring): those with an 8-neighbour on the
    other side of dark / not dark."""
    dark = (bits.astype(np.uint32) & 3) == 0
    near = np.zeros_like(dark)
    h, w = dark.shape
    padded = np.pad(dark, 1, mode="edge")
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            near |= padded[1 + dy:1 + dy + h, 1 + dx:1 + dx + w] != dark
    return near


def classes_of(bits: np.ndarray) -> np.ndarray:
    b = bits.astype(np.uint32)
    return np.where(b & 1, 1, np.where(b & 2, 2, 0))
