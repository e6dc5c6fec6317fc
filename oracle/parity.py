"""Parity of a traced frame against the reference's CPU trace of the same rays: test infrastructure for
the `-m gpu` parity tests and bench.py's CPU leg.  Nothing in the product imports it.

The reference computes in FP32 (src/software/lens.inc), and so does the bulk of every fast trace.  Two
FP32 traces that round differently disagree, and the disagreement is not uniform: the hashed-lattice
stars (lens.inc:69-86, 322-324; a tent of 0.1 or 0.17 of a cell at 90 or 240 cells a unit, ~7e-4 rad)
and the sky and disc texels make the radiance change by about 3e-3 for 1e-6 of escape direction, the
size of FP32's own rounding after some 40 steps.  On such pixels the reference is itself not within
1e-3 of the same algorithm evaluated in FP64 (0.24 % of the 1080p x 4 frame's pixels outside the
photon ring).  So the comparison names two sets of pixels:

  kept      outside one pixel of the photon ring (the shadow's edge in the reference's image), as the
            pixel-class criterion does;
  resolved  kept, and the FP64 evaluation of the reference's algorithm moves by at most `tol` (5e-4 by
            default) when every ray moves by `eps` (1e-6, a thousandth of a pixel) along either image
            axis: the radiance is fixed to that tolerance by the rays' positions at FP32's resolution.
            The moved rays are four FP64 renders of a frame whose forward vector is shifted by
            +-eps right, +-eps up (the same as moving each ray's image position).

and reports, for each pair of images, the share of pixels within 1e-3 relative (of the RGB sum, floor
1e-3) on both sets.  Even on the resolved pixels a few stay apart: the trajectory's moves do not cover
the rounding inside the shading itself (a colour or ring row chosen by truncating an FP32 product), and
on them the reference is not within 1e-3 of its own FP64 evaluation either (23 of the 2.07 million
resolved pixels of the 1080p x 4 frame).
"""
from __future__ import annotations

import numpy as np

from . import binding

EPS = 1e-6
TOL = 5e-4


def ring_mask(bits: np.ndarray) -> np.ndarray:
    """Pixels within one pixel of the shadow's edge: those with an 8-neighbour on the other side of
    dark / not dark (neither disc light nor sky: class bits 1 and 2 clear)."""
    dark = (bits.astype(np.uint32) & 3) == 0
    near = np.zeros_like(dark)
    h, w = dark.shape
    padded = np.pad(dark, 1, mode="edge")
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            near |= padded[1 + dy:1 + dy + h, 1 + dx:1 + dx + w] != dark
    return near


def classes_of(bits: np.ndarray) -> np.ndarray:
    """Disc (1) if any disc light, else sky (2) if the ray escaped, else horizon (0)."""
    b = bits.astype(np.uint32)
    return np.where(b & 1, 1, np.where(b & 2, 2, 0))


def relative(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Relative difference of two images' RGB sums, against b (floor 1e-3)."""
    la = a[..., :3].astype(np.float64).sum(-1)
    lb = b[..., :3].astype(np.float64).sum(-1)
    return np.abs(la - lb) / np.maximum(np.abs(lb), 1e-3)


class Reference:
    """The reference's trace of a frame on the CPU (the oracle port, the reference's bits), its FP64
    evaluation from the same frame, and the conditioning of each pixel."""

    def __init__(self, frame, map_, fluid, jitter: int, seed: int, eps: float = EPS, tol: float = TOL,
                 threads: int = 0):
        kw = dict(jitter=jitter, seed=seed, threads=threads)
        self.fp32 = binding.render32(frame, map_, fluid, **kw)
        self.fp64 = binding.render64(frame, binding.widened(frame), map_, fluid, **kw)
        moved = np.zeros(self.fp32.shape[:2])
        for shift in ((eps, 0.0), (-eps, 0.0), (0.0, eps), (0.0, -eps)):
            other = binding.render64(frame, binding.widened(frame, shift), map_, fluid, **kw)
            moved = np.maximum(moved, relative(other, self.fp64))
        self.kept = ~ring_mask(self.fp32[..., 3])
        self.resolved = self.kept & (moved <= tol)
        self.eps, self.tol = eps, tol

    def report(self, image: np.ndarray) -> dict:
        """An image of the same rays against the reference: classes on kept pixels; radiance within 1e-3
        on kept and on resolved pixels; and, beside it, the reference's own FP32 against its FP64."""
        keep, res = self.kept, self.resolved
        to_ref = relative(image, self.fp32)
        to_fp64 = relative(image, self.fp64)
        own = relative(self.fp32, self.fp64)
        agree = classes_of(image[..., 3])[keep] == classes_of(self.fp32[..., 3])[keep]
        return {
            "class_agreement_outside_ring": float(agree.mean()),
            "ring_share": float(1.0 - keep.mean()),
            "radiance_within_1e-3": float(np.mean(to_ref[keep] <= 1e-3)),
            "radiance_over_1e-3_pixels": int(np.sum(to_ref[keep] > 1e-3)),
            "radiance_rel_p99": float(np.quantile(to_ref[keep], 0.99)),
            "resolved_share_of_kept": float(res.sum() / max(1, keep.sum())),
            "radiance_within_1e-3_resolved": float(np.mean(to_ref[res] <= 1e-3)),
            "radiance_over_1e-3_resolved_pixels": int(np.sum(to_ref[res] > 1e-3)),
            "radiance_rel_max_resolved": float(to_ref[res].max()),
            "reference_fp32_vs_fp64_within_1e-3": float(np.mean(own[keep] <= 1e-3)),
            "reference_fp32_vs_fp64_over_1e-3_pixels": int(np.sum(own[keep] > 1e-3)),
            "reference_fp32_vs_fp64_over_1e-3_resolved_pixels": int(np.sum(own[res] > 1e-3)),
            "image_vs_fp64_within_1e-3": float(np.mean(to_fp64[keep] <= 1e-3)),
            "image_vs_fp64_over_1e-3_pixels": int(np.sum(to_fp64[keep] > 1e-3)),
            "image_vs_fp64_over_1e-3_resolved_pixels": int(np.sum(to_fp64[res] > 1e-3)),
            "conditioning": {"eps": self.eps, "tol": self.tol},
        }
