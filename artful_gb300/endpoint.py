"""Endpoint error of a trace against another trace of the same rays (normally the plain FP64 trace, at
the same or half the step): from the ray-end records (ArtfCudaRayEnd) and the HDR frames that
artfCudaHoleTrace writes.

Per ray: the disc-hit radius (relative) and azimuth (turns, on the circle) where both rays lit the
disc, and the escape direction (unit vectors) where both escaped; a ray's error is the largest of
those it has.  Per pixel: the radiance (the RGB sum) relative to the other frame's, floor 1e-3.
"""
from __future__ import annotations

import numpy as np

END_DTYPE = np.dtype([("hitR", "<f4"), ("hitPhi", "<f4"), ("dir", "<f4", (3,)), ("mino", "<f4"),
                      ("steps", "<u2"), ("crossings", "u1"), ("kind", "u1"), ("fp64Steps", "<u2"),
                      ("reserved", "<u2")])


def ray_errors(e: np.ndarray, r: np.ndarray):
    """Each ray's endpoint error against r's, and which rays are comparable (both lit the disc, or both
    escaped)."""
    both_hit = np.isfinite(e["hitR"]) & np.isfinite(r["hitR"])
    both_sky = ((e["kind"] & 15) == 1) & ((r["kind"] & 15) == 1)
    per_ray = np.zeros(len(e))
    with np.errstate(invalid="ignore", divide="ignore"):
        dr = np.abs(e["hitR"].astype(np.float64) - r["hitR"]) / np.abs(r["hitR"])
        dphi = np.abs(e["hitPhi"].astype(np.float64) - r["hitPhi"])
    dphi = np.minimum(dphi, 1.0 - dphi)
    ddir = np.linalg.norm(e["dir"].astype(np.float64) - r["dir"], axis=1)
    per_ray[both_hit] = np.maximum(dr, dphi)[both_hit]
    per_ray[both_sky] = np.maximum(per_ray[both_sky], ddir[both_sky])
    return per_ray, both_hit | both_sky, (dr[both_hit], dphi[both_hit], ddir[both_sky])


def endpoint_error(e: np.ndarray, r: np.ndarray, img: np.ndarray, img_ref: np.ndarray) -> dict:
    """The share of comparable rays within 1e-4, of rays that end alike, the quantiles of each endpoint
    quantity, and the pixels' radiance against the other frame's."""
    per_ray, comparable, (dr, dphi, ddir) = ray_errors(e, r)
    lum = img[..., :3].astype(np.float64).sum(-1)
    lum_ref = img_ref[..., :3].astype(np.float64).sum(-1)
    drad = (np.abs(lum - lum_ref) / np.maximum(lum_ref, 1e-3)).ravel()

    def q(a, p):
        return float(np.quantile(a, p)) if len(a) else None

    return {
        "rays_within_1e-4": float(np.mean(per_ray[comparable] <= 1e-4)),
        "same_end_kind": float(np.mean((e["kind"] & 15) == (r["kind"] & 15))),
        "hit_r_rel": {"median": q(dr, .5), "p99": q(dr, .99)},
        "hit_phi_turns": {"median": q(dphi, .5), "p99": q(dphi, .99)},
        "escape_dir": {"median": q(ddir, .5), "p99": q(ddir, .99)},
        "radiance_rel": {"median": q(drad, .5), "p99": q(drad, .99), "pixels_within_1e-3": float(np.mean(drad <= 1e-3))},
    }
