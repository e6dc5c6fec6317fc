"""Host side of the gradients (no GPU): scenes from the five parameters, their frames and the Jacobian of
the frame fields that the adjoint and the forward-mode reference chain through, the fit workloads."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

from artful_gb300 import capi, fit


def _fields(f64) -> np.ndarray:
    """The 28 frame fields in the Jacobian's row order."""
    out = []
    for name, n in (("forward", 3), ("right", 3), ("up", 3), ("metric", 4), ("place", 4), ("er", 3), ("etheta", 3),
                    ("ephi", 3)):
        out += list(getattr(f64, name))[:n]
    out += [f64.spin[0], f64.disc[0]]
    return np.array(out)


@pytest.fixture(scope="module")
def start(lib):
    return fit.config4_params()[1]


def test_params_scene(lib, start):
    cam, desc = capi.Camera(), capi.BlackHoleDesc()
    capi.check(lib.artfCudaHoleParamsScene(C.byref(start), C.byref(cam), C.byref(desc)))
    assert cam.position.x == 0.0
    assert cam.position.y == pytest.approx(32.0 * math.cos(math.radians(55.0)), rel=1e-6)
    assert cam.position.z == pytest.approx(32.0 * math.sin(math.radians(55.0)), rel=1e-6)
    assert desc.spin == pytest.approx(0.6, rel=1e-7)
    assert desc.discInner == pytest.approx(1.1 * lib.artfCudaIsco(0.6), rel=1e-6)
    assert desc.discOuter == 12.0 and desc.bloom == 0.0 and desc.samples == 1


def test_jacobian_structure(lib, start):
    f, f64, jac = fit.frames(start, 64, 36)
    assert f.size[0] == 64 and f.size[1] == 36 and f.size[2] == 1
    assert f.boost[3] <= 1.0  # an eye at rest: the adjoint's set-up has no aberration
    np.testing.assert_allclose(jac[26], [1, 0, 0, 0, 0], atol=1e-9)  # d a / d theta
    assert jac[27, 2] == pytest.approx(lib.artfCudaIsco(0.6), rel=1e-6)  # d r_in / d scale = ISCO
    assert jac[27, 0] < 0                                           # the ISCO shrinks as a grows
    np.testing.assert_array_equal(jac[:, 3], 0)                     # q reaches no frame field
    # the eye's basis in its local frame does not move (it looks at the hole); inclination turns the local
    # frame and moves the eye in latitude; distance moves the metric at the eye
    np.testing.assert_allclose(jac[0:9], 0, atol=1e-9)
    assert np.abs(jac[17:26, 1]).max() > 0.1 and abs(jac[16, 1]) > 0.1
    assert np.abs(jac[9:17, 4]).max() > 0.5


def test_jacobian_against_wider_differences(lib, start):
    """The Jacobian (central differences of step 1e-6) against differences of step 1e-4: the same to the
    truncation error of the wider step."""
    _, _, jac = fit.frames(start, 64, 36)
    theta = fit.theta_of(start)
    for q in range(5):
        h = 1e-4 * max(1.0, abs(theta[q]))
        up, down = theta.copy(), theta.copy()
        up[q] += h
        down[q] -= h
        fu = _fields(fit.frames(fit.with_theta(start, up), 64, 36)[1])
        fd = _fields(fit.frames(fit.with_theta(start, down), 64, 36)[1])
        np.testing.assert_allclose(jac[:, q], (fu - fd) / (2 * h), rtol=1e-5, atol=1e-7)


def test_params_map_rings(lib, start):
    """The map of a parameter scene: glow (r / r_in)^-q and orbit speed 1 / (2 pi (r^1.5 + a)) by row."""
    m = fit.param_map(start)
    cam, desc = capi.Camera(), capi.BlackHoleDesc()
    capi.check(lib.artfCudaHoleParamsScene(C.byref(start), C.byref(cam), C.byref(desc)))
    inner, outer = float(desc.discInner), float(desc.discOuter)
    rho = np.arange(capi.MAP_HEIGHT) / (capi.MAP_HEIGHT - 1)
    r = inner / (1.0 - rho * (1.0 - inner / outer))
    glow = m[capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT]
    np.testing.assert_allclose(glow, (r / inner) ** -start.emissivity, rtol=2e-6)
    speed = m[capi.ROWS_AT:capi.ROWS_AT + 2 * capi.MAP_HEIGHT:2]
    np.testing.assert_allclose(speed, 1.0 / (2 * np.pi * (r ** 1.5 + float(desc.spin))), rtol=2e-6)


def test_params_rejects_bad_scenes(lib, start):
    f, f64 = capi.HoleFrame(), capi.HoleFrame64()
    assert lib.artfCudaHoleParamsFrames(None, 64, 36, C.byref(f), C.byref(f64), None) != 0
    assert lib.artfCudaHoleParamsMap(C.byref(start), None) != 0
    theta = fit.theta_of(start)
    for q, bad in ((0, 1.2), (0, float("nan")), (1, -0.1), (2, 0.0), (2, 20.0), (4, 2.0)):
        t = theta.copy()
        t[q] = bad
        p = fit.with_theta(start, t)
        assert lib.artfCudaHoleParamsFrames(C.byref(p), 64, 36, C.byref(f), C.byref(f64), None) != 0, (q, bad)
        cam, desc = capi.Camera(), capi.BlackHoleDesc()
        assert lib.artfCudaHoleParamsScene(C.byref(p), C.byref(cam), C.byref(desc)) != 0


def test_fit_workloads():
    target, start = fit.config4_params()
    np.testing.assert_allclose(fit.theta_of(target), [0.7, math.radians(60), 1.0, 3.0, 30.0])
    np.testing.assert_allclose(fit.theta_of(start), [0.6, math.radians(55), 1.1, 2.7, 32.0])
    fits = fit.config5_fits()
    assert len(fits) == 32
    for t, s in fits:
        tt, ss = fit.theta_of(t), fit.theta_of(s)
        assert 0.1 <= tt[0] <= 0.99 and math.radians(20) <= tt[1] <= math.radians(85) and 1.0 <= tt[2] <= 1.5
        off = np.abs(ss / tt - 1.0)
        # the drawn parameters start 15% off (the spin capped), the emissivity index and distance on target
        assert np.all(np.abs(off[1:3] - 0.15) < 1e-12) and np.all(off[3:] == 0.0)
        assert ss[0] <= fit.SPIN_LIMIT
    again = fit.config5_fits()
    assert all(np.array_equal(fit.theta_of(a[1]), fit.theta_of(b[1])) for a, b in zip(fits, again))
    every = fit.config5_fits(offset=range(5))
    for (t, s), (t3, _) in zip(every, fits):
        tt, ss = fit.theta_of(t), fit.theta_of(s)
        assert np.array_equal(tt, fit.theta_of(t3))  # the same targets either way
        assert np.all(np.abs(np.abs(ss / tt - 1.0)[1:] - 0.15) < 1e-12)


def test_projection_keeps_scenes_valid():
    theta = np.array([[1.5, -0.2, 0.1, 3.0, 1.0]])
    kept = fit.project(theta)
    assert kept[0, 0] == fit.SPIN_LIMIT and kept[0, 1] > 0 and kept[0, 2] == 0.5 and kept[0, 4] == 4.0
