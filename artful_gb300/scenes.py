"""The synthetic workloads, seeded: the views of the benchmark configurations and of the parity tests,
built through the C ABI's host set-up (the clamps, the synthetic map) so that every caller (tests,
bench.py, the golden-fixture script) traces the same inputs.

Geometry for all of them: the hole's axis +y, the eye at r_obs (0, cos i, sin i) looking at the hole
with +y up, a pinhole of vertical field 0.6 rad; a geometrically thin disc (height 1e-3, the
reference's floor) from the ISCO to 12 M with emissivity r^-q, and a sky of 2000 seeded stars.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math

import numpy as np

from . import capi


@dataclasses.dataclass
class Scene:
    name: str
    desc: capi.BlackHoleDesc
    camera: capi.Camera
    width: int
    height: int
    seed: int = 0            # of the synthetic map
    emissivity: float = 3.0  # q
    jitter: int = 0          # 0: the reference's stratified samples; n: n jittered rays a pixel
    jitter_seed: int = 0
    whole: bool = False      # golden: record the whole frame
    classes: bool = False    # golden: record the pixel classes


def hole_desc(spin: float, inner: float = 0.0, outer: float = 12.0, doppler: float = 1.0, stars: float = 1.0,
              samples: int = 1, shutter: float = 0.0, time: float = 0.0, velocity=(0.0, 0.0, 0.0),
              height: float = 1e-3) -> capi.BlackHoleDesc:
    d = capi.load().artfCudaBlackHoleDefaults()
    d.axis = capi.Vec3(0.0, 1.0, 0.0)
    d.spin = spin
    d.discInner = inner
    d.discOuter = outer
    d.discHeight = height
    d.doppler = doppler
    d.stars = stars
    d.bloom = 0.0
    d.samples = samples
    d.shutter = shutter
    d.time = time
    d.velocity = capi.Vec3(*velocity)
    return d


def camera(inclination_deg: float, r_obs: float, fov: float = 0.6) -> capi.Camera:
    i = math.radians(inclination_deg)
    return capi.Camera(capi.Vec3(0.0, r_obs * math.cos(i), r_obs * math.sin(i)), capi.Vec3(0.0, 0.0, 0.0),
                       capi.Vec3(0.0, 1.0, 0.0), fov, 0.1)


def clamp(desc: capi.BlackHoleDesc) -> capi.BlackHoleDesc:
    out = capi.BlackHoleDesc()
    capi.load().artfCudaHoleClamp(C.byref(desc), C.byref(out))
    return out


def frame(scene: Scene, fluid_time: float | None = None):
    """The FP32 and FP64 frames of a scene, and its clamped description.  The fluid's moment defaults to
    the description's time: what a fluid started for this disc at that time holds (fluid.c:255-316)."""
    lib = capi.load()
    d = clamp(scene.desc)
    if fluid_time is None:
        fluid_time = float(d.time)
    f = capi.HoleFrame()
    if lib.artfCudaHoleFrame(C.byref(scene.camera), C.byref(d), fluid_time, scene.width, scene.height,
                             C.byref(f)) == 0:
        raise ValueError("bad frame arguments")
    f64 = capi.HoleFrame64()
    capi.check(lib.artfCudaHoleFrame64(C.byref(scene.camera), C.byref(d), fluid_time, scene.width, scene.height,
                                       C.byref(f64)))
    return f, f64, d


def synth_map(lib, clamped: capi.BlackHoleDesc, seed: int, emissivity: float, stars: int = 2000) -> np.ndarray:
    m = np.zeros(capi.MAP_FLOATS, np.float32)
    sd = capi.SynthDesc(seed, clamped.discInner, clamped.discOuter, clamped.spin, emissivity, stars)
    capi.check(lib.artfCudaSynthMap(C.byref(sd), m.ctypes.data))
    return m


def unit_fluid() -> np.ndarray:
    """A fluid field of 1 everywhere: the disc's density is then the map's alone (0.9 + 0.1 * 1)."""
    return np.ones(capi.FLUID_FLOATS, np.float32)


def config1() -> Scene:
    """Plain method, small: a = 0.9, r_obs = 30, i = 80 deg, 320 x 180, one ray at each pixel centre."""
    return Scene("c1", hole_desc(0.9), camera(80.0, 30.0), 320, 180, seed=0, emissivity=3.0, whole=True,
                 classes=True)


def config2(jitter: int = 4) -> Scene:
    """Mixed precision at scale: a = 0.998, r_obs = 50, i = 85 deg, 1920 x 1080, 4 jittered rays a pixel."""
    return Scene("c2", hole_desc(0.998), camera(85.0, 50.0), 1920, 1080, seed=1, emissivity=3.0, jitter=jitter,
                 jitter_seed=1)


def config3_views(count: int = 64, seed: int = 2):
    """Batched uneven views: resolution, spin, inclination and distance drawn from seed 2."""
    rng = np.random.default_rng(seed)
    views = []
    for k in range(count):
        w = int(rng.integers(128, 1281)) & ~15
        w = max(w, 128)
        h = w * 9 // 16
        spin = float(rng.uniform(0.0, 0.998))
        incl = float(rng.uniform(5.0, 89.0))
        r_obs = float(rng.uniform(20.0, 80.0))
        views.append(Scene(f"c3_{k}", hole_desc(spin), camera(incl, r_obs), w, h, seed=seed, emissivity=3.0))
    return views


def config4_target() -> Scene:
    return Scene("c4_target", hole_desc(0.7), camera(60.0, 30.0), 512, 288, seed=4, emissivity=3.0)


def config4_start() -> Scene:
    isco = capi.load().artfCudaIsco(0.6)
    return Scene("c4_start", hole_desc(0.6, inner=1.1 * isco), camera(55.0, 32.0), 512, 288, seed=4,
                 emissivity=2.7)


def timeline():
    """A hole over time as an application animates one: its description set every frame, a frame drawn
    after most.  The gas takes single steps, two settings come between two draws, a jump hits the 48-step
    cap, the clock falls behind the gas and then far back (the gas's clock restarts there), the spin
    changes (the disc repainted, a new gas), then the disc, then both come back, and the camera moves.
    Returns (width, height, [(camera, clamped-before description, draw after it)])."""
    def at(t, spin=0.9, outer=12.0, bloom=4.5):
        d = hole_desc(spin, outer=outer, time=t)
        d.bloom = bloom
        return d
    near, far = camera(80.0, 30.0), camera(72.0, 34.0)
    steps = [(near, at(0.0), True), (near, at(0.1), True), (near, at(1.05), False), (near, at(2.3), True),
             (near, at(30.0), True), (near, at(29.0), True), (near, at(5.0), True), (near, at(5.5), True),
             (near, at(6.0, spin=0.6), True), (near, at(6.4, spin=0.6, outer=16.0), True),
             (near, at(7.0), True), (far, at(7.3), True), (far, at(7.35), False), (far, at(9.0), True)]
    return 160, 90, steps


def golden_scenes():
    """The views whose reference outputs are recorded in tests/golden/."""
    c1 = config1()
    scenes = {
        "c1": c1,
        "c2": Scene("c2", hole_desc(0.998), camera(85.0, 50.0), 1920, 1080, seed=1),
        "c4_target": config4_target(),
        "c4_start": config4_start(),
        "odd_101x67": Scene("odd_101x67", hole_desc(0.9), camera(80.0, 30.0), 101, 67, seed=0, whole=True),
        "odd_3x2": Scene("odd_3x2", hole_desc(0.9), camera(80.0, 30.0), 3, 2, seed=0, whole=True),
        "odd_1x1": Scene("odd_1x1", hole_desc(0.9), camera(80.0, 30.0), 1, 1, seed=0, whole=True),
        "moving_2x2": Scene("moving_2x2", hole_desc(0.6, samples=2, shutter=3.0, time=7.0, velocity=(0.3, 0.0, 0.1),
                                                    doppler=0.6),
                            camera(70.0, 26.0), 96, 64, seed=5, emissivity=2.5, whole=True),
        "retro_edge": Scene("retro_edge", hole_desc(-0.5, doppler=0.0), camera(89.5, 20.0), 80, 45, seed=6,
                            emissivity=2.0, whole=True),
        "spinless_3x3": Scene("spinless_3x3", hole_desc(0.0, samples=3, outer=20.0), camera(30.0, 14.0), 40, 30,
                              seed=7, whole=True),
    }
    return scenes
