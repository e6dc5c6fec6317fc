"""The oracle against the reference: the golden fixtures (the reference's own outputs) bit for bit,
and, where oracle/_ref was built from the reference's sources, the reference live on fresh random
rays with its own painted disc and fluid."""
import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from oracle import binding


def _inputs(lib, name):
    scene = scenes.golden_scenes()[name]
    frame, frame64, clamped = scenes.frame(scene)
    return scene, frame, frame64, scenes.synth_map(lib, clamped, scene.seed, scene.emissivity), scenes.unit_fluid()


@pytest.mark.parametrize("name", list(scenes.golden_scenes()))
def test_oracle_rays_bit_exact(lib, oracle_lib, golden, name):
    _, arrays = golden
    scene, frame, _, m, fluid = _inputs(lib, name)
    rays = arrays[f"{name}_rays"]
    rgb = binding.trace32(frame, m, fluid, rays[:, 0], rays[:, 1], rays[:, 2])
    want = arrays[f"{name}_rgb"]
    assert np.array_equal(rgb.view(np.uint32), want.view(np.uint32)), np.argwhere(rgb != want)[:5]


@pytest.mark.parametrize("name", [n for n, s in scenes.golden_scenes().items() if s.whole])
def test_oracle_frames_bit_exact(lib, oracle_lib, golden, name):
    meta, arrays = golden
    scene, frame, _, m, fluid = _inputs(lib, name)
    hdr = binding.render32(frame, m, fluid)
    rgb = np.ascontiguousarray(hdr[..., :3])
    assert hashlib.sha256(rgb.tobytes()).hexdigest() == meta["views"][name]["hdr_sha256"]
    if f"{name}_hdr" in arrays:
        assert np.array_equal(rgb, arrays[f"{name}_hdr"])


def test_oracle_pixel_classes_match_reference(lib, oracle_lib, golden):
    _, arrays = golden
    scene, frame, _, m, fluid = _inputs(lib, "c1")
    bits = binding.render32(frame, m, fluid)[..., 3].astype(np.uint32)
    mine = np.where(bits & 1, 1, np.where(bits & 2, 2, 0))
    want = arrays["c1_classes"]
    assert np.mean(mine == want) >= 0.9999, np.mean(mine == want)


def test_oracle_jittered_rows_bit_exact(lib, oracle_lib, golden):
    meta, arrays = golden
    scene = scenes.config2(4)
    frame, _, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    for i, y in enumerate(meta["c2_rows"]["rows"]):
        hdr = binding.render32(frame, m, scenes.unit_fluid(), jitter=4, seed=scene.jitter_seed, rows=(y, y + 1))
        assert np.array_equal(hdr[y, :, :3], arrays["c2_rows"][i])


def _draw_case(name):
    from tests.golden.make_golden import draw_cases
    for case, view, bloom, exposure in draw_cases():
        if case == name:
            d = capi.BlackHoleDesc.from_buffer_copy(view.desc)
            d.bloom, d.exposure = bloom, exposure
            return scenes.Scene(**{**view.__dict__, "desc": d})
    raise KeyError(name)


DRAW_CASES = ["c1_bloom", "c1_dim", "moving_2x2_bloom", "odd_101x67_bloom", "odd_3x2", "spinless_3x3_bloom"]


@pytest.mark.parametrize("name", DRAW_CASES)
def test_oracle_bloom_and_tone_map_match_reference_frames(lib, oracle_lib, golden, name):
    """The whole picture: the oracle's trace, bloom and tone map against the reference renderer's BGRA."""
    meta, arrays = golden
    scene = _draw_case(name)
    frame, _, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    bgra = binding.post(frame, binding.render32(frame, m, scenes.unit_fluid()))
    assert hashlib.sha256(bgra.tobytes()).hexdigest() == meta["draw"][name]["bgra_sha256"]
    if f"draw_{name}" in arrays:
        assert np.array_equal(bgra, arrays[f"draw_{name}"])


def test_oracle_half_step_converges(lib, oracle_lib):
    """The discretisation error of the reference's fixed-step Nystrom: halving the step moves disc hits
    and escape directions far less than a pixel for rays away from the photon ring."""
    scene, frame, frame64, m, fluid = _inputs(lib, "c1")
    rng = np.random.default_rng(3)
    nx = rng.uniform(-1, 1, 4000).astype(np.float32)
    ny = rng.uniform(-1, 1, 4000).astype(np.float32)
    _, e1 = binding.trace32(frame, m, fluid, nx, ny, 0.0, ends=True)
    _, e2 = binding.trace32(frame, m, fluid, nx, ny, 0.0, step_scale=0.5, ends=True)
    sky = ((e1["kind"] & 15) == 1) & ((e2["kind"] & 15) == 1)
    gap = np.linalg.norm(e1["dir"][sky] - e2["dir"][sky], axis=1)
    assert np.median(gap) < 1e-4


@pytest.mark.skipif(not binding.ref_available(), reason="the reference was not built here (oracle/ref.mk)")
def test_oracle_matches_reference_live_with_painted_disc(lib, oracle_lib):
    """The reference's own painted gas (hole.c:136 buildDisc) and fluid (fluid.c), not in the fixtures."""
    from tests.golden.make_golden import RefView
    ref = binding.ref()
    rng = np.random.default_rng(11)
    for spin, incl, dist in [(0.6, 84.0, 26.0), (0.95, 70.0, 15.0), (-0.3, 45.0, 40.0)]:
        scene = scenes.Scene("live", scenes.hole_desc(spin, outer=34.0, stars=0.4, height=0.03),
                             scenes.camera(incl, dist), 256, 144)
        v = RefView(scene.camera, scene.desc, scene.width, scene.height)
        frame = capi.HoleFrame()
        ref.refFrame(C.byref(v), C.byref(frame), None)
        painted = np.zeros(capi.MAP_FLOATS, np.float32)
        ref.refMap(C.byref(v), painted.ctypes.data)
        fluid = np.zeros(capi.FLUID_FLOATS, np.float32)
        ref.refFluid(C.byref(v), fluid.ctypes.data)
        n = 8 * 2000
        nx = rng.uniform(-1, 1, n).astype(np.float32)
        ny = rng.uniform(-1, 1, n).astype(np.float32)
        t = np.repeat(rng.uniform(0, 20, n // 8).astype(np.float32), 8)
        want = np.zeros((n, 3), np.float32)
        ref.refTrace(C.byref(frame), painted.ctypes.data, fluid.ctypes.data, n, nx.ctypes.data, ny.ctypes.data,
                     t.ctypes.data, want.ctypes.data)
        got = binding.trace32(frame, painted, fluid, nx, ny, t)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
