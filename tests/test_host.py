"""The host set-up (artful_gb300/csrc/holeHost.c) against the reference's hole.c, through the golden
fixtures the reference produced: frames, clamps, ISCO, orbit speed bit for bit; the synthetic map
generator against its recorded hash (the same bits on x86 and Arm)."""
import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes


def test_isco_matches_reference(lib, golden):
    meta, _ = golden
    for s, r in zip(meta["isco"]["spins"], meta["isco"]["r"]):
        assert lib.artfCudaIsco(s) == np.float32(r)


def test_isco_known_values(lib):
    # Bardeen, Press & Teukolsky: 6 M at rest, 1 M prograde and 9 M retrograde at the extremes
    assert abs(lib.artfCudaIsco(0.0) - 6.0) < 1e-6
    assert abs(lib.artfCudaIsco(0.9999) - 1.0) < 0.1
    assert abs(lib.artfCudaIsco(-0.9999) - 9.0) < 0.01


def test_orbit_speed_matches_reference(lib, golden):
    meta, _ = golden
    o = meta["orbit"]
    for s, row in zip(o["spins"], o["v"]):
        for r, v in zip(o["radii"], row):
            assert lib.artfCudaOrbitSpeed(s, r) == np.float32(v)


@pytest.mark.parametrize("name", list(scenes.golden_scenes()))
def test_frame_and_clamps_match_reference(lib, golden, name):
    meta, _ = golden
    scene = scenes.golden_scenes()[name]
    frame, _, clamped = scenes.frame(scene)
    rec = meta["views"][name]
    assert bytes(clamped).hex() == rec["clamped_hex"]
    assert bytes(frame).hex() == rec["frame_hex"]


@pytest.mark.parametrize("name", ["c1", "moving_2x2", "retro_edge"])
def test_frame64_agrees_with_frame32(name):
    scene = scenes.golden_scenes()[name]
    f32, f64, _ = scenes.frame(scene)
    for field in capi.FRAME_FIELDS:
        a = np.array(getattr(f32, field), np.float64)
        b = np.array(getattr(f64, field), np.float64)
        assert np.allclose(a, b, rtol=2e-6, atol=2e-6), (field, a, b)


@pytest.mark.parametrize("name", list(scenes.golden_scenes()))
def test_synthetic_map_is_reproducible(lib, golden, name):
    meta, _ = golden
    scene = scenes.golden_scenes()[name]
    _, _, clamped = scenes.frame(scene)
    m = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    assert hashlib.sha256(m.tobytes()).hexdigest() == meta["views"][name]["map_sha256"]


@pytest.mark.parametrize("name", list(scenes.golden_scenes()))
def test_synthetic_map_from_the_oracle_library(golden, name):
    """The CPU arm reads its map from the oracle's library (the same generator source): the same bytes,
    made from the reference's clamped description alone."""
    from oracle import binding
    meta, _ = golden
    scene = scenes.golden_scenes()[name]
    clamped = capi.BlackHoleDesc.from_buffer_copy(bytes.fromhex(meta["views"][name]["clamped_hex"]))
    m = binding.synth_map(clamped.discInner, clamped.discOuter, clamped.spin, scene.seed, scene.emissivity)
    assert hashlib.sha256(m.tobytes()).hexdigest() == meta["views"][name]["map_sha256"]


def test_synthetic_map_contents(lib):
    scene = scenes.config1()
    _, _, d = scenes.frame(scene)
    m = scenes.synth_map(lib, d, 0, 3.0)
    gas = m[:capi.ROWS_AT]
    assert 0.5 <= gas.min() and gas.max() < 1.5
    glow = m[capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT]
    assert glow[0] == pytest.approx(1.0, rel=1e-6)
    # rows are even in 1/r: the last row is the outer radius, so glow there is (outer/inner)^-3
    assert glow[-1] == pytest.approx((d.discOuter / d.discInner) ** -3.0, rel=1e-5)
    assert np.all(np.diff(glow) < 0)
    sky = m[capi.SKY_AT:capi.SKY_AT + capi.SKY_WIDTH * capi.SKY_HEIGHT]
    assert sky.min() == np.float32(.0006)
    total = float((sky - np.float32(.0006)).astype(np.float64).sum())
    assert 5 < total < 400  # 2000 stars, log-uniform in [1e-3, 1]: mean about 0.145
    assert not m[capi.DUST_AT:].any()
    # rows: the reference's orbit rate and heat (hole.c:191-192)
    rows = m[capi.ROWS_AT:capi.ROWS_AT + 2 * capi.MAP_HEIGHT].reshape(-1, 2)
    assert np.all(rows[:, 1] == np.float32(4500.0) / np.float32(6500.0))
    r0 = d.discInner
    assert rows[0, 0] == pytest.approx(1 / (2 * np.pi * (r0 ** 1.5 + d.spin)), rel=1e-6)


def test_set_rings_is_the_reference_disc_glow(lib):
    m = np.zeros(capi.MAP_FLOATS, np.float32)
    lib.artfCudaSetRings(m.ctypes.data, 3.0, 30.0, 0.5)
    glow = m[capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT]
    assert glow[0] == pytest.approx(6.0)
    assert glow[-1] == pytest.approx(6 * 10 ** 1.5, rel=1e-5)


def test_frame_rejects_bad_sizes(lib):
    scene = scenes.config1()
    d = scenes.clamp(scene.desc)
    f = capi.HoleFrame()
    assert lib.artfCudaHoleFrame(C.byref(scene.camera), C.byref(d), 0.0, 0, 10, C.byref(f)) == 0
    assert lib.artfCudaHoleFrame(None, C.byref(d), 0.0, 10, 10, C.byref(f)) == 0
