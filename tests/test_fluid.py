"""The disc fluid's oracle (no GPU): the restatement of the reference's fluid.c (oracle/fluidOracle.c)
against the golden hashes recorded from the reference, and against the reference itself where it is built
here (oracle/_ref), byte for byte."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from oracle import binding


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def replay(lib, prefix, case):
    """The states of a recorded case, replayed: (stepped, time, field sha256) after the start and each
    advance."""
    fl = binding.Fluid(lib, prefix, case["inner"], case["outer"], case["spin"], case["time"])
    field, t = fl.read()
    states = [(None, t, _sha(field))]
    for s in case["states"][1:]:
        stepped = fl.advance(s["advance_to"])
        field, t = fl.read()
        states.append((stepped, t, _sha(field)))
    fl.free()
    return states


@pytest.mark.parametrize("name", ["a0.9", "a0.998", "a-0.5"])
def test_oracle_fluid_matches_the_reference_bytes(oracle_lib, golden, name):
    meta, arrays = golden
    case = meta["fluid"][name]
    got = replay(oracle_lib, "oracle", case)
    for (stepped, t, sha), want in zip(got, case["states"]):
        assert sha == want["field_sha256"], (name, want["advance_to"])
        assert t == want["time"]
        assert stepped == want["stepped"]


def test_oracle_fluid_row_values(oracle_lib, golden):
    meta, arrays = golden
    case = meta["fluid"]["a0.9"]
    fl = binding.Fluid(oracle_lib, "oracle", case["inner"], case["outer"], case["spin"], case["time"])
    field, _ = fl.read()
    fl.free()
    np.testing.assert_array_equal(field.reshape(256, 1024)[100], arrays["fluid_a0.9_row100"])
    assert np.isfinite(field).all() and field.min() >= 0.0 and field.max() > 0.1


@pytest.mark.skipif(not binding.ref_available(), reason="the reference is not built here")
def test_oracle_fluid_equals_the_reference_live(oracle_lib):
    """A disc the fixtures do not hold: the oracle's field equals the reference's, byte for byte."""
    inner, outer, spin = 1.7, 20.0, 0.6
    a = binding.Fluid(oracle_lib, "oracle", inner, outer, spin, 3.3)
    b = binding.Fluid(binding.ref(), "ref", inner, outer, spin, 3.3)
    for target in (None, 4.1, 9.7):
        if target is not None:
            assert a.advance(target) == b.advance(target)
        fa, ta = a.read()
        fb, tb = b.read()
        assert ta == tb
        np.testing.assert_array_equal(fa.view(np.uint32), fb.view(np.uint32))
    a.free()
    b.free()


# ---- the gas's clock on the host (artfCudaFluidClock) and the scene that keeps it --------------------

def _clock(lib, clock, target):
    import ctypes as C
    c = C.c_double(clock)
    steps = lib.artfCudaFluidClock(C.byref(c), target)
    return steps, c.value


@pytest.mark.parametrize("name", ["a0.9", "a0.998", "a-0.5"])
def test_the_gas_clock_is_the_reference_clock(lib, golden, name):
    """Over each recorded case: the reference's time after every advance, and a step taken exactly when the
    reference's field changed (fluid.c:319-333)."""
    meta, _ = golden
    case = meta["fluid"][name]
    clock = case["states"][0]["time"]
    for state in case["states"][1:]:
        steps, clock = _clock(lib, clock, state["advance_to"])
        assert clock == state["time"], (name, state["advance_to"])
        assert (steps > 0) == state["stepped"]


def test_the_gas_clock_counts_steps(lib):
    assert _clock(lib, 0.0, 0.19) == (0, 0.0)
    steps, clock = _clock(lib, 0.0, 1.0)
    assert steps == 4 or steps == 5
    assert abs(clock - steps * np.float64(np.float32(0.2))) < 1e-12
    steps, clock = _clock(lib, 0.0, 100.0)            # the cap: 48 steps, ending at 100
    assert steps == 48 and abs(clock - 100.0) < 1e-9
    assert _clock(lib, 10.0, 1.5) == (0, 1.5)          # more than 8 back: the clock restarts there
    assert _clock(lib, 10.0, 5.0) == (0, 10.0)         # behind by less than 8: nothing
    assert _clock(lib, 1.0, float("nan")) == (0, 1.0)


@pytest.mark.skipif(not binding.ref_available(), reason="the reference is not built here")
def test_the_gas_clock_against_the_reference_live(lib):
    """Random advances (small ones, so that the reference's gas steps little): the same times."""
    rng = np.random.default_rng(11)
    f = binding.Fluid(binding.ref(), "ref", 2.32, 12.0, 0.9, 1.5)
    clock = 1.5
    try:
        for _ in range(12):
            target = clock + float(rng.choice([-9.0, -0.5, 0.05, 0.21, 0.6, 1.3]))
            stepped = f.advance(target)
            steps, clock = _clock(lib, clock, target)
            assert clock == f.read()[1] and (steps > 0) == stepped
    finally:
        f.free()


def test_scene_keeps_the_reference_gas(lib, golden):
    """The library's scene over the recorded timeline: its gas's clock is the reference scene's fluid time
    after every setting (hole.c:264-270), a new gas starts exactly at each new disc or spin, and the steps
    it counts bring a gas from its start to that clock."""
    import ctypes as C
    from artful_gb300 import capi, scenes
    meta, _ = golden
    want = meta["timeline"]["fluid_times"]
    _, _, steps = scenes.timeline()
    s = lib.artfCudaSceneNew()
    try:
        generations = []
        for (cam, desc, _), t in zip(steps, want):
            lib.artfCudaSceneSetCamera(s, C.byref(cam))
            lib.artfCudaSceneSetBlackHole(s, C.byref(desc))
            inputs = capi.HoleInputs()
            assert lib.artfCudaSceneReadHole(s, C.byref(inputs))
            assert inputs.gasClock == t
            generations.append(inputs.gasGeneration)
            # the count replays: from the start, each step adds 0.2f, unless a cap or a restart of the
            # clock intervened (both in this timeline); at least it never exceeds what the time allows
            assert inputs.gasSteps <= max(0.0, (t - inputs.gasStart) / 0.2 + 48)
        assert generations[0] != 0
        changes = [i for i in range(1, len(generations)) if generations[i] != generations[i - 1]]
        assert changes == [8, 9, 10]   # spin 0.6; outer 16; back to the first disc
    finally:
        lib.artfCudaSceneFree(s)
