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
