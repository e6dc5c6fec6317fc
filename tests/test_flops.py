"""The roofline's algorithmic work: the constants of artful_gb300/csrc/lensFlops.h against an exact count
of the trace's own formulas (tests/flops_count.cpp instantiates lensCore.cuh on the host with an
operation-counting number type).  No GPU."""
from __future__ import annotations

import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "artful_gb300", "csrc")

# The products of the ray's constants each Nystrom sub-step's formulas recompute (lensCore.cuh
# radialStep: a^2, h^2, h/2, h^2/8, h^2/2, h^2/6, h/6; polarStep: the same and 2a^2): computed once a ray.
STEP_INVARIANTS = 7 + 8
PIXEL_SUM = 3   # the ray's light added to its pixel
PLANE_TEST = 1  # n_z n_z' < 0


@pytest.fixture(scope="module")
def counts(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("flops") / "flops_count")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                    os.path.join(ROOT, "tests", "flops_count.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {name: int(value) for name, value in (line.split() for line in out.splitlines())}


@pytest.fixture(scope="module")
def constants():
    text = open(os.path.join(CSRC, "lensFlops.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define ARTF_FLOPS_(\w+) (\d+)", text)}


def test_per_ray(counts, constants):
    assert constants["RAY"] == counts["setup"] + STEP_INVARIANTS + PIXEL_SUM
    assert constants["RAY_SPINLESS"] == counts["setup_spinless"] + STEP_INVARIANTS + PIXEL_SUM


def test_per_step(counts, constants):
    assert constants["STEP"] == counts["step_as_written"] - STEP_INVARIANTS + PLANE_TEST
    assert constants["STEP_SPINLESS"] == counts["step_as_written_spinless"] - STEP_INVARIANTS + PLANE_TEST


def test_per_crossing(counts, constants):
    assert constants["CROSSING"] == counts["crossing"] == counts["crossing_spinless"]
    assert constants["CROSSING_DOPPLER"] == counts["crossing"] - counts["crossing_nodoppler"]


def test_per_escape(counts, constants):
    assert constants["ESCAPE"] == counts["escape"] == counts["escape_spinless"]
    assert constants["SKY"] == counts["sky"] == counts["sky_spinless"]
    # a star drawn in both layers' cells: the most the lower bound leaves out
    assert counts["sky_with_stars"] - counts["sky"] == 63


def test_mixed_fp64_work(counts, constants):
    """The mixed trace's wide work (about FP64's precision: double-float pairs, or FP64 in the horizon's
    band): a ray's set-up with its view's terms given (and its step's terms formed), a whole radial
    sub-step (the horizon's band), the radial motion alone (a turning point of u) and the polar axis
    component alone (a turning point of n_z), with those terms given."""
    assert constants["WIDE_START"] == counts["wide_start"] == counts["wide_start_spinless"]
    assert constants["WIDE_RADIAL"] == counts["wide_radial"]
    assert constants["WIDE_RADIAL_SPINLESS"] == counts["wide_radial_spinless"]
    assert constants["WIDE_TURN"] == counts["wide_turn"] == counts["wide_turn_spinless"]
    assert constants["WIDE_AXIS"] == counts["wide_axis"] == counts["wide_axis_spinless"]
    # each part is a subset of its whole sub-step's operations
    assert counts["wide_axis"] < counts["wide_polar_whole"] and counts["wide_turn"] < counts["wide_radial"]
