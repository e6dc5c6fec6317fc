"""The reference's painted disc map (hole.c:136-197 buildDisc and setRings): the oracle's restatement
(oracle/discOracle.c) against the golden hashes recorded from the reference and against the reference
itself where it is built here; the host ring and colour tables against the oracle's.  No GPU."""
from __future__ import annotations

import ctypes as C
import hashlib

import numpy as np
import pytest

from artful_gb300 import capi, scenes
from oracle import binding


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def painted(oracle_lib):
    """The oracle's painted map, without the rings' tables (painting takes a second or two)."""
    m = np.zeros(capi.MAP_FLOATS, np.float32)
    oracle_lib.oraclePaintDisc(m.ctypes.data)
    return m


@pytest.mark.parametrize("name", ["c1", "retro_edge", "spinless_3x3"])
def test_oracle_painted_map_is_the_reference(oracle_lib, golden, painted, name):
    meta, _ = golden
    case = meta["painted"][name]
    m = painted.copy()
    oracle_lib.oracleSetRings(m.ctypes.data, case["inner"], case["outer"], case["spin"])
    assert _sha(m) == case["map_sha256"]


def test_host_tables_are_the_oracle(lib, oracle_lib, golden, painted):
    """The rings' and colours' tables of the host set-up (holeHost.c) that the GPU painter copies in."""
    case = golden[0]["painted"]["c1"]
    m = painted.copy()
    oracle_lib.oracleSetRings(m.ctypes.data, case["inner"], case["outer"], case["spin"])
    rows = np.zeros(capi.MAP_HEIGHT * 2, np.float32)
    glow = np.zeros(capi.MAP_HEIGHT, np.float32)
    colours = np.zeros(capi.COLORS * 3, np.float32)
    lib.artfCudaHoleRings(rows.ctypes.data, glow.ctypes.data, case["inner"], case["outer"], case["spin"])
    lib.artfCudaHoleColours(colours.ctypes.data)
    np.testing.assert_array_equal(rows, m[capi.ROWS_AT:capi.ROWS_AT + capi.MAP_HEIGHT * 2])
    np.testing.assert_array_equal(glow, m[capi.GLOW_AT:capi.GLOW_AT + capi.MAP_HEIGHT])
    np.testing.assert_array_equal(colours, m[capi.COLORS_AT:capi.COLORS_AT + capi.COLORS * 3])


@pytest.mark.skipif(not binding.ref_available(), reason="the reference is not built here")
def test_oracle_painted_map_equals_the_reference_live(oracle_lib, painted):
    """A disc the fixtures do not hold, against the reference's own scene map."""
    class RefView(C.Structure):
        _fields_ = [("camera", capi.Camera), ("desc", capi.BlackHoleDesc), ("width", C.c_int), ("height", C.c_int)]
    desc = scenes.hole_desc(0.3, inner=4.0, outer=17.0)
    v = RefView(scenes.camera(45.0, 25.0), desc, 64, 36)
    want = np.zeros(capi.MAP_FLOATS, np.float32)
    binding.ref().refMap(C.byref(v), want.ctypes.data)
    clamped = scenes.clamp(desc)
    m = painted.copy()
    oracle_lib.oracleSetRings(m.ctypes.data, clamped.discInner, clamped.discOuter, clamped.spin)
    np.testing.assert_array_equal(m.view(np.uint32), want.view(np.uint32))


def test_gas_scale_is_the_same_float_in_the_gpus_order(oracle_lib):
    """The painted gas takes no disc parameter, so its inner-half scale is one number for every disc.
    Its 2^20 float texels add up exactly in double in any order (each has a 24-bit significand, and the
    partial sums never need more than double's 53 bits at these magnitudes): the GPU painter's order
    (1024 runs, strided threads and a tree) and the reference's texel order give the same double, hence
    the same float scale, which lies well away from float's rounding boundary."""
    import ctypes as C
    sums = (C.c_double * 2)()
    scales = (C.c_float * 2)()
    oracle_lib.oracleGasSums(1024, sums, scales)
    assert sums[0] == sums[1] and scales[0] == scales[1]
    texels = 2048 * 512
    q = [texels / sums[0], texels / sums[1]]
    f = np.float32(q[0])
    ulp = float(np.spacing(f))
    margin = min(abs(q[0] - (float(f) - ulp / 2)), abs(q[0] - (float(f) + ulp / 2)))
    assert abs(q[0] - q[1]) * 1e6 < margin, (q, margin)
