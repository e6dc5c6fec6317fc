"""Python access to the oracle (oracle/liboracle.so) and, where it has been built from the reference's
sources, to the reference itself (oracle/_ref/libartref.so).  Test infrastructure: only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, to check results and to time the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libartref.so")

MAP_FLOATS = 2887424
FLUID_FLOATS = 1024 * 256


class OracleEnd(C.Structure):
    _fields_ = [("hitR", C.c_float), ("hitPhi", C.c_float), ("dir", C.c_float * 3), ("mino", C.c_float),
                ("steps", C.c_uint16), ("crossings", C.c_uint8), ("kind", C.c_uint8),
                ("fp64Steps", C.c_uint16), ("reserved", C.c_uint16)]


FRAME_FIELDS = ("er", "etheta", "ephi", "right", "up", "forward", "metric", "place", "spin", "flow", "boost", "disc",
                "look", "image")


class Frame64(C.Structure):
    """The frame's fields in double (oracle.h OracleFrame64)."""
    _fields_ = [(n, C.c_double * 4) for n in FRAME_FIELDS]


def widened(frame, shift=(0.0, 0.0)) -> Frame64:
    """The FP32 frame's fields in double, the same values: what an FP64 trace of the reference's own rays
    starts from.  shift moves every ray's image position by (dx, dy) (forward += dx right + dy up)."""
    w = Frame64()
    for n in FRAME_FIELDS:
        src, dst = getattr(frame, n), getattr(w, n)
        for k in range(4):
            dst[k] = float(src[k])
    for k in range(3):
        w.forward[k] += shift[0] * w.right[k] + shift[1] * w.up[k]
    return w


class SynthDesc(C.Structure):
    """The synthetic scene's description (include/artful_cuda.h ArtfCudaSynthDesc)."""
    _fields_ = [("seed", C.c_uint64), ("inner", C.c_float), ("outer", C.c_float), ("spin", C.c_float),
                ("emissivity", C.c_float), ("stars", C.c_int)]


class OracleOptions(C.Structure):
    _fields_ = [("stepScale", C.c_float)]


END_DTYPE = np.dtype([("hitR", "<f4"), ("hitPhi", "<f4"), ("dir", "<f4", (3,)), ("mino", "<f4"),
                      ("steps", "<u2"), ("crossings", "u1"), ("kind", "u1"), ("fp64Steps", "<u2"),
                      ("reserved", "<u2")])
assert END_DTYPE.itemsize == C.sizeof(OracleEnd) == 32


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_LIB


_oracle = None


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        vp = C.c_void_p
        lib.oracleTrace32.argtypes = [vp, vp, vp, C.POINTER(OracleOptions), C.c_int, vp, vp, vp, vp, vp]
        lib.oracleTrace64.argtypes = [vp, vp, vp, C.POINTER(OracleOptions), C.c_int, vp, vp, vp, vp, vp]
        lib.oracleRender32.argtypes = [vp, vp, vp, C.POINTER(OracleOptions), C.c_int, C.c_uint32, C.c_int, C.c_int,
                                       C.c_int, vp, vp]
        lib.oracleRender64.argtypes = [vp, vp, vp, vp, C.POINTER(OracleOptions), C.c_int, C.c_uint32, C.c_int,
                                       C.c_int, C.c_int, vp, vp]
        lib.oracleJitter.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.oraclePost.argtypes = [vp, vp, vp]
        lib.oracleThreads.restype = C.c_int
        lib.oracleFluidNew.argtypes = [C.c_float, C.c_float, C.c_float, C.c_double]
        lib.oracleFluidNew.restype = vp
        lib.oracleFluidAdvance.argtypes = [vp, C.c_double]
        lib.oracleFluidRead.argtypes = [vp, vp]
        lib.oracleFluidRead.restype = C.c_double
        lib.oracleFluidFree.argtypes = [vp]
        lib.oraclePaintDisc.argtypes = [vp]
        lib.oracleSetRings.argtypes = [vp, C.c_float, C.c_float, C.c_float]
        lib.oracleGasSums.argtypes = [C.c_int, vp, vp]
        lib.artfCudaSynthMap.argtypes = [C.POINTER(SynthDesc), vp]
        lib.artfCudaSynthMap.restype = C.c_int
        _oracle = lib
    return _oracle


class Fluid:
    """The disc fluid of the oracle (prefix "oracle") or of the reference itself (prefix "ref"): made,
    advanced, read (the field as float32 and the moment it is of), freed."""

    def __init__(self, lib, prefix: str, inner: float, outer: float, spin: float, time: float):
        self.lib, self.prefix = lib, prefix
        self.handle = getattr(lib, prefix + "FluidNew")(inner, outer, spin, time)
        if not self.handle:
            raise RuntimeError("fluid allocation failed")

    def advance(self, time: float) -> bool:
        return bool(getattr(self.lib, self.prefix + "FluidAdvance")(self.handle, time))

    def read(self):
        out = np.empty(FLUID_FLOATS, np.float32)
        t = getattr(self.lib, self.prefix + "FluidRead")(self.handle, out.ctypes.data)
        return out, t

    def free(self):
        if self.handle:
            getattr(self.lib, self.prefix + "FluidFree")(self.handle)
            self.handle = None


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def trace32(frame, map_, fluid, nx, ny, time, step_scale=1.0, ends=False):
    """Per-ray FP32 oracle: rgb (n, 3) float32 and, if asked, the endpoint records."""
    nx = np.ascontiguousarray(nx, np.float32)
    ny = np.ascontiguousarray(ny, np.float32)
    time = np.ascontiguousarray(np.broadcast_to(time, nx.shape), np.float32)
    rgb = np.zeros((nx.size, 3), np.float32)
    e = np.zeros(nx.size, END_DTYPE) if ends else None
    oracle().oracleTrace32(C.byref(frame), _ptr(map_), _ptr(fluid), C.byref(OracleOptions(step_scale)), nx.size,
                           _ptr(nx), _ptr(ny), _ptr(time), _ptr(rgb), _ptr(e))
    return (rgb, e) if ends else rgb


def render32(frame, map_, fluid, jitter=0, seed=0, threads=0, rows=None, step_scale=1.0, ends=False):
    """Whole-frame FP32 oracle: (H, W, 4) float32, RGB and the pixel-class bits."""
    w, h = frame.size[0], frame.size[1]
    y0, y1 = rows if rows else (0, h)
    rays = jitter if jitter else frame.size[2] ** 2
    hdr = np.zeros((h, w, 4), np.float32)
    e = np.zeros(w * h * rays, END_DTYPE) if ends else None
    oracle().oracleRender32(C.byref(frame), _ptr(map_), _ptr(fluid), C.byref(OracleOptions(step_scale)), jitter,
                            seed, threads, y0, y1, _ptr(hdr), _ptr(e))
    return (hdr, e) if ends else hdr


def render64(frame, frame64, map_, fluid, jitter=0, seed=0, threads=0, rows=None, step_scale=1.0, ends=False):
    w, h = frame.size[0], frame.size[1]
    y0, y1 = rows if rows else (0, h)
    rays = jitter if jitter else frame.size[2] ** 2
    hdr = np.zeros((h, w, 4), np.float64)
    e = np.zeros(w * h * rays, END_DTYPE) if ends else None
    oracle().oracleRender64(C.byref(frame), C.byref(frame64), _ptr(map_), _ptr(fluid),
                            C.byref(OracleOptions(step_scale)), jitter, seed, threads, y0, y1, _ptr(hdr), _ptr(e))
    return (hdr, e) if ends else hdr


def synth_map(inner: float, outer: float, spin: float, seed: int, emissivity: float, stars: int = 2000):
    """The benchmark's synthetic map for a disc (the library's generator source, built into the oracle's
    library): what the CPU arm reads, with no CUDA library loaded."""
    m = np.zeros(MAP_FLOATS, np.float32)
    status = oracle().artfCudaSynthMap(C.byref(SynthDesc(seed, inner, outer, spin, emissivity, stars)), m.ctypes.data)
    if status != 0:
        raise ValueError("bad synthetic scene")
    return m


def post(frame, hdr):
    """Bloom and tone map of an (H, W, 4) float32 light frame: (H, W) uint32 BGRA."""
    hdr = np.ascontiguousarray(hdr, np.float32)
    out = np.zeros(hdr.shape[:2], np.uint32)
    oracle().oraclePost(C.byref(frame), _ptr(hdr), _ptr(out))
    return out


def jitter_offsets(seed: int, pixel: int, k: int):
    dx, dy = C.c_float(), C.c_float()
    oracle().oracleJitter(seed, pixel, k, C.byref(dx), C.byref(dy))
    return dx.value, dy.value


# ---- the reference itself (only where oracle/_ref was built from its sources) ---------------------

def ref_available() -> bool:
    return os.path.exists(REF_LIB)


_ref = None


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_LIB)
        vp = C.c_void_p
        lib.refFrame.argtypes = [vp, vp, vp]
        lib.refFrame.restype = C.c_uint32
        lib.refMap.argtypes = [vp, vp]
        lib.refFluid.argtypes = [vp, vp]
        lib.refFluid.restype = C.c_double
        lib.refTrace.argtypes = [vp, vp, vp, C.c_int, vp, vp, vp, vp]
        lib.refRender.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        lib.refRender.restype = C.c_double
        lib.refIsco.argtypes = [C.c_float]
        lib.refIsco.restype = C.c_float
        lib.refOrbitSpeed.argtypes = [C.c_float, C.c_float]
        lib.refOrbitSpeed.restype = C.c_float
        lib.refPoolThreads.argtypes = [C.c_int]
        lib.refPoolThreads.restype = C.c_int
        lib.refFluidNew.argtypes = [C.c_float, C.c_float, C.c_float, C.c_double]
        lib.refFluidNew.restype = vp
        lib.refFluidAdvance.argtypes = [vp, C.c_double]
        lib.refFluidRead.argtypes = [vp, vp]
        lib.refFluidRead.restype = C.c_double
        lib.refFluidFree.argtypes = [vp]
        _ref = lib
    return _ref
