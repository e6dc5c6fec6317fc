"""ctypes view of include/artful_cuda.h: struct layouts and the library's entry points.

The product is the C ABI in libartful_cuda.so; this module only declares it for Python callers (the
tests, bench.py).  Loading fails loudly when the library has not been built: there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libartful_cuda.so")
DEBUG_LIB_PATH = os.path.join(HERE, "libartful_cuda_debug.so")  # the bounds-checked build (build --debug)
ENOMEM = -3
EBOUNDS = -7

MAP_WIDTH, MAP_HEIGHT = 2048, 1024
DUST_WIDTH, DUST_HEIGHT = 1024, 256
FLUID_WIDTH, FLUID_HEIGHT = 1024, 256
COLORS = 256
SKY_WIDTH, SKY_HEIGHT = 1024, 512
ROWS_AT = MAP_WIDTH * MAP_HEIGHT
COLORS_AT = ROWS_AT + MAP_HEIGHT * 2
SKY_AT = COLORS_AT + COLORS * 3
GLOW_AT = SKY_AT + SKY_WIDTH * SKY_HEIGHT
DUST_AT = GLOW_AT + MAP_HEIGHT
MAP_FLOATS = DUST_AT + DUST_WIDTH * DUST_HEIGHT
FLUID_FLOATS = FLUID_WIDTH * FLUID_HEIGHT

EXACT, FP32, FP64, MIXED = 0, 1, 2, 3
PRECISIONS = {"exact": EXACT, "fp32": FP32, "fp64": FP64, "mixed": MIXED}

END_HORIZON, END_SKY, END_OPAQUE, END_CAP, END_LIT = 0, 1, 2, 3, 0x10


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("position", Vec3), ("target", Vec3), ("up", Vec3), ("fovY", C.c_float), ("near_", C.c_float)]


class BlackHoleDesc(C.Structure):
    _fields_ = [("position", Vec3), ("axis", Vec3)] + [
        (n, C.c_float)
        for n in ("mass", "spin", "discInner", "discOuter", "discHeight", "discThickness", "discGain", "doppler",
                  "stars", "bloom", "exposure", "time", "shutter")
    ] + [("velocity", Vec3), ("samples", C.c_int)]


_F4 = C.c_float * 4
_D4 = C.c_double * 4
FRAME_FIELDS = ("er", "etheta", "ephi", "right", "up", "forward", "metric", "place", "spin", "flow", "boost", "disc",
                "look", "image")


class HoleFrame(C.Structure):
    _fields_ = [(n, _F4) for n in FRAME_FIELDS] + [("size", C.c_uint32 * 4), ("bloom", (C.c_uint32 * 4) * 8)]


class HoleFrame64(C.Structure):
    _fields_ = [(n, _D4) for n in FRAME_FIELDS]


class SynthDesc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("inner", C.c_float), ("outer", C.c_float), ("spin", C.c_float),
                ("emissivity", C.c_float), ("stars", C.c_int)]


class TraceOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("jitter", C.c_int), ("seed", C.c_uint32), ("stepScale", C.c_float),
                ("horizonBand", C.c_float), ("blockSize", C.c_int), ("compactEvery", C.c_int),
                ("persistent", C.c_int), ("guards", C.c_uint32), ("fp64Batch", C.c_int),
                ("refillBatch", C.c_int), ("bandRays", C.c_int64), ("order", C.c_int)]


ORDER_HEAVY_FIRST, ORDER_PIXELS = 0, 1
BACKEND = 4  # ARTF_CUDA_BACKEND: Artful's ArtfBackend with this backend appended (artful_cuda_renderer.h)
GUARD_MOTION, GUARD_HORIZON, GUARD_RADIAL, GUARD_POLAR, GUARD_PSI, GUARD_ALL = 1, 2, 4, 8, 16, 31


class RayEnd(C.Structure):
    _fields_ = [("hitR", C.c_float), ("hitPhi", C.c_float), ("dir", C.c_float * 3), ("mino", C.c_float),
                ("steps", C.c_uint16), ("crossings", C.c_uint8), ("kind", C.c_uint8),
                ("fp64Steps", C.c_uint16), ("reserved", C.c_uint16)]


class TraceStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("steps", C.c_uint64), ("crossings", C.c_uint64), ("escapes", C.c_uint64),
                ("fp64Steps", C.c_uint64), ("fp64Horizon", C.c_uint64), ("fp64Radial", C.c_uint64),
                ("fp64Polar", C.c_uint64), ("fp64Rounds", C.c_uint64), ("flops", C.c_double), ("ms", C.c_float),
                ("bands", C.c_uint32), ("flops64", C.c_double)]


class View(C.Structure):
    _fields_ = [("frame", HoleFrame), ("frame64", HoleFrame64), ("map", C.c_void_p), ("fluid", C.c_void_p),
                ("hdr", C.c_void_p), ("ends", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("blockSize", C.c_int), ("compactEvery", C.c_int), ("fp64Batch", C.c_int), ("refillBatch", C.c_int),
                ("ms", C.c_float), ("defaultMs", C.c_float), ("trials", C.c_int)]


class HoleParams(C.Structure):
    _fields_ = [(name, C.c_double) for name in ("spin", "inclination", "innerScale", "emissivity", "distance", "fovY",
                                                "outer", "height", "thickness", "gain", "doppler", "stars", "time")] + \
               [("seed", C.c_uint64)]


class AdjointResult(C.Structure):
    _fields_ = [("loss", C.c_double), ("grad", C.c_double * 5)]


GRAD_FIELDS = 28
ADJOINT_MIN_CHECKPOINT, ADJOINT_MAX_CHECKPOINT, ADJOINT_MAX_VIEWS = 1, 64, 1024

assert C.sizeof(HoleFrame) == 368 and C.sizeof(BlackHoleDesc) == 92 and C.sizeof(Camera) == 44
assert C.sizeof(RayEnd) == 32 and C.sizeof(HoleParams) == 112 and C.sizeof(AdjointResult) == 48

P = C.POINTER
_vp = C.c_void_p
_fp = P(C.c_float)

# name: (restype, argtypes)
SIGNATURES = {
    "artfCudaLastError": (C.c_char_p, []),
    "artfCudaBlackHoleDefaults": (BlackHoleDesc, []),
    "artfCudaIsco": (C.c_float, [C.c_float]),
    "artfCudaOrbitSpeed": (C.c_float, [C.c_float, C.c_float]),
    "artfCudaHoleClamp": (None, [P(BlackHoleDesc), P(BlackHoleDesc)]),
    "artfCudaHoleFrame": (C.c_uint32, [P(Camera), P(BlackHoleDesc), C.c_double, C.c_int, C.c_int, P(HoleFrame)]),
    "artfCudaHoleFrame64": (C.c_int, [P(Camera), P(BlackHoleDesc), C.c_double, C.c_int, C.c_int, P(HoleFrame64)]),
    "artfCudaSetRings": (None, [_vp, C.c_float, C.c_float, C.c_float]),
    "artfCudaSynthMap": (C.c_int, [P(SynthDesc), _vp]),
    "artfCudaSynthRings": (None, [P(SynthDesc), _vp]),
    "artfCudaCreate": (C.c_int, [C.c_int, P(_vp)]),
    "artfCudaDestroy": (None, [_vp]),
    "artfCudaSetMap": (C.c_int, [_vp, _vp, C.c_uint64]),
    "artfCudaSetFluid": (C.c_int, [_vp, _vp, C.c_uint64]),
    "artfCudaDeviceMap": (_vp, [_vp]),
    "artfCudaDeviceFluid": (_vp, [_vp]),
    "artfCudaStream": (_vp, [_vp]),
    "artfCudaHoleTrace": (C.c_int, [_vp, P(HoleFrame), P(HoleFrame64), _vp, _vp, P(TraceOptions), _vp, _vp,
                                    P(TraceStats)]),
    "artfCudaHoleRender": (C.c_int, [_vp, P(HoleFrame), P(HoleFrame64), _vp, C.c_uint64, _vp, C.c_uint64,
                                     P(TraceOptions), _vp, P(TraceStats)]),
    "artfCudaHoleTraceRays": (C.c_int, [_vp, P(HoleFrame), P(HoleFrame64), _vp, _vp, C.c_int, C.c_float, C.c_int,
                                        _vp, _vp, _vp, _vp, _vp, P(TraceStats)]),
    "artfCudaProbePeaks": (C.c_int, [_vp, C.c_int, P(C.c_double), P(C.c_double)]),
    "artfCudaCheckConversions": (C.c_int, [_vp, C.c_uint64, P(C.c_uint64)]),
    "artfCudaCheckPairs": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "artfCudaFailAfter": (C.c_int, [_vp, C.c_int]),
    "artfCudaHoleBatch": (C.c_int, [_vp, P(View), C.c_int, P(TraceOptions), P(TraceStats)]),
    "artfCudaBatchGraphCreate": (C.c_int, [_vp, P(View), C.c_int, P(TraceOptions), P(_vp)]),
    "artfCudaBatchGraphUpdate": (C.c_int, [_vp, P(View), C.c_int]),
    "artfCudaBatchGraphLaunch": (C.c_int, [_vp, P(TraceStats)]),
    "artfCudaBatchGraphDestroy": (None, [_vp]),
    "artfCudaAutotune": (C.c_int, [_vp, P(View), C.c_int, P(TraceOptions), P(Tuning)]),
    "artfCudaHoleBatchNoAlloc": (C.c_int, [P(View), C.c_int, P(TraceOptions), _vp, P(TraceStats)]),
    "artfCudaHoleDraw": (C.c_int, [_vp, P(HoleFrame), P(HoleFrame64), _vp, C.c_uint64, _vp, C.c_uint64,
                                   P(TraceOptions), _vp, _vp, P(TraceStats)]),
    "artfCudaPostLaunch": (C.c_int, [P(HoleFrame), _vp, P(_vp), _vp, _vp]),
    # gradients of an image loss in the scene's five parameters
    "artfCudaHoleParamsScene": (C.c_int, [P(HoleParams), P(Camera), P(BlackHoleDesc)]),
    "artfCudaHoleParamsFrames": (C.c_int, [P(HoleParams), C.c_int, C.c_int, P(HoleFrame), P(HoleFrame64), _vp]),
    "artfCudaHoleParamsMap": (C.c_int, [P(HoleParams), _vp]),
    "artfCudaHoleTangents": (C.c_int, [_vp, P(HoleParams), P(HoleFrame), P(HoleFrame64), _vp, _vp, _vp, _vp]),
    "artfCudaHoleAdjoint": (C.c_int, [_vp, P(HoleParams), C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp,
                                      _vp, P(AdjointResult), P(TraceStats)]),
    # the reference's painted disc, made on the GPU
    "artfCudaPaintDisc": (C.c_int, [_vp, _vp, C.c_float, C.c_float, C.c_float]),
    "artfCudaHoleRings": (None, [_vp, _vp, C.c_float, C.c_float, C.c_float]),
    "artfCudaHoleColours": (None, [_vp]),
    # the disc's fluid on the GPU
    "artfCudaFluidNew": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, C.c_double, P(_vp)]),
    "artfCudaFluidAdvance": (C.c_int, [_vp, C.c_double, P(C.c_int)]),
    "artfCudaFluidField": (_vp, [_vp]),
    "artfCudaFluidTime": (C.c_double, [_vp]),
    "artfCudaFluidRead": (C.c_int, [_vp, _vp]),
    "artfCudaFluidFree": (None, [_vp]),
    "artfCudaFluidClock": (C.c_int, [P(C.c_double), C.c_double]),
    "artfCudaFluidStep": (C.c_int, [_vp, C.c_int64, C.c_double]),
    "artfCudaUseFluid": (C.c_int, [_vp, _vp]),
    # the renderer backend (artful_cuda_renderer.h)
    "artfCudaRendererSetDeviceInputs": (None, [_vp, C.c_bool]),
    "artfCudaFrameRead": (C.c_int, [_vp, _vp, _vp]),
    "artfCudaFailAllocAfter": (C.c_int, [_vp, C.c_int]),
    "artfCudaNew": (_vp, [_vp]),
    "artfCudaNewWithReader": (_vp, [_vp, _vp]),
    "artfCudaRendererReadLight": (C.c_bool, [_vp, _vp]),
    "artfCudaRendererSetPrecision": (None, [_vp, C.c_int]),
    "artfCudaRendererContext": (_vp, [_vp]),
    "artfCudaSceneNew": (_vp, []),
    "artfCudaSceneFree": (None, [_vp]),
    "artfCudaSceneSetCamera": (None, [_vp, P(Camera)]),
    "artfCudaSceneSetBlackHole": (None, [_vp, P(BlackHoleDesc)]),
    "artfCudaSceneSetHoleMap": (None, [_vp, _vp, _vp, C.c_double]),
    "artfCudaSceneSetSeed": (None, [_vp, C.c_uint64, C.c_float]),
    "artfCudaSceneReadHole": (C.c_bool, [_vp, _vp]),
}


class Surface(C.Structure):
    _fields_ = [("kind", C.c_int), ("a", C.c_void_p), ("b", C.c_void_p)]


class RendererOptions(C.Structure):
    """Layout of Artful's ArtfRendererOptions (include/artful/renderer.h:51-71)."""
    _fields_ = [("backend", C.c_int), ("surface", Surface), ("width", C.c_int), ("height", C.c_int),
                ("noVsync", C.c_bool), ("threads", C.c_int), ("simd", C.c_int), ("antialias", C.c_bool),
                ("hdr", C.c_bool), ("compressTextures", C.c_bool), ("pipelineCache", C.c_char_p)]


class FrameStats(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("cpuMs", "cullMs", "geometryMs", "rasterMs", "lensMs")] + \
               [(n, C.c_uint32) for n in ("instancesDrawn", "trianglesBinned", "tilesSkipped", "instancesHidden",
                                          "traceSamples")] + [("gpuMs", C.c_double), ("shadowMapsDrawn", C.c_uint32)]


class Overlay(C.Structure):
    _fields_ = [("pixels", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("stride", C.c_int),
                ("partial", C.c_bool), ("damage", C.c_void_p), ("damageCount", C.c_size_t)]


class HoleInputs(C.Structure):
    """What a renderer reads of a scene (artful_cuda_renderer.h ArtfCudaHoleInputs)."""
    _fields_ = [("on", C.c_bool), ("camera", Camera), ("desc", BlackHoleDesc), ("map", C.c_void_p),
                ("mapVersion", C.c_uint64), ("fluid", C.c_void_p), ("fluidVersion", C.c_uint64),
                ("fluidTime", C.c_double), ("gasGeneration", C.c_uint64), ("gasStart", C.c_double),
                ("gasSteps", C.c_uint64), ("gasClock", C.c_double)]


class RendererVtbl(C.Structure):
    """The eight entries of Artful's ArtfRendererVtbl (src/render/rendererInternal.h:7-16)."""
    _fields_ = [("description", C.CFUNCTYPE(C.c_char_p, C.c_void_p)),
                ("resize", C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int)),
                ("setOverlay", C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)),
                ("draw", C.CFUNCTYPE(C.c_bool, C.c_void_p, C.c_void_p)),
                ("readPixels", C.CFUNCTYPE(C.c_bool, C.c_void_p, C.c_void_p)),
                ("pixels", C.CFUNCTYPE(C.c_void_p, C.c_void_p)),
                ("stats", C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)),
                ("destroy", C.CFUNCTYPE(None, C.c_void_p))]


class RendererHead(C.Structure):
    """struct ArtfRenderer's head (src/render/rendererInternal.h:18-27)."""
    _fields_ = [("vt", C.POINTER(RendererVtbl)), ("backend", C.c_int), ("trialFrame", C.c_int),
                ("trialMs", C.c_double * 2)]


assert C.sizeof(RendererOptions) == 64 and C.sizeof(FrameStats) == 80

NOALLOC_MAX_VIEWS = 64

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """The product library, with every declared entry point typed.  Raises when it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError: the library lacks a declared symbol
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, lib=None) -> None:
    if status != 0:
        lib = lib or load()
        msg = lib.artfCudaLastError()
        raise RuntimeError(f"artful_cuda status {status}: {msg.decode() if msg else ''}")
