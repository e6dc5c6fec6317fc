"""Generates the golden fixtures of tests/golden/ from the reference renderer itself.

It needs the reference built from its own sources (`make -f oracle/ref.mk`, which reads the reference
checkout) and the product library (for the synthetic map generator, whose output is pinned here by
its hash).  Everything recorded is the reference's output: frames from hole.c:273 artfHoleFrame,
clamped descriptions from hole.c:242, rays from lens.inc:99 lensTrace, whole frames from the tile
loop lens.inc:355 (through the reference's thread pool), pixel classes from three renders of the
same view (normal, stars 0, disc gain 0: the disc-only and the sky-only light).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from artful_gb300 import capi  # noqa: E402
from oracle import binding  # noqa: E402
from artful_gb300 import scenes  # noqa: E402


class RefView(C.Structure):
    _fields_ = [("camera", capi.Camera), ("desc", capi.BlackHoleDesc), ("width", C.c_int), ("height", C.c_int)]


def ref_frame(ref, scene):
    v = RefView(scene.camera, scene.desc, scene.width, scene.height)
    frame, clamped = capi.HoleFrame(), capi.BlackHoleDesc()
    ref.refFrame(C.byref(v), C.byref(frame), C.byref(clamped))
    return frame, clamped


def aligned(n):
    raw = np.zeros(n + 16, np.float32)
    off = (-raw.ctypes.data % 64) // 4
    return raw[off:off + n]


def ref_render(ref, frame, map_, fluid):
    w, h = frame.size[0], frame.size[1]
    stride = (w + 7) & ~7
    planes = [aligned(stride * h) for _ in range(3)]
    ref.refRender(C.byref(frame), map_.ctypes.data, fluid.ctypes.data, 0, 0, 1, *[p.ctypes.data for p in planes])
    return np.stack([p.reshape(h, stride)[:, :w] for p in planes], -1).copy()


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def draw_cases():
    """Views drawn whole through the reference's renderer: (name, scene, bloom, exposure)."""
    g = scenes.golden_scenes()
    return [("c1_bloom", g["c1"], 4.5, 1.0), ("c1_dim", g["c1"], 1.0, 0.3),
            ("moving_2x2_bloom", g["moving_2x2"], 2.0, 1.5), ("odd_101x67_bloom", g["odd_101x67"], 4.5, 1.0),
            ("odd_3x2", g["odd_3x2"], 4.5, 1.0), ("spinless_3x3_bloom", g["spinless_3x3"], 3.0, 2.0)]


def fluid_cases():
    """Discs whose fluid is recorded (name, spin, start time, the moments it is advanced to in turn): the
    inner edge at the ISCO, the outer at 12.  The moments cover a step, several, the 48-step cap, a clock
    behind the gas (no step) and one set far back (the gas restarts its clock there)."""
    return [("a0.9", 0.9, 0.0, [1.0, 3.05, 20.0, 19.9, 5.0, 6.0]),
            ("a0.998", 0.998, 7.0, [7.8, 10.0, 27.0]),
            ("a-0.5", -0.5, 0.0, [0.6])]


def main():
    if not binding.ref_available():
        sys.exit("the reference is not built: make -f oracle/ref.mk")
    ref = binding.ref()
    lib = capi.load()
    out = {"views": {}, "isco": {}, "orbit": {}}
    arrays = {}
    rng = np.random.default_rng(20261203)

    # ISCO and orbit speed (hole.c:207, 215)
    spins = np.linspace(-.998, .998, 25).astype(np.float32)
    out["isco"] = {"spins": spins.tolist(), "r": [float(ref.refIsco(float(s))) for s in spins]}
    radii = np.array([2.5, 4., 7., 12., 40.], np.float32)
    out["orbit"] = {"spins": spins[::4].tolist(), "radii": radii.tolist(),
                    "v": [[float(ref.refOrbitSpeed(float(s), float(r))) for r in radii] for s in spins[::4]]}

    for name, scene in scenes.golden_scenes().items():
        frame, clamped = ref_frame(ref, scene)
        map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
        fluid = scenes.unit_fluid()
        rec = {"frame_hex": bytes(frame).hex(), "clamped_hex": bytes(clamped).hex(),
               "map_sha256": sha(map_), "synth": {"seed": scene.seed, "emissivity": scene.emissivity}}
        # rays at random image positions, eight at one moment (the harness traces eight lanes at a time)
        n = 1024
        nx = rng.uniform(-1.05, 1.05, n).astype(np.float32)
        ny = rng.uniform(-1.05, 1.05, n).astype(np.float32)
        t = np.repeat(rng.uniform(0, 5, n // 8).astype(np.float32), 8) if scene.desc.shutter else \
            np.full(n, scene.desc.time, np.float32)
        rgb = np.zeros((n, 3), np.float32)
        ref.refTrace(C.byref(frame), map_.ctypes.data, fluid.ctypes.data, n, nx.ctypes.data, ny.ctypes.data,
                     t.ctypes.data, rgb.ctypes.data)
        arrays[f"{name}_rays"] = np.stack([nx, ny, t], -1)
        arrays[f"{name}_rgb"] = rgb
        if scene.whole:
            hdr = ref_render(ref, frame, map_, fluid)
            rec["hdr_sha256"] = sha(hdr)
            rec["hdr_sum"] = float(hdr.astype(np.float64).sum())
            if hdr.size <= 120000:
                arrays[f"{name}_hdr"] = hdr
            if scene.classes:
                # the disc-only and the sky-only light, for the pixel classes
                d = capi.BlackHoleDesc.from_buffer_copy(scene.desc)
                d.stars = 0.
                only_disc, _ = ref_frame(ref, scenes.Scene(**{**scene.__dict__, "desc": d}))
                d = capi.BlackHoleDesc.from_buffer_copy(scene.desc)
                d.discGain = 0.
                only_sky, _ = ref_frame(ref, scenes.Scene(**{**scene.__dict__, "desc": d}))
                disc = ref_render(ref, only_disc, map_, fluid).max(-1) > 0
                sky = ref_render(ref, only_sky, map_, fluid).max(-1) > 0
                classes = np.where(disc, 1, np.where(sky, 2, 0)).astype(np.uint8)
                arrays[f"{name}_classes"] = classes
        out["views"][name] = rec
        print(name, rec.get("hdr_sha256", "")[:16], rec["map_sha256"][:16])

    # jittered rays of the 1080p configuration (four a pixel at seeded offsets), two rows
    scene = scenes.config2(1)
    frame, clamped = ref_frame(ref, scene)
    map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    fluid = scenes.unit_fluid()
    rows = [300, 541]
    nx, ny, t = [], [], []
    for y in rows:
        for x in range(scene.width):
            for k in range(4):
                dx, dy = binding.jitter_offsets(scene.jitter_seed, y * scene.width + x, k)
                nx.append(np.float32((np.float32(x) + np.float32(dx)) * frame.image[1] - np.float32(1)))
                ny.append(np.float32(np.float32(1) - (np.float32(y) + np.float32(dy)) * frame.image[2]))
    nx = np.array(nx, np.float32)
    ny = np.array(ny, np.float32)
    t = np.zeros(nx.size, np.float32)
    rgb = np.zeros((nx.size, 3), np.float32)
    ref.refTrace(C.byref(frame), map_.ctypes.data, fluid.ctypes.data, nx.size, nx.ctypes.data, ny.ctypes.data,
                 t.ctypes.data, rgb.ctypes.data)
    rgb = rgb.reshape(len(rows), scene.width, 4, 3)
    pix = np.zeros((len(rows), scene.width, 3), np.float32)
    for k in range(4):
        pix = pix + rgb[:, :, k]
    pix = pix * np.float32(.25)
    arrays["c2_rows"] = pix
    out["c2_rows"] = {"rows": rows, "frame_hex": bytes(frame).hex(), "map_sha256": sha(map_)}

    # whole BGRA frames from the reference's software renderer (artfRendererNew / Draw / ReadPixels),
    # bloom and tone map included, for a scene holding only the hole, with the synthetic map in place
    ref.refDraw.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    out["draw"] = {}
    for name, view, bloom, exposure in draw_cases():
        d = capi.BlackHoleDesc.from_buffer_copy(view.desc)
        d.bloom, d.exposure = bloom, exposure
        view = scenes.Scene(**{**view.__dict__, "desc": d})
        frame, clamped = ref_frame(ref, view)
        map_ = scenes.synth_map(lib, clamped, view.seed, view.emissivity)
        bgra = np.zeros((view.height, view.width), np.uint32)
        v = RefView(view.camera, d, view.width, view.height)
        fluid = scenes.unit_fluid()  # (kept alive across the call)
        ref.refDraw(C.byref(v), map_.ctypes.data, fluid.ctypes.data, 0, bgra.ctypes.data)
        out["draw"][name] = {"bgra_sha256": sha(bgra), "bloom": bloom, "exposure": exposure, "base": view.name}
        if bgra.size <= 40000:
            arrays[f"draw_{name}"] = bgra
        print("draw", name, sha(bgra)[:16])

    # the reference's painted disc map (hole.c:136-197 buildDisc and setRings) for some discs
    out["painted"] = {}
    for name in ("c1", "retro_edge", "spinless_3x3"):
        view = scenes.golden_scenes()[name]
        v = RefView(view.camera, view.desc, view.width, view.height)
        frame, clamped = ref_frame(ref, view)
        painted = np.zeros(capi.MAP_FLOATS, np.float32)
        ref.refMap(C.byref(v), painted.ctypes.data)
        out["painted"][name] = {"inner": float(clamped.discInner), "outer": float(clamped.discOuter),
                                "spin": float(clamped.spin), "map_sha256": sha(painted)}
        print("painted", name, sha(painted)[:16])

    # the reference's disc fluid (fluid.c): its field's bytes after its start and after each advance
    out["fluid"] = {}
    for name, spin, t0, times in fluid_cases():
        inner = float(lib.artfCudaIsco(spin))
        fl = binding.Fluid(ref, "ref", inner, 12.0, spin, t0)
        field, t = fl.read()
        states = [{"advance_to": None, "stepped": None, "time": t, "field_sha256": sha(field)}]
        arrays[f"fluid_{name}_row100"] = field.reshape(256, 1024)[100].copy()
        for target in times:
            stepped = fl.advance(target)
            field, t = fl.read()
            states.append({"advance_to": target, "stepped": stepped, "time": t, "field_sha256": sha(field)})
        fl.free()
        out["fluid"][name] = {"inner": inner, "outer": 12.0, "spin": spin, "time": t0, "states": states}
        print("fluid", name, [s["field_sha256"][:12] for s in states])

    # the reference's own scene over time (hole.c:242-271: its painted disc, its gas started and advanced
    # by artfSceneSetBlackHole), drawn by its software renderer after the marked settings
    ref.refDrawScene.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    width, height, steps = scenes.timeline()
    views = (RefView * len(steps))(*[RefView(cam, d, width, height) for cam, d, _ in steps])
    marks = np.array([int(draw) for _, _, draw in steps], np.int32)
    frames = np.zeros((int(marks.sum()), height, width), np.uint32)
    times = np.zeros(len(steps), np.float64)
    ref.refDrawScene(views, marks.ctypes.data, len(steps), 0, frames.ctypes.data, times.ctypes.data)
    out["timeline"] = {"width": width, "height": height, "fluid_times": times.tolist(),
                       "bgra_sha256": [sha(f) for f in frames]}
    arrays["timeline_last"] = frames[-1]
    print("timeline", [sha(f)[:8] for f in frames])

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.npz"))


if __name__ == "__main__":
    main()
