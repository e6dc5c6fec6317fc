"""Benchmark of the Kerr hole trace on GB300: geodesics/s at 1080p.

The headline is the mixed-precision trace of the 1920 x 1080, 4-jittered-rays-a-pixel view (a = 0.998,
r_obs = 50 M, i = 85 deg), next to the plain FP64 trace of the same frame (the ratio is the target's
4x), each with its endpoint error against FP64 at half step.  A step is one trace of the whole frame
(8,294,400 geodesics) with the inputs resident in HBM; L2 is flushed (a 256 MB write) before every timed
step, outside the timed region.  `e2e` is the same metric through the host-buffer C ABI call
(artfCudaHoleRender): the map and fluid copied from pinned host memory and the HDR frame copied back,
every step.

Beside it, on rank 0: the 64-view batch (one graph-captured persistent launch, autotuned); the adjoint at
512 x 288 (its time over the forward trace's); and 32 inverse fits of 256 x 144 by Adam on the adjoint's
gradients, with their recovery error and wall time per fit beside the same fit on FP64 central
differences.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--fd-fits F]

--impl reference times the reference's CPU path on this host's cores: the oracle port (the reference's
lensTrace in scalar C, bit for bit; its own sources are not on this machine), with all host threads, on
the same whole frame every step, its inputs made without the CUDA library.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from artful_gb300.endpoint import END_DTYPE, endpoint_error  # noqa: E402  (numpy only: loads no library)

METRIC = "geodesics/s @1080p: mixed-prec vs FP64 GPU at ≤1e-4 endpoint err; adj/fwd time"
UNIT = "geodesics/s"
WORKLOAD = "kerr-hole 1920x1080, 4 jittered rays/px, a=0.998, r_obs=50 M, i=85 deg, disc ISCO..12 M r^-3, 2000 stars"
# Kernels one mixed frame launches: the tile probe, the heavy-first order, the trace, the ray-plane sum.
LAUNCHES_PER_MIXED_FRAME = 4
# DRAM bytes (read + write) of one launch of the mixed trace kernel at this workload, from one ncu
# capture (dram__bytes_read.sum 17.23 MB + dram__bytes_write.sum 73.95 MB): the map read once, and the
# part of the 133 MB of ray planes that leaves L2 before the sum reads it back.
TRACE_TRAFFIC_BYTES = 91_173_120
TRACE_TRAFFIC_GEODESICS = 1920 * 1080 * 4
FLOPS_WIDE_RADIAL = 61  # lensFlops.h: a whole radial sub-step in the horizon's band (spin != 0)
# How busy the mixed trace keeps its pipes, from one ncu --set full capture of its kernel at 960x540 x 4
# (the counted work above counts a double-float operation, some 3 to 10 FP32 instructions, as one): the
# FP64 pipe's instructions, the FP32 FMA pipe's cycles, the integer pipe's instructions and the
# schedulers' issue slots, of peak.
MIXED_PIPES_BUSY = {"fp64": 0.035, "fp32_fma": 0.398, "alu": 0.370, "issue": 0.690,
                    "source": "ncu sm__inst_executed_pipe_fp64, sm__pipe_fma_cycles_active, sm__inst_executed_pipe_alu, "
                              "smsp__issue_active "
                              "of traceMixedQueueOneAll at 960x540 x 4"}
TRACE_TRAFFIC_SOURCE = "ncu dram__bytes of one launch of the mixed trace kernel at 1920x1080 x 4 jittered rays"
# The adjoint's checkpoint interval: 32, a ray's state kept every 32 steps and each segment recomputed in
# the reverse pass; 1, every state kept (48 bytes a step) and nothing recomputed.
ADJOINT_CHECKPOINT = 1


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--quick", action="store_true", help="skip the slow side measurements")
    p.add_argument("--profile", choices=["mixed", "fp64", "exact", "fp32", "adjoint", "frame"],
                   help="trace one frame of that precision (after one untimed one), or run the adjoint twice, "
                        "or draw five of the reference's frames through the backend, and exit: the case for ncu")
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--views", type=int, default=1, help="views of --profile adjoint")
    p.add_argument("--checkpoint", type=int, default=ADJOINT_CHECKPOINT,
                   help="checkpoint interval of --profile adjoint (1: every state kept)")
    p.add_argument("--guards", type=int, default=0,
                   help="the mixed trace's FP64 guards for --profile mixed (ARTF_CUDA_GUARD_* bits; 0: all)")
    p.add_argument("--persistent", action="store_true", help="the persistent form of --profile exact/fp32/fp64")
    p.add_argument("--sweep", action="store_true",
                   help="time the mixed trace's guard, band and batch variants, each with its endpoint error")
    p.add_argument("--fd-fits", type=int, default=4,
                   help="fits of the inverse-fit workload also run with FP64 central-difference gradients")
    p.add_argument("--gradient-bias", type=int, default=0, metavar="FITS",
                   help="compare the adjoint's gradient with FP64 central differences of several steps on the "
                        "first FITS inverse fits, and print the loss along each parameter, then exit")
    return p.parse_args()


def scale_of(p):
    """A parameter point's scale for finite-difference steps: each parameter's size, at least 0.1."""
    from artful_gb300 import fit
    return np.array([max(abs(x), 1e-1) for x in fit.theta_of(p)])


def gradient_bias(args):
    """Why the inverse fits do not recover their parameters.  On the first fits of the configuration-5
    workload (256 x 144, targets from seed 3, starts 15% off): the adjoint's gradient against central
    differences of the FP64 loss at steps of 1e-2 .. 1e-4 of each parameter, at the start and halfway to
    the target (cosine per fit, sign agreement and the ratio of the components); and the FP64 loss along
    the straight line start -> target and along each parameter alone around the target.  One JSON line."""
    import torch
    from artful_gb300 import capi, fit, scenes
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.artfCudaCreate(0, C.byref(ctx)))
    fits = fit.config5_fits(32, seed=3)[:args.gradient_bias]
    m = fit.param_map(fits[0][0])
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    unit = scenes.unit_fluid()
    capi.check(lib.artfCudaSetFluid(ctx, unit.ctypes.data, 0))
    w, h = 256, 144
    adj = fit.Adjoint(lib, ctx, w, h, checkpoint=ADJOINT_CHECKPOINT)
    targets = adj.render([t for t, _ in fits])
    fp64 = fit.Fp64Loss(lib, ctx, w, h, m, lib.artfCudaDeviceFluid(ctx), 10 * len(fits))

    def differences(params, step):
        """Central differences of the FP64 loss, each parameter moved by step times its size."""
        moved, views = [], []
        for k, p in enumerate(params):
            th, sc = fit.theta_of(p), scale_of(p)
            for q in range(5):
                for sign in (1.0, -1.0):
                    t = th.copy()
                    t[q] += sign * step * sc[q]
                    moved.append(fit.with_theta(p, fit.project(t)))
                    views.append(k)
        out = np.empty(len(moved))
        for lo in range(0, len(moved), fp64.capacity):
            idx = torch.tensor(views[lo:lo + fp64.capacity], device="cuda")
            out[lo:lo + len(moved[lo:lo + fp64.capacity])] = fp64.losses(moved[lo:lo + fp64.capacity],
                                                                         targets.index_select(0, idx))
        out = out.reshape(len(params), 5, 2)
        return (out[..., 0] - out[..., 1]) / (2 * step * np.stack([scale_of(p) for p in params]))

    table = {}
    for point in ("start", "halfway"):
        params = [fit.with_theta(s, fit.theta_of(s) if point == "start" else 0.5 * (fit.theta_of(s) + fit.theta_of(t)))
                  for t, s in fits]
        _, g_adj, _ = adj(params, targets)
        sc = np.stack([scale_of(p) for p in params])
        rows = {}
        for step in (1e-2, 3e-3, 1e-3, 1e-4):
            g = differences(params, step)
            cos = [float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30)) for a, b in zip(g_adj, g)]
            with np.errstate(invalid="ignore", divide="ignore"):
                ratio = np.where(np.abs(g * sc) > 1e-12, (g_adj * sc) / (g * sc), np.nan)
            rows[f"{step:g}"] = {
                "median_cosine": float(np.median(cos)),
                "sign_agreement": dict(zip(fit.PARAM_NAMES, np.mean(np.sign(g_adj) == np.sign(g), 0).tolist())),
                "median_ratio": dict(zip(fit.PARAM_NAMES, np.nanmedian(ratio, 0).tolist()))}
        table[point] = rows
    line = []
    for frac in np.linspace(0.0, 1.0, 11):
        params = [fit.with_theta(s, (1 - frac) * fit.theta_of(s) + frac * fit.theta_of(t)) for t, s in fits]
        line.append(float(np.median(fp64.losses(params, targets))))
    alone = {}
    offsets = (-0.15, -0.1, -0.05, -0.02, 0.0, 0.02, 0.05, 0.1, 0.15)
    for q, name in enumerate(fit.PARAM_NAMES):
        row = []
        for frac in offsets:
            params = []
            for t, _ in fits:
                th = fit.theta_of(t).copy()
                th[q] *= 1 + frac
                params.append(fit.with_theta(t, fit.project(th)))
            row.append(float(np.median(fp64.losses(params, targets))))
        alone[name] = row
    print(json.dumps({"gradient_bias": table, "fits": len(fits),
                      "loss_start_to_target_median": line, "loss_alone_offsets": list(offsets),
                      "loss_alone_median": alone, "pixels": pixel_decomposition(adj, fits, targets)}),
          flush=True)
    lib.artfCudaDestroy(ctx)


def pixel_decomposition(adj, fits, targets, step=1e-3, fine=1e-4):
    """Where the adjoint's gradient and the finite differences part, pixel by pixel, at the fits' starts.
    Each pixel's loss (its squared RGB error over 3 x pixels) by the adjoint's own forward renders (FP32,
    the function the adjoint differentiates) at theta +- step and theta +- fine (each times the
    parameter's size).  A pixel is *smooth* in a parameter when its two
    central differences agree within 5 % (the loss is differentiable there at the step's scale), else
    it is *rough*: an edge, a truncated colour or ring row, a class change or a star's tent crossed
    within the step.  Per parameter: the central-difference gradient at `step` summed over all pixels,
    and the share of it on the rough pixels; the adjoint's sum (its per-pixel gradients) over all and
    over the smooth pixels, against the fine differences on the smooth pixels; how many pixels are
    rough."""
    import torch
    from artful_gb300 import fit
    n = len(fits)
    start = [s for _, s in fits]
    h, w = adj.height, adj.width
    grads = torch.zeros((n, h, w, 5), dtype=torch.float32, device="cuda")
    adj(start, targets, pixel_grads=grads)
    grads = grads.double().cpu().numpy()

    def pixel_losses(params):
        """Each pixel's loss, rendered by the adjoint's own forward pass (the function it differentiates)."""
        out = []
        for lo in range(0, len(params), n):
            chunk = params[lo:lo + n]
            d = adj.render(chunk)[..., :3].double() - targets[:len(chunk), ..., :3].double()
            out.append(((d * d).sum(-1) / (3 * h * w)).cpu().numpy())
        return np.concatenate(out)

    def central(q, size):
        moved = []
        for sign in (1.0, -1.0):
            for p in start:
                th = fit.theta_of(p)
                th[q] += sign * size * scale_of(p)[q]
                moved.append(fit.with_theta(p, th))
        lm = pixel_losses(moved)
        sc = np.array([size * scale_of(p)[q] for p in start])[:, None, None]
        return (lm[:n] - lm[n:]) / (2 * sc)

    rows = {}
    for q, name in enumerate(fit.PARAM_NAMES):
        coarse, near = central(q, step), central(q, fine)
        floor = 1e-6 * np.abs(near).max()
        smooth = np.abs(coarse - near) <= 0.05 * np.abs(near) + floor
        g = grads[..., q]
        rows[name] = {
            "fd_all": float(coarse.sum() / n), "fd_share_on_rough_pixels":
                float(np.abs(coarse[~smooth]).sum() / max(np.abs(coarse).sum(), 1e-30)),
            "adjoint_all": float(g.sum() / n), "adjoint_over_fd_all": float(g.sum() / coarse.sum()),
            "adjoint_over_fine_fd_smooth": float(g[smooth].sum() / near[smooth].sum())
            if abs(near[smooth].sum()) > 1e-30 else None,
            "smooth_pixels_within_2pct": float(np.mean(np.abs(g - near)[smooth] <= 0.02 * np.abs(near)[smooth] + floor)),
            "smooth_cosine": float(np.dot(g[smooth], near[smooth]) /
                                   (np.linalg.norm(g[smooth]) * np.linalg.norm(near[smooth]) + 1e-30)),
            "smooth_l1_error": float(np.abs(g - near)[smooth].sum() / max(np.abs(near)[smooth].sum(), 1e-30)),
            "rough_pixels": float(1.0 - smooth.mean())}
    return {"step": step, "fine": fine, "per_parameter": rows}


def sweep(args):
    """One JSON line per variant of the mixed trace: time, FP64 work by reason, endpoint error against
    FP64 at the same step and at half step."""
    import torch
    from artful_gb300 import capi, scenes
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.artfCudaCreate(0, C.byref(ctx)))
    scene = scenes.config2(4)
    frame, frame64, clamped = scenes.frame(scene)
    map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    capi.check(lib.artfCudaSetMap(ctx, map_.ctypes.data, 1))
    unit = scenes.unit_fluid()  # (kept alive across the call: the ABI reads it)
    capi.check(lib.artfCudaSetFluid(ctx, unit.ctypes.data, 1))
    w, h, rays = scene.width, scene.height, 4
    hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ends = torch.empty((w * h * rays * 32,), dtype=torch.uint8, device="cuda")

    def run(opts, with_ends=False, steps=0):
        s = capi.TraceStats()
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(opts),
                                         hdr.data_ptr(), ends.data_ptr() if with_ends else None, C.byref(s)))
        times = []
        for _ in range(steps):
            t = capi.TraceStats()
            capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(opts),
                                             hdr.data_ptr(), None, C.byref(t)))
            times.append(t.ms)
        e = np.frombuffer(ends.cpu().numpy().tobytes(), END_DTYPE).copy() if with_ends else None
        return s, (statistics.median(times) if times else s.ms), e, hdr.cpu().numpy().copy()

    def o(precision, scale=1.0, guards=0, band=0.0, batch=0, wait=0, refill=0, block=0):
        return capi.TraceOptions(precision, rays, scene.jitter_seed, scale, band, block, wait, 1, guards, batch,
                                 refill)

    _, ms64, e64, img64 = run(o(capi.FP64), True, 2)
    _, _, e64h, img64h = run(o(capi.FP64, 0.5), True, 0)
    _, ms32, e32, img32 = run(o(capi.FP32), True, 5)
    print(json.dumps({"variant": "fp64", "ms": ms64}), flush=True)
    print(json.dumps({"variant": "fp32 (no guards at all)", "ms": ms32,
                      "vs_fp64": endpoint_error(e32, e64, img32, img64),
                      "vs_fp64_half": endpoint_error(e32, e64h, img32, img64h)}), flush=True)
    G = capi
    variants = [
        ("defaults: all guards, band 0.95, batch 32, refill 32, wait 256, block 128", dict()),
        ("band 0.8", dict(band=0.8)),
        ("band 0.99", dict(band=0.99)),
        ("batch 16", dict(batch=16)),
        ("batch 24", dict(batch=24)),
        ("refill 8", dict(refill=8)),
        ("refill 24", dict(refill=24)),
        ("refill 32", dict(refill=32)),
        ("wait 16", dict(wait=16)),
        ("wait 256", dict(wait=256)),
        ("block 64", dict(block=64)),
        ("block 256", dict(block=256)),
        ("motion + psi only", dict(guards=G.GUARD_MOTION | G.GUARD_PSI)),
        ("motion + horizon + psi", dict(guards=G.GUARD_MOTION | G.GUARD_HORIZON | G.GUARD_PSI)),
        ("motion + turning points + psi", dict(guards=G.GUARD_MOTION | G.GUARD_RADIAL | G.GUARD_POLAR | G.GUARD_PSI)),
        ("no motion guard", dict(guards=G.GUARD_ALL & ~G.GUARD_MOTION)),
    ]
    for name, kw in variants:
        s, ms, e, img = run(o(capi.MIXED, **kw), True, 5)
        print(json.dumps({"variant": name, "ms": ms, "over_fp64": ms64 / ms,
                          "fp64_steps": s.fp64Steps, "steps": s.steps, "horizon": s.fp64Horizon,
                          "radial": s.fp64Radial, "polar": s.fp64Polar, "rounds": s.fp64Rounds,
                          "vs_fp64": endpoint_error(e, e64, img, img64),
                          "vs_fp64_half": endpoint_error(e, e64h, img, img64h)}), flush=True)
    lib.artfCudaDestroy(ctx)


def profile_case(args):
    """One warm-up and one traced frame of one precision at the given size, nothing else; or, for
    `adjoint`, two adjoint launches over `--views` views of the adjoint workload at the given size."""
    from artful_gb300 import capi, scenes
    import torch
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.artfCudaCreate(0, C.byref(ctx)))
    if args.profile == "frame":
        out = reference_frame_measurement(lib, frames=3, warm=2, cpu=False)
        print(json.dumps({"profile": "frame", **{k: v for k, v in out.items() if k.endswith("ms")}}))
        lib.artfCudaDestroy(ctx)
        return
    if args.profile == "adjoint":
        from artful_gb300 import fit
        target, start = fit.config4_params()
        m = fit.param_map(start)
        capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 1))
        unit = scenes.unit_fluid()
        capi.check(lib.artfCudaSetFluid(ctx, unit.ctypes.data, 1))
        adj = fit.Adjoint(lib, ctx, args.width, args.height, checkpoint=args.checkpoint)
        targets = adj.render([target] * args.views)
        for _ in range(2):
            loss, grad, s = adj([start] * args.views, targets)
        print(json.dumps({"profile": "adjoint", "width": args.width, "height": args.height, "views": args.views,
                          "checkpoint": args.checkpoint, "ms": s.ms, "rays": s.rays, "steps": s.steps, "grad": grad[0].tolist()}))
        lib.artfCudaDestroy(ctx)
        return
    scene = scenes.config2(4)
    scene.width, scene.height = args.width, args.height
    frame, frame64, clamped = scenes.frame(scene)
    map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    capi.check(lib.artfCudaSetMap(ctx, map_.ctypes.data, 1))
    unit = scenes.unit_fluid()  # (kept alive across the call: the ABI reads it)
    capi.check(lib.artfCudaSetFluid(ctx, unit.ctypes.data, 1))
    hdr = torch.empty((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
    o = capi.TraceOptions(capi.PRECISIONS[args.profile], 4, scene.jitter_seed, 1.0, 0.0, 0, 0,
                          1 if args.persistent else 0, args.guards)
    for _ in range(2):
        s = capi.TraceStats()
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(o),
                                         hdr.data_ptr(), None, C.byref(s)))
    print(json.dumps({"profile": args.profile, "width": scene.width, "height": scene.height, "ms": s.ms,
                      "rays": s.rays, "steps": s.steps, "fp64Steps": s.fp64Steps, "flops": s.flops}))
    lib.artfCudaDestroy(ctx)


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(frame, map_, fluid, jitter, seed):
    """The oracle port (the reference's lensTrace in scalar C, bit for bit) on all host threads over the
    whole frame: one untimed frame, then the better of two."""
    from oracle import binding
    threads = binding.oracle().oracleThreads()
    geodesics = int(frame.size[0]) * int(frame.size[1]) * jitter
    binding.render32(frame, map_, fluid, jitter=jitter, seed=seed, threads=threads)
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        binding.render32(frame, map_, fluid, jitter=jitter, seed=seed, threads=threads)
        times.append(time.perf_counter() - t0)
    dt = min(times)
    return {"value": geodesics / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the whole 1920x1080 frame, {jitter} jittered rays a pixel ({geodesics} geodesics, "
                      f"{dt:.2f} s); the oracle port, scalar C, {threads} threads (the reference's AVX2 build "
                      f"ran {REFERENCE_SIMD_X86['avx2_over_port']}x the port on an x86 host)"}


def vs_reference_cpu(frame, map_, fluid, image, jitter, seed):
    """The GPU frame against the reference's CPU trace of the same rays (the oracle port, the reference's
    bits) and against the same algorithm in FP64 (oracle/parity.py): classes outside the photon ring,
    radiance within 1e-3 outside the ring and on the pixels resolved at FP32's precision, and the
    reference's own FP32 against its FP64 beside it."""
    from oracle import parity
    out = parity.Reference(frame, map_, fluid, jitter, seed).report(image)
    out["reference"] = "the oracle port, the reference's lensTrace bit for bit, whole frame"
    return out


def reference_inputs():
    """The headline view's inputs for the CPU arm, without the CUDA library: the frame block the
    reference's own artfHoleFrame filled (recorded from the reference in the golden fixtures), and the
    synthetic map from the oracle's library, checked against the recorded hash."""
    import hashlib
    from artful_gb300 import capi  # (ctypes layouts only: nothing is loaded)
    from oracle import binding
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as fh:
        meta = json.load(fh)
    frame = capi.HoleFrame.from_buffer_copy(bytes.fromhex(meta["c2_rows"]["frame_hex"]))
    clamped = capi.BlackHoleDesc.from_buffer_copy(bytes.fromhex(meta["views"]["c2"]["clamped_hex"]))
    synth = meta["views"]["c2"]["synth"]
    map_ = binding.synth_map(clamped.discInner, clamped.discOuter, clamped.spin, synth["seed"], synth["emissivity"])
    if hashlib.sha256(map_.tobytes()).hexdigest() != meta["c2_rows"]["map_sha256"]:
        raise RuntimeError("the CPU arm's synthetic map differs from the recorded one")
    return frame, map_, np.ones(binding.FLUID_FLOATS, np.float32)


# The reference's own SIMD build against the oracle port, measured on an x86 host where the reference's
# sources are (the AVX2 kernels: 8 lanes): the headline view with 2 x 2 stratified rays a pixel, best of
# three, 8 threads each.  The Arm host has the reference's NEON kernels (4 lanes) but not its sources.
REFERENCE_SIMD_X86 = {"avx2_ms": 160.9, "port_ms": 1643.1, "reference_portable_ms": 1228.7, "threads": 8,
                      "avx2_over_port": 10.2, "view": "1920x1080, 2x2 stratified rays a pixel, a=0.998, i=85 deg",
                      "same_bits": True}


def run_reference(args, rank, world):
    """The reference's CPU path of the headline workload on this host's cores: every step one whole frame
    (1920 x 1080, 4 jittered rays a pixel) through the oracle port, the reference's lensTrace restated in
    scalar C and equal to it bit for bit, on all host threads.  Rank 0 alone; no CUDA library is loaded."""
    if rank != 0:
        return
    from oracle import binding
    frame, map_, fluid = reference_inputs()
    threads = binding.oracle().oracleThreads()
    geodesics = 1920 * 1080 * 4
    for _ in range(args.warmup):
        binding.render32(frame, map_, fluid, jitter=4, seed=1, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        binding.render32(frame, map_, fluid, jitter=4, seed=1, threads=threads)
    step_s = (time.perf_counter() - t0) / args.steps
    value = geodesics / step_s
    sample = (f"the whole 1920x1080 frame, 4 jittered rays a pixel ({geodesics} geodesics) a step; the oracle "
              f"port (the reference's lensTrace in scalar C, bit for bit) on {threads} threads.  It stands in for "
              f"the reference's NEON build, whose sources are not on this host; on an x86 host the reference's "
              f"AVX2 build ran this view {REFERENCE_SIMD_X86['avx2_over_port']}x the port "
              f"({REFERENCE_SIMD_X86['avx2_ms']} against {REFERENCE_SIMD_X86['port_ms']} ms, 8 threads)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "reference_simd_x86": REFERENCE_SIMD_X86,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_config(world):
    """The workload both arms name."""
    return {"workload": WORKLOAD, "parallelism": f"replicas{world}"}


def main():
    args = parse()
    if args.profile:
        profile_case(args)
        return
    if args.sweep:
        sweep(args)
        return
    if args.gradient_bias:
        gradient_bias(args)
        return
    rank, world, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    from artful_gb300 import capi, scenes
    torch.cuda.set_device(local)
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.artfCudaCreate(local, C.byref(ctx)))
    stream = torch.cuda.ExternalStream(lib.artfCudaStream(ctx), device=f"cuda:{local}")

    scene = scenes.config2(4)
    # the reference's own frame block: the traces that work in double widen it (a NULL FP64 frame), so
    # every trace here and the reference's CPU trace follow the same rays
    frame, _, clamped = scenes.frame(scene)
    map_ = scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)
    fluid = scenes.unit_fluid()
    capi.check(lib.artfCudaSetMap(ctx, map_.ctypes.data, 1))
    capi.check(lib.artfCudaSetFluid(ctx, fluid.ctypes.data, 1))
    w, h, rays = scene.width, scene.height, 4
    geodesics = w * h * rays
    hdr = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def opts(precision, step_scale=1.0):
        return capi.TraceOptions(precision, rays, scene.jitter_seed, step_scale, 0.0, 0, 0, 1)

    def timed(precision, steps, warmup):
        o = opts(precision)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(o),
                                                 hdr.data_ptr(), None, None))
            stream.synchronize()
            barrier(world)
            total = 0.0
            for _ in range(steps):
                flush.fill_(1)
                start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                start.record(stream)
                capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(o),
                                                 hdr.data_ptr(), None, None))
                stop.record(stream)
                stop.synchronize()
                total += start.elapsed_time(stop)
            torch.cuda.synchronize()
            barrier(world)
        return max_over_ranks(total / steps, world)

    def stats_of(precision):
        s = capi.TraceStats()
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(opts(precision)),
                                         hdr.data_ptr(), None, C.byref(s)))
        return s

    # the headline: mixed precision, timed (clocks sampled meanwhile)
    with Clocks(local) as clocks:
        ms_mixed = timed(capi.MIXED, args.steps, args.warmup)
    s_mixed = stats_of(capi.MIXED)
    side = {}
    fp64_steps = max(2, args.steps // 3)
    ms_fp64 = timed(capi.FP64, fp64_steps, 1)
    side["fp64"] = {"geodesics_per_s": geodesics / (ms_fp64 * 1e-3), "ms_per_frame": ms_fp64}
    for name, prec in (("fp32_exact", capi.EXACT), ("fp32_fast", capi.FP32)):
        ms = timed(prec, args.steps, 1)
        s = stats_of(prec)
        side[name] = {"geodesics_per_s": geodesics / (ms * 1e-3), "ms_per_frame": ms,
                      "steps_per_s": s.steps / (ms * 1e-3), "flops_per_frame": s.flops}
    side["fp64"]["flops_per_frame"] = stats_of(capi.FP64).flops

    # the same view with the reference's own 2 x 2 stratified rays a pixel (the frame's samples, no
    # jitter), through the same public call: mixed and the exact FP32 trace (the reference's bits)
    strat_scene = scenes.Scene("c2_2x2", scenes.hole_desc(0.998, samples=2), scenes.camera(85.0, 50.0), w, h,
                               seed=scene.seed, emissivity=scene.emissivity)
    strat_frame = scenes.frame(strat_scene)[0]

    def timed_strat(precision, steps):
        o = capi.TraceOptions(precision, 0, 0, 1.0, 0.0, 0, 0, 1)
        with torch.cuda.stream(stream):
            capi.check(lib.artfCudaHoleTrace(ctx, C.byref(strat_frame), None, None, None, C.byref(o),
                                             hdr.data_ptr(), None, None))
            total = 0.0
            for _ in range(steps):
                flush.fill_(1)
                start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                start.record(stream)
                capi.check(lib.artfCudaHoleTrace(ctx, C.byref(strat_frame), None, None, None, C.byref(o),
                                                 hdr.data_ptr(), None, None))
                stop.record(stream)
                stop.synchronize()
                total += start.elapsed_time(stop)
        return total / steps

    stratified = {}
    for name, prec in (("mixed", capi.MIXED), ("fp32_exact", capi.EXACT)):
        ms = timed_strat(prec, args.steps)
        stratified[name] = {"ms_per_frame": ms, "geodesics_per_s": geodesics / (ms * 1e-3)}

    # endpoint error of the mixed trace: against FP64 at the same step (precision) and at half step
    # (precision and discretisation), over every ray of the frame
    def ends_of(precision, step_scale=1.0):
        e = torch.empty((geodesics * 32,), dtype=torch.uint8, device="cuda")
        o = opts(precision, step_scale)
        capi.check(lib.artfCudaHoleTrace(ctx, C.byref(frame), None, None, None, C.byref(o),
                                         hdr.data_ptr(), e.data_ptr(), None))
        torch.cuda.synchronize()
        return np.frombuffer(e.cpu().numpy().tobytes(), END_DTYPE), hdr.cpu().numpy().copy()

    endpoint = {}
    if not args.quick:
        e_mixed, img_mixed = ends_of(capi.MIXED)
        for label, scale in (("vs_fp64_same_step", 1.0), ("vs_fp64_half_step", 0.5)):
            e_ref, img_ref = ends_of(capi.FP64, scale)
            endpoint[label] = endpoint_error(e_mixed, e_ref, img_mixed, img_ref)

    # roofline of the trace: the mixed kernel runs on the FP32 pipe, its FP32 steps and its wide work (the
    # set-ups and the turning points as double-float pairs) alike, all but the horizon band's FP64
    # sub-steps; no tensor cores.  Its algorithmic operations (the FP32 ones and the wide ones, each
    # counted once) over the step time, against the FP32 pipe's measured peak
    fp32_peak, fp64_peak = C.c_double(), C.c_double()
    capi.check(lib.artfCudaProbePeaks(lib.artfCudaStream(ctx), local, C.byref(fp32_peak), C.byref(fp64_peak)))
    achieved = (s_mixed.flops + s_mixed.flops64) / (ms_mixed * 1e-3) / 1e12
    peak = fp32_peak.value / 1e12
    peak64 = fp64_peak.value / 1e12
    horizon64 = s_mixed.fp64Horizon * FLOPS_WIDE_RADIAL  # (what still runs on the FP64 pipe)
    # HBM beside it, to show it is not the bound: the trace's DRAM bytes a frame against the measured copy
    traffic = TRACE_TRAFFIC_BYTES * geodesics / TRACE_TRAFFIC_GEODESICS  # (scaled by the rays traced)
    hbm = {"achieved": traffic / (ms_mixed * 1e-3) / 1e9, "unit": "GB/s", "traffic_source": TRACE_TRAFFIC_SOURCE}
    peaks_path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            hbm.update(peak=float(json.load(fh)["hbm_gbs"]), peak_source="MEASURED_PEAKS.json, of measured")
    else:
        hbm.update(peak=6800.0, peak_source="6.8 TB/s, of fallback")
    hbm["frac"] = hbm["achieved"] / hbm["peak"]
    # the other traces against their own pipe: FP32 (exact, fast) and FP64 (plain), of the measured peaks
    for name, pipe_peak in (("fp32_exact", peak), ("fp32_fast", peak), ("fp64", peak64)):
        entry = side[name]
        entry["pipe_frac"] = entry["flops_per_frame"] / (entry["ms_per_frame"] * 1e-3) / 1e12 / pipe_peak

    # end to end through the host-buffer entry point
    pin_map = torch.from_numpy(map_).pin_memory()
    pin_fluid = torch.from_numpy(fluid).pin_memory()
    pin_hdr = torch.empty((h, w, 4), dtype=torch.float32).pin_memory()
    o = opts(capi.MIXED)
    for _ in range(args.warmup):
        capi.check(lib.artfCudaHoleRender(ctx, C.byref(frame), None, pin_map.data_ptr(), 0,
                                          pin_fluid.data_ptr(), 0, C.byref(o), pin_hdr.data_ptr(), None))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        capi.check(lib.artfCudaHoleRender(ctx, C.byref(frame), None, pin_map.data_ptr(), 0,
                                          pin_fluid.data_ptr(), 0, C.byref(o), pin_hdr.data_ptr(), None))
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, world)

    cpu = None
    batch = None
    adjoint = fitting = next_rows = whole_frame = None
    if rank == 0 and not args.quick:
        cpu = cpu_baseline(frame, map_, fluid, rays, scene.jitter_seed)
        versus_cpu = vs_reference_cpu(frame, map_, fluid, img_mixed, rays, scene.jitter_seed)
        batch = batch_measurement(lib, ctx, args.steps, flush)
        adjoint = adjoint_measurement(lib, ctx, args.steps, flush)
        fitting = fit_measurement(lib, ctx, args.fd_fits)
        next_rows = next_rows_measurement(lib, ctx)
        whole_frame = reference_frame_measurement(lib)

    lib.artfCudaDestroy(ctx)
    if rank != 0:
        return
    value = world * geodesics / (ms_mixed * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "precision": "mixed",
        "config": bench_config(world), "l2": "flushed (256 MB write) before every timed step",
        "mixed_over_fp64": side["fp64"]["ms_per_frame"] / ms_mixed,
        "steps_per_s": s_mixed.steps / (ms_mixed * 1e-3) * world,
        "fp64_step_share": s_mixed.fp64Steps / max(1, s_mixed.steps),
        "fp64_substeps": {"horizon_band": s_mixed.fp64Horizon, "radial_turn": s_mixed.fp64Radial,
                          "polar_turn": s_mixed.fp64Polar, "warp_rounds": s_mixed.fp64Rounds},
        "side": side,
        "stratified_2x2": stratified,
        "endpoint_error": endpoint,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "measured FMA-chain probe (artfCudaProbePeaks), of measured; "
                                    "MEASURED_PEAKS.json has no FP64- or FP32-pipe figure",
                     "flops_per_frame": s_mixed.flops, "wide_flops_per_frame": s_mixed.flops64,
                     "fp64": {"achieved": horizon64 / (ms_mixed * 1e-3) / 1e12, "peak": peak64,
                              "frac": horizon64 / (ms_mixed * 1e-3) / 1e12 / peak64,
                              "flops_per_frame": horizon64,
                              "what": "the horizon band's FP64 sub-steps, all that still runs on the FP64 pipe"},
                     "hbm": hbm,
                     "time": "the whole timed step (probe, order, trace, combine)",
                     "pipes_busy": MIXED_PIPES_BUSY},
        "e2e": {"value": world * geodesics / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": (map_.nbytes + fluid.nbytes), "d2h_bytes_per_step": h * w * 16},
        "gpu_launches": args.steps * LAUNCHES_PER_MIXED_FRAME,
        "clocks": clocks.summary(),
    }
    if cpu:
        line["cpu_baseline"] = cpu
        line["mixed_vs_reference_cpu"] = versus_cpu
    if batch:
        line["batch_64_views"] = batch
    if adjoint:
        line["adjoint"] = adjoint
    if fitting:
        line["inverse_fit"] = fitting
    if next_rows:
        line["disc_inputs"] = next_rows
    if whole_frame:
        line["reference_frame"] = whole_frame
    print(json.dumps(line), flush=True)


def _median_ms(run, steps, flush=None):
    """Median over `steps` runs of the device time a run reports (its own CUDA events), after a flush of L2
    before each when a flush buffer is given.  The flush runs on torch's stream and the library's launches
    on the context's own (non-blocking) stream, so the flush is waited for: overlapping the timed launch
    it would slow it."""
    import torch
    times = []
    for _ in range(max(3, steps)):
        if flush is not None:
            flush.fill_(1)
            torch.cuda.synchronize()
        times.append(run())
    return statistics.median(times)


def adjoint_measurement(lib, ctx, steps, flush):
    """Configuration 4: the adjoint at 512 x 288 (a = 0.6, i = 55 deg, r_in = 1.1 r_ISCO, q = 2.7,
    r_obs = 32 against the image of a = 0.7, i = 60 deg, r_in = r_ISCO, q = 3, r_obs = 30), with its
    checkpoint interval (ADJOINT_CHECKPOINT), beside the forward traces of the same rays (FP32 and mixed
    precision); eight such views in one adjoint launch beside one forward trace of as many pixels; and
    both again with the other interval (every state kept, or a checkpoint every 32 steps)."""
    import torch
    from artful_gb300 import capi, fit
    target, start = fit.config4_params()
    m = fit.param_map(start)
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    w, h = 512, 288
    adj = fit.Adjoint(lib, ctx, w, h, checkpoint=ADJOINT_CHECKPOINT)
    targets = adj.render([target])
    torch.cuda.synchronize()
    last = {}

    def run_adjoint(views, tg, k=ADJOINT_CHECKPOINT):
        def go():
            loss, grad, st = adj(views, tg, checkpoint=k)
            last.update(loss=loss, grad=grad, stats=st)
            return st.ms
        return go

    def run_forward(p, width, height, precision):
        f, f64, _ = fit.frames(p, width, height)
        hdr = torch.empty((height, width, 4), dtype=torch.float32, device="cuda")
        opts = capi.TraceOptions(precision, 0, 0, 1.0, 0.0, 0, 0, 0, 0, 0, 0)

        def go():
            s = capi.TraceStats()
            capi.check(lib.artfCudaHoleTrace(ctx, C.byref(f), C.byref(f64), None, None, C.byref(opts), hdr.data_ptr(),
                                             None, C.byref(s)))
            last["fwd_steps"] = s.steps
            return s.ms
        return go

    ms_adj = _median_ms(run_adjoint([start], targets), steps, flush)
    one = dict(last)
    ms_fp32 = _median_ms(run_forward(start, w, h, capi.FP32), steps, flush)
    ms_mixed = _median_ms(run_forward(start, w, h, capi.MIXED), steps, flush)
    eight = targets.repeat(8, 1, 1, 1)
    ms_adj8 = _median_ms(run_adjoint([start] * 8, eight), steps, flush)
    steps8 = last["stats"].steps
    ms_fp32_big = _median_ms(run_forward(start, 1448, 816, capi.FP32), steps, flush)
    other = 32 if ADJOINT_CHECKPOINT == 1 else 1
    ms_other = _median_ms(run_adjoint([start], targets, other), steps, flush)
    grad_other = last["grad"][0]
    ms_other8 = _median_ms(run_adjoint([start] * 8, eight, other), steps, flush)
    return {
        "workload": "512x288, 1 ray at each pixel centre, loss = MSE of linear RGB against the target's image, "
                    f"K={ADJOINT_CHECKPOINT}" + (" (every state kept)" if ADJOINT_CHECKPOINT == 1 else ""),
        "adjoint_ms": ms_adj, "forward_fp32_ms": ms_fp32, "forward_mixed_ms": ms_mixed,
        "adjoint_over_forward_fp32": ms_adj / ms_fp32, "adjoint_over_forward_mixed": ms_adj / ms_mixed,
        "steps": one["stats"].steps, "loss": float(one["loss"][0]),
        "gradient": dict(zip(fit.PARAM_NAMES, map(float, one["grad"][0]))),
        "batched_8_views": {"adjoint_ms": ms_adj8, "steps": steps8,
                            "forward_fp32_1448x816_ms": ms_fp32_big,
                            "adjoint_over_forward_fp32": ms_adj8 / ms_fp32_big},
        "other_checkpoint": {"checkpoint": other, "adjoint_ms": ms_other, "adjoint_over_forward_fp32": ms_other / ms_fp32,
                             "batched_8_views_ms": ms_other8, "batched_8_over_forward_fp32": ms_other8 / ms_fp32_big,
                             "gradient_max_rel_diff": float(np.max(np.abs(grad_other - one["grad"][0]))
                                                            / np.max(np.abs(one["grad"][0])))},
    }


def next_rows_measurement(lib, ctx):
    """The disc's inputs made on the GPU, byte for byte the reference's: the painted map (hole.c
    buildDisc + setRings) and the fluid's step (fluid.c), each beside the oracle's scalar C restatement
    of the same code timed on one host core (the reference runs them on all cores)."""
    import torch
    from artful_gb300 import capi
    from oracle import binding
    inner, outer, spin = float(lib.artfCudaIsco(0.998)), 12.0, 0.998
    dev = torch.empty(capi.MAP_FLOATS, dtype=torch.float32, device="cuda")
    paint = []
    for _ in range(5):
        t0 = time.perf_counter()
        capi.check(lib.artfCudaPaintDisc(ctx, dev.data_ptr(), inner, outer, spin))  # (synchronous)
        paint.append((time.perf_counter() - t0) * 1e3)
    fluid = C.c_void_p()
    t0 = time.perf_counter()
    capi.check(lib.artfCudaFluidNew(ctx, inner, outer, spin, 0.0, C.byref(fluid)))
    fluid_new_ms = (time.perf_counter() - t0) * 1e3
    stream = torch.cuda.ExternalStream(lib.artfCudaStream(ctx))
    steps = {}
    for n in (1, 48):
        times = []
        for _ in range(5):
            start_t = lib.artfCudaFluidTime(fluid)
            begin, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            begin.record(stream)
            capi.check(lib.artfCudaFluidAdvance(fluid, start_t + n * 0.2 + 1e-3, None))
            end.record(stream)
            end.synchronize()
            times.append(begin.elapsed_time(end))
        steps[n] = statistics.median(times) / n
    lib.artfCudaFluidFree(fluid)
    orc = binding.oracle()
    host = np.zeros(capi.MAP_FLOATS, np.float32)
    t0 = time.perf_counter()
    orc.oraclePaintDisc(host.ctypes.data)
    oracle_paint_ms = (time.perf_counter() - t0) * 1e3
    fl = binding.Fluid(orc, "oracle", inner, outer, spin, 0.0)
    t0 = time.perf_counter()
    fl.advance(48 * 0.2 + 1e-3)
    oracle_step_ms = (time.perf_counter() - t0) * 1e3 / 48
    fl.free()
    return {"paint_disc_ms": statistics.median(paint), "fluid_new_ms": fluid_new_ms,
            "fluid_step_ms": steps[1], "fluid_step_ms_in_48": steps[48],
            "cpu_baseline": {"paint_disc_ms": oracle_paint_ms, "fluid_step_ms": oracle_step_ms, "cores": 1,
                             "kind": "port", "sample": "one painted map; 48 fluid steps"}}


def reference_frame_measurement(lib, frames=30, warm=5, cpu=True):
    """The reference's own published frame (its README's `blackhole` figure: 1920 x 1080, one ray a pixel,
    a fluid step and bloom; 23 ms on a Vega 8 in Vulkan, 141 ms in its software renderer on a 4-core Ryzen
    3200G), drawn through this backend's eight-entry table with device inputs: the reference's own scene (its
    painted disc and its gas, made and stepped on the GPU), the exact trace (the reference's bits), bloom,
    tone map and dither, the BGRA frame read back to the host every frame.  The hole's clock moves one gas
    step (0.2) a frame.  Beside it the oracle port of the same frame's parts on the host cores."""
    from artful_gb300 import capi, scenes
    w, h = 1920, 1080
    opts = capi.RendererOptions(capi.BACKEND)
    opts.width, opts.height = w, h
    r = lib.artfCudaNew(C.byref(opts))
    if not r:
        raise RuntimeError(lib.artfCudaLastError())
    vt = C.cast(r, C.POINTER(capi.RendererHead)).contents.vt.contents
    lib.artfCudaRendererSetDeviceInputs(r, True)
    scene = lib.artfCudaSceneNew()
    cam = scenes.camera(80.0, 30.0)
    lib.artfCudaSceneSetCamera(scene, C.byref(cam))
    bgra = np.zeros((h, w), np.uint32)

    def desc_at(k):
        d = scenes.hole_desc(0.9, time=0.2 * k)
        d.bloom = 4.5
        return d

    import torch
    pinned = torch.empty((h, w), dtype=torch.int32, pin_memory=True)
    times, draws, reads, lens, pinned_times = [], [], [], [], []
    try:
        for k in range(warm + 2 * frames):
            d = desc_at(k)
            lib.artfCudaSceneSetBlackHole(scene, C.byref(d))
            # the first frames read back into pageable memory (a plain host array), the rest into pinned
            into = bgra.ctypes.data if k < warm + frames else pinned.data_ptr()
            t0 = time.perf_counter()
            if not vt.draw(r, scene):
                raise RuntimeError(lib.artfCudaLastError())
            t1 = time.perf_counter()
            if not vt.readPixels(r, into):
                raise RuntimeError(lib.artfCudaLastError())
            t2 = time.perf_counter()
            if warm <= k < warm + frames:
                times.append((t2 - t0) * 1e3)
                draws.append((t1 - t0) * 1e3)
                reads.append((t2 - t1) * 1e3)
                st = capi.FrameStats()
                vt.stats(r, C.cast(C.pointer(st), C.c_void_p))
                lens.append(st.lensMs)
            elif k >= warm + frames:
                pinned_times.append((t2 - t0) * 1e3)
    finally:
        vt.destroy(r)
        lib.artfCudaSceneFree(scene)
    out = {"workload": "the reference's blackhole frame: 1920x1080, 1 ray a pixel, a = 0.9, i = 80 deg, r = 30 M, "
                       "painted disc, a gas step a frame, bloom 4.5, ACES and dither to BGRA, read back to the host",
           "ms_per_frame": statistics.median(times), "ms_per_frame_min": min(times),
           "draw_ms": statistics.median(draws), "read_pixels_ms": statistics.median(reads),
           "lens_ms": statistics.median(lens), "frames": frames,
           "ms_per_frame_into_pinned": statistics.median(pinned_times),
           "reference_published_ms": {"vega8_vulkan": 23.0, "ryzen_3200g_4_cores_software": 141.0}}
    if not cpu:
        return out
    # the oracle port of the frame's parts on the host: a gas step, the trace (all host threads), bloom and
    # tone map (one thread), on the synthetic disc of the same hole
    from oracle import binding
    view = scenes.Scene("frame", desc_at(warm), cam, w, h, seed=0)
    frame, _, clamped = scenes.frame(view)
    m = binding.synth_map(clamped.discInner, clamped.discOuter, clamped.spin, 0, 3.0)
    fl = binding.Fluid(binding.oracle(), "oracle", clamped.discInner, clamped.discOuter, clamped.spin, 0.0)
    t0 = time.perf_counter()
    fl.advance(0.2 + 1e-3)
    field, _ = fl.read()
    t1 = time.perf_counter()
    hdr = binding.render32(frame, m, field)
    t2 = time.perf_counter()
    binding.post(frame, hdr)
    t3 = time.perf_counter()
    fl.free()
    out["cpu_baseline"] = {"ms_per_frame": (t3 - t0) * 1e3, "fluid_step_ms": (t1 - t0) * 1e3,
                             "trace_ms": (t2 - t1) * 1e3, "post_ms": (t3 - t2) * 1e3, "cores": os.cpu_count(),
                             "kind": "port", "sample": "one frame: the oracle's gas step and bloom on one thread, "
                                                       "its trace on all host threads"}
    return out


def fit_measurement(lib, ctx, fd_fits):
    """Configuration 5: 32 independent fits of 256 x 144 (targets from seed 3, starts 15% off in the three
    drawn parameters, spin, inclination and inner radius, the emissivity index and distance held at their
    known values), 200 Adam steps of lr 1e-2, every step one adjoint launch over all 32 views; beside the
    same fit with gradients by central differences (h = 1e-4) of FP64 renders, on the first `fd_fits` fits;
    and, harder, the same 32 fits with every one of the five parameters started 15% off and fitted."""
    import torch
    from artful_gb300 import capi, fit
    fits = fit.config5_fits(32, seed=3)
    m = fit.param_map(fits[0][0])
    capi.check(lib.artfCudaSetMap(ctx, m.ctypes.data, 0))
    w, h = 256, 144
    adj = fit.Adjoint(lib, ctx, w, h, checkpoint=ADJOINT_CHECKPOINT)
    fit.fit_batch(adj, fits[:2], steps=3)  # warm-up
    theta, history, wall = fit.fit_batch(adj, fits, steps=200, lr=1e-2)
    err = fit.recovery_error(theta, fits)

    def summary(e, free=fit.DRAWN):
        names = [fit.PARAM_NAMES[q] for q in free]
        e = e[:, list(free)]
        return {"median": dict(zip(names, map(float, np.median(e, 0)))),
                "p90": dict(zip(names, map(float, np.percentile(e, 90, 0)))),
                "fits_within_5pct": int((e.max(1) < 0.05).sum()), "fits_within_10pct": int((e.max(1) < 0.10).sum())}

    out = {"workload": "32 fits of 256x144, spin, inclination and inner radius started 15% off and fitted "
                       "(q = 3, r_obs = 30 held), 200 Adam steps, lr 1e-2 (relative to the start), "
                       f"adjoint K={ADJOINT_CHECKPOINT}",
           "wall_s": wall, "wall_per_fit_s": wall / len(fits), "start_error": 0.15,
           "loss_first_last": [float(history[0]), float(history[-1])], "recovery_error": summary(err)}
    # why: the adjoint's gradient against finite differences of its own forward renders, pixel by pixel,
    # at the first six fits' starts (the share of the gradient on pixels where the loss is not smooth)
    six = adj.render([t for t, _ in fits[:6]])
    out["gradient_decomposition"] = pixel_decomposition(adj, fits[:6], six)
    all5 = fit.config5_fits(32, seed=3, offset=range(5))
    theta5, history5, wall5 = fit.fit_batch(adj, all5, steps=200, lr=1e-2, free=range(5))
    out["five_parameters"] = {"workload": "the same fits with all five parameters started 15% off and fitted",
                              "wall_s": wall5, "loss_first_last": [float(history5[0]), float(history5[-1])],
                              "recovery_error": summary(fit.recovery_error(theta5, all5), range(5))}
    if fd_fits > 0:
        targets = adj.render([t for t, _ in fits[:fd_fits]])
        fp64 = fit.Fp64Loss(lib, ctx, w, h, m, lib.artfCudaDeviceFluid(ctx), 11 * fd_fits)
        theta_fd, history_fd, wall_fd = fit.fit_batch_fd(fp64, fits[:fd_fits], targets, steps=200, lr=1e-2)
        err_fd = fit.recovery_error(theta_fd, fits[:fd_fits])
        out["fp64_fd_baseline"] = {
            "fits": fd_fits, "wall_s": wall_fd, "wall_per_fit_s": wall_fd / fd_fits,
            "loss_first_last": [float(history_fd[0]), float(history_fd[-1])],
            "recovery_error": summary(err_fd), "adjoint_same_fits": summary(err[:fd_fits]),
            "adjoint_speedup_per_fit": (wall_fd / fd_fits) / (wall / len(fits))}
        del fp64
        torch.cuda.empty_cache()
    return out


def batch_measurement(lib, ctx, steps, flush):
    """Configuration 3: 64 views of uneven size, spin, inclination and distance (seed 2), each with its own
    disc map, traced by one persistent launch captured in a CUDA graph, after the autotuner picked its
    launch shape; next to the same views as 64 separate launches."""
    import torch
    from artful_gb300 import capi, scenes
    stream = torch.cuda.ExternalStream(lib.artfCudaStream(ctx))
    views, keep, geodesics = [], [], 0
    for scene in scenes.config3_views(64, seed=2):
        frame, frame64, clamped = scenes.frame(scene)
        m = torch.from_numpy(scenes.synth_map(lib, clamped, scene.seed, scene.emissivity)).cuda()
        fluid = torch.from_numpy(scenes.unit_fluid()).cuda()
        hdr = torch.empty((scene.height, scene.width, 4), dtype=torch.float32, device="cuda")
        views.append(capi.View(frame, frame64, m.data_ptr(), fluid.data_ptr(), hdr.data_ptr(), None))
        keep.append((m, fluid, hdr))
        geodesics += scene.width * scene.height
    table = (capi.View * len(views))(*views)
    opts = capi.TraceOptions(capi.MIXED, 0, 2, 1.0, 0.0, 0, 0, 1)
    tuning = capi.Tuning()
    capi.check(lib.artfCudaAutotune(ctx, table, len(views), C.byref(opts), C.byref(tuning)))
    graph = C.c_void_p()
    capi.check(lib.artfCudaBatchGraphCreate(ctx, table, len(views), C.byref(opts), C.byref(graph)))
    stats = capi.TraceStats()
    capi.check(lib.artfCudaBatchGraphLaunch(graph, C.byref(stats)))
    times = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.fill_(1)
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            capi.check(lib.artfCudaBatchGraphLaunch(graph, None))
            stop.record(stream)
            stop.synchronize()
            times.append(start.elapsed_time(stop))
    lib.artfCudaBatchGraphDestroy(graph)
    ms_batch = statistics.median(times)
    # the same views one launch each
    separate = []
    for _ in range(max(1, steps // 2)):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            for v in views:
                capi.check(lib.artfCudaHoleTrace(ctx, C.byref(v.frame), C.byref(v.frame64), v.map, v.fluid,
                                                 C.byref(opts), v.hdr, None, None))
            stop.record(stream)
            stop.synchronize()
            separate.append(start.elapsed_time(stop))
    ms_sep = statistics.median(separate)
    return {"views": len(views), "geodesics": geodesics, "ms_per_batch": ms_batch,
            "geodesics_per_s": geodesics / (ms_batch * 1e-3), "separate_launches_ms": ms_sep,
            "batch_over_separate": ms_sep / ms_batch, "fp64_step_share": stats.fp64Steps / max(1, stats.steps),
            "autotune": {"blockSize": tuning.blockSize, "compactEvery": tuning.compactEvery,
                         "fp64Batch": tuning.fp64Batch, "refillBatch": tuning.refillBatch,
                         "tuned_ms": tuning.ms, "default_ms": tuning.defaultMs, "trials": tuning.trials}}


if __name__ == "__main__":
    main()
