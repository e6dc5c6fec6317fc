/* artful_cuda — the trace kernels, generic in the arithmetic type.  Included by lensExact.cu,
 * lensFast.cu and lensFp64.cu, whose compile flags fix how float rounds.
 *
 * Work layout: a warp owns an 8 x 4 tile of pixels (rays of neighbouring pixels bend alike, so the
 * lanes of a warp take similar numbers of steps and cross the disc at similar moments), a thread owns
 * one pixel and traces its rays one after the other, summing them in the reference's order.  The HDR
 * frame is width * height float4: linear RGB and the pixel's class bits.  A persistent variant, where
 * each warp pulls tiles from a device queue, lives in the same file. */
#pragma once

#include "lensCore.cuh"
#include "lensLaunch.h"

namespace artf {
namespace {

template <typename R> struct KernelParams {
    Frame<R> f;                 /* the frame in R: kernel parameters sit in the constant bank */
    ArtfCudaHoleFrame h;        /* sample positions come from the FP32 frame, as the reference's */
    const float* map;
    const float* fluid;
    float4* hdr;
    ArtfCudaRayEnd* ends;
    unsigned long long* counters;
    int jitter;
    uint32_t seed;
    R stepScale;
    int maxSteps;
    int rays;
    float share;
    int tilesX, tiles;          /* 8 x 4 pixel tiles: this launch's count */
    int tileBegin;              /* the first (a band of the frame starts further down) */
};

/* What a thread counts, reduced over the warp before it reaches the device counters. */
struct Tally {
    unsigned rays = 0, steps = 0, crossings = 0, escapes = 0;
};

__device__ __forceinline__ void flushTally(const Tally& t, unsigned long long* counters) {
    const unsigned rays = __reduce_add_sync(0xFFFFFFFFu, t.rays);
    const unsigned steps = __reduce_add_sync(0xFFFFFFFFu, t.steps);
    const unsigned crossings = __reduce_add_sync(0xFFFFFFFFu, t.crossings);
    const unsigned escapes = __reduce_add_sync(0xFFFFFFFFu, t.escapes);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters + CRays, (unsigned long long)rays);
        atomicAdd(counters + CSteps, (unsigned long long)steps);
        atomicAdd(counters + CCrossings, (unsigned long long)crossings);
        atomicAdd(counters + CEscapes, (unsigned long long)escapes);
    }
}

__device__ __forceinline__ unsigned classBits(unsigned kind) {
    unsigned bits = (kind & ARTF_CUDA_END_LIT) ? 1u : 0u;
    if ((kind & 15u) == ARTF_CUDA_END_SKY) bits |= 2u;
    else if (!(kind & ARTF_CUDA_END_LIT)) bits |= 4u;
    return bits;
}

/* One ray, from its image position to its end (lens.inc:99-351).  Adds its light to sum (3). */
template <typename R>
__device__ __forceinline__ unsigned traceRay(const KernelParams<R>& p, R nx, R ny, R time, R* sum,
                                             ArtfCudaRayEnd* end, Tally& t) {
    const Frame<R>& f = p.f;
    RayConst<R> c;
    RayState<R> s;
    rayStart(f, nx, ny, time, p.stepScale, c, s);
    const R a = f.a, a2 = a * a;
    if (a != R(0)) s.drag = dragAt(a, a2, c.xiA, s.u);
    const R rhoScale = recipR(R(1) - divR(f.inner, f.outer));

    R raySum[3] = {R(0), R(0), R(0)}, through = R(1);
    unsigned kind = ARTF_CUDA_END_CAP, crossings = 0;
    bool lit = false;
    R hitR = R(NAN), hitPhi = R(NAN), mino = R(p.maxSteps) * c.step, dir[3] = {R(0), R(0), R(0)};
    int i = 0;
    for (; i < p.maxSteps; ++i) {
        StepOut<R> o;
        nystromStep(a, c, s, o);
        Crossing<R> x;
        if (crossingOf(f, rhoScale, c, s, o, x)) {
            ++crossings;
            R turn;
            const R light = shadeCrossing(f, rhoScale, p.map, p.fluid, c, x, through, raySum, &turn);
            if (light > R(0) && !lit) {
                lit = true;
                hitR = recipR(x.uc);
                hitPhi = turn - floorR(turn);
            }
        }
        if (R(0) > o.next.u) {
            const R part = divR(s.u, s.u - o.next.u);
            R away[3];
            for (int k = 0; k < 3; ++k) away[k] = s.n[k] + part * (o.next.n[k] - s.n[k]);
            const R awayPsi = s.psi + part * (o.next.psi - s.psi);
            skyDirection(away, awayPsi, dir);
            if (f.stars > R(0)) shadeSky(f, p.map, c, dir, through, raySum);
            kind = ARTF_CUDA_END_SKY;
            mino = (R(i) + part) * c.step;
            ++i;
            break;
        }
        if (o.next.u > f.uHorizon) { kind = ARTF_CUDA_END_HORIZON; mino = R(i + 1) * c.step; ++i; break; }
        if (!(through > KF(.004))) { kind = ARTF_CUDA_END_OPAQUE; mino = R(i + 1) * c.step; ++i; break; }
        s = o.next;
    }
    for (int k = 0; k < 3; ++k) sum[k] = sum[k] + raySum[k];
    if (lit) kind |= ARTF_CUDA_END_LIT;
    t.rays += 1;
    t.steps += (unsigned)i;
    t.crossings += crossings;
    t.escapes += (kind & 15u) == ARTF_CUDA_END_SKY;
    if (end) {
        ArtfCudaRayEnd e;
        e.hitR = (float)hitR;
        e.hitPhi = (float)hitPhi;
        for (int k = 0; k < 3; ++k) e.dir[k] = (float)dir[k];
        e.mino = (float)mino;
        e.steps = (uint16_t)i;
        e.crossings = (uint8_t)(crossings > 255u ? 255u : crossings);
        e.kind = (uint8_t)kind;
        e.fp64Steps = (uint16_t)(sizeof(R) == 8 ? i : 0);
        e.reserved = 0;
        *end = e;
    }
    return kind;
}

/* All rays of one pixel, summed in the reference's order and scaled by 1 / rays (lens.inc:364-380). */
template <typename R> __device__ __forceinline__ void tracePixel(const KernelParams<R>& p, int32_t x, int32_t y,
                                                                  Tally& t) {
    const size_t pixel = (size_t)y * (size_t)p.f.width + (size_t)x;
    R sum[3] = {R(0), R(0), R(0)};
    unsigned bits = 0;
    for (int k = 0; k < p.rays; ++k) {
        float nx, ny, moment;
        samplePosition(p.h, p.jitter, p.seed, x, y, k, &nx, &ny, &moment);
        const float time = p.h.disc[2] + p.h.spin[3] * moment;
        const int64_t endAt = (int64_t)pixel * p.rays + k;
        ArtfCudaRayEnd* end = p.ends && inBounds(p.f.fault, kBoundsRayEnd, endAt,
                                                 (int64_t)p.f.width * p.f.height * p.rays)
                                  ? p.ends + endAt
                                  : nullptr;
        bits |= classBits(traceRay(p, R(nx), R(ny), R(time), sum, end, t));
    }
    const R share = R(p.share);
    if (inBounds(p.f.fault, kBoundsPixel, (int64_t)pixel, (int64_t)p.f.width * p.f.height))
        p.hdr[pixel] = make_float4((float)(sum[0] * share), (float)(sum[1] * share), (float)(sum[2] * share), (float)bits);
}

/* One warp per 8 x 4 tile, one thread per pixel. */
template <typename R> __global__ void __launch_bounds__(256) traceTiles(const KernelParams<R> p) {
    const int lane = threadIdx.x & 31;
    const int local = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), tile = p.tileBegin + local;
    Tally t;
    if (local < p.tiles) {
        const int32_t x = (tile % p.tilesX) * 8 + (lane & 7), y = (tile / p.tilesX) * 4 + (lane >> 3);
        if (x < p.f.width && y < p.f.height) tracePixel(p, x, y, t);
    }
    flushTally(t, p.counters);
}

/* Persistent: a grid of resident warps that pull tiles from the queue counter until none is left. */
template <typename R> __global__ void __launch_bounds__(256) traceQueue(const KernelParams<R> p) {
    const int lane = threadIdx.x & 31;
    Tally t;
    for (;;) {
        int local = 0;
        if (lane == 0) local = (int)atomicAdd(p.counters + CQueue, 1ull);
        local = __shfl_sync(0xFFFFFFFFu, local, 0);
        if (local >= p.tiles) break;
        const int tile = p.tileBegin + local;
        const int32_t x = (tile % p.tilesX) * 8 + (lane & 7), y = (tile / p.tilesX) * 4 + (lane >> 3);
        if (x < p.f.width && y < p.f.height) tracePixel(p, x, y, t);
        __syncwarp();
    }
    flushTally(t, p.counters);
}

/* A list of rays at given image positions, one a thread (the per-ray entry point). */
struct RayList {
    int n;
    const float* nx;
    const float* ny;
    const float* time;
    float* rgb;
};

template <typename R> __global__ void __launch_bounds__(128) traceList(const KernelParams<R> p, const RayList l) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Tally t;
    if (i < l.n) {
        R sum[3] = {R(0), R(0), R(0)};
        traceRay(p, R(l.nx[i]), R(l.ny[i]), R(l.time[i]), sum, p.ends ? p.ends + i : nullptr, t);
        for (int k = 0; k < 3; ++k) l.rgb[3 * i + k] = (float)sum[k];
    }
    flushTally(t, p.counters);
}

template <typename R> cudaError_t launchUniform(const TraceLaunch& l, const void* frameSource) {
    KernelParams<R> p;
    if (sizeof(R) == 8) p.f.load(*(const ArtfCudaHoleFrame64*)frameSource, l.frame);
    else p.f.load(*(const ArtfCudaHoleFrame*)frameSource, l.frame);
    p.f.fault = l.counters + CBoundsKind;
    p.h = l.frame;
    p.map = l.map;
    p.fluid = l.fluid;
    p.hdr = l.hdr;
    p.ends = l.ends;
    p.counters = l.counters;
    p.jitter = l.jitter;
    p.seed = l.seed;
    p.stepScale = R(l.stepScale);
    p.maxSteps = l.stepScale < .75f ? 384 : 192;
    p.rays = l.jitter ? l.jitter : (int)(l.frame.size[2] * l.frame.size[2]);
    p.share = l.jitter ? 1.f / (float)l.jitter : l.frame.image[3];
    p.tilesX = ((int)l.frame.size[0] + 7) / 8;
    const int tileRows = ((int)l.frame.size[1] + 3) / 4;
    const int bandBegin = l.tileRows > 0 ? l.tileRowBegin : 0;
    const int bandRows = l.tileRows > 0 ? l.tileRows : tileRows;
    p.tileBegin = bandBegin * p.tilesX;
    p.tiles = p.tilesX * bandRows;
    const int block = l.blockSize > 0 ? l.blockSize : 128;
    if (l.rayCount > 0) {
        const RayList list = {l.rayCount, l.rayX, l.rayY, l.rayTime, l.rayRgb};
        traceList<R><<<(l.rayCount + block - 1) / block, block, 0, l.stream>>>(p, list);
    } else if (l.persistent) {
        int perSm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, traceQueue<R>, block, 0);
        int grid = (perSm > 0 ? perSm : 1) * l.smCount;
        const int needed = (p.tiles * 32 + block - 1) / block;
        if (grid > needed) grid = needed;
        traceQueue<R><<<grid, block, 0, l.stream>>>(p);
    } else {
        const int grid = (p.tiles * 32 + block - 1) / block;
        traceTiles<R><<<grid, block, 0, l.stream>>>(p);
    }
    return cudaGetLastError();
}

}  // namespace
}  // namespace artf
