/* artful_cuda — the mixed-precision trace: FP32 for the bulk of each geodesic, FP64 only where
 * stability needs it.
 *
 *   - the constants of motion (E, xi = L_z / E, Carter's eta, K) and the first state come from the ray
 *     at the eye in FP64, from the frame computed in double;
 *   - a step runs in FP64 when the ray is within a band of the outer horizon (u > band * 0.995/r+),
 *     where Delta / r^2 in the frame-drag rate loses most of its bits to cancellation, or when the FP32
 *     step brought a turning point: the radial (du/ds changes sign) or the polar one (the axis part of
 *     dn/ds changes sign);
 *   - psi, the frame-drag angle, is summed with a compensated (two-sum) accumulator, and the Mino time
 *     of the endpoint is formed in FP64 from the step count, so that neither drifts over 192 steps.
 * The disc and sky shading stay in FP32.  Built with the fast FP32 flags of lensFast.cu; double
 * arithmetic is IEEE throughout. */
#include "lensKernel.cuh"

namespace artf {
namespace {

struct MixedParams {
    Frame<float> f;
    Frame<double> d;
    ArtfCudaHoleFrame h;
    const float* map;
    const float* fluid;
    float4* hdr;
    ArtfCudaRayEnd* ends;
    unsigned long long* counters;
    int jitter;
    uint32_t seed;
    float stepScale;
    int maxSteps;
    int rays;
    float share;
    int tilesX, tiles;
    float uGuard;  /* FP64 steps above this u */
};

template <typename A, typename B> __device__ __forceinline__ void convertState(const RayState<A>& s, RayState<B>& o) {
    o.u = B(s.u), o.w = B(s.w), o.psi = B(s.psi), o.drag = B(s.drag);
    for (int k = 0; k < 3; ++k) o.n[k] = B(s.n[k]), o.v[k] = B(s.v[k]);
}

__device__ __forceinline__ unsigned traceRayMixed(const MixedParams& p, float nx, float ny, float time, float* sum,
                                                  ArtfCudaRayEnd* end, Tally& t, unsigned& wideSteps) {
    const Frame<float>& f = p.f;
    /* the ray at the eye and its constants of motion in FP64 */
    RayConst<double> cd;
    RayState<double> sd;
    rayStart(p.d, (double)nx, (double)ny, (double)time, (double)p.stepScale, cd, sd);
    const double ad = p.d.a, a2d = ad * ad;
    if (ad != 0.0) sd.drag = dragAt(ad, a2d, cd.xiA, sd.u);
    RayConst<float> c;
    c.invEnergy = (float)cd.invEnergy, c.xi = (float)cd.xi, c.moved = (float)cd.moved, c.big = (float)cd.big;
    c.step = (float)cd.step, c.uA = (float)cd.uA, c.uB = (float)cd.uB, c.uC = (float)cd.uC, c.xiA = (float)cd.xiA;
    c.time = time;
    RayState<float> s;
    convertState(sd, s);
    s.psi = 0.f; /* the steps return psi's increment; the sum is kept apart, compensated */
    const float a = f.a;
    const float rhoScale = 1.f / (1.f - f.inner / f.outer);

    float psiHi = 0.f, psiLo = 0.f;
    float raySum[3] = {0.f, 0.f, 0.f}, through = 1.f;
    unsigned kind = ARTF_CUDA_END_CAP, crossings = 0, wide = 0;
    bool lit = false;
    float hitR = NAN, hitPhi = NAN, dir[3] = {0.f, 0.f, 0.f};
    double mino = (double)p.maxSteps * cd.step;
    int i = 0;
    for (; i < p.maxSteps; ++i) {
        StepOut<float> o;
        bool inFp64 = s.u > p.uGuard;
        if (!inFp64) {
            nystromStep(a, c, s, o);
            /* a turning point inside the step: take it again in FP64 */
            inFp64 = (s.w > 0.f) != (o.next.w > 0.f) || (s.v[2] > 0.f) != (o.next.v[2] > 0.f);
        }
        if (inFp64) {
            RayState<double> wideState;
            convertState(s, wideState);
            StepOut<double> od;
            nystromStep(ad, cd, wideState, od);
            convertState(od.next, o.next);
            o.k1 = (float)od.k1;
            for (int k = 0; k < 3; ++k) o.a1[k] = (float)od.a1[k];
            ++wide;
        }
        const float increment = o.next.psi;

        Crossing<float> x;
        if (crossingOf(f, rhoScale, c, s, o, x)) {
            x.psiC = psiHi + (psiLo + x.part * increment);
            ++crossings;
            float turn;
            const float light = shadeCrossing(f, rhoScale, p.map, p.fluid, c, x, through, raySum, &turn);
            if (light > 0.f && !lit) {
                lit = true;
                hitR = 1.f / x.uc;
                hitPhi = turn - floorf(turn);
            }
        }
        if (0.f > o.next.u) {
            const float part = s.u / (s.u - o.next.u);
            float away[3];
            for (int k = 0; k < 3; ++k) away[k] = s.n[k] + part * (o.next.n[k] - s.n[k]);
            const float awayPsi = psiHi + (psiLo + part * increment);
            skyDirection(away, awayPsi, dir);
            if (f.stars > 0.f) shadeSky(f, p.map, c, dir, through, raySum);
            kind = ARTF_CUDA_END_SKY;
            mino = ((double)i + (double)part) * cd.step;
            ++i;
            break;
        }
        if (o.next.u > f.uHorizon) { kind = ARTF_CUDA_END_HORIZON; mino = (double)(i + 1) * cd.step; ++i; break; }
        if (!(through > .004f)) { kind = ARTF_CUDA_END_OPAQUE; mino = (double)(i + 1) * cd.step; ++i; break; }
        /* psi += increment, with the rounding error carried (Knuth's two-sum) */
        const float sumHi = psiHi + increment, back = sumHi - psiHi;
        psiLo += (psiHi - (sumHi - back)) + (increment - back);
        psiHi = sumHi;
        s = o.next;
        s.psi = 0.f;
    }
    for (int k = 0; k < 3; ++k) sum[k] = sum[k] + raySum[k];
    if (lit) kind |= ARTF_CUDA_END_LIT;
    t.rays += 1;
    t.steps += (unsigned)i;
    t.crossings += crossings;
    t.escapes += (kind & 15u) == ARTF_CUDA_END_SKY;
    wideSteps += wide;
    if (end) {
        ArtfCudaRayEnd e;
        e.hitR = hitR;
        e.hitPhi = hitPhi;
        for (int k = 0; k < 3; ++k) e.dir[k] = dir[k];
        e.mino = (float)mino;
        e.steps = (uint16_t)i;
        e.crossings = (uint8_t)(crossings > 255u ? 255u : crossings);
        e.kind = (uint8_t)kind;
        e.fp64Steps = (uint16_t)wide;
        e.reserved = 0;
        *end = e;
    }
    return kind;
}

__global__ void __launch_bounds__(128) traceMixedTiles(const MixedParams p) {
    const int lane = threadIdx.x & 31;
    const int tile = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    Tally t;
    unsigned wideSteps = 0;
    if (tile < p.tiles) {
        const int32_t x = (tile % p.tilesX) * 8 + (lane & 7), y = (tile / p.tilesX) * 4 + (lane >> 3);
        if (x < p.f.width && y < p.f.height) {
            const size_t pixel = (size_t)y * (size_t)p.f.width + (size_t)x;
            float sum[3] = {0.f, 0.f, 0.f};
            unsigned bits = 0;
            for (int k = 0; k < p.rays; ++k) {
                float nx, ny, moment;
                samplePosition(p.h, p.jitter, p.seed, x, y, k, &nx, &ny, &moment);
                const float time = p.h.disc[2] + p.h.spin[3] * moment;
                ArtfCudaRayEnd* end = p.ends ? p.ends + pixel * (size_t)p.rays + (size_t)k : nullptr;
                bits |= classBits(traceRayMixed(p, nx, ny, time, sum, end, t, wideSteps));
            }
            p.hdr[pixel] = make_float4(sum[0] * p.share, sum[1] * p.share, sum[2] * p.share, (float)bits);
        }
    }
    flushTally(t, p.counters);
    const unsigned wide = __reduce_add_sync(0xFFFFFFFFu, wideSteps);
    if (lane == 0) atomicAdd(p.counters + CFp64Steps, (unsigned long long)wide);
}

__global__ void __launch_bounds__(128) traceMixedList(const MixedParams p, const int n, const float* nx,
                                                      const float* ny, const float* time, float* rgb) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Tally t;
    unsigned wideSteps = 0;
    if (i < n) {
        float sum[3] = {0.f, 0.f, 0.f};
        traceRayMixed(p, nx[i], ny[i], time[i], sum, p.ends ? p.ends + i : nullptr, t, wideSteps);
        for (int k = 0; k < 3; ++k) rgb[3 * i + k] = sum[k];
    }
    flushTally(t, p.counters);
    const unsigned wide = __reduce_add_sync(0xFFFFFFFFu, wideSteps);
    if ((threadIdx.x & 31) == 0) atomicAdd(p.counters + CFp64Steps, (unsigned long long)wide);
}

}  // namespace

cudaError_t launchMixed(const TraceLaunch& l) {
    MixedParams p;
    p.f.load(l.frame64, l.frame);
    p.d.load(l.frame64, l.frame);
    p.h = l.frame;
    p.map = l.map;
    p.fluid = l.fluid;
    p.hdr = l.hdr;
    p.ends = l.ends;
    p.counters = l.counters;
    p.jitter = l.jitter;
    p.seed = l.seed;
    p.stepScale = l.stepScale;
    p.maxSteps = l.stepScale < .75f ? 384 : 192;
    p.rays = l.jitter ? l.jitter : (int)(l.frame.size[2] * l.frame.size[2]);
    p.share = l.jitter ? 1.f / (float)l.jitter : l.frame.image[3];
    p.tilesX = ((int)l.frame.size[0] + 7) / 8;
    p.tiles = p.tilesX * (((int)l.frame.size[1] + 3) / 4);
    p.uGuard = (float)((double)(l.horizonBand > 0.f ? l.horizonBand : .5f) * l.frame64.spin[1]);
    const int block = 128;
    if (l.rayCount > 0) {
        traceMixedList<<<(l.rayCount + block - 1) / block, block, 0, l.stream>>>(p, l.rayCount, l.rayX, l.rayY,
                                                                                 l.rayTime, l.rayRgb);
        return cudaGetLastError();
    }
    const int grid = (p.tiles * 32 + block - 1) / block;
    traceMixedTiles<<<grid, block, 0, l.stream>>>(p);
    return cudaGetLastError();
}

}  // namespace artf
