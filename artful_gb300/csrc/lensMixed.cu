/* artful_cuda — the mixed-precision trace: FP32 for the bulk of each geodesic, extended precision
 * (about FP64's) only where stability needs it.  "Wide" work runs as double-float pairs on the FP32 pipe
 * (Dekker's double-length arithmetic, about 48 bits), or in FP64 where it divides:
 *
 *   MOTION   the constants of motion (E, xi = L_z / E, Carter's eta, K and the radial equation's
 *            coefficients) come from the ray at the eye in double-float, from the frame's doubles split
 *            into pairs; the first state's w and v and the step, the integrator's FP32 quantities, are
 *            formed from them in FP32 (the step by the reference's rule from the rounded K, so every
 *            sub-step of a ray, FP32 or wide, takes the same one);
 *   HORIZON  within a band of the outer horizon (u > band * 0.995 / r+) the radial sub-step of
 *            (u, du/ds, psi) runs in FP64: Delta / r^2 in the frame-drag rate loses most of its bits to
 *            cancellation there;
 *   RADIAL   the step in which du/ds changes sign (the radial potential's zero) has its motion of
 *            (u, du/ds) in double-float (psi and its rate, smooth there, stay the FP32 step's);
 *   POLAR    the step in which the axis part of dn/ds changes sign (the polar potential's zero) has
 *            the axis component (n_z, dn_z/ds) in double-float: n_z'' depends on n_z alone, and the
 *            turning point is its (the components about the axis stay the FP32 step's);
 *   PSI      psi, the frame-drag angle, is summed with a compensated (two-sum) accumulator, and the
 *            endpoint's Mino time is formed in FP64 from the step count: neither drifts over 192 steps.
 * The radial and polar sub-steps are independent (u'' depends on u alone, n'' on n alone), so a guard
 * costs wide work only for the part that needs it.  The disc and sky shading stay in FP32.  Built with
 * the fast FP32 flags; in double, + - * are IEEE and / and sqrt are refined hardware estimates (within
 * an ulp or two, lensCore.cuh), as in the plain FP64 trace.  At the headline frame the double-float
 * sub-steps give the FP64 ones' bits, rounded to float, for every pixel.
 *
 * Scheduling (traceMixedQueue): a warp pays for a wide sub-step whatever number of its lanes take part.
 * So wide work runs in warp-wide rounds: lanes that need a wide sub-step (or a new ray's set-up) wait,
 * keeping their FP32 results, while the others keep stepping in FP32; a round runs when `batch` lanes
 * wait, when no lane can move without one, or after a bounded wait.  Pixels of every view of a batch
 * come from one device queue (work stealing across views of uneven size), a lane at a time, by warp
 * ballot and shuffle.  Every lane computes exactly what the per-ray path (traceRayMixed) computes, in
 * the same order: the schedule changes when, never what.  A single frame is a batch of one view. */
#define ARTF_FAST_FP64 1 /* FP64 division and square roots by refined hardware estimates (lensCore.cuh) */
#define ARTF_FP64_NEWTON_STEPS 1 /* one refinement: ~40 bits, far below float's rounding (3.4 % faster) */
#include "lensKernel.cuh"
#include "lensMixed.h"

#include <string.h>

namespace artf {

/* A view as the kernel reads it, from the device view table. */
/* A value as the unevaluated sum hi + lo of two floats, |lo| at most half an ulp of hi: Dekker's
 * double-length arithmetic (1971), about 48 significant bits from FP32 instructions, which this GPU
 * issues 64 times as fast as FP64 ones. */
struct Ff {
    float hi, lo;
};

/* What a ray's set-up under the MOTION guard takes from the view, in double-float: the eye's basis, the
 * metric's four factors, rho, a and the start terms. */
struct MotionTermsFf {
    Ff forward[3], right[3], up[3], metric[4], rho, a, a2, mu0Squared, minusTwoA2;
};

struct MixedView {
    Frame<float> f;
    Frame<double> d;
    ArtfCudaHoleFrame h; /* sample positions come from the FP32 frame, as the reference's */
    const float* map;
    const float* fluid;
    float4* hdr;
    ArtfCudaRayEnd* ends;
    /* Rays of the view's pixels, plane k for ray k (radiance, class bits), or NULL.  With planes, a work
     * unit is one ray and mixedCombine sums each pixel's rays afterwards; without, a unit is a pixel
     * whose rays one lane traces in turn. */
    float4* rayOut;
    double wideA2;            /* a^2 in double, for the horizon band's FP64 sub-step */
    StartTerms<double> start64; /* what a moving eye's rays' FP64 set-up takes from the view alone */
    MotionTermsFf motion;       /* the same and the frame's, for the set-up of an eye at rest, as pairs */
    float startNarrow[4];     /* the eye's e_r and 1/r in float, where every ray's set-up starts */
    float wScaleNarrow;       /* -u0^2 sqrt(Delta) sqrt(Sigma), in float: w's factor from the eye */
    float stepBaseNarrow;     /* the step rule's (pi / 24) x step scale, in float */
    float rhoScale, uGuard, share;
    int tilesX, pixelUnits, units, unitBase, tileBase, rays, jitter;
    int rowBegin, rows; /* the pixel rows this launch traces (a band of the frame, or all of it) */
    uint32_t seed;
};
static_assert(sizeof(MixedView) <= kMixedViewBytesMax, "a view table slot outgrew kMixedViewBytesMax");

namespace {

struct MixedParams {
    const MixedView* views;
    int viewCount;
    int totalUnits;
    /* the queue's slots (32 units: one ray plane of one tile) in the order handed out, each (view | plane
     * << 12, tile); NULL: pixel order, view after view */
    const uint2* order;
    unsigned long long* counters;
    float stepScale;
    int maxSteps;
    uint32_t guards;  /* ARTF_CUDA_GUARD_* */
    int batch;        /* lanes waiting before a warp runs an FP64 round */
    int refill;       /* idle lanes before a warp starts new rays (an FP64 set-up each) */
    int maxWait;      /* iterations a lane waits at most */
};

/* One ray's state between steps. */
struct MixedRay {
    RayConst<float> c;
    Ff big, uA, uB, uC, xiA;           /* the coefficients the wide sub-steps use, as double-float pairs */
    double step;
    RayState<float> s;                 /* s.psi stays 0: a step returns psi's increment */
    float psiHi, psiLo, through, sum[3], hitR, hitPhi;
    int i;
    unsigned crossings, wide;
    bool lit;
};

/* Float <-> double conversions on the integer pipe.  On this GPU a conversion to double costs an FP64
 * instruction and one to float two, on the narrow FP64 pipe, while the integer pipe idles: these take a
 * handful of integer instructions instead, for the same bits as the hardware's conversions under this
 * unit's flags (flush-to-zero; round to nearest even), NaN aside (a NaN stays a NaN, its payload is not
 * kept).  artfCudaCheckConversions checks them against the hardware's.  The narrowing is a call, not
 * inlined at its sites in the FP64 paths: inlined, those copies overflowed the instruction cache (warps
 * stalled waiting for instructions; 3.97 ms against 3.50 at 1080p x 4). */
__device__ __forceinline__ double widen(float f) {
    const uint32_t b = __float_as_uint(f), sign = b & 0x80000000u, mag = b & 0x7fffffffu, e = mag >> 23;
    uint32_t hi = sign | ((mag >> 3) + 0x38000000u), lo = mag << 29;  /* rebias 127 -> 1023 */
    if (e == 0u) hi = sign, lo = 0u;                                    /* zero (a subnormal flushes) */
    if (e == 255u) hi = sign | 0x7ff00000u | ((mag & 0x7fffffu) >> 3);  /* infinity, NaN */
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __noinline__ float narrow(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t sign = hi & 0x80000000u, e = (hi >> 20) & 0x7ffu;
    /* the top 23 bits of the 52-bit fraction, and the 29 below them that rounding looks at */
    const uint32_t keep = ((hi & 0xfffffu) << 3) | (lo >> 29), rest = lo & 0x1fffffffu;
    uint32_t bits;
    if (e >= 897u && e <= 1150u) {
        bits = ((e - 896u) << 23) | keep;
        bits += (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) ? 1u : 0u; /* (may carry to inf) */
    } else if (e == 896u) {
        /* in [2^-127, 2^-126): rounded to 24 significant bits as if the exponent went on, only what then
         * reaches 2^-126 is not flushed (the fraction's top 23 bits all ones, and the rest half or more) */
        bits = (keep == 0x7fffffu && rest >= 0x10000000u) ? 0x00800000u : 0u;
    } else if (e < 896u) {
        bits = 0u;
    } else if (e == 0x7ffu && ((hi & 0xfffffu) | lo)) {
        bits = 0x7fffffffu; /* NaN */
    } else {
        bits = 0x7f800000u; /* too large, or infinite */
    }
    return __uint_as_float(sign | bits);
}

__device__ __forceinline__ double ffWide(Ff a);
__device__ __forceinline__ RayConst<double> wideConst(const MixedRay& r) {
    RayConst<double> c;
    c.big = ffWide(r.big), c.step = r.step, c.uA = ffWide(r.uA), c.uB = ffWide(r.uB), c.uC = ffWide(r.uC);
    c.xiA = ffWide(r.xiA);
    c.invEnergy = c.xi = c.moved = c.time = 0.0; /* (not read by the sub-steps) */
    return c;
}

/* ---- double-float arithmetic --------------------------------------------------------------------------
 * Sums by Knuth's error-free TwoSum, products by an FMA's residual (the exact error of a rounded product),
 * each result renormalised by Dekker's fast two-sum; the reciprocal and the reciprocal square root are
 * the float estimates refined by one Newton-Raphson step in double-float, as this unit's FP64 ones are
 * refined from float estimates (about 46 and 43 bits).  No step contracts: the only products are the
 * explicit FMAs. */
__device__ __forceinline__ Ff ffNorm(float s, float e) {
    const float hi = s + e;
    return Ff{hi, e - (hi - s)};
}
__device__ __forceinline__ Ff ffAdd(Ff a, Ff b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    return ffNorm(s, ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo));
}
__device__ __forceinline__ Ff ffNeg(Ff a) { return Ff{-a.hi, -a.lo}; }
__device__ __forceinline__ Ff ffSub(Ff a, Ff b) { return ffAdd(a, ffNeg(b)); }
__device__ __forceinline__ Ff ffMul(Ff a, Ff b) {
    const float p = a.hi * b.hi;
    return ffNorm(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p))));
}
__device__ __forceinline__ Ff ffMulF(Ff a, float b) {
    const float p = a.hi * b;
    return ffNorm(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
}
__device__ __forceinline__ Ff ffRecip(Ff x) {
    const float y = 1.f / x.hi;
    const Ff r = ffSub(Ff{1.f, 0.f}, ffMulF(x, y)); /* 1 - x y */
    return ffNorm(y, y * r.hi);
}
__device__ __forceinline__ Ff ffRsqrt(Ff x) {
    const float y = rsqrtf(x.hi);
    const Ff r = ffSub(Ff{1.f, 0.f}, ffMulF(ffMulF(x, y), y)); /* 1 - x y^2 */
    return ffNorm(y, .5f * y * r.hi);
}
/* hi + lo as a double: exact, since the pair holds at most 48 significant bits. */
__device__ __forceinline__ double ffWide(Ff a) { return widen(a.hi) + widen(a.lo); }
__device__ __forceinline__ Ff ffSplit(double x) {
    const float hi = narrow(x);
    return Ff{hi, narrow(x - widen(hi))};
}
__device__ __forceinline__ Ff ffProd(float a, float b) {
    const float p = a * b;
    return Ff{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ Ff ffScale(Ff a, float powerOfTwo) { return Ff{a.hi * powerOfTwo, a.lo * powerOfTwo}; }

/* The step's terms (stepTerms in lensCore.cuh) in double-float from the float step: its square is exact
 * as a pair, the halves and eighth exact, the sixths products by the float 1/6 as there. */
struct StepTermsFf {
    Ff half, eighth, halfSquare, sixthSquare, sixth;
};
__device__ __forceinline__ StepTermsFf stepTermsFf(float step) {
    const Ff step2 = ffProd(step, step);
    StepTermsFf t;
    t.half = Ff{step * .5f, 0.f}, t.eighth = ffScale(step2, .125f), t.halfSquare = ffScale(step2, .5f);
    t.sixthSquare = ffMulF(step2, 1.f / 6.f), t.sixth = ffProd(step, 1.f / 6.f);
    return t;
}
__device__ __forceinline__ StepTerms<double> wideTerms(const StepTermsFf& t) {
    StepTerms<double> w;
    w.half = ffWide(t.half), w.eighth = ffWide(t.eighth), w.halfSquare = ffWide(t.halfSquare);
    w.sixthSquare = ffWide(t.sixthSquare), w.sixth = ffWide(t.sixth);
    return w;
}
/* bendAt: x (uA + x (uB + x uC)) */
__device__ __forceinline__ Ff ffBend(const MixedRay& r, Ff x) {
    return ffMul(x, ffAdd(r.uA, ffMul(x, ffAdd(r.uB, ffMul(x, r.uC)))));
}
/* radialMotionWith (lensCore.cuh) in double-float, in its order of operations. */
__device__ __forceinline__ void radialMotionFf(const MixedRay& r, const StepTermsFf& t, float u, float w, Ff& nextU,
                                               Ff& nextW, Ff& k1) {
    const Ff uf{u, 0.f};
    k1 = ffBend(r, uf);
    const Ff midU = ffAdd(ffAdd(uf, ffMulF(t.half, w)), ffMul(t.eighth, k1));
    const Ff k2 = ffBend(r, midU);
    const Ff uw = ffAdd(uf, ffProd(r.c.step, w));
    const Ff endU = ffAdd(uw, ffMul(t.halfSquare, k2));
    const Ff k3 = ffBend(r, endU);
    nextU = ffAdd(uw, ffMul(t.sixthSquare, ffAdd(k1, ffAdd(k2, k2))));
    nextW = ffAdd(Ff{w, 0.f}, ffMul(t.sixth, ffAdd(ffAdd(k1, k3), ffMulF(k2, 4.f))));
}
/* polarAxisWith (lensCore.cuh) in double-float, in its order of operations. */
__device__ __forceinline__ void polarAxisFf(Ff a2, const MixedRay& r, const StepTermsFf& t, float nz, float vz,
                                            Ff& nextNz, Ff& nextVz, Ff& a1) {
    const Ff twoA2 = ffScale(a2, 2.f), nzf{nz, 0.f};
    const Ff c1 = ffAdd(r.big, ffMul(twoA2, ffProd(nz, nz)));
    a1 = ffSub(ffMulF(a2, nz), ffMulF(c1, nz));
    const Ff midN = ffAdd(ffAdd(nzf, ffMulF(t.half, vz)), ffMul(t.eighth, a1));
    const Ff c2 = ffAdd(r.big, ffMul(twoA2, ffMul(midN, midN)));
    const Ff a2s = ffSub(ffMul(a2, midN), ffMul(c2, midN));
    const Ff nv = ffAdd(nzf, ffProd(r.c.step, vz));
    const Ff endN = ffAdd(nv, ffMul(t.halfSquare, a2s));
    const Ff c3 = ffAdd(r.big, ffMul(twoA2, ffMul(endN, endN)));
    const Ff a3 = ffSub(ffMul(a2, endN), ffMul(c3, endN));
    nextNz = ffAdd(nv, ffMul(t.sixthSquare, ffAdd(a1, ffAdd(a2s, a2s))));
    nextVz = ffAdd(Ff{vz, 0.f}, ffMul(t.sixth, ffAdd(ffAdd(a1, a3), ffMulF(a2s, 4.f))));
}

/* The constants of motion alone, for an eye at rest (lens.inc:125-142 without the aberration of
 * 110-122), in double-float, in rayStartWith's order of operations with the direction normalised first: E,
 * the axial momentum xi, eta and K = eta + xi^2 and the radial equation's coefficients, rounded to float
 * (a pair's hi is its value rounded to nearest) into r.c, the five the wide sub-steps take into r as
 * pairs, and the factors the first state is made of (d_x, 1 / (|d| E), across and the axial component
 * of the direction over E), which the caller forms in FP32 as the reference's integrator has them. */
__device__ __forceinline__ void motionConstantsFf(const MotionTermsFf& t, float nx, float ny, MixedRay& r,
                                                  float& dx, float& over, float& across, float& xiAxis) {
    Ff d[3];
    for (int k = 0; k < 3; ++k) d[k] = ffAdd(ffAdd(t.forward[k], ffMulF(t.right[k], nx)), ffMulF(t.up[k], ny));
    const Ff invLength = ffRsqrt(ffAdd(ffAdd(ffMul(d[0], d[0]), ffMul(d[1], d[1])), ffMul(d[2], d[2])));
    const Ff dz = ffMul(d[2], invLength);
    const Ff invEnergy = ffRecip(ffSub(t.metric[0], ffMul(t.metric[1], dz)));
    const Ff overFf = ffMul(invLength, invEnergy);
    const Ff xi = ffNeg(ffMul(ffMul(t.metric[2], dz), invEnergy));
    const Ff xiAxisFf = ffMul(ffMul(t.metric[3], d[2]), overFf);
    const Ff acrossFf = ffMul(ffMul(t.rho, d[1]), overFf);
    const Ff eta = ffAdd(ffMul(acrossFf, acrossFf), ffMul(t.mu0Squared, ffSub(ffMul(xiAxisFf, xiAxisFf), t.a2)));
    const Ff big = ffAdd(eta, ffMul(xi, xi));
    const Ff uA = ffSub(t.a2, big);
    const Ff xiOff = ffSub(xi, t.a);
    const Ff uB = ffMulF(ffAdd(eta, ffMul(xiOff, xiOff)), 3.f);
    const Ff uC = ffMul(t.minusTwoA2, eta);
    const Ff xiA = ffMul(xi, t.a);
    r.c.invEnergy = invEnergy.hi, r.c.xi = xi.hi, r.c.moved = 1.f;
    r.c.big = big.hi, r.c.uA = uA.hi, r.c.uB = uB.hi, r.c.uC = uC.hi, r.c.xiA = xiA.hi;
    r.big = big, r.uA = uA, r.uB = uB, r.uC = uC, r.xiA = xiA;
    dx = d[0].hi, over = overFf.hi, across = acrossFf.hi, xiAxis = xiAxisFf.hi;
}

/* The helpers below take the guards apart from the parameters, so that a kernel built for all of them
 * passes a constant and its tests fold away. */

/* A ray's start: its constants of motion and first state, in double-float under the MOTION guard. */
__device__ __forceinline__ void mixedStart(const MixedParams& p, uint32_t guards, const MixedView& v, float nx,
                                           float ny, float time, MixedRay& r) {
    if ((guards & ARTF_CUDA_GUARD_MOTION) && v.d.boost[3] > 1.0) {
        /* a moving eye: the whole set-up with its aberration in FP64 */
        RayConst<double> cd;
        RayState<double> sd;
        rayStartWith(v.d, v.start64, widen(nx), widen(ny), widen(time), cd, sd);
        r.c.invEnergy = narrow(cd.invEnergy), r.c.xi = narrow(cd.xi), r.c.moved = narrow(cd.moved);
        r.c.big = narrow(cd.big), r.c.step = narrow(cd.step), r.c.uA = narrow(cd.uA), r.c.uB = narrow(cd.uB);
        r.c.uC = narrow(cd.uC), r.c.xiA = narrow(cd.xiA);
        r.big = ffSplit(cd.big), r.step = cd.step, r.uA = ffSplit(cd.uA), r.uB = ffSplit(cd.uB);
        r.uC = ffSplit(cd.uC), r.xiA = ffSplit(cd.xiA);
        r.s.u = v.startNarrow[3], r.s.w = narrow(sd.w);
        for (int k = 0; k < 3; ++k) r.s.n[k] = v.startNarrow[k], r.s.v[k] = narrow(sd.v[k]);
    } else if (guards & ARTF_CUDA_GUARD_MOTION) {
        float dx, over, across, xiAxis;
        motionConstantsFf(v.motion, nx, ny, r, dx, over, across, xiAxis);
        r.c.step = divSqrtR(v.stepBaseNarrow, maxX(r.c.big, 4.f));
        r.step = widen(r.c.step);
        /* (u and n start at the eye's: the view's, narrowed once) */
        r.s.u = v.startNarrow[3];
        r.s.w = v.wScaleNarrow * dx * over;
        for (int k = 0; k < 3; ++k)
            r.s.n[k] = v.startNarrow[k], r.s.v[k] = across * v.f.etheta[k] + xiAxis * v.f.ephi[k];
    } else {
        rayStart(v.f, nx, ny, time, p.stepScale, r.c, r.s);
        r.big = Ff{r.c.big, 0.f}, r.step = r.c.step, r.uA = Ff{r.c.uA, 0.f}, r.uB = Ff{r.c.uB, 0.f};
        r.uC = Ff{r.c.uC, 0.f}, r.xiA = Ff{r.c.xiA, 0.f};
    }
    r.c.time = time;
    r.s.psi = 0.f;
    r.s.drag = v.f.a != 0.f ? dragAt(v.f.a, v.f.a * v.f.a, r.c.xiA, r.s.u) : 0.f;
    r.psiHi = r.psiLo = 0.f;
    r.through = 1.f;
    r.sum[0] = r.sum[1] = r.sum[2] = 0.f;
    r.hitR = r.hitPhi = NAN;
    r.i = 0;
    r.crossings = r.wide = 0;
    r.lit = false;
}

/* Which sub-steps of this FP32 step must run again wide. */
__device__ __forceinline__ void mixedNeeds(uint32_t guards, const MixedView& v, const MixedRay& r,
                                           const StepOut<float>& o, bool& radial, bool& polar, unsigned& reason) {
    const bool band = (guards & ARTF_CUDA_GUARD_HORIZON) && r.s.u > v.uGuard;
    const bool turnR = (guards & ARTF_CUDA_GUARD_RADIAL) && ((r.s.w > 0.f) != (o.next.w > 0.f));
    polar = (guards & ARTF_CUDA_GUARD_POLAR) && ((r.s.v[2] > 0.f) != (o.next.v[2] > 0.f));
    radial = band || turnR;
    reason = (band ? 1u : 0u) | (turnR && !band ? 2u : 0u) | (polar ? 4u : 0u);
}

/* The wide sub-steps, with the ray's step terms (stepTermsFf, formed once a ray).  Radial: in the
 * horizon's band the whole sub-step in FP64 (the frame-drag rate's Delta / r^2 cancels there, and it
 * divides), from the pairs widened; at a turning point of u the motion (u, du/ds) alone in double-float,
 * psi and its rate staying the FP32 step's. */
__device__ __forceinline__ void radialWide(const MixedView& v, const MixedRay& r, const StepTermsFf& t, bool band,
                                           StepOut<float>& o) {
    if (band) {
        const RayConst<double> c = wideConst(r);
        double k1;
        RayState<double> s, next;
        s.u = widen(r.s.u), s.w = widen(r.s.w), s.psi = 0.0, s.drag = widen(r.s.drag);
        radialStepWith(v.d.a, v.wideA2, c, wideTerms(t), s, next, k1);
        o.next.u = narrow(next.u), o.next.w = narrow(next.w), o.next.psi = narrow(next.psi);
        o.next.drag = narrow(next.drag);
        o.k1 = narrow(k1);
    } else {
        Ff u, w, k1;
        radialMotionFf(r, t, r.s.u, r.s.w, u, w, k1);
        o.next.u = u.hi, o.next.w = w.hi, o.k1 = k1.hi;
    }
}

/* Polar: at the turning point of n_z, the axis component (n_z, dn_z/ds); the components about the axis
 * stay the FP32 step's. */
__device__ __forceinline__ void polarWide(const MixedView& v, const MixedRay& r, const StepTermsFf& t,
                                          StepOut<float>& o) {
    Ff nz, vz, a1z;
    polarAxisFf(v.motion.a2, r, t, r.s.n[2], r.s.v[2], nz, vz, a1z);
    o.next.n[2] = nz.hi, o.next.v[2] = vz.hi, o.a1[2] = a1z.hi;
}

/* After a step: the disc crossing, escape, horizon, opacity and the step cap.  Returns the end's kind
 * (ARTF_CUDA_END_*) + 1, or 0 when the ray goes on. */
__device__ __forceinline__ unsigned mixedAdvance(const MixedParams& p, uint32_t guards, const MixedView& v,
                                                 MixedRay& r, const StepOut<float>& o) {
    const Frame<float>& f = v.f;
    const bool compensated = guards & ARTF_CUDA_GUARD_PSI;
    const float increment = o.next.psi;
    Crossing<float> x;
    if (crossingOf(f, v.rhoScale, r.c, r.s, o, x)) {
        x.psiC = compensated ? r.psiHi + (r.psiLo + x.part * increment) : r.psiHi + x.part * increment;
        ++r.crossings;
        float turn;
        const float light = shadeCrossing(f, v.rhoScale, v.map, v.fluid, r.c, x, r.through, r.sum, &turn);
        if (light > 0.f && !r.lit) {
            r.lit = true;
            r.hitR = 1.f / x.uc;
            r.hitPhi = turn - floorf(turn);
        }
    }
    ++r.i;
    if (0.f > o.next.u) {
        const float part = r.s.u / (r.s.u - o.next.u);
        float away[3], dir[3];
        for (int k = 0; k < 3; ++k) away[k] = r.s.n[k] + part * (o.next.n[k] - r.s.n[k]);
        const float awayPsi = compensated ? r.psiHi + (r.psiLo + part * increment) : r.psiHi + part * increment;
        skyDirection(away, awayPsi, dir);
        if (f.stars > 0.f) shadeSky(f, v.map, r.c, dir, r.through, r.sum);
        /* (the escape's direction and moment travel in the slots the ray no longer needs) */
        r.s.n[0] = dir[0], r.s.n[1] = dir[1], r.s.n[2] = dir[2];
        r.s.w = part;
        return ARTF_CUDA_END_SKY + 1;
    }
    if (o.next.u > f.uHorizon) return ARTF_CUDA_END_HORIZON + 1;
    if (!(r.through > .004f)) return ARTF_CUDA_END_OPAQUE + 1;
    if (compensated) {
        const float sumHi = r.psiHi + increment, back = sumHi - r.psiHi;
        r.psiLo += (r.psiHi - (sumHi - back)) + (increment - back);
        r.psiHi = sumHi;
    } else {
        r.psiHi += increment;
    }
    r.s = o.next;
    r.s.psi = 0.f;
    return r.i >= p.maxSteps ? ARTF_CUDA_END_CAP + 1 : 0u;
}

/* The end record of a finished ray, and its tallies. */
__device__ __forceinline__ unsigned mixedFinish(const MixedRay& r, unsigned ended, ArtfCudaRayEnd* end, Tally& t) {
    unsigned kind = ended - 1;
    if (r.lit) kind |= ARTF_CUDA_END_LIT;
    t.rays += 1;
    t.steps += (unsigned)r.i;
    t.crossings += r.crossings;
    const bool sky = (kind & 15u) == ARTF_CUDA_END_SKY;
    t.escapes += sky;
    if (end) {
        ArtfCudaRayEnd e;
        e.hitR = r.hitR;
        e.hitPhi = r.hitPhi;
        for (int k = 0; k < 3; ++k) e.dir[k] = sky ? r.s.n[k] : 0.f;
        e.mino = (float)(sky ? ((double)(r.i - 1) + (double)r.s.w) * r.step : (double)r.i * r.step);
        e.steps = (uint16_t)r.i;
        e.crossings = (uint8_t)(r.crossings > 255u ? 255u : r.crossings);
        e.kind = (uint8_t)kind;
        e.fp64Steps = (uint16_t)r.wide;
        e.reserved = 0;
        *end = e;
    }
    return kind;
}

struct Reasons {
    unsigned wide = 0, horizon = 0, radial = 0, polar = 0, rounds = 0;
};

__device__ __forceinline__ void countReason(unsigned reason, Reasons& n) {
    n.wide += 1;
    n.horizon += reason & 1u;
    n.radial += (reason >> 1) & 1u;
    n.polar += (reason >> 2) & 1u;
}

/* The per-ray path: one ray from start to end, each step's wide sub-steps at once. */
__device__ __forceinline__ unsigned traceRayMixed(const MixedParams& p, const MixedView& v, float nx, float ny,
                                                  float time, float* sum, ArtfCudaRayEnd* end, Tally& t, Reasons& n) {
    MixedRay r;
    mixedStart(p, p.guards, v, nx, ny, time, r);
    unsigned ended = 0;
    while (!ended) {
        StepOut<float> o;
        nystromStep(v.f.a, r.c, r.s, o);
        bool radial, polar;
        unsigned reason;
        mixedNeeds(p.guards, v, r, o, radial, polar, reason);
        if (radial || polar) {
            const StepTermsFf terms = stepTermsFf(r.c.step);
            if (radial) radialWide(v, r, terms, (reason & 1u) != 0u, o);
            if (polar) polarWide(v, r, terms, o);
        }
        if (radial || polar) {
            ++r.wide;
            countReason(reason, n);
        }
        ended = mixedAdvance(p, p.guards, v, r, o);
    }
    for (int k = 0; k < 3; ++k) sum[k] = sum[k] + r.sum[k];
    return mixedFinish(r, ended, end, t);
}

__device__ __forceinline__ void flushReasons(const Reasons& n, unsigned long long* counters) {
    const unsigned wide = __reduce_add_sync(0xFFFFFFFFu, n.wide);
    const unsigned horizon = __reduce_add_sync(0xFFFFFFFFu, n.horizon);
    const unsigned radial = __reduce_add_sync(0xFFFFFFFFu, n.radial);
    const unsigned polar = __reduce_add_sync(0xFFFFFFFFu, n.polar);
    const unsigned rounds = __reduce_add_sync(0xFFFFFFFFu, n.rounds);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters + CFp64Steps, (unsigned long long)wide);
        atomicAdd(counters + CFp64Horizon, (unsigned long long)horizon);
        atomicAdd(counters + CFp64Radial, (unsigned long long)radial);
        atomicAdd(counters + CFp64Polar, (unsigned long long)polar);
        atomicAdd(counters + CFp64Rounds, (unsigned long long)rounds);
    }
}

/* The view a queue unit belongs to: the last whose first unit is at or below it. */
__device__ __forceinline__ int viewOf(const MixedParams& p, int unit) {
    int lo = 0, hi = p.viewCount - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&p.views[mid].unitBase) <= unit) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* ---- heavy first --------------------------------------------------------------------------------
 * After the queue empties the persistent grid drains, and a lane that took a long ray late holds its SM
 * while the others idle (a photon-ring ray runs to the step cap, ten times a sky ray's steps).  So the
 * queue hands out the heaviest tiles first and leaves short rays for the end.  A tile's weight is the
 * step count of one FP32 ray through its middle, stepped without shading (the disc is thin: it seldom
 * ends a ray) up to 64 steps (a sky ray takes about 25; what goes on longer is heavy); tiles are
 * counting-sorted by weight class, heaviest first.  The order changes when a ray is traced, never what
 * it computes, so the frame is the same bits in any order. */

constexpr int kWeightClasses = 9; /* steps / 8 up to 64: the probe stops there (all heavier tiles, class 8) */
constexpr int kProbeSteps = 64;

/* The view a batch-wide tile belongs to: the last whose first tile is at or below it. */
__device__ __forceinline__ int tileView(const MixedParams& p, int tile) {
    int lo = 0, hi = p.viewCount - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&p.views[mid].tileBase) <= tile) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

/* Each tile's weight class, and each class's count of queue slots (a tile has one a ray plane), counted
 * in the block first so that each class takes one global atomic a block. */
__global__ void __launch_bounds__(128) probeTiles(const MixedParams p, int totalTiles, int* weights,
                                                  unsigned* classes) {
    __shared__ unsigned counts[kWeightClasses];
    if (threadIdx.x < kWeightClasses) counts[threadIdx.x] = 0;
    __syncthreads();
    const int g = (int)(blockIdx.x * 128 + threadIdx.x);
    if (g < totalTiles) {
        const MixedView& v = p.views[tileView(p, g)];
        const int tile = g - v.tileBase;
        const int x = min((tile % v.tilesX) * 8 + 4, (int)v.f.width - 1);
        const int y = min(v.rowBegin + (tile / v.tilesX) * 4 + 2, v.rowBegin + v.rows - 1);
        float nx, ny, moment;
        samplePosition(v.h, v.jitter, v.seed, x, y, 0, &nx, &ny, &moment);
        RayConst<float> c;
        RayState<float> s;
        rayStart(v.f, nx, ny, v.h.disc[2] + v.h.spin[3] * moment, p.stepScale, c, s);
        const float a = v.f.a;
        if (a != 0.f) s.drag = dragAt(a, a * a, c.xiA, s.u);
        const int most = min(p.maxSteps, kProbeSteps);
        int i = 0;
        while (i < most) {
            StepOut<float> o;
            nystromStep(a, c, s, o);
            ++i;
            if (0.f > o.next.u || o.next.u > v.f.uHorizon) break;
            s = o.next;
        }
        const int w = min(i >> 3, kWeightClasses - 1);
        weights[g] = w;
        atomicAdd(counts + w, v.rayOut ? (unsigned)v.rays : 1u);
    }
    __syncthreads();
    if (threadIdx.x < kWeightClasses && counts[threadIdx.x]) atomicAdd(classes + threadIdx.x, counts[threadIdx.x]);
}

/* Each tile's slots into the order, its planes together, heavier classes first (within a class in the
 * order the atomics give): a block reserves each class's run with one global atomic, its tiles take
 * places within the run by shared ones. */
__global__ void __launch_bounds__(128) placeTiles(const MixedParams p, int totalTiles, const int* weights,
                                                  const unsigned* classes, unsigned* cursors, uint2* order) {
    __shared__ unsigned counts[kWeightClasses], runs[kWeightClasses];
    if (threadIdx.x < kWeightClasses) counts[threadIdx.x] = 0;
    __syncthreads();
    const int g = (int)(blockIdx.x * 128 + threadIdx.x);
    const bool active = g < totalTiles;
    int vi = 0, w = 0;
    unsigned planes = 0, within = 0;
    if (active) {
        vi = tileView(p, g);
        w = weights[g];
        planes = p.views[vi].rayOut ? (unsigned)p.views[vi].rays : 1u;
        within = atomicAdd(counts + w, planes);
    }
    __syncthreads();
    if (threadIdx.x < kWeightClasses) {
        unsigned before = 0;
        for (int c = kWeightClasses - 1; c > (int)threadIdx.x; --c) before += classes[c];
        runs[threadIdx.x] = counts[threadIdx.x] ? before + atomicAdd(cursors + threadIdx.x, counts[threadIdx.x]) : 0u;
    }
    __syncthreads();
    if (!active) return;
    const unsigned at = runs[w] + within;
    const unsigned tile = (unsigned)(g - p.views[vi].tileBase);
    for (unsigned k = 0; k < planes; ++k) order[at + k] = make_uint2((unsigned)vi | k << 12, tile);
}

/* FP32 steps a lane takes between two of the warp's votes on refills and FP64 rounds (measured at
 * 1080p x 4: 3 steps 2.64 ms, 4 steps 2.62, 6 steps 2.60, 8 steps 2.60, 10 steps 2.62; the 64-view batch
 * alike). */
constexpr int kInnerSteps = 6;

/* This lane's step terms, from the block's table. */
__device__ __forceinline__ StepTermsFf laneTerms(const Ff (*terms)[256]) {
    StepTermsFf t;
    t.half = terms[0][threadIdx.x], t.eighth = terms[1][threadIdx.x], t.halfSquare = terms[2][threadIdx.x];
    t.sixthSquare = terms[3][threadIdx.x], t.sixth = terms[4][threadIdx.x];
    return t;
}

/* The warp-scheduled trace (see the file's head).  kOne: a single view, read from `one` (a kernel
 * parameter) rather than from the view table.  kAll: every guard on (the default), the step's tests of
 * them as constants. */
template <bool kOne, bool kAll>
__device__ __forceinline__ void mixedQueue(const MixedParams& p, const MixedView* one) {
    const uint32_t guards = kAll ? (uint32_t)ARTF_CUDA_GUARD_ALL : p.guards;
    /* each lane's ray's step terms as pairs, formed at its set-up: a wide round then loads them where
     * it would multiply them out again */
    __shared__ Ff terms[5][256];
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    Tally t;
    Reasons n;
    int unit = -1, x = 0, y = 0, k = 0, kEnd = 1; /* this lane's unit: rays k .. kEnd - 1 of pixel (x, y) */
    const MixedView* v = kOne ? one : p.views;
    bool exhausted = false, live = false, haveStep = false, waitR = false, waitP = false;
    unsigned reason = 0, bits = 0;
    float pixel[3] = {0.f, 0.f, 0.f};
    MixedRay r;
    StepOut<float> o;
    int sinceStart = 0, sinceRadial = 0, sincePolar = 0;
    /* Every iteration either advances some lane's ray by a step, starts rays, or ends the loop: the queue
     * is finite and a ray ends within maxSteps steps, so the loop ends. */
    for (;;) {
        /* (1) refill, batched: the set-up of a ray is wide work */
        const unsigned idle = __ballot_sync(full, !live && !exhausted);
        const unsigned liveMask = __ballot_sync(full, live);
        if (idle && (__popc(idle) >= p.refill || liveMask == 0 || sinceStart >= p.maxWait)) {
            sinceStart = 0;
            const bool needPixel = !live && !exhausted && (unit < 0 || k >= kEnd);
            const unsigned fetch = __ballot_sync(full, needPixel);
            if (fetch) {
                const int leader = __ffs(fetch) - 1;
                int base = 0;
                if (lane == leader) base = (int)atomicAdd(p.counters + CQueue, (unsigned long long)__popc(fetch));
                base = __shfl_sync(full, base, leader);
                if (needPixel) {
                    unit = base + __popc(fetch & below);
                    k = 0, bits = 0;
                    pixel[0] = pixel[1] = pixel[2] = 0.f;
                    if (unit >= p.totalUnits) {
                        exhausted = true;
                        unit = -1;
                    } else {
                        /* a slot of 32 units is one ray plane of one tile: a warp's lanes take
                         * neighbouring pixels */
                        int plane, tile;
                        const int within = unit & 31; /* (every view's first unit is a multiple of 32) */
                        if (p.order) {
                            const uint2 slot = __ldg(p.order + (unit >> 5));
                            if (!kOne) v = p.views + (slot.x & 4095u);
                            plane = v->rayOut ? (int)(slot.x >> 12) : 0;
                            tile = (int)slot.y;
                        } else {
                            if (!kOne) v = p.views + viewOf(p, unit);
                            int local = unit - v->unitBase;
                            plane = v->rayOut ? local / v->pixelUnits : 0;
                            local -= plane * v->pixelUnits;
                            tile = local >> 5;
                        }
                        x = (tile % v->tilesX) * 8 + (within & 7);
                        y = v->rowBegin + (tile / v->tilesX) * 4 + (within >> 3);
                        k = plane;
                        kEnd = v->rayOut ? plane + 1 : v->rays;
                        if (x >= v->f.width || y >= v->rowBegin + v->rows) k = kEnd; /* (off the band: fetch again) */
                    }
                }
            }
            if (!live && unit >= 0 && k < kEnd) {
                float nx, ny, moment;
                samplePosition(v->h, v->jitter, v->seed, x, y, k, &nx, &ny, &moment);
                /* (the set-up keeps its guard test at run time: made constant there too, the batch ran
                 * 7.61 ms against 7.13, a matter of code layout) */
                mixedStart(p, p.guards, *v, nx, ny, v->h.disc[2] + v->h.spin[3] * moment, r);
                const StepTermsFf t = stepTermsFf(r.c.step);
                terms[0][threadIdx.x] = t.half, terms[1][threadIdx.x] = t.eighth;
                terms[2][threadIdx.x] = t.halfSquare, terms[3][threadIdx.x] = t.sixthSquare;
                terms[4][threadIdx.x] = t.sixth;
                live = true;
            }
        } else if (idle) {
            ++sinceStart;
        }
        if (__all_sync(full, exhausted && !live)) break;

        /* (2) wide rounds, when enough lanes wait or no other lane can move */
        const unsigned ready = __ballot_sync(full, live && !waitR && !waitP);
        const unsigned needR = __ballot_sync(full, waitR), needP = __ballot_sync(full, waitP);
        if (needR && (__popc(needR) >= p.batch || ready == 0 || sinceRadial >= p.maxWait)) {
            if (waitR) {
                radialWide(*v, r, laneTerms(terms), (reason & 1u) != 0u, o);
                waitR = false;
            }
            sinceRadial = 0;
            n.rounds += lane == 0;
        } else if (needR) {
            ++sinceRadial;
        }
        if (needP && (__popc(needP) >= p.batch || ready == 0 || sincePolar >= p.maxWait)) {
            if (waitP) {
                polarWide(*v, r, laneTerms(terms), o);
                waitP = false;
            }
            sincePolar = 0;
            n.rounds += lane == 0;
        } else if (needP) {
            ++sincePolar;
        }
        /* (3) up to kInnerSteps FP32 steps a lane between the warp's votes: a lane commits its complete
         * step (one a round just finished, or a plain one) and takes the next, until a step needs an FP64
         * sub-step or the ray ends */
        for (int j = 0; j < kInnerSteps; ++j) {
            if (haveStep && !waitR && !waitP) {
                haveStep = false;
                const unsigned ended = mixedAdvance(p, guards, *v, r, o);
                if (ended) {
                    const size_t index = (size_t)y * (size_t)v->f.width + (size_t)x;
                    const int64_t pixels = (int64_t)v->f.width * v->f.height;
                    ArtfCudaRayEnd* end = v->ends && inBounds(v->f.fault, kBoundsRayEnd,
                                                              (int64_t)(index * (size_t)v->rays + (size_t)k),
                                                              pixels * v->rays)
                                              ? v->ends + index * (size_t)v->rays + (size_t)k
                                              : nullptr;
                    const unsigned rayBits = classBits(mixedFinish(r, ended, end, t));
                    live = false;
                    if (v->rayOut) {
                        /* (a plane holds the band's pixels) */
                        const size_t plane = (size_t)v->f.width * (size_t)v->rows;
                        const size_t inBand = (size_t)(y - v->rowBegin) * (size_t)v->f.width + (size_t)x;
                        if (inBounds(v->f.fault, kBoundsRayPlane, (int64_t)((size_t)k * plane + inBand),
                                     (int64_t)plane * v->rays))
                            v->rayOut[(size_t)k * plane + inBand] =
                                make_float4(r.sum[0], r.sum[1], r.sum[2], (float)rayBits);
                        ++k;
                    } else {
                        bits |= rayBits;
                        for (int c = 0; c < 3; ++c) pixel[c] = pixel[c] + r.sum[c];
                        if (++k == kEnd && inBounds(v->f.fault, kBoundsPixel, (int64_t)index, pixels))
                            v->hdr[index] = make_float4(pixel[0] * v->share, pixel[1] * v->share,
                                                        pixel[2] * v->share, (float)bits);
                    }
                }
            }
            if (live && !haveStep) {
                nystromStep(v->f.a, r.c, r.s, o);
                mixedNeeds(guards, *v, r, o, waitR, waitP, reason);
                haveStep = true;
                if (waitR || waitP) {
                    ++r.wide;
                    countReason(reason, n);
                }
            }
        }
    }
    flushTally(t, p.counters);
    flushReasons(n, p.counters);
}

/* The views from the table (a batch).  The kernels come in pairs: the guards chosen at run time, and all
 * of them as constants, which every trace with all guards runs (frames, bands and batches alike, so that
 * their bits agree): its dead branches fold away and its code is smaller. */
__global__ void __launch_bounds__(256) traceMixedQueue(const MixedParams p) { mixedQueue<false, false>(p, nullptr); }
__global__ void __launch_bounds__(256) traceMixedQueueAll(const MixedParams p) { mixedQueue<false, true>(p, nullptr); }

/* A single view (a frame) as a kernel parameter: its fields are then read from the constant bank where
 * they are used, not loaded from the view table in global memory at every step. */
__global__ void __launch_bounds__(256) traceMixedQueueOne(const MixedParams p, const __grid_constant__ MixedView view) {
    mixedQueue<true, false>(p, &view);
}
__global__ void __launch_bounds__(256) traceMixedQueueOneAll(const MixedParams p,
                                                             const __grid_constant__ MixedView view) {
    mixedQueue<true, true>(p, &view);
}

/* Each pixel of the views with ray planes: its rays' radiance summed in ray order and scaled by
 * 1 / rays, and their class bits; the same operations, in the same order, as the per-pixel path. */
__global__ void __launch_bounds__(256) mixedCombine(const MixedView* views) {
    const MixedView& v = views[blockIdx.y];
    if (!v.rayOut) return;
    const size_t pixels = (size_t)v.f.width * (size_t)v.rows; /* the band's */
    const size_t i = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (i >= pixels) return;
    float sum[3] = {0.f, 0.f, 0.f};
    unsigned bits = 0;
    for (int k = 0; k < v.rays; ++k) {
        const float4 q = v.rayOut[(size_t)k * pixels + i];
        sum[0] = sum[0] + q.x, sum[1] = sum[1] + q.y, sum[2] = sum[2] + q.z;
        bits |= (unsigned)q.w;
    }
    const size_t at = (size_t)v.rowBegin * (size_t)v.f.width + i;
    if (inBounds(v.f.fault, kBoundsPixel, (int64_t)at, (int64_t)v.f.width * v.f.height))
        v.hdr[at] = make_float4(sum[0] * v.share, sum[1] * v.share, sum[2] * v.share, (float)bits);
}

/* The per-ray entry point: rays at given image positions in the table's first view. */
__global__ void __launch_bounds__(128) traceMixedList(const MixedParams p, const int count, const float* nx,
                                                      const float* ny, const float* time, float* rgb) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Tally t;
    Reasons n;
    if (i < count) {
        float sum[3] = {0.f, 0.f, 0.f};
        const MixedView& v = p.views[0];
        traceRayMixed(p, v, nx[i], ny[i], time[i], sum, v.ends ? v.ends + i : nullptr, t, n);
        for (int k = 0; k < 3; ++k) rgb[3 * i + k] = sum[k];
    }
    flushTally(t, p.counters);
    flushReasons(n, p.counters);
}

MixedParams paramsOf(const TraceLaunch& l, const void* deviceTable, int viewCount, int totalUnits) {
    MixedParams p;
    p.views = (const MixedView*)deviceTable;
    p.viewCount = viewCount;
    p.totalUnits = totalUnits;
    p.counters = l.counters;
    p.stepScale = l.stepScale;
    p.maxSteps = l.stepScale < .75f ? 384 : 192;
    p.guards = l.guards ? l.guards : ARTF_CUDA_GUARD_ALL;
    p.batch = l.fp64Batch > 0 ? (l.fp64Batch > 32 ? 32 : l.fp64Batch) : 32;
    p.refill = l.refillBatch > 0 ? (l.refillBatch > 32 ? 32 : l.refillBatch) : 32;
    /* (256 votes: the best of the autotuner's choices on both the 1080p frame and the 64-view batch) */
    p.maxWait = l.compactEvery > 0 ? l.compactEvery : 256;
    p.order = nullptr;
    return p;
}

}  // namespace

namespace {

/* widen against the hardware's float-to-double conversion, on every float bit pattern (256 a thread);
 * bad[0] counts differing results (two NaNs agree), bad[2] keeps the least differing input. */
__global__ void __launch_bounds__(256) checkWiden(unsigned long long* bad) {
    const uint32_t first = (blockIdx.x * 256u + threadIdx.x) << 8;
    for (uint32_t k = 0; k < 256u; ++k) {
        const float f = __uint_as_float(first | k);
        const double want = (double)f, got = widen(f);
        const bool same = (want != want && got != got) || __double_as_longlong(want) == __double_as_longlong(got);
        if (!same) {
            atomicAdd(bad, 1ull);
            atomicMin(bad + 2, (unsigned long long)(first | k));
        }
    }
}

__device__ __forceinline__ unsigned long long mixBits(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* narrow against the hardware's double-to-float conversion, on `perThread` doubles a thread: exponents
 * around float's range and random fractions, a quarter of them with the 29 bits rounding looks at set
 * to a tie or next to one, an eighth with the kept bits all ones; one in sixteen a random bit pattern.
 * bad[1] counts differing results, bad[3] keeps the least differing input. */
__global__ void __launch_bounds__(256) checkNarrow(unsigned long long* bad, uint32_t perThread) {
    const unsigned long long id = blockIdx.x * 256ull + threadIdx.x;
    for (uint32_t k = 0; k < perThread; ++k) {
        const unsigned long long r = mixBits(id * perThread + k), s = mixBits(r);
        unsigned long long bits;
        if ((r & 15u) == 0u) {
            bits = s;
        } else {
            const unsigned long long e = 880u + (r >> 8) % 290u;
            unsigned long long fraction = s & 0xFFFFFFFFFFFFFull;
            const uint32_t rests[4] = {0x10000000u, 0x0FFFFFFFu, 0x10000001u, 0u};
            if (((r >> 4) & 3u) == 0u) fraction = (fraction & ~0x1FFFFFFFull) | rests[(r >> 6) & 3u];
            if (((r >> 20) & 7u) == 0u) fraction |= 0x7FFFFFull << 29;
            bits = ((r >> 63) << 63) | (e << 52) | fraction;
        }
        const double d = __longlong_as_double((long long)bits);
        const float want = (float)d, got = narrow(d);
        const bool same = (want != want && got != got) || __float_as_uint(want) == __float_as_uint(got);
        if (!same) {
            atomicAdd(bad + 1, 1ull);
            atomicMin(bad + 3, bits);
        }
    }
}

}  // namespace

size_t mixedViewBytes() { return sizeof(MixedView); }

int mixedFillView(const TraceLaunch& l, const ArtfCudaHoleFrame& frame, const ArtfCudaHoleFrame64& frame64,
                  const float* map, const float* fluid, float4* hdr, ArtfCudaRayEnd* ends, float4* rayOut, int unitBase,
                  int tileBase, void* slot, int* tiles) {
    MixedView v;
    memset(&v, 0, sizeof v);
    v.f.load(frame64, frame);
    v.d.load(frame64, frame);
    v.f.fault = v.d.fault = l.counters + CBoundsKind;
    v.h = frame;
    v.map = map;
    v.fluid = fluid;
    v.hdr = hdr;
    v.ends = ends;
    v.wideA2 = v.d.a * v.d.a;
    v.start64 = startTerms(v.d, (double)l.stepScale);
    for (int k = 0; k < 3; ++k) v.startNarrow[k] = (float)v.d.er[k];
    v.startNarrow[3] = (float)v.d.place[2];
    v.wScaleNarrow = (float)v.start64.wScale;
    v.stepBaseNarrow = (float)v.start64.stepBase;
    auto split = [](double x) {
        const float hi = (float)x;
        return Ff{hi, (float)(x - (double)hi)};
    };
    for (int k = 0; k < 3; ++k) {
        v.motion.forward[k] = split(v.d.forward[k]);
        v.motion.right[k] = split(v.d.right[k]);
        v.motion.up[k] = split(v.d.up[k]);
    }
    for (int k = 0; k < 4; ++k) v.motion.metric[k] = split(v.d.metric[k]);
    v.motion.rho = split(v.d.place[0]), v.motion.a = split(v.d.a), v.motion.a2 = split(v.start64.a2);
    v.motion.mu0Squared = split(v.start64.mu0Squared), v.motion.minusTwoA2 = split(v.start64.minusTwoA2);
    v.rhoScale = 1.f / (1.f - v.f.inner / v.f.outer);
    v.uGuard = (float)((double)(l.horizonBand > 0.f ? l.horizonBand : .95f) * frame64.spin[1]);
    v.rays = l.jitter ? l.jitter : (int)(frame.size[2] * frame.size[2]);
    v.share = l.jitter ? 1.f / (float)l.jitter : frame.image[3];
    v.jitter = l.jitter;
    v.seed = l.seed;
    v.tilesX = ((int)frame.size[0] + 7) / 8;
    const int tileRows = ((int)frame.size[1] + 3) / 4;
    const int bandBegin = l.tileRows > 0 ? l.tileRowBegin : 0, bandRows = l.tileRows > 0 ? l.tileRows : tileRows;
    v.rowBegin = bandBegin * 4;
    v.rows = (bandBegin + bandRows) * 4 < (int)frame.size[1] ? bandRows * 4 : (int)frame.size[1] - v.rowBegin;
    v.pixelUnits = v.tilesX * bandRows * 32;
    v.rayOut = v.rays > 1 ? rayOut : nullptr; /* (one ray a pixel: the pixel is the ray) */
    v.units = v.pixelUnits * (v.rayOut ? v.rays : 1);
    v.unitBase = unitBase;
    v.tileBase = tileBase;
    memcpy(slot, &v, sizeof v);
    *tiles = v.tilesX * bandRows;
    return v.units;
}

/* The heavy-first scratch: the weight classes' counts and cursors, a weight a tile, a slot a 32 units. */
constexpr size_t kOrderHead = 2 * 32 * sizeof(unsigned);

size_t mixedOrderBytes(int totalTiles, int totalUnits) {
    const size_t weights = ((size_t)totalTiles * sizeof(int) + 15) & ~(size_t)15;
    return kOrderHead + weights + (size_t)(totalUnits / 32) * sizeof(uint2);
}

int mixedGrid(const TraceLaunch& l, int totalUnits, const void* kernel) {
    const int block = l.blockSize > 0 ? l.blockSize : 128;
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, block, 0);
    int grid = (perSm > 0 ? perSm : 1) * l.smCount;
    const int needed = (totalUnits + block - 1) / block;
    return grid > needed ? needed : (grid < 1 ? 1 : grid);
}

cudaError_t launchMixedTable(const TraceLaunch& l, const void* deviceTable, int viewCount, int totalUnits,
                             size_t combinePixels, int totalTiles, void* orderScratch, const void* hostView) {
    MixedParams p = paramsOf(l, deviceTable, viewCount, totalUnits);
    const int block = l.blockSize > 0 ? l.blockSize : 128;
    if (l.rayCount > 0) {
        traceMixedList<<<(l.rayCount + 127) / 128, 128, 0, l.stream>>>(p, l.rayCount, l.rayX, l.rayY, l.rayTime,
                                                                       l.rayRgb);
        return cudaGetLastError();
    }
    if (orderScratch && l.order == ARTF_CUDA_ORDER_HEAVY_FIRST && totalTiles > 0) {
        unsigned* classes = (unsigned*)orderScratch;
        unsigned* cursors = classes + 32;
        int* weights = (int*)((char*)orderScratch + kOrderHead);
        uint2* order = (uint2*)((char*)weights + (((size_t)totalTiles * sizeof(int) + 15) & ~(size_t)15));
        const cudaError_t e = cudaMemsetAsync(orderScratch, 0, kOrderHead, l.stream);
        if (e != cudaSuccess) return e;
        const unsigned grid = (unsigned)((totalTiles + 127) / 128);
        probeTiles<<<grid, 128, 0, l.stream>>>(p, totalTiles, weights, classes);
        placeTiles<<<grid, 128, 0, l.stream>>>(p, totalTiles, weights, classes, cursors, order);
        p.order = order;
    }
    const bool all = p.guards == ARTF_CUDA_GUARD_ALL;
    if (hostView && viewCount == 1) {
        MixedView one;
        memcpy(&one, hostView, sizeof one);
        const void* kernel = all ? (const void*)traceMixedQueueOneAll : (const void*)traceMixedQueueOne;
        const int grid = mixedGrid(l, totalUnits, kernel);
        if (all) traceMixedQueueOneAll<<<grid, block, 0, l.stream>>>(p, one);
        else traceMixedQueueOne<<<grid, block, 0, l.stream>>>(p, one);
    } else {
        const void* kernel = all ? (const void*)traceMixedQueueAll : (const void*)traceMixedQueue;
        const int grid = mixedGrid(l, totalUnits, kernel);
        if (all) traceMixedQueueAll<<<grid, block, 0, l.stream>>>(p);
        else traceMixedQueue<<<grid, block, 0, l.stream>>>(p);
    }
    if (combinePixels > 0)
        mixedCombine<<<dim3((unsigned)((combinePixels + 255) / 256), (unsigned)viewCount), 256, 0, l.stream>>>(p.views);
    return cudaGetLastError();
}

}  // namespace artf

namespace artf {
int failWith(int status, const char* message);

namespace {
/* The pair arithmetic the wide sub-steps use, one record a thread: (a.hi, a.lo, b.hi, b.lo) in,
 * a + b, a b, 1 / a and 1 / sqrt(|a|) out, each as (hi, lo). */
__global__ void checkPairs(const float4* in, float* out, int count) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= count) return;
    const float4 r = in[i];
    const Ff a{r.x, r.y}, b{r.z, r.w};
    const Ff sum = ffAdd(a, b), product = ffMul(a, b), recip = ffRecip(a);
    const Ff root = ffRsqrt(Ff{fabsf(a.hi), a.hi < 0.f ? -a.lo : a.lo});
    float* o = out + (size_t)i * 8;
    o[0] = sum.hi, o[1] = sum.lo, o[2] = product.hi, o[3] = product.lo;
    o[4] = recip.hi, o[5] = recip.lo, o[6] = root.hi, o[7] = root.lo;
}
}  // namespace
}  // namespace artf

extern "C" int artfCudaCheckPairs(void* stream, const float* hostIn, int count, float* hostOut) {
    if (!hostIn || !hostOut || count < 1 || count > (1 << 24))
        return artf::failWith(ARTF_CUDA_EINVAL, "pairs check: inputs, outputs and 1 .. 2^24 records");
    const cudaStream_t s = (cudaStream_t)stream;
    void* buffer = nullptr;
    const size_t inBytes = sizeof(float) * 4 * (size_t)count, outBytes = sizeof(float) * 8 * (size_t)count;
    cudaError_t e = cudaMalloc(&buffer, inBytes + outBytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return artf::failWith(ARTF_CUDA_ENOMEM, "pairs check: device allocation");
    }
    float4* in = (float4*)buffer;
    float* out = (float*)((char*)buffer + inBytes);
    e = cudaMemcpyAsync(in, hostIn, inBytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        artf::checkPairs<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(in, out, count);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hostOut, out, outBytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buffer);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaCheckConversions(void* stream, uint64_t narrowCount, uint64_t* mismatches) {
    if (!mismatches) return artf::failWith(ARTF_CUDA_EINVAL, "mismatches is NULL");
    const cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* bad = nullptr;
    cudaError_t e = cudaMalloc(&bad, sizeof(unsigned long long) * 4);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ENOMEM, "conversion check: device allocation");
    const unsigned long long init[4] = {0ull, 0ull, ~0ull, ~0ull};
    e = cudaMemcpyAsync(bad, init, sizeof init, cudaMemcpyHostToDevice, s);
    const uint32_t threads = 1u << 20;
    const uint32_t perThread = (uint32_t)((narrowCount + threads - 1) / threads);
    if (e == cudaSuccess) {
        artf::checkWiden<<<1u << 16, 256, 0, s>>>(bad); /* 2^24 threads x 256: every float */
        if (perThread > 0) artf::checkNarrow<<<threads / 256, 256, 0, s>>>(bad, perThread);
        e = cudaGetLastError();
    }
    unsigned long long out[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, bad, sizeof out, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(bad);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    for (int k = 0; k < 4; ++k) mismatches[k] = out[k];
    return ARTF_CUDA_OK;
}
