/* artful_cuda — one ray around a Kerr hole, for one GPU thread: the integrator, the disc crossing and
 * its shading, and the sky.  Generic in the arithmetic type R (float or double).  Each translation
 * unit that instantiates it fixes how float rounds by its compile flags: lensExact.cu without
 * contraction and with IEEE / and sqrt (the reference's bits), lensFast.cu with fused multiply-adds
 * and fast reciprocals.
 *
 * The physics and its discretisation are the reference's (eugeniobenfica/artful v0.4.0,
 * src/software/lens.inc): Carter-separated null geodesics in Mino time with u = 1/r, a unit vector n on
 * the sphere and the frame-drag angle psi,
 *     u'' = u (uA + u (uB + u uC)),   n'' = -(K + 2 a^2 m^2) n + a^2 m z,   psi' = -a u (2 - a xi u) / (1 - 2u + a^2 u^2),
 * integrated by a fixed-step three-stage Nystrom method of step (pi/24) / sqrt(max(K, 4)), at most 192
 * steps (lens.inc:3-23, 133, 165-192).  Within an expression the operations keep the reference's order:
 * in float, order decides the rounding, and the exact trace is checked bit for bit.
 *
 * Layout in device memory: the map is one float block (ArtfCudaHoleFrame's companion, 11.5 MB: it stays
 * resident in the 126 MB L2 for a whole frame); the fluid 1 MB; the frame constants travel as a kernel
 * parameter (constant bank).  Every map read has its index clamped into the map: for the reference's
 * inputs the clamp never moves an index, and no input can make a thread read outside the buffers. */
#pragma once

#include "artful_cuda.h"

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define ARTF_HD __host__ __device__ __forceinline__
#else
#define ARTF_HD inline
#endif

namespace artf {

/* ---- scalar helpers -------------------------------------------------------------------------- */

ARTF_HD float sqrtR(float x) { return sqrtf(x); }
ARTF_HD double sqrtR(double x) { return sqrt(x); }
ARTF_HD float floorR(float x) { return floorf(x); }
ARTF_HD double floorR(double x) { return floor(x); }
ARTF_HD float absR(float x) { return fabsf(x); }
ARTF_HD double absR(double x) { return fabs(x); }
/* x86's minimum and maximum (the reference's SIMD layer defines them so on every ISA): with a NaN
 * operand, the second operand.  Bounds written second therefore also catch NaN. */
template <typename R> ARTF_HD R minX(R a, R b) { return a < b ? a : b; }
template <typename R> ARTF_HD R maxX(R a, R b) { return a > b ? a : b; }
/* Truncation toward zero (cvttps2dq for values in range; NaN gives 0 here, INT32_MIN there: both mask
 * to the same column, and every other use is preceded by a clamp). */
ARTF_HD int32_t truncI(float x) {
#if defined(__CUDA_ARCH__)
    return __float2int_rz(x);
#else
    return (x > -2147483648.f && x < 2147483648.f) ? (int32_t)x : 0;
#endif
}
ARTF_HD int32_t truncI(double x) {
#if defined(__CUDA_ARCH__)
    return __double2int_rz(x);
#else
    return (x > -2147483648.0 && x < 2147483648.0) ? (int32_t)x : 0;
#endif
}
ARTF_HD int32_t clampI(int32_t i, int32_t lo, int32_t hi) { return i < lo ? lo : i > hi ? hi : i; }

/* Division, reciprocal and square roots.  In float these are the plain operations: the unit's flags
 * decide their rounding (IEEE in the exact trace).  In double, units that define ARTF_FAST_FP64 take the
 * hardware's 20-bit estimates (PTX rcp.approx.ftz.f64, rsqrt.approx.f64) and refine them by
 * Newton-Raphson iterations, each doubling the correct bits (e = 1 - x y, y += y e for the reciprocal;
 * e = 1 - x y^2, y += y e / 2 for the inverse square root): two of them (the default) land within an ulp
 * or two of the IEEE result, for a fraction of the FP64 instructions of the correctly rounded sequences;
 * a unit that defines ARTF_FP64_NEWTON_STEPS 1 takes one, about 40 correct bits, where the result only
 * has to be far finer than float's 24.  Operands here are normal and positive where square roots are
 * taken. */
#if defined(__CUDA_ARCH__) && defined(ARTF_FAST_FP64)
#ifndef ARTF_FP64_NEWTON_STEPS
#define ARTF_FP64_NEWTON_STEPS 2
#endif
__device__ __forceinline__ double recipR(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
#if ARTF_FP64_NEWTON_STEPS > 1
    e = fma(-x, y, 1.0);
    y = fma(y, e, y);
#endif
    return y;
}
__device__ __forceinline__ double invSqrtR(double x) {
    double y;
    asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x * y, y, 1.0);
    y = fma(y * .5, e, y);
#if ARTF_FP64_NEWTON_STEPS > 1
    e = fma(-x * y, y, 1.0);
    y = fma(y * .5, e, y);
#endif
    return y;
}
__device__ __forceinline__ double divR(double a, double b) { return a * recipR(b); }
#else
ARTF_HD double recipR(double x) { return 1.0 / x; }
ARTF_HD double invSqrtR(double x) { return 1.0 / sqrt(x); }
ARTF_HD double divR(double a, double b) { return a / b; }
#endif
ARTF_HD float recipR(float x) { return 1.f / x; }
ARTF_HD float invSqrtR(float x) { return 1.f / sqrtf(x); }
ARTF_HD float divR(float a, float b) { return a / b; }
/* a / sqrt(x), and sqrt(x) itself */
ARTF_HD float divSqrtR(float a, float x) { return a / sqrtf(x); }
#if defined(__CUDA_ARCH__) && defined(ARTF_FAST_FP64)
__device__ __forceinline__ double divSqrtR(double a, double x) { return a * invSqrtR(x); }
__device__ __forceinline__ double rootR(double x) { return x * invSqrtR(fmax(x, 1e-300)); }
#else
ARTF_HD double divSqrtR(double a, double x) { return a / sqrt(x); }
ARTF_HD double rootR(double x) { return sqrt(x); }
#endif
ARTF_HD float rootR(float x) { return sqrtf(x); }

/* ---- the debug build's bounds checks -------------------------------------------------------------
 * Built with ARTF_CUDA_DEBUG_BOUNDS, every table row or entry the shading reads is checked against its
 * own region of the map or fluid (not only the buffer, which the clamps below keep every read inside),
 * and every write against the frame or buffer it goes to.  The first index found outside is recorded in
 * the fault word a frame carries (the launch's CBoundsKind, CBoundsIndex counters) and the C ABI
 * returns ARTF_CUDA_EBOUNDS; the read still goes through the clamp, as in the release build, and the
 * write is skipped.  In the release build the checks compile to nothing. */
enum BoundsKind : uint32_t {
    kBoundsGasRow = 1, kBoundsFluidRow, kBoundsDustRow, kBoundsSkyRow, kBoundsRingRow, kBoundsColour,
    kBoundsPixel, kBoundsRayPlane, kBoundsRayEnd
};

ARTF_HD bool inBounds(unsigned long long* fault, uint32_t kind, int64_t i, int64_t count) {
#if defined(ARTF_CUDA_DEBUG_BOUNDS) && defined(__CUDA_ARCH__)
    if (i >= 0 && i < count) return true;
    if (fault && atomicCAS(fault, 0ull, (unsigned long long)kind) == 0ull) atomicExch(fault + 1, (unsigned long long)i);
    return false;
#else
    (void)fault, (void)kind, (void)i, (void)count;
    return true;
#endif
}

/* A read of the read-only map or fluid (through the non-coherent path on the GPU). */
ARTF_HD float fetch(const float* p, int32_t i) {
#if defined(__CUDA_ARCH__)
    return __ldg(p + i);
#else
    return p[i];
#endif
}

/* The reference's float constants, exactly: a double trace evaluates its formulas with the same
 * constant values. */
#define KF(x) R(x##f)

/* ---- the frame ---------------------------------------------------------------------------------- */

template <typename R> struct Frame {
    R er[3], etheta[3], ephi[3], right[3], up[3], forward[3];
    R metric[4], place[4];
    R a, uHorizon, discHeight, shutter, flow, boost[4];
    R inner, outer, time, thickness, gain, doppler, stars;
    R pixelX, pixelY, share; /* 2/width, 2/height, 1/(rays a pixel) */
    int32_t width, height, side;
    unsigned long long* fault; /* the debug build's fault word (two counters), or NULL */
    /* The differentiated traces evaluate the two map tables that depend on the scene's parameters (the
     * rings' orbit speed and their glow, (r / inner)^-q) from their formulas, so that the parameters'
     * derivatives flow through them; every other trace reads the tables. */
    int32_t analyticTables;
    R emissivity;

    template <typename F> ARTF_HD void load(const F& f, const ArtfCudaHoleFrame& sizes) {
        for (int c = 0; c < 3; ++c) {
            er[c] = R(f.er[c]), etheta[c] = R(f.etheta[c]), ephi[c] = R(f.ephi[c]);
            right[c] = R(f.right[c]), up[c] = R(f.up[c]), forward[c] = R(f.forward[c]);
        }
        for (int c = 0; c < 4; ++c) metric[c] = R(f.metric[c]), place[c] = R(f.place[c]), boost[c] = R(f.boost[c]);
        a = R(f.spin[0]), uHorizon = R(f.spin[1]), discHeight = R(f.spin[2]), shutter = R(f.spin[3]);
        flow = R(f.flow[0]);
        inner = R(f.disc[0]), outer = R(f.disc[1]), time = R(f.disc[2]), thickness = R(f.disc[3]);
        gain = R(f.look[0]), doppler = R(f.look[1]), stars = R(f.look[2]);
        pixelX = R(f.image[1]), pixelY = R(f.image[2]), share = R(f.image[3]);
        width = (int32_t)sizes.size[0], height = (int32_t)sizes.size[1], side = (int32_t)sizes.size[2];
        fault = nullptr;
        analyticTables = 0;
        emissivity = R(0);
    }
};

ARTF_HD float expR(float x) { return expf(x); }
ARTF_HD double expR(double x) { return exp(x); }
ARTF_HD float logR(float x) { return logf(x); }
ARTF_HD double logR(double x) { return log(x); }

/* The rings' orbit speed at a map row (hole.c:186-191 setRings, rows even in 1/r). */
template <typename R> ARTF_HD R ringSpeedAt(const Frame<R>& f, const float* map, int32_t row) {
    if (f.analyticTables) {
        const R rho = R((float)row / (float)(ARTF_CUDA_MAP_HEIGHT - 1));
        const R r = divR(f.inner, R(1) - rho * (R(1) - divR(f.inner, f.outer)));
        return recipR(KF(6.2831853) * (r * rootR(r) + f.a));
    }
    return R(fetch(map, clampI(ARTF_CUDA_ROWS_AT + row + row, 0, ARTF_CUDA_MAP_FLOATS - 1)));
}

/* The rings' glow at a map row: (r / inner)^-q of the synthetic disc. */
template <typename R> ARTF_HD R ringGlowAt(const Frame<R>& f, const float* map, int32_t row) {
    if (f.analyticTables) {
        const R rho = R((float)row / (float)(ARTF_CUDA_MAP_HEIGHT - 1));
        const R span = R(1) - rho * (R(1) - divR(f.inner, f.outer)); /* inner / r */
        return expR(f.emissivity * logR(span));
    }
    return R(fetch(map, clampI(ARTF_CUDA_GLOW_AT + row, 0, ARTF_CUDA_MAP_FLOATS - 1)));
}

/* ---- per ray ------------------------------------------------------------------------------------ */

/* What stays fixed along a ray (lens.inc:125-142). */
template <typename R> struct RayConst {
    R invEnergy, xi, moved;          /* 1/E, the axial momentum over E, the eye's aberration factor */
    R big, step;                     /* K = eta + xi^2, and the Nystrom step */
    R uA, uB, uC, xiA;               /* u'' = u (uA + u (uB + u uC)); a xi */
    R time;                          /* the moment this ray sees the gas at */
};

/* The integrated state (lens.inc:146-152). */
template <typename R> struct RayState {
    R u, w;                          /* 1/r and du/ds */
    R n[3], v[3];                    /* the unit vector toward the ray in the disc frame, and dn/ds */
    R psi, drag;                     /* the frame-drag angle and its rate */
};

/* Where the ray stands after a step, with the first-stage derivatives the crossing test needs. */
template <typename R> struct StepOut {
    RayState<R> next;
    R k1, a1[3];
};

/* What a ray's start takes from the frame alone (lens.inc:125-152), fixed for a view and a step scale:
 * a caller may form it once and hand it to rayStartWith, with the same values. */
template <typename R> struct StartTerms {
    R a2, mu0Squared, minusTwoA2, stepBase, wScale;
};

template <typename R> ARTF_HD StartTerms<R> startTerms(const Frame<R>& f, R stepScale) {
    const R u0 = f.place[2];
    StartTerms<R> t;
    t.a2 = f.a * f.a;
    t.mu0Squared = f.place[3] * f.place[3];
    t.minusTwoA2 = KF(-2.) * t.a2;
    t.stepBase = KF(.13089969) * stepScale;
    t.wScale = (-u0) * u0 * f.place[1] * f.place[0];
    return t;
}

/* lens.inc:101-152: the ray of image position (nx, ny), its constants of motion, its first state. */
template <typename R> ARTF_HD void rayStartWith(const Frame<R>& f, const StartTerms<R>& t, R nx, R ny, R time,
                                                RayConst<R>& c, RayState<R>& s) {
    R d[3];
    for (int k = 0; k < 3; ++k) d[k] = f.forward[k] + nx * f.right[k] + ny * f.up[k];
    const R invLength = invSqrtR(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int k = 0; k < 3; ++k) d[k] = d[k] * invLength;

    /* 110-122: light reaching a moving eye from d left, for one at rest, from elsewhere */
    R moved = R(1);
    const R gamma = f.boost[3];
    if (gamma > R(1)) {
        const R share = divR(gamma, gamma + R(1));
        const R cosine = R(0) - (d[0] * f.boost[0] + d[1] * f.boost[1] + d[2] * f.boost[2]);
        const R push = gamma * (R(1) + share * cosine);
        const R over = recipR(gamma * (R(1) + cosine));
        for (int k = 0; k < 3; ++k) d[k] = (d[k] - f.boost[k] * push) * over;
        moved = over;
    }

    const R a = f.a, a2 = t.a2, rho = f.place[0], u0 = f.place[2];
    const R energy = f.metric[0] - f.metric[1] * d[2];
    c.invEnergy = recipR(energy);
    c.xi = R(0) - f.metric[2] * d[2] * c.invEnergy;
    const R xiAxis = f.metric[3] * d[2] * c.invEnergy;
    const R across = rho * d[1] * c.invEnergy;
    const R eta = across * across + t.mu0Squared * (xiAxis * xiAxis - a2);
    c.big = eta + c.xi * c.xi;
    c.step = divSqrtR(t.stepBase, maxX(c.big, KF(4.)));
    c.uA = a2 - c.big;
    const R xiOff = c.xi - a;
    c.uB = KF(3.) * (eta + xiOff * xiOff);
    c.uC = t.minusTwoA2 * eta;
    c.xiA = c.xi * a;
    c.moved = moved;
    c.time = time;

    s.u = u0;
    s.w = t.wScale * d[0] * c.invEnergy;
    for (int k = 0; k < 3; ++k) s.n[k] = f.er[k], s.v[k] = across * f.etheta[k] + xiAxis * f.ephi[k];
    s.psi = R(0);
    s.drag = R(0);
}

template <typename R> ARTF_HD void rayStart(const Frame<R>& f, R nx, R ny, R time, R stepScale, RayConst<R>& c,
                                            RayState<R>& s) {
    rayStartWith(f, startTerms(f, stepScale), nx, ny, time, c, s);
}

/* The constants of motion alone, for an eye at rest (lens.inc:125-142 without the aberration of
 * 110-122): E, the axial momentum xi, eta and K = eta + xi^2, the radial equation's coefficients, and the
 * factors the first state is made of (the ray's unnormalised x component, and across and the axial
 * component of its direction over E).  The mixed trace evaluates these in double-float pairs, in this
 * order (motionConstantsFf), and forms the first state and the step from them in FP32, as the reference's
 * integrator has them; the flop count counts them here. */
template <typename R> struct MotionFactors {
    R dx, over, across, xiAxis; /* d_x, 1 / (|d| E), across, xi_axis */
};

template <typename R> ARTF_HD void motionConstants(const Frame<R>& f, const StartTerms<R>& t, R nx, R ny,
                                                   RayConst<R>& c, MotionFactors<R>& m) {
    R d[3];
    for (int k = 0; k < 3; ++k) d[k] = f.forward[k] + nx * f.right[k] + ny * f.up[k];
    const R invLength = invSqrtR(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const R dz = d[2] * invLength;
    const R energy = f.metric[0] - f.metric[1] * dz;
    c.invEnergy = recipR(energy);
    m.over = invLength * c.invEnergy;
    c.xi = R(0) - f.metric[2] * dz * c.invEnergy;
    m.xiAxis = f.metric[3] * d[2] * m.over;
    m.across = f.place[0] * d[1] * m.over;
    const R eta = m.across * m.across + t.mu0Squared * (m.xiAxis * m.xiAxis - t.a2);
    c.big = eta + c.xi * c.xi;
    c.uA = t.a2 - c.big;
    const R xiOff = c.xi - f.a;
    c.uB = KF(3.) * (eta + xiOff * xiOff);
    c.uC = t.minusTwoA2 * eta;
    c.xiA = c.xi * f.a;
    m.dx = d[0];
}

/* psi' at u (lens.inc:144 DRAG); the denominator is Delta / r^2, kept off zero. */
template <typename R> ARTF_HD R dragAt(R a, R a2, R xiA, R x) {
    return divR((-a) * x * (KF(2.) - xiA * x), maxX(R(1) - (x + x) + a2 * x * x, KF(1e-3)));
}

template <typename R> ARTF_HD R bendAt(const RayConst<R>& c, R x) { return x * (c.uA + x * (c.uB + x * c.uC)); }

/* The step decouples: u'' depends on u alone and n'' on n alone (lens.inc:7-8), and psi' on u alone.
 * So one Nystrom step is a radial sub-step of (u, w, psi) and a polar sub-step of (n, v), with the same
 * operations either way; the mixed-precision trace runs each in the precision it needs. */

/* The products of a ray's step that every sub-step takes (lens.inc:165-192): fixed along the ray, so a
 * caller may form them once and hand them to the sub-steps below, with the same values. */
template <typename R> struct StepTerms {
    R half, eighth, halfSquare, sixthSquare, sixth;
};

template <typename R> ARTF_HD StepTerms<R> stepTerms(R step) {
    const R step2 = step * step;
    StepTerms<R> t;
    t.half = step * KF(.5), t.eighth = step2 * KF(.125), t.halfSquare = step2 * KF(.5);
    t.sixthSquare = step2 * R(1.f / 6.f), t.sixth = step * R(1.f / 6.f);
    return t;
}

/* lens.inc:165-192, the radial part: u, du/ds, and Simpson's rule for psi, with the step's terms and
 * a2 = a * a given. */
template <typename R>
ARTF_HD void radialStepWith(R a, R a2, const RayConst<R>& c, const StepTerms<R>& t, const RayState<R>& s,
                            RayState<R>& next, R& k1Out) {
    const R step = c.step;
    const R half = t.half, eighth = t.eighth, halfSquare = t.halfSquare;
    const R sixthSquare = t.sixthSquare, sixth = t.sixth;
    const R k1 = bendAt(c, s.u);
    const R midU = s.u + half * s.w + eighth * k1;
    const R k2 = bendAt(c, midU);
    const R endU = s.u + step * s.w + halfSquare * k2;
    const R k3 = bendAt(c, endU);
    next.u = s.u + step * s.w + sixthSquare * (k1 + (k2 + k2));
    next.w = s.w + sixth * (k1 + k3 + KF(4.) * k2);
    if (a != R(0)) {
        next.drag = dragAt(a, a2, c.xiA, next.u);
        next.psi = s.psi + sixth * (s.drag + next.drag + KF(4.) * dragAt(a, a2, c.xiA, midU));
    } else {
        next.drag = R(0);
        next.psi = R(0);
    }
    k1Out = k1;
}

template <typename R>
ARTF_HD void radialStep(R a, const RayConst<R>& c, const RayState<R>& s, RayState<R>& next, R& k1Out) {
    radialStepWith(a, a * a, c, stepTerms(c.step), s, next, k1Out);
}

/* The radial sub-step's motion alone, u and du/ds, by the same operations as radialStepWith's: the part
 * a turning point of u concerns (the mixed trace runs it in FP64 there). */
template <typename R>
ARTF_HD void radialMotionWith(const RayConst<R>& c, const StepTerms<R>& t, R u, R w, R& nextU, R& nextW, R& k1Out) {
    const R step = c.step;
    const R k1 = bendAt(c, u);
    const R midU = u + t.half * w + t.eighth * k1;
    const R k2 = bendAt(c, midU);
    const R endU = u + step * w + t.halfSquare * k2;
    const R k3 = bendAt(c, endU);
    nextU = u + step * w + t.sixthSquare * (k1 + (k2 + k2));
    nextW = w + t.sixth * (k1 + k3 + KF(4.) * k2);
    k1Out = k1;
}

/* The polar sub-step's axis component alone, n_z and dn_z/ds, by the same operations as polarStepWith's
 * for it: n_z'' depends on n_z alone, and the polar turning point is n_z's (the mixed trace runs this in
 * FP64 there). */
template <typename R>
ARTF_HD void polarAxisWith(R a2, R twoA2, const RayConst<R>& c, const StepTerms<R>& t, R nz, R vz, R& nextNz,
                           R& nextVz, R& a1z) {
    const R step = c.step;
    const R c1 = c.big + twoA2 * (nz * nz);
    const R a1 = a2 * nz - c1 * nz;
    const R midN = nz + t.half * vz + t.eighth * a1;
    const R c2 = c.big + twoA2 * (midN * midN);
    const R a2s = a2 * midN - c2 * midN;
    const R endN = nz + step * vz + t.halfSquare * a2s;
    const R c3 = c.big + twoA2 * (endN * endN);
    const R a3 = a2 * endN - c3 * endN;
    nextNz = nz + step * vz + t.sixthSquare * (a1 + (a2s + a2s));
    nextVz = vz + t.sixth * (a1 + a3 + KF(4.) * a2s);
    a1z = a1;
}

/* lens.inc:165-192, the polar part: n on the sphere and dn/ds, with the step's terms, a2 = a * a and
 * twoA2 = 2 * a2 given. */
template <typename R>
ARTF_HD void polarStepWith(R a2, R twoA2, const RayConst<R>& c, const StepTerms<R>& t, const RayState<R>& s,
                           RayState<R>& next, R* a1Out) {
    const R step = c.step;
    const R half = t.half, eighth = t.eighth, halfSquare = t.halfSquare;
    const R sixthSquare = t.sixthSquare, sixth = t.sixth;
    const R c1 = c.big + twoA2 * (s.n[2] * s.n[2]);
    const R a1[3] = {R(0) - c1 * s.n[0], R(0) - c1 * s.n[1], a2 * s.n[2] - c1 * s.n[2]};
    R midN[3];
    for (int k = 0; k < 3; ++k) midN[k] = s.n[k] + half * s.v[k] + eighth * a1[k];
    const R c2 = c.big + twoA2 * (midN[2] * midN[2]);
    const R a2s[3] = {R(0) - c2 * midN[0], R(0) - c2 * midN[1], a2 * midN[2] - c2 * midN[2]};
    R endN[3];
    for (int k = 0; k < 3; ++k) endN[k] = s.n[k] + step * s.v[k] + halfSquare * a2s[k];
    const R c3 = c.big + twoA2 * (endN[2] * endN[2]);
    const R a3[3] = {R(0) - c3 * endN[0], R(0) - c3 * endN[1], a2 * endN[2] - c3 * endN[2]};
    for (int k = 0; k < 3; ++k) {
        next.n[k] = s.n[k] + step * s.v[k] + sixthSquare * (a1[k] + (a2s[k] + a2s[k]));
        next.v[k] = s.v[k] + sixth * (a1[k] + a3[k] + KF(4.) * a2s[k]);
        a1Out[k] = a1[k];
    }
}

template <typename R>
ARTF_HD void polarStep(R a, const RayConst<R>& c, const RayState<R>& s, RayState<R>& next, R* a1Out) {
    const R a2 = a * a;
    polarStepWith(a2, KF(2.) * a2, c, stepTerms(c.step), s, next, a1Out);
}

/* lens.inc:165-192: one Nystrom step of (u, n) and Simpson's rule for psi. */
template <typename R> ARTF_HD void nystromStep(R a, const RayConst<R>& c, const RayState<R>& s, StepOut<R>& o) {
    radialStep(a, c, s, o.next, o.k1);
    polarStep(a, c, s, o.next, o.a1);
}

/* A disc crossing inside one step: the ray's state at the plane (lens.inc:197-208, second-order Taylor
 * from the step's start). */
template <typename R> struct Crossing {
    R part, uc, wc, cx, cy, vx, vy, vz, psiC, dragC;
};

/* lens.inc:195-202: did the step cross the disc's plane within its radial range?  Fills x when so. */
template <typename R> ARTF_HD bool crossingOf(const Frame<R>& f, R rhoScale, const RayConst<R>& c,
                                              const RayState<R>& s, const StepOut<R>& o, Crossing<R>& x) {
    if (!(s.n[2] * o.next.n[2] < R(0))) return false;
    const R part = divR(s.n[2], s.n[2] - o.next.n[2]);
    const R hu = part * c.step, hh = hu * hu * KF(.5);
    const R uc = s.u + hu * s.w + hh * o.k1;
    const R rhoCenter = (R(1) - f.inner * uc) * rhoScale;
    if (!(rhoCenter > KF(-.03) && rhoCenter < KF(1.02))) return false;
    x.part = part;
    x.uc = uc;
    x.wc = s.w + hu * o.k1;
    x.cx = s.n[0] + hu * s.v[0] + hh * o.a1[0];
    x.cy = s.n[1] + hu * s.v[1] + hh * o.a1[1];
    x.vx = s.v[0] + hu * o.a1[0];
    x.vy = s.v[1] + hu * o.a1[1];
    x.vz = s.v[2] + hu * o.a1[2];
    x.psiC = s.psi + part * (o.next.psi - s.psi);
    x.dragC = s.drag + part * (o.next.drag - s.drag);
    return true;
}

/* lens.inc:30-41: the angle of (x, y) in turns, by the reference's polynomial arctangent. */
template <typename R> ARTF_HD R turnsOf(R y, R x) {
    const R ax = absR(x), ay = absR(y);
    const R most = maxX(maxX(ax, ay), KF(1e-20)), least = minX(ax, ay);
    const R q = divR(least, most), s = q * q;
    R r = KF(-.0464964749) * s + KF(.15931422);
    r = r * s - KF(.327622764);
    r = r * s * q + q;
    if (ay > ax) r = KF(1.57079633) - r;
    if (x < R(0)) r = KF(3.14159265) - r;
    if (y < R(0)) r = R(0) - r;
    return r * KF(.15915494);
}

/* lens.inc:44-54: sine of an angle in turns, folded to a quarter turn, odd polynomial. */
template <typename R> ARTF_HD R sineOf(R turns) {
    R t = turns - floorR(turns + KF(.5));
    if (t > KF(.25)) t = KF(.5) - t;
    if (t < KF(-.25)) t = KF(-.5) - t;
    const R x = t * KF(6.2831853), x2 = x * x;
    R p = x2 * KF(2.7557319e-6) + KF(-1.9841270e-4);
    p = p * x2 + KF(8.3333333e-3);
    p = p * x2 + KF(-.16666667);
    return p * x2 * x + x;
}

/* lens.inc:89-96: a row of a region of `width` (a power of two) columns starting `at` floats into a
 * buffer of `count` floats, read at a turn, linear in between.  The index is clamped to the buffer,
 * not the region: wherever the reference reads inside its buffer, this reads the same float. */
template <typename R>
ARTF_HD R rowAt(const float* buffer, int32_t count, int32_t at, int32_t width, int32_t row, R turn) {
    const R pos = (turn - floorR(turn)) * R(width);
    const R column = floorR(pos), part = pos - column;
    const int32_t c0 = truncI(column) & (width - 1), c1 = (c0 + 1) & (width - 1);
    const int32_t base = at + row * width;
    const R lo = R(fetch(buffer, clampI(base + c0, 0, count - 1)));
    const R hi = R(fetch(buffer, clampI(base + c1, 0, count - 1)));
    return lo + (hi - lo) * part;
}

/* lens.inc:56-61: the star lattice's cube hash. */
ARTF_HD uint32_t cubeHash(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = x * 73856093u ^ y * 19349663u ^ z * 83492791u;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

/* lens.inc:69-86: one layer of hashed-cube stars at direction dir, added to rgb. */
template <typename R> ARTF_HD void starLayer(const R* dir, R cells, int32_t density, float size, R gain, R* rgb) {
    const R px = dir[0] * cells, py = dir[1] * cells, pz = dir[2] * cells;
    const R cx = floorR(px), cy = floorR(py), cz = floorR(pz);
    const uint32_t h = cubeHash((uint32_t)truncI(cx), (uint32_t)truncI(cy), (uint32_t)truncI(cz));
    if (!(density > (int32_t)(h & 255u))) return;
    const R inv255 = R(1.f / 255.f);
    const R ex = px - cx - R(float((h >> 8) & 255u)) * inv255;
    const R ey = py - cy - R(float((h >> 16) & 255u)) * inv255;
    const R ez = pz - cz - R(float((h >> 24) & 255u)) * inv255;
    const R d2 = ex * ex + ey * ey + ez * ez;
    R light = maxX(R(1) - d2 * R(1.f / (size * size)), R(0));
    light = light * light * gain;
    const R warm = R(float((h >> 3) & 255u)) * inv255;
    rgb[0] = rgb[0] + light * (KF(.75) + warm * KF(.25));
    rgb[1] = rgb[1] + light * KF(.82);
    rgb[2] = rgb[2] + light * (R(1) - warm * KF(.45));
}

/* What a crossing gives: lens.inc:204-289.  Adds its light to sum, and leaves the disc's transmission
 * in `through`.  Returns the light (> 0 when the disc lit the ray). */
template <typename R> ARTF_HD R shadeCrossing(const Frame<R>& f, R rhoScale, const float* map, const float* fluid,
                                              const RayConst<R>& c, const Crossing<R>& x, R& through, R* sum,
                                              R* turnOut) {
    const R turn = turnsOf(x.cy, x.cx) + x.psiC * KF(.15915494);
    const R rate = (divR(x.cx * x.vy - x.cy * x.vx, maxX(x.cx * x.cx + x.cy * x.cy, KF(1e-6))) + x.dragC) * KF(.15915494);
    /* gas seen at a slant is deeper */
    const R slope = divR(x.wc, x.uc);
    const R speed2 = x.vx * x.vx + x.vy * x.vy + (x.vz * x.vz + slope * slope);
    const R mu = maxX(divSqrtR(absR(x.vz), speed2), KF(.02));
    const R slant = divR(divR(f.thickness, R(3)), mu);
    const R reach = minX(divR(f.discHeight, maxX(absR(x.vz), KF(1e-5))), c.step * KF(1.5));
    const int32_t mapCount = ARTF_CUDA_MAP_FLOATS, fluidCount = ARTF_CUDA_FLUID_FLOATS;
    const R fluidTime = c.time - f.flow;

    R glow = R(0), clear = through;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const R t = R(((float)k + .5f) * (2.f / 3.f) - 1.f);
        const R ds = reach * t;
        const R uk = x.uc + x.wc * ds;
        const R rhoK = (R(1) - f.inner * uk) * rhoScale;
        const bool inside = rhoK > R(0) && rhoK < R(1);
        const R rowPos = (inside ? rhoK : R(0)) * R(ARTF_CUDA_MAP_HEIGHT - 1);
        const R rowFloor = minX(floorR(rowPos), R(ARTF_CUDA_MAP_HEIGHT - 2));
        const R rowPart = rowPos - rowFloor;
        const int32_t row0 = truncI(rowFloor), row1 = row0 + 1;
        inBounds(f.fault, kBoundsGasRow, row0, ARTF_CUDA_MAP_HEIGHT - 1); /* (row0 and row1) */
        const R speed0 = ringSpeedAt(f, map, row0), speed1 = ringSpeedAt(f, map, row1);
        const R turnK = turn + (inside ? rate * ds : R(0));
        const R d0 = rowAt(map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0, turnK - speed0 * c.time);
        const R d1 = rowAt(map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row1, turnK - speed1 * c.time);
        R density = d0 + (d1 - d0) * rowPart;
        /* the fluid, each ring turned on since it was stepped */
        const R fluidPos = (inside ? rhoK : R(0)) * R(ARTF_CUDA_FLUID_HEIGHT - 1);
        const R fluidFloor = minX(floorR(fluidPos), R(ARTF_CUDA_FLUID_HEIGHT - 2));
        const int32_t fluidRow = truncI(fluidFloor);
        inBounds(f.fault, kBoundsFluidRow, fluidRow, ARTF_CUDA_FLUID_HEIGHT - 1); /* (and the row after) */
        const R fluidTurn = turnK - speed0 * fluidTime;
        const R g0 = rowAt(fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow, fluidTurn);
        const R g1 = rowAt(fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow + 1, fluidTurn);
        const R gas = g0 + (g1 - g0) * (fluidPos - fluidFloor);
        density = density * (R(1.f - .1f) + KF(.1) * gas);
        /* dust: less light, more opacity */
        const R dustPos = (inside ? rhoK : R(0)) * R(ARTF_CUDA_DUST_HEIGHT - 1);
        const int32_t dustRow = truncI(minX(floorR(dustPos), R(ARTF_CUDA_DUST_HEIGHT - 1)));
        inBounds(f.fault, kBoundsDustRow, dustRow, ARTF_CUDA_DUST_HEIGHT);
        const R dusty = rowAt(map, mapCount, ARTF_CUDA_DUST_AT, ARTF_CUDA_DUST_WIDTH, dustRow, turnK - speed0 * c.time);
        const R lit = R(1) - KF(.97) * dusty;
        /* how far from the disc's middle plane, and what the slice stops and gives */
        const R height = t * divR(reach, f.discHeight);
        const R level = maxX(R(1) - x.vz * x.vz * (height * height), R(0));
        density = inside ? density * level : R(0);
        const R depth = slant * density * (R(1) + KF(25.) * dusty);
        const R alpha = divR(depth, R(1) + depth);
        glow = glow + clear * alpha * (density * lit);
        clear = clear * (R(1) - alpha);
    }

    /* the ring's heat and glow; its orbit's Doppler and the hole's pull */
    const R rhoCenter = (R(1) - f.inner * x.uc) * rhoScale;
    const R rhoSafe = minX(maxX(rhoCenter, R(0)), R(1));
    const int32_t rowIndex = truncI(rhoSafe * R(ARTF_CUDA_MAP_HEIGHT - 1));
    inBounds(f.fault, kBoundsRingRow, rowIndex, ARTF_CUDA_MAP_HEIGHT);
    R heat = R(fetch(map, clampI(ARTF_CUDA_ROWS_AT + rowIndex + rowIndex + 1, 0, mapCount - 1)));
    const R gives = ringGlowAt(f, map, rowIndex);
    R light = f.gain * glow * gives;
    if (f.doppler != R(0)) {
        const R safeU = maxX(x.uc, KF(1e-4));
        const R root = safeU * rootR(safeU);
        const R lift = R(1) + f.a * root;
        const R spinRate = divR(root, lift);
        const R beneath = maxX(R(1) - KF(3.) * safeU + (KF(2.) * f.a) * root, KF(1e-4));
        const R shift = divR(rootR(beneath) * (c.invEnergy * c.moved), lift * (R(1) - spinRate * c.xi));
        const R g = R(1) + f.doppler * (shift - R(1));
        const R g2 = g * g;
        light = light * (g2 * g2);
        heat = heat * g;
    }
    const R colorPos = minX(heat * R(ARTF_CUDA_COLORS / 2), R(ARTF_CUDA_COLORS - 1));
    const int32_t color = truncI(colorPos);
    inBounds(f.fault, kBoundsColour, color, ARTF_CUDA_COLORS);
    const int32_t at = ARTF_CUDA_COLORS_AT + color + color + color;
    sum[0] = sum[0] + light * R(fetch(map, clampI(at, 0, mapCount - 1)));
    sum[1] = sum[1] + light * R(fetch(map, clampI(at + 1, 0, mapCount - 1)));
    sum[2] = sum[2] + light * R(fetch(map, clampI(at + 2, 0, mapCount - 1)));
    through = clear;
    *turnOut = turn;
    return light;
}

/* The escape direction in the sky's frame: the last chord's end turned by psi (lens.inc:316-321). */
template <typename R> ARTF_HD void skyDirection(const R* away, R awayPsi, R* dir) {
    const R invAway = invSqrtR(maxX(away[0] * away[0] + away[1] * away[1] + away[2] * away[2], KF(1e-12)));
    const R psiTurns = awayPsi * KF(.15915494);
    const R sine = sineOf(psiTurns), cosine = sineOf(psiTurns + KF(.25));
    const R x = away[0] * invAway, y = away[1] * invAway, m = away[2] * invAway;
    dir[0] = x * cosine - y * sine;
    dir[1] = x * sine + y * cosine;
    dir[2] = m;
}

/* lens.inc:322-346: the stars and the sky's dust toward dir, seen through what the disc let through. */
template <typename R> ARTF_HD void shadeSky(const Frame<R>& f, const float* map, const RayConst<R>& c, const R* dir,
                                            R through, R* sum) {
    R rgb[3] = {R(0), R(0), R(0)};
    starLayer(dir, KF(90.), 26, .1f, KF(1.6), rgb);
    starLayer(dir, KF(240.), 70, .17f, KF(.22), rgb);
    const R skyTurn = turnsOf(dir[1], dir[0]);
    const R heightPos = (dir[2] * KF(.5) + KF(.5)) * R(ARTF_CUDA_SKY_HEIGHT - 1);
    const R skyFloor = minX(floorR(heightPos), R(ARTF_CUDA_SKY_HEIGHT - 2));
    const int32_t skyRow = truncI(skyFloor);
    inBounds(f.fault, kBoundsSkyRow, skyRow, ARTF_CUDA_SKY_HEIGHT - 1); /* (and the row after) */
    const R s0 = rowAt(map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH, skyRow, skyTurn);
    const R s1 = rowAt(map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH, skyRow + 1, skyTurn);
    const R dust = s0 + (s1 - s0) * (heightPos - skyFloor);
    rgb[0] = rgb[0] + dust * KF(.92);
    rgb[1] = rgb[1] + dust * KF(.86);
    rgb[2] = rgb[2] + dust;
    R shown = through * f.stars;
    if (f.doppler != R(0)) {
        const R g1 = R(1) + f.doppler * (c.invEnergy * c.moved - R(1));
        const R g2 = g1 * g1;
        shown = shown * (g2 * g2);
    }
    for (int k = 0; k < 3; ++k) sum[k] = sum[k] + rgb[k] * shown;
}

/* ---- sample positions ---------------------------------------------------------------------------- */

ARTF_HD uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

/* A float product rounded on its own, never fused with the sum it feeds: the sample positions below are
 * the reference's to the bit in every unit, including those built with contraction and fast division. */
ARTF_HD float mulRn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
/* A correctly rounded float quotient, whatever the unit's division flags. */
ARTF_HD float divRn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

/* Ray k of pixel (x, y): its image position and its moment within the shutter.  jitter 0: the
 * reference's stratified side x side samples, with its float arithmetic (lens.inc:365-371: the
 * eight-pixel group's base column plus the lane); jitter n: n uniform offsets hashed from the seed. */
ARTF_HD void samplePosition(const ArtfCudaHoleFrame& h, int jitter, uint32_t seed, int32_t x, int32_t y, int32_t k,
                            float* nx, float* ny, float* moment) {
    if (!jitter) {
        const int32_t side = (int32_t)h.size[2];
        const int32_t sy = k / side, sx = k - sy * side;
        const float dx = divRn((float)sx + .5f, (float)side), dy = divRn((float)sy + .5f, (float)side);
        const int32_t group = x & ~7, lane = x & 7;
        *nx = mulRn((float)lane + ((float)group + dx), h.image[1]) - 1.f;
        *ny = 1.f - mulRn((float)y + dy, h.image[2]);
        *moment = mulRn((float)((sy * side + sx) * 5 % (side * side)) + .5f, h.image[3]) - .5f;
    } else {
        const uint32_t base = mix32(mix32(seed ^ 0xA511E9B3u) ^ ((uint32_t)y * h.size[0] + (uint32_t)x));
        const float dx = mulRn((float)(mix32(base + 2u * (uint32_t)k) >> 8), 1.f / 16777216.f);
        const float dy = mulRn((float)(mix32(base + 2u * (uint32_t)k + 1u) >> 8), 1.f / 16777216.f);
        *nx = mulRn((float)x + dx, h.image[1]) - 1.f;
        *ny = 1.f - mulRn((float)y + dy, h.image[2]);
        *moment = divRn((float)(k * 5 % jitter) + .5f, (float)jitter) - .5f;
    }
}

}  // namespace artf
