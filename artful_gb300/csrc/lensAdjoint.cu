/* artful_cuda — the adjoint of the trace: the gradient of an image loss with respect to the scene's five
 * parameters theta = (spin, inclination, inner radius / ISCO, emissivity index q, distance), by
 * reverse-mode differentiation written out by hand, in FP32.
 *
 * Loss of a view: L = sum over pixels and colour channels of (radiance - target)^2 / (3 * pixels), one
 * ray at each pixel's centre.  Theta reaches the trace through the frame's fields (the eye's basis, the
 * metric at the eye, the spin, the inner radius: ARTF_CUDA_GRAD_FIELDS of them, whose Jacobian in theta
 * the host supplies), through the rings' glow (r / inner)^-q and orbit speed, evaluated here from their
 * formulas, and through the spin in the equations of motion.
 *
 * Two kernels.  The forward one traces each pixel's ray with its shading, keeps a checkpoint at the start
 * of each segment of K steps in a trail in device memory (field by field across rays), and leaves the
 * ray's loss adjoint and end there.  The reverse one walks each ray back from its last step that added
 * radiance, a segment at a time, each segment recomputed from its checkpoint into a ring of K kept
 * states in the thread's local memory; or, with K = 1 (every state kept, 48 bytes a step), a warp's rays
 * together from the warp's highest step, their states read back through shared memory with nothing
 * recomputed.  At each step, in reverse order, it
 * applies the transposed derivatives of the sky (at the escape), of the disc crossing (its three slices,
 * the ring's glow and the Doppler shift) and of the Nystrom step's radial and polar parts, accumulating
 * the adjoints of the constants of motion; at the ray's start it takes them through the set-up to the
 * frame's fields, and projects those onto theta at once, so a thread carries six sums.  Choices with no
 * derivative (which texel or star cell, the 0.004 opacity cut-off, the step cap) contribute none: the
 * pathwise derivative.
 *
 * Work layout: a view table in device memory; grid (blocks of four 8 x 4 tiles, views), the tiles of a
 * view heaviest first, each block copying its view's entry to shared memory, each warp tracing one tile.
 * Each tile's six sums go to the tile's own slot; a last kernel adds them in a fixed order, in double, so
 * the result does not depend on scheduling. */
#include "lensKernel.cuh"
#include "lensTangent.h"

#include <string.h>

namespace artf {

struct alignas(16) AdjointView {
    Frame<float> f;             /* with analyticTables set and the emissivity index */
    ArtfCudaHoleFrame h;
    float jacobian[ARTF_CUDA_GRAD_FIELDS][5];
    const float* map;
    const float* fluid;
    const float4* target;
    float4* hdr;                /* the radiance the forward pass found, or NULL */
    float* pixelGrads;          /* each pixel's share of the gradient (5 floats a pixel), or NULL */
    float lossScale;            /* 1 / (3 * pixels) */
    int pixels;
};

namespace {

constexpr int kThreads = 128;
constexpr int kMaxK = ARTF_CUDA_ADJOINT_MAX_CHECKPOINT;
/* With every state kept: the steps a warp's reads run ahead of its step back, through shared memory. */
constexpr int kStage = 4;
constexpr int kMaxSteps = 192;
constexpr int kAdjointClasses = kMaxSteps / 8 + 1; /* a tile's weight: its steps / 8 */
constexpr int kClassStride = 32;                   /* a view's class counters */
constexpr float kTurn = .15915494f; /* 1 / 2 pi, the reference's constant */

/* Adjoints of what a ray's constants of motion and the frame's scalars feed. */
struct ConstBar {
    float step, uA, uB, uC, xiA, big, invEnergy, xi, a, inner, q;
};

/* ---- the equations' pieces ----------------------------------------------------------------------- */

/* k = x (uA + x (uB + x uC)) taken back. */
__device__ __forceinline__ void bendBack(const RayConst<float>& c, float x, float kBar, float& xBar, ConstBar& g) {
    xBar += kBar * (c.uA + x * (2.f * c.uB + 3.f * c.uC * x));
    g.uA += kBar * x;
    g.uB += kBar * x * x;
    g.uC += kBar * x * x * x;
}

/* psi' = -a x (2 - xiA x) / max(1 - 2x + a^2 x^2, 1e-3) taken back. */
__device__ __forceinline__ void dragBack(float a, float xiA, float x, float dBar, float& xBar, ConstBar& g) {
    const float num = -a * x * (2.f - xiA * x);
    const float raw = 1.f - (x + x) + a * a * x * x;
    const bool held = !(raw > 1e-3f);
    const float den = held ? 1e-3f : raw;
    const float numBar = dBar / den, denBar = held ? 0.f : -numBar * num / den;
    xBar += numBar * (-a * (2.f - 2.f * xiA * x)) + denBar * (2.f * a * a * x - 2.f);
    g.a += numBar * (-x * (2.f - xiA * x)) + denBar * 2.f * a * x * x;
    g.xiA += numBar * a * x * x;
}

/* The drag rate at x with the pieces its adjoint takes: the numerator, the reciprocal of the denominator
 * and whether the denominator was held at its floor.  One reciprocal serves the rate and its adjoint
 * (four reciprocals a step fewer than dragAt and dragBack apart: 1.314 -> 1.293 ms for 8 views). */
struct DragTerms {
    float rate, num, inv;
    bool held;
};

__device__ __forceinline__ DragTerms dragTerms(float a, float a2, float xiA, float x) {
    DragTerms d;
    d.num = -a * x * (2.f - xiA * x);
    const float raw = 1.f - (x + x) + a2 * x * x;
    d.held = !(raw > 1e-3f);
    d.inv = 1.f / (d.held ? 1e-3f : raw);
    d.rate = d.num * d.inv;
    return d;
}

/* dragBack with the rate's pieces already at hand. */
__device__ __forceinline__ void dragBackWith(float a, float xiA, float x, const DragTerms& d, float dBar, float& xBar,
                                             ConstBar& g) {
    const float numBar = dBar * d.inv, denBar = d.held ? 0.f : -numBar * d.rate;
    xBar += numBar * (-a * (2.f - 2.f * xiA * x)) + denBar * (2.f * a * a * x - 2.f);
    g.a += numBar * (-x * (2.f - xiA * x)) + denBar * 2.f * a * x * x;
    g.xiA += numBar * a * x * x;
}

/* lens.inc:30-41's polynomial arctangent (in turns): its slopes in y and x. */
__device__ __forceinline__ void turnsSlope(float y, float x, float& dy, float& dx) {
    const float ax = fabsf(x), ay = fabsf(y);
    const bool steep = ay > ax;
    const float most = fmaxf(steep ? ay : ax, 1e-20f), least = steep ? ax : ay;
    const float q = least / most, s = q * q;
    const float slope = 1.f + s * (-3.f * .327622764f + s * (5.f * .15931422f + s * (7.f * -.0464964749f)));
    float sign = steep ? -1.f : 1.f;
    if (x < 0.f) sign = -sign;
    if (y < 0.f) sign = -sign;
    const float k = kTurn * sign * slope;
    const float dqLeast = 1.f / most, dqMost = -q / most;
    dx = k * (steep ? dqLeast : dqMost) * (x < 0.f ? -1.f : 1.f);
    dy = k * (steep ? dqMost : dqLeast) * (y < 0.f ? -1.f : 1.f);
}

/* lens.inc:44-54's polynomial sine of an angle in turns: its slope. */
__device__ __forceinline__ float sineSlope(float turns) {
    float t = turns - floorf(turns + .5f), sign = 1.f;
    if (t > .25f) t = .5f - t, sign = -sign;
    if (t < -.25f) t = -.5f - t, sign = -sign;
    const float x = t * 6.2831853f, x2 = x * x;
    const float d = 1.f + x2 * (3.f * -.16666667f +
                                x2 * (5.f * 8.3333333e-3f + x2 * (7.f * -1.9841270e-4f + x2 * (9.f * 2.7557319e-6f))));
    return sign * 6.2831853f * d;
}

/* A map row read at a turn (rowAt): its slope in the turn. */
__device__ __forceinline__ float rowSlope(const float* buffer, int32_t count, int32_t at, int32_t width, int32_t row,
                                          float turn) {
    const float pos = (turn - floorf(turn)) * (float)width;
    const int32_t c0 = truncI(floorf(pos)) & (width - 1), c1 = (c0 + 1) & (width - 1);
    const int32_t base = at + row * width;
    const float lo = fetch(buffer, clampI(base + c0, 0, count - 1)), hi = fetch(buffer, clampI(base + c1, 0, count - 1));
    return (hi - lo) * (float)width;
}

/* The rings' orbit speed 1 / (2 pi (r^1.5 + a)) at a row, r = inner / span: its slopes in a and inner. */
__device__ __forceinline__ void speedSlopes(const Frame<float>& f, int32_t row, float speed, float& dA, float& dInner) {
    const float rho = (float)row / (float)(ARTF_CUDA_MAP_HEIGHT - 1);
    const float span = 1.f - rho * (1.f - f.inner / f.outer), dspan = rho / f.outer;
    const float r = f.inner / span, dr = 1.f / span - f.inner * dspan / (span * span);
    dA = -6.2831853f * speed * speed;
    dInner = dA * 1.5f * sqrtf(r) * dr;
}

/* ---- the Nystrom step taken back (lens.inc:165-192) ------------------------------------------------ */

/* What every step of a ray taken back takes from the ray alone, formed once a ray: the step's products
 * (as stepTerms forms them) and the spin's. */
struct BackTerms {
    float h, half, eighth, halfSq, sixthSq, sixth, a, a2, twoA2, fourA2, fourA, twoA;
};

__device__ __forceinline__ BackTerms backTerms(float a, float step) {
    BackTerms t;
    const StepTerms<float> st = stepTerms(step);
    t.h = step, t.half = st.half, t.eighth = st.eighth, t.halfSq = st.halfSquare, t.sixthSq = st.sixthSquare;
    t.sixth = st.sixth;
    t.a = a, t.a2 = a * a, t.twoA2 = 2.f * t.a2, t.fourA2 = 4.f * t.a2, t.fourA = 4.f * a, t.twoA = 2.f * a;
    return t;
}

/* A(x) = (-c x0, -c x1, a^2 x2 - c x2), c = K + 2 a^2 x2^2 as the forward step forms it; returns c. */
__device__ __forceinline__ float accelWith(const BackTerms& t, float big, const float* x, float* out) {
    const float cc = big + t.twoA2 * (x[2] * x[2]);
    out[0] = 0.f - cc * x[0], out[1] = 0.f - cc * x[1], out[2] = t.a2 * x[2] - cc * x[2];
    return cc;
}

/* A(x) taken back from its adjoint y, with its c. */
__device__ __forceinline__ void accelBackWith(const BackTerms& t, float cc, const float* x, const float* y, float* xBar,
                                              ConstBar& g) {
    const float cBar = -(x[0] * y[0] + x[1] * y[1] + x[2] * y[2]);
    xBar[0] += -cc * y[0];
    xBar[1] += -cc * y[1];
    xBar[2] += (t.a2 - cc) * y[2] + cBar * t.fourA2 * x[2];
    g.a += x[2] * (t.twoA * y[2] + cBar * t.fourA * x[2]);
    g.big += cBar;
}

/* The polar part: from the adjoints of (n', v') and of the first stage's a1 (which a crossing reads), adds
 * to those of (n, v) and the constants. */
__device__ __forceinline__ void polarBack(const BackTerms& t, float big, const float* n, const float* v,
                                          const float* nNextBar, const float* vNextBar, const float* a1Extra,
                                          bool extra, float* nBar, float* vBar, ConstBar& g, ConstBar& gs) {
    const float h = t.h, half = t.half, eighth = t.eighth, halfSq = t.halfSq, sixthSq = t.sixthSq, sixth = t.sixth;
    float a1[3], midN[3], a2s[3], endN[3], a3[3];
    const float c1 = accelWith(t, big, n, a1);
    for (int k = 0; k < 3; ++k) midN[k] = n[k] + half * v[k] + eighth * a1[k];
    const float c2 = accelWith(t, big, midN, a2s);
    for (int k = 0; k < 3; ++k) endN[k] = n[k] + h * v[k] + halfSq * a2s[k];
    const float c3 = accelWith(t, big, endN, a3);
    (void)a3;
    float a1Bar[3], a2Bar[3], a3Bar[3], midBar[3] = {0.f, 0.f, 0.f}, endBar[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 3; ++k) {
        /* n' = n + h v + h^2/6 (a1 + 2 a2);  v' = v + h/6 (a1 + a3 + 4 a2) */
        nBar[k] += nNextBar[k];
        vBar[k] += h * nNextBar[k] + vNextBar[k];
        a1Bar[k] = sixthSq * nNextBar[k] + sixth * vNextBar[k];
        a2Bar[k] = 2.f * sixthSq * nNextBar[k] + 4.f * sixth * vNextBar[k];
        a3Bar[k] = sixth * vNextBar[k];
    }
    accelBackWith(t, c3, endN, a3Bar, endBar, gs);
    for (int k = 0; k < 3; ++k) { /* endN = n + h v + h^2/2 a2 */
        nBar[k] += endBar[k];
        vBar[k] += h * endBar[k];
        a2Bar[k] += halfSq * endBar[k];
    }
    accelBackWith(t, c2, midN, a2Bar, midBar, gs);
    for (int k = 0; k < 3; ++k) { /* midN = n + h/2 v + h^2/8 a1 */
        nBar[k] += midBar[k];
        vBar[k] += half * midBar[k];
        a1Bar[k] += eighth * midBar[k];
    }
    accelBackWith(t, c1, n, a1Bar, nBar, gs);
    if (extra) accelBackWith(t, c1, n, a1Extra, nBar, g); /* (what a crossing read of a1: not the step's) */
}

/* The radial part: from the adjoints of (u', w', psi', drag') and of k1, adds to those of (u, w, psi,
 * drag) and the constants. */
__device__ __forceinline__ void radialBack(const BackTerms& t, const RayConst<float>& c, float u, float w, float drag,
                                           float uNextBar, float wNextBar, float psiNextBar, float dragNextBar,
                                           float k1Extra, bool extra, float& uBar, float& wBar, float& psiBar,
                                           float& dragBar, ConstBar& g, ConstBar& gs) {
    const float h = t.h, half = t.half, eighth = t.eighth, halfSq = t.halfSq, sixthSq = t.sixthSq, sixth = t.sixth;
    const float k1 = bendAt(c, u);
    const float midU = u + half * w + eighth * k1;
    const float k2 = bendAt(c, midU);
    const float endU = u + h * w + halfSq * k2;
    float midBar = 0.f;
    if (t.a != 0.f) {
        /* drag' = drag(u');  psi' = psi + h/6 (drag + drag' + 4 drag(midU)): the step length's explicit
         * share here; its share through u' and midU is the motion's, taken over the whole ray */
        const float uNext = u + h * w + sixthSq * (k1 + (k2 + k2));
        const DragTerms dNext = dragTerms(t.a, t.a2, c.xiA, uNext), dMid = dragTerms(t.a, t.a2, c.xiA, midU);
        const float s6 = psiNextBar * sixth;
        psiBar += psiNextBar;
        dragBar += s6;
        g.step += psiNextBar * (drag + dNext.rate + 4.f * dMid.rate) * (1.f / 6.f);
        dragBackWith(t.a, c.xiA, midU, dMid, 4.f * s6, midBar, g);
        dragBackWith(t.a, c.xiA, uNext, dNext, dragNextBar + s6, uNextBar, g);
    }
    /* u' = u + h w + h^2/6 (k1 + 2 k2);  w' = w + h/6 (k1 + k3 + 4 k2) */
    uBar += uNextBar;
    wBar += h * uNextBar + wNextBar;
    float k1Bar = sixthSq * uNextBar + sixth * wNextBar;
    float k2Bar = 2.f * sixthSq * uNextBar + 4.f * sixth * wNextBar;
    const float k3Bar = sixth * wNextBar;
    float endBar = 0.f; /* endU = u + h w + h^2/2 k2 */
    bendBack(c, endU, k3Bar, endBar, gs);
    uBar += endBar;
    wBar += h * endBar;
    k2Bar += halfSq * endBar;
    bendBack(c, midU, k2Bar, midBar, gs); /* midU = u + h/2 w + h^2/8 k1 */
    uBar += midBar;
    wBar += half * midBar;
    k1Bar += eighth * midBar;
    bendBack(c, u, k1Bar, uBar, gs);
    if (extra) bendBack(c, u, k1Extra, uBar, g); /* (what a crossing read of k1: not the step's) */
}

/* The adjoints of one step's start state and of what the crossing and the sky read of its end. */
struct StepBar {
    float u, w, n[3], v[3], psi, drag;
    float k1, a1[3];
    float nextU, nextN[3], nextPsi, nextDrag;
};

/* ---- a disc crossing taken back (lens.inc:195-289) ------------------------------------------------- */

__device__ void crossingBack(const AdjointView& v, float rhoScale, const RayConst<float>& c, const RayState<float>& s,
                             const StepOut<float>& o, const Crossing<float>& x, float throughBefore,
                             const float* sumBar, float& throughBar, StepBar& b, ConstBar& g) {
    const Frame<float>& f = v.f;
    const int32_t mapCount = ARTF_CUDA_MAP_FLOATS, fluidCount = ARTF_CUDA_FLUID_FLOATS;
    /* the shading's values, as shadeCrossing finds them */
    const float turn = turnsOf(x.cy, x.cx) + x.psiC * kTurn;
    const float m2raw = x.cx * x.cx + x.cy * x.cy, m2 = maxX(m2raw, 1e-6f);
    const float num = x.cx * x.vy - x.cy * x.vx;
    const float rate = (num / m2 + x.dragC) * kTurn;
    const float slope = x.wc / x.uc;
    const float speed2 = x.vx * x.vx + x.vy * x.vy + (x.vz * x.vz + slope * slope);
    const float invSpeed = 1.f / sqrtf(speed2);
    const float muRaw = fabsf(x.vz) * invSpeed, mu = maxX(muRaw, .02f);
    const float slant = f.thickness / 3.f / mu;
    const float reachA = f.discHeight / maxX(fabsf(x.vz), 1e-5f), reachB = c.step * 1.5f;
    const float reach = minX(reachA, reachB);
    const float fluidTime = c.time - f.flow;
    float clearK[3], alphaK[3], densK[3], litK[3], glow = 0.f, clear = throughBefore;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float t = ((float)k + .5f) * (2.f / 3.f) - 1.f;
        const float ds = reach * t, uk = x.uc + x.wc * ds, rhoK = (1.f - f.inner * uk) * rhoScale;
        const bool inside = rhoK > 0.f && rhoK < 1.f;
        float dens = 0.f, dusty = 0.f;
        if (inside) {
            const float rowPos = rhoK * (float)(ARTF_CUDA_MAP_HEIGHT - 1);
            const float rowFloor = minX(floorf(rowPos), (float)(ARTF_CUDA_MAP_HEIGHT - 2));
            const int32_t row0 = truncI(rowFloor);
            const float sp0 = ringSpeedAt(f, v.map, row0), sp1 = ringSpeedAt(f, v.map, row0 + 1);
            const float turnK = turn + rate * ds;
            const float d0 = rowAt(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0, turnK - sp0 * c.time);
            const float d1 = rowAt(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0 + 1, turnK - sp1 * c.time);
            const float fluidPos = rhoK * (float)(ARTF_CUDA_FLUID_HEIGHT - 1);
            const float fluidFloor = minX(floorf(fluidPos), (float)(ARTF_CUDA_FLUID_HEIGHT - 2));
            const int32_t fluidRow = truncI(fluidFloor);
            const float g0 = rowAt(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow, turnK - sp0 * fluidTime);
            const float g1 = rowAt(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow + 1, turnK - sp0 * fluidTime);
            const float gas = g0 + (g1 - g0) * (fluidPos - fluidFloor);
            const float dustPos = rhoK * (float)(ARTF_CUDA_DUST_HEIGHT - 1);
            const int32_t dustRow = truncI(minX(floorf(dustPos), (float)(ARTF_CUDA_DUST_HEIGHT - 1)));
            dusty = rowAt(v.map, mapCount, ARTF_CUDA_DUST_AT, ARTF_CUDA_DUST_WIDTH, dustRow, turnK - sp0 * c.time);
            const float height = t * (reach / f.discHeight);
            const float level = maxX(1.f - x.vz * x.vz * (height * height), 0.f);
            dens = (d0 + (d1 - d0) * (rowPos - rowFloor)) * ((1.f - .1f) + .1f * gas) * level;
        }
        const float depth = slant * dens * (1.f + 25.f * dusty);
        clearK[k] = clear;
        alphaK[k] = depth / (1.f + depth);
        densK[k] = dens;
        litK[k] = 1.f - .97f * dusty;
        glow = glow + clear * alphaK[k] * (dens * litK[k]);
        clear = clear * (1.f - alphaK[k]);
    }
    const float rhoCenter = (1.f - f.inner * x.uc) * rhoScale;
    const int32_t rowIndex = truncI(minX(maxX(rhoCenter, 0.f), 1.f) * (float)(ARTF_CUDA_MAP_HEIGHT - 1));
    float heat = fetch(v.map, clampI(ARTF_CUDA_ROWS_AT + rowIndex + rowIndex + 1, 0, mapCount - 1));
    const float gives = ringGlowAt(f, v.map, rowIndex);
    const float light0 = f.gain * glow * gives;
    float g4 = 1.f;
    float safeU = 0.f, root = 0.f, lift = 1.f, spinRate = 0.f, sqrtB = 0.f, pShift = 0.f, qShift = 1.f, gShift = 1.f;
    bool uHeld = false, bHeld = false;
    if (f.doppler != 0.f) {
        uHeld = !(x.uc > 1e-4f);
        safeU = maxX(x.uc, 1e-4f);
        root = safeU * sqrtf(safeU);
        lift = 1.f + f.a * root;
        spinRate = root / lift;
        const float bRaw = 1.f - 3.f * safeU + (2.f * f.a) * root;
        bHeld = !(bRaw > 1e-4f);
        sqrtB = sqrtf(maxX(bRaw, 1e-4f));
        pShift = c.invEnergy * c.moved;
        qShift = lift * (1.f - spinRate * c.xi);
        gShift = 1.f + f.doppler * (sqrtB * pShift / qShift - 1.f);
        g4 = (gShift * gShift) * (gShift * gShift);
        heat = heat * gShift;
    }
    const int32_t color = truncI(minX(heat * (float)(ARTF_CUDA_COLORS / 2), (float)(ARTF_CUDA_COLORS - 1)));
    const int32_t at = ARTF_CUDA_COLORS_AT + color + color + color;
    const float lightBar = sumBar[0] * fetch(v.map, clampI(at, 0, mapCount - 1)) +
                           sumBar[1] * fetch(v.map, clampI(at + 1, 0, mapCount - 1)) +
                           sumBar[2] * fetch(v.map, clampI(at + 2, 0, mapCount - 1));

    /* ---- back: light = gain glow gives g^4 ---- */
    float ucBar = 0.f, wcBar = 0.f, cxBar = 0.f, cyBar = 0.f, vxBar = 0.f, vyBar = 0.f, vzBar = 0.f, psiCBar = 0.f,
          dragCBar = 0.f;
    if (f.doppler != 0.f) {
        const float shiftBar = lightBar * light0 * 4.f * (gShift * gShift * gShift) * f.doppler;
        const float shift = sqrtB * pShift / qShift;
        const float sqrtBBar = shiftBar * pShift / qShift, pBar = shiftBar * sqrtB / qShift;
        const float qBar = -shiftBar * shift / qShift;
        const float beneathBar = bHeld ? 0.f : sqrtBBar * .5f / sqrtB;
        float safeUBar = -3.f * beneathBar, rootBar = 2.f * f.a * beneathBar;
        g.a += 2.f * root * beneathBar;
        float liftBar = qBar * (1.f - spinRate * c.xi);
        const float spinRateBar = -qBar * lift * c.xi;
        g.xi += -qBar * lift * spinRate;
        rootBar += spinRateBar / lift;
        liftBar += -spinRateBar * root / (lift * lift);
        g.a += liftBar * root;
        rootBar += liftBar * f.a;
        safeUBar += rootBar * 1.5f * sqrtf(safeU);
        if (!uHeld) ucBar += safeUBar;
        g.invEnergy += pBar * c.moved;
    }
    const float light0Bar = lightBar * g4;
    const float glowBar = light0Bar * f.gain * gives;
    {
        /* gives = span^q, span = 1 - rho (1 - inner / outer) */
        const float givesBar = light0Bar * f.gain * glow;
        const float rho = (float)rowIndex / (float)(ARTF_CUDA_MAP_HEIGHT - 1);
        const float span = 1.f - rho * (1.f - f.inner / f.outer);
        g.q += givesBar * gives * logf(span);
        g.inner += givesBar * f.emissivity * gives / span * (rho / f.outer);
    }
    float clearBar = throughBar; /* the transmission after the crossing is the last slice's clear */
    float reachBar = 0.f, slantBar = 0.f, rateBar = 0.f, turnBar = 0.f;
    for (int k = 2; k >= 0; --k) {
        const float t = ((float)k + .5f) * (2.f / 3.f) - 1.f;
        /* glow += clear alpha dens lit;  clear' = clear (1 - alpha) */
        const float alphaBar = glowBar * clearK[k] * densK[k] * litK[k] - clearBar * clearK[k];
        float densBar = glowBar * clearK[k] * alphaK[k] * litK[k];
        const float litBar = glowBar * clearK[k] * alphaK[k] * densK[k];
        clearBar = clearBar * (1.f - alphaK[k]) + glowBar * alphaK[k] * densK[k] * litK[k];
        const float ds = reach * t, uk = x.uc + x.wc * ds, rhoK = (1.f - f.inner * uk) * rhoScale;
        if (!(rhoK > 0.f && rhoK < 1.f)) continue; /* no gas there: nothing reaches back */
        const float rowPos = rhoK * (float)(ARTF_CUDA_MAP_HEIGHT - 1);
        const float rowFloor = minX(floorf(rowPos), (float)(ARTF_CUDA_MAP_HEIGHT - 2)), rowPart = rowPos - rowFloor;
        const int32_t row0 = truncI(rowFloor);
        const float sp0 = ringSpeedAt(f, v.map, row0), sp1 = ringSpeedAt(f, v.map, row0 + 1);
        const float turnK = turn + rate * ds;
        const float T0 = turnK - sp0 * c.time, T1 = turnK - sp1 * c.time, TF = turnK - sp0 * fluidTime;
        const float d0 = rowAt(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0, T0);
        const float d1 = rowAt(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0 + 1, T1);
        const float fluidPos = rhoK * (float)(ARTF_CUDA_FLUID_HEIGHT - 1);
        const float fluidFloor = minX(floorf(fluidPos), (float)(ARTF_CUDA_FLUID_HEIGHT - 2));
        const float fluidPart = fluidPos - fluidFloor;
        const int32_t fluidRow = truncI(fluidFloor);
        const float g0 = rowAt(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow, TF);
        const float g1 = rowAt(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow + 1, TF);
        const float gas = g0 + (g1 - g0) * fluidPart;
        const float dens0 = d0 + (d1 - d0) * rowPart, gasFactor = (1.f - .1f) + .1f * gas;
        const int32_t dustRow =
            truncI(minX(floorf(rhoK * (float)(ARTF_CUDA_DUST_HEIGHT - 1)), (float)(ARTF_CUDA_DUST_HEIGHT - 1)));
        const float dusty = rowAt(v.map, mapCount, ARTF_CUDA_DUST_AT, ARTF_CUDA_DUST_WIDTH, dustRow, T0);
        const float height = t * (reach / f.discHeight);
        const float levelRaw = 1.f - x.vz * x.vz * (height * height), level = maxX(levelRaw, 0.f);
        const float dens = dens0 * gasFactor * level, dust25 = 1.f + 25.f * dusty;
        /* alpha = depth / (1 + depth), depth = slant dens (1 + 25 dusty) */
        const float depth = slant * dens * dust25;
        const float depthBar = alphaBar / ((1.f + depth) * (1.f + depth));
        slantBar += depthBar * dens * dust25;
        densBar += depthBar * slant * dust25;
        const float dustyBar = depthBar * slant * dens * 25.f - .97f * litBar;
        if (levelRaw > 0.f) {
            const float levelBar = densBar * dens0 * gasFactor;
            vzBar += levelBar * (-2.f * x.vz * height * height);
            reachBar += levelBar * (-2.f * x.vz * x.vz * height) * (t / f.discHeight);
        }
        const float dens0Bar = densBar * gasFactor * level, gasBar = densBar * dens0 * level * .1f;
        const float rhoKBar = dens0Bar * (d1 - d0) * (float)(ARTF_CUDA_MAP_HEIGHT - 1) +
                              gasBar * (g1 - g0) * (float)(ARTF_CUDA_FLUID_HEIGHT - 1);
        const float T0Bar = dens0Bar * (1.f - rowPart) * rowSlope(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0, T0) +
                            dustyBar * rowSlope(v.map, mapCount, ARTF_CUDA_DUST_AT, ARTF_CUDA_DUST_WIDTH, dustRow, T0);
        const float T1Bar = dens0Bar * rowPart * rowSlope(v.map, mapCount, 0, ARTF_CUDA_MAP_WIDTH, row0 + 1, T1);
        const float TFBar =
            gasBar * ((1.f - fluidPart) * rowSlope(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow, TF) +
                      fluidPart * rowSlope(v.fluid, fluidCount, 0, ARTF_CUDA_FLUID_WIDTH, fluidRow + 1, TF));
        const float turnKBar = T0Bar + T1Bar + TFBar;
        {
            /* T = turnK - speed time: the rings' speeds in a and inner */
            float dA, dInner;
            const float sp0Bar = -T0Bar * c.time - TFBar * fluidTime, sp1Bar = -T1Bar * c.time;
            speedSlopes(f, row0, sp0, dA, dInner);
            g.a += sp0Bar * dA;
            g.inner += sp0Bar * dInner;
            speedSlopes(f, row0 + 1, sp1, dA, dInner);
            g.a += sp1Bar * dA;
            g.inner += sp1Bar * dInner;
        }
        turnBar += turnKBar;
        rateBar += turnKBar * ds;
        /* rhoK = (1 - inner uk) rhoScale, rhoScale = 1 / (1 - inner / outer);  uk = uc + wc ds;  ds = reach t */
        const float ukBar = -rhoKBar * f.inner * rhoScale;
        g.inner += rhoKBar * (-uk * rhoScale + (1.f - f.inner * uk) * rhoScale * rhoScale / f.outer);
        ucBar += ukBar;
        wcBar += ukBar * ds;
        reachBar += (turnKBar * rate + ukBar * x.wc) * t;
    }
    throughBar = clearBar;
    /* reach = min(height / max(|vz|, 1e-5), 1.5 step) */
    if (reachA < reachB) {
        if (fabsf(x.vz) > 1e-5f) vzBar += -reachBar * reachA / x.vz;
    } else {
        g.step += reachBar * 1.5f;
    }
    /* slant = thickness / 3 / mu;  mu = max(|vz| / sqrt(speed2), .02);  speed2 = vx^2 + vy^2 + vz^2 + slope^2 */
    if (muRaw > .02f) {
        const float muBar = -slantBar * slant / mu;
        vzBar += muBar * invSpeed * (x.vz < 0.f ? -1.f : 1.f);
        const float speed2Bar = muBar * fabsf(x.vz) * -.5f * invSpeed / speed2;
        vxBar += speed2Bar * 2.f * x.vx;
        vyBar += speed2Bar * 2.f * x.vy;
        vzBar += speed2Bar * 2.f * x.vz;
        const float slopeBar = speed2Bar * 2.f * slope; /* slope = wc / uc */
        wcBar += slopeBar / x.uc;
        ucBar += -slopeBar * slope / x.uc;
    }
    {
        /* rate = ((cx vy - cy vx) / max(cx^2 + cy^2, 1e-6) + dragC) / 2 pi */
        const float r = rateBar * kTurn;
        dragCBar += r;
        const float numBar = r / m2, m2Bar = -r * num / (m2 * m2);
        cxBar += numBar * x.vy;
        vyBar += numBar * x.cx;
        cyBar += -numBar * x.vx;
        vxBar += -numBar * x.cy;
        if (m2raw > 1e-6f) cxBar += m2Bar * 2.f * x.cx, cyBar += m2Bar * 2.f * x.cy;
    }
    {
        /* turn = turns(cy, cx) + psiC / 2 pi */
        float dy, dx;
        turnsSlope(x.cy, x.cx, dy, dx);
        cyBar += turnBar * dy;
        cxBar += turnBar * dx;
        psiCBar += turnBar * kTurn;
    }
    /* the crossing's state, a second-order step of hu = part h from the step's start */
    const float h = c.step, hu = x.part * h, hh = hu * hu * .5f;
    const float huBar = ucBar * (s.w + hu * o.k1) + wcBar * o.k1 + cxBar * (s.v[0] + hu * o.a1[0]) +
                        cyBar * (s.v[1] + hu * o.a1[1]) + vxBar * o.a1[0] + vyBar * o.a1[1] + vzBar * o.a1[2];
    b.u += ucBar;
    b.w += ucBar * hu + wcBar;
    b.k1 += ucBar * hh + wcBar * hu;
    b.n[0] += cxBar;
    b.n[1] += cyBar;
    b.v[0] += cxBar * hu + vxBar;
    b.v[1] += cyBar * hu + vyBar;
    b.v[2] += vzBar;
    b.a1[0] += cxBar * hh + vxBar * hu;
    b.a1[1] += cyBar * hh + vyBar * hu;
    b.a1[2] += vzBar * hu;
    b.psi += psiCBar * (1.f - x.part);
    b.nextPsi += psiCBar * x.part;
    b.drag += dragCBar * (1.f - x.part);
    b.nextDrag += dragCBar * x.part;
    g.step += huBar * x.part;
    /* part = nz / (nz - nz') */
    const float partBar = huBar * h + psiCBar * (o.next.psi - s.psi) + dragCBar * (o.next.drag - s.drag);
    const float den = s.n[2] - o.next.n[2];
    b.n[2] += -partBar * o.next.n[2] / (den * den);
    b.nextN[2] += partBar * s.n[2] / (den * den);
}

/* ---- the escape taken back (lens.inc:316-346) ------------------------------------------------------ */

__device__ void skyBack(const AdjointView& v, const RayConst<float>& c, const RayState<float>& s,
                        const RayState<float>& next, float through, const float* sumBar, float& throughBar,
                        StepBar& b, ConstBar& g) {
    const Frame<float>& f = v.f;
    const float part = s.u / (s.u - next.u);
    float away[3];
    for (int k = 0; k < 3; ++k) away[k] = s.n[k] + part * (next.n[k] - s.n[k]);
    const float awayPsi = s.psi + part * (next.psi - s.psi);
    const float len2raw = away[0] * away[0] + away[1] * away[1] + away[2] * away[2];
    const float invA = 1.f / sqrtf(maxX(len2raw, 1e-12f));
    const float psiT = awayPsi * kTurn;
    const float sine = sineOf(psiT), cosine = sineOf(psiT + .25f);
    const float x = away[0] * invA, y = away[1] * invA, m = away[2] * invA;
    const float dir[3] = {x * cosine - y * sine, x * sine + y * cosine, m};
    float rgb[3] = {0.f, 0.f, 0.f};
    starLayer(dir, 90.f, 26, .1f, 1.6f, rgb);
    starLayer(dir, 240.f, 70, .17f, .22f, rgb);
    const float skyTurn = turnsOf(dir[1], dir[0]);
    const float heightPos = (dir[2] * .5f + .5f) * (float)(ARTF_CUDA_SKY_HEIGHT - 1);
    const float skyFloor = minX(floorf(heightPos), (float)(ARTF_CUDA_SKY_HEIGHT - 2)), skyPart = heightPos - skyFloor;
    const int32_t skyRow = truncI(skyFloor);
    const float s0 = rowAt(v.map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH, skyRow, skyTurn);
    const float s1 = rowAt(v.map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH, skyRow + 1, skyTurn);
    const float dust = s0 + (s1 - s0) * skyPart;
    rgb[0] = rgb[0] + dust * .92f;
    rgb[1] = rgb[1] + dust * .86f;
    rgb[2] = rgb[2] + dust;
    float g1 = 1.f, g14 = 1.f;
    if (f.doppler != 0.f) {
        g1 = 1.f + f.doppler * (c.invEnergy * c.moved - 1.f);
        g14 = (g1 * g1) * (g1 * g1);
    }
    const float shown = through * f.stars * g14;
    /* back */
    const float rgbBar[3] = {sumBar[0] * shown, sumBar[1] * shown, sumBar[2] * shown};
    const float shownBar = sumBar[0] * rgb[0] + sumBar[1] * rgb[1] + sumBar[2] * rgb[2];
    throughBar += shownBar * f.stars * g14;
    if (f.doppler != 0.f) g.invEnergy += shownBar * through * f.stars * 4.f * (g1 * g1 * g1) * f.doppler * c.moved;
    float dirBar[3] = {0.f, 0.f, 0.f};
    {
        /* the dust: rows by height, columns by the turn */
        const float dustBar = rgbBar[0] * .92f + rgbBar[1] * .86f + rgbBar[2];
        dirBar[2] += dustBar * (s1 - s0) * .5f * (float)(ARTF_CUDA_SKY_HEIGHT - 1);
        const float turnBar =
            dustBar * ((1.f - skyPart) * rowSlope(v.map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH,
                                                  skyRow, skyTurn) +
                       skyPart * rowSlope(v.map, ARTF_CUDA_MAP_FLOATS, ARTF_CUDA_SKY_AT, ARTF_CUDA_SKY_WIDTH,
                                          skyRow + 1, skyTurn));
        float dy, dx;
        turnsSlope(dir[1], dir[0], dy, dx);
        dirBar[1] += turnBar * dy;
        dirBar[0] += turnBar * dx;
    }
    /* the two star layers (lens.inc:69-86): light = max(1 - d^2 / size^2, 0)^2 gain */
    const float layer[2][4] = {{90.f, 26.f, .1f, 1.6f}, {240.f, 70.f, .17f, .22f}};
    for (int l = 0; l < 2; ++l) {
        const float cells = layer[l][0], size = layer[l][2], gain = layer[l][3];
        const float px = dir[0] * cells, py = dir[1] * cells, pz = dir[2] * cells;
        const float cx = floorf(px), cy = floorf(py), cz = floorf(pz);
        const uint32_t hash = cubeHash((uint32_t)truncI(cx), (uint32_t)truncI(cy), (uint32_t)truncI(cz));
        if (!((int32_t)layer[l][1] > (int32_t)(hash & 255u))) continue;
        const float inv255 = 1.f / 255.f;
        const float e[3] = {px - cx - (float)((hash >> 8) & 255u) * inv255, py - cy - (float)((hash >> 16) & 255u) * inv255,
                            pz - cz - (float)((hash >> 24) & 255u) * inv255};
        const float base = 1.f - (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * (1.f / (size * size));
        if (!(base > 0.f)) continue;
        const float warm = (float)((hash >> 3) & 255u) * inv255;
        const float lightBar = rgbBar[0] * (.75f + warm * .25f) + rgbBar[1] * .82f + rgbBar[2] * (1.f - warm * .45f);
        const float d2Bar = -lightBar * 2.f * base * gain / (size * size);
        for (int k = 0; k < 3; ++k) dirBar[k] += d2Bar * 2.f * e[k] * cells;
    }
    /* dir = (x cos - y sin, x sin + y cos, m), (x, y, m) = away / |away|, the angle psi / 2 pi */
    const float xBar = dirBar[0] * cosine + dirBar[1] * sine, yBar = dirBar[1] * cosine - dirBar[0] * sine;
    const float psiTBar = (dirBar[1] * x - dirBar[0] * y) * sineSlope(psiT) + (dirBar[0] * x + dirBar[1] * y) * sineSlope(psiT + .25f);
    const float awayPsiBar = psiTBar * kTurn;
    float awayBar[3] = {xBar * invA, yBar * invA, dirBar[2] * invA};
    if (len2raw > 1e-12f) {
        const float k = -(xBar * away[0] + yBar * away[1] + dirBar[2] * away[2]) * invA * invA * invA;
        for (int i = 0; i < 3; ++i) awayBar[i] += k * away[i];
    }
    /* away = n + part (n' - n);  awayPsi = psi + part (psi' - psi);  part = u / (u - u') */
    float partBar = awayPsiBar * (next.psi - s.psi);
    for (int k = 0; k < 3; ++k) {
        b.n[k] += awayBar[k] * (1.f - part);
        b.nextN[k] += awayBar[k] * part;
        partBar += awayBar[k] * (next.n[k] - s.n[k]);
    }
    b.psi += awayPsiBar * (1.f - part);
    b.nextPsi += awayPsiBar * part;
    const float den = s.u - next.u;
    b.u += -partBar * next.u / (den * den);
    b.nextU += partBar * s.u / (den * den);
}

/* ---- the ray's set-up taken back (lens.inc:101-152), and onto theta ---------------------------------- */

__device__ void startBack(const AdjointView& v, float nx, float ny, const RayConst<float>& c, const StepBar& x0,
                          ConstBar g, float* grad) {
    const Frame<float>& f = v.f;
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = f.forward[k] + nx * f.right[k] + ny * f.up[k];
    const float inv = 1.f / sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const float e[3] = {d[0] * inv, d[1] * inv, d[2] * inv};
    const float a = f.a, rho = f.place[0], rootDelta = f.place[1], u0 = f.place[2], mu0 = f.place[3];
    const float iE = c.invEnergy, xi = c.xi;
    const float xa = f.metric[3] * e[2] * iE, ac = rho * e[1] * iE;
    const float eta = ac * ac + mu0 * mu0 * (xa * xa - a * a);
    const float P = -u0 * u0 * rootDelta * rho;
    float fieldBar[ARTF_CUDA_GRAD_FIELDS];
#pragma unroll
    for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS; ++k) fieldBar[k] = 0.f;
    /* the first state: u = u0, w = P e_x / E, n = er, v = ac etheta + xa ephi, drag = drag(u0) */
    float u0Bar = x0.u, acBar = 0.f, xaBar = 0.f, eBar[3] = {0.f, 0.f, 0.f}, iEBar = g.invEnergy, xiBar = g.xi;
    if (a != 0.f) dragBack(a, c.xiA, u0, x0.drag, u0Bar, g);
    for (int k = 0; k < 3; ++k) {
        fieldBar[17 + k] += x0.n[k];
        fieldBar[20 + k] += x0.v[k] * ac;
        fieldBar[23 + k] += x0.v[k] * xa;
        acBar += x0.v[k] * f.etheta[k];
        xaBar += x0.v[k] * f.ephi[k];
    }
    const float PBar = x0.w * e[0] * iE;
    eBar[0] += x0.w * P * iE;
    iEBar += x0.w * P * e[0];
    u0Bar += PBar * (-2.f * u0 * rootDelta * rho);
    const float rootDeltaBar = PBar * (-u0 * u0 * rho);
    float rhoBar = PBar * (-u0 * u0 * rootDelta);
    /* xiA = xi a;  uC = -2 a^2 eta;  uB = 3 (eta + (xi - a)^2);  uA = a^2 - K;  K = eta + xi^2 */
    xiBar += g.xiA * a;
    g.a += g.xiA * xi;
    float etaBar = -2.f * a * a * g.uC + 3.f * g.uB;
    g.a += -4.f * a * eta * g.uC;
    const float offBar = 6.f * (xi - a) * g.uB;
    xiBar += offBar;
    g.a += -offBar + 2.f * a * g.uA;
    float bigBar = g.big - g.uA;
    if (c.big > 4.f) bigBar += g.step * (-.5f * c.step / c.big); /* step = C / sqrt(max(K, 4)) */
    etaBar += bigBar;
    xiBar += 2.f * xi * bigBar;
    /* eta = ac^2 + mu0^2 (xa^2 - a^2) */
    acBar += 2.f * ac * etaBar;
    const float mu0Bar = 2.f * mu0 * (xa * xa - a * a) * etaBar;
    xaBar += 2.f * mu0 * mu0 * xa * etaBar;
    g.a += -2.f * a * mu0 * mu0 * etaBar;
    /* ac = rho e_y / E;  xa = m3 e_z / E;  xi = -m2 e_z / E;  E = m0 - m1 e_z */
    rhoBar += acBar * e[1] * iE;
    eBar[1] += acBar * rho * iE;
    iEBar += acBar * rho * e[1] + xaBar * f.metric[3] * e[2] - xiBar * f.metric[2] * e[2];
    fieldBar[12] += xaBar * e[2] * iE;
    fieldBar[11] += -xiBar * e[2] * iE;
    eBar[2] += (xaBar * f.metric[3] - xiBar * f.metric[2]) * iE;
    const float EBar = -iEBar * iE * iE;
    fieldBar[9] += EBar;
    fieldBar[10] += -EBar * e[2];
    eBar[2] += -EBar * f.metric[1];
    /* e = d / |d|, d = forward + nx right + ny up */
    const float dot = (eBar[0] * d[0] + eBar[1] * d[1] + eBar[2] * d[2]) * inv * inv * inv;
    for (int k = 0; k < 3; ++k) {
        const float dBar = eBar[k] * inv - dot * d[k];
        fieldBar[k] += dBar;
        fieldBar[3 + k] += dBar * nx;
        fieldBar[6 + k] += dBar * ny;
    }
    fieldBar[13] += rhoBar;
    fieldBar[14] += rootDeltaBar;
    fieldBar[15] += u0Bar;
    fieldBar[16] += mu0Bar;
    fieldBar[26] += g.a;
    fieldBar[27] += g.inner;
#pragma unroll
    for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS; ++k)
#pragma unroll
        for (int q = 0; q < 5; ++q) grad[q] += fieldBar[k] * v.jacobian[k][q];
    grad[3] += g.q;
}

/* ---- the kernels -------------------------------------------------------------------------------- */

struct alignas(16) Kept {
    RayState<float> s;
    float through; /* the disc's transmission before this step's crossing */
};

/* Each ray's trail from the forward kernel to the reverse one, in device memory, field by field across
 * rays (a warp's 32 rays are adjacent in every field: its loads and stores coalesce):
 *   head  (steps, top, escaped, 0) as ints: steps taken, and steps 0 .. top - 1 go back
 *   bar   (dL/dR, dL/dG, dL/dB, the transmission at the end)
 *   end   the state after the last step (three float4)
 *   saved the state at the start of each segment of K steps (three float4 a segment)
 * A state is (u, w, n0, n1), (n2, v0, v1, v2), (psi, drag, through, 0). */
struct Trail {
    int4* head;
    float4* bar;
    float4* end;    /* 3 x rays */
    float4* saved;  /* 3 x segments x rays */
    size_t rays;
};

/* (streaming stores: the trail, larger than L2, is marked to leave it first, so that the map the forward
 * kernel shades from stays; 0.182 -> 0.180 ms at 512x288) */
__device__ __forceinline__ void storeState(float4* at, size_t stride, const RayState<float>& s, float through) {
    __stcs(at, make_float4(s.u, s.w, s.n[0], s.n[1]));
    __stcs(at + stride, make_float4(s.n[2], s.v[0], s.v[1], s.v[2]));
    __stcs(at + 2 * stride, make_float4(s.psi, s.drag, through, 0.f));
}

__device__ __forceinline__ void loadState(const float4* at, size_t stride, RayState<float>& s, float& through) {
    const float4 a = at[0], b = at[stride], c = at[2 * stride];
    s.u = a.x, s.w = a.y, s.n[0] = a.z, s.n[1] = a.w;
    s.n[2] = b.x, s.v[0] = b.y, s.v[1] = b.z, s.v[2] = b.w;
    s.psi = c.x, s.drag = c.y, through = c.z;
}

struct AdjointLaunch {
    const AdjointView* views;
    float* partials; /* 8 floats a tile: the loss, the five gradient components, two unused */
    unsigned long long* counters;
    const int* order;  /* each view's tiles for the reverse kernel, heaviest first (tilesPerView a view) */
    int* weights;      /* each tile's weight for that order, and each view's count of tiles a weight, */
    unsigned* classes; /* both written by the forward kernel */
    Trail trail;
    int tilesX, tilesPerView, totalTiles, K;
};

/* One step from s, with its crossing's shading. */
__device__ __forceinline__ void stepOnce(const AdjointView& v, float rhoScale, const RayConst<float>& c,
                                         const RayState<float>& s, StepOut<float>& o, float& through, float* sum,
                                         unsigned& crossings) {
    nystromStep(v.f.a, c, s, o);
    Crossing<float> x;
    if (crossingOf(v.f, rhoScale, c, s, o, x)) {
        float turn;
        shadeCrossing(v.f, rhoScale, v.map, v.fluid, c, x, through, sum, &turn);
        ++crossings;
    }
}

/* The ray of pixel (px, py) at its centre: its image position, constants of motion and first state. */
__device__ __forceinline__ void adjointStart(const AdjointView& v, int px, int py, float& nx, float& ny,
                                             RayConst<float>& c, RayState<float>& s) {
    float moment;
    samplePosition(v.h, 0, 0, px, py, 0, &nx, &ny, &moment);
    rayStart(v.f, nx, ny, v.h.disc[2] + v.h.spin[3] * moment, 1.f, c, s);
    if (v.f.a != 0.f) s.drag = dragAt(v.f.a, v.f.a * v.f.a, c.xiA, s.u);
}

/* A warp an 8 x 4 tile of pixels (rays of neighbouring pixels take similar numbers of steps, so a warp's
 * lanes stay busy together), a block four tiles of one view (blockIdx.y).  Each warp writes its tile's
 * sums to the tile's own slot and leaves: no warp waits for another once the view is in shared memory.
 * A tile's rays are trail entries (view * tilesPerView + tile) * 32 + lane. */
struct TileLane {
    int local, px, py;
    size_t tile, ray;
    bool inside;
};

__device__ __forceinline__ bool tileLane(const AdjointLaunch& L, const int* order, const AdjointView& v, TileLane& t) {
    const int lane = (int)(threadIdx.x & 31);
    const int slot = (int)(blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5));
    if (slot >= L.tilesPerView) return false; /* the whole warp: its tile lies past the view */
    t.local = order ? order[(size_t)blockIdx.y * L.tilesPerView + slot] : slot;
    t.px = (t.local % L.tilesX) * 8 + (lane & 7), t.py = (t.local / L.tilesX) * 4 + (lane >> 3);
    t.tile = (size_t)blockIdx.y * L.tilesPerView + t.local;
    t.ray = t.tile * 32 + (size_t)lane;
    t.inside = t.px < v.f.width && t.py < v.f.height;
    return true;
}

__device__ __forceinline__ void copyView(const AdjointLaunch& L, AdjointView& v) {
    const int4* src = reinterpret_cast<const int4*>(L.views + blockIdx.y);
    int4* dst = reinterpret_cast<int4*>(&v);
    for (int k = threadIdx.x; k < (int)(sizeof(AdjointView) / 16); k += kThreads) dst[k] = src[k];
}

/* The forward kernel: each ray traced with its shading, the state kept at the start of every segment of K
 * steps, the loss and its adjoint in the radiance; the tile's loss to its slot.  kK: the checkpoint
 * interval as a constant (the default, 32: segment indices are shifts), or 0 to read it from L. */
template <int kK> __global__ void __launch_bounds__(kThreads, 6) adjointForward(const AdjointLaunch L) {
    __shared__ AdjointView v;
    copyView(L, v);
    __syncthreads();
    TileLane t;
    if (!tileLane(L, nullptr, v, t)) return;
    const int K = kK ? kK : L.K;
    const Trail& tr = L.trail;
    float loss = 0.f;
    int top = 0;
    Tally tally;
    if (t.inside) {
        const Frame<float>& f = v.f;
        float nx, ny;
        RayConst<float> c;
        RayState<float> s;
        adjointStart(v, t.px, t.py, nx, ny, c, s);
        const float rhoScale = recipR(1.f - divR(f.inner, f.outer));
        float sum[3] = {0.f, 0.f, 0.f}, through = 1.f;
        int steps = 0, lastCrossing = -1;
        unsigned crossings = 0;
        bool escaped = false;
        RayState<float> end = s;
        for (int step = 0; step < kMaxSteps; ++step) {
            if (step % K == 0) storeState(tr.saved + (size_t)(3 * (step / K)) * tr.rays + t.ray, tr.rays, s, through);
            StepOut<float> o;
            const unsigned crossed = crossings;
            stepOnce(v, rhoScale, c, s, o, through, sum, crossings);
            if (crossings != crossed) lastCrossing = step;
            ++steps;
            end = o.next;
            if (0.f > o.next.u) {
                const float part = s.u / (s.u - o.next.u);
                float away[3], dir[3];
                for (int k = 0; k < 3; ++k) away[k] = s.n[k] + part * (o.next.n[k] - s.n[k]);
                skyDirection(away, s.psi + part * (o.next.psi - s.psi), dir);
                if (f.stars > 0.f) shadeSky(f, v.map, c, dir, through, sum);
                escaped = true;
                break;
            }
            if (o.next.u > f.uHorizon || !(through > .004f)) break;
            s = o.next;
        }
        const float4 want = v.target[t.py * f.width + t.px];
        const float diff[3] = {sum[0] - want.x, sum[1] - want.y, sum[2] - want.z};
        loss = (diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]) * v.lossScale;
        if (v.hdr) v.hdr[t.py * f.width + t.px] = make_float4(sum[0], sum[1], sum[2], 0.f);
        /* Back from the last step that added to the radiance (the escape, when the sky is shown; else the
         * last disc crossing): after it every adjoint is zero, and a step taken back with zero adjoints
         * adds exactly nothing, so those steps, and the recomputation of segments holding only them, are
         * skipped. */
        top = escaped && f.stars > 0.f ? steps : lastCrossing + 1;
        tr.head[t.ray] = make_int4(steps, top, escaped ? 1 : 0, 0);
        tr.bar[t.ray] = make_float4(2.f * diff[0] * v.lossScale, 2.f * diff[1] * v.lossScale,
                                    2.f * diff[2] * v.lossScale, through);
        storeState(tr.end + t.ray, tr.rays, end, through);
        tally.rays += 1;
        tally.steps += (unsigned)steps;
        tally.crossings += crossings;
        tally.escapes += escaped;
    } else {
        tr.head[t.ray] = make_int4(0, 0, 0, 0);
    }
    flushTally(tally, L.counters);
    for (int off = 16; off > 0; off >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, off);
    /* the tile's weight in the reverse kernel's order: the most steps one of its rays takes back */
    const int most = __reduce_max_sync(0xFFFFFFFFu, top);
    if ((threadIdx.x & 31) == 0) {
        L.partials[t.tile * 8] = loss;
        const int w = min(most >> 3, kAdjointClasses - 1);
        L.weights[t.tile] = w;
        atomicAdd(L.classes + blockIdx.y * kClassStride + w, 1u);
    }
}

/* The reverse kernel: each ray's steps taken back from its last contributing one, then the ray's set-up;
 * the tile's gradient to its slot.  With a checkpoint every K > 1 steps each segment is recomputed from
 * its kept state into a ring of K states and taken back from there; with K = 1 every state was kept and
 * nothing is recomputed: each warp's kept states come through a ring of kStage steps in shared memory,
 * copied there by cp.async kStage - 1 steps ahead of their use. */
template <int kK> __global__ void __launch_bounds__(kThreads, 3) adjointReverse(const AdjointLaunch L) {
    __shared__ AdjointView v;
    copyView(L, v);
    __syncthreads();
    TileLane t;
    if (!tileLane(L, L.order, v, t)) return;
    const int K = kK ? kK : L.K;
    const Trail& tr = L.trail;
    float grad[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int4 head = t.inside ? tr.head[t.ray] : make_int4(0, 0, 0, 0);
    const int steps = head.x, top = head.y;
    const bool escaped = head.z != 0;
    if (top > 0) {
        const Frame<float>& f = v.f;
        const float a = f.a;
        float nx, ny;
        RayConst<float> c;
        RayState<float> start;
        adjointStart(v, t.px, t.py, nx, ny, c, start);
        const float rhoScale = recipR(1.f - divR(f.inner, f.outer));
        const float4 bar = tr.bar[t.ray];
        const float sumBar[3] = {bar.x, bar.y, bar.z}, throughEnd = bar.w;
        const BackTerms bt = backTerms(a, c.step);
        StepBar next;
        memset(&next, 0, sizeof next);
        ConstBar g, gs; /* gs: what the steps' own maps give the constants the step length scales */
        memset(&g, 0, sizeof g);
        memset(&gs, 0, sizeof gs);
        float throughBar = 0.f, direct = 0.f; /* direct: velocities against what crossings add to their adjoints */
        RayState<float> after; /* the state after the step being taken back */
        /* One step taken back: k, the state it started from; after, the state it ended in. */
        auto back = [&](const Kept& k, int step) {
            StepOut<float> o;
            o.next = after;
            o.k1 = bendAt(c, k.s.u);
            accelWith(bt, c.big, k.s.n, o.a1);
            StepBar b;
            memset(&b, 0, sizeof b);
            b.nextU = next.u;
            for (int j = 0; j < 3; ++j) b.nextN[j] = next.n[j];
            b.nextPsi = next.psi;
            b.nextDrag = next.drag;
            if (escaped && step == steps - 1 && f.stars > 0.f)
                skyBack(v, c, k.s, o.next, throughEnd, sumBar, throughBar, b, g);
            Crossing<float> x;
            const bool crossed = crossingOf(f, rhoScale, c, k.s, o, x);
            if (crossed) {
                crossingBack(v, rhoScale, c, k.s, o, x, k.through, sumBar, throughBar, b, g);
                direct += k.s.w * b.w + k.s.v[0] * b.v[0] + k.s.v[1] * b.v[1] + k.s.v[2] * b.v[2];
            }
            radialBack(bt, c, k.s.u, k.s.w, k.s.drag, b.nextU, next.w, b.nextPsi, b.nextDrag, b.k1, crossed, b.u, b.w,
                       b.psi, b.drag, g, gs);
            polarBack(bt, c.big, k.s.n, k.s.v, b.nextN, next.v, b.a1, crossed, b.n, b.v, g, gs);
            next = b;
            after = k.s;
        };
        float unused;
        if constexpr (kK == 1) {
            /* the state after the last step taken back: the ray's end when that step was its last, else kept */
            loadState(top == steps ? tr.end + t.ray : tr.saved + (size_t)(3 * top) * tr.rays + t.ray, tr.rays, after,
                      unused);
            /* The warp walks back together from its highest step, each lane taking back only its own steps
             * (below its top): at each step the active lanes' kept states are one run of 512 bytes in each
             * of the trail's three planes. */
            const int warpTop = __reduce_max_sync(__activemask(), top);
            const float4* lane = tr.saved + t.ray;
            __shared__ float4 stage[kThreads / 32][kStage][3][32];
            float4(*mine)[3][32] = stage[threadIdx.x >> 5];
            const int me = (int)(threadIdx.x & 31);
            auto fetch = [&](int s) {
                if (s >= 0 && s < top) {
                    const float4* from = lane + (size_t)(3 * s) * tr.rays;
                    for (int q = 0; q < 3; ++q) {
                        const unsigned to = (unsigned)__cvta_generic_to_shared(&mine[s % kStage][q][me]);
                        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(to), "l"(from + q * tr.rays)
                                     : "memory");
                    }
                }
                asm volatile("cp.async.commit_group;\n" ::: "memory");
            };
            for (int j = 0; j < kStage - 1; ++j) fetch(warpTop - 1 - j);
            for (int step = warpTop - 1; step >= 0; --step) {
                fetch(step - (kStage - 1)); /* into the slot the step before this one was read from */
                asm volatile("cp.async.wait_group %0;\n" ::"n"(kStage - 1) : "memory");
                if (step < top) {
                    const float4(*at)[32] = mine[step % kStage];
                    const float4 p0 = at[0][me], p1 = at[1][me], p2 = at[2][me];
                    Kept k;
                    k.s.u = p0.x, k.s.w = p0.y, k.s.n[0] = p0.z, k.s.n[1] = p0.w;
                    k.s.n[2] = p1.x, k.s.v[0] = p1.y, k.s.v[1] = p1.z, k.s.v[2] = p1.w;
                    k.s.psi = p2.x, k.s.drag = p2.y, k.through = p2.z;
                    back(k, step);
                }
            }
        } else {
            Kept ring[kK ? kK : kMaxK];
            for (int first = ((top - 1) / K) * K; first >= 0; first -= K) {
                const int last = min(first + K, top); /* steps first .. last - 1 */
                /* the segment's states from its kept start; the state after its last step is the ray's end
                 * when that step was the ray's last, else one more step on */
                RayState<float> r;
                float through;
                loadState(tr.saved + (size_t)(3 * (first / K)) * tr.rays + t.ray, tr.rays, r, through);
                float junk[3] = {0.f, 0.f, 0.f};
                unsigned n = 0;
                for (int step = first; step < last; ++step) {
                    ring[step - first] = Kept{r, through};
                    if (step == steps - 1) break;
                    StepOut<float> o;
                    stepOnce(v, rhoScale, c, r, o, through, junk, n);
                    r = o.next;
                }
                after = r;
                if (last == steps) loadState(tr.end + t.ray, tr.rays, after, unused);
                for (int step = last - 1; step >= first; --step) back(ring[step - first], step);
            }
        }
        /* The step length's adjoint from the motion, over the whole ray at once.  A Nystrom step of length h
         * is the step of length 1 of the motion with its velocities scaled by h and its accelerations'
         * coefficients (K and a^2 for n; uA, uB, uC for u) by h^2, the velocities coming out divided by h;
         * summed over the ray the terms telescope to the first state's velocities against their adjoints,
         * less the velocities against what crossings added to their adjoints, and the scaled coefficients
         * against what the steps gave their adjoints (for a: 2 a^2 d/d(a^2) = a d/da). */
        g.step += (start.w * next.w + start.v[0] * next.v[0] + start.v[1] * next.v[1] + start.v[2] * next.v[2] -
                   direct + 2.f * (c.uA * gs.uA + c.uB * gs.uB + c.uC * gs.uC + c.big * gs.big) + a * gs.a) /
                  c.step;
        g.a += gs.a, g.big += gs.big, g.uA += gs.uA, g.uB += gs.uB, g.uC += gs.uC;
        startBack(v, nx, ny, c, next, g, grad);
    }
    if (t.inside && v.pixelGrads)
        for (int q = 0; q < 5; ++q) v.pixelGrads[(size_t)(t.py * v.f.width + t.px) * 5 + q] = grad[q];
    const int lane = (int)(threadIdx.x & 31);
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        float sum = grad[q];
        for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xFFFFFFFFu, sum, off);
        if (lane == 0) L.partials[t.tile * 8 + 1 + q] = sum;
    }
}

/* ---- heavy tiles first ----------------------------------------------------------------------------
 * Blocks are dispatched in order and a ray's step back costs in proportion to its steps, so the reverse
 * kernel's heaviest tiles go to its first blocks: the launch does not end on a few photon-ring tiles
 * while the rest of the GPU idles.  A tile's weight is what the forward kernel found, the most steps a ray
 * of the tile takes back, in classes of 8 up to 192; a counting sort a view orders the tiles.  (The
 * forward kernel runs in tile order: ordering it too, by a probe ray a tile, cost more than it saved.)
 * Each tile still writes its own partial sums and adjointSums adds them in tile order, so the gradients
 * are the same bits in any order. */

__global__ void __launch_bounds__(128) adjointPlace(const AdjointLaunch L, const int* weights, const unsigned* classes,
                                                    unsigned* cursors, int* order) {
    __shared__ unsigned counts[kAdjointClasses], runs[kAdjointClasses];
    if (threadIdx.x < kAdjointClasses) counts[threadIdx.x] = 0;
    __syncthreads();
    const int local = (int)(blockIdx.x * 128 + threadIdx.x);
    const bool active = local < L.tilesPerView;
    int w = 0;
    unsigned within = 0;
    if (active) {
        w = weights[(size_t)blockIdx.y * L.tilesPerView + local];
        within = atomicAdd(counts + w, 1u);
    }
    __syncthreads();
    if (threadIdx.x < kAdjointClasses) {
        const unsigned* mine = classes + blockIdx.y * kClassStride;
        unsigned before = 0;
        for (int c = kAdjointClasses - 1; c > (int)threadIdx.x; --c) before += mine[c];
        runs[threadIdx.x] = counts[threadIdx.x]
                                ? before + atomicAdd(cursors + blockIdx.y * kClassStride + threadIdx.x, counts[threadIdx.x])
                                : 0u;
    }
    __syncthreads();
    if (active) order[(size_t)blockIdx.y * L.tilesPerView + runs[w] + within] = local;
}

/* Knuth's TwoSum: s + e equals a + b exactly (no products, so no contraction applies). */
__device__ __forceinline__ void twoSum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

/* A sum kept as an unevaluated pair hi + lo of floats: hi + lo += h + l, renormalised. */
__device__ __forceinline__ void addPair(float& hi, float& lo, float h, float l) {
    float s, e;
    twoSum(hi, h, s, e);
    e += lo + l;
    hi = s + e;
    lo = e - (hi - s);
}

/* Each view's six sums in a fixed order: a block a view, each thread adding a stride of the view's tiles,
 * then the threads' sums pairwise within each warp and the warps' in turn.  Every sum is a pair of floats
 * (hi + lo, about 48 bits), so the float pipe does the work that double would give on this GPU's narrow
 * FP64 pipe, and the result does not depend on scheduling. */
__global__ void __launch_bounds__(1024) adjointSums(const float* partials, int tilesPerView, double* results) {
    __shared__ float part[32][6][2];
    const int view = (int)blockIdx.x, lane = (int)(threadIdx.x & 31), warp = (int)(threadIdx.x >> 5);
    const float4* mine = reinterpret_cast<const float4*>(partials + (size_t)view * tilesPerView * 8);
    float hi[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, lo[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int b = (int)threadIdx.x; b < tilesPerView; b += 1024) {
        const float4 x = mine[(size_t)b * 2], y = mine[(size_t)b * 2 + 1];
        const float v[6] = {x.x, x.y, x.z, x.w, y.x, y.y};
#pragma unroll
        for (int k = 0; k < 6; ++k) addPair(hi[k], lo[k], v[k], 0.f);
    }
    for (int round = 0; round < 2; ++round) {
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const float h = __shfl_down_sync(0xFFFFFFFFu, hi[k], off);
                const float l = __shfl_down_sync(0xFFFFFFFFu, lo[k], off);
                addPair(hi[k], lo[k], h, l);
            }
        if (round == 1) break;
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < 6; ++k) part[warp][k][0] = hi[k], part[warp][k][1] = lo[k];
        __syncthreads();
        if (warp != 0) return;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const bool held = lane < (int)(blockDim.x >> 5);
            hi[k] = held ? part[lane][k][0] : 0.f, lo[k] = held ? part[lane][k][1] : 0.f;
        }
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) results[(size_t)view * 8 + k] = (double)hi[k] + (double)lo[k];
}

}  // namespace

size_t adjointViewBytes() { return sizeof(AdjointView); }

int adjointTiles(int width, int height) { return ((width + 7) / 8) * ((height + 3) / 4); }

void adjointFillView(void* slot, const ArtfCudaHoleFrame& frame, const double* jacobian, double emissivity,
                     const float* map, const float* fluid, const float* target, float* hdr, float* pixelGrads) {
    AdjointView v;
    memset(&v, 0, sizeof v);
    v.f.load(frame, frame);
    v.f.analyticTables = 1;
    v.f.emissivity = (float)emissivity;
    v.h = frame;
    for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS; ++k)
        for (int q = 0; q < 5; ++q) v.jacobian[k][q] = (float)jacobian[k * 5 + q];
    v.map = map;
    v.fluid = fluid;
    v.target = (const float4*)target;
    v.hdr = (float4*)hdr;
    v.pixelGrads = pixelGrads;
    v.pixels = (int)(frame.size[0] * frame.size[1]);
    v.lossScale = 1.f / (3.f * (float)v.pixels);
    memcpy(slot, &v, sizeof v);
}

/* The order's scratch: class counts and cursors (zeroed before each launch), then the tiles' weights and
 * order. */
static size_t orderHead(int count) { return sizeof(unsigned) * 2 * kClassStride * (size_t)count; }

size_t adjointOrderBytes(int count, int width, int height) {
    return orderHead(count) + sizeof(int) * 2 * (size_t)count * adjointTiles(width, height);
}

/* The trail's rays: 32 a tile, padding lanes included. */
static size_t trailRays(int count, int width, int height) { return (size_t)count * adjointTiles(width, height) * 32; }

static int trailSegments(int K) { return (kMaxSteps + K - 1) / K; }

size_t adjointTrailBytes(int count, int width, int height, int K) {
    return trailRays(count, width, height) * sizeof(float4) * (2 + 3 + 3 * (size_t)trailSegments(K));
}

cudaError_t launchAdjoint(const void* table, int count, int width, int height, int K, unsigned long long* counters,
                          float* partials, double* results, cudaStream_t stream, void* orderScratch, void* trail) {
    AdjointLaunch L;
    L.views = (const AdjointView*)table;
    L.partials = partials;
    L.counters = counters;
    L.tilesX = (width + 7) / 8;
    L.tilesPerView = adjointTiles(width, height);
    L.totalTiles = L.tilesPerView * count;
    L.K = K;
    L.trail.rays = trailRays(count, width, height);
    L.trail.head = (int4*)trail;
    L.trail.bar = (float4*)(L.trail.head + L.trail.rays);
    L.trail.end = L.trail.bar + L.trail.rays;
    L.trail.saved = L.trail.end + 3 * L.trail.rays;
    if (!orderScratch) return cudaErrorInvalidValue;
    const size_t tiles = (size_t)count * L.tilesPerView;
    unsigned* classes = (unsigned*)orderScratch;
    unsigned* cursors = classes + kClassStride * (size_t)count;
    int* weights = (int*)(cursors + kClassStride * (size_t)count);
    int* order = weights + tiles;
    const cudaError_t e = cudaMemsetAsync(orderScratch, 0, orderHead(count), stream);
    if (e != cudaSuccess) return e;
    const dim3 placeGrid((unsigned)((L.tilesPerView + 127) / 128), (unsigned)count);
    L.order = order;
    L.weights = weights;
    L.classes = classes;
    const unsigned blocks = (unsigned)((L.tilesPerView + kThreads / 32 - 1) / (kThreads / 32));
    const dim3 grid(blocks, (unsigned)count);
    /* the forward kernel, the reverse kernel's order from what it found, the reverse kernel */
    if (K == 32)
        adjointForward<32><<<grid, kThreads, 0, stream>>>(L);
    else if (K == 1)
        adjointForward<1><<<grid, kThreads, 0, stream>>>(L);
    else
        adjointForward<0><<<grid, kThreads, 0, stream>>>(L);
    adjointPlace<<<placeGrid, 128, 0, stream>>>(L, weights, classes, cursors, order);
    if (K == 32)
        adjointReverse<32><<<grid, kThreads, 0, stream>>>(L);
    else if (K == 1)
        adjointReverse<1><<<grid, kThreads, 0, stream>>>(L);
    else
        adjointReverse<0><<<grid, kThreads, 0, stream>>>(L);
    adjointSums<<<(unsigned)count, 1024, 0, stream>>>(partials, L.tilesPerView, results);
    return cudaGetLastError();
}

}  // namespace artf
