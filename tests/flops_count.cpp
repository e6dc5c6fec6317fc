// Counts the floating-point operations of the trace's own formulas (artful_gb300/csrc/lensCore.cuh),
// instantiated on the host with a number type that counts each + - * / sqrt min max as one operation
// (comparisons, floor, abs, sign flips, conversions and loads count none).  Prints one "name count"
// line for each piece the roofline's constants (lensFlops.h) are made of; tests/test_flops.py compiles
// and runs this and checks the constants.
#include <stdio.h>

#include <cmath>
#include <cstdint>

struct Op {
    double v;
    Op() : v(0) {}
    Op(double x) : v(x) {}
};

static long g_ops = 0;

static inline Op operator+(Op a, Op b) { ++g_ops; return Op(a.v + b.v); }
static inline Op operator-(Op a, Op b) { ++g_ops; return Op(a.v - b.v); }
static inline Op operator*(Op a, Op b) { ++g_ops; return Op(a.v * b.v); }
static inline Op operator/(Op a, Op b) { ++g_ops; return Op(a.v / b.v); }
static inline Op operator-(Op a) { return Op(-a.v); }
static inline bool operator<(Op a, Op b) { return a.v < b.v; }
static inline bool operator>(Op a, Op b) { return a.v > b.v; }
static inline bool operator!=(Op a, Op b) { return a.v != b.v; }

/* The core's scalar helpers for Op, found by argument-dependent lookup from its templates. */
static inline Op sqrtR(Op x) { ++g_ops; return Op(std::sqrt(x.v)); }
static inline Op floorR(Op x) { return Op(std::floor(x.v)); }
static inline Op absR(Op x) { return Op(std::fabs(x.v)); }
static inline Op recipR(Op x) { ++g_ops; return Op(1.0 / x.v); }
static inline Op invSqrtR(Op x) { g_ops += 2; return Op(1.0 / std::sqrt(x.v)); }     /* a sqrt, a division */
static inline Op divR(Op a, Op b) { ++g_ops; return Op(a.v / b.v); }
static inline Op divSqrtR(Op a, Op x) { g_ops += 2; return Op(a.v / std::sqrt(x.v)); } /* the same */
static inline Op rootR(Op x) { ++g_ops; return Op(std::sqrt(x.v)); }
static inline Op expR(Op x) { ++g_ops; return Op(std::exp(x.v)); }
static inline Op logR(Op x) { ++g_ops; return Op(std::log(x.v)); }
static inline int32_t truncI(Op x) { return (int32_t)x.v; }

#include "lensCore.cuh"

namespace artf {
template <> inline Op minX<Op>(Op a, Op b) { ++g_ops; return a.v < b.v ? a : b; }
template <> inline Op maxX<Op>(Op a, Op b) { ++g_ops; return a.v > b.v ? a : b; }
}  // namespace artf

using namespace artf;

static float g_map[ARTF_CUDA_MAP_FLOATS];
static float g_fluid[ARTF_CUDA_FLUID_FLOATS];

/* A frame of plausible values; the counts depend on them only through the branches named. */
static Frame<Op> frame(double spin, double doppler) {
    Frame<Op> f;
    for (int c = 0; c < 3; ++c) {
        f.er[c] = Op(c == 2 ? 1.0 : 0.0), f.etheta[c] = Op(c == 0 ? 1.0 : 0.0), f.ephi[c] = Op(c == 1 ? 1.0 : 0.0);
        f.right[c] = Op(c == 1 ? 0.3 : 0.0), f.up[c] = Op(c == 0 ? 0.3 : 0.0), f.forward[c] = Op(c == 2 ? -1.0 : 0.0);
    }
    f.metric[0] = 0.96, f.metric[1] = 0.001, f.metric[2] = 29.0, f.metric[3] = 30.0;
    f.place[0] = 30.0, f.place[1] = 29.0, f.place[2] = 1.0 / 30.0, f.place[3] = 0.2;
    f.a = spin, f.uHorizon = 0.5, f.discHeight = 1e-3, f.shutter = 0.0, f.flow = 0.0;
    for (int c = 0; c < 4; ++c) f.boost[c] = 0.0;
    f.inner = 2.3, f.outer = 12.0, f.time = 0.0, f.thickness = 0.5, f.gain = 1.0, f.doppler = doppler, f.stars = 1.0;
    f.pixelX = f.pixelY = f.share = 1.0;
    f.width = f.height = 64, f.side = 1;
    f.analyticTables = 0;
    f.emissivity = 0.0;
    return f;
}

int main() {
    for (int i = 0; i < ARTF_CUDA_MAP_FLOATS; ++i) g_map[i] = 0.5f;
    for (int i = 0; i < ARTF_CUDA_FLUID_FLOATS; ++i) g_fluid[i] = 1.f;
    for (int spin = 0; spin < 2; ++spin) {
        const char* tag = spin ? "" : "_spinless";
        const Frame<Op> f = frame(spin ? 0.9 : 0.0, 1.0);
        RayConst<Op> c;
        RayState<Op> s;
        /* per ray: the set-up, the first drag and the disc's radial scale (lens.inc:101-163) */
        g_ops = 0;
        rayStart(f, Op(0.1), Op(0.2), Op(0.0), Op(1.0), c, s);
        if (f.a != Op(0.0)) s.drag = dragAt(f.a, f.a * f.a, c.xiA, s.u);
        const Op rhoScale = recipR(Op(1.0) - divR(f.inner, f.outer));
        printf("setup%s %ld\n", tag, g_ops);
        /* the mixed trace's wide work: a ray's set-up (what it takes from the view formed once a view,
         * its step's terms formed once a ray), and one radial and one polar sub-step with those given */
        {
            const StartTerms<Op> view = startTerms(f, Op(1.0));
            const Op a2 = f.a * f.a, twoA2 = Op(2.0) * a2;
            RayConst<Op> cw;
            RayState<Op> sw, next;
            Op k1, a1[3];
            rayStartWith(f, view, Op(0.1), Op(0.2), Op(0.0), cw, sw);
            /* (the mixed trace's wide set-up: the constants of motion alone, and the step's terms; the
             * first state and the step are its FP32 work) */
            RayConst<Op> cm;
            MotionFactors<Op> mf;
            g_ops = 0;
            motionConstants(f, view, Op(0.1), Op(0.2), cm, mf);
            const StepTerms<Op> terms = stepTerms(cw.step);
            printf("wide_start%s %ld\n", tag, g_ops);
            g_ops = 0;
            radialStepWith(f.a, a2, cw, terms, sw, next, k1);
            printf("wide_radial%s %ld\n", tag, g_ops);
            g_ops = 0;
            polarStepWith(a2, twoA2, cw, terms, sw, next, a1);
            printf("wide_polar_whole%s %ld\n", tag, g_ops);
            /* what the turning-point guards run: the radial motion alone, the polar axis component alone */
            Op nu, nw, nz, vz, a1z;
            g_ops = 0;
            radialMotionWith(cw, terms, sw.u, sw.w, nu, nw, k1);
            printf("wide_turn%s %ld\n", tag, g_ops);
            g_ops = 0;
            polarAxisWith(a2, twoA2, cw, terms, sw.n[2], sw.v[2], nz, vz, a1z);
            printf("wide_axis%s %ld\n", tag, g_ops);
        }
        /* one Nystrom step as written: each sub-step recomputes the ray's constant products */
        StepOut<Op> o;
        g_ops = 0;
        nystromStep(f.a, c, s, o);
        printf("step_as_written%s %ld\n", tag, g_ops);
        /* one accepted crossing: its position and its shading, with and without the Doppler shift */
        s.n[0] = Op(0.7), s.n[1] = Op(0.7), s.n[2] = Op(0.1), s.u = Op(0.2), s.w = Op(0.01);
        o.next = s, o.next.n[2] = Op(-0.1), o.k1 = Op(0.0);
        for (int k = 0; k < 3; ++k) s.v[k] = Op(0.3), o.a1[k] = Op(0.0);
        for (int dop = 0; dop < 2; ++dop) {
            Frame<Op> g = f;
            g.doppler = Op(dop ? 1.0 : 0.0);
            Crossing<Op> x;
            Op through = Op(1.0), sum[3] = {Op(0.0), Op(0.0), Op(0.0)}, turn;
            g_ops = 0;
            const bool accepted = crossingOf(g, rhoScale, c, s, o, x);
            shadeCrossing(g, rhoScale, g_map, g_fluid, c, x, through, sum, &turn);
            if (!accepted) return 1;
            printf("crossing%s%s %ld\n", dop ? "" : "_nodoppler", tag, g_ops);
        }
        /* an escape: the last chord's end and the direction in the sky's frame (lens.inc:293-321) */
        o.next.u = Op(-0.01);
        g_ops = 0;
        const Op part = divR(s.u, s.u - o.next.u);
        Op away[3], dir[3];
        for (int k = 0; k < 3; ++k) away[k] = s.n[k] + part * (o.next.n[k] - s.n[k]);
        const Op awayPsi = s.psi + part * (o.next.psi - s.psi);
        skyDirection(away, awayPsi, dir);
        printf("escape%s %ld\n", tag, g_ops);
        /* the stars and sky dust toward it, with the Doppler shift (lens.inc:322-347): the least over
         * directions (no star in either layer's cell) and the most (a star drawn in both) */
        long least = 1L << 30, most = 0;
        for (int d = 0; d < 4096; ++d) {
            const double z = -1.0 + (d + 0.5) * (2.0 / 4096), r = std::sqrt(1.0 - z * z), t = d * 2.399963;
            const Op toward[3] = {Op(r * std::cos(t)), Op(r * std::sin(t)), Op(z)};
            Op sum[3] = {Op(0.0), Op(0.0), Op(0.0)};
            g_ops = 0;
            shadeSky(f, g_map, c, toward, Op(1.0), sum);
            least = g_ops < least ? g_ops : least;
            most = g_ops > most ? g_ops : most;
        }
        printf("sky%s %ld\nsky_with_stars%s %ld\n", tag, least, tag, most);
    }
    return 0;
}
