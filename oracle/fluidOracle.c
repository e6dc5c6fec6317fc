/* Oracle (test infrastructure): the reference's disc fluid, src/scene/fluid.c, restated in
 * scalar C on one thread.  Only tests/ use it, to check the GPU fluid step (artful_gb300/csrc/fluid.cu)
 * byte for byte; it is pinned in turn against the reference's own fluid.c (oracle/_ref, refFluid*) and
 * against the golden hashes in tests/golden/.
 *
 * The model (fluid.c:1-23): isothermal compressible flow on 256 rings of 1024 cells between the disc's
 * edges, density S and the velocity's departure from a circular orbit (vr, w), Kerr's orbital and
 * epicyclic frequencies, eddies stirred in at random, a FARGO-style shift of each ring along itself by
 * its orbit.  Each float expression keeps the reference's order of operations (built without
 * contraction, as the reference is), which is what makes the bytes equal. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define FW 1024                         /* cells around a ring (ARTF_FLUID_WIDTH) */
#define FH 256                          /* rings (ARTF_FLUID_HEIGHT) */
#define DT .2f                          /* fluid.c:28 STEP */
#define ARC (6.2831853f / (float)FW)    /* fluid.c:29 DPHI */
#define MAX_STEPS 48                    /* fluid.c:30 */
#define WARM_STEPS 60                   /* fluid.c:31 */
#define WOUND_TIME 900.f                /* fluid.c:32 */

struct OracleFluid {
    float inner, outer;
    float* dens[2];
    float* radial[2];
    float* orbital[2];
    float* field;
    int cur;
    float radius[FH], rowWidth[FH], angular[FH], epicyclic[FH], sound2[FH], slide[FH], envelope[FH], fall[FH];
    uint32_t state;
    double time;
};

static float clampF(float v, float lo, float hi) { return v < lo ? lo : v > hi ? hi : v; }
static float lesser(float a, float b) { return b < a ? b : a; }
static float greater(float a, float b) { return a < b ? b : a; }
static int atMost(int a, int b) { return a < b ? a : b; }
static int atLeast(int a, int b) { return a > b ? a : b; }

/* fluid.c:49-56: xorshift32, and a uniform float from its top 24 bits */
static uint32_t draw(OracleFluid* f) {
    uint32_t x = f->state;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    f->state = x;
    return x;
}
static float uniform(OracleFluid* f) { return (float)(draw(f) >> 8) * (1.f / 16777216.f); }

/* fluid.c:58-61: smoothstep from a to b */
static float ease(float a, float b, float x) {
    const float t = clampF((x - a) / (b - a), 0.f, 1.f);
    return t * t * (3.f - 2.f * t);
}

/* fluid.c:63-69 */
static uint32_t cellHash(uint32_t x, uint32_t y, uint32_t seed) {
    uint32_t h = x * 0x9E3779B1u ^ y * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

/* fluid.c:71-80: value noise wrapping every `period` across x */
static float noise(float x, float y, uint32_t period, uint32_t seed) {
    const float fx = floorf(x), fy = floorf(y), tx = x - fx, ty = y - fy;
    const uint32_t x0 = (uint32_t)fx & (period - 1), x1 = (x0 + 1) & (period - 1), y0 = (uint32_t)fy, y1 = y0 + 1;
    const float v00 = (float)(cellHash(x0, y0, seed) >> 8), v10 = (float)(cellHash(x1, y0, seed) >> 8);
    const float v01 = (float)(cellHash(x0, y1, seed) >> 8), v11 = (float)(cellHash(x1, y1, seed) >> 8);
    const float sx = tx * tx * (3.f - 2.f * tx), sy = ty * ty * (3.f - 2.f * ty);
    const float lo = v00 + (v10 - v00) * sx, hi = v01 + (v11 - v01) * sx;
    return (lo + (hi - lo) * sy) * (1.f / 16777216.f);
}

/* fluid.c:82-93: bilinear, wrapping around the ring, held at the first and last rings */
static float bilinear(const float* a, float x, float y) {
    const float fy = clampF(y, 0.f, (float)(FH - 1) - .001f);
    const int y0 = (int)fy;
    const float py = fy - (float)y0;
    const float fx = floorf(x), px = x - fx;
    const int x0 = (int)fx & (FW - 1), x1 = (x0 + 1) & (FW - 1);
    const float* lo = a + (size_t)y0 * FW;
    const float* hi = lo + FW;
    const float top = lo[x0] + (lo[x1] - lo[x0]) * px, bottom = hi[x0] + (hi[x1] - hi[x0]) * px;
    return top + (bottom - top) * py;
}

/* fluid.c:96-124: the velocities carried along themselves, then pushed (w first, its new value used at once) */
static void velocities(OracleFluid* f) {
    const int n = f->cur;
    const float* s = f->dens[n];
    const float* vr = f->radial[n];
    const float* w = f->orbital[n];
    for (int j = 0; j < FH; ++j) {
        float* outR = f->radial[n ^ 1] + (size_t)j * FW;
        float* outW = f->orbital[n ^ 1] + (size_t)j * FW;
        const float r = f->radius[j], invR = 1.f / r, c2 = f->sound2[j], om = f->angular[j], sw = f->epicyclic[j];
        const float toCells = DT / (r * ARC), toRows = DT / f->rowWidth[j];
        const int up = atMost(j + 1, FH - 1), down = atLeast(j - 1, 0);
        const float invSpan = 1.f / (f->radius[up] - f->radius[down]), invArc = 1.f / (2.f * r * ARC);
        const float keep = 1.f - DT * .04f * om;
        for (int i = 0; i < FW; ++i) {
            const size_t at = (size_t)j * FW + i;
            const float x = (float)i - w[at] * toCells, y = (float)j - vr[at] * toRows;
            const float v0 = bilinear(vr, x, y), w0 = bilinear(w, x, y);
            const float inv = 1.f / s[at];
            const float gradR = (s[(size_t)up * FW + i] - s[(size_t)down * FW + i]) * invSpan * inv;
            const float gradPhi = (s[(size_t)j * FW + ((i + 1) & (FW - 1))] - s[(size_t)j * FW + ((i - 1) & (FW - 1))]) *
                                  invArc * inv;
            const float w1 = w0 + DT * (-sw * v0 - v0 * w0 * invR - c2 * gradPhi);
            const float v1 = v0 + DT * (2.f * om * w1 + w1 * w1 * invR - c2 * gradR);
            outW[i] = clampF(w1 * keep, -.4f, .4f);
            outR[i] = clampF(v1 * keep, -.4f, .4f);
        }
    }
}

/* fluid.c:126-151: the density carried by the new velocities, spread or heaped, drifting in, refilled */
static void densities(OracleFluid* f) {
    const int n = f->cur;
    const float* s = f->dens[n];
    const float* vr = f->radial[n ^ 1];
    const float* w = f->orbital[n ^ 1];
    for (int j = 0; j < FH; ++j) {
        float* out = f->dens[n ^ 1] + (size_t)j * FW;
        const float r = f->radius[j], invR = 1.f / r;
        const float toCells = DT / (r * ARC), toRows = DT / f->rowWidth[j];
        const int up = atMost(j + 1, FH - 1), down = atLeast(j - 1, 0);
        const float rUp = f->radius[up], rDown = f->radius[down], invSpan = 1.f / (rUp - rDown);
        const float invArc = 1.f / (2.f * r * ARC);
        const float drift = -.004f, refill = DT * .002f * f->angular[j];
        for (int i = 0; i < FW; ++i) {
            const size_t at = (size_t)j * FW + i;
            const float x = (float)i - w[at] * toCells, y = (float)j - (vr[at] + drift) * toRows;
            const float moved = bilinear(s, x, y);
            const float spread = (rUp * vr[(size_t)up * FW + i] - rDown * vr[(size_t)down * FW + i]) * invSpan * invR +
                                 (w[(size_t)j * FW + ((i + 1) & (FW - 1))] - w[(size_t)j * FW + ((i - 1) & (FW - 1))]) *
                                     invArc;
            const float next = moved * (1.f - DT * clampF(spread, -2.f, 2.f));
            out[i] = clampF(next + (1.f - next) * refill, .03f, 8.f);
        }
    }
}

/* fluid.c:153-161: a ring moved along itself by `cells`, by a Catmull-Rom cubic held within its two middle
 * neighbours */
static void slideRing(const float* in, float* out, float cells) {
    const float whole = floorf(cells), t = 1.f - (cells - whole), t2 = t * t, t3 = t2 * t;
    const int b = -(int)whole - 1;
    const float k0 = -.5f * t + t2 - .5f * t3, k1 = 1.f - 2.5f * t2 + 1.5f * t3;
    const float k2 = .5f * t + 2.f * t2 - 1.5f * t3, k3 = -.5f * t2 + .5f * t3;
    for (int i = 0; i < FW; ++i) {
        const float p0 = in[(i + b - 1) & (FW - 1)], p1 = in[(i + b) & (FW - 1)];
        const float p2 = in[(i + b + 1) & (FW - 1)], p3 = in[(i + b + 2) & (FW - 1)];
        out[i] = clampF(k0 * p0 + k1 * p1 + k2 * p2 + k3 * p3, lesser(p1, p2), greater(p1, p2));
    }
}

/* fluid.c:163-173: every ring by its own orbit, from the new fields back into the current ones */
static void slideAll(OracleFluid* f) {
    const int n = f->cur ^ 1;
    for (int j = 0; j < FH; ++j) {
        const size_t at = (size_t)j * FW;
        slideRing(f->dens[n] + at, f->dens[n ^ 1] + at, f->slide[j]);
        slideRing(f->radial[n] + at, f->radial[n ^ 1] + at, f->slide[j]);
        slideRing(f->orbital[n] + at, f->orbital[n ^ 1] + at, f->slide[j]);
    }
}

/* fluid.c:175-186: what the backends read, where the density tears below the disc's envelope */
static void showField(OracleFluid* f) {
    for (int j = 0; j < FH; ++j) {
        const float* s = f->dens[f->cur] + (size_t)j * FW;
        float* out = f->field + (size_t)j * FW;
        for (int i = 0; i < FW; ++i) {
            const float v = s[i] * f->envelope[j];
            out[i] = f->fall[j] * ease(.1f, 1.1f, v) * lesser(v, 2.2f);
        }
    }
}

/* fluid.c:188-219: one eddy (a whirl with a clump of gas at its heart), its draws in the reference's order */
static void eddy(OracleFluid* f, int small) {
    float* s = f->dens[f->cur];
    float* vr = f->radial[f->cur];
    float* w = f->orbital[f->cur];
    const float u = uniform(f), r0 = f->inner + (f->outer - f->inner) * u * u;
    int j0 = 0;
    while (j0 < FH - 1 && f->radius[j0] < r0) ++j0;
    const int i0 = (int)(draw(f) & (FW - 1));
    const float size = r0 * (small ? .006f + .02f * uniform(f) : .02f + .1f * uniform(f));
    const float c = sqrtf(f->sound2[j0]);
    float strength = 0.f;
    if (!small) {
        const float sign = uniform(f) < .5f ? -1.f : 1.f;
        strength = sign * c * (.3f + .7f * uniform(f));
    }
    const float clump = (uniform(f) - .42f) * (small ? 1.5f : .5f);
    const float invSize2 = 1.f / (size * size);
    const int reach = atMost((int)(2.5f * size / (r0 * ARC)) + 1, FW / 2 - 1);
    for (int j = 0; j < FH; ++j) {
        const float dr = f->radius[j] - r0;
        if (dr * dr > 6.25f * size * size) continue;
        for (int di = -reach; di <= reach; ++di) {
            const float dx = (float)di * f->radius[j] * ARC;
            const float d2 = (dr * dr + dx * dx) * invSize2;
            if (d2 > 6.25f) continue;
            const float g = 1.f - d2 * .16f, shape = g * g * g;
            const size_t at = (size_t)j * FW + (size_t)((i0 + di) & (FW - 1));
            vr[at] -= strength * shape * dx / size;
            w[at] += strength * shape * dr / size;
            s[at] = clampF(s[at] * (1.f + clump * shape), .03f, 8.f);
        }
    }
}

/* fluid.c:221-229: each ring's mean density drawn back towards 1 (a sum in ring order) */
static void balance(OracleFluid* f) {
    for (int j = 0; j < FH; ++j) {
        float* s = f->dens[f->cur] + (size_t)j * FW;
        float sum = 0;
        for (int i = 0; i < FW; ++i) sum += s[i];
        const float mean = sum * (1.f / (float)FW), scale = 1.f + .03f * (1.f / mean - 1.f);
        for (int i = 0; i < FW; ++i) s[i] = clampF(s[i] * scale, .03f, 8.f);
    }
}

/* fluid.c:231-241 */
static void advanceOnce(OracleFluid* f) {
    for (int k = 0; k < 2; ++k) eddy(f, 0);
    for (int k = 0; k < 14; ++k) eddy(f, 1);
    velocities(f);
    densities(f);
    slideAll(f);
    balance(f);
    f->time += DT;
}

void oracleFluidFree(OracleFluid* f) {
    if (!f) return;
    for (int k = 0; k < 2; ++k) free(f->dens[k]), free(f->radial[k]), free(f->orbital[k]);
    free(f->field);
    free(f);
}

/* fluid.c:255-317 */
OracleFluid* oracleFluidNew(float inner, float outer, float spin, double time) {
    OracleFluid* f = calloc(1, sizeof *f);
    if (!f) return NULL;
    f->inner = inner, f->outer = outer, f->state = 0x9E3779B9u, f->time = time;
    for (int k = 0; k < 2; ++k) {
        f->dens[k] = calloc((size_t)FW * FH, sizeof(float));
        f->radial[k] = calloc((size_t)FW * FH, sizeof(float));
        f->orbital[k] = calloc((size_t)FW * FH, sizeof(float));
    }
    f->field = calloc((size_t)FW * FH, sizeof(float));
    const float k = 1.f - inner / outer;
    for (int j = 0; j < FH; ++j) {
        const float rho = (float)j / (float)(FH - 1), r = inner / (1.f - rho * k);
        f->radius[j] = r;
        const float root = sqrtf(r), om = 1.f / (r * root + spin);
        f->angular[j] = om;
        const float kappa2 = om * om * (1.f - 6.f / r + 8.f * spin / (r * root) - 3.f * spin * spin / (r * r));
        f->epicyclic[j] = greater(kappa2, -.5f * om * om) / (2.f * om);
        const float c = .03f * r * om;
        f->sound2[j] = c * c;
        f->slide[j] = om * DT / ARC;
        f->envelope[j] = ease(inner + .5f, inner + 2.2f, r) * (1.f - .86f * ease(outer * .12f, outer * .8f, r));
        f->fall[j] = sqrtf(inner / r);
    }
    for (int j = 0; j < FH; ++j)
        f->rowWidth[j] = (f->radius[atMost(j + 1, FH - 1)] - f->radius[atLeast(j - 1, 0)]) * (j == 0 || j == FH - 1 ? 1.f : .5f);
    /* the gas as clumps the shear has long been drawing out (fluid.c:291-311) */
    float* s = f->dens[0];
    for (int j = 0; j < FH; ++j) {
        const float rho = (float)j / (float)(FH - 1), wound = f->angular[j] * WOUND_TIME / 6.2831853f;
        for (int i = 0; i < FW; ++i) {
            float turn = (float)i / (float)FW - wound;
            turn -= floorf(turn);
            float sum = 0, amplitude = .5f, total = 0, across = 14.f;
            uint32_t period = 16;
            for (uint32_t o = 0; o < 5; ++o) {
                sum += amplitude * noise(turn * (float)period, rho * across, period, 7 + o);
                total += amplitude;
                amplitude *= .72f;
                period *= 2;
                across *= 2.f;
            }
            const float v = sum / total;
            s[(size_t)j * FW + i] = .06f + 3.4f * ease(.34f, .68f, v) * ease(.34f, .68f, v);
        }
    }
    for (int e = 0; e < 200; ++e) eddy(f, 0);
    for (int e = 0; e < WARM_STEPS; ++e) advanceOnce(f);
    f->time = time;
    showField(f);
    return f;
}

/* fluid.c:319-333 */
int oracleFluidAdvance(OracleFluid* f, double time) {
    if (time - f->time < DT) {
        if (time < f->time - 8.0) f->time = time;
        return 0;
    }
    int steps = (int)((time - f->time) / DT);
    if (steps > MAX_STEPS) {
        f->time = time - (double)MAX_STEPS * DT;
        steps = MAX_STEPS;
    }
    for (int e = 0; e < steps; ++e) advanceOnce(f);
    showField(f);
    return 1;
}

double oracleFluidRead(const OracleFluid* f, float* out) {
    memcpy(out, f->field, sizeof(float) * FW * FH);
    return f->time;
}
