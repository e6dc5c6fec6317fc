/* Oracle (test infrastructure): the reference's painted disc map, src/scene/hole.c:14-197
 * (buildDisc and setRings), restated in scalar C.  Only tests/ use it, to check the GPU painter
 * (artful_gb300/csrc/disc.cu) byte for byte; it is pinned against the reference's own map (oracle/_ref,
 * refMap) and against the golden hash in tests/golden/.
 *
 * The map: gas as strands along each orbit and torn clouds (2048 x 1024, rows even in 1/r), scaled to a
 * mean of 1 over its inner half; dust lanes (1024 x 256); a black-body colour table (256); the sky's dust
 * band (1024 x 512); per row the ring's orbit speed, heat and glow for a disc (inner, outer, spin).  No
 * libm beyond floor, fabs and sqrt: the same bits on every host (hole.c:5-6). */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>

#define MAP_W 2048
#define MAP_H 1024
#define ROWS_AT (MAP_W * MAP_H)
#define NCOLOURS 256
#define COLOURS_AT (ROWS_AT + MAP_H * 2)
#define SKY_W 1024
#define SKY_H 512
#define SKY_AT (COLOURS_AT + NCOLOURS * 3)
#define GLOW_AT (SKY_AT + SKY_W * SKY_H)
#define DUST_W 1024
#define DUST_H 256
#define DUST_AT (GLOW_AT + MAP_H)
#define DISC_KELVIN 4500.f  /* hole.c:180 */
#define TABLE_KELVIN 6500.f /* the colour table's middle (sceneInternal.h ARTF_HOLE_KELVIN) */

static float clampF(float v, float lo, float hi) { return v < lo ? lo : v > hi ? hi : v; }
static float greater(float a, float b) { return a < b ? b : a; }

/* hole.c:14-21 */
static uint32_t texHash(uint32_t x, uint32_t y, uint32_t seed) {
    uint32_t h = x * 0x9E3779B1u ^ y * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    return h ^ h >> 15;
}

/* hole.c:23-26 */
static float ease(float a, float b, float x) {
    const float t = clampF((x - a) / (b - a), 0.f, 1.f);
    return t * t * (3.f - 2.f * t);
}

/* hole.c:29-39: value noise repeating every period in x (coordinates through a signed integer) */
static float lattice(float x, float y, uint32_t period, uint32_t seed) {
    const float fx = floorf(x), fy = floorf(y), tx = x - fx, ty = y - fy;
    const uint32_t x0 = (uint32_t)(int32_t)fx % period, x1 = (x0 + 1) % period, y0 = (uint32_t)(int32_t)fy, y1 = y0 + 1;
    const float v00 = (float)(texHash(x0, y0, seed) >> 8), v10 = (float)(texHash(x1, y0, seed) >> 8);
    const float v01 = (float)(texHash(x0, y1, seed) >> 8), v11 = (float)(texHash(x1, y1, seed) >> 8);
    const float sx = tx * tx * (3.f - 2.f * tx), sy = ty * ty * (3.f - 2.f * ty);
    const float lo = v00 + (v10 - v00) * sx, hi = v01 + (v11 - v01) * sx;
    return (lo + (hi - lo) * sy) * (1.f / 16777216.f);
}

/* hole.c:42-53: octaves, 0 to 1 */
static float octaves(float x, float y, uint32_t period, float scaleY, float falloff, float stretch, int count,
                     uint32_t seed) {
    float sum = 0, amplitude = .5f, total = 0;
    for (int o = 0; o < count; ++o) {
        sum += amplitude * lattice(x * (float)period, y * scaleY, period, seed + (uint32_t)o);
        total += amplitude;
        amplitude *= falloff;
        period *= 2;
        scaleY *= stretch;
    }
    return sum / total;
}

/* hole.c:56-60: e^x as (1 + x / 2^20)^(2^20) */
static double powerExp(double x) {
    double v = 1.0 + x / 1048576.0;
    for (int i = 0; i < 20; ++i) v *= v;
    return v;
}

/* hole.c:63-89: Planck's law at three wavelengths, balanced at 6500 K, film's dyes, at most 1 */
static void bodyColour(double kelvin, float* rgb) {
    static const double metres[3] = {611e-9, 549e-9, 464e-9};
    double v[3], white[3], most = 0;
    for (int c = 0; c < 3; ++c) {
        const double l = metres[c], l2 = l * l;
        v[c] = 1.0 / (l2 * l2 * l * (powerExp(.014388 / (l * kelvin)) - 1.0));
        white[c] = 1.0 / (l2 * l2 * l * (powerExp(.014388 / (l * 6500.0)) - 1.0));
    }
    for (int c = 0; c < 3; ++c) {
        v[c] /= white[c];
        if (v[c] > most) most = v[c];
    }
    v[1] *= .6;
    v[2] *= .72;
    for (int c = 0; c < 3; ++c) rgb[c] = (float)(v[c] / most);
}

/* hole.c:92-95 */
static float crest(float v) {
    const float r = 1.f - fabsf(2.f * v - 1.f);
    return r * r;
}

/* hole.c:101-124: strands along each orbit, wandering, torn clouds, a fraying outer edge */
static float gasAt(float turn, float rho) {
    const float wander = .045f * (octaves(turn, rho, 3, 5.f, .5f, 2.f, 4, 101) - .5f) +
                         .012f * (octaves(turn, rho, 11, 24.f, .5f, 2.f, 3, 107) - .5f);
    float along = turn + .03f * (octaves(turn, rho, 5, 9.f, .5f, 2.f, 3, 113) - .5f);
    along -= floorf(along);
    const float across = rho + wander;
    float hair = 0, amplitude = .5f, total = 0, scale = 600.f;
    uint32_t period = 6;
    for (int o = 0; o < 6; ++o) {
        hair += amplitude * crest(lattice(along * (float)period, across * scale, period, 120u + (uint32_t)o));
        total += amplitude;
        amplitude *= .62f;
        period *= 2;
        scale *= 1.75f;
    }
    hair /= total;
    const float cloud = octaves(along, across, 7, 34.f, .55f, 2.f, 5, 131);
    const float outer = ease(.85f, 1.f, rho);
    const float torn = ease(.3f + .08f * outer, .7f + .08f * outer, cloud);
    const float gaps = 1.f + (torn - 1.f) * ease(.1f, .6f, rho);
    const float edge = ease(0.f, .02f, rho) * (1.f - ease(.9f, 1.f, across));
    return edge * (.25f + 2.2f * hair) * (.04f + 1.5f * gaps);
}

void oraclePaintDisc(float* map) {
    for (int y = 0; y < MAP_H; ++y) {
        const float rho = (float)y / (float)(MAP_H - 1), thin = 1.f - .887f * rho;
        for (int x = 0; x < MAP_W; ++x) {
            float turn = (float)x / (float)MAP_W + rho * .09f;
            turn -= floorf(turn);
            map[(size_t)y * MAP_W + x] = gasAt(turn, rho) * thin * thin;
        }
    }
    /* the gas to a mean of 1 over the inner half (hole.c:143-147: a double sum in texel order) */
    double sum = 0;
    for (size_t i = 0; i < (size_t)MAP_W * (MAP_H / 2); ++i) sum += map[i];
    const float scale = (float)((double)MAP_W * (MAP_H / 2) / sum);
    for (size_t i = 0; i < (size_t)MAP_W * MAP_H; ++i) map[i] *= scale;
    /* dust lanes (hole.c:150-159) */
    for (int y = 0; y < DUST_H; ++y) {
        const float rho = (float)y / (float)(DUST_H - 1), outward = ease(.25f, .8f, rho);
        for (int x = 0; x < DUST_W; ++x) {
            const float turn = (float)x / (float)DUST_W;
            map[DUST_AT + y * DUST_W + x] = outward * ease(.45f, .7f, octaves(turn, rho, 4, 90.f, .55f, 2.f, 5, 151));
        }
    }
    /* colours (hole.c:161-166) */
    for (int i = 0; i < NCOLOURS; ++i) {
        const double kelvin = greater(TABLE_KELVIN * (double)i / (NCOLOURS / 2), 400.0);
        bodyColour(kelvin, map + COLOURS_AT + i * 3);
    }
    /* the sky's dust band (hole.c:168-177) */
    for (int y = 0; y < SKY_H; ++y) {
        const float height = (float)y / (float)(SKY_H - 1);
        for (int x = 0; x < SKY_W; ++x) {
            const float turn = (float)x / (float)SKY_W;
            const float bent = height - .5f + .22f * (lattice(turn * 2.f, 3.f, 2, 41) - .5f) +
                               .1f * (lattice(turn * 3.f, 5.f, 3, 42) - .5f);
            const float band = 1.f - ease(0.f, .3f, fabsf(bent));
            const float dust = octaves(turn, height, 8, 8.f, .58f, 2.f, 6, 51);
            map[SKY_AT + y * SKY_W + x] = .0006f + band * band * ease(.3f, .75f, dust) * .006f;
        }
    }
}

/* The inner half's sum of the unscaled gas two ways: in texel order (hole.c:143-144, the reference's)
 * and in the order the GPU's painter adds it (`blocks` runs of texels, each run summed by 256 strided
 * threads and a pairwise tree, then the runs in order), with the float scale each gives.  The gas takes
 * no disc parameter, so these are the same for every disc. */
void oracleGasSums(int blocks, double* sums, float* scales) {
    const size_t texels = (size_t)MAP_W * (MAP_H / 2);
    float* gas = (float*)malloc(sizeof(float) * texels);
    for (int y = 0; y < MAP_H / 2; ++y) {
        const float rho = (float)y / (float)(MAP_H - 1), thin = 1.f - .887f * rho;
        for (int x = 0; x < MAP_W; ++x) {
            float turn = (float)x / (float)MAP_W + rho * .09f;
            turn -= floorf(turn);
            gas[(size_t)y * MAP_W + x] = gasAt(turn, rho) * thin * thin;
        }
    }
    double ordered = 0;
    for (size_t i = 0; i < texels; ++i) ordered += gas[i];
    const size_t per = texels / (size_t)blocks;
    double tree = 0, part[256];
    for (int b = 0; b < blocks; ++b) {
        const float* run = gas + (size_t)b * per;
        for (int t = 0; t < 256; ++t) {
            double s = 0;
            for (size_t i = (size_t)t; i < per; i += 256) s += run[i];
            part[t] = s;
        }
        for (int width = 128; width > 0; width >>= 1)
            for (int t = 0; t < width; ++t) part[t] += part[t + width];
        tree += part[0];
    }
    free(gas);
    sums[0] = ordered, sums[1] = tree;
    scales[0] = (float)((double)texels / ordered), scales[1] = (float)((double)texels / tree);
}

/* hole.c:186-197: each ring's orbit speed (turns a unit time), heat, and glow */
void oracleSetRings(float* map, float inner, float outer, float spin) {
    for (int y = 0; y < MAP_H; ++y) {
        const float rho = (float)y / (float)(MAP_H - 1), r = inner / (1.f - rho * (1.f - inner / outer));
        map[ROWS_AT + y * 2] = 1.f / (6.2831853f * (r * sqrtf(r) + spin));
        map[ROWS_AT + y * 2 + 1] = DISC_KELVIN / TABLE_KELVIN;
        const float out = r / inner;
        map[GLOW_AT + y] = 6.f * out * sqrtf(out);
    }
}
