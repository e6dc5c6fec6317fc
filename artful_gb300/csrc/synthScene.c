/* artful_cuda — the synthetic scenes of the benchmark configurations, and the map tables they share
 * with the reference's painted disc, in C11.  The rings' tables restate the reference's
 * src/scene/hole.c:10-12, 186-197 (setRings) and its colour table hole.c:54-85, 159-164; the synthetic
 * disc and sky (value noise in (row, azimuth) with emissivity r^-q through the glow table, and a seeded
 * star catalogue splatted into the sky) are this library's own workload generator.
 *
 * The library builds this file, and so does the oracle's library: both arms of the benchmark trace the
 * same inputs without the CPU arm loading the CUDA library.  Nothing here calls exp, log or pow: the maps
 * are integer hashing and IEEE + - * / sqrt (built with -ffp-contract=off), so that an x86 host and an
 * Arm host write the same bits. */
#include "artful_cuda.h"

#include <math.h>
#include <stdint.h>
#include <string.h>

static float fmaxRef(float a, float b) { return a < b ? b : a; }
/* ---- map tables ----------------------------------------------------------------------------- */

/* Map rows are even in 1/r between inner (row 0) and outer (the last row). */
static float rowRadius(float rho, float inner, float outer) { return inner / (1.f - rho * (1.f - inner / outer)); }

#define DISC_KELVIN 4500.f  /* the disc's one temperature (the reference's HOLE_KELVIN) */
#define TABLE_KELVIN 6500.0 /* heat 1 is this; the colour table's middle */

static void ringSpeedHeatRows(float* rows, float inner, float outer, float spin) {
    for (int y = 0; y < ARTF_CUDA_MAP_HEIGHT; ++y) {
        const float r = rowRadius((float)y / (float)(ARTF_CUDA_MAP_HEIGHT - 1), inner, outer);
        rows[y * 2] = 1.f / (6.2831853f * (r * sqrtf(r) + spin));
        rows[y * 2 + 1] = DISC_KELVIN / (float)TABLE_KELVIN;
    }
}

static void ringSpeedHeat(float* map, float inner, float outer, float spin) {
    ringSpeedHeatRows(map + ARTF_CUDA_ROWS_AT, inner, outer, spin);
}

void artfCudaHoleRings(float* rows, float* glow, float inner, float outer, float spin) {
    ringSpeedHeatRows(rows, inner, outer, spin);
    for (int y = 0; y < ARTF_CUDA_MAP_HEIGHT; ++y) {
        const float r = rowRadius((float)y / (float)(ARTF_CUDA_MAP_HEIGHT - 1), inner, outer);
        const float out = r / inner;
        glow[y] = 6.f * out * sqrtf(out);
    }
}

void artfCudaSetRings(float* map, float inner, float outer, float spin) {
    artfCudaHoleRings(map + ARTF_CUDA_ROWS_AT, map + ARTF_CUDA_GLOW_AT, inner, outer, spin);
}

/* e^x as (1 + x / 2^20)^(2^20): multiplications only (the reference's exactExp). */
static double expBySquaring(double x) {
    double v = 1.0 + x / 1048576.0;
    for (int i = 0; i < 20; ++i) v *= v;
    return v;
}

/* Planck's spectral radiance at the three wavelengths that stand for a screen's primaries. */
static void planckRgb(double kelvin, double* v) {
    static const double metres[3] = {611e-9, 549e-9, 464e-9};
    for (int c = 0; c < 3; ++c) {
        const double l = metres[c], l2 = l * l;
        v[c] = 1.0 / (l2 * l2 * l * (expBySquaring(.014388 / (l * kelvin)) - 1.0));
    }
}

/* A black body's colour on film balanced so that 6500 K is white, brightest channel 1. */
static void blackBodyRgb(double kelvin, float* rgb) {
    double v[3], white[3], most = 0;
    planckRgb(kelvin, v);
    planckRgb(6500.0, white);
    for (int c = 0; c < 3; ++c) {
        v[c] /= white[c];
        if (v[c] > most) most = v[c];
    }
    v[1] *= .6;
    v[2] *= .72;
    for (int c = 0; c < 3; ++c) rgb[c] = (float)(v[c] / most);
}

static void colourTable(float* map) { artfCudaHoleColours(map + ARTF_CUDA_COLORS_AT); }

void artfCudaHoleColours(float* colors) {
    for (int i = 0; i < ARTF_CUDA_COLORS; ++i) {
        /* (through float, as the reference's artfMaxf takes it) */
        const double kelvin = fmaxRef((float)(TABLE_KELVIN * (double)i / (ARTF_CUDA_COLORS / 2)), 400.f);
        blackBodyRgb(kelvin, colors + i * 3);
    }
}

/* ---- deterministic elementary functions (double, IEEE + - * / only) ------------------------------ */

#define LN2 0.6931471805599453

/* ln x for x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)), then 2 atanh((m - 1) / (m + 1)) by its series. */
static double detLog(double x) {
    int e = 0;
    while (x >= 1.4142135623730951) { x *= .5; ++e; }
    while (x < .7071067811865476) { x *= 2.0; --e; }
    const double s = (x - 1.0) / (x + 1.0), s2 = s * s;
    double term = s, sum = 0;
    for (int k = 0; k < 30; ++k) {
        sum += term / (double)(2 * k + 1);
        term *= s2;
    }
    return 2.0 * sum + (double)e * LN2;
}

/* e^x: x = k ln 2 + t with |t| <= ln2 / 2, e^t by its Taylor series, times 2^k by halving or doubling. */
static double detExp(double x) {
    const double kf = floor(x / LN2 + .5);
    const double t = x - kf * LN2;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k < 28; ++k) {
        term *= t / (double)k;
        sum += term;
    }
    int k = (int)kf;
    while (k > 0) { sum *= 2.0; --k; }
    while (k < 0) { sum *= .5; ++k; }
    return sum;
}

/* ---- the synthetic disc and sky -------------------------------------------------------------- */

/* splitmix64's finaliser: a well-mixed 64-bit value of a 64-bit key. */
static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* A uniform value in [0, 1) with 24 bits, from a stream (seed, kind) at index i. */
static double uniform24(uint64_t seed, uint64_t kind, uint64_t i) {
    const uint64_t h = mix64(mix64(seed * 0x100000001B3ull ^ kind) ^ i);
    return (double)(h >> 40) * (1.0 / 16777216.0);
}

#define LATTICE 64

static float smoothWeight(float t) { return t * t * (3.f - 2.f * t); }

/* The gas: value noise on a LATTICE x LATTICE grid over (azimuth, row), periodic in azimuth, each lattice
 * value uniform in [0.5, 1.5], read between lattice points with smoothstep weights. */
static void gasNoise(uint64_t seed, float* map) {
    float lattice[LATTICE][LATTICE];
    for (int j = 0; j < LATTICE; ++j)
        for (int i = 0; i < LATTICE; ++i) lattice[j][i] = (float)(.5 + uniform24(seed, 1, (uint64_t)(j * LATTICE + i)));
    for (int y = 0; y < ARTF_CUDA_MAP_HEIGHT; ++y) {
        const float v = (float)y * ((float)(LATTICE - 1) / (float)(ARTF_CUDA_MAP_HEIGHT - 1));
        int j0 = (int)v;
        if (j0 > LATTICE - 2) j0 = LATTICE - 2;
        const float ty = smoothWeight(v - (float)j0);
        for (int x = 0; x < ARTF_CUDA_MAP_WIDTH; ++x) {
            const float u = (float)x * ((float)LATTICE / (float)ARTF_CUDA_MAP_WIDTH);
            const int i0 = (int)u % LATTICE, i1 = (i0 + 1) % LATTICE;
            const float tx = smoothWeight(u - (float)(int)u);
            const float top = lattice[j0][i0] + (lattice[j0][i1] - lattice[j0][i0]) * tx;
            const float bottom = lattice[j0 + 1][i0] + (lattice[j0 + 1][i1] - lattice[j0 + 1][i0]) * tx;
            map[(size_t)y * ARTF_CUDA_MAP_WIDTH + x] = top + (bottom - top) * ty;
        }
    }
}

void artfCudaSynthRings(const ArtfCudaSynthDesc* s, float* map) {
    ringSpeedHeat(map, s->inner, s->outer, s->spin);
    float* glow = map + ARTF_CUDA_GLOW_AT;
    for (int y = 0; y < ARTF_CUDA_MAP_HEIGHT; ++y) {
        const float r = rowRadius((float)y / (float)(ARTF_CUDA_MAP_HEIGHT - 1), s->inner, s->outer);
        /* (r / inner)^-q */
        glow[y] = (float)detExp(-(double)s->emissivity * detLog((double)r / (double)s->inner));
    }
}

/* The sky: a floor of faint dust and a catalogue of point stars splatted between texels, so that the
 * trace's bilinear read of the sky map finds each star where it is. */
static void starSky(uint64_t seed, int stars, float* map) {
    float* sky = map + ARTF_CUDA_SKY_AT;
    for (int i = 0; i < ARTF_CUDA_SKY_WIDTH * ARTF_CUDA_SKY_HEIGHT; ++i) sky[i] = .0006f;
    for (int s = 0; s < stars; ++s) {
        const double height = 2.0 * uniform24(seed, 2, (uint64_t)s) - 1.0; /* uniform on the sphere */
        const double turn = uniform24(seed, 3, (uint64_t)s);
        const double brightness = detExp((-3.0 + 3.0 * uniform24(seed, 4, (uint64_t)s)) * 2.302585092994046);
        const float at = (float)turn * (float)ARTF_CUDA_SKY_WIDTH;
        const float rowAt = ((float)height * .5f + .5f) * (float)(ARTF_CUDA_SKY_HEIGHT - 1);
        const int c0 = (int)at & (ARTF_CUDA_SKY_WIDTH - 1), c1 = (c0 + 1) & (ARTF_CUDA_SKY_WIDTH - 1);
        int r0 = (int)rowAt;
        if (r0 > ARTF_CUDA_SKY_HEIGHT - 2) r0 = ARTF_CUDA_SKY_HEIGHT - 2;
        const float fx = at - (float)(int)at, fy = rowAt - (float)r0, b = (float)brightness;
        sky[r0 * ARTF_CUDA_SKY_WIDTH + c0] += b * (1.f - fx) * (1.f - fy);
        sky[r0 * ARTF_CUDA_SKY_WIDTH + c1] += b * fx * (1.f - fy);
        sky[(r0 + 1) * ARTF_CUDA_SKY_WIDTH + c0] += b * (1.f - fx) * fy;
        sky[(r0 + 1) * ARTF_CUDA_SKY_WIDTH + c1] += b * fx * fy;
    }
}

int artfCudaSynthMap(const ArtfCudaSynthDesc* s, float* map) {
    if (!s || !map || !(s->inner > 0) || !(s->outer > s->inner) || s->stars < 0) return ARTF_CUDA_EINVAL;
    memset(map, 0, sizeof(float) * ARTF_CUDA_MAP_FLOATS);
    gasNoise(s->seed, map);
    artfCudaSynthRings(s, map);
    colourTable(map);
    starSky(s->seed, s->stars, map);
    /* dust: none (the memset) */
    return ARTF_CUDA_OK;
}
