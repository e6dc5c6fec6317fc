/* The oracle's entry points: the per-ray trace of lensOracleBody.h in float and in double, and the
 * reference's tile loop (src/software/lens.inc:355-383) over whole frames on host threads.
 * Test infrastructure: see oracle.h. */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* lens.inc:56-61 lensHash: a hash of a lattice cube, for the stars. */
static uint32_t oracleCubeHash(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = x * 73856093u ^ y * 19349663u ^ z * 83492791u;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

#define REAL float
#define FRAME OracleFrame
#define SFX 32
#define SQRT sqrtf
#define FLOOR floorf
#define FABS fabsf
#include "lensOracleBody.h"
#undef REAL
#undef FRAME
#undef SFX
#undef SQRT
#undef FLOOR
#undef FABS

#define REAL double
#define FRAME OracleFrame64
#define SFX 64
#define SQRT sqrt
#define FLOOR floor
#define FABS fabs
#include "lensOracleBody.h"

/* A 32-bit integer mixer (two multiply-xorshift rounds). */
static uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

void oracleJitter(uint32_t seed, uint32_t pixel, uint32_t k, float* dx, float* dy) {
    const uint32_t base = mix32(mix32(seed ^ 0xA511E9B3u) ^ pixel);
    *dx = (float)(mix32(base + 2u * k) >> 8) * (1.f / 16777216.f);
    *dy = (float)(mix32(base + 2u * k + 1u) >> 8) * (1.f / 16777216.f);
}

void oracleTrace32(const OracleFrame* h, const float* map, const float* fluid, const OracleOptions* o, int n,
                   const float* nx, const float* ny, const float* time, float* rgb, OracleEnd* ends) {
    const float scale = o && o->stepScale > 0 ? o->stepScale : 1.f;
    for (int i = 0; i < n; ++i) traceRay32(h, map, fluid, scale, nx[i], ny[i], time[i], rgb + 3 * i, ends ? ends + i : 0);
}

void oracleTrace64(const OracleFrame64* h, const float* map, const float* fluid, const OracleOptions* o, int n,
                   const double* nx, const double* ny, const double* time, double* rgb, OracleEnd* ends) {
    const double scale = o && o->stepScale > 0 ? o->stepScale : 1.0;
    for (int i = 0; i < n; ++i) traceRay64(h, map, fluid, scale, nx[i], ny[i], time[i], rgb + 3 * i, ends ? ends + i : 0);
}

/* ---- whole frames ------------------------------------------------------------------------------- */

typedef struct RenderJob {
    const OracleFrame* h32;
    const OracleFrame64* h64; /* NULL: the FP32 trace */
    const float* map;
    const float* fluid;
    float stepScale;
    int jitter;
    uint32_t seed;
    int y0, y1;
    float* hdr32;
    double* hdr64;
    OracleEnd* ends;
    int next; /* the next row to take */
    pthread_mutex_t lock;
} RenderJob;

/* The sample positions of one pixel's rays, as lens.inc:365-371 makes them for stratified sampling
 * (the eight-lane group's base column, then the lane, in float), or from oracleJitter. */
static void samplePosition(const OracleFrame* h, int jitter, uint32_t seed, int x, int y, int k, float* nx, float* ny,
                           float* moment) {
    const int side = (int)h->size[2];
    if (!jitter) {
        const int sy = k / side, sx = k % side;
        const float dx = ((float)sx + .5f) / (float)side, dy = ((float)sy + .5f) / (float)side;
        const int group = x & ~7, lane = x & 7;
        *nx = ((float)lane + ((float)group + dx)) * h->image[1] - 1.f;
        *ny = 1.f - ((float)y + dy) * h->image[2];
        *moment = ((float)((sy * side + sx) * 5 % (side * side)) + .5f) * h->image[3] - .5f;
    } else {
        float dx, dy;
        oracleJitter(seed, (uint32_t)y * h->size[0] + (uint32_t)x, (uint32_t)k, &dx, &dy);
        *nx = ((float)x + dx) * h->image[1] - 1.f;
        *ny = 1.f - ((float)y + dy) * h->image[2];
        *moment = ((float)(k * 5 % jitter) + .5f) / (float)jitter - .5f;
    }
}

static uint32_t classBits(uint8_t kind) {
    uint32_t bits = kind & ORACLE_LIT ? 1u : 0u;
    if ((kind & 15) == ORACLE_SKY) bits |= 2u;
    else if (!(kind & ORACLE_LIT)) bits |= 4u;
    return bits;
}

static void renderRow(RenderJob* j, int y) {
    const OracleFrame* h = j->h32;
    const int width = (int)h->size[0];
    const int rays = j->jitter ? j->jitter : (int)(h->size[2] * h->size[2]);
    for (int x = 0; x < width; ++x) {
        const size_t pixel = (size_t)y * width + x;
        float sum32[3] = {0, 0, 0};
        double sum64[3] = {0, 0, 0};
        uint32_t bits = 0;
        for (int k = 0; k < rays; ++k) {
            float nx, ny, moment;
            samplePosition(h, j->jitter, j->seed, x, y, k, &nx, &ny, &moment);
            OracleEnd end;
            OracleEnd* e = j->ends ? j->ends + pixel * rays + k : &end;
            if (!j->h64) {
                float rgb[3];
                const float time = h->disc[2] + h->spin[3] * moment;
                traceRay32(h, j->map, j->fluid, j->stepScale, nx, ny, time, rgb, e);
                for (int c = 0; c < 3; ++c) sum32[c] = sum32[c] + rgb[c];
            } else {
                double rgb[3];
                const double time = j->h64->disc[2] + j->h64->spin[3] * (double)moment;
                traceRay64(j->h64, j->map, j->fluid, (double)j->stepScale, (double)nx, (double)ny, time, rgb, e);
                for (int c = 0; c < 3; ++c) sum64[c] = sum64[c] + rgb[c];
            }
            bits |= classBits(e->kind);
        }
        if (!j->h64) {
            const float share = j->jitter ? 1.f / (float)j->jitter : h->image[3];
            for (int c = 0; c < 3; ++c) j->hdr32[pixel * 4 + c] = sum32[c] * share;
            j->hdr32[pixel * 4 + 3] = (float)bits;
        } else {
            const double share = 1.0 / (double)rays;
            for (int c = 0; c < 3; ++c) j->hdr64[pixel * 4 + c] = sum64[c] * share;
            j->hdr64[pixel * 4 + 3] = (double)bits;
        }
    }
}

static void* renderWorker(void* user) {
    RenderJob* j = user;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        const int y = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (y >= j->y1) return 0;
        renderRow(j, y);
    }
}

static void renderAll(RenderJob* j, int threads) {
    if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    j->next = j->y0;
    pthread_mutex_init(&j->lock, 0);
    pthread_t ids[256];
    int started = 0;
    for (int t = 1; t < threads; ++t)
        if (!pthread_create(&ids[started], 0, renderWorker, j)) ++started;
    renderWorker(j);
    for (int t = 0; t < started; ++t) pthread_join(ids[t], 0);
    pthread_mutex_destroy(&j->lock);
}

void oracleRender32(const OracleFrame* h, const float* map, const float* fluid, const OracleOptions* o, int jitter,
                    uint32_t seed, int threads, int y0, int y1, float* hdr, OracleEnd* ends) {
    RenderJob j;
    memset(&j, 0, sizeof j);
    j.h32 = h, j.map = map, j.fluid = fluid, j.stepScale = o && o->stepScale > 0 ? o->stepScale : 1.f;
    j.jitter = jitter, j.seed = seed, j.y0 = y0, j.y1 = y1, j.hdr32 = hdr, j.ends = ends;
    renderAll(&j, threads);
}

void oracleRender64(const OracleFrame* h32, const OracleFrame64* h, const float* map, const float* fluid,
                    const OracleOptions* o, int jitter, uint32_t seed, int threads, int y0, int y1, double* hdr,
                    OracleEnd* ends) {
    RenderJob j;
    memset(&j, 0, sizeof j);
    j.h32 = h32, j.h64 = h, j.map = map, j.fluid = fluid, j.stepScale = o && o->stepScale > 0 ? o->stepScale : 1.f;
    j.jitter = jitter, j.seed = seed, j.y0 = y0, j.y1 = y1, j.hdr64 = hdr, j.ends = ends;
    renderAll(&j, threads);
}

int oracleThreads(void) { return (int)sysconf(_SC_NPROCESSORS_ONLN); }
