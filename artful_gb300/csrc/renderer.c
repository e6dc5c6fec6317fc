/* artful_cuda — the GB300 hole tracer as an Artful renderer backend (C11), and the library's own
 * minimal hole scene.  The backend fills the eight-entry table every Artful renderer has
 * (src/render/rendererInternal.h:7-27) and draws through the C ABI: the trace, its bloom and tone
 * map on the GPU, and the frame read back for readPixels.  Its rules are the reference's:
 *   - draw returns false when the device is lost; the renderer must then be freed, and the scene
 *     survives for a new one (include/artful/renderer.h:107-109);
 *   - failures are reported once (artfCudaLastError) and never abort (include/artful/core.h:56-57);
 *   - an overlay's pixels are read in setOverlay or the next draw (include/artful/renderer.h:91-105);
 *   - a scene without a hole draws black, as the hole is all this backend draws. */
#define _POSIX_C_SOURCE 200809L /* clock_gettime */
#include "artful_cuda_renderer.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---- the scene ---------------------------------------------------------------------------------- */

struct ArtfCudaScene {
    uint64_t id;
    ArtfCudaCamera camera;
    bool on;
    ArtfCudaBlackHoleDesc desc; /* clamped */
    float* map;
    uint64_t mapVersion;
    float* fluid;
    uint64_t fluidVersion;
    double fluidTime;
    bool ownMap;                /* the caller's map, not the synthetic one */
    uint64_t seed;
    float emissivity;
    uint32_t gasGeneration;     /* the gas's clock, kept as artfSceneSetBlackHole keeps its fluid's */
    double gasStart, gasClock;
    uint64_t gasSteps;
};

static uint64_t nextSceneId = 1;

ArtfCudaScene* artfCudaSceneNew(void) {
    ArtfCudaScene* s = (ArtfCudaScene*)calloc(1, sizeof(ArtfCudaScene));
    if (!s) return NULL;
    s->id = nextSceneId++;
    s->camera.position.z = 30.f;
    s->camera.up.y = 1.f;
    s->camera.fovY = .9f;
    s->camera.near_ = .1f;
    s->emissivity = 3.f;
    return s;
}

void artfCudaSceneFree(ArtfCudaScene* s) {
    if (!s) return;
    free(s->map);
    free(s->fluid);
    free(s);
}

void artfCudaSceneSetCamera(ArtfCudaScene* s, const ArtfCudaCamera* camera) {
    if (s && camera) s->camera = *camera;
}

void artfCudaSceneSetSeed(ArtfCudaScene* s, uint64_t seed, float emissivity) {
    if (!s) return;
    s->seed = seed;
    s->emissivity = emissivity;
    if (s->on && !s->ownMap && s->map) {
        const ArtfCudaSynthDesc synth = {s->seed, s->desc.discInner, s->desc.discOuter, s->desc.spin, s->emissivity, 2000};
        artfCudaSynthMap(&synth, s->map);
        ++s->mapVersion;
    }
}

void artfCudaSceneSetBlackHole(ArtfCudaScene* s, const ArtfCudaBlackHoleDesc* desc) {
    if (!s) return;
    if (!desc) {
        s->on = false;
        return;
    }
    ArtfCudaBlackHoleDesc d;
    artfCudaHoleClamp(desc, &d);
    const bool sameDisc = s->map && s->desc.discInner == d.discInner && s->desc.discOuter == d.discOuter;
    const bool sameSpin = sameDisc && s->desc.spin == d.spin;
    s->on = true;
    s->desc = d;
    s->fluidTime = d.time;
    if (!s->map) s->map = (float*)malloc(sizeof(float) * ARTF_CUDA_MAP_FLOATS);
    if (!s->fluid) {
        s->fluid = (float*)malloc(sizeof(float) * ARTF_CUDA_FLUID_FLOATS);
        if (s->fluid)
            for (size_t i = 0; i < ARTF_CUDA_FLUID_FLOATS; ++i) s->fluid[i] = 1.f;
        ++s->fluidVersion;
    }
    if (!s->map || !s->fluid) {
        s->on = false; /* (out of host memory: the scene keeps no hole) */
        return;
    }
    if (!sameSpin && !s->ownMap) {
        const ArtfCudaSynthDesc synth = {s->seed, d.discInner, d.discOuter, d.spin, s->emissivity, 2000};
        artfCudaSynthMap(&synth, s->map);
        ++s->mapVersion;
    }
    /* hole.c:264-270: a new gas for a new disc or spin, else the old one advanced to the time */
    if (!sameSpin) {
        ++s->gasGeneration;
        s->gasStart = s->gasClock = d.time;
        s->gasSteps = 0;
    } else {
        s->gasSteps += (uint64_t)artfCudaFluidClock(&s->gasClock, d.time);
    }
}

void artfCudaSceneSetHoleMap(ArtfCudaScene* s, const float* map, const float* fluid, double fluidTime) {
    if (!s || !map || !fluid) return;
    if (!s->map) s->map = (float*)malloc(sizeof(float) * ARTF_CUDA_MAP_FLOATS);
    if (!s->fluid) s->fluid = (float*)malloc(sizeof(float) * ARTF_CUDA_FLUID_FLOATS);
    if (!s->map || !s->fluid) return;
    memcpy(s->map, map, sizeof(float) * ARTF_CUDA_MAP_FLOATS);
    memcpy(s->fluid, fluid, sizeof(float) * ARTF_CUDA_FLUID_FLOATS);
    s->ownMap = true;
    s->fluidTime = fluidTime;
    ++s->mapVersion;
    ++s->fluidVersion;
}

bool artfCudaSceneReadHole(const void* scene, ArtfCudaHoleInputs* out) {
    const ArtfCudaScene* s = (const ArtfCudaScene*)scene;
    if (!s || !out) return false;
    memset(out, 0, sizeof *out);
    out->on = s->on && s->map && s->fluid;
    out->camera = s->camera;
    out->desc = s->desc;
    out->map = s->map;
    out->mapVersion = s->id << 32 | (s->mapVersion & 0xFFFFFFFFu);
    out->fluid = s->fluid;
    out->fluidVersion = s->id << 32 | (s->fluidVersion & 0xFFFFFFFFu);
    out->fluidTime = s->fluidTime;
    out->gasGeneration = s->id << 32 | s->gasGeneration;
    out->gasStart = s->gasStart;
    out->gasSteps = s->gasSteps;
    out->gasClock = s->gasClock;
    return true;
}

/* ---- the renderer -------------------------------------------------------------------------------- */

typedef struct CudaRenderer {
    ArtfCudaRenderer base;
    ArtfCuda* ctx;
    ArtfCudaSceneReader reader;
    int width, height;
    int precision;
    uint32_t* bgra;
    float* light;
    bool bgraOnDevice;          /* the last frame's BGRA is the context's (read back at readPixels), not bgra */
    bool lightOnDevice;         /* the last frame's light is the context's, not light */
    uint32_t* overlay;          /* a copy of the last overlay, width * height, or NULL */
    int overlayWidth, overlayHeight;
    char description[160];
    ArtfCudaFrameStats stats;
    bool deviceInputs;
    bool painted;               /* the context's map is the painted disc of paintedDisc (inner, outer, spin) */
    float paintedDisc[3];
    ArtfCudaFluid* gas;         /* the scene's gas, on the device */
    bool gasShown;              /* the context's fluid is the gas's field */
    uint64_t gasGeneration, gasSteps;
} CudaRenderer;

static double nowMs(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec * 1e3 + (double)t.tv_nsec * 1e-6;
}

static const char* cudaDescription(const ArtfCudaRenderer* r) { return ((const CudaRenderer*)r)->description; }

static bool allocFrame(CudaRenderer* c, int width, int height) {
    const size_t pixels = (size_t)(width > 0 ? width : 1) * (size_t)(height > 0 ? height : 1);
    uint32_t* bgra = (uint32_t*)calloc(pixels, sizeof(uint32_t));
    float* light = (float*)calloc(pixels * 4, sizeof(float));
    if (!bgra || !light) {
        free(bgra);
        free(light);
        return false;
    }
    free(c->bgra);
    free(c->light);
    c->bgra = bgra;
    c->light = light;
    c->bgraOnDevice = c->lightOnDevice = false;
    c->width = width > 0 ? width : 1;
    c->height = height > 0 ? height : 1;
    return true;
}

static void cudaResize(ArtfCudaRenderer* r, int width, int height) {
    CudaRenderer* c = (CudaRenderer*)r;
    if (width != c->width || height != c->height) allocFrame(c, width, height);
}

static void cudaSetOverlay(ArtfCudaRenderer* r, const ArtfCudaOverlay* o) {
    CudaRenderer* c = (CudaRenderer*)r;
    free(c->overlay);
    c->overlay = NULL;
    if (!o || !o->pixels || o->width < 1 || o->height < 1) return;
    const int stride = o->stride ? o->stride : o->width;
    c->overlay = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)o->width * (size_t)o->height);
    if (!c->overlay) return;
    for (int y = 0; y < o->height; ++y)
        memcpy(c->overlay + (size_t)y * o->width, o->pixels + (size_t)y * stride, sizeof(uint32_t) * (size_t)o->width);
    c->overlayWidth = o->width;
    c->overlayHeight = o->height;
}

/* byte * rest / 255, rounded (the software backend's timesRest) */
static uint32_t timesRest(uint32_t byte, uint32_t rest) {
    const uint32_t t = byte * rest + 128u;
    return (t + (t >> 8)) >> 8;
}

/* The overlay, premultiplied, over the frame. */
static void composite(CudaRenderer* c) {
    if (!c->overlay) return;
    const int w = c->overlayWidth < c->width ? c->overlayWidth : c->width;
    const int h = c->overlayHeight < c->height ? c->overlayHeight : c->height;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const uint32_t o = c->overlay[(size_t)y * c->overlayWidth + x];
            uint32_t* p = c->bgra + (size_t)y * c->width + x;
            const uint32_t rest = 255u - (o >> 24);
            uint32_t out = 0;
            for (int s = 0; s < 32; s += 8) {
                const uint32_t v = (o >> s & 255u) + timesRest(*p >> s & 255u, rest);
                out |= (v > 255u ? 255u : v) << s;
            }
            *p = out;
        }
}

/* The scene's painted map and gas made on the device, as hole.c:249-270 makes them on the host: the map
 * painted again when the disc or the spin changes; the gas started afresh when the scene's starts
 * afresh, else stepped as many steps as the scene's clock has counted since the last draw.  A reader
 * that knows no clock (gasGeneration 0) gets the reference's rule applied at each draw instead.  Returns
 * an ArtfCuda status; *fluidTime: the gas's time. */
static int deviceInputs(CudaRenderer* c, const ArtfCudaHoleInputs* in, double* fluidTime) {
    const ArtfCudaBlackHoleDesc* d = &in->desc;
    const bool sameDisc = c->painted && c->paintedDisc[0] == d->discInner && c->paintedDisc[1] == d->discOuter;
    const bool sameSpin = sameDisc && c->paintedDisc[2] == d->spin;
    int status;
    if (!sameSpin) {
        c->painted = false;
        if ((status = artfCudaPaintDisc(c->ctx, NULL, d->discInner, d->discOuter, d->spin))) return status;
        c->paintedDisc[0] = d->discInner, c->paintedDisc[1] = d->discOuter, c->paintedDisc[2] = d->spin;
        c->painted = true;
    }
    const bool known = in->gasGeneration != 0;
    const bool restart = !c->gas || (known ? in->gasGeneration != c->gasGeneration || in->gasSteps < c->gasSteps
                                           : !sameSpin);
    bool changed = restart || !c->gasShown;
    if (restart) {
        artfCudaFluidFree(c->gas);
        c->gas = NULL;
        if ((status = artfCudaFluidNew(c->ctx, d->discInner, d->discOuter, d->spin, known ? in->gasStart : d->time,
                                       &c->gas)))
            return status;
        c->gasGeneration = in->gasGeneration;
        c->gasSteps = 0;
    }
    if (known) {
        const uint64_t steps = in->gasSteps - c->gasSteps;
        if ((status = artfCudaFluidStep(c->gas, (int64_t)steps, in->gasClock))) return status;
        c->gasSteps = in->gasSteps;
        changed = changed || steps > 0;
    } else if (!restart) {
        int stepped = 0;
        if ((status = artfCudaFluidAdvance(c->gas, d->time, &stepped))) return status;
        changed = changed || stepped;
    }
    c->gasShown = false;
    if (changed && (status = artfCudaUseFluid(c->ctx, c->gas))) return status;
    c->gasShown = true;
    *fluidTime = artfCudaFluidTime(c->gas);
    return ARTF_CUDA_OK;
}

static bool cudaDraw(ArtfCudaRenderer* r, void* scene) {
    CudaRenderer* c = (CudaRenderer*)r;
    const double t0 = nowMs();
    ArtfCudaHoleInputs in;
    memset(&c->stats, 0, sizeof c->stats);
    if (!c->reader(scene, &in) || !in.on) {
        c->bgraOnDevice = c->lightOnDevice = false;
        for (size_t i = 0; i < (size_t)c->width * c->height; ++i) c->bgra[i] = 0xFF000000u;
        memset(c->light, 0, sizeof(float) * 4 * (size_t)c->width * c->height);
        composite(c);
        c->stats.cpuMs = nowMs() - t0;
        return true;
    }
    double fluidTime = in.fluidTime;
    if (c->deviceInputs) {
        if (deviceInputs(c, &in, &fluidTime)) return false;
    } else {
        c->painted = c->gasShown = false; /* (the context's map and fluid are the host's from here on) */
    }
    ArtfCudaHoleFrame frame;
    ArtfCudaHoleFrame64 frame64;
    if (!artfCudaHoleFrame(&in.camera, &in.desc, fluidTime, c->width, c->height, &frame) ||
        artfCudaHoleFrame64(&in.camera, &in.desc, fluidTime, c->width, c->height, &frame64))
        return true; /* (nothing to draw at this size; the device is fine) */
    ArtfCudaTraceOptions options;
    memset(&options, 0, sizeof options);
    options.precision = c->precision;
    options.stepScale = 1.f;
    options.persistent = 1;
    ArtfCudaTraceStats stats;
    /* The frame stays on the device until readPixels (or the light until artfCudaRendererReadLight) asks
     * for it; with an overlay the BGRA comes back now, to be composited as drawn. */
    uint32_t* bgraNow = c->overlay ? c->bgra : NULL;
    c->bgraOnDevice = c->lightOnDevice = false;
    const int status = c->deviceInputs
                           ? artfCudaHoleDraw(c->ctx, &frame, &frame64, NULL, 0, NULL, 0, &options, NULL, bgraNow,
                                              &stats)
                           : artfCudaHoleDraw(c->ctx, &frame, &frame64, in.map, in.mapVersion, in.fluid,
                                              in.fluidVersion, &options, NULL, bgraNow, &stats);
    if (status) return false; /* the device is lost (or unusable): the renderer must be freed */
    c->bgraOnDevice = bgraNow == NULL;
    c->lightOnDevice = true;
    composite(c);
    c->stats.lensMs = stats.ms;
    c->stats.gpuMs = stats.ms;
    c->stats.traceSamples = frame.size[2] * frame.size[2];
    c->stats.cpuMs = nowMs() - t0;
    return true;
}

static bool cudaReadPixels(ArtfCudaRenderer* r, uint32_t* dst) {
    CudaRenderer* c = (CudaRenderer*)r;
    if (!dst) return false;
    if (c->bgraOnDevice) return artfCudaFrameRead(c->ctx, NULL, dst) == ARTF_CUDA_OK;
    memcpy(dst, c->bgra, sizeof(uint32_t) * (size_t)c->width * c->height);
    return true;
}

static uint32_t* cudaPixels(ArtfCudaRenderer* r) {
    (void)r;
    return NULL; /* (a GPU backend's frame is not in host memory between calls) */
}

static void cudaStats(const ArtfCudaRenderer* r, ArtfCudaFrameStats* out) {
    if (out) *out = ((const CudaRenderer*)r)->stats;
}

static void cudaDestroy(ArtfCudaRenderer* r) {
    CudaRenderer* c = (CudaRenderer*)r;
    artfCudaFluidFree(c->gas);
    artfCudaDestroy(c->ctx);
    free(c->bgra);
    free(c->light);
    free(c->overlay);
    free(c);
}

static const ArtfCudaRendererVtbl cudaTable = {cudaDescription, cudaResize, cudaSetOverlay, cudaDraw,
                                               cudaReadPixels, cudaPixels, cudaStats, cudaDestroy};

ArtfCudaRenderer* artfCudaNewWithReader(const ArtfCudaRendererOptions* options, ArtfCudaSceneReader reader) {
    if (!options || !reader) return NULL;
    CudaRenderer* c = (CudaRenderer*)calloc(1, sizeof(CudaRenderer));
    if (!c) return NULL;
    c->base.vt = &cudaTable;
    c->base.backend = ARTF_CUDA_BACKEND;
    c->reader = reader;
    c->precision = ARTF_CUDA_EXACT;
    if (artfCudaCreate(0, &c->ctx) || !allocFrame(c, options->width, options->height)) {
        artfCudaDestroy(c->ctx);
        free(c->bgra);
        free(c->light);
        free(c);
        return NULL;
    }
    snprintf(c->description, sizeof c->description, "CUDA, GB300 (sm_103a), Kerr hole tracer");
    return &c->base;
}

ArtfCudaRenderer* artfCudaNew(const ArtfCudaRendererOptions* options) {
    return artfCudaNewWithReader(options, artfCudaSceneReadHole);
}

bool artfCudaRendererReadLight(ArtfCudaRenderer* r, float* dst) {
    CudaRenderer* c = (CudaRenderer*)r;
    if (!c || !dst) return false;
    if (c->lightOnDevice) return artfCudaFrameRead(c->ctx, dst, NULL) == ARTF_CUDA_OK;
    memcpy(dst, c->light, sizeof(float) * 4 * (size_t)c->width * c->height);
    return true;
}

void artfCudaRendererSetPrecision(ArtfCudaRenderer* r, int precision) {
    if (r && precision >= ARTF_CUDA_EXACT && precision <= ARTF_CUDA_MIXED) ((CudaRenderer*)r)->precision = precision;
}

ArtfCuda* artfCudaRendererContext(ArtfCudaRenderer* r) { return r ? ((CudaRenderer*)r)->ctx : NULL; }

void artfCudaRendererSetDeviceInputs(ArtfCudaRenderer* r, bool on) {
    if (r) ((CudaRenderer*)r)->deviceInputs = on;
}
