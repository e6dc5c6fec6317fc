/* The renderer backend's host logic (renderer.c: the scene API, device inputs and the gas clock, the
 * frame kept on the device until read, the overlay, resizes, a hole removed) driven through its table over
 * a fake device, built by tests/test_host_sanitized.py with AddressSanitizer and UndefinedBehaviorSanitizer.
 * The fake "draws" a frame whose every pixel encodes its own index, so the read-back paths can be checked. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "artful_cuda.h"
#include "artful_cuda_renderer.h"

/* ---- the fake device ------------------------------------------------------------------------------- */

struct ArtfCuda { size_t drawn; int draws; };
struct ArtfCudaFluid { double time; };

static uint32_t pixelOf(size_t i) { return 0xFF000000u | (uint32_t)(i * 2654435761u & 0xFFFFFFu); }

static void fill(size_t n, float* hdr, uint32_t* bgra) {
    for (size_t i = 0; i < n; ++i) {
        if (hdr) hdr[4 * i] = (float)i, hdr[4 * i + 1] = hdr[4 * i + 2] = 0.5f, hdr[4 * i + 3] = 1.f;
        if (bgra) bgra[i] = pixelOf(i);
    }
}

int artfCudaCreate(int device, ArtfCuda** out) {
    (void)device;
    *out = (ArtfCuda*)calloc(1, sizeof(ArtfCuda));
    return *out ? 0 : -3;
}
void artfCudaDestroy(ArtfCuda* ctx) { free(ctx); }
int artfCudaHoleDraw(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                     const float* hostMap, uint64_t mapVersion, const float* hostFluid, uint64_t fluidVersion,
                     const ArtfCudaTraceOptions* options, float* hostHdr, uint32_t* hostBgra,
                     ArtfCudaTraceStats* stats) {
    (void)frame64, (void)mapVersion, (void)fluidVersion, (void)options;
    if (hostMap) { volatile float touch = hostMap[ARTF_CUDA_MAP_FLOATS - 1]; (void)touch; }
    if (hostFluid) { volatile float touch = hostFluid[ARTF_CUDA_FLUID_FLOATS - 1]; (void)touch; }
    ctx->drawn = (size_t)frame->size[0] * frame->size[1];
    ++ctx->draws;
    fill(ctx->drawn, hostHdr, hostBgra);
    if (stats) { memset(stats, 0, sizeof *stats); stats->ms = 1.f; }
    return 0;
}
int artfCudaFrameRead(ArtfCuda* ctx, float* hostHdr, uint32_t* hostBgra) {
    if (!ctx->drawn) return -1;
    fill(ctx->drawn, hostHdr, hostBgra);
    return 0;
}
int artfCudaPaintDisc(ArtfCuda* ctx, float* map, float inner, float outer, float spin) {
    (void)ctx, (void)map, (void)inner, (void)outer, (void)spin;
    return 0;
}
int artfCudaFluidNew(ArtfCuda* ctx, float inner, float outer, float spin, double time, ArtfCudaFluid** out) {
    (void)ctx, (void)inner, (void)outer, (void)spin;
    *out = (ArtfCudaFluid*)calloc(1, sizeof(ArtfCudaFluid));
    if (!*out) return -3;
    (*out)->time = time;
    return 0;
}
int artfCudaFluidAdvance(ArtfCudaFluid* f, double time, int* stepped) {
    *stepped = 0;
    f->time = time;
    return 0;
}
int artfCudaFluidStep(ArtfCudaFluid* f, int64_t steps, double time) {
    (void)steps;
    f->time = time;
    return 0;
}
int artfCudaUseFluid(ArtfCuda* ctx, const ArtfCudaFluid* f) { (void)ctx, (void)f; return 0; }
double artfCudaFluidTime(const ArtfCudaFluid* f) { return f->time; }
void artfCudaFluidFree(ArtfCudaFluid* f) { free(f); }

/* ---- the driver ------------------------------------------------------------------------------------ */

static int fails;
#define EXPECT(c) do { if (!(c)) { fprintf(stderr, "expected %s (line %d)\n", #c, __LINE__); ++fails; } } while (0)

static bool frameIsPattern(const uint32_t* got, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (got[i] != pixelOf(i)) return false;
    return true;
}

int main(void) {
    ArtfCudaRendererOptions o;
    memset(&o, 0, sizeof o);
    o.backend = ARTF_CUDA_BACKEND;
    o.width = 37, o.height = 21;
    ArtfCudaRenderer* r = artfCudaNew(&o);
    EXPECT(r != NULL);
    if (!r) return 1;
    const ArtfCudaRendererVtbl* vt = r->vt;
    ArtfCudaScene* s = artfCudaSceneNew();
    ArtfCudaCamera cam;
    memset(&cam, 0, sizeof cam);
    cam.position.y = 5.f, cam.position.z = 29.f, cam.up.y = 1.f, cam.fovY = .6f, cam.near_ = .1f;
    artfCudaSceneSetCamera(s, &cam);
    artfCudaSceneSetSeed(s, 4, 3.f);
    ArtfCudaBlackHoleDesc d = artfCudaBlackHoleDefaults();
    d.axis.y = 1.f, d.spin = .9f, d.discOuter = 12.f, d.bloom = 4.5f;
    artfCudaSceneSetBlackHole(s, &d);

    size_t n = 37 * 21;
    uint32_t* bgra = (uint32_t*)calloc(n, sizeof(uint32_t));
    float* light = (float*)calloc(n * 4, sizeof(float));
    /* host inputs: drawn, the frame read back at readPixels, the light when asked */
    EXPECT(vt->draw(r, s));
    EXPECT(vt->readPixels(r, bgra) && frameIsPattern(bgra, n));
    EXPECT(artfCudaRendererReadLight(r, light) && light[4 * (n - 1)] == (float)(n - 1));
    EXPECT(vt->pixels(r) == NULL);
    ArtfCudaFrameStats st;
    vt->stats(r, &st);
    EXPECT(st.lensMs == 1.0);
    /* an overlay: composited as drawn, over the frame */
    uint32_t over[6 * 4];
    for (int i = 0; i < 24; ++i) over[i] = 0xFF00FF00u;
    ArtfCudaOverlay ov;
    memset(&ov, 0, sizeof ov);
    ov.pixels = over, ov.width = 6, ov.height = 4;
    vt->setOverlay(r, &ov);
    EXPECT(vt->draw(r, s));
    EXPECT(vt->readPixels(r, bgra) && bgra[0] == 0xFF00FF00u && bgra[37 * 5] == pixelOf(37 * 5));
    vt->setOverlay(r, NULL);
    /* device inputs, the hole's clock moving; resizes to the reference's odd sizes and back */
    artfCudaRendererSetDeviceInputs(r, true);
    const int sizes[][2] = {{160, 90}, {101, 67}, {3, 2}, {1, 1}, {37, 21}};
    for (int k = 0; k < 5; ++k) {
        d.time = 0.2f * (float)(k + 1);
        artfCudaSceneSetBlackHole(s, &d);
        vt->resize(r, sizes[k][0], sizes[k][1]);
        const size_t m = (size_t)sizes[k][0] * (size_t)sizes[k][1];
        uint32_t* frame = (uint32_t*)calloc(m, sizeof(uint32_t));
        EXPECT(vt->readPixels(r, frame)); /* (after a resize and before a draw: the new frame, empty) */
        EXPECT(vt->draw(r, s));
        EXPECT(vt->readPixels(r, frame) && frameIsPattern(frame, m));
        free(frame);
    }
    /* a caller's own map and fluid, then the hole removed: black */
    float* map = (float*)calloc(ARTF_CUDA_MAP_FLOATS, sizeof(float));
    float* fluid = (float*)calloc(ARTF_CUDA_FLUID_FLOATS, sizeof(float));
    artfCudaRendererSetDeviceInputs(r, false);
    artfCudaSceneSetHoleMap(s, map, fluid, 1.0);
    EXPECT(vt->draw(r, s));
    artfCudaSceneSetBlackHole(s, NULL);
    EXPECT(vt->draw(r, s));
    EXPECT(vt->readPixels(r, bgra) && bgra[0] == 0xFF000000u && bgra[n - 1] == 0xFF000000u);
    EXPECT(artfCudaRendererReadLight(r, light) && light[0] == 0.f);
    free(map);
    free(fluid);
    free(bgra);
    free(light);
    vt->destroy(r);
    artfCudaSceneFree(s);
    printf("renderer checks failed: %d\n", fails);
    return fails ? 1 : 0;
}
