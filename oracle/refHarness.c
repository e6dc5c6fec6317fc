/* Test-only harness around the reference renderer, built from the reference's own sources by
 * oracle/ref.mk into oracle/_ref/libartref.so.  It pins the oracle: the oracle restatement
 * (oracle/lensOracle.c) and the golden fixtures under tests/golden/ are pinned against what these
 * entry points return.  Nothing in the product links or loads it.
 *
 * It compiles the reference's tile kernels (src/software/kernels.inc, which includes
 * src/software/lens.inc) into this translation unit, so that the reference's static per-ray trace
 * (lens.inc:99 lensTrace) can be called with arbitrary sub-pixel positions, as the jittered
 * configurations need, and not only through the stratified tile loop (lens.inc:355 lensTile). */
#define KERNELS refHarnessKernels
#define KERNELS_NAME "harness"
#include "software/kernels.inc"

#include "core/threads.h"
#include "render/rendererInternal.h"

#include <string.h>
#include <time.h>

/* A hole and the camera that looks at it, as the reference's public API takes them. */
typedef struct RefView {
    ArtfCamera camera;
    ArtfBlackHoleDesc desc;
    int width, height;
} RefView;

static ArtfScene* scene;

static ArtfScene* sceneFor(const RefView* v) {
    if (!scene) scene = artfSceneNew();
    artfSceneSetCamera(scene, &v->camera);
    artfSceneSetBlackHole(scene, &v->desc);
    return scene;
}

/* The frame block the reference fills for this view (hole.c:273 artfHoleFrame), and the description as
 * artfSceneSetBlackHole clamped it (hole.c:242). Returns the bloom pixel count. */
uint32_t refFrame(const RefView* v, ArtfHoleFrame* out, ArtfBlackHoleDesc* clamped) {
    ArtfScene* s = sceneFor(v);
    uint32_t bloomPixels = 0;
    artfHoleFrame(s, v->width, v->height, out, &bloomPixels);
    if (clamped) *clamped = s->hole.desc;
    return bloomPixels;
}

/* The reference's own painted map (hole.c:136 buildDisc + hole.c:186 setRings) for this view's disc. */
void refMap(const RefView* v, float* out) {
    ArtfScene* s = sceneFor(v);
    memcpy(out, s->hole.map, sizeof(float) * ARTF_HOLE_MAP_FLOATS);
}

/* The reference's fluid field for this view (fluid.c:335), and the moment it is of. */
double refFluid(const RefView* v, float* out) {
    ArtfScene* s = sceneFor(v);
    memcpy(out, artfFluidField(s->hole.fluid), sizeof(float) * ARTF_FLUID_WIDTH * ARTF_FLUID_HEIGHT);
    return artfFluidTime(s->hole.fluid);
}

/* The reference's disc fluid by itself (fluid.c:255-336): made, advanced, read, freed. */
void* refFluidNew(float inner, float outer, float spin, double time) { return artfFluidNew(inner, outer, spin, time); }
int refFluidAdvance(void* f, double time) { return artfFluidAdvance((ArtfFluid*)f, time); }
double refFluidRead(const void* f, float* out) {
    memcpy(out, artfFluidField((const ArtfFluid*)f), sizeof(float) * ARTF_FLUID_WIDTH * ARTF_FLUID_HEIGHT);
    return artfFluidTime((const ArtfFluid*)f);
}
void refFluidFree(void* f) { artfFluidFree((ArtfFluid*)f); }

/* n rays at image positions (nx, ny) in -1..1 and moments time[]: linear RGB of each, 3 floats a ray. */
void refTrace(const ArtfHoleFrame* h, const float* map, const float* fluid, int n, const float* nx, const float* ny,
              const float* time, float* rgb) {
    for (int i = 0; i < n; i += 8) {
        float x[8], y[8];
        const int lanes = n - i < 8 ? n - i : 8;
        for (int k = 0; k < 8; ++k) {
            x[k] = nx[i + (k < lanes ? k : 0)];
            y[k] = ny[i + (k < lanes ? k : 0)];
        }
        /* one moment for the eight: the harness calls with one moment per group of eight */
        V8F r, g, b;
        lensTrace(h, map, fluid, v8fLoad(x), v8fLoad(y), time[i], &r, &g, &b);
        float rr[8], gg[8], bb[8];
        v8fStore(rr, r);
        v8fStore(gg, g);
        v8fStore(bb, b);
        for (int k = 0; k < lanes; ++k) {
            rgb[(i + k) * 3 + 0] = rr[k];
            rgb[(i + k) * 3 + 1] = gg[k];
            rgb[(i + k) * 3 + 2] = bb[k];
        }
    }
}

typedef struct RenderJob {
    ArtfSoftFrame* f;
    const ArtfKernels* kernels;
} RenderJob;

static void renderTile(void* user, uint32_t tile, uint32_t worker) {
    (void)worker;
    RenderJob* j = user;
    j->kernels->lens(j->f, tile);
}

static double nowMs(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec * 1e3 + (double)t.tv_nsec * 1e-6;
}

/* The whole frame through the reference's tile loop (software.c:417, lens.inc:355) on `threads`
 * threads (0: all, at most 16), into three planes of stride (width + 7) & ~7 (software.c:391).
 * simd: 0 the widest kernels here, 1 portable. Best of `repeat` runs, in ms. */
double refRender(const ArtfHoleFrame* h, const float* map, const float* fluid, int threads, int simd, int repeat,
                 float* r, float* g, float* b) {
    ArtfSoftFrame f;
    memset(&f, 0, sizeof f);
    f.width = (int)h->size[0];
    f.height = (int)h->size[1];
    f.tilesX = (f.width + ARTF_TILE - 1) / ARTF_TILE;
    f.tilesY = (f.height + ARTF_TILE - 1) / ARTF_TILE;
    f.hdrStride = (f.width + 7) & ~7;
    f.hdr[0] = r;
    f.hdr[1] = g;
    f.hdr[2] = b;
    f.holeData = *h;
    f.holeMap = map;
    f.holeFluid = fluid;
    RenderJob job = {&f, &artfKernelsPortable};
#ifdef ARTFUL_HAVE_AVX2
    if (!simd && __builtin_cpu_supports("avx2")) job.kernels = &artfKernelsAvx2;
#endif
    ArtfPool* pool = artfPoolNew(threads);
    double best = 1e30;
    for (int k = 0; k < (repeat > 0 ? repeat : 1); ++k) {
        const double t0 = nowMs();
        artfPoolRun(pool, renderTile, &job, (uint32_t)(f.tilesX * f.tilesY));
        const double t = nowMs() - t0;
        if (t < best) best = t;
    }
    artfPoolFree(pool);
    return best;
}

int refPoolThreads(int threads) {
    ArtfPool* pool = artfPoolNew(threads);
    const int n = artfPoolSize(pool);
    artfPoolFree(pool);
    return n;
}

/* A whole BGRA frame from the reference's software renderer, through its public API
 * (artfRendererNew / Draw / ReadPixels, renderer.c:189-254), for a scene holding only this view's hole,
 * with the given map and fluid field put in place of the scene's own (the same inputs the GPU reads). */
void refDraw(const RefView* v, const float* map, const float* fluid, int threads, uint32_t* bgra) {
    ArtfScene* s = artfSceneNew();
    artfSceneSetCamera(s, &v->camera);
    artfSceneSetBlackHole(s, &v->desc);
    memcpy(s->hole.map, map, sizeof(float) * ARTF_HOLE_MAP_FLOATS);
    memcpy((float*)artfFluidField(s->hole.fluid), fluid, sizeof(float) * ARTF_FLUID_WIDTH * ARTF_FLUID_HEIGHT);
    ArtfRendererOptions o = artfRendererDefaults(v->width, v->height);
    o.backend = ARTF_BACKEND_SOFTWARE;
    o.threads = threads;
    ArtfRenderer* r = artfRendererNew(&o);
    artfRendererDraw(r, s);
    artfRendererReadPixels(r, bgra);
    artfRendererFree(r);
    artfSceneFree(s);
}

/* The reference's own scene over time: one scene and one software renderer of the first view's size;
 * each view's camera and description set in turn (artfSceneSetBlackHole paints the disc, starts and
 * advances the gas: hole.c:242-271), and after each view marked in `drawAfter` a frame drawn and read
 * into the next width * height of bgra; the gas's time after each view into fluidTimes (may be NULL).
 * Nothing is put in place of the scene's own map or fluid. */
void refDrawScene(const RefView* views, const int* drawAfter, int count, int threads, uint32_t* bgra,
                  double* fluidTimes) {
    ArtfScene* s = artfSceneNew();
    ArtfRendererOptions o = artfRendererDefaults(views[0].width, views[0].height);
    o.backend = ARTF_BACKEND_SOFTWARE;
    o.threads = threads;
    ArtfRenderer* r = artfRendererNew(&o);
    const size_t pixels = (size_t)views[0].width * (size_t)views[0].height;
    for (int i = 0; i < count; ++i) {
        artfSceneSetCamera(s, &views[i].camera);
        artfSceneSetBlackHole(s, &views[i].desc);
        if (fluidTimes) fluidTimes[i] = artfFluidTime(s->hole.fluid);
        if (!drawAfter[i]) continue;
        artfRendererDraw(r, s);
        artfRendererReadPixels(r, bgra);
        bgra += pixels;
    }
    artfRendererFree(r);
    artfSceneFree(s);
}

/* The reference's ISCO and orbit speed (hole.c:207, hole.c:215). */
float refIsco(float spin) { return artfHoleIsco(spin); }
float refOrbitSpeed(float spin, float r) { return artfBlackHoleOrbitSpeed(spin, r); }

/* Sizes of what the harness hands across, for the caller to check its own layout against. */
void refSizes(int* out) {
    out[0] = (int)sizeof(ArtfHoleFrame);
    out[1] = (int)sizeof(ArtfBlackHoleDesc);
    out[2] = (int)sizeof(ArtfCamera);
    out[3] = (int)sizeof(RefView);
    out[4] = ARTF_HOLE_MAP_FLOATS;
    out[5] = ARTF_FLUID_WIDTH * ARTF_FLUID_HEIGHT;
}
