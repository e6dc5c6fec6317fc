/* artful_cuda — the GB300 hole tracer as an Artful renderer backend, beside Vulkan and software.
 *
 * The renderer is an object that begins with a table of eight functions, as every Artful backend does
 * (src/render/rendererInternal.h:7-27: ArtfRendererVtbl and struct ArtfRenderer): Artful's public
 * calls (artfRendererDraw, ReadPixels, Stats, ...) dispatch through it unchanged.  This backend draws
 * the black hole only: the trace on the GPU, then its bloom and tone map, to BGRA.
 *
 * A backend reads the scene.  In Artful's own tree the scene is the internal ArtfScene; this library
 * cannot include it, so the renderer reads a scene through an ArtfCudaSceneReader, a function that
 * fills ArtfCudaHoleInputs from whatever the scene pointer points at.  The reader for Artful's scene is
 * a few lines in the backend file a maintainer adds to Artful's tree (src/cuda/, beside its other
 * backends); the reader for ArtfCudaScene, this library's own minimal hole scene, is built in. */
#ifndef ARTFUL_CUDA_RENDERER_H
#define ARTFUL_CUDA_RENDERER_H

#include "artful_cuda.h"

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ArtfBackend (include/artful/renderer.h:24) with this backend appended. */
enum { ARTF_CUDA_BACKEND = 4 };

/* Layout-compatible with ArtfSurface and ArtfRendererOptions (include/artful/renderer.h:37-71). */
typedef struct ArtfCudaSurface {
    int kind;
    void* a;
    void* b;
} ArtfCudaSurface;

typedef struct ArtfCudaRendererOptions {
    int backend;
    ArtfCudaSurface surface; /* not used: the frame stays in memory */
    int width, height;
    bool noVsync;
    int threads;
    int simd;
    bool antialias;
    bool hdr;
    bool compressTextures;
    const char* pipelineCache;
} ArtfCudaRendererOptions;

/* Layout-compatible with ArtfOverlay and ArtfRect (include/artful/renderer.h:86-105). */
typedef struct ArtfCudaRect { int x, y, w, h; } ArtfCudaRect;
typedef struct ArtfCudaOverlay {
    const uint32_t* pixels;
    int width, height;
    int stride;
    bool partial;
    const ArtfCudaRect* damage;
    size_t damageCount;
} ArtfCudaOverlay;

/* Layout-compatible with ArtfFrameStats (include/artful/renderer.h:118-131). */
typedef struct ArtfCudaFrameStats {
    double cpuMs, cullMs, geometryMs, rasterMs, lensMs;
    uint32_t instancesDrawn, trianglesBinned, tilesSkipped, instancesHidden, traceSamples;
    double gpuMs;
    uint32_t shadowMapsDrawn;
} ArtfCudaFrameStats;

typedef struct ArtfCudaRenderer ArtfCudaRenderer;

/* The table every backend fills (src/render/rendererInternal.h:7-16). */
typedef struct ArtfCudaRendererVtbl {
    const char* (*description)(const ArtfCudaRenderer* r);
    void (*resize)(ArtfCudaRenderer* r, int width, int height);
    void (*setOverlay)(ArtfCudaRenderer* r, const ArtfCudaOverlay* overlay);
    bool (*draw)(ArtfCudaRenderer* r, void* scene);
    bool (*readPixels)(ArtfCudaRenderer* r, uint32_t* dst);
    uint32_t* (*pixels)(ArtfCudaRenderer* r);
    void (*stats)(const ArtfCudaRenderer* r, ArtfCudaFrameStats* out);
    void (*destroy)(ArtfCudaRenderer* r);
} ArtfCudaRendererVtbl;

/* The head every renderer starts with (src/render/rendererInternal.h:18-27). */
struct ArtfCudaRenderer {
    const ArtfCudaRendererVtbl* vt;
    int backend;
    int trialFrame;
    double trialMs[2];
};

/* What the backend reads of a scene each frame. */
typedef struct ArtfCudaHoleInputs {
    bool on;                    /* a hole is set (artfSceneSetBlackHole with a description) */
    ArtfCudaCamera camera;
    ArtfCudaBlackHoleDesc desc; /* as artfSceneSetBlackHole clamped it */
    const float* map;           /* ARTF_CUDA_MAP_FLOATS, host, borrowed for the call */
    uint64_t mapVersion;        /* changes when the map does (with the scene's identity folded in) */
    const float* fluid;         /* ARTF_CUDA_FLUID_FLOATS, host, borrowed */
    uint64_t fluidVersion;
    double fluidTime;           /* the moment the fluid field is of */
    /* The scene's gas by its clock, for a backend that steps the gas on the device
     * (artfCudaRendererSetDeviceInputs): a number that changes whenever the gas starts afresh (hole.c:265,
     * a new disc or spin; 0: not known, and the backend then follows desc.time at each draw), the moment
     * it started, the steps taken since (artfCudaFluidClock's count over every advance) and its clock. */
    uint64_t gasGeneration;
    double gasStart;
    uint64_t gasSteps;
    double gasClock;
} ArtfCudaHoleInputs;

typedef bool (*ArtfCudaSceneReader)(const void* scene, ArtfCudaHoleInputs* out);

/* A renderer on the first sm_103 device, or NULL (logged through artfCudaLastError) when there is
 * none.  artfCudaNew reads ArtfCudaScene; artfCudaNewWithReader reads any scene through `reader`. */
ArtfCudaRenderer* artfCudaNew(const ArtfCudaRendererOptions* options);
ArtfCudaRenderer* artfCudaNewWithReader(const ArtfCudaRendererOptions* options, ArtfCudaSceneReader reader);

/* Beyond the table: the last frame's linear light, width * height float4 (RGB, pixel-class bits),
 * before bloom and tone map; the trace's precision (ArtfCudaPrecision, default ARTF_CUDA_EXACT: the
 * software backend's pixels); the context, for fault injection in tests. */
bool artfCudaRendererReadLight(ArtfCudaRenderer* r, float* dst);
void artfCudaRendererSetPrecision(ArtfCudaRenderer* r, int precision);
ArtfCuda* artfCudaRendererContext(ArtfCudaRenderer* r);
/* Device inputs: the renderer ignores the scene's host map and fluid and makes the reference's own on
 * the GPU from the description, as artfSceneSetBlackHole makes them on the CPU (hole.c:249-270): the
 * painted disc (artfCudaPaintDisc) whenever the disc or the spin changes, and the gas (ArtfCudaFluid),
 * started then and stepped as the scene's clock says (the inputs' gas fields).  No map or fluid crosses
 * from the host.  Off by default (the scene's host inputs are drawn). */
void artfCudaRendererSetDeviceInputs(ArtfCudaRenderer* r, bool on);

/* ---- the library's own minimal hole scene (Artful's scene API for this path, restated) ------------ */

typedef struct ArtfCudaScene ArtfCudaScene;
ArtfCudaScene* artfCudaSceneNew(void);
void artfCudaSceneFree(ArtfCudaScene* s);
/* scene.h:322 artfSceneSetCamera */
void artfCudaSceneSetCamera(ArtfCudaScene* s, const ArtfCudaCamera* camera);
/* scene.h:500 artfSceneSetBlackHole: NULL removes the hole.  The description is clamped as the
 * reference clamps it; the disc is the synthetic one (artfCudaSynthMap: seed, emissivity 3), rebuilt when
 * the disc or the spin changes; the fluid field is 1 everywhere.  The gas's clock runs as the
 * reference's (a new gas when the disc or the spin changes, else an advance to the description's time),
 * for renderers that draw with device inputs. */
void artfCudaSceneSetBlackHole(ArtfCudaScene* s, const ArtfCudaBlackHoleDesc* desc);
/* A caller's own map and fluid field in place of the synthetic ones (copied). */
void artfCudaSceneSetHoleMap(ArtfCudaScene* s, const float* map, const float* fluid, double fluidTime);
void artfCudaSceneSetSeed(ArtfCudaScene* s, uint64_t seed, float emissivity);
bool artfCudaSceneReadHole(const void* scene, ArtfCudaHoleInputs* out);

#ifdef __cplusplus
}
#endif

#endif
