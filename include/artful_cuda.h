/* artful_cuda — Artful's Kerr black-hole tracer on one GB300 (sm_103a).
 *
 * The C ABI between a C11 host and the CUDA kernels.  Plain pointers and sizes only.  Every call
 * returns 0 or a negative ArtfCudaStatus, and never aborts.  Pointers are borrowed for the call
 * unless a comment says otherwise.
 *
 * What it replaces in the reference (eugeniobenfica/artful v0.4.0):
 *   - the per-pixel trace `lensTrace` / `lensTile` of the software backend (src/software/lens.inc:99,
 *     355) and the Vulkan hole compute shader (src/vulkan/shaders.c:1957 artfShaderHoleTrace), as
 *     dispatched by `drawHole` (src/software/software.c:410-417) and `traceHole`
 *     (src/vulkan/vulkan.c:1758-1781);
 *   - the host set-up those read: `artfHoleFrame` (src/scene/hole.c:273), `artfHoleIsco` (hole.c:207),
 *     `artfBlackHoleOrbitSpeed` (hole.c:215), `artfBlackHoleDefaults` (hole.c:225), the clamps of
 *     `artfSceneSetBlackHole` (hole.c:242-258) and the ring tables of `setRings` (hole.c:186).
 * The renderer backend that plugs all of this behind `artfRendererNew` is in artful_cuda_renderer.h. */
#ifndef ARTFUL_CUDA_H
#define ARTFUL_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ARTF_CUDA_ABI_VERSION 1

/* ---- data layouts shared with the reference ----------------------------------------------------- */

/* The map every backend reads, one block of floats (src/scene/sceneInternal.h:18-32, 324-329):
 * painted gas 2048 x 1024 (rows even in 1/r), per row (turns per unit time, heat), black-body colours
 * 256 x 3, sky dust 1024 x 512, per row glow, dust 1024 x 256.  The fluid is 1024 x 256. */
#define ARTF_CUDA_MAP_WIDTH 2048
#define ARTF_CUDA_MAP_HEIGHT 1024
#define ARTF_CUDA_DUST_WIDTH 1024
#define ARTF_CUDA_DUST_HEIGHT 256
#define ARTF_CUDA_FLUID_WIDTH 1024
#define ARTF_CUDA_FLUID_HEIGHT 256
#define ARTF_CUDA_COLORS 256
#define ARTF_CUDA_SKY_WIDTH 1024
#define ARTF_CUDA_SKY_HEIGHT 512
#define ARTF_CUDA_BLOOM_LEVELS 8
#define ARTF_CUDA_ROWS_AT (ARTF_CUDA_MAP_WIDTH * ARTF_CUDA_MAP_HEIGHT)
#define ARTF_CUDA_COLORS_AT (ARTF_CUDA_ROWS_AT + ARTF_CUDA_MAP_HEIGHT * 2)
#define ARTF_CUDA_SKY_AT (ARTF_CUDA_COLORS_AT + ARTF_CUDA_COLORS * 3)
#define ARTF_CUDA_GLOW_AT (ARTF_CUDA_SKY_AT + ARTF_CUDA_SKY_WIDTH * ARTF_CUDA_SKY_HEIGHT)
#define ARTF_CUDA_DUST_AT (ARTF_CUDA_GLOW_AT + ARTF_CUDA_MAP_HEIGHT)
#define ARTF_CUDA_MAP_FLOATS (ARTF_CUDA_DUST_AT + ARTF_CUDA_DUST_WIDTH * ARTF_CUDA_DUST_HEIGHT)
#define ARTF_CUDA_FLUID_FLOATS (ARTF_CUDA_FLUID_WIDTH * ARTF_CUDA_FLUID_HEIGHT)

/* Layout-compatible with the reference's public ArtfVec3 and ArtfCamera (include/artful/core.h,
 * include/artful/scene.h:314-320). */
typedef struct ArtfCudaVec3 { float x, y, z; } ArtfCudaVec3;
typedef struct ArtfCudaCamera {
    ArtfCudaVec3 position, target, up;
    float fovY;  /* radians */
    float near_;
} ArtfCudaCamera;

/* Layout-compatible with the reference's ArtfBlackHoleDesc (include/artful/scene.h:470-490). */
typedef struct ArtfCudaBlackHoleDesc {
    ArtfCudaVec3 position, axis;
    float mass, spin, discInner, discOuter, discHeight, discThickness, discGain, doppler, stars, bloom, exposure,
        time, shutter;
    ArtfCudaVec3 velocity;
    int samples;
} ArtfCudaBlackHoleDesc;

/* Per-frame constants, the reference's uniform block (src/scene/sceneInternal.h:302-319): 368 bytes. */
typedef struct ArtfCudaHoleFrame {
    float er[4];      /* the eye on the unit sphere in the disc frame (x, z, axis); w: its distance */
    float etheta[4], ephi[4];
    float right[4], up[4], forward[4]; /* a pixel's ray along (r, theta, phi) at the eye */
    float metric[4];  /* lapse, frame-drag rate times radius, that radius, radius per sine */
    float place[4];   /* sqrt(Sigma), sqrt(Delta), 1/r, cos(theta) */
    float spin[4];    /* a, 0.995 / r+, disc height, shutter */
    float flow[4];    /* the moment the fluid field is of */
    float boost[4];   /* eye velocity along (r, theta, phi); w: gamma */
    float disc[4];    /* inner, outer, time, thickness */
    float look[4];    /* gain, doppler, stars, bloom */
    float image[4];   /* exposure, 2/width, 2/height, 1/rays a pixel */
    uint32_t size[4]; /* width, height, rays a side, bloom levels */
    uint32_t bloom[ARTF_CUDA_BLOOM_LEVELS][4];
} ArtfCudaHoleFrame;

/* The same constants computed in double from the same description (no reference counterpart: the
 * reference fills its frame in FP32).  The FP64 and mixed-precision traces read it. */
typedef struct ArtfCudaHoleFrame64 {
    double er[4], etheta[4], ephi[4], right[4], up[4], forward[4], metric[4], place[4], spin[4], flow[4], boost[4],
        disc[4], look[4], image[4];
} ArtfCudaHoleFrame64;

/* ---- status ------------------------------------------------------------------------------------- */

typedef enum ArtfCudaStatus {
    ARTF_CUDA_OK = 0,
    ARTF_CUDA_EINVAL = -1,     /* a NULL pointer, a size out of range, an unknown option */
    ARTF_CUDA_ENODEVICE = -2,  /* no sm_103 device, or the device asked for does not exist */
    ARTF_CUDA_ENOMEM = -3,     /* a device allocation failed */
    ARTF_CUDA_ELAUNCH = -4,    /* a launch or copy failed; the context should be destroyed */
    ARTF_CUDA_ETIMEOUT = -5,   /* a bounded device wait gave up (the persistent queue) */
    ARTF_CUDA_ELOST = -6,      /* the context was marked lost (a fault injected on the host) */
    ARTF_CUDA_EBOUNDS = -7     /* (the debug build, ARTF_CUDA_DEBUG_BOUNDS) an index outside its table or
                                * frame: the read was kept inside the buffer and the write skipped */
} ArtfCudaStatus;

/* A line about the last error of this thread's calls; borrowed. */
const char* artfCudaLastError(void);

/* ---- host set-up: the reference's hole.c, restated (C11, no GPU needed) ------------------------- */

/* hole.c:225 artfBlackHoleDefaults */
ArtfCudaBlackHoleDesc artfCudaBlackHoleDefaults(void);
/* hole.c:207 artfHoleIsco: the innermost stable circular orbit, in masses */
float artfCudaIsco(float spin);
/* hole.c:215 artfBlackHoleOrbitSpeed */
float artfCudaOrbitSpeed(float spin, float r);
/* The clamps artfSceneSetBlackHole applies (hole.c:245-258): spin to +-0.998, inner to the ISCO when 0 or
 * at least r+ + 0.2, outer at least inner + 1, height at least 1e-3, samples 1..8, mass at least 1e-6. */
void artfCudaHoleClamp(const ArtfCudaBlackHoleDesc* in, ArtfCudaBlackHoleDesc* out);
/* hole.c:273 artfHoleFrame for a clamped description, the camera, and the moment the fluid field is of.
 * Returns the bloom pixel count; 0 on a bad argument. */
uint32_t artfCudaHoleFrame(const ArtfCudaCamera* camera, const ArtfCudaBlackHoleDesc* clamped, double fluidTime,
                           int width, int height, ArtfCudaHoleFrame* out);
/* The same frame in double (for the FP64 and mixed traces). Returns 0, or ARTF_CUDA_EINVAL. */
int artfCudaHoleFrame64(const ArtfCudaCamera* camera, const ArtfCudaBlackHoleDesc* clamped, double fluidTime,
                        int width, int height, ArtfCudaHoleFrame64* out);
/* hole.c:186 setRings: per map row its orbit speed and heat, and its glow (the reference's painted disc). */
void artfCudaSetRings(float* map, float inner, float outer, float spin);
/* The same tables by themselves: rows (ARTF_CUDA_MAP_HEIGHT x 2) and glow (ARTF_CUDA_MAP_HEIGHT). */
void artfCudaHoleRings(float* rows, float* glow, float inner, float outer, float spin);
/* hole.c:161-166: the black-body colour table (ARTF_CUDA_COLORS x 3 floats). */
void artfCudaHoleColours(float* colors);

/* The synthetic disc and sky of the benchmark configurations, written into a whole map.
 *   gas:   value noise on a 64 x 64 lattice in (radius row, azimuth), seeded, in [0.5, 1.5];
 *   glow:  (r / inner)^-emissivity, so the emission falls as r^-q;
 *   rows:  the reference's orbit speed and heat (hole.c:186-192);
 *   colours: the reference's black-body table (hole.c:159-164);
 *   sky:   a floor of 0.0006 plus `stars` point stars, uniform on the sphere, brightness log-uniform in
 *          [1e-3, 1], splatted bilinearly;  dust: none.
 * Every value comes from integer hashing and IEEE + - * / sqrt only: the same bits on every host. */
typedef struct ArtfCudaSynthDesc {
    uint64_t seed;
    float inner, outer, spin;  /* the clamped disc */
    float emissivity;          /* q */
    int stars;                 /* how many catalogue stars: 2000 in the benchmarks */
} ArtfCudaSynthDesc;
int artfCudaSynthMap(const ArtfCudaSynthDesc* desc, float* map);
/* Only the rows and glow of a synthetic map (what changes with spin, inner and q). */
void artfCudaSynthRings(const ArtfCudaSynthDesc* desc, float* map);

/* ---- device context ------------------------------------------------------------------------------ */

typedef struct ArtfCuda ArtfCuda;

/* Opens `device` (an sm_103 GPU) and its stream; owns the device copies of the map and fluid. */
int artfCudaCreate(int device, ArtfCuda** out);
void artfCudaDestroy(ArtfCuda* ctx);
/* Copies a whole map (ARTF_CUDA_MAP_FLOATS) / fluid field (ARTF_CUDA_FLUID_FLOATS) from the host when
 * `version` differs from the one held (0 always copies). */
int artfCudaSetMap(ArtfCuda* ctx, const float* hostMap, uint64_t version);
int artfCudaSetFluid(ArtfCuda* ctx, const float* hostFluid, uint64_t version);
/* Fault injection on the host, for tests of device loss (the reference's artfVulkanSubmitsLeft,
 * src/render/rendererInternal.h:29-30): after `launches` more launches the context reports
 * ARTF_CUDA_ELOST, as after a device loss, without the GPU being touched.  -1 turns it off. */
int artfCudaFailAfter(ArtfCuda* ctx, int launches);
/* Allocation failure injected on the host (the reference counts allocations for its tests,
 * src/core/base.c:32-33): after `allocations` more device or page-locked allocations the context's next
 * one fails, as on an exhausted device, without the driver being asked, and the call reports
 * ARTF_CUDA_ENOMEM; the context stays usable.  -1 turns it off. */
int artfCudaFailAllocAfter(ArtfCuda* ctx, int allocations);
/* The device copies, for callers that launch on their own buffers. */
const float* artfCudaDeviceMap(const ArtfCuda* ctx);
const float* artfCudaDeviceFluid(const ArtfCuda* ctx);
/* The context's stream (a cudaStream_t). */
void* artfCudaStream(const ArtfCuda* ctx);

/* ---- the trace ----------------------------------------------------------------------------------- */

typedef enum ArtfCudaPrecision {
    ARTF_CUDA_EXACT = 0,  /* FP32 with the reference's rounding (no contraction, IEEE / and sqrt): the same
                           * bits as the software backend */
    ARTF_CUDA_FP32 = 1,   /* FP32 with fused multiply-adds and fast reciprocals */
    ARTF_CUDA_FP64 = 2,   /* plain FP64 throughout, from the FP64 frame */
    ARTF_CUDA_MIXED = 3   /* FP32 steps; FP64 constants of motion, turning-point and near-horizon steps */
} ArtfCudaPrecision;

typedef struct ArtfCudaTraceOptions {
    int precision;       /* ArtfCudaPrecision */
    int jitter;          /* 0: the reference's side x side stratified samples (frame size[2]);
                          * n > 0: n rays a pixel at seeded uniform sub-pixel offsets */
    uint32_t seed;       /* of the jitter */
    float stepScale;     /* 1: the reference's step (pi/24 / sqrt(max(K, 4))); 0.5: half steps, with twice
                          * the step cap. 0 means 1 */
    float horizonBand;   /* mixed: FP64 radial sub-steps where u > band * (0.995 / r+), i.e. within about
                          * r+ / band of the hole; 0 means the default 0.95 */
    int blockSize;       /* threads a block: 0 picks the tuned value */
    int compactEvery;    /* steps between warp refills: 0 picks the tuned value */
    int persistent;      /* 1: one block per SM slot, rays pulled from a queue; 0: one ray a thread */
    uint32_t guards;     /* mixed: which FP64 guards run (ARTF_CUDA_GUARD_*); 0 means all */
    int fp64Batch;       /* mixed: lanes that wait for a wide sub-step before a warp runs them; 0: 32 */
    int refillBatch;     /* mixed: idle lanes before a warp starts new rays (wide set-ups); 0: 32 */
    int64_t bandRays;    /* a frame of more rays than this goes out in bands of whole rows of at most this
                          * many rays, each launched and waited for, so that no launch holds the GPU long
                          * (vulkan.c:1729-1756).  0: the reference's choice, bands of 8e6 rays for frames
                          * above 6.4e7 (a 4K frame of 64 rays a pixel is seconds of work); < 0: never.
                          * Single frames only; the result is the same bits either way */
    int order;           /* mixed: the order the queue hands out work.  0: heavy first (one probe ray a tile
                          * estimates each 8 x 4 tile's steps, and the heaviest go first, so that the
                          * launch does not end on long rays started late); 1: pixel order.  The result is
                          * the same bits either way */
} ArtfCudaTraceOptions;

enum { ARTF_CUDA_ORDER_HEAVY_FIRST = 0, ARTF_CUDA_ORDER_PIXELS = 1 };

/* The mixed trace's guards: work carried at about FP64's precision ("wide"), as double-float pairs on the
 * FP32 pipe, or in FP64 within the horizon's band. */
enum {
    ARTF_CUDA_GUARD_MOTION = 1,   /* the constants of motion from the ray, wide (the first state from them) */
    ARTF_CUDA_GUARD_HORIZON = 2,  /* FP64 radial sub-steps within the band of the outer horizon */
    ARTF_CUDA_GUARD_RADIAL = 4,   /* the step where du/ds changes sign, its radial motion wide */
    ARTF_CUDA_GUARD_POLAR = 8,    /* the step where the axis part of dn/ds changes sign, its axis part wide */
    ARTF_CUDA_GUARD_PSI = 16,     /* compensated summation of psi */
    ARTF_CUDA_GUARD_ALL = 31
};

/* Endpoint of each ray (optional output), 32 bytes. */
typedef struct ArtfCudaRayEnd {
    float hitR, hitPhi;  /* first lit disc crossing: radius in masses, azimuth in turns [0, 1); NaN: none */
    float dir[3];        /* escape direction, after the frame-drag rotation; 0: did not escape */
    float mino;          /* the Mino time at the endpoint */
    uint16_t steps;      /* integration steps taken */
    uint8_t crossings;   /* accepted disc crossings */
    uint8_t kind;        /* ARTF_CUDA_END_*, | ARTF_CUDA_END_LIT when a crossing gave light */
    uint16_t fp64Steps;  /* of those, how many ran wide (the mixed trace) */
    uint16_t reserved;
} ArtfCudaRayEnd;

enum {
    ARTF_CUDA_END_HORIZON = 0,  /* fell through 0.995 r+ */
    ARTF_CUDA_END_SKY = 1,      /* escaped (u < 0) */
    ARTF_CUDA_END_OPAQUE = 2,   /* the disc let through 0.004 or less */
    ARTF_CUDA_END_CAP = 3,      /* ran out of steps */
    ARTF_CUDA_END_LIT = 0x10
};

/* Pixel classes written into the alpha of each HDR pixel: bit 0 a ray was lit by the disc, bit 1 a ray
 * escaped, bit 2 a ray ended dark (horizon, cap or opaque). */

/* What a trace did, counted on the device. */
typedef struct ArtfCudaTraceStats {
    uint64_t rays, steps, crossings, escapes, fp64Steps;
    uint64_t fp64Horizon, fp64Radial, fp64Polar; /* mixed: the wide (FP64-precision) steps by reason */
    uint64_t fp64Rounds;                         /* mixed: warp rounds of wide steps */
    double flops;        /* algorithmic FP32-pipe operations (the counting rule is in lensFlops.h) */
    float ms;            /* device time of the trace kernel(s), CUDA events on the context's stream */
    uint32_t bands;      /* launches the frame went out in (ArtfCudaTraceOptions.bandRays) */
    double flops64;      /* of the work, what ran at FP64's precision (FP64: all of flops; mixed: the wide
                          * set-ups and sub-steps by the same rule, as double-float pairs on the FP32 pipe
                          * or, in the horizon's band, in FP64) */
} ArtfCudaTraceStats;

/* Traces one frame into `hdr` (device memory, width * height float4: linear RGB and the class bits).
 * map, fluid: device pointers (NULL: the context's copies).  frame64: needed for FP64 and MIXED (NULL:
 * promoted from `frame`).  ends: device memory for width * height * rays-a-pixel records, or NULL.
 * stats: filled when not NULL (it synchronises the stream).  Asynchronous otherwise. */
int artfCudaHoleTrace(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                      const float* map, const float* fluid, const ArtfCudaTraceOptions* options, float* hdr,
                      ArtfCudaRayEnd* ends, ArtfCudaTraceStats* stats);

/* Traces n rays at given image positions and moments (device arrays of n floats each) into rgb (device,
 * 3 floats a ray): the per-ray form of the reference's trace (src/software/lens.inc:99 lensTrace), for
 * callers that make their own sample positions.  precision: ArtfCudaPrecision.  ends may be NULL. */
int artfCudaHoleTraceRays(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                          const float* map, const float* fluid, int precision, float stepScale, int n, const float* nx,
                          const float* ny, const float* time, float* rgb, ArtfCudaRayEnd* ends,
                          ArtfCudaTraceStats* stats);

/* A whole frame as a renderer backend draws it, from host buffers: the trace, then the bloom pyramid
 * and the tone map with its dither (src/software/software.c:320-427, src/software/lens.inc:387-440) to
 * premultiplied BGRA (alpha 255).  Copies back the linear light (width * height float4) to hostHdr and
 * the BGRA frame (width * height uint32) to hostBgra, each when not NULL.  Synchronous.  stats->ms is
 * the device time of trace and bloom together (the reference's lensMs).  A NULL hostMap or hostFluid
 * draws with what the context holds (artfCudaPaintDisc, artfCudaUseFluid, an earlier upload). */
int artfCudaHoleDraw(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                     const float* hostMap, uint64_t mapVersion, const float* hostFluid, uint64_t fluidVersion,
                     const ArtfCudaTraceOptions* options, float* hostHdr, uint32_t* hostBgra,
                     ArtfCudaTraceStats* stats);
/* The last frame artfCudaHoleDraw drew on this context, copied back when it is wanted rather than at
 * every draw: its linear light (width * height float4) to hostHdr and its BGRA (width * height uint32)
 * to hostBgra, each when not NULL.  ARTF_CUDA_EINVAL when no draw has finished since the context's frame
 * buffers last changed (artfCudaHoleRender uses the light buffer too).  Synchronous.  (The renderer's
 * readPixels, software.c's frame in host memory, has no counterpart call in the reference: a GPU
 * backend's frame is read back at readPixels.) */
int artfCudaFrameRead(ArtfCuda* ctx, float* hostHdr, uint32_t* hostBgra);
/* The bloom and tone map alone, on device buffers: hdr (width * height float4) to bgra, with three bloom
 * planes of the frame's bloom pixel count (artfCudaHoleFrame's return value), on `stream`. */
int artfCudaPostLaunch(const ArtfCudaHoleFrame* frame, const float* hdr, float* const bloomPlanes[3], uint32_t* bgra,
                       void* stream);

/* ---- batches of views (mixed precision) ---------------------------------------------------------- */

/* One view of a batch: its frames, and device pointers to its inputs and outputs. */
typedef struct ArtfCudaView {
    ArtfCudaHoleFrame frame;
    ArtfCudaHoleFrame64 frame64;
    const float* map;        /* device; NULL: the context's map */
    const float* fluid;      /* device; NULL: the context's fluid */
    float* hdr;              /* device: width * height float4 */
    ArtfCudaRayEnd* ends;    /* device, or NULL */
} ArtfCudaView;

#define ARTF_CUDA_MAX_VIEWS 4096

/* Traces `count` views of any sizes in one persistent launch (mixed precision): every view's pixels
 * feed one device work queue that the resident warps steal from, so uneven views balance.  The view
 * table is copied to the device on the context's stream.  Asynchronous unless stats is given.  No
 * counterpart in the reference (it draws one view a frame). */
int artfCudaHoleBatch(ArtfCuda* ctx, const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options,
                      ArtfCudaTraceStats* stats);

/* The same batch captured once in a CUDA graph (table copy, counter reset, launch), then replayed.
 * Update replaces the views' frames and pointers (same count and sizes) for the next launch.  The graph
 * owns its device table and pinned staging; the views are copied in at create and update. */
typedef struct ArtfCudaGraph ArtfCudaGraph;
int artfCudaBatchGraphCreate(ArtfCuda* ctx, const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options,
                             ArtfCudaGraph** out);
int artfCudaBatchGraphUpdate(ArtfCudaGraph* graph, const ArtfCudaView* views, int count);
int artfCudaBatchGraphLaunch(ArtfCudaGraph* graph, ArtfCudaTraceStats* stats);
void artfCudaBatchGraphDestroy(ArtfCudaGraph* graph);

/* A batch trace that allocates nothing, for callers that cannot call cudaMalloc: a host engine or
 * plug-in framework that owns all device memory through its own allocator, or a render thread that
 * must not stall on an allocation.  No counterpart in the reference.  It needs no context: it traces on
 * the current device and on the caller's `stream` (a cudaStream_t, or NULL), and every view's map,
 * fluid and hdr must be device pointers the caller owns.  Its scratch (the view table and the queue
 * counters) is one fixed array on each device that loads the library, held until the process exits
 * (82 KB): so a batch holds at most ARTF_CUDA_NOALLOC_MAX_VIEWS views, and more is refused with
 * ARTF_CUDA_EINVAL.  No room is left for ray planes or the heavy-first order: each work unit is a pixel,
 * whose rays one lane traces in turn, in pixel order (options->order is ignored), which can be slower
 * than the context's batch for views of several rays a pixel.  The first call on each device looks up
 * the array's device address there and keeps it; after a device reset the process must restart before
 * calling this again.  A call on a stream that is being captured is refused (ARTF_CUDA_EINVAL): the
 * graph API is the form to capture.  Calls share the array: calls whose work overlaps on the GPU race,
 * so order them on one stream.  Asynchronous; stats, when given, synchronises the stream and fills the
 * counts (not ms or flops). */
#define ARTF_CUDA_NOALLOC_MAX_VIEWS 64
int artfCudaHoleBatchNoAlloc(const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options, void* stream,
                             ArtfCudaTraceStats* stats);

/* The autotuner: times the batch under candidate launch shapes (threads a block, steps a lane waits at
 * most before a refill or an FP64 round, the FP64 and refill batch sizes), by coordinate descent from
 * the defaults, and keeps the fastest in the context: later mixed traces whose options leave these at 0
 * use it.  Synchronous; a few hundred launches. */
typedef struct ArtfCudaTuning {
    int blockSize, compactEvery, fp64Batch, refillBatch;
    float ms;         /* the best time found */
    float defaultMs;  /* the defaults' time */
    int trials;
} ArtfCudaTuning;
int artfCudaAutotune(ArtfCuda* ctx, const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options,
                     ArtfCudaTuning* result);

/* The same from host memory to host memory: copies the map and fluid (when their versions changed; NULL:
 * the context's own), traces, and brings width * height float4 back to `hostHdr`: a page-locked buffer
 * (cudaHostAlloc, or registered) is written by the trace's kernels directly, any other is copied into
 * from the device's frame.  Synchronous. */
int artfCudaHoleRender(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                       const float* hostMap, uint64_t mapVersion, const float* hostFluid, uint64_t fluidVersion,
                       const ArtfCudaTraceOptions* options, float* hostHdr, ArtfCudaTraceStats* stats);

/* ---- gradients of an image loss (no reference counterpart) ---------------------------------------- */

/* A scene by its five physical parameters, theta = (spin a, inclination i in radians from the axis,
 * inner disc radius as a multiple of the ISCO, emissivity index q, observer distance r_obs), the eye at
 * r_obs (0, cos i, sin i) looking at the hole with +y up, the hole's axis +y, one ray at each pixel's
 * centre, and the synthetic disc (artfCudaSynthMap) of emissivity r^-q.  The remaining fields hold
 * fixed. */
typedef struct ArtfCudaHoleParams {
    double spin, inclination, innerScale, emissivity, distance;
    double fovY, outer, height, thickness, gain, doppler, stars, time;
    uint64_t seed;
} ArtfCudaHoleParams;

/* The frame fields the parameters reach: forward, right, up (3 each), metric (4), place (4), er,
 * etheta, ephi (3 each), the spin, the inner radius. */
#define ARTF_CUDA_GRAD_FIELDS 28

/* The scene's camera and description; its FP32 and FP64 frames and the Jacobian of the frame fields in
 * theta (ARTF_CUDA_GRAD_FIELDS x 5, row-major: central differences of the FP64 frame); its map.  Any
 * output may be NULL.  The inner radius is used as given (not clamped). */
int artfCudaHoleParamsScene(const ArtfCudaHoleParams* params, ArtfCudaCamera* camera, ArtfCudaBlackHoleDesc* desc);
int artfCudaHoleParamsFrames(const ArtfCudaHoleParams* params, int width, int height, ArtfCudaHoleFrame* frame,
                             ArtfCudaHoleFrame64* frame64, double* jacobian);
int artfCudaHoleParamsMap(const ArtfCudaHoleParams* params, float* map);

/* The FP64 forward-mode reference: for each pixel and colour channel, its radiance and the radiance's
 * five derivatives in theta, into `out` (device, width * height * 3 * 6 doubles).  map and fluid: device
 * pointers (NULL: the context's).  Synchronous. */
int artfCudaHoleTangents(ArtfCuda* ctx, const ArtfCudaHoleParams* params, const ArtfCudaHoleFrame* frame,
                         const ArtfCudaHoleFrame64* frame64, const double* jacobian, const float* map,
                         const float* fluid, double* out);

#define ARTF_CUDA_ADJOINT_MIN_CHECKPOINT 1
#define ARTF_CUDA_ADJOINT_MAX_CHECKPOINT 64
#define ARTF_CUDA_ADJOINT_MAX_VIEWS 1024

/* A view's loss, L = sum over pixels and colour channels of (radiance - target)^2 / (3 * pixels), and
 * its gradient in theta = (spin, inclination, innerScale, emissivity, distance). */
typedef struct ArtfCudaAdjointResult {
    double loss;
    double grad[5];
} ArtfCudaAdjointResult;

/* The adjoint: reverse-mode derivatives of the FP32 trace, checkpointing the ray's state every
 * `checkpointEvery` steps (ARTF_CUDA_ADJOINT_MIN_CHECKPOINT .. ARTF_CUDA_ADJOINT_MAX_CHECKPOINT) and
 * recomputing in between; 1 keeps every state (up to 192 a ray, 48 bytes each) and recomputes nothing.  `count` views (params[0 .. count - 1]) of one size, one ray at each pixel's
 * centre, in one launch.  The rings' orbit speed and glow come from their formulas; the map's other
 * tables (gas, dust, sky, colours) and the fluid are shared by the views: device pointers (NULL: the
 * context's).  targets: device, count * width * height float4 (linear RGB, the fourth unused).  hdr:
 * device, the same size, or NULL: the radiance the adjoint's forward pass found.  pixelGrads: device,
 * count * width * height * 5 floats, or NULL: each pixel's share of its view's gradient.  results: host,
 * count entries.  stats: rays, steps, crossings, escapes of the forward pass, and the launch's device
 * time.  Synchronous. */
int artfCudaHoleAdjoint(ArtfCuda* ctx, const ArtfCudaHoleParams* params, int count, int width, int height,
                        const float* map, const float* fluid, const float* targets, int checkpointEvery, float* hdr,
                        float* pixelGrads, ArtfCudaAdjointResult* results, ArtfCudaTraceStats* stats);

/* ---- the reference's painted disc, made on the GPU (src/scene/hole.c:136-197) ----------------------- */

/* buildDisc then setRings: the map Artful draws a hole with (gas strands and clouds, dust lanes, the
 * sky's dust band, black-body colours, the rings' tables for a disc from inner to outer around a hole of
 * this spin), byte for byte the reference's, into a device map of ARTF_CUDA_MAP_FLOATS (NULL: the
 * context's, which the trace then reads).  The reference paints it on the CPU at start-up.  Synchronous. */
int artfCudaPaintDisc(ArtfCuda* ctx, float* map, float inner, float outer, float spin);

/* ---- the disc's gas, stepped on the GPU (src/scene/fluid.c) --------------------------------------- */

/* The reference steps the disc's fluid on the CPU every frame and uploads its 1 MB field; this one lives
 * on the context's device, where the trace reads it, and its bytes equal the reference's (fluid.c is
 * deterministic: + - * / and comparisons in a fixed order). */
typedef struct ArtfCudaFluid ArtfCudaFluid;
/* fluid.c:255 artfFluidNew: the gas of a disc from inner to outer around a hole of this spin, as of
 * `time` (its start: 200 eddies and 60 steps).  Synchronous. */
int artfCudaFluidNew(ArtfCuda* ctx, float inner, float outer, float spin, double time, ArtfCudaFluid** out);
/* fluid.c:319 artfFluidAdvance: steps of 0.2 up to `time`, at most 48 a call (the gas does not run back);
 * *stepped (may be NULL): whether the field changed.  On the context's stream. */
int artfCudaFluidAdvance(ArtfCudaFluid* f, double time, int* stepped);
/* The clock of fluid.c:319-333 alone, on the host: how many steps artfFluidAdvance takes from a gas whose
 * time is *clock towards `time`, with *clock moved to the gas's time after them (a step adds 0.2f).  The
 * field after any run of advances depends only on the steps taken since its start, so a caller that
 * counts them can bring a gas up to date later in one call (artfCudaFluidStep). */
int artfCudaFluidClock(double* clock, double time);
/* `steps` steps now (any number), the field after them, and the gas's time set to `time`.  On the
 * context's stream. */
int artfCudaFluidStep(ArtfCudaFluid* f, int64_t steps, double time);
/* The field copied into the context's fluid (on the device, on its stream), which traces and draws with
 * no fluid given then read.  f must be of this context. */
int artfCudaUseFluid(ArtfCuda* ctx, const ArtfCudaFluid* f);
/* fluid.c:335-336: the field (device, ARTF_CUDA_FLUID_FLOATS, owned by f; valid after the stream's work)
 * and the moment it is of. */
const float* artfCudaFluidField(const ArtfCudaFluid* f);
double artfCudaFluidTime(const ArtfCudaFluid* f);
/* The field copied to host memory.  Synchronous. */
int artfCudaFluidRead(const ArtfCudaFluid* f, float* host);
/* fluid.c:243 */
void artfCudaFluidFree(ArtfCudaFluid* f);

/* ---- measurement ------------------------------------------------------------------------------- */

/* The device's FP32 and FP64 fused multiply-add throughput, measured (flop/s, a multiply-add two):
 * the denominators of the trace's roofline.  No reference counterpart.  stream: a cudaStream_t or NULL. */
int artfCudaProbePeaks(void* stream, int device, double* fp32Flops, double* fp64Flops);
/* The mixed trace converts between float and double with integer instructions (the FP64 pipe that bounds
 * it does the hardware's conversions slowly); this checks those against the hardware's conversions:
 * float to double on every float, double to float on narrowCount doubles around float's range and its
 * rounding ties.  mismatches[0], [1]: differing results of each (two NaNs agree); [2], [3]: the least
 * differing input's bits (all ones: none).  Synchronous on `stream` (a cudaStream_t or NULL). */
int artfCudaCheckConversions(void* stream, uint64_t narrowCount, uint64_t* mismatches);
/* The mixed trace's wide sub-steps compute with double-float pairs (hi + lo, about 48 bits) on the FP32
 * pipe; this runs that arithmetic on `count` records of hostIn (a.hi, a.lo, b.hi, b.lo: host, 4 floats
 * a record) into hostOut (host, 8 floats a record: a + b, a b, 1 / a and 1 / sqrt(|a|), each hi, lo), for
 * a test to compare with exact arithmetic.  Synchronous on `stream` (a cudaStream_t or NULL). */
int artfCudaCheckPairs(void* stream, const float* hostIn, int count, float* hostOut);

#ifdef __cplusplus
}
#endif

#endif
