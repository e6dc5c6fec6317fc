/* artful_cuda — the C ABI's device side: contexts, uploads, the trace dispatch, batches of views, their
 * CUDA graphs and the autotuner.  Every entry point checks its arguments and every CUDA call, and
 * reports failure by status, never by abort. */
#include "nvtxRange.h"
#include "artful_cuda.h"
#include "lensFlops.h"
#include "lensLaunch.h"
#include "lensMixed.h"
#include "lensTangent.h"

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static thread_local char lastError[256];

static int fail(int status, const char* format, ...) {
    va_list args;
    va_start(args, format);
    vsnprintf(lastError, sizeof lastError, format, args);
    va_end(args);
    return status;
}

#define CUDA_OR(status, call)                                                                       \
    do {                                                                                            \
        const cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(status, "%s: %s", #call, cudaGetErrorString(e_));        \
    } while (0)

extern "C" const char* artfCudaLastError(void) { return lastError; }

struct ArtfCuda {
    int device;
    int smCount;
    cudaStream_t stream;
    cudaEvent_t start, stop;
    float* map;
    float* fluid;
    uint64_t mapVersion, fluidVersion;
    bool mapHeld, fluidHeld;
    unsigned long long* counters; /* artf::CCount */
    float4* hdr;                  /* the host path's frame buffer */
    size_t hdrPixels;
    uint32_t* bgra;               /* the draw path's tone-mapped frame */
    size_t bgraPixels;
    size_t drawnPixels;           /* the last artfCudaHoleDraw's frame size (its light in hdr, its BGRA in
                                   * bgra), for artfCudaFrameRead; 0: none since */
    float* bloom;                 /* three planes of bloomPixels floats */
    size_t bloomPixels;
    /* the mixed trace's view table: device copy, pinned staging, and when the staging was last read */
    void* table;
    void* stage;
    size_t tableBytes;
    cudaEvent_t staged;
    bool stagedPending;
    ArtfCudaTuning tuned;
    bool hasTuning;
    /* the mixed trace's ray planes (one float4 a ray of a pixel), for views of several rays a pixel */
    float4* planes;
    size_t planeCount;
    /* the mixed trace's heavy-first order (artf::mixedOrderBytes) */
    void* order;
    size_t orderBytes;
    /* the adjoint's view table (device and pinned staging), block sums and per-view results */
    void* adjTable;
    void* adjStage;
    size_t adjViews;
    float* adjPartials;
    size_t adjPartialCount;
    double* adjResults;
    double* adjResultsHost;
    size_t adjResultViews;
    void* adjOrder;               /* the adjoint's heavy-first tile order (artf::adjointOrderBytes) */
    size_t adjOrderBytes;
    void* adjTrail;               /* the rays' kept states between the adjoint's kernels (artf::adjointTrailBytes) */
    size_t adjTrailBytes;
    uint32_t lastBands; /* launches of the last trace (1 but for a frame in bands) */
    int launchesLeft; /* host-side fault injection: launches before the context reports loss; -1 off */
    int allocsLeft;   /* host-side fault injection: allocations before the next one fails; -1 off */
    bool lost;
};

/* Makes the context's device current for this thread. */
static int enter(ArtfCuda* ctx) {
    if (!ctx) return fail(ARTF_CUDA_EINVAL, "no context");
    if (ctx->lost) return fail(ARTF_CUDA_ELOST, "the context was lost; destroy it and make another");
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaSetDevice(ctx->device));
    return ARTF_CUDA_OK;
}

/* Counts a launch against the injected-fault budget: when it runs out the context is lost, as a device
 * loss would leave it, without the GPU being touched. */
static int spendLaunch(ArtfCuda* ctx) {
    if (ctx->launchesLeft < 0) return ARTF_CUDA_OK;
    if (ctx->launchesLeft == 0) {
        ctx->lost = true;
        return fail(ARTF_CUDA_ELOST, "device loss injected on the host (artfCudaFailAfter)");
    }
    --ctx->launchesLeft;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaFailAfter(ArtfCuda* ctx, int launches) {
    if (!ctx) return fail(ARTF_CUDA_EINVAL, "no context");
    ctx->launchesLeft = launches < 0 ? -1 : launches;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaFailAllocAfter(ArtfCuda* ctx, int allocations) {
    if (!ctx) return fail(ARTF_CUDA_EINVAL, "no context");
    ctx->allocsLeft = allocations < 0 ? -1 : allocations;
    return ARTF_CUDA_OK;
}

/* A context's device or page-locked allocation, counted against the injected-failure budget: when it has
 * run out the allocation fails as an exhausted device's would, without the driver being asked. */
static cudaError_t ctxAlloc(ArtfCuda* ctx, void** p, size_t bytes, bool pageLocked = false) {
    if (ctx->allocsLeft == 0) return cudaErrorMemoryAllocation;
    if (ctx->allocsLeft > 0) --ctx->allocsLeft;
    const cudaError_t e = pageLocked ? cudaMallocHost(p, bytes) : cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        /* An allocation's failure is not sticky, but it stays the runtime's last error: cleared here, or
         * the next launch's check would report it. */
        (void)cudaGetLastError();
        *p = nullptr;
    }
    return e;
}

extern "C" int artfCudaCreate(int device, ArtfCuda** out) {
    if (!out) return fail(ARTF_CUDA_EINVAL, "out is NULL");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(ARTF_CUDA_ENODEVICE, "no CUDA device");
    if (device < 0 || device >= count) return fail(ARTF_CUDA_ENODEVICE, "device %d of %d", device, count);
    cudaDeviceProp prop;
    CUDA_OR(ARTF_CUDA_ENODEVICE, cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(ARTF_CUDA_ENODEVICE, "device %d is sm_%d%d; this library is built for sm_103a", device, prop.major,
                    prop.minor);
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaSetDevice(device));
    ArtfCuda* ctx = (ArtfCuda*)calloc(1, sizeof(ArtfCuda));
    if (!ctx) return fail(ARTF_CUDA_ENOMEM, "host allocation");
    ctx->device = device;
    ctx->smCount = prop.multiProcessorCount;
    ctx->launchesLeft = -1;
    ctx->allocsLeft = -1;
    int status = ARTF_CUDA_OK;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->start) != cudaSuccess || cudaEventCreate(&ctx->stop) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->staged, cudaEventDisableTiming) != cudaSuccess)
        status = fail(ARTF_CUDA_ELAUNCH, "stream or event creation failed");
    if (!status && (cudaMalloc(&ctx->map, sizeof(float) * ARTF_CUDA_MAP_FLOATS) != cudaSuccess ||
                    cudaMalloc(&ctx->fluid, sizeof(float) * ARTF_CUDA_FLUID_FLOATS) != cudaSuccess ||
                    cudaMalloc(&ctx->counters, sizeof(unsigned long long) * artf::CCount) != cudaSuccess))
        status = fail(ARTF_CUDA_ENOMEM, "device allocation of the map, fluid or counters failed");
    if (status) {
        artfCudaDestroy(ctx);
        return status;
    }
    *out = ctx;
    return ARTF_CUDA_OK;
}

extern "C" void artfCudaDestroy(ArtfCuda* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->map);
    cudaFree(ctx->fluid);
    cudaFree(ctx->counters);
    cudaFree(ctx->hdr);
    cudaFree(ctx->bgra);
    cudaFree(ctx->bloom);
    cudaFree(ctx->table);
    cudaFreeHost(ctx->stage);
    cudaFree(ctx->planes);
    cudaFree(ctx->order);
    cudaFree(ctx->adjTable);
    cudaFreeHost(ctx->adjStage);
    cudaFree(ctx->adjPartials);
    cudaFree(ctx->adjResults);
    cudaFreeHost(ctx->adjResultsHost);
    cudaFree(ctx->adjOrder);
    cudaFree(ctx->adjTrail);
    if (ctx->start) cudaEventDestroy(ctx->start);
    if (ctx->stop) cudaEventDestroy(ctx->stop);
    if (ctx->staged) cudaEventDestroy(ctx->staged);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    free(ctx);
}

static int upload(ArtfCuda* ctx, float* dst, const float* src, size_t floats, uint64_t version, uint64_t* held,
                  bool* isHeld) {
    if (!src) return fail(ARTF_CUDA_EINVAL, "host buffer is NULL");
    if (*isHeld && version != 0 && version == *held) return ARTF_CUDA_OK;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(dst, src, sizeof(float) * floats, cudaMemcpyHostToDevice, ctx->stream));
    *held = version;
    *isHeld = true;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaSetMap(ArtfCuda* ctx, const float* hostMap, uint64_t version) {
    int status = enter(ctx);
    if (status) return status;
    return upload(ctx, ctx->map, hostMap, ARTF_CUDA_MAP_FLOATS, version, &ctx->mapVersion, &ctx->mapHeld);
}

extern "C" int artfCudaSetFluid(ArtfCuda* ctx, const float* hostFluid, uint64_t version) {
    int status = enter(ctx);
    if (status) return status;
    return upload(ctx, ctx->fluid, hostFluid, ARTF_CUDA_FLUID_FLOATS, version, &ctx->fluidVersion, &ctx->fluidHeld);
}

/* A host map and fluid for a draw, each copied when its version changed; NULL: the context's own. */
static int hostInputs(ArtfCuda* ctx, const float* hostMap, uint64_t mapVersion, const float* hostFluid,
                      uint64_t fluidVersion) {
    if (!hostMap && !ctx->mapHeld) return fail(ARTF_CUDA_EINVAL, "no map: pass one or paint the context's");
    if (!hostFluid && !ctx->fluidHeld) return fail(ARTF_CUDA_EINVAL, "no fluid: pass one or give the context one");
    if (hostMap)
        if (int s = upload(ctx, ctx->map, hostMap, ARTF_CUDA_MAP_FLOATS, mapVersion, &ctx->mapVersion, &ctx->mapHeld))
            return s;
    if (hostFluid)
        if (int s = upload(ctx, ctx->fluid, hostFluid, ARTF_CUDA_FLUID_FLOATS, fluidVersion, &ctx->fluidVersion,
                           &ctx->fluidHeld))
            return s;
    return ARTF_CUDA_OK;
}

extern "C" const float* artfCudaDeviceMap(const ArtfCuda* ctx) { return ctx ? ctx->map : nullptr; }
extern "C" const float* artfCudaDeviceFluid(const ArtfCuda* ctx) { return ctx ? ctx->fluid : nullptr; }
extern "C" void* artfCudaStream(const ArtfCuda* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

/* The double frame from the float one, where the caller gave none. */
static void promoteFrame(const ArtfCudaHoleFrame* f, ArtfCudaHoleFrame64* d) {
    const float* src[] = {f->er, f->etheta, f->ephi, f->right, f->up, f->forward, f->metric,
                          f->place, f->spin, f->flow, f->boost, f->disc, f->look, f->image};
    double* dst[] = {d->er, d->etheta, d->ephi, d->right, d->up, d->forward, d->metric,
                     d->place, d->spin, d->flow, d->boost, d->disc, d->look, d->image};
    for (int i = 0; i < 14; ++i)
        for (int c = 0; c < 4; ++c) dst[i][c] = src[i][c];
}

static int checkOptions(const ArtfCudaTraceOptions* o) {
    if (!o) return fail(ARTF_CUDA_EINVAL, "options is NULL");
    if (o->jitter < 0 || o->jitter > 256) return fail(ARTF_CUDA_EINVAL, "jitter %d out of 0..256", o->jitter);
    if (o->precision < ARTF_CUDA_EXACT || o->precision > ARTF_CUDA_MIXED)
        return fail(ARTF_CUDA_EINVAL, "unknown precision %d", o->precision);
    if (o->stepScale < 0.f || o->stepScale > 1.f) return fail(ARTF_CUDA_EINVAL, "stepScale out of [0, 1]");
    if (o->guards > ARTF_CUDA_GUARD_ALL) return fail(ARTF_CUDA_EINVAL, "unknown guard bits %#x", o->guards);
    if (o->fp64Batch < 0 || o->fp64Batch > 32) return fail(ARTF_CUDA_EINVAL, "fp64Batch out of 0..32");
    if (o->refillBatch < 0 || o->refillBatch > 32) return fail(ARTF_CUDA_EINVAL, "refillBatch out of 0..32");
    if (o->blockSize != 0 && (o->blockSize < 32 || o->blockSize > 256 || o->blockSize % 32))
        return fail(ARTF_CUDA_EINVAL, "blockSize %d: 0, or a multiple of 32 up to 256", o->blockSize);
    if (o->compactEvery < 0 || o->compactEvery > 4096) return fail(ARTF_CUDA_EINVAL, "compactEvery out of range");
    if (o->horizonBand < 0.f || o->horizonBand > 1.f) return fail(ARTF_CUDA_EINVAL, "horizonBand out of [0, 1]");
    if (o->order != ARTF_CUDA_ORDER_HEAVY_FIRST && o->order != ARTF_CUDA_ORDER_PIXELS)
        return fail(ARTF_CUDA_EINVAL, "unknown order %d", o->order);
    return ARTF_CUDA_OK;
}

static int checkFrame(const ArtfCudaHoleFrame* f, const ArtfCudaTraceOptions* o) {
    if (!f) return fail(ARTF_CUDA_EINVAL, "frame is NULL");
    if (int s = checkOptions(o)) return s;
    if (f->size[0] < 1 || f->size[1] < 1 || f->size[0] > 32768 || f->size[1] > 32768)
        return fail(ARTF_CUDA_EINVAL, "frame size %u x %u out of range", f->size[0], f->size[1]);
    if (!o->jitter && (f->size[2] < 1 || f->size[2] > 8))
        return fail(ARTF_CUDA_EINVAL, "rays a side %u out of 1..8", f->size[2]);
    return ARTF_CUDA_OK;
}

/* The launch options of a trace, with the context's tuning where the caller left a value at 0. */
static artf::TraceLaunch launchOf(const ArtfCuda* ctx, const ArtfCudaTraceOptions* o) {
    artf::TraceLaunch l;
    memset(&l, 0, sizeof l);
    l.jitter = o->jitter;
    l.seed = o->seed;
    l.stepScale = o->stepScale > 0.f ? o->stepScale : 1.f;
    l.horizonBand = o->horizonBand;
    l.blockSize = o->blockSize;
    l.compactEvery = o->compactEvery;
    l.persistent = o->persistent;
    l.guards = o->guards;
    l.fp64Batch = o->fp64Batch;
    l.refillBatch = o->refillBatch;
    l.order = o->order;
    if (ctx->hasTuning && o->precision == ARTF_CUDA_MIXED) {
        if (!l.blockSize) l.blockSize = ctx->tuned.blockSize;
        if (!l.compactEvery) l.compactEvery = ctx->tuned.compactEvery;
        if (!l.fp64Batch) l.fp64Batch = ctx->tuned.fp64Batch;
        if (!l.refillBatch) l.refillBatch = ctx->tuned.refillBatch;
    }
    l.counters = ctx->counters;
    l.smCount = ctx->smCount;
    l.stream = ctx->stream;
    return l;
}

/* Room for `count` views in the context's table and its staging. */
static int reserveTable(ArtfCuda* ctx, int count) {
    const size_t bytes = artf::mixedViewBytes() * (size_t)count;
    if (bytes <= ctx->tableBytes) return ARTF_CUDA_OK;
    if (ctx->stagedPending) CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventSynchronize(ctx->staged));
    ctx->stagedPending = false;
    cudaFree(ctx->table);
    cudaFreeHost(ctx->stage);
    ctx->table = ctx->stage = nullptr;
    ctx->tableBytes = 0;
    CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, &ctx->table, bytes));
    CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, &ctx->stage, bytes, true));
    ctx->tableBytes = bytes;
    return ARTF_CUDA_OK;
}

/* The ray planes a batch of views needs (float4 each). */
static size_t planesOf(const artf::TraceLaunch& l, const ArtfCudaView* views, int count) {
    size_t total = 0;
    for (int i = 0; i < count; ++i)
        total += (size_t)views[i].frame.size[0] * views[i].frame.size[1] * artf::mixedRayPlanes(l, views[i].frame);
    return total;
}

/* Room for `count` float4 of ray planes in the context. */
static int reservePlanes(ArtfCuda* ctx, size_t count) {
    if (count <= ctx->planeCount) return ARTF_CUDA_OK;
    cudaFree(ctx->planes); /* (synchronises: no launch still writes the old planes) */
    ctx->planes = nullptr;
    ctx->planeCount = 0;
    CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, (void**)&ctx->planes, sizeof(float4) * count));
    ctx->planeCount = count;
    return ARTF_CUDA_OK;
}

/* The heavy-first order's scratch for this many tiles and units. */
static int reserveOrder(ArtfCuda* ctx, int tiles, int units) {
    const size_t bytes = artf::mixedOrderBytes(tiles, units);
    if (bytes <= ctx->orderBytes) return ARTF_CUDA_OK;
    cudaFree(ctx->order); /* (synchronises: no launch still reads the old order) */
    ctx->order = nullptr;
    ctx->orderBytes = 0;
    CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, &ctx->order, bytes));
    ctx->orderBytes = bytes;
    return ARTF_CUDA_OK;
}

/* Fills the staging table from views; the total queue units in *units and tiles in *tiles.  planes: room
 * for the views' ray planes (planesOf), or NULL to trace a pixel a unit; *combinePixels: the largest view
 * with planes. */
static int fillTable(ArtfCuda* ctx, const artf::TraceLaunch& l, const ArtfCudaView* views, int count,
                     const ArtfCudaTraceOptions* o, void* stage, float4* planes, int* units, size_t* combinePixels,
                     int* tiles) {
    long long total = 0, tileTotal = 0;
    size_t offset = 0, widest = 0;
    for (int i = 0; i < count; ++i) {
        const ArtfCudaView& v = views[i];
        if (int s = checkFrame(&v.frame, o)) return s;
        if (!v.hdr) return fail(ARTF_CUDA_EINVAL, "view %d: hdr is NULL", i);
        if ((!v.map && !ctx->mapHeld) || (!v.fluid && !ctx->fluidHeld))
            return fail(ARTF_CUDA_EINVAL, "view %d: no map or fluid, and none set on the context", i);
        const size_t pixels = (size_t)v.frame.size[0] * v.frame.size[1], np = artf::mixedRayPlanes(l, v.frame);
        float4* rayOut = planes && np ? planes + offset : nullptr;
        if (rayOut) {
            offset += pixels * np;
            widest = pixels > widest ? pixels : widest;
        }
        int viewTiles = 0;
        const int n = artf::mixedFillView(l, v.frame, v.frame64, v.map ? v.map : ctx->map, v.fluid ? v.fluid : ctx->fluid,
                                (float4*)v.hdr, v.ends, rayOut, (int)total, (int)tileTotal,
                                (char*)stage + artf::mixedViewBytes() * i, &viewTiles);
        total += n;
        tileTotal += viewTiles;
        if (total > 0x7FFFFFFFLL) return fail(ARTF_CUDA_EINVAL, "batch of %lld rays is too large", total);
    }
    *units = (int)total;
    *tiles = (int)tileTotal;
    *combinePixels = widest;
    return ARTF_CUDA_OK;
}

/* Copies the staged table to the device, after the previous copy has read the staging. */
static int sendTable(ArtfCuda* ctx, int count) {
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(ctx->table, ctx->stage, artf::mixedViewBytes() * (size_t)count,
                                               cudaMemcpyHostToDevice, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->staged, ctx->stream));
    ctx->stagedPending = true;
    return ARTF_CUDA_OK;
}

static int waitStaging(ArtfCuda* ctx) {
    if (ctx->stagedPending) CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventSynchronize(ctx->staged));
    ctx->stagedPending = false;
    return ARTF_CUDA_OK;
}

static int readStats(ArtfCuda* ctx, const ArtfCudaHoleFrame& frame, int precision, uint32_t guards,
                     ArtfCudaTraceStats* stats) {
    unsigned long long c[artf::CCount];
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(c, ctx->counters, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventElapsedTime(&ms, ctx->start, ctx->stop));
    stats->rays = c[artf::CRays];
    stats->steps = c[artf::CSteps];
    stats->crossings = c[artf::CCrossings];
    stats->escapes = c[artf::CEscapes];
    stats->fp64Steps = precision == ARTF_CUDA_FP64 ? c[artf::CSteps] : c[artf::CFp64Steps];
    stats->fp64Horizon = c[artf::CFp64Horizon];
    stats->fp64Radial = c[artf::CFp64Radial];
    stats->fp64Polar = c[artf::CFp64Polar];
    stats->fp64Rounds = c[artf::CFp64Rounds];
    stats->flops = artfFlops(stats->rays, stats->steps, stats->crossings, stats->escapes, frame.spin[0] != 0.f,
                             frame.look[1] != 0.f, frame.look[2] > 0.f);
    if (precision == ARTF_CUDA_FP64) {
        stats->flops64 = stats->flops;
    } else if (precision == ARTF_CUDA_MIXED) {
        const bool motion = (guards ? guards : ARTF_CUDA_GUARD_ALL) & ARTF_CUDA_GUARD_MOTION;
        stats->flops64 = artfFlops64(motion ? stats->rays : 0, stats->fp64Horizon, stats->fp64Radial,
                                     stats->fp64Polar, frame.spin[0] != 0.f);
    } else {
        stats->flops64 = 0.0;
    }
    stats->ms = ms;
    stats->bands = ctx->lastBands;
    return ARTF_CUDA_OK;
}

/* The debug build's fault word, read after a trace (ARTF_CUDA_DEBUG_BOUNDS: lensCore.cuh). */
static int checkBounds(ArtfCuda* ctx) {
#if defined(ARTF_CUDA_DEBUG_BOUNDS)
    static const char* const kinds[] = {"", "gas row", "fluid row", "dust row", "sky row", "ring row",
                                        "colour", "pixel", "ray plane", "ray end"};
    unsigned long long w[2];
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(w, ctx->counters + artf::CBoundsKind, sizeof w, cudaMemcpyDeviceToHost,
                                               ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    if (w[0])
        return fail(ARTF_CUDA_EBOUNDS, "%s index %lld outside its table or frame",
                    w[0] < sizeof kinds / sizeof kinds[0] ? kinds[w[0]] : "unknown", (long long)w[1]);
#else
    (void)ctx;
#endif
    return ARTF_CUDA_OK;
}

/* Frames that go out in bands (vulkan.c:1733-1734): above this many rays, bands of that many. */
static const int64_t kRaysApart = 64000000, kRaysABand = 8000000;

/* One launch of the frame's tile rows l.tileRowBegin .. + l.tileRows (all when 0 rows), or of its ray
 * list, in the given precision. */
static int launchBand(ArtfCuda* ctx, artf::TraceLaunch& l, int precision) {
    if (precision == ARTF_CUDA_MIXED) {
        if (int s = reserveTable(ctx, 1)) return s;
        const int height = (int)l.frame.size[1];
        const int rowBegin = l.tileRows > 0 ? l.tileRowBegin * 4 : 0;
        const int rows = l.tileRows > 0 ? (rowBegin + l.tileRows * 4 < height ? l.tileRows * 4 : height - rowBegin)
                                        : height;
        const size_t pixels = (size_t)l.frame.size[0] * rows;
        const size_t np = l.rayCount > 0 ? 0 : artf::mixedRayPlanes(l, l.frame);
        if (np)
            if (int s = reservePlanes(ctx, pixels * np)) return s;
        if (int s = waitStaging(ctx)) return s;
        int tiles = 0;
        const int units = artf::mixedFillView(l, l.frame, l.frame64, l.map, l.fluid, l.hdr, l.ends,
                                              np ? ctx->planes : nullptr, 0, 0, ctx->stage, &tiles);
        if (int s = reserveOrder(ctx, tiles, units)) return s;
        if (int s = sendTable(ctx, 1)) return s;
        const cudaError_t e = artf::launchMixedTable(l, ctx->table, 1, units, np ? pixels : 0, tiles, ctx->order,
                                                     ctx->stage);
        if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "mixed trace launch: %s", cudaGetErrorString(e));
        return ARTF_CUDA_OK;
    }
    cudaError_t e = cudaSuccess;
    switch (precision) {
    case ARTF_CUDA_EXACT: e = artf::launchExact(l); break;
    case ARTF_CUDA_FP32: e = artf::launchFast(l); break;
    default: e = artf::launchFp64(l); break;
    }
    if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "trace launch: %s", cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}

/* One frame (or ray list) of any precision: its launches (a band of whole tile rows each, waited for,
 * when the frame has more rays than bandRays allows: ArtfCudaTraceOptions), bracketed by events, and
 * the stats.  Every pixel's rays are traced within one band, so the bands change when, not what. */
static int runTrace(ArtfCuda* ctx, artf::TraceLaunch& l, int precision, int64_t bandRays, ArtfCudaTraceStats* stats) {
    if (int s = spendLaunch(ctx)) return s;
    const int tileRows = ((int)l.frame.size[1] + 3) / 4;
    const int64_t perPixel = l.jitter ? l.jitter : (int64_t)l.frame.size[2] * l.frame.size[2];
    const int64_t total = (int64_t)l.frame.size[0] * l.frame.size[1] * perPixel;
    const int64_t perTileRow = (int64_t)l.frame.size[0] * 4 * perPixel;
    int64_t band = 0;
    if (l.rayCount == 0 && bandRays == 0 && total > kRaysApart) band = kRaysABand;
    if (l.rayCount == 0 && bandRays > 0 && total > bandRays) band = bandRays;
    const int rowsABand = band > 0 ? (int)(band / perTileRow > 1 ? band / perTileRow : 1) : tileRows;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
    int bands = 0, status = ARTF_CUDA_OK;
    for (int first = 0; first < tileRows && !status; first += rowsABand) {
        if (band > 0) {
            l.tileRowBegin = first;
            l.tileRows = rowsABand < tileRows - first ? rowsABand : tileRows - first;
            if (bands > 0) { /* each band its own launch, waited for (vulkan.c:1740-1754) */
                CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
                CUDA_OR(ARTF_CUDA_ELAUNCH,
                        cudaMemsetAsync(ctx->counters + artf::CQueue, 0, sizeof(unsigned long long), ctx->stream));
            }
        }
        status = launchBand(ctx, l, precision);
        ++bands;
        if (l.rayCount > 0) break;
    }
    l.tileRowBegin = l.tileRows = 0;
    if (status) return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    ctx->lastBands = (uint32_t)bands;
    if ((status = checkBounds(ctx))) return status;
    return stats ? readStats(ctx, l.frame, precision, l.guards, stats) : ARTF_CUDA_OK;
}

extern "C" int artfCudaHoleTraceRays(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                     const float* map, const float* fluid, int precision, float stepScale, int n,
                                     const float* nx, const float* ny, const float* time, float* rgb,
                                     ArtfCudaRayEnd* ends, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleTraceRays");
    int status = enter(ctx);
    if (status) return status;
    ArtfCudaTraceOptions o;
    memset(&o, 0, sizeof o);
    o.precision = precision;
    o.stepScale = stepScale;
    o.jitter = 1; /* (the frame's samples are not read) */
    if ((status = checkFrame(frame, &o))) return status;
    if (n < 1 || !nx || !ny || !time || !rgb) return fail(ARTF_CUDA_EINVAL, "ray list: n %d or a NULL array", n);
    if (!map && !ctx->mapHeld) return fail(ARTF_CUDA_EINVAL, "no map: pass one or call artfCudaSetMap");
    if (!fluid && !ctx->fluidHeld) return fail(ARTF_CUDA_EINVAL, "no fluid: pass one or call artfCudaSetFluid");
    artf::TraceLaunch l = launchOf(ctx, &o);
    l.frame = *frame;
    if (frame64) l.frame64 = *frame64;
    else promoteFrame(frame, &l.frame64);
    l.map = map ? map : ctx->map;
    l.fluid = fluid ? fluid : ctx->fluid;
    l.ends = ends;
    l.jitter = 0;
    l.rayCount = n;
    l.rayX = nx, l.rayY = ny, l.rayTime = time, l.rayRgb = rgb;
    return runTrace(ctx, l, precision, -1, stats);
}

extern "C" int artfCudaHoleTrace(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                 const float* map, const float* fluid, const ArtfCudaTraceOptions* options, float* hdr,
                                 ArtfCudaRayEnd* ends, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleTrace");
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkFrame(frame, options))) return status;
    if (!hdr) return fail(ARTF_CUDA_EINVAL, "hdr is NULL");
    if (!map && !ctx->mapHeld) return fail(ARTF_CUDA_EINVAL, "no map: pass one or call artfCudaSetMap");
    if (!fluid && !ctx->fluidHeld) return fail(ARTF_CUDA_EINVAL, "no fluid: pass one or call artfCudaSetFluid");
    artf::TraceLaunch l = launchOf(ctx, options);
    l.frame = *frame;
    if (frame64) l.frame64 = *frame64;
    else promoteFrame(frame, &l.frame64);
    l.map = map ? map : ctx->map;
    l.fluid = fluid ? fluid : ctx->fluid;
    l.hdr = (float4*)hdr;
    l.ends = ends;
    return runTrace(ctx, l, options->precision, options->bandRays, stats);
}

extern "C" int artfCudaHoleRender(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                  const float* hostMap, uint64_t mapVersion, const float* hostFluid,
                                  uint64_t fluidVersion, const ArtfCudaTraceOptions* options, float* hostHdr,
                                  ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleRender");
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkFrame(frame, options))) return status;
    if (!hostHdr) return fail(ARTF_CUDA_EINVAL, "hostHdr is NULL");
    ctx->drawnPixels = 0; /* (the light buffer is this path's from here on) */
    if ((status = hostInputs(ctx, hostMap, mapVersion, hostFluid, fluidVersion))) return status;
    const size_t pixels = (size_t)frame->size[0] * frame->size[1];
    /* A page-locked host buffer, which the device addresses, takes the frame straight from the trace's
     * kernels, over the link as they write it; any other buffer gets a copy of the device's frame. */
    cudaPointerAttributes where;
    if (cudaPointerGetAttributes(&where, hostHdr) == cudaSuccess && where.type == cudaMemoryTypeHost &&
        where.devicePointer) {
        if ((status = artfCudaHoleTrace(ctx, frame, frame64, nullptr, nullptr, options, (float*)where.devicePointer,
                                        nullptr, stats)))
            return status;
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
        return ARTF_CUDA_OK;
    }
    cudaGetLastError(); /* (a pointer the runtime does not know is no error to keep) */
    if (pixels > ctx->hdrPixels) {
        cudaFree(ctx->hdr);
        ctx->hdr = nullptr;
        ctx->hdrPixels = 0;
        CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, (void**)&ctx->hdr, sizeof(float4) * pixels));
        ctx->hdrPixels = pixels;
    }
    if ((status = artfCudaHoleTrace(ctx, frame, frame64, nullptr, nullptr, options, (float*)ctx->hdr, nullptr, stats)))
        return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH,
            cudaMemcpyAsync(hostHdr, ctx->hdr, sizeof(float4) * pixels, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    return ARTF_CUDA_OK;
}

/* Grows a device buffer to at least `count` elements of `size` bytes. */
static int reserve(ArtfCuda* ctx, void** buffer, size_t* held, size_t count, size_t size) {
    if (count <= *held) return ARTF_CUDA_OK;
    cudaFree(*buffer);
    *buffer = nullptr;
    *held = 0;
    CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, buffer, count * size));
    *held = count;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaHoleDraw(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                const float* hostMap, uint64_t mapVersion, const float* hostFluid,
                                uint64_t fluidVersion, const ArtfCudaTraceOptions* options, float* hostHdr,
                                uint32_t* hostBgra, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleDraw");
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkFrame(frame, options))) return status;
    ctx->drawnPixels = 0;
    if ((status = hostInputs(ctx, hostMap, mapVersion, hostFluid, fluidVersion))) return status;
    const size_t pixels = (size_t)frame->size[0] * frame->size[1];
    size_t bloomPixels = 0;
    for (uint32_t i = 0; i < frame->size[3] && i < ARTF_CUDA_BLOOM_LEVELS; ++i)
        bloomPixels += (size_t)frame->bloom[i][1] * frame->bloom[i][2];
    if (frame->size[3] < 1 || bloomPixels == 0) return fail(ARTF_CUDA_EINVAL, "the frame has no bloom levels");
    if ((status = reserve(ctx, (void**)&ctx->hdr, &ctx->hdrPixels, pixels, sizeof(float4)))) return status;
    if ((status = reserve(ctx, (void**)&ctx->bgra, &ctx->bgraPixels, pixels, sizeof(uint32_t)))) return status;
    if ((status = reserve(ctx, (void**)&ctx->bloom, &ctx->bloomPixels, bloomPixels * 3, sizeof(float)))) return status;
    artf::TraceLaunch l = launchOf(ctx, options);
    l.frame = *frame;
    if (frame64) l.frame64 = *frame64;
    else promoteFrame(frame, &l.frame64);
    l.map = ctx->map;
    l.fluid = ctx->fluid;
    l.hdr = ctx->hdr;
    /* trace (its own events), then the pyramid and tone map, timed from the trace's start */
    if ((status = runTrace(ctx, l, options->precision, options->bandRays, nullptr))) return status;
    float* planes[3] = {ctx->bloom, ctx->bloom + bloomPixels, ctx->bloom + 2 * bloomPixels};
    if ((status = artfCudaPostLaunch(frame, (const float*)ctx->hdr, planes, ctx->bgra, ctx->stream)))
        return fail(status, "bloom and tone map launch: %s", cudaGetErrorString(cudaGetLastError()));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    if (stats) {
        if ((status = readStats(ctx, *frame, options->precision, options->guards, stats))) return status;
    }
    if (hostHdr)
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(hostHdr, ctx->hdr, sizeof(float4) * pixels,
                                                   cudaMemcpyDeviceToHost, ctx->stream));
    if (hostBgra)
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(hostBgra, ctx->bgra, sizeof(uint32_t) * pixels,
                                                   cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    ctx->drawnPixels = pixels;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaFrameRead(ArtfCuda* ctx, float* hostHdr, uint32_t* hostBgra) {
    artf::Range range("artfCudaFrameRead");
    int status = enter(ctx);
    if (status) return status;
    if (!ctx->drawnPixels) return fail(ARTF_CUDA_EINVAL, "no frame drawn since the frame buffers last changed");
    if (hostHdr)
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(hostHdr, ctx->hdr, sizeof(float4) * ctx->drawnPixels,
                                                   cudaMemcpyDeviceToHost, ctx->stream));
    if (hostBgra)
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(hostBgra, ctx->bgra, sizeof(uint32_t) * ctx->drawnPixels,
                                                   cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaHoleTangents(ArtfCuda* ctx, const ArtfCudaHoleParams* params, const ArtfCudaHoleFrame* frame,
                                    const ArtfCudaHoleFrame64* frame64, const double* jacobian, const float* map,
                                    const float* fluid, double* out) {
    artf::Range range("artfCudaHoleTangents");
    int status = enter(ctx);
    if (status) return status;
    if (!params || !frame || !frame64 || !jacobian || !out) return fail(ARTF_CUDA_EINVAL, "a NULL argument");
    if (frame->size[0] < 1 || frame->size[1] < 1 || (size_t)frame->size[0] * frame->size[1] > (1u << 24))
        return fail(ARTF_CUDA_EINVAL, "frame size out of range for the forward-mode reference");
    if ((!map && !ctx->mapHeld) || (!fluid && !ctx->fluidHeld)) return fail(ARTF_CUDA_EINVAL, "no map or fluid");
    if ((status = spendLaunch(ctx))) return status;
    artf::TraceLaunch l;
    memset(&l, 0, sizeof l);
    l.frame = *frame;
    l.frame64 = *frame64;
    l.map = map ? map : ctx->map;
    l.fluid = fluid ? fluid : ctx->fluid;
    l.counters = ctx->counters;
    l.stream = ctx->stream;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
    const cudaError_t e = artf::launchTangents(l, jacobian, params->emissivity, out);
    if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "tangent launch: %s", cudaGetErrorString(e));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    return ARTF_CUDA_OK;
}

/* Grows the adjoint's table, staging, block sums and results to `count` views of `blocks` blocks. */
static int reserveAdjoint(ArtfCuda* ctx, int count, int blocks, int width, int height, int K) {
    if ((size_t)count > ctx->adjViews) {
        cudaFree(ctx->adjTable);
        cudaFreeHost(ctx->adjStage);
        ctx->adjTable = ctx->adjStage = nullptr;
        ctx->adjViews = 0;
        CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, &ctx->adjTable, artf::adjointViewBytes() * count));
        CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, &ctx->adjStage, artf::adjointViewBytes() * count, true));
        ctx->adjViews = (size_t)count;
    }
    if ((size_t)count > ctx->adjResultViews) {
        cudaFree(ctx->adjResults);
        cudaFreeHost(ctx->adjResultsHost);
        ctx->adjResults = ctx->adjResultsHost = nullptr;
        ctx->adjResultViews = 0;
        CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, (void**)&ctx->adjResults, sizeof(double) * 8 * count));
        CUDA_OR(ARTF_CUDA_ENOMEM, ctxAlloc(ctx, (void**)&ctx->adjResultsHost, sizeof(double) * 8 * count, true));
        ctx->adjResultViews = (size_t)count;
    }
    if (int s = reserve(ctx, (void**)&ctx->adjPartials, &ctx->adjPartialCount, (size_t)count * blocks * 8, sizeof(float)))
        return s;
    if (int s = reserve(ctx, &ctx->adjOrder, &ctx->adjOrderBytes, artf::adjointOrderBytes(count, width, height), 1))
        return s;
    return reserve(ctx, &ctx->adjTrail, &ctx->adjTrailBytes, artf::adjointTrailBytes(count, width, height, K), 1);
}

extern "C" int artfCudaHoleAdjoint(ArtfCuda* ctx, const ArtfCudaHoleParams* params, int count, int width, int height,
                                   const float* map, const float* fluid, const float* targets, int checkpointEvery,
                                   float* hdr, float* pixelGrads, ArtfCudaAdjointResult* results,
                                   ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleAdjoint");
    int status = enter(ctx);
    if (status) return status;
    if (!params || !targets || !results) return fail(ARTF_CUDA_EINVAL, "params, targets and results are required");
    if (count < 1 || count > ARTF_CUDA_ADJOINT_MAX_VIEWS)
        return fail(ARTF_CUDA_EINVAL, "%d views (1 .. %d)", count, ARTF_CUDA_ADJOINT_MAX_VIEWS);
    if (width < 1 || height < 1 || width > 16384 || height > 16384 || (size_t)width * height > (1u << 24))
        return fail(ARTF_CUDA_EINVAL, "size %d x %d out of range", width, height);
    if (checkpointEvery < ARTF_CUDA_ADJOINT_MIN_CHECKPOINT || checkpointEvery > ARTF_CUDA_ADJOINT_MAX_CHECKPOINT)
        return fail(ARTF_CUDA_EINVAL, "checkpoint interval %d (%d .. %d)", checkpointEvery,
                    ARTF_CUDA_ADJOINT_MIN_CHECKPOINT, ARTF_CUDA_ADJOINT_MAX_CHECKPOINT);
    if ((!map && !ctx->mapHeld) || (!fluid && !ctx->fluidHeld)) return fail(ARTF_CUDA_EINVAL, "no map or fluid");
    const int pixels = width * height, blocks = artf::adjointTiles(width, height);
    if ((status = reserveAdjoint(ctx, count, blocks, width, height, checkpointEvery))) return status;
    /* (the staging is free: every call ends synchronised) */
    const size_t slot = artf::adjointViewBytes();
    for (int v = 0; v < count; ++v) {
        ArtfCudaHoleFrame frame;
        double jacobian[ARTF_CUDA_GRAD_FIELDS * 5];
        if ((status = artfCudaHoleParamsFrames(params + v, width, height, &frame, nullptr, jacobian)))
            return fail(status, "view %d: parameters out of range", v);
        if (frame.boost[3] > 1.f) return fail(ARTF_CUDA_EINVAL, "view %d: a moving eye", v);
        artf::adjointFillView((char*)ctx->adjStage + slot * v, frame, jacobian, params[v].emissivity,
                              map ? map : ctx->map, fluid ? fluid : ctx->fluid, targets + (size_t)v * pixels * 4,
                              hdr ? hdr + (size_t)v * pixels * 4 : nullptr,
                              pixelGrads ? pixelGrads + (size_t)v * pixels * 5 : nullptr);
    }
    if ((status = spendLaunch(ctx))) return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH,
            cudaMemcpyAsync(ctx->adjTable, ctx->adjStage, slot * count, cudaMemcpyHostToDevice, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
    const cudaError_t e = artf::launchAdjoint(ctx->adjTable, count, width, height, checkpointEvery, ctx->counters,
                                              ctx->adjPartials, ctx->adjResults, ctx->stream, ctx->adjOrder,
                                              ctx->adjTrail);
    if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "adjoint launch: %s", cudaGetErrorString(e));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(ctx->adjResultsHost, ctx->adjResults, sizeof(double) * 8 * count,
                                               cudaMemcpyDeviceToHost, ctx->stream));
    unsigned long long c[artf::CCount];
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemcpyAsync(c, ctx->counters, sizeof c, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    for (int v = 0; v < count; ++v) {
        results[v].loss = ctx->adjResultsHost[v * 8];
        for (int q = 0; q < 5; ++q) results[v].grad[q] = ctx->adjResultsHost[v * 8 + 1 + q];
    }
    if (stats) {
        float ms = 0.f;
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventElapsedTime(&ms, ctx->start, ctx->stop));
        memset(stats, 0, sizeof *stats);
        stats->rays = c[artf::CRays];
        stats->steps = c[artf::CSteps];
        stats->crossings = c[artf::CCrossings];
        stats->escapes = c[artf::CEscapes];
        stats->ms = ms;
        stats->bands = 1;
    }
    return ARTF_CUDA_OK;
}

/* For the other C ABI units (noAlloc.cu): the same error line and argument checks. */
namespace artf {
int failWith(int status, const char* message) { return fail(status, "%s", message); }
/* For the other units that work on a context (fluid.cu): its device made current, and its stream. */
int contextStream(ArtfCuda* ctx, cudaStream_t* stream) {
    if (int s = enter(ctx)) return s;
    *stream = ctx->stream;
    return ARTF_CUDA_OK;
}
/* The context's map, about to be written on the device (disc.cu): held from now on, under version 0 so
 * that the next artfCudaSetMap copies whatever it is given. */
int contextMap(ArtfCuda* ctx, float** map) {
    if (int s = enter(ctx)) return s;
    *map = ctx->map;
    ctx->mapHeld = true;
    ctx->mapVersion = 0;
    return ARTF_CUDA_OK;
}
/* The same for the context's fluid (fluid.cu). */
int contextFluid(ArtfCuda* ctx, float** fluid) {
    if (int s = enter(ctx)) return s;
    *fluid = ctx->fluid;
    ctx->fluidHeld = true;
    ctx->fluidVersion = 0;
    return ARTF_CUDA_OK;
}
int checkTraceFrame(const ArtfCudaHoleFrame* frame, const ArtfCudaTraceOptions* options) {
    return checkFrame(frame, options);
}
}  // namespace artf

/* ---- batches ------------------------------------------------------------------------------------- */

static int checkBatch(const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options) {
    if (!views || count < 1 || count > ARTF_CUDA_MAX_VIEWS)
        return fail(ARTF_CUDA_EINVAL, "batch of %d views: 1..%d", count, ARTF_CUDA_MAX_VIEWS);
    if (int s = checkOptions(options)) return s;
    if (options->precision != ARTF_CUDA_MIXED)
        return fail(ARTF_CUDA_EINVAL, "batches trace in mixed precision (ARTF_CUDA_MIXED) only");
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaHoleBatch(ArtfCuda* ctx, const ArtfCudaView* views, int count,
                                 const ArtfCudaTraceOptions* options, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleBatch");
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkBatch(views, count, options))) return status;
    if ((status = spendLaunch(ctx))) return status;
    const artf::TraceLaunch l = launchOf(ctx, options);
    if ((status = reserveTable(ctx, count))) return status;
    if ((status = reservePlanes(ctx, planesOf(l, views, count)))) return status;
    if ((status = waitStaging(ctx))) return status;
    int units = 0, tiles = 0;
    size_t combine = 0;
    if ((status = fillTable(ctx, l, views, count, options, ctx->stage, ctx->planes, &units, &combine, &tiles)))
        return status;
    if ((status = reserveOrder(ctx, tiles, units))) return status;
    if ((status = sendTable(ctx, count))) return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
    const cudaError_t e = artf::launchMixedTable(l, ctx->table, count, units, combine, tiles, ctx->order,
                                                     count == 1 ? ctx->stage : nullptr);
    if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "batch launch: %s", cudaGetErrorString(e));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    ctx->lastBands = 1;
    if ((status = checkBounds(ctx))) return status;
    return stats ? readStats(ctx, views[0].frame, ARTF_CUDA_MIXED, l.guards, stats) : ARTF_CUDA_OK;
}

struct ArtfCudaGraph {
    ArtfCuda* ctx;
    int count, units, tiles;
    size_t combine;
    ArtfCudaTraceOptions options;
    ArtfCudaHoleFrame first; /* (for the stats' counting rule) */
    void* table;
    void* stage;
    float4* planes; /* the graph's own ray planes: its captured launches keep the pointer */
    size_t planeCount;
    void* order;    /* and its own heavy-first order */
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

extern "C" void artfCudaBatchGraphDestroy(ArtfCudaGraph* g) {
    if (!g) return;
    cudaSetDevice(g->ctx->device);
    cudaStreamSynchronize(g->ctx->stream);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->table);
    cudaFreeHost(g->stage);
    cudaFree(g->planes);
    cudaFree(g->order);
    free(g);
}

extern "C" int artfCudaBatchGraphCreate(ArtfCuda* ctx, const ArtfCudaView* views, int count,
                                        const ArtfCudaTraceOptions* options, ArtfCudaGraph** out) {
    artf::Range range("artfCudaBatchGraphCreate");
    int status = enter(ctx);
    if (status) return status;
    if (!out) return fail(ARTF_CUDA_EINVAL, "out is NULL");
    *out = nullptr;
    if ((status = checkBatch(views, count, options))) return status;
    ArtfCudaGraph* g = (ArtfCudaGraph*)calloc(1, sizeof(ArtfCudaGraph));
    if (!g) return fail(ARTF_CUDA_ENOMEM, "host allocation");
    g->ctx = ctx;
    g->count = count;
    g->options = *options;
    g->first = views[0].frame;
    const size_t bytes = artf::mixedViewBytes() * (size_t)count;
    const artf::TraceLaunch l = launchOf(ctx, options);
    const size_t planes = planesOf(l, views, count);
    g->planeCount = planes;
    if (ctxAlloc(ctx, &g->table, bytes) != cudaSuccess || ctxAlloc(ctx, &g->stage, bytes, true) != cudaSuccess ||
        (planes && ctxAlloc(ctx, (void**)&g->planes, sizeof(float4) * planes) != cudaSuccess)) {
        artfCudaBatchGraphDestroy(g);
        return fail(ARTF_CUDA_ENOMEM, "graph table allocation");
    }
    if ((status = fillTable(ctx, l, views, count, options, g->stage, g->planes, &g->units, &g->combine, &g->tiles))) {
        artfCudaBatchGraphDestroy(g);
        return status;
    }
    if (ctxAlloc(ctx, &g->order, artf::mixedOrderBytes(g->tiles, g->units)) != cudaSuccess) {
        artfCudaBatchGraphDestroy(g);
        return fail(ARTF_CUDA_ENOMEM, "graph order allocation");
    }
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        /* (a failed call ends the capture all the same, so the stream is left out of capture mode) */
        cudaError_t captured = cudaMemcpyAsync(g->table, g->stage, bytes, cudaMemcpyHostToDevice, ctx->stream);
        if (captured == cudaSuccess)
            captured = cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream);
        if (captured == cudaSuccess)
            captured = artf::launchMixedTable(l, g->table, count, g->units, g->combine, g->tiles, g->order,
                                              nullptr); /* (an update rewrites the table, not a captured copy) */
        e = cudaStreamEndCapture(ctx->stream, &g->graph);
        if (e == cudaSuccess && captured != cudaSuccess) e = captured;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        artfCudaBatchGraphDestroy(g);
        return fail(ARTF_CUDA_ELAUNCH, "graph capture: %s", cudaGetErrorString(e));
    }
    *out = g;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaBatchGraphUpdate(ArtfCudaGraph* g, const ArtfCudaView* views, int count) {
    if (!g) return fail(ARTF_CUDA_EINVAL, "no graph");
    int status = enter(g->ctx);
    if (status) return status;
    if (!views || count != g->count) return fail(ARTF_CUDA_EINVAL, "update needs the graph's %d views", g->count);
    /* (a launch in flight may still be reading the staging) */
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(g->ctx->stream));
    const artf::TraceLaunch l = launchOf(g->ctx, &g->options);
    int units = 0;
    size_t combine = 0;
    /* (the planes the graph holds must cover the new views: sizes may differ at equal tile counts) */
    if (planesOf(l, views, count) != g->planeCount)
        return fail(ARTF_CUDA_EINVAL, "update changed the views' sizes; make a new graph");
    int tiles = 0;
    if ((status = fillTable(g->ctx, l, views, count, &g->options, g->stage, g->planes, &units, &combine, &tiles)))
        return status;
    if (units != g->units || combine != g->combine || tiles != g->tiles)
        return fail(ARTF_CUDA_EINVAL, "update changed the views' sizes; make a new graph");
    g->first = views[0].frame;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaBatchGraphLaunch(ArtfCudaGraph* g, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaBatchGraphLaunch");
    if (!g) return fail(ARTF_CUDA_EINVAL, "no graph");
    ArtfCuda* ctx = g->ctx;
    int status = enter(ctx);
    if (status) return status;
    if ((status = spendLaunch(ctx))) return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaGraphLaunch(g->exec, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    ctx->lastBands = 1;
    if ((status = checkBounds(ctx))) return status;
    return stats ? readStats(ctx, g->first, ARTF_CUDA_MIXED, g->options.guards, stats) : ARTF_CUDA_OK;
}

/* ---- the autotuner ------------------------------------------------------------------------------ */

/* Median time of `repeats` launches of the batch already in the context's table. */
static int timeBatch(ArtfCuda* ctx, const artf::TraceLaunch& l, int count, int units, size_t combine, int tiles,
                     int repeats, float* ms) {
    float times[8];
    for (int r = -1; r < repeats; ++r) {
        CUDA_OR(ARTF_CUDA_ELAUNCH,
                cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
        const cudaError_t e = artf::launchMixedTable(l, ctx->table, count, units, combine, tiles, ctx->order,
                                                     count == 1 ? ctx->stage : nullptr);
        if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "autotune launch: %s", cudaGetErrorString(e));
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
        CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventSynchronize(ctx->stop));
        if (r >= 0) CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventElapsedTime(&times[r], ctx->start, ctx->stop));
    }
    for (int i = 1; i < repeats; ++i)
        for (int j = i; j > 0 && times[j] < times[j - 1]; --j) {
            const float t = times[j];
            times[j] = times[j - 1];
            times[j - 1] = t;
        }
    *ms = times[repeats / 2];
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaAutotune(ArtfCuda* ctx, const ArtfCudaView* views, int count,
                                const ArtfCudaTraceOptions* options, ArtfCudaTuning* result) {
    artf::Range range("artfCudaAutotune");
    int status = enter(ctx);
    if (status) return status;
    if (!result) return fail(ARTF_CUDA_EINVAL, "result is NULL");
    if ((status = checkBatch(views, count, options))) return status;
    ArtfCudaTraceOptions o = *options;
    o.blockSize = o.compactEvery = o.fp64Batch = o.refillBatch = 0;
    ctx->hasTuning = false;
    artf::TraceLaunch l = launchOf(ctx, &o);
    if ((status = reserveTable(ctx, count))) return status;
    if ((status = reservePlanes(ctx, planesOf(l, views, count)))) return status;
    if ((status = waitStaging(ctx))) return status;
    int units = 0, tiles = 0;
    size_t combine = 0;
    if ((status = fillTable(ctx, l, views, count, &o, ctx->stage, ctx->planes, &units, &combine, &tiles)))
        return status;
    if ((status = reserveOrder(ctx, tiles, units))) return status;
    if ((status = sendTable(ctx, count))) return status;

    /* coordinate descent over the launch shape, from the defaults */
    static const int blocks[] = {64, 128, 192, 256};
    static const int waits[] = {16, 32, 64, 128, 256};
    static const int batches[] = {16, 24, 28, 32};
    static const int refills[] = {16, 24, 28, 32};
    int best[4] = {128, 64, 32, 32};
    const int* values[4] = {blocks, waits, batches, refills};
    const int counts[4] = {4, 5, 4, 4};
    const int repeats = 3;
    float bestMs = 0.f;
    int trials = 0;
    l.blockSize = best[0], l.compactEvery = best[1], l.fp64Batch = best[2], l.refillBatch = best[3];
    if ((status = timeBatch(ctx, l, count, units, combine, tiles, repeats, &bestMs))) return status;
    const float defaultMs = bestMs;
    ++trials;
    for (int pass = 0; pass < 2; ++pass)
        for (int d = 0; d < 4; ++d)
            for (int c = 0; c < counts[d]; ++c) {
                int trial[4] = {best[0], best[1], best[2], best[3]};
                if (values[d][c] == best[d]) continue;
                trial[d] = values[d][c];
                l.blockSize = trial[0], l.compactEvery = trial[1], l.fp64Batch = trial[2], l.refillBatch = trial[3];
                float ms = 0.f;
                if ((status = timeBatch(ctx, l, count, units, combine, tiles, repeats, &ms))) return status;
                ++trials;
                if (ms < bestMs * 0.99f) {
                    bestMs = ms;
                    memcpy(best, trial, sizeof best);
                }
            }
    ctx->tuned.blockSize = best[0];
    ctx->tuned.compactEvery = best[1];
    ctx->tuned.fp64Batch = best[2];
    ctx->tuned.refillBatch = best[3];
    ctx->tuned.ms = bestMs;
    ctx->tuned.defaultMs = defaultMs;
    ctx->tuned.trials = trials;
    ctx->hasTuning = true;
    *result = ctx->tuned;
    return ARTF_CUDA_OK;
}
