/* artful_cuda — the C ABI's device side: contexts, uploads and the trace dispatch.  Every entry point
 * checks its arguments and every CUDA call, and reports failure by status, never by abort. */
#include "artful_cuda.h"
#include "lensFlops.h"
#include "lensLaunch.h"

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
    bool lost;
};

/* Makes the context's device current for this thread. */
static int enter(ArtfCuda* ctx) {
    if (!ctx) return fail(ARTF_CUDA_EINVAL, "no context");
    if (ctx->lost) return fail(ARTF_CUDA_ELOST, "the context was lost; destroy it and make another");
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaSetDevice(ctx->device));
    return ARTF_CUDA_OK;
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
    int status = ARTF_CUDA_OK;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->start) != cudaSuccess || cudaEventCreate(&ctx->stop) != cudaSuccess)
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
    if (ctx->start) cudaEventDestroy(ctx->start);
    if (ctx->stop) cudaEventDestroy(ctx->stop);
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

static int checkFrame(const ArtfCudaHoleFrame* f, const ArtfCudaTraceOptions* o) {
    if (!f || !o) return fail(ARTF_CUDA_EINVAL, "frame or options is NULL");
    if (f->size[0] < 1 || f->size[1] < 1 || f->size[0] > 32768 || f->size[1] > 32768)
        return fail(ARTF_CUDA_EINVAL, "frame size %u x %u out of range", f->size[0], f->size[1]);
    if (!o->jitter && (f->size[2] < 1 || f->size[2] > 8))
        return fail(ARTF_CUDA_EINVAL, "rays a side %u out of 1..8", f->size[2]);
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
    return ARTF_CUDA_OK;
}

/* Launches what l describes and, when stats is given, waits and reads the counters and the time. */
static int runTrace(ArtfCuda* ctx, artf::TraceLaunch& l, int precision, ArtfCudaTraceStats* stats) {
    l.counters = ctx->counters;
    l.smCount = ctx->smCount;
    l.stream = ctx->stream;
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaMemsetAsync(ctx->counters, 0, sizeof(unsigned long long) * artf::CCount, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->start, ctx->stream));
    cudaError_t e = cudaSuccess;
    switch (precision) {
    case ARTF_CUDA_EXACT: e = artf::launchExact(l); break;
    case ARTF_CUDA_FP32: e = artf::launchFast(l); break;
    case ARTF_CUDA_FP64: e = artf::launchFp64(l); break;
    default: e = artf::launchMixed(l); break;
    }
    if (e != cudaSuccess) return fail(ARTF_CUDA_ELAUNCH, "trace launch: %s", cudaGetErrorString(e));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaEventRecord(ctx->stop, ctx->stream));
    if (stats) {
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
        stats->flops = artfFlops(stats->rays, stats->steps, stats->crossings, stats->escapes, l.frame.spin[0] != 0.f,
                                 l.frame.look[1] != 0.f, l.frame.look[2] > 0.f);
        stats->ms = ms;
    }
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaHoleTraceRays(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                     const float* map, const float* fluid, int precision, float stepScale, int n,
                                     const float* nx, const float* ny, const float* time, float* rgb,
                                     ArtfCudaRayEnd* ends, ArtfCudaTraceStats* stats) {
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
    artf::TraceLaunch l;
    memset(&l, 0, sizeof l);
    l.frame = *frame;
    if (frame64) l.frame64 = *frame64;
    else promoteFrame(frame, &l.frame64);
    l.map = map ? map : ctx->map;
    l.fluid = fluid ? fluid : ctx->fluid;
    l.ends = ends;
    l.stepScale = stepScale > 0.f ? stepScale : 1.f;
    l.rayCount = n;
    l.rayX = nx, l.rayY = ny, l.rayTime = time, l.rayRgb = rgb;
    return runTrace(ctx, l, precision, stats);
}

extern "C" int artfCudaHoleTrace(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                 const float* map, const float* fluid, const ArtfCudaTraceOptions* options, float* hdr,
                                 ArtfCudaRayEnd* ends, ArtfCudaTraceStats* stats) {
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkFrame(frame, options))) return status;
    if (!hdr) return fail(ARTF_CUDA_EINVAL, "hdr is NULL");
    if (!map && !ctx->mapHeld) return fail(ARTF_CUDA_EINVAL, "no map: pass one or call artfCudaSetMap");
    if (!fluid && !ctx->fluidHeld) return fail(ARTF_CUDA_EINVAL, "no fluid: pass one or call artfCudaSetFluid");
    artf::TraceLaunch l;
    memset(&l, 0, sizeof l);
    l.frame = *frame;
    if (frame64) l.frame64 = *frame64;
    else promoteFrame(frame, &l.frame64);
    l.map = map ? map : ctx->map;
    l.fluid = fluid ? fluid : ctx->fluid;
    l.hdr = (float4*)hdr;
    l.ends = ends;
    l.counters = ctx->counters;
    l.jitter = options->jitter;
    l.seed = options->seed;
    l.stepScale = options->stepScale > 0.f ? options->stepScale : 1.f;
    l.horizonBand = options->horizonBand;
    l.blockSize = options->blockSize;
    l.compactEvery = options->compactEvery;
    l.persistent = options->persistent;
    l.guards = options->guards;
    l.fp64Batch = options->fp64Batch;
    l.refillBatch = options->refillBatch;
    return runTrace(ctx, l, options->precision, stats);
}

extern "C" int artfCudaHoleRender(ArtfCuda* ctx, const ArtfCudaHoleFrame* frame, const ArtfCudaHoleFrame64* frame64,
                                  const float* hostMap, uint64_t mapVersion, const float* hostFluid,
                                  uint64_t fluidVersion, const ArtfCudaTraceOptions* options, float* hostHdr,
                                  ArtfCudaTraceStats* stats) {
    int status = enter(ctx);
    if (status) return status;
    if ((status = checkFrame(frame, options))) return status;
    if (!hostHdr) return fail(ARTF_CUDA_EINVAL, "hostHdr is NULL");
    if ((status = artfCudaSetMap(ctx, hostMap, mapVersion))) return status;
    if ((status = artfCudaSetFluid(ctx, hostFluid, fluidVersion))) return status;
    const size_t pixels = (size_t)frame->size[0] * frame->size[1];
    if (pixels > ctx->hdrPixels) {
        cudaFree(ctx->hdr);
        ctx->hdr = nullptr;
        ctx->hdrPixels = 0;
        CUDA_OR(ARTF_CUDA_ENOMEM, cudaMalloc(&ctx->hdr, sizeof(float4) * pixels));
        ctx->hdrPixels = pixels;
    }
    if ((status = artfCudaHoleTrace(ctx, frame, frame64, nullptr, nullptr, options, (float*)ctx->hdr, nullptr, stats)))
        return status;
    CUDA_OR(ARTF_CUDA_ELAUNCH,
            cudaMemcpyAsync(hostHdr, ctx->hdr, sizeof(float4) * pixels, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_OR(ARTF_CUDA_ELAUNCH, cudaStreamSynchronize(ctx->stream));
    return ARTF_CUDA_OK;
}
