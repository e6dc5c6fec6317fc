/* artful_cuda — a batch trace that allocates nothing.
 *
 * Some callers cannot call cudaMalloc: a host engine or plug-in framework that owns every byte of
 * device memory through its own allocator and memory budget, or a render thread that must not take the
 * device-wide synchronisation an allocation can cause in the middle of a frame.  The context-based
 * entry points allocate (at artfCudaCreate and when a batch outgrows the view table), so this entry
 * point keeps its only scratch, the batch's view table and its work-queue and tally counters, in one
 * file-scope device array of fixed size, and takes every input and output from the caller.
 *
 * The array lives on every GPU that loads the library until the process exits (82 KB).  Host code
 * cannot use the array's name as a device address, so the first call on each device looks the address
 * up there (cudaGetSymbolAddress, with that device current) and keeps it; after a device reset
 * (cudaDeviceReset, or a reset of the primary context) the kept address is stale, and the process must
 * restart before it calls this entry point again.  All calls share the array and it keeps the last
 * call's contents; each call writes the table and clears the counters before its launch.  Calls whose
 * work overlaps on the GPU (on different streams, or from different threads) race on the array: order
 * them on one stream.  The table is built in a file-scope host buffer, not on the caller's stack (a
 * render thread may have a small one), under a lock held until its copy has been staged.  A call made
 * while its stream is being captured is refused: the graph would record a copy from that host buffer,
 * which later calls overwrite, and the stats read would end the capture. */
#include "nvtxRange.h"
#include "artful_cuda.h"
#include "lensLaunch.h"
#include "lensMixed.h"

#include <cuda_runtime.h>
#include <mutex>
#include <stdio.h>
#include <string.h>

namespace artf {
int failWith(int status, const char* message);
int checkTraceFrame(const ArtfCudaHoleFrame* frame, const ArtfCudaTraceOptions* options);
}  // namespace artf

namespace {

constexpr size_t kCounterBytes = 256; /* artf::CCount counters, padded */
static_assert(sizeof(unsigned long long) * artf::CCount <= kCounterBytes, "counters outgrew their slot");
constexpr size_t kScratchBytes = kCounterBytes + ARTF_CUDA_NOALLOC_MAX_VIEWS * artf::kMixedViewBytesMax;

/* The scratch: counters first, then the view table. */
static __device__ __align__(256) unsigned char noAllocScratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex setupLock;
void* scratchOn[kMaxDevices]; /* device address of the array, per device; NULL until looked up */
/* The view table's host side, built and copied under stageLock (a copy from pageable memory is staged
 * before cudaMemcpyAsync returns, so the buffer is free again once the lock is released). */
std::mutex stageLock;
alignas(16) unsigned char stage[ARTF_CUDA_NOALLOC_MAX_VIEWS * artf::kMixedViewBytesMax];

/* The array's device address on the current device, looked up on the first call there. */
int scratchAddress(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return artf::failWith(ARTF_CUDA_ENODEVICE, "device index out of range");
    std::lock_guard<std::mutex> hold(setupLock);
    if (!scratchOn[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, noAllocScratch);
        if (e != cudaSuccess || !ptr) {
            char line[160];
            snprintf(line, sizeof line, "cudaGetSymbolAddress of the scratch array: %s", cudaGetErrorString(e));
            return artf::failWith(ARTF_CUDA_ELAUNCH, line);
        }
        scratchOn[device] = ptr;
    }
    *out = (unsigned char*)scratchOn[device];
    return ARTF_CUDA_OK;
}

}  // namespace

extern "C" int artfCudaHoleBatchNoAlloc(const ArtfCudaView* views, int count, const ArtfCudaTraceOptions* options,
                                        void* stream, ArtfCudaTraceStats* stats) {
    artf::Range range("artfCudaHoleBatchNoAlloc");
    char line[200];
    if (!views || !options) return artf::failWith(ARTF_CUDA_EINVAL, "views or options is NULL");
    if (count < 1 || count > ARTF_CUDA_NOALLOC_MAX_VIEWS) {
        snprintf(line, sizeof line, "batch of %d views: the allocation-free entry point holds 1..%d views", count,
                 ARTF_CUDA_NOALLOC_MAX_VIEWS);
        return artf::failWith(ARTF_CUDA_EINVAL, line);
    }
    if (options->precision != ARTF_CUDA_MIXED)
        return artf::failWith(ARTF_CUDA_EINVAL, "batches trace in mixed precision (ARTF_CUDA_MIXED) only");
    for (int i = 0; i < count; ++i) {
        if (int s = artf::checkTraceFrame(&views[i].frame, options)) return s;
        if (!views[i].map || !views[i].fluid || !views[i].hdr) {
            snprintf(line, sizeof line, "view %d: map, fluid and hdr must be device pointers (no context here)", i);
            return artf::failWith(ARTF_CUDA_EINVAL, line);
        }
    }
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &capturing) != cudaSuccess ||
        capturing != cudaStreamCaptureStatusNone)
        return artf::failWith(ARTF_CUDA_EINVAL, "the allocation-free batch is not made for a stream being captured "
                                                "(use the graph API: artfCudaBatchGraphCreate)");
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return artf::failWith(ARTF_CUDA_ENODEVICE, "no current CUDA device");
    unsigned char* scratch = nullptr;
    if (int s = scratchAddress(device, &scratch)) return s;

    artf::TraceLaunch l;
    memset(&l, 0, sizeof l);
    l.jitter = options->jitter;
    l.seed = options->seed;
    l.stepScale = options->stepScale > 0.f ? options->stepScale : 1.f;
    l.horizonBand = options->horizonBand;
    l.blockSize = options->blockSize;
    l.compactEvery = options->compactEvery;
    l.guards = options->guards;
    l.fp64Batch = options->fp64Batch;
    l.refillBatch = options->refillBatch;
    l.counters = (unsigned long long*)scratch;
    l.smCount = sms;
    l.stream = (cudaStream_t)stream;

    /* the table, built in the file's host buffer and copied in */
    std::unique_lock<std::mutex> staging(stageLock);
    long long units = 0, tiles = 0;
    for (int i = 0; i < count; ++i) {
        /* (no ray planes nor heavy-first order: the fixed scratch cannot hold them, so a work unit is a
         * pixel, in pixel order) */
        int viewTiles = 0;
        units += artf::mixedFillView(l, views[i].frame, views[i].frame64, views[i].map, views[i].fluid,
                                     (float4*)views[i].hdr, views[i].ends, nullptr, (int)units, (int)tiles,
                                     stage + artf::mixedViewBytes() * (size_t)i, &viewTiles);
        tiles += viewTiles;
        if (units > 0x7FFFFFFFLL) return artf::failWith(ARTF_CUDA_EINVAL, "batch is too large");
    }
    unsigned char* table = scratch + kCounterBytes;
    cudaError_t e = cudaMemcpyAsync(table, stage, artf::mixedViewBytes() * (size_t)count, cudaMemcpyHostToDevice,
                                    l.stream);
    staging.unlock();
    if (e == cudaSuccess) e = cudaMemsetAsync(scratch, 0, kCounterBytes, l.stream);
    if (e == cudaSuccess) e = artf::launchMixedTable(l, table, count, (int)units, 0, (int)tiles, nullptr, nullptr);
    if (e != cudaSuccess) {
        snprintf(line, sizeof line, "allocation-free batch launch: %s", cudaGetErrorString(e));
        return artf::failWith(ARTF_CUDA_ELAUNCH, line);
    }
    if (stats) {
        unsigned long long c[artf::CCount];
        e = cudaMemcpyAsync(c, scratch, sizeof c, cudaMemcpyDeviceToHost, l.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(l.stream);
        if (e != cudaSuccess) {
            snprintf(line, sizeof line, "allocation-free batch stats: %s", cudaGetErrorString(e));
            return artf::failWith(ARTF_CUDA_ELAUNCH, line);
        }
        memset(stats, 0, sizeof *stats);
        stats->rays = c[artf::CRays];
        stats->steps = c[artf::CSteps];
        stats->crossings = c[artf::CCrossings];
        stats->escapes = c[artf::CEscapes];
        stats->fp64Steps = c[artf::CFp64Steps];
        stats->fp64Horizon = c[artf::CFp64Horizon];
        stats->fp64Radial = c[artf::CFp64Radial];
        stats->fp64Polar = c[artf::CFp64Polar];
        stats->fp64Rounds = c[artf::CFp64Rounds];
        stats->bands = 1;
    }
    return ARTF_CUDA_OK;
}
