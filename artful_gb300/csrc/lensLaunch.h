/* artful_cuda — what the C ABI (abi.cu) hands the kernel translation units: one struct of launch
 * parameters, and one launcher per precision, each in its own .cu with its own float flags. */
#pragma once

#include "artful_cuda.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace artf {

/* Device counters a trace adds to (unsigned 64-bit each).  CBoundsKind and CBoundsIndex: in the
 * debug build (ARTF_CUDA_DEBUG_BOUNDS), the first index found outside its table or frame (kind, index). */
enum Counter {
    CRays, CSteps, CCrossings, CEscapes, CFp64Steps, CQueue, CStatus,
    CFp64Horizon, CFp64Radial, CFp64Polar, CFp64Rounds, CBoundsKind, CBoundsIndex, CCount
};

struct TraceLaunch {
    ArtfCudaHoleFrame frame;      /* the FP32 frame (sample positions always come from it) */
    ArtfCudaHoleFrame64 frame64;  /* the FP64 frame (FP64 and mixed traces) */
    const float* map;
    const float* fluid;
    float4* hdr;                  /* width * height */
    ArtfCudaRayEnd* ends;         /* width * height * rays, or NULL */
    unsigned long long* counters; /* CCount of them, zeroed by the caller */
    int jitter;
    uint32_t seed;
    float stepScale;
    float horizonBand;
    int blockSize;
    int compactEvery;
    int persistent;
    uint32_t guards;
    int fp64Batch;
    int refillBatch;
    int order;                    /* ARTF_CUDA_ORDER_* (the mixed trace's queue) */
    int smCount;
    cudaStream_t stream;
    /* a band of the frame: 4-pixel tile rows [tileRowBegin, tileRowBegin + tileRows); 0 rows: all */
    int tileRowBegin;
    int tileRows;
    /* a list of rays in place of a frame's pixels (rayCount > 0) */
    int rayCount;
    const float* rayX;
    const float* rayY;
    const float* rayTime;
    float* rayRgb;
};

cudaError_t launchExact(const TraceLaunch& l);
cudaError_t launchFast(const TraceLaunch& l);
cudaError_t launchFp64(const TraceLaunch& l);
/* (the mixed trace launches from a view table: lensMixed.h) */

}  // namespace artf
