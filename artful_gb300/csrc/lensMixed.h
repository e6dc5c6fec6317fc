/* artful_cuda — the mixed-precision trace's view table, between the C ABI and lensMixed.cu.
 *
 * A batch of views is traced by one persistent launch that reads a table of per-view constants from
 * device memory: the FP32 and FP64 frames, the map, fluid and output pointers, and each view's first
 * unit in the shared work queue (8 x 4 pixel tiles, 32 units a tile).  The caller fills the table on
 * the host (mixedFillView, one slot of mixedViewBytes() bytes a view), copies it to the device, zeroes
 * the counters and launches. */
#pragma once

#include "lensLaunch.h"

#include <stddef.h>

namespace artf {

/* A table slot never takes more than this (lensMixed.cu checks it at compile time). */
constexpr size_t kMixedViewBytesMax = 1024;

size_t mixedViewBytes();
/* Fills one table slot; returns the view's unit count. */
int mixedFillView(const TraceLaunch& options, const ArtfCudaHoleFrame& frame, const ArtfCudaHoleFrame64& frame64,
                  const float* map, const float* fluid, float4* hdr, ArtfCudaRayEnd* ends, int unitBase, void* slot);
/* The persistent grid for a batch of this many units. */
int mixedGrid(const TraceLaunch& options, int totalUnits);
/* Launches the trace of a table already on the device (or, with options.rayCount > 0, the ray list of
 * its first view). */
cudaError_t launchMixedTable(const TraceLaunch& options, const void* deviceTable, int viewCount, int totalUnits);

}  // namespace artf
