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
constexpr size_t kMixedViewBytesMax = 1312;

size_t mixedViewBytes();
/* Fills one table slot; returns the view's unit count and, in *tiles, its 8 x 4 tiles.  rayOut: the
 * view's ray planes (width * height float4 a ray of a pixel, mixedRayPlanes of them), or NULL.  With
 * planes a work unit is one ray, so no lane is left with a pixel's several long rays after the queue
 * empties; without, a unit is a pixel.  unitBase, tileBase: the view's first unit and tile in the
 * batch. */
int mixedFillView(const TraceLaunch& options, const ArtfCudaHoleFrame& frame, const ArtfCudaHoleFrame64& frame64,
                  const float* map, const float* fluid, float4* hdr, ArtfCudaRayEnd* ends, float4* rayOut, int unitBase,
                  int tileBase, void* slot, int* tiles);
/* Device bytes of the heavy-first order of a batch of this many tiles and units. */
size_t mixedOrderBytes(int totalTiles, int totalUnits);
/* The planes a view needs: rays a pixel when above one, else none. */
inline size_t mixedRayPlanes(const TraceLaunch& l, const ArtfCudaHoleFrame& frame) {
    const size_t rays = l.jitter ? (size_t)l.jitter : (size_t)frame.size[2] * frame.size[2];
    return rays > 1 ? rays : 0;
}
/* The persistent grid of the given queue kernel for a batch of this many units. */
int mixedGrid(const TraceLaunch& options, int totalUnits, const void* kernel);
/* Launches the trace of a table already on the device (or, with options.rayCount > 0, the ray list of
 * its first view); then, when combinePixels (the largest view's pixel count) is above 0, the sum of
 * the views' ray planes into their frames.  With orderScratch (mixedOrderBytes of device memory) and
 * options.order heavy-first, the tiles are probed and ordered first (two short launches); NULL: the
 * queue runs in pixel order.  hostView: the host's copy of the table's one view (viewCount 1), which the
 * trace then takes as a kernel parameter; NULL where the table may change under a captured launch. */
cudaError_t launchMixedTable(const TraceLaunch& options, const void* deviceTable, int viewCount, int totalUnits,
                             size_t combinePixels, int totalTiles, void* orderScratch, const void* hostView);

}  // namespace artf
