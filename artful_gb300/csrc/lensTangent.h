/* artful_cuda — the differentiated traces' shared pieces: which frame fields the scene parameters reach
 * (the rows of ArtfCudaHoleParams' Jacobian), and the launchers of the forward-mode reference
 * (lensTangent.cu) and of the adjoint (lensAdjoint.cu). */
#pragma once

#include "lensCore.cuh"
#include "lensLaunch.h"

namespace artf {

/* Field k of the frame in the Jacobian's order: forward, right, up (3 each), metric (4), place (4), er,
 * etheta, ephi (3 each), the spin, the disc's inner radius. */
template <typename R> ARTF_HD R* gradField(Frame<R>& f, int k) {
    if (k < 3) return &f.forward[k];
    if (k < 6) return &f.right[k - 3];
    if (k < 9) return &f.up[k - 6];
    if (k < 13) return &f.metric[k - 9];
    if (k < 17) return &f.place[k - 13];
    if (k < 20) return &f.er[k - 17];
    if (k < 23) return &f.etheta[k - 20];
    if (k < 26) return &f.ephi[k - 23];
    if (k == 26) return &f.a;
    return &f.inner;
}

cudaError_t launchTangents(const TraceLaunch& l, const double* jacobian, double emissivity, double* out);

/* The adjoint's view table: one entry of adjointViewBytes() a view, filled on the host. */
size_t adjointViewBytes();
int adjointTiles(int width, int height); /* 8 x 4 tiles of pixels a view */
void adjointFillView(void* slot, const ArtfCudaHoleFrame& frame, const double* jacobian, double emissivity,
                     const float* map, const float* fluid, const float* target, float* hdr, float* pixelGrads);
/* The adjoint over `count` views of width x height; partials: count * adjointTiles(width, height) * 8
 * floats of scratch; results: count * 8 doubles (the loss, the five gradient components, two unused);
 * trail: adjointTrailBytes of scratch, where the forward kernel leaves each ray's kept states for the
 * reverse one. */
cudaError_t launchAdjoint(const void* table, int count, int width, int height, int K, unsigned long long* counters,
                          float* partials, double* results, cudaStream_t stream, void* orderScratch, void* trail);
size_t adjointTrailBytes(int count, int width, int height, int K);
/* Device bytes of the adjoint's order scratch (orderScratch above, required): the reverse kernel's
 * heavy-first tile order, with the weights and class counts it is sorted from. */
size_t adjointOrderBytes(int count, int width, int height);

}  // namespace artf
