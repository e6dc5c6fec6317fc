/* artful_cuda — the FP64 forward-mode reference for the adjoint: every pixel's radiance and its
 * derivatives along the five scene parameters (spin, inclination, inner radius scale, emissivity index,
 * distance), carried through the trace's own templated core in dual numbers (lensDual.cuh).  The frame's
 * fields enter with their derivatives (the Jacobian of the frame in the parameters), the emissivity
 * index as the fourth direction, and the two parameter-dependent map tables from their formulas.
 * One thread a pixel, one ray at its centre; slow (five tangents in double) and exact: a reference for
 * the adjoint's gradients to be checked against. */
#include "lensDual.cuh"
#include "lensKernel.cuh"
#include "lensTangent.h"

namespace artf {
namespace {

using D5 = Dual<5>;

__global__ void __launch_bounds__(64) traceTangents(const KernelParams<D5> p, double* out) {
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    Tally t;
    const int pixels = p.f.width * p.f.height;
    if (i < pixels) {
        const int x = i % p.f.width, y = i / p.f.width;
        float nx, ny, moment;
        samplePosition(p.h, 0, 0, x, y, 0, &nx, &ny, &moment);
        D5 sum[3] = {D5(0.0), D5(0.0), D5(0.0)};
        traceRay(p, D5(nx), D5(ny), D5(p.h.disc[2] + p.h.spin[3] * moment), sum, nullptr, t);
        for (int c = 0; c < 3; ++c) {
            double* o = out + ((size_t)i * 3 + c) * 6;
            o[0] = sum[c].v;
            for (int k = 0; k < 5; ++k) o[1 + k] = sum[c].d[k];
        }
    }
    flushTally(t, p.counters);
}

}  // namespace

cudaError_t launchTangents(const TraceLaunch& l, const double* jacobian, double emissivity, double* out) {
    KernelParams<D5> p;
    p.f.load(l.frame64, l.frame);
    for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS; ++k) {
        D5* field = gradField(p.f, k);
        for (int q = 0; q < 5; ++q) field->d[q] = jacobian[k * 5 + q];
    }
    p.f.analyticTables = 1;
    p.f.emissivity = D5(emissivity);
    p.f.emissivity.d[3] = 1.0;
    p.h = l.frame;
    p.map = l.map;
    p.fluid = l.fluid;
    p.hdr = nullptr;
    p.ends = nullptr;
    p.counters = l.counters;
    p.jitter = 0;
    p.seed = 0;
    p.stepScale = D5(1.0);
    p.maxSteps = 192;
    p.rays = 1;
    p.share = 1.f;
    p.tilesX = p.tiles = p.tileBegin = 0;
    const int pixels = (int)(l.frame.size[0] * l.frame.size[1]);
    traceTangents<<<(pixels + 63) / 64, 64, 0, l.stream>>>(p, out);
    return cudaGetLastError();
}

}  // namespace artf
