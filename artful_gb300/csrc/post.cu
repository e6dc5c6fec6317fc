/* artful_cuda — a traced frame to what a screen shows: the bloom pyramid and the tone map with its
 * dither, on the GPU.  Restates the software backend's bloomDownRow / bloomUpRow / bloomTap
 * (src/software/software.c:320-387) and lensToneMap / lensFill (src/software/lens.inc:387-440), with
 * the same float operations in the same order: built with the exact flags (no contraction, IEEE
 * division and square root), the BGRA frame comes out bit for bit the software backend's.
 *
 * The pyramid's levels are the frame's bloom table (ArtfCudaHoleFrame.bloom: offset, width, height),
 * three float planes of the frame's bloom pixel count.  Level 0 takes the mean of four pixels' light
 * above the threshold (2) and under the ceiling (48); each next level four bilinear taps of the one
 * before; then each level, from the top down, adds four taps of the one above, times 0.85.  The tone
 * map reads level 0 between its texels, turns its glow toward grey (0.9), adds it times bloom * 0.15,
 * scales by the exposure, applies Narkowicz's ACES fit and a square root, and dithers by a hash. */
#include "nvtxRange.h"
#include "artful_cuda.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr float kThreshold = 2.f, kCeiling = 48.f, kFade = .85f, kWhite = .9f;

__device__ __forceinline__ float minRef(float a, float b) { return b < a ? b : a; } /* core.h artfMinf */
__device__ __forceinline__ float maxRef(float a, float b) { return a < b ? b : a; } /* core.h artfMaxf */
__device__ __forceinline__ int clampRef(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
__device__ __forceinline__ float minX(float a, float b) { return a < b ? a : b; }   /* simd.h v8fMin */
__device__ __forceinline__ float maxX(float a, float b) { return a > b ? a : b; }   /* simd.h v8fMax */

__device__ __forceinline__ float bright(float v) { return minRef(maxRef(v - kThreshold, 0.f), kCeiling); }

/* software.c:320-328 bloomTap: a level at (sx, sy) in its texels, bilinear, clamped at the edges. */
__device__ __forceinline__ float tap(const float* level, int width, int height, float sx, float sy) {
    const float baseX = floorf(sx), baseY = floorf(sy), partX = sx - baseX, partY = sy - baseY;
    const int x0 = clampRef((int)baseX, 0, width - 1), x1 = clampRef((int)baseX + 1, 0, width - 1);
    const float* r0 = level + (size_t)clampRef((int)baseY, 0, height - 1) * width;
    const float* r1 = level + (size_t)clampRef((int)baseY + 1, 0, height - 1) * width;
    const float top = r0[x0] + (r0[x1] - r0[x0]) * partX, bottom = r1[x0] + (r1[x1] - r1[x0]) * partX;
    return top + (bottom - top) * partY;
}

struct Planes {
    float* c[3];
};

/* software.c:334-351: level 0 from the frame's light. */
__global__ void bloomFirst(const float4* hdr, int width, int height, Planes bloom, uint32_t at, int toW, int toH) {
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)blockIdx.y;
    if (x >= toW || y >= toH) return;
    const int lastX = width - 1, lastY = height - 1;
    const int y0 = min(y * 2, lastY), y1 = min(y * 2 + 1, lastY), x0 = min(x * 2, lastX), x1 = min(x * 2 + 1, lastX);
    const float4 a0 = hdr[(size_t)y0 * width + x0], a1 = hdr[(size_t)y0 * width + x1];
    const float4 b0 = hdr[(size_t)y1 * width + x0], b1 = hdr[(size_t)y1 * width + x1];
    const float s[3][4] = {{a0.x, a1.x, b0.x, b1.x}, {a0.y, a1.y, b0.y, b1.y}, {a0.z, a1.z, b0.z, b1.z}};
    for (int c = 0; c < 3; ++c)
        bloom.c[c][at + (size_t)y * toW + x] = (bright(s[c][0]) + bright(s[c][1]) + bright(s[c][2]) + bright(s[c][3])) * .25f;
}

/* software.c:353-365: level L from level L - 1, four taps. */
__global__ void bloomDown(Planes bloom, uint32_t fromAt, int fromW, int fromH, uint32_t toAt, int toW, int toH) {
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)blockIdx.y;
    if (x >= toW || y >= toH) return;
    const float cy = (float)y * 2.f + .5f, cx = (float)x * 2.f + .5f;
    for (int c = 0; c < 3; ++c) {
        const float* level = bloom.c[c] + fromAt;
        float sum = 0;
        for (int k = 0; k < 4; ++k) sum += tap(level, fromW, fromH, cx + (k & 1 ? 1.f : -1.f), cy + (k & 2 ? 1.f : -1.f));
        bloom.c[c][toAt + (size_t)y * toW + x] = sum * .25f;
    }
}

/* software.c:368-386: level L gains four taps of level L + 1. */
__global__ void bloomUp(Planes bloom, uint32_t fromAt, int fromW, int fromH, uint32_t toAt, int toW, int toH) {
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)blockIdx.y;
    if (x >= toW || y >= toH) return;
    const float sy = ((float)y + .5f) * .5f - .5f, sx = ((float)x + .5f) * .5f - .5f;
    for (int c = 0; c < 3; ++c) {
        const float* level = bloom.c[c] + fromAt;
        float sum = 0;
        for (int k = 0; k < 4; ++k) sum += tap(level, fromW, fromH, sx + (k & 1 ? .5f : -.5f), sy + (k & 2 ? .5f : -.5f));
        float* out = bloom.c[c] + toAt + (size_t)y * toW + x;
        *out += sum * (.25f * kFade);
    }
}

/* lens.inc:56-61: the dither's hash (the star lattice's). */
__device__ __forceinline__ uint32_t hash3(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t h = x * 73856093u ^ y * 19349663u ^ z * 83492791u;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

/* lens.inc:387-391: Narkowicz's fit to ACES, and a square root for the screen. */
__device__ __forceinline__ float toneCurve(float x) {
    const float top = x * (x * 2.51f + .03f);
    const float bottom = x * (x * 2.43f + .59f) + .14f;
    return sqrtf(minX(top / bottom, 1.f));
}

/* lens.inc:395-440: light plus glow, exposed, tone mapped and dithered to premultiplied BGRA. */
__global__ void toneMap(const float4* hdr, int width, int height, Planes bloom, uint32_t at, int bw, int bh,
                        float exposure, float spread, uint32_t* bgra) {
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)blockIdx.y;
    if (x >= width || y >= height) return;
    const float sy = ((float)y + .5f) * .5f - .5f, baseY = floorf(sy), partY = sy - baseY;
    const int y0 = clampRef((int)baseY, 0, bh - 1), y1 = clampRef((int)baseY + 1, 0, bh - 1);
    const float pixel = (float)x;
    const float sx = (pixel + .5f) * .5f - .5f;
    const float baseX = floorf(sx), partX = sx - baseX, lastX = (float)(bw - 1);
    const int x0 = (int)minX(maxX(baseX, 0.f), lastX), x1 = (int)minX(maxX(baseX + 1.f, 0.f), lastX);
    float glows[3];
    for (int c = 0; c < 3; ++c) {
        const float* plane = bloom.c[c] + at;
        const float a = plane[y0 * bw + x0], b = plane[y0 * bw + x1];
        const float d = plane[y1 * bw + x0], e = plane[y1 * bw + x1];
        const float upper = a + (b - a) * partX, lower = d + (e - d) * partX;
        glows[c] = upper + (lower - upper) * partY;
    }
    const float grey = glows[0] * .3f + glows[1] * .59f + glows[2] * .11f;
    const float4 h = hdr[(size_t)y * width + x];
    const float light[3] = {h.x, h.y, h.z};
    const float dither = (float)(int)(hash3((uint32_t)(x + y * 8192), 7u, 13u) & 255u) * (1.f / 255.f);
    uint32_t bytes[3];
    for (int c = 0; c < 3; ++c) {
        const float glow = glows[c] + (grey - glows[c]) * kWhite;
        const float shown = toneCurve((light[c] + glow * spread) * exposure);
        bytes[c] = (uint32_t)(int)minX(shown * 255.f + dither, 255.f);
    }
    bgra[(size_t)y * width + x] = bytes[0] << 16 | bytes[1] << 8 | bytes[2] | 0xFF000000u;
}

}  // namespace

/* The pyramid and tone map of one frame; bloom: three planes of the frame's bloom pixel count. */
extern "C" int artfCudaPostLaunch(const ArtfCudaHoleFrame* frame, const float* hdr, float* const bloomPlanes[3],
                                  uint32_t* bgra, void* stream) {
    artf::Range range("artfCudaPostLaunch");
    if (!frame || !hdr || !bloomPlanes || !bgra) return ARTF_CUDA_EINVAL;
    const int width = (int)frame->size[0], height = (int)frame->size[1], levels = (int)frame->size[3];
    if (width < 1 || height < 1 || levels < 1 || levels > ARTF_CUDA_BLOOM_LEVELS) return ARTF_CUDA_EINVAL;
    cudaStream_t s = (cudaStream_t)stream;
    Planes planes = {{bloomPlanes[0], bloomPlanes[1], bloomPlanes[2]}};
    const int block = 128;
    const uint32_t(*table)[4] = frame->bloom;
    for (int i = 0; i < levels; ++i) {
        const dim3 grid((table[i][1] + block - 1) / block, table[i][2]);
        if (i == 0) bloomFirst<<<grid, block, 0, s>>>((const float4*)hdr, width, height, planes, table[0][0],
                                                      (int)table[0][1], (int)table[0][2]);
        else bloomDown<<<grid, block, 0, s>>>(planes, table[i - 1][0], (int)table[i - 1][1], (int)table[i - 1][2],
                                              table[i][0], (int)table[i][1], (int)table[i][2]);
    }
    for (int i = levels - 1; i-- > 0;) {
        const dim3 grid((table[i][1] + block - 1) / block, table[i][2]);
        bloomUp<<<grid, block, 0, s>>>(planes, table[i + 1][0], (int)table[i + 1][1], (int)table[i + 1][2], table[i][0],
                                       (int)table[i][1], (int)table[i][2]);
    }
    const float spread = frame->look[3] * (1.f - kFade);
    toneMap<<<dim3((width + block - 1) / block, height), block, 0, s>>>(
        (const float4*)hdr, width, height, planes, table[0][0], (int)table[0][1], (int)table[0][2], frame->image[0],
        spread, bgra);
    return cudaGetLastError() == cudaSuccess ? ARTF_CUDA_OK : ARTF_CUDA_ELAUNCH;
}
