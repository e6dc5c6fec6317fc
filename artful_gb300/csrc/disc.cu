/* artful_cuda — the reference's painted disc map, made on the GPU (src/scene/hole.c:14-197 buildDisc and
 * setRings), byte for byte.
 *
 * The reference paints it on every core at start-up, about 0.6 s: two million gas texels of some thirty
 * lattice lookups each (strands along each orbit, torn clouds, a fraying edge), dust lanes, the sky's
 * dust band, a black-body colour table and the rings' tables.  Every texel is its own, so one thread a
 * texel computes what the reference does; this unit is built without contraction and with IEEE division
 * and square root, and each float expression keeps the reference's order.  The one reduction, the gas's
 * mean over the map's inner half (a double sum the reference adds in texel order), is added here in a
 * fixed tree order: the sum is of floats of moderate range, its double rounding leaves the float scale
 * derived from it unchanged, and the test holds the whole map to the reference's bytes.  The colour and
 * ring tables (4 K floats) come from the host set-up (holeHost.c), as the reference computes them. */
#include "nvtxRange.h"
#include "artful_cuda.h"

#include <cuda_runtime.h>

namespace artf {
int contextStream(ArtfCuda* ctx, cudaStream_t* stream);
int contextMap(ArtfCuda* ctx, float** map);
int failWith(int status, const char* message);
}  // namespace artf

namespace {

constexpr int MW = ARTF_CUDA_MAP_WIDTH, MH = ARTF_CUDA_MAP_HEIGHT;
constexpr int HALF = MW * (MH / 2);   /* the inner half the gas is scaled over */
constexpr int SUM_BLOCKS = 1024;      /* HALF / SUM_BLOCKS texels a block */

__device__ __forceinline__ float clampF(float v, float lo, float hi) { return v < lo ? lo : v > hi ? hi : v; }

/* hole.c:14-21 */
__device__ __forceinline__ uint32_t texHash(uint32_t x, uint32_t y, uint32_t seed) {
    uint32_t h = x * 0x9E3779B1u ^ y * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    return h ^ h >> 15;
}

/* hole.c:23-26 */
__device__ __forceinline__ float ease(float a, float b, float x) {
    const float t = clampF((x - a) / (b - a), 0.f, 1.f);
    return t * t * (3.f - 2.f * t);
}

/* hole.c:29-39: value noise repeating every period in x, coordinates through a signed integer */
__device__ __forceinline__ float lattice(float x, float y, uint32_t period, uint32_t seed) {
    const float fx = floorf(x), fy = floorf(y), tx = x - fx, ty = y - fy;
    const uint32_t x0 = (uint32_t)(int32_t)fx % period, x1 = (x0 + 1) % period, y0 = (uint32_t)(int32_t)fy, y1 = y0 + 1;
    const float v00 = (float)(texHash(x0, y0, seed) >> 8), v10 = (float)(texHash(x1, y0, seed) >> 8);
    const float v01 = (float)(texHash(x0, y1, seed) >> 8), v11 = (float)(texHash(x1, y1, seed) >> 8);
    const float sx = tx * tx * (3.f - 2.f * tx), sy = ty * ty * (3.f - 2.f * ty);
    const float lo = v00 + (v10 - v00) * sx, hi = v01 + (v11 - v01) * sx;
    return (lo + (hi - lo) * sy) * (1.f / 16777216.f);
}

/* hole.c:42-53 */
__device__ float octaves(float x, float y, uint32_t period, float scaleY, float falloff, float stretch, int count,
                         uint32_t seed) {
    float sum = 0, amplitude = .5f, total = 0;
    for (int o = 0; o < count; ++o) {
        sum += amplitude * lattice(x * (float)period, y * scaleY, period, seed + (uint32_t)o);
        total += amplitude;
        amplitude *= falloff;
        period *= 2;
        scaleY *= stretch;
    }
    return sum / total;
}

__device__ __forceinline__ float crest(float v) {
    const float r = 1.f - fabsf(2.f * v - 1.f);
    return r * r;
}

/* hole.c:101-124 */
__device__ float gasAt(float turn, float rho) {
    const float wander = .045f * (octaves(turn, rho, 3, 5.f, .5f, 2.f, 4, 101) - .5f) +
                         .012f * (octaves(turn, rho, 11, 24.f, .5f, 2.f, 3, 107) - .5f);
    float along = turn + .03f * (octaves(turn, rho, 5, 9.f, .5f, 2.f, 3, 113) - .5f);
    along -= floorf(along);
    const float across = rho + wander;
    float hair = 0, amplitude = .5f, total = 0, scale = 600.f;
    uint32_t period = 6;
    for (int o = 0; o < 6; ++o) {
        hair += amplitude * crest(lattice(along * (float)period, across * scale, period, 120u + (uint32_t)o));
        total += amplitude;
        amplitude *= .62f;
        period *= 2;
        scale *= 1.75f;
    }
    hair /= total;
    const float cloud = octaves(along, across, 7, 34.f, .55f, 2.f, 5, 131);
    const float outer = ease(.85f, 1.f, rho);
    const float torn = ease(.3f + .08f * outer, .7f + .08f * outer, cloud);
    const float gaps = 1.f + (torn - 1.f) * ease(.1f, .6f, rho);
    const float edge = ease(0.f, .02f, rho) * (1.f - ease(.9f, 1.f, across));
    return edge * (.25f + 2.2f * hair) * (.04f + 1.5f * gaps);
}

/* hole.c:128-138: a thread a gas texel */
__global__ void __launch_bounds__(256) paintGas(float* __restrict__ map) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= MW * MH) return;
    const int y = t / MW, x = t - y * MW;
    const float rho = (float)y / (float)(MH - 1), thin = 1.f - .887f * rho;
    float turn = (float)x / (float)MW + rho * .09f;
    turn -= floorf(turn);
    map[t] = gasAt(turn, rho) * thin * thin;
}

/* The inner half's sum in double, a fixed order: each block its own run of texels (its threads
 * strided, then a tree), then one thread the blocks in order, and the scale (hole.c:143-146). */
__global__ void __launch_bounds__(256) sumHalf(const float* __restrict__ map, double* __restrict__ partial) {
    __shared__ double part[256];
    const int per = HALF / SUM_BLOCKS;
    const float* run = map + (size_t)blockIdx.x * per;
    double s = 0.0;
    for (int i = (int)threadIdx.x; i < per; i += 256) s += (double)run[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int width = 128; width > 0; width >>= 1) {
        if ((int)threadIdx.x < width) part[threadIdx.x] += part[threadIdx.x + width];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = part[0];
}

__global__ void finishScale(const double* __restrict__ partial, float* __restrict__ scale) {
    double sum = 0.0;
    for (int b = 0; b < SUM_BLOCKS; ++b) sum += partial[b];
    *scale = (float)((double)HALF / sum);
}

__global__ void __launch_bounds__(256) scaleGas(float* __restrict__ map, const float* __restrict__ scale) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t < MW * MH) map[t] *= *scale;
}

/* hole.c:150-159: dust lanes */
__global__ void __launch_bounds__(256) paintDust(float* __restrict__ map) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= ARTF_CUDA_DUST_WIDTH * ARTF_CUDA_DUST_HEIGHT) return;
    const int y = t / ARTF_CUDA_DUST_WIDTH, x = t - y * ARTF_CUDA_DUST_WIDTH;
    const float rho = (float)y / (float)(ARTF_CUDA_DUST_HEIGHT - 1), outward = ease(.25f, .8f, rho);
    const float turn = (float)x / (float)ARTF_CUDA_DUST_WIDTH;
    map[ARTF_CUDA_DUST_AT + t] = outward * ease(.45f, .7f, octaves(turn, rho, 4, 90.f, .55f, 2.f, 5, 151));
}

/* hole.c:168-177: the sky's dust band */
__global__ void __launch_bounds__(256) paintSky(float* __restrict__ map) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= ARTF_CUDA_SKY_WIDTH * ARTF_CUDA_SKY_HEIGHT) return;
    const int y = t / ARTF_CUDA_SKY_WIDTH, x = t - y * ARTF_CUDA_SKY_WIDTH;
    const float height = (float)y / (float)(ARTF_CUDA_SKY_HEIGHT - 1), turn = (float)x / (float)ARTF_CUDA_SKY_WIDTH;
    const float bent = height - .5f + .22f * (lattice(turn * 2.f, 3.f, 2, 41) - .5f) +
                       .1f * (lattice(turn * 3.f, 5.f, 3, 42) - .5f);
    const float band = 1.f - ease(0.f, .3f, fabsf(bent));
    const float dust = octaves(turn, height, 8, 8.f, .58f, 2.f, 6, 51);
    map[ARTF_CUDA_SKY_AT + t] = .0006f + band * band * ease(.3f, .75f, dust) * .006f;
}

}  // namespace

extern "C" int artfCudaPaintDisc(ArtfCuda* ctx, float* map, float inner, float outer, float spin) {
    artf::Range range("artfCudaPaintDisc");
    cudaStream_t stream = nullptr;
    if (int s = artf::contextStream(ctx, &stream)) return s;
    if (!(inner > 0.f) || !(outer > inner) || !(fabsf(spin) <= 1.f))
        return artf::failWith(ARTF_CUDA_EINVAL, "paint disc: needs 0 < inner < outer and |spin| <= 1");
    if (!map)
        if (int s = artf::contextMap(ctx, &map)) return s;
    /* the tables on the host: rows and colours lie together, the glow apart */
    static_assert(ARTF_CUDA_COLORS_AT == ARTF_CUDA_ROWS_AT + ARTF_CUDA_MAP_HEIGHT * 2, "map layout");
    float tables[ARTF_CUDA_MAP_HEIGHT * 2 + ARTF_CUDA_COLORS * 3], glow[ARTF_CUDA_MAP_HEIGHT];
    artfCudaHoleRings(tables, glow, inner, outer, spin);
    artfCudaHoleColours(tables + ARTF_CUDA_MAP_HEIGHT * 2);
    void* scratch = nullptr;
    cudaError_t e = cudaMalloc(&scratch, sizeof(double) * SUM_BLOCKS + 16);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ENOMEM, "paint disc: scratch allocation");
    double* partial = (double*)scratch;
    float* scale = (float*)(partial + SUM_BLOCKS);
    paintGas<<<(MW * MH + 255) / 256, 256, 0, stream>>>(map);
    sumHalf<<<SUM_BLOCKS, 256, 0, stream>>>(map, partial);
    finishScale<<<1, 1, 0, stream>>>(partial, scale);
    scaleGas<<<(MW * MH + 255) / 256, 256, 0, stream>>>(map, scale);
    paintDust<<<(ARTF_CUDA_DUST_WIDTH * ARTF_CUDA_DUST_HEIGHT + 255) / 256, 256, 0, stream>>>(map);
    paintSky<<<(ARTF_CUDA_SKY_WIDTH * ARTF_CUDA_SKY_HEIGHT + 255) / 256, 256, 0, stream>>>(map);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(map + ARTF_CUDA_ROWS_AT, tables, sizeof tables, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(map + ARTF_CUDA_GLOW_AT, glow, sizeof glow, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream); /* (the tables are on this frame) */
    cudaFree(scratch);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}
