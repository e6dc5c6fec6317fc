/* artful_cuda — the disc's gas on the GPU: the reference's fluid step (src/scene/fluid.c), byte for byte.
 *
 * The model (fluid.c:1-23): isothermal compressible flow in the disc's plane on 256 rings of 1024 cells,
 * density S and the velocity's departure from a circular orbit (vr along the radius, w along the orbit),
 * Kerr's orbital and epicyclic frequencies; eddies stirred in at random; a FARGO-style shift of each ring
 * along itself by its own orbit.  The reference steps it on the CPU every frame and uploads the 1 MB
 * field; here it stays on the device, where the trace reads it.
 *
 * Same bytes: this unit is built without contraction and with IEEE division and square root, and each
 * float expression keeps the reference's order of operations.  The reference's cell loops are
 * independent within a pass (each pass reads one copy of the fields and writes the other), so one thread
 * a cell computes what it computes.  Two things are ordered: the eddies, which overlap and so run one
 * after another in one block, each eddy's cells in parallel (an eddy touches each cell once); and each
 * ring's mean density, a sum in cell order, which one thread a ring adds up.  The random draws that place
 * the eddies (a xorshift sequence) are made on the host, in the reference's order, for all the steps of
 * a call at once, and copied to the device with their shapes.
 *
 * Work layout: 7 fields of 256 x 1024 floats (7 MB, L2-resident), one allocation; per step five launches
 * on the context's stream (stir, velocities, densities, shift, balance), and the field after the last. */
#include "nvtxRange.h"
#include "artful_cuda.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

namespace artf {
int contextStream(ArtfCuda* ctx, cudaStream_t* stream);
int contextFluid(ArtfCuda* ctx, float** fluid);
int failWith(int status, const char* message);
}  // namespace artf

namespace {

constexpr int FW = ARTF_CUDA_FLUID_WIDTH;  /* cells around a ring */
constexpr int FH = ARTF_CUDA_FLUID_HEIGHT; /* rings */
constexpr float DT = .2f;                  /* fluid.c:28 */
#define ARC (6.2831853f / (float)FW)       /* fluid.c:29 */
constexpr int MAX_STEPS = 48;              /* fluid.c:30 */
constexpr int WARM_STEPS = 60;             /* fluid.c:31 */
constexpr float WOUND_TIME = 900.f;        /* fluid.c:32 */
constexpr int EDDIES_A_STEP = 16;          /* fluid.c:232-234: two large, fourteen small */
constexpr int START_EDDIES = 200;          /* fluid.c:312 */
constexpr int FIELD = FW * FH;

/* Per ring: radius, the row's width in radius, orbital and epicyclic terms, sound speed squared, the
 * ring's shift a step in cells, the envelope and fall-off of what shows (fluid.c:270-287). */
struct Rings {
    float radius[FH], rowWidth[FH], angular[FH], epicyclic[FH], sound2[FH], slide[FH], envelope[FH], fall[FH];
};

/* One eddy, placed and shaped on the host (fluid.c:188-201). */
struct Eddy {
    float r0, size, strength, clump, invSize2;
    int i0, reach;
};

__host__ __device__ __forceinline__ float clampF(float v, float lo, float hi) { return v < lo ? lo : v > hi ? hi : v; }
__host__ __device__ __forceinline__ float lesser(float a, float b) { return b < a ? b : a; }
__host__ __device__ __forceinline__ float greater(float a, float b) { return a < b ? b : a; }
__host__ __device__ __forceinline__ int atMost(int a, int b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ int atLeast(int a, int b) { return a > b ? a : b; }

__host__ __device__ __forceinline__ float ease(float a, float b, float x) {
    const float t = clampF((x - a) / (b - a), 0.f, 1.f);
    return t * t * (3.f - 2.f * t);
}

__device__ __forceinline__ uint32_t cellHash(uint32_t x, uint32_t y, uint32_t seed) {
    uint32_t h = x * 0x9E3779B1u ^ y * 0x85EBCA77u ^ seed * 0xC2B2AE3Du;
    h = (h ^ h >> 15) * 0x2C1B3C6Du;
    h = (h ^ h >> 12) * 0x297A2D39u;
    return h ^ h >> 15;
}

/* fluid.c:71-80 */
__device__ __forceinline__ float noise(float x, float y, uint32_t period, uint32_t seed) {
    const float fx = floorf(x), fy = floorf(y), tx = x - fx, ty = y - fy;
    const uint32_t x0 = (uint32_t)fx & (period - 1), x1 = (x0 + 1) & (period - 1), y0 = (uint32_t)fy, y1 = y0 + 1;
    const float v00 = (float)(cellHash(x0, y0, seed) >> 8), v10 = (float)(cellHash(x1, y0, seed) >> 8);
    const float v01 = (float)(cellHash(x0, y1, seed) >> 8), v11 = (float)(cellHash(x1, y1, seed) >> 8);
    const float sx = tx * tx * (3.f - 2.f * tx), sy = ty * ty * (3.f - 2.f * ty);
    const float lo = v00 + (v10 - v00) * sx, hi = v01 + (v11 - v01) * sx;
    return (lo + (hi - lo) * sy) * (1.f / 16777216.f);
}

/* fluid.c:82-93 (an index never leaves the field: y0 <= FH - 2, columns wrap) */
__device__ __forceinline__ float bilinear(const float* __restrict__ a, float x, float y) {
    const float fy = clampF(y, 0.f, (float)(FH - 1) - .001f);
    const int y0 = (int)fy;
    const float py = fy - (float)y0;
    const float fx = floorf(x), px = x - fx;
    const int x0 = (int)fx & (FW - 1), x1 = (x0 + 1) & (FW - 1);
    const float* lo = a + (size_t)y0 * FW;
    const float* hi = lo + FW;
    const float top = lo[x0] + (lo[x1] - lo[x0]) * px, bottom = hi[x0] + (hi[x1] - hi[x0]) * px;
    return top + (bottom - top) * py;
}

/* ---- kernels: one thread a cell, unless said otherwise ------------------------------------------ */

/* fluid.c:291-311: the start, clumps the shear has long been drawing out */
__global__ void __launch_bounds__(256) seedDensity(float* __restrict__ s, const Rings* __restrict__ rings) {
    const int cell = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (cell >= FIELD) return;
    const int j = cell / FW, i = cell - j * FW;
    const float rho = (float)j / (float)(FH - 1), wound = rings->angular[j] * WOUND_TIME / 6.2831853f;
    float turn = (float)i / (float)FW - wound;
    turn -= floorf(turn);
    float sum = 0, amplitude = .5f, total = 0, across = 14.f;
    uint32_t period = 16;
    for (uint32_t o = 0; o < 5; ++o) {
        sum += amplitude * noise(turn * (float)period, rho * across, period, 7 + o);
        total += amplitude;
        amplitude *= .72f;
        period *= 2;
        across *= 2.f;
    }
    const float v = sum / total;
    s[cell] = .06f + 3.4f * ease(.34f, .68f, v) * ease(.34f, .68f, v);
}

/* fluid.c:202-218: eddies one after another (they overlap), each one's cells at once; one block.  The
 * rows an eddy can reach (its radial test passed) are found first and only they are visited: the test
 * still runs on each, so every cell gets the update the reference gives it. */
__global__ void __launch_bounds__(1024) stir(float* __restrict__ s, float* __restrict__ vr, float* __restrict__ w,
                                             const Rings* __restrict__ rings, const Eddy* __restrict__ eddies,
                                             int count) {
    __shared__ int lo, hi;
    for (int e = 0; e < count; ++e) {
        const Eddy q = eddies[e];
        if (threadIdx.x == 0) lo = FH, hi = -1;
        __syncthreads();
        if ((int)threadIdx.x < FH) {
            const float dr = rings->radius[threadIdx.x] - q.r0;
            if (!(dr * dr > 6.25f * q.size * q.size)) {
                atomicMin(&lo, (int)threadIdx.x);
                atomicMax(&hi, (int)threadIdx.x);
            }
        }
        __syncthreads();
        const int span = 2 * q.reach + 1; /* columns -reach .. reach: fewer than FW, so each cell once */
        const int rows = hi - lo + 1;     /* (none reached: not positive) */
        for (int k = (int)threadIdx.x; k < rows * span; k += (int)blockDim.x) {
            const int row = k / span, j = lo + row, di = k - row * span - q.reach;
            const float dr = rings->radius[j] - q.r0;
            if (dr * dr > 6.25f * q.size * q.size) continue;
            const float dx = (float)di * rings->radius[j] * ARC;
            const float d2 = (dr * dr + dx * dx) * q.invSize2;
            if (d2 > 6.25f) continue;
            const float g = 1.f - d2 * .16f, shape = g * g * g;
            const size_t at = (size_t)j * FW + (size_t)((q.i0 + di) & (FW - 1));
            vr[at] -= q.strength * shape * dx / q.size;
            w[at] += q.strength * shape * dr / q.size;
            s[at] = clampF(s[at] * (1.f + q.clump * shape), .03f, 8.f);
        }
        __syncthreads();
    }
}

/* fluid.c:96-124 */
__global__ void __launch_bounds__(256) velocities(const float* __restrict__ s, const float* __restrict__ vr,
                                                  const float* __restrict__ w, float* __restrict__ outR,
                                                  float* __restrict__ outW, const Rings* __restrict__ rings) {
    const int cell = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (cell >= FIELD) return;
    const int j = cell / FW, i = cell - j * FW;
    const float r = rings->radius[j], invR = 1.f / r, c2 = rings->sound2[j], om = rings->angular[j];
    const float sw = rings->epicyclic[j];
    const float toCells = DT / (r * ARC), toRows = DT / rings->rowWidth[j];
    const int up = atMost(j + 1, FH - 1), down = atLeast(j - 1, 0);
    const float invSpan = 1.f / (rings->radius[up] - rings->radius[down]), invArc = 1.f / (2.f * r * ARC);
    const float keep = 1.f - DT * .04f * om;
    const float x = (float)i - w[cell] * toCells, y = (float)j - vr[cell] * toRows;
    const float v0 = bilinear(vr, x, y), w0 = bilinear(w, x, y);
    const float inv = 1.f / s[cell];
    const float gradR = (s[(size_t)up * FW + i] - s[(size_t)down * FW + i]) * invSpan * inv;
    const float gradPhi = (s[(size_t)j * FW + ((i + 1) & (FW - 1))] - s[(size_t)j * FW + ((i - 1) & (FW - 1))]) *
                          invArc * inv;
    const float w1 = w0 + DT * (-sw * v0 - v0 * w0 * invR - c2 * gradPhi);
    const float v1 = v0 + DT * (2.f * om * w1 + w1 * w1 * invR - c2 * gradR);
    outW[cell] = clampF(w1 * keep, -.4f, .4f);
    outR[cell] = clampF(v1 * keep, -.4f, .4f);
}

/* fluid.c:126-151 */
__global__ void __launch_bounds__(256) densities(const float* __restrict__ s, const float* __restrict__ vr,
                                                 const float* __restrict__ w, float* __restrict__ out,
                                                 const Rings* __restrict__ rings) {
    const int cell = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (cell >= FIELD) return;
    const int j = cell / FW, i = cell - j * FW;
    const float r = rings->radius[j], invR = 1.f / r;
    const float toCells = DT / (r * ARC), toRows = DT / rings->rowWidth[j];
    const int up = atMost(j + 1, FH - 1), down = atLeast(j - 1, 0);
    const float rUp = rings->radius[up], rDown = rings->radius[down], invSpan = 1.f / (rUp - rDown);
    const float invArc = 1.f / (2.f * r * ARC);
    const float drift = -.004f, refill = DT * .002f * rings->angular[j];
    const float x = (float)i - w[cell] * toCells, y = (float)j - (vr[cell] + drift) * toRows;
    const float moved = bilinear(s, x, y);
    const float spread = (rUp * vr[(size_t)up * FW + i] - rDown * vr[(size_t)down * FW + i]) * invSpan * invR +
                         (w[(size_t)j * FW + ((i + 1) & (FW - 1))] - w[(size_t)j * FW + ((i - 1) & (FW - 1))]) * invArc;
    const float next = moved * (1.f - DT * clampF(spread, -2.f, 2.f));
    out[cell] = clampF(next + (1.f - next) * refill, .03f, 8.f);
}

/* fluid.c:153-173: each ring moved along itself by its orbit, a Catmull-Rom cubic held within its two
 * middle neighbours, for the three fields, from the new copies back into the current ones */
__device__ __forceinline__ float slideCell(const float* __restrict__ in, int i, int b, float k0, float k1, float k2,
                                           float k3) {
    const float p0 = in[(i + b - 1) & (FW - 1)], p1 = in[(i + b) & (FW - 1)];
    const float p2 = in[(i + b + 1) & (FW - 1)], p3 = in[(i + b + 2) & (FW - 1)];
    return clampF(k0 * p0 + k1 * p1 + k2 * p2 + k3 * p3, lesser(p1, p2), greater(p1, p2));
}

__global__ void __launch_bounds__(256) slide(const float* __restrict__ s, const float* __restrict__ vr,
                                             const float* __restrict__ w, float* __restrict__ outS,
                                             float* __restrict__ outR, float* __restrict__ outW,
                                             const Rings* __restrict__ rings) {
    const int cell = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (cell >= FIELD) return;
    const int j = cell / FW, i = cell - j * FW;
    const float cells = rings->slide[j];
    const float whole = floorf(cells), t = 1.f - (cells - whole), t2 = t * t, t3 = t2 * t;
    const int b = -(int)whole - 1;
    const float k0 = -.5f * t + t2 - .5f * t3, k1 = 1.f - 2.5f * t2 + 1.5f * t3;
    const float k2 = .5f * t + 2.f * t2 - 1.5f * t3, k3 = -.5f * t2 + .5f * t3;
    const size_t row = (size_t)j * FW;
    outS[cell] = slideCell(s + row, i, b, k0, k1, k2, k3);
    outR[cell] = slideCell(vr + row, i, b, k0, k1, k2, k3);
    outW[cell] = slideCell(w + row, i, b, k0, k1, k2, k3);
}

/* fluid.c:221-229: a block a ring; its sum in cell order by one thread, as the reference adds it */
__global__ void __launch_bounds__(256) balance(float* __restrict__ s) {
    __shared__ float ring[FW];
    __shared__ float scale;
    float* row = s + (size_t)blockIdx.x * FW;
    for (int i = (int)threadIdx.x; i < FW; i += (int)blockDim.x) ring[i] = row[i];
    __syncthreads();
    if (threadIdx.x == 0) {
        float sum = 0;
        for (int i = 0; i < FW; ++i) sum += ring[i];
        const float mean = sum * (1.f / (float)FW);
        scale = 1.f + .03f * (1.f / mean - 1.f);
    }
    __syncthreads();
    for (int i = (int)threadIdx.x; i < FW; i += (int)blockDim.x) row[i] = clampF(ring[i] * scale, .03f, 8.f);
}

/* fluid.c:175-186 */
__global__ void __launch_bounds__(256) showField(const float* __restrict__ s, float* __restrict__ out,
                                                 const Rings* __restrict__ rings) {
    const int cell = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (cell >= FIELD) return;
    const int j = cell / FW;
    const float v = s[cell] * rings->envelope[j];
    out[cell] = rings->fall[j] * ease(.1f, 1.1f, v) * lesser(v, 2.2f);
}

}  // namespace

struct ArtfCudaFluid {
    ArtfCuda* ctx;
    cudaStream_t stream;
    float inner, outer;
    float* block;          /* the seven fields, one allocation */
    float* dens[2];
    float* radial[2];
    float* orbital[2];
    float* field;
    Rings* rings;          /* device copy */
    Eddy* eddies;          /* device: a call's eddies, in order */
    Eddy* staged;          /* pinned host: the same */
    int eddyRoom;
    Rings host;
    uint32_t state;        /* fluid.c:49 xorshift32 */
    double time;
};

namespace {

uint32_t draw(ArtfCudaFluid* f) {
    uint32_t x = f->state;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    f->state = x;
    return x;
}
float uniform(ArtfCudaFluid* f) { return (float)(draw(f) >> 8) * (1.f / 16777216.f); }

/* fluid.c:188-201: where an eddy goes and its shape, with the reference's draws in its order */
Eddy placeEddy(ArtfCudaFluid* f, bool small) {
    Eddy q;
    const float u = uniform(f);
    q.r0 = f->inner + (f->outer - f->inner) * u * u;
    int j0 = 0;
    while (j0 < FH - 1 && f->host.radius[j0] < q.r0) ++j0;
    q.i0 = (int)(draw(f) & (FW - 1));
    q.size = q.r0 * (small ? .006f + .02f * uniform(f) : .02f + .1f * uniform(f));
    const float c = sqrtf(f->host.sound2[j0]);
    q.strength = 0.f;
    if (!small) {
        const float sign = uniform(f) < .5f ? -1.f : 1.f;
        q.strength = sign * c * (.3f + .7f * uniform(f));
    }
    q.clump = (uniform(f) - .42f) * (small ? 1.5f : .5f);
    q.invSize2 = 1.f / (q.size * q.size);
    q.reach = atMost((int)(2.5f * q.size / (q.r0 * ARC)) + 1, FW / 2 - 1);
    return q;
}

int reserveEddies(ArtfCudaFluid* f, int count) {
    if (count <= f->eddyRoom) return ARTF_CUDA_OK;
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, "fluid: sync");
    cudaFree(f->eddies);
    cudaFreeHost(f->staged);
    f->eddies = nullptr, f->staged = nullptr, f->eddyRoom = 0;
    if (cudaMalloc(&f->eddies, sizeof(Eddy) * count) != cudaSuccess ||
        cudaMallocHost(&f->staged, sizeof(Eddy) * count) != cudaSuccess)
        return artf::failWith(ARTF_CUDA_ENOMEM, "fluid: eddy table allocation");
    f->eddyRoom = count;
    return ARTF_CUDA_OK;
}

/* `steps` steps (fluid.c:231-241), after `extra` eddies of the start, and the field after them. */
int advanceSteps(ArtfCudaFluid* f, int extra, int steps) {
    const int count = extra + steps * EDDIES_A_STEP;
    if (int s = reserveEddies(f, count)) return s;
    /* (the previous call's copy may still read the staging) */
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, "fluid: sync");
    int n = 0;
    for (int e = 0; e < extra; ++e) f->staged[n++] = placeEddy(f, false);
    for (int k = 0; k < steps; ++k) {
        for (int e = 0; e < 2; ++e) f->staged[n++] = placeEddy(f, false);
        for (int e = 0; e < 14; ++e) f->staged[n++] = placeEddy(f, true);
    }
    cudaError_t e = n ? cudaMemcpyAsync(f->eddies, f->staged, sizeof(Eddy) * n, cudaMemcpyHostToDevice, f->stream)
                      : cudaSuccess;
    const int cur = 0; /* each step's shift writes back into the current copies */
    const unsigned blocks = (FIELD + 255) / 256;
    if (e == cudaSuccess && extra > 0) {
        stir<<<1, 1024, 0, f->stream>>>(f->dens[cur], f->radial[cur], f->orbital[cur], f->rings, f->eddies, extra);
        e = cudaGetLastError();
    }
    for (int k = 0; k < steps && e == cudaSuccess; ++k) {
        stir<<<1, 1024, 0, f->stream>>>(f->dens[cur], f->radial[cur], f->orbital[cur], f->rings,
                                         f->eddies + extra + k * EDDIES_A_STEP, EDDIES_A_STEP);
        velocities<<<blocks, 256, 0, f->stream>>>(f->dens[cur], f->radial[cur], f->orbital[cur], f->radial[cur ^ 1],
                                                  f->orbital[cur ^ 1], f->rings);
        densities<<<blocks, 256, 0, f->stream>>>(f->dens[cur], f->radial[cur ^ 1], f->orbital[cur ^ 1],
                                                 f->dens[cur ^ 1], f->rings);
        slide<<<blocks, 256, 0, f->stream>>>(f->dens[cur ^ 1], f->radial[cur ^ 1], f->orbital[cur ^ 1], f->dens[cur],
                                             f->radial[cur], f->orbital[cur], f->rings);
        balance<<<FH, 256, 0, f->stream>>>(f->dens[cur]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        showField<<<blocks, 256, 0, f->stream>>>(f->dens[cur], f->field, f->rings);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}

}  // namespace

extern "C" void artfCudaFluidFree(ArtfCudaFluid* f) {
    if (!f) return;
    cudaStreamSynchronize(f->stream);
    cudaFree(f->block);
    cudaFree(f->rings);
    cudaFree(f->eddies);
    cudaFreeHost(f->staged);
    free(f);
}

extern "C" int artfCudaFluidNew(ArtfCuda* ctx, float inner, float outer, float spin, double time,
                                ArtfCudaFluid** out) {
    artf::Range range("artfCudaFluidNew");
    if (!out) return artf::failWith(ARTF_CUDA_EINVAL, "out is NULL");
    *out = nullptr;
    if (!(inner > 0.f) || !(outer > inner) || !(fabsf(spin) <= 1.f) || !isfinite(time))
        return artf::failWith(ARTF_CUDA_EINVAL, "fluid: a disc needs 0 < inner < outer and |spin| <= 1");
    cudaStream_t stream = nullptr;
    if (int s = artf::contextStream(ctx, &stream)) return s;
    ArtfCudaFluid* f = (ArtfCudaFluid*)calloc(1, sizeof(ArtfCudaFluid));
    if (!f) return artf::failWith(ARTF_CUDA_ENOMEM, "host allocation");
    f->ctx = ctx, f->stream = stream, f->inner = inner, f->outer = outer;
    f->state = 0x9E3779B9u, f->time = time;
    if (cudaMalloc(&f->block, sizeof(float) * FIELD * 7) != cudaSuccess ||
        cudaMalloc(&f->rings, sizeof(Rings)) != cudaSuccess) {
        artfCudaFluidFree(f);
        return artf::failWith(ARTF_CUDA_ENOMEM, "fluid: device allocation");
    }
    for (int k = 0; k < 2; ++k)
        f->dens[k] = f->block + FIELD * (3 * k), f->radial[k] = f->block + FIELD * (3 * k + 1),
        f->orbital[k] = f->block + FIELD * (3 * k + 2);
    f->field = f->block + FIELD * 6;
    /* the rings (fluid.c:270-290), on the host in float as the reference has them */
    Rings& g = f->host;
    const float k = 1.f - inner / outer;
    for (int j = 0; j < FH; ++j) {
        const float rho = (float)j / (float)(FH - 1), r = inner / (1.f - rho * k);
        g.radius[j] = r;
        const float root = sqrtf(r), om = 1.f / (r * root + spin);
        g.angular[j] = om;
        const float kappa2 = om * om * (1.f - 6.f / r + 8.f * spin / (r * root) - 3.f * spin * spin / (r * r));
        g.epicyclic[j] = greater(kappa2, -.5f * om * om) / (2.f * om);
        const float c = .03f * r * om;
        g.sound2[j] = c * c;
        g.slide[j] = om * DT / ARC;
        g.envelope[j] = ease(inner + .5f, inner + 2.2f, r) * (1.f - .86f * ease(outer * .12f, outer * .8f, r));
        g.fall[j] = sqrtf(inner / r);
    }
    for (int j = 0; j < FH; ++j)
        g.rowWidth[j] = (g.radius[atMost(j + 1, FH - 1)] - g.radius[atLeast(j - 1, 0)]) * (j == 0 || j == FH - 1 ? 1.f : .5f);
    cudaError_t e = cudaMemcpyAsync(f->rings, &f->host, sizeof(Rings), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(f->block, 0, sizeof(float) * FIELD * 7, stream);
    if (e == cudaSuccess) {
        seedDensity<<<(FIELD + 255) / 256, 256, 0, stream>>>(f->dens[0], f->rings);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream); /* (the rings' staging is on this frame) */
    int status = e == cudaSuccess ? advanceSteps(f, START_EDDIES, WARM_STEPS)
                                  : artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    if (status) {
        artfCudaFluidFree(f);
        return status;
    }
    f->time = time;
    *out = f;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaFluidAdvance(ArtfCudaFluid* f, double time, int* stepped) {
    artf::Range range("artfCudaFluidAdvance");
    if (stepped) *stepped = 0;
    if (!f || !isfinite(time)) return artf::failWith(ARTF_CUDA_EINVAL, "no fluid, or a time that is not finite");
    cudaStream_t stream = nullptr;
    if (int s = artf::contextStream(f->ctx, &stream)) return s;
    double clock = f->time;
    const int steps = artfCudaFluidClock(&clock, time);
    if (steps > 0)
        if (int s = advanceSteps(f, 0, steps)) return s;
    f->time = clock;
    if (stepped) *stepped = steps > 0;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaFluidStep(ArtfCudaFluid* f, int64_t steps, double time) {
    artf::Range range("artfCudaFluidStep");
    if (!f || steps < 0 || !isfinite(time)) return artf::failWith(ARTF_CUDA_EINVAL, "fluid step: no fluid, or bad steps or time");
    cudaStream_t stream = nullptr;
    if (int s = artf::contextStream(f->ctx, &stream)) return s;
    /* in runs of at most 4 x 48 steps, so that the eddy staging stays small */
    for (int64_t done = 0; done < steps;) {
        const int run = (int)(steps - done < 4 * MAX_STEPS ? steps - done : 4 * MAX_STEPS);
        if (int s = advanceSteps(f, 0, run)) return s;
        done += run;
    }
    f->time = time;
    return ARTF_CUDA_OK;
}

extern "C" int artfCudaUseFluid(ArtfCuda* ctx, const ArtfCudaFluid* f) {
    if (!f || f->ctx != ctx) return artf::failWith(ARTF_CUDA_EINVAL, "use fluid: no fluid, or one of another context");
    float* dst = nullptr;
    if (int s = artf::contextFluid(ctx, &dst)) return s;
    const cudaError_t e = cudaMemcpyAsync(dst, f->field, sizeof(float) * FIELD, cudaMemcpyDeviceToDevice, f->stream);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}

extern "C" const float* artfCudaFluidField(const ArtfCudaFluid* f) { return f ? f->field : nullptr; }
extern "C" double artfCudaFluidTime(const ArtfCudaFluid* f) { return f ? f->time : 0.0; }

extern "C" int artfCudaFluidRead(const ArtfCudaFluid* f, float* host) {
    if (!f || !host) return artf::failWith(ARTF_CUDA_EINVAL, "no fluid or no buffer");
    cudaError_t e = cudaMemcpyAsync(host, f->field, sizeof(float) * FIELD, cudaMemcpyDeviceToHost, f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) return artf::failWith(ARTF_CUDA_ELAUNCH, cudaGetErrorString(e));
    return ARTF_CUDA_OK;
}
