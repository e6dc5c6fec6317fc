/* artful_cuda — the FP32 and FP64 pipes' measured peaks on this device, the denominators of the trace's
 * roofline (the trace is bound by the FP32 pipe, not by memory and not by tensor cores).  Each thread runs
 * eight independent chains of fused multiply-adds; the grid fills every SM several times over. */
#include "artful_cuda.h"

#include <cuda_runtime.h>

namespace {

template <typename T> __global__ void __launch_bounds__(256) fmaChains(T* out, int rounds, T x) {
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = x + T(threadIdx.x + k);
    const T m = T(0.999999), c = T(1e-7);
    for (int i = 0; i < rounds; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a[k] * m + c;
    }
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == T(-12345)) out[0] = s; /* (never true: keeps the chains alive) */
}

template <typename T> double measure(int smCount, int rounds, cudaStream_t stream) {
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1;
    const int blocks = smCount * 8, threads = 256;
    cudaEvent_t start, stop;
    cudaEventCreate(&start);
    cudaEventCreate(&stop);
    fmaChains<T><<<blocks, threads, 0, stream>>>(out, rounds / 8, T(1));
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(start, stream);
        fmaChains<T><<<blocks, threads, 0, stream>>>(out, rounds, T(1));
        cudaEventRecord(stop, stream);
        cudaEventSynchronize(stop);
        float ms = 0;
        cudaEventElapsedTime(&ms, start, stop);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    cudaFree(out);
    const double flops = 2.0 * 8.0 * (double)rounds * blocks * threads;
    return cudaGetLastError() == cudaSuccess ? flops / (best * 1e-3) : -1;
}

}  // namespace

extern "C" int artfCudaProbePeaks(void* streamHandle, int device, double* fp32Flops, double* fp64Flops) {
    if (!fp32Flops || !fp64Flops) return ARTF_CUDA_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return ARTF_CUDA_ENODEVICE;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return ARTF_CUDA_ENODEVICE;
    cudaStream_t stream = (cudaStream_t)streamHandle;
    *fp32Flops = measure<float>(sms, 1 << 14, stream);
    *fp64Flops = measure<double>(sms, 1 << 9, stream);
    return (*fp32Flops > 0 && *fp64Flops > 0) ? ARTF_CUDA_OK : ARTF_CUDA_ELAUNCH;
}
