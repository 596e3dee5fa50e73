// fma_peak.cu -- measurement support, not part of the library's C ABI: the FMA issue
// ceiling of the FP64 or FP32 pipe that the ALU-bound kernels are measured against.
// Built into libhype_probes.so (test and benchmark use only).
#include <cuda_runtime.h>

#include "hype_common.cuh"
#include "probes.h"

// ------------------------------------------------------------------ FMA peak probe
// Eight independent FMA chains per thread, 8 blocks of 256 threads per SM: the
// issue-rate ceiling of the FP64 (or FP32) pipe that the ALU-bound kernels are
// measured against.
namespace hype {
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) x[q] = (T)(threadIdx.x + q);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = x[q] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += x[q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
static int probe(int iters, double* tflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    T* d = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaMalloc((void**)&d, sizeof(T) * blocks * threads);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_fma_probe<T><<<blocks, threads>>>(d, 16, (T)0.999, (T)0.001);
        cudaEventRecord(e0);
        k_fma_probe<T><<<blocks, threads>>>(d, iters, (T)0.999, (T)0.001);
        cudaEventRecord(e1);
        count_launch(2);
        e = cudaEventSynchronize(e1);
    }
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_last_error("hype_probe_fma_peak", e);
        return HYPE_ERR_CUDA;
    }
    *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
    return HYPE_OK;
}
}  // namespace hype

extern "C" int hype_probe_fma_peak(int precision, double* tflops) {
    if (!tflops) return HYPE_ERR_ARG;
    if (precision == HYPE_PREC_FP64) return hype::probe<double>(4096, tflops);
    if (precision == HYPE_PREC_FP32) return hype::probe<float>(65536, tflops);
    return HYPE_ERR_ARG;
}
