// df64_probe.cu -- elementwise probe of the double-float primitives of df64.cuh, for the
// tests: the split of an FP64 value into its FP32 pair and back, and the pair arithmetic.
// Built into libhype_probes.so (test use only), not part of the library's C ABI.
#include <cuda_runtime.h>

#include "df64.cuh"
#include "hype_common.cuh"
#include "probes.h"

namespace hype {

__global__ void k_df64_probe(const double* __restrict__ x, const double* __restrict__ y, long long n,
                             double* __restrict__ out) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const df64 a = df_from_double(x[q]), b = df_from_double(y[q]);
    double* o = out + 7 * q;
    o[0] = df_f2d(a.hi);
    o[1] = df_f2d(a.lo);
    o[2] = df_to_double(a);
    o[3] = df_to_double(a + b);
    o[4] = df_to_double(a - b);
    o[5] = df_to_double(a * b);
    o[6] = df_to_double(df_div(a, b));
}

}  // namespace hype

extern "C" int hype_df64_probe(const double* x, const double* y, long long n, double* out) {
    if (!x || !y || !out || n < 1) return HYPE_ERR_ARG;
    double *dx = nullptr, *dy = nullptr, *dout = nullptr;
    cudaError_t ce = cudaMalloc((void**)&dx, sizeof(double) * n);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&dy, sizeof(double) * n);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&dout, sizeof(double) * 7 * n);
    if (ce == cudaSuccess) ce = cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(dy, y, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) {
        hype::k_df64_probe<<<(unsigned)((n + 255) / 256), 256>>>(dx, dy, n, dout);
        hype::count_launch(1);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpy(out, dout, sizeof(double) * 7 * n, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dout);
    if (ce != cudaSuccess) {
        hype::set_last_error("hype_df64_probe", ce);
        return HYPE_ERR_CUDA;
    }
    return HYPE_OK;
}
