// hype_common.cuh -- shared helpers of the sm_103a library (error handling,
// launch accounting, boundary index maps).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/hype_gpu.h"

namespace hype {

// thread-local last CUDA error text (returned by hype_last_error)
void set_last_error(const char* where, cudaError_t e);
// process-wide kernel launch counter (hype_launch_count)
void count_launch(long long n = 1);

#define HYPE_CK(call)                                        \
    do {                                                     \
        cudaError_t e__ = (call);                            \
        if (e__ != cudaSuccess) {                            \
            ::hype::set_last_error(#call, e__);              \
            return e__ == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA; \
        }                                                    \
    } while (0)

#define HYPE_LAUNCHED(n)                                     \
    do {                                                     \
        ::hype::count_launch(n);                             \
        cudaError_t e__ = cudaGetLastError();                \
        if (e__ != cudaSuccess) {                            \
            ::hype::set_last_error("kernel launch", e__);    \
            return HYPE_ERR_CUDA;                            \
        }                                                    \
    } while (0)

// Map an index of a ghost cell onto the cell that supplies its value
// (3d/weno4/Navier-Stokes-3D/rhs_function.c:52-181): periodic wrap,
// transmissive copy of the edge cell, reflective mirror (-1-i / 2n-1-i) with
// the normal momentum negated (*flip).
__host__ __device__ __forceinline__ int bmap(int i, int n, int blo, int bhi, int* flip) {
    if (i < 0) {
        if (blo == HYPE_BC_PERIODIC) return i + n;
        if (blo == HYPE_BC_TRANSMISSIVE) return 0;
        *flip = 1;
        return -1 - i;
    }
    if (i >= n) {
        if (bhi == HYPE_BC_PERIODIC) return i - n;
        if (bhi == HYPE_BC_TRANSMISSIVE) return n - 1;
        *flip = 1;
        return 2 * n - 1 - i;
    }
    return i;
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace hype
