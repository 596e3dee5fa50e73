// mlp_kernels.cuh -- the troubled-cell indicator network (no counterpart in the reference).
//
// 25 -> 32 (ReLU) -> 32 (ReLU) -> 1 logit, BF16 weights, FP32 accumulation.
// Input: the normalised 5-point stencil (along one face normal) of each of the
// 5 conserved variables; a cell is scored by the max of its three directional
// logits.  Parameter layout (FP32 master copy, 1921 values):
//   W1[32][25] b1[32] W2[32][32] b2[32] W3[32] b3[1]
#pragma once

#include <cuda_bf16.h>

namespace hype {
namespace mlp {

constexpr int NIN = 25, NH = 32;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NH, NPARAM = OFF_B3 + 1;

// normalised 5-point stencil: (s_k - mean) / (range + delta), delta = 1e-2 (|mean| + 1e-3):
// variations of less than about a percent of the local magnitude (grid noise, small
// acoustic perturbations) read as flat, a jump of the order of the state as O(1)
__host__ __device__ __forceinline__ void normalise5(const float* s, float* out) {
    const float mu = 0.2f * (s[0] + s[1] + s[2] + s[3] + s[4]);
    float lo = s[0], hi = s[0];
    for (int k = 1; k < 5; ++k) {
        lo = s[k] < lo ? s[k] : lo;
        hi = s[k] > hi ? s[k] : hi;
    }
    const float inv = 1.0f / ((hi - lo) + 1e-2f * ((mu < 0 ? -mu : mu) + 1e-3f));
    for (int k = 0; k < 5; ++k) out[k] = (s[k] - mu) * inv;
}

// forward pass of one input with weights p (bf16 in shared or global memory)
__device__ __forceinline__ float forward(const __nv_bfloat16* __restrict__ p, const float* x) {
    float h1[NH];
#pragma unroll 4
    for (int j = 0; j < NH; ++j) {
        float a = __bfloat162float(p[OFF_B1 + j]);
#pragma unroll
        for (int k = 0; k < NIN; ++k) a = fmaf(__bfloat162float(p[OFF_W1 + j * NIN + k]), x[k], a);
        h1[j] = fmaxf(a, 0.0f);
    }
    float out = __bfloat162float(p[OFF_B3]);
#pragma unroll 4
    for (int j = 0; j < NH; ++j) {
        float a = __bfloat162float(p[OFF_B2 + j]);
#pragma unroll
        for (int k = 0; k < NH; ++k) a = fmaf(__bfloat162float(p[OFF_W2 + j * NH + k]), h1[k], a);
        out = fmaf(__bfloat162float(p[OFF_W3 + j]), fmaxf(a, 0.0f), out);
    }
    return out;
}

}  // namespace mlp
}  // namespace hype
