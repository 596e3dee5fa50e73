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

// magnitude of conserved variable c in a cell of density rho and total energy E:
// |rho|, |E|, and for the momenta sqrt(2 |rho E|), which bounds |m| while the pressure
// is positive (a momentum near zero is measured against the cell's energy, not itself)
template <typename T>
__host__ __device__ __forceinline__ T var_scale(int c, T rho, T E) {
    const T ar = rho < 0 ? -rho : rho, ae = E < 0 ? -E : E;
    return c == 0 ? ar : c == 4 ? ae : sqrt((T)2 * ar * ae);
}

// normalised 5-point stencil: (s_k - mean) / (range + floor) with floor = 1e-2 of the
// variable's magnitude in the cell: variations below about a percent of the state
// (grid noise, weak acoustics) read as flat, a jump of the order of the state as O(1)
__host__ __device__ __forceinline__ void normalise5(const float* s, float scale, float* out) {
    const float mu = 0.2f * (s[0] + s[1] + s[2] + s[3] + s[4]);
#ifdef __CUDA_ARCH__
    // three-input min / max (the same extremes for finite values; a signed zero they may pick
    // differently cancels in hi - lo + floor)
    float lo, hi;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(lo) : "f"(s[0]), "f"(s[1]), "f"(s[2]));
    asm("min.f32 %0, %1, %2, %3;" : "=f"(lo) : "f"(lo), "f"(s[3]), "f"(s[4]));
    asm("max.f32 %0, %1, %2, %3;" : "=f"(hi) : "f"(s[0]), "f"(s[1]), "f"(s[2]));
    asm("max.f32 %0, %1, %2, %3;" : "=f"(hi) : "f"(hi), "f"(s[3]), "f"(s[4]));
#else
    float lo = s[0], hi = s[0];
    for (int k = 1; k < 5; ++k) {
        lo = s[k] < lo ? s[k] : lo;
        hi = s[k] > hi ? s[k] : hi;
    }
#endif
#ifdef __CUDA_ARCH__
    const float inv = __frcp_rn((hi - lo) + (1e-2f * scale + 1e-30f));  // = 1 / x, correctly rounded
#else
    const float inv = 1.0f / ((hi - lo) + (1e-2f * scale + 1e-30f));
#endif
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

// ---- tensor-core inference (mma.sync m16n8k16, BF16 operands, FP32 accumulation) ----
// A warp scores 32 cells x 3 directions = 96 rows (3D), or x 2 directions = 64 rows (2D).  Inputs and the first hidden layer
// are rounded to BF16 (the operand type); b1 rides in W1's padding column 25 against a
// constant-1 input, b2 initialises the second accumulator.
constexpr int KP = 32;       // padded input width (25 features, the bias input, zeros)
constexpr int ROWS = 96;     // rows per warp
constexpr int RSTRIDE = 40;  // BF16 row stride of the staging buffer (conflict-free fragment loads)

struct MmaWeights {
    unsigned w1[NH * KP / 2];  // W1 | b1 | 0, BF16 pairs, [n][k]
    unsigned w2[NH * NH / 2];  // W2, BF16 pairs, [n][k]
    float b2[NH], w3[NH], b3;
};

// the fragment layout of the BF16 parameters p (host or device)
__host__ __device__ inline void pack_weights(const __nv_bfloat16* __restrict__ p, MmaWeights& w, int t = 0, int nt = 1) {
    __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(w.w1);
    __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(w.w2);
    for (int q = t; q < NH * KP; q += nt) {
        const int n = q / KP, k = q % KP;
        w1[q] = k < NIN ? p[OFF_W1 + n * NIN + k] : (k == NIN ? p[OFF_B1 + n] : __float2bfloat16_rn(0.0f));
    }
    for (int q = t; q < NH * NH; q += nt) w2[q] = p[OFF_W2 + q];
    for (int q = t; q < NH; q += nt) {
        w.b2[q] = __bfloat162float(p[OFF_B2 + q]);
        w.w3[q] = __bfloat162float(p[OFF_W3 + q]);
    }
    if (t == 0) w.b3 = __bfloat162float(p[OFF_B3]);
}

// one row of the staging buffer: 25 features, the bias input 1, zeros
__device__ __forceinline__ void stage_row(__nv_bfloat16* row, const float* x, bool valid) {
#pragma unroll
    for (int k = 0; k < KP; k += 2) {
        const float lo = !valid ? 0.0f : k < NIN ? x[k] : (k == NIN ? 1.0f : 0.0f);
        const float hi = !valid ? 0.0f : k + 1 < NIN ? x[k + 1] : (k + 1 == NIN ? 1.0f : 0.0f);
        *reinterpret_cast<__nv_bfloat162*>(row + k) = __floats2bfloat162_rn(lo, hi);
    }
}

__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_relu(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(fmaxf(lo, 0.0f), fmaxf(hi, 0.0f));
    return *reinterpret_cast<unsigned*>(&v);
}

// logits of the warp's NROWS staged rows (shared memory) into lg[NROWS] (shared memory);
// w is the packed network in global memory (L1-resident after the first warp);
// every lane of the warp must call it
template <int NROWS = ROWS>
__device__ __forceinline__ void warp_logits(const MmaWeights* __restrict__ w, const __nv_bfloat16* rows, float* lg) {
    static_assert(NROWS % 16 == 0, "rows come in m16 tiles");
    const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
    unsigned bw1[4][2][2], bw2[4][2][2];
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            const int o = (n * 8 + g) * (KP / 2) + kt * 8 + tg;
            bw1[n][kt][0] = __ldg(&w->w1[o]);
            bw1[n][kt][1] = __ldg(&w->w1[o + 4]);
            bw2[n][kt][0] = __ldg(&w->w2[o]);
            bw2[n][kt][1] = __ldg(&w->w2[o + 4]);
        }
    const float b3 = __ldg(&w->b3);
    const unsigned* r32 = reinterpret_cast<const unsigned*>(rows);
#pragma unroll 1
    for (int mt = 0; mt < NROWS / 16; ++mt) {
        unsigned a[2][4];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            const int r0 = (mt * 16 + g) * (RSTRIDE / 2) + kt * 8 + tg, r1 = r0 + 8 * (RSTRIDE / 2);
            a[kt][0] = r32[r0];
            a[kt][1] = r32[r1];
            a[kt][2] = r32[r0 + 4];
            a[kt][3] = r32[r1 + 4];
        }
        float c1[4][4];
#pragma unroll
        for (int n = 0; n < 4; ++n) {
            c1[n][0] = c1[n][1] = c1[n][2] = c1[n][3] = 0.0f;
            mma_bf16(c1[n], a[0], bw1[n][0][0], bw1[n][0][1]);
            mma_bf16(c1[n], a[1], bw1[n][1][0], bw1[n][1][1]);
        }
        unsigned h[2][4];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            h[kt][0] = pack_relu(c1[2 * kt][0], c1[2 * kt][1]);
            h[kt][1] = pack_relu(c1[2 * kt][2], c1[2 * kt][3]);
            h[kt][2] = pack_relu(c1[2 * kt + 1][0], c1[2 * kt + 1][1]);
            h[kt][3] = pack_relu(c1[2 * kt + 1][2], c1[2 * kt + 1][3]);
        }
        float o0 = 0.0f, o1 = 0.0f;
#pragma unroll
        for (int n = 0; n < 4; ++n) {
            const int col = n * 8 + tg * 2;
            const float b20 = __ldg(&w->b2[col]), b21 = __ldg(&w->b2[col + 1]);
            const float w30 = __ldg(&w->w3[col]), w31 = __ldg(&w->w3[col + 1]);
            float c2[4] = {b20, b21, b20, b21};
            mma_bf16(c2, h[0], bw2[n][0][0], bw2[n][0][1]);
            mma_bf16(c2, h[1], bw2[n][1][0], bw2[n][1][1]);
            o0 = fmaf(w30, fmaxf(c2[0], 0.0f), fmaf(w31, fmaxf(c2[1], 0.0f), o0));
            o1 = fmaf(w30, fmaxf(c2[2], 0.0f), fmaf(w31, fmaxf(c2[3], 0.0f), o1));
        }
        o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
        o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
        o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
        if (tg == 0) {
            lg[mt * 16 + g] = o0 + b3;
            lg[mt * 16 + g + 8] = o1 + b3;
        }
    }
}

}  // namespace mlp
}  // namespace hype
