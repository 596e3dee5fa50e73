// mlp.cu -- training and evaluation of the troubled-cell indicator on the GPU.
//
// Hand-written forward / backward / Adam kernels (no framework).  A sample is a
// cell: X[s][3][25] (normalised stencils along x, y, z), label y[s] in {0,1}.
// The cell's logit is the max over its three directional logits; the loss is
// binary cross-entropy with a positive-class weight.  Training uses the
// BF16-rounded weights with FP32 activations and accumulation and an FP32 master
// copy updated by Adam; inference (k_score and the gated reconstruction) runs the
// same network on the tensor cores with BF16 inputs and first-layer activations.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "hype_common.cuh"
#include "mlp_kernels.cuh"

namespace hype {
namespace mlp {

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ q, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) q[i] = __float2bfloat16_rn(p[i]);
}

// cell scores on the tensor cores, the same code path as the gated reconstruction
__global__ void __launch_bounds__(128) k_score(const float* __restrict__ X, int n, const MmaWeights* __restrict__ w,
                                               float* __restrict__ score) {
    __shared__ __align__(16) __nv_bfloat16 rows[4][ROWS * RSTRIDE];
    __shared__ float lg[4][ROWS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    for (int d = 0; d < 3; ++d) {
        float x[NIN];
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = s < n ? X[((long long)s * 3 + d) * NIN + k] : 0.0f;
        stage_row(rows[warp] + (lane * 3 + d) * RSTRIDE, x, s < n);
    }
    __syncwarp();
    warp_logits(w, rows[warp], lg[warp]);
    __syncwarp();
    if (s < n) score[s] = fmaxf(lg[warp][lane * 3], fmaxf(lg[warp][lane * 3 + 1], lg[warp][lane * 3 + 2]));
}

__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }

// per-sample loss gradient of the max-pooled logit, block-reduced in shared memory
__global__ void __launch_bounds__(128) k_grad(const float* __restrict__ X, const float* __restrict__ Y,
                                              const int* __restrict__ idx, int nb, const __nv_bfloat16* __restrict__ pg,
                                              float pos_w, float* __restrict__ grad, double* __restrict__ loss) {
    __shared__ __nv_bfloat16 p[NPARAM];
    __shared__ float g[NPARAM];
    __shared__ float lsum[128];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
        p[i] = pg[i];
        g[i] = 0.0f;
    }
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    float my_loss = 0.0f;
    if (t < nb) {
        const int s = idx ? idx[t] : t;
        const float y = Y[s];
        float x[NIN], best = -INFINITY;
        int bd = 0;
        for (int d = 0; d < 3; ++d) {
            float xx[NIN];
#pragma unroll
            for (int k = 0; k < NIN; ++k) xx[k] = X[((long long)s * 3 + d) * NIN + k];
            const float z = forward(p, xx);
            if (z > best) {
                best = z;
                bd = d;
            }
        }
#pragma unroll
        for (int k = 0; k < NIN; ++k) x[k] = X[((long long)s * 3 + bd) * NIN + k];
        // forward of the winning direction, keeping the activations
        float a1[NH], h1[NH], a2[NH];
        for (int j = 0; j < NH; ++j) {
            float a = __bfloat162float(p[OFF_B1 + j]);
            for (int k = 0; k < NIN; ++k) a = fmaf(__bfloat162float(p[OFF_W1 + j * NIN + k]), x[k], a);
            a1[j] = a;
            h1[j] = fmaxf(a, 0.0f);
        }
        float z = __bfloat162float(p[OFF_B3]);
        for (int j = 0; j < NH; ++j) {
            float a = __bfloat162float(p[OFF_B2 + j]);
            for (int k = 0; k < NH; ++k) a = fmaf(__bfloat162float(p[OFF_W2 + j * NH + k]), h1[k], a);
            a2[j] = a;
            z = fmaf(__bfloat162float(p[OFF_W3 + j]), fmaxf(a, 0.0f), z);
        }
        // BCE with positive weight: -(w y log s(z) + (1-y) log(1-s(z)))
        my_loss = pos_w * y * softplus(-z) + (1.0f - y) * softplus(z);
        const float sg = 1.0f / (1.0f + expf(-z));
        const float dz = pos_w * y * (sg - 1.0f) + (1.0f - y) * sg;
        atomicAdd(&g[OFF_B3], dz);
        float ga2[NH];
        for (int j = 0; j < NH; ++j) {
            atomicAdd(&g[OFF_W3 + j], dz * fmaxf(a2[j], 0.0f));
            ga2[j] = a2[j] > 0.0f ? dz * __bfloat162float(p[OFF_W3 + j]) : 0.0f;
            atomicAdd(&g[OFF_B2 + j], ga2[j]);
        }
        for (int k = 0; k < NH; ++k) {
            float dh = 0.0f;
            for (int j = 0; j < NH; ++j) {
                atomicAdd(&g[OFF_W2 + j * NH + k], ga2[j] * h1[k]);
                dh = fmaf(ga2[j], __bfloat162float(p[OFF_W2 + j * NH + k]), dh);
            }
            const float ga1 = a1[k] > 0.0f ? dh : 0.0f;
            atomicAdd(&g[OFF_B1 + k], ga1);
            for (int i = 0; i < NIN; ++i) atomicAdd(&g[OFF_W1 + k * NIN + i], ga1 * x[i]);
        }
    }
    lsum[threadIdx.x] = my_loss;
    __syncthreads();
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) atomicAdd(&grad[i], g[i]);
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) s += lsum[q];
        atomicAdd(loss, s);
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, int t, float scale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * scale;
    m[i] = b1 * m[i] + (1.0f - b1) * gi;
    v[i] = b2 * v[i] + (1.0f - b2) * gi * gi;
    const float mh = m[i] / (1.0f - powf(b1, (float)t)), vh = v[i] / (1.0f - powf(b2, (float)t));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace mlp
}  // namespace hype

using namespace hype;
using namespace hype::mlp;

extern "C" int hype_mlp_nparam(void) { return NPARAM; }

namespace {
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { cudaFree(p); }
};
}  // namespace

#define MLP_ALLOC(buf, bytes)                              \
    do {                                                   \
        cudaError_t e__ = cudaMalloc(&(buf).p, (bytes));   \
        if (e__ != cudaSuccess) {                          \
            set_last_error("cudaMalloc", e__);             \
            return HYPE_ERR_NOMEM;                         \
        }                                                  \
    } while (0)

extern "C" int hype_mlp_score(const float* X, int n, const float* params, float* score) {
    if (!X || !params || !score || n < 0) return HYPE_ERR_ARG;
    if (n == 0) return HYPE_OK;
    DevBuf dX, dw, ds;
    MLP_ALLOC(dX, sizeof(float) * (size_t)n * 3 * NIN);
    MLP_ALLOC(dw, sizeof(MmaWeights));
    MLP_ALLOC(ds, sizeof(float) * (size_t)n);
    std::vector<__nv_bfloat16> q(NPARAM);
    for (int i = 0; i < NPARAM; ++i) q[i] = __float2bfloat16_rn(params[i]);
    MmaWeights hw;
    pack_weights(q.data(), hw);
    HYPE_CK(cudaMemcpy(dX.p, X, sizeof(float) * (size_t)n * 3 * NIN, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemcpy(dw.p, &hw, sizeof(MmaWeights), cudaMemcpyHostToDevice));
    k_score<<<cdiv(n, 128), 128>>>((const float*)dX.p, n, (const MmaWeights*)dw.p, (float*)ds.p);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpy(score, ds.p, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
    return HYPE_OK;
}

extern "C" int hype_mlp_grad(const float* X, const float* y, int n, const float* params, float pos_weight, float* grad,
                             double* loss) {
    if (!X || !y || !params || !grad || n <= 0) return HYPE_ERR_ARG;
    DevBuf dX, dy, dp, dq, dg, dl;
    MLP_ALLOC(dX, sizeof(float) * (size_t)n * 3 * NIN);
    MLP_ALLOC(dy, sizeof(float) * (size_t)n);
    MLP_ALLOC(dp, sizeof(float) * NPARAM);
    MLP_ALLOC(dq, sizeof(__nv_bfloat16) * NPARAM);
    MLP_ALLOC(dg, sizeof(float) * NPARAM);
    MLP_ALLOC(dl, sizeof(double));
    HYPE_CK(cudaMemcpy(dX.p, X, sizeof(float) * (size_t)n * 3 * NIN, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemcpy(dy.p, y, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemcpy(dp.p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemset(dg.p, 0, sizeof(float) * NPARAM));
    HYPE_CK(cudaMemset(dl.p, 0, sizeof(double)));
    k_to_bf16<<<cdiv(NPARAM, 256), 256>>>((const float*)dp.p, (__nv_bfloat16*)dq.p, NPARAM);
    k_grad<<<cdiv(n, 128), 128>>>((const float*)dX.p, (const float*)dy.p, nullptr, n, (const __nv_bfloat16*)dq.p, pos_weight,
                                  (float*)dg.p, (double*)dl.p);
    HYPE_LAUNCHED(2);
    HYPE_CK(cudaMemcpy(grad, dg.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    double l = 0.0;
    HYPE_CK(cudaMemcpy(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost));
    if (loss) *loss = l;
    return HYPE_OK;
}

// Adam on minibatches drawn by a seeded shuffle; params (FP32) in and out.
extern "C" int hype_mlp_train(const float* X, const float* y, int n, float* params, int epochs, int batch, float lr,
                              float pos_weight, unsigned seed, double* final_loss) {
    if (!X || !y || !params || n <= 0 || epochs < 0 || batch <= 0) return HYPE_ERR_ARG;
    DevBuf dX, dy, dp, dq, dg, dm, dv, dl, di;
    MLP_ALLOC(dX, sizeof(float) * (size_t)n * 3 * NIN);
    MLP_ALLOC(dy, sizeof(float) * (size_t)n);
    MLP_ALLOC(dp, sizeof(float) * NPARAM);
    MLP_ALLOC(dq, sizeof(__nv_bfloat16) * NPARAM);
    MLP_ALLOC(dg, sizeof(float) * NPARAM);
    MLP_ALLOC(dm, sizeof(float) * NPARAM);
    MLP_ALLOC(dv, sizeof(float) * NPARAM);
    MLP_ALLOC(dl, sizeof(double));
    MLP_ALLOC(di, sizeof(int) * (size_t)n);
    HYPE_CK(cudaMemcpy(dX.p, X, sizeof(float) * (size_t)n * 3 * NIN, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemcpy(dy.p, y, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemcpy(dp.p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    HYPE_CK(cudaMemset(dm.p, 0, sizeof(float) * NPARAM));
    HYPE_CK(cudaMemset(dv.p, 0, sizeof(float) * NPARAM));
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    unsigned long long st = seed * 6364136223846793005ull + 1442695040888963407ull;
    int t = 0;
    double last = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = n - 1; i > 0; --i) {  // Fisher-Yates with a 64-bit LCG
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            const int j = (int)((st >> 33) % (unsigned long long)(i + 1));
            const int tmp = order[i];
            order[i] = order[j];
            order[j] = tmp;
        }
        HYPE_CK(cudaMemcpy(di.p, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
        double eloss = 0.0;
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nb = (n - b0) < batch ? (n - b0) : batch;
            HYPE_CK(cudaMemsetAsync(dg.p, 0, sizeof(float) * NPARAM));
            HYPE_CK(cudaMemsetAsync(dl.p, 0, sizeof(double)));
            k_to_bf16<<<cdiv(NPARAM, 256), 256>>>((const float*)dp.p, (__nv_bfloat16*)dq.p, NPARAM);
            k_grad<<<cdiv(nb, 128), 128>>>((const float*)dX.p, (const float*)dy.p, (const int*)di.p + b0, nb,
                                           (const __nv_bfloat16*)dq.p, pos_weight, (float*)dg.p, (double*)dl.p);
            ++t;
            k_adam<<<cdiv(NPARAM, 256), 256>>>((float*)dp.p, (const float*)dg.p, (float*)dm.p, (float*)dv.p, NPARAM, lr, 0.9f,
                                               0.999f, 1e-8f, t, 1.0f / nb);
            HYPE_LAUNCHED(3);
            double l = 0.0;
            HYPE_CK(cudaMemcpy(&l, dl.p, sizeof(double), cudaMemcpyDeviceToHost));
            eloss += l;
        }
        last = eloss / n;
    }
    HYPE_CK(cudaMemcpy(params, dp.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
    if (final_loss) *final_loss = last;
    return HYPE_OK;
}
