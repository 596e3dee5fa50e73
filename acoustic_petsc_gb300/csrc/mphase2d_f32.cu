// mphase2d_f32.cu -- the FP32 recon/flux form of the 2D multiphase RHS (HYPE_PREC_FP32),
// in its own translation unit so that it compiles with FMA contraction: the FP64 kernels
// in mphase2d.cu keep the reference's rounding and are compiled without it.
#include "hype_common.cuh"
#include "mphase2d_dev.cuh"

namespace hype {
namespace mp2d {

// the reconstruction (plain or indicator-gated) and the two face-flux launches of one RHS
int launch_rhs_f32(int model, bool learned, const double* P, void* T, double* F, double* G, const Geo& g, const Eos& e,
                   DevScalars* ds, int slot, const mlp::MmaWeights* mlp, float logit_thr, unsigned long long* flagged,
                   cudaStream_t st) {
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4));
    const dim3 gx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4)), gy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4));
#define MP_LAUNCH_F32(M)                                                                                       \
    do {                                                                                                       \
        if (learned)                                                                                           \
            k_mp_recon_learned<float, M><<<gr, br, 0, st>>>(P, (float*)T, g, e, ds, mlp, logit_thr, flagged);  \
        else                                                                                                   \
            k_mp_recon<float, M><<<gr, br, 0, st>>>(P, (float*)T, g, e, ds);                                   \
        k_mp_faces<float, M, 0><<<gx, br, 0, st>>>((const float*)T, F, g, e, ds, slot);                        \
        k_mp_faces<float, M, 1><<<gy, br, 0, st>>>((const float*)T, G, g, e, ds, slot);                        \
    } while (0)
    if (model == HYPE_MP_DI4) MP_LAUNCH_F32(HYPE_MP_DI4);
    else MP_LAUNCH_F32(HYPE_MP_KAPILA5);
#undef MP_LAUNCH_F32
    return HYPE_OK;
}

}  // namespace mp2d
}  // namespace hype
