// mphase2d_f32.cu -- the FP32 recon/flux form of the 2D multiphase RHS (HYPE_PREC_FP32),
// in its own translation unit so that it compiles with FMA contraction: the FP64 kernels
// in mphase2d.cu keep the reference's rounding and are compiled without it.
#include "euler_kernels.cuh"
#include "hype_common.cuh"
#include "mphase2d_dev.cuh"

namespace hype {
namespace mp2d {

// conserved -> primitive for the FP32 form: the pressure (p = (g - 1)(E - rho |u|^2 / 2) - g pi,
// where the stiffness term cancels most of E) and every other value formed in FP64 as cons2prim
// does, with its divisions as FP64 reciprocals within an ulp (the values are rounded to FP32 next),
// written as the FP32 copy the reconstruction reads
// the mixture rules' constants, formed once on the host: (g1 - 1)(g2 - 1), g_k p_k / (g_k - 1)
struct MixConst {
    double c, s1, s2;
};

__global__ void __launch_bounds__(256) k_mp_prim_f32(const double* __restrict__ U, float* __restrict__ P, Eos e,
                                                     MixConst mc, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    const double c = mc.c, s1 = mc.s1, s2 = mc.s2;
    if (e.model == HYPE_MP_DI4) {
        const double Q0 = U[q], Q1 = U[N + q], Q2 = U[2 * N + q], Q3 = U[3 * N + q], phi = U[4 * N + q];
        const double g = 1.0 + c * euler::recip_wide((1.0 - phi) * (e.g1 - 1.0) + phi * (e.g2 - 1.0));
        const double pi = ((g - 1.0) * euler::recip_wide(g)) * (s1 * phi + s2 * (1.0 - phi));
        const double irho = euler::recip_wide(Q0);
        P[q] = (float)Q0;
        P[N + q] = (float)(irho * Q1);
        P[2 * N + q] = (float)(irho * Q2);
        P[3 * N + q] = (float)((g - 1.0) * (Q3 - 0.5 * irho * (Q1 * Q1 + Q2 * Q2)) - g * pi);
        P[4 * N + q] = (float)phi;
    } else {
        const double Q0 = U[q], Q1 = U[N + q], Q2 = U[2 * N + q], Q3 = U[3 * N + q], Q4 = U[4 * N + q];
        const double a1 = U[5 * N + q], a2 = 1.0 - a1;
        const double g = 1.0 + c * euler::recip_wide((e.g2 - 1.0) * a1 + (e.g1 - 1.0) * a2);
        const double pi = ((g - 1.0) * euler::recip_wide(g)) * (s1 * a1 + s2 * a2);
        const double rho = Q0 + Q1, irho = euler::recip_wide(rho);
        const double u = Q2 * irho, v = Q3 * irho;
        P[q] = (float)(Q0 * euler::recip_wide(a1));
        P[N + q] = (float)(Q1 * euler::recip_wide(a2));
        P[2 * N + q] = (float)u;
        P[3 * N + q] = (float)v;
        P[4 * N + q] = (float)((g - 1.0) * (Q4 - 0.5 * rho * (u * u + v * v)) - g * pi);
        P[5 * N + q] = (float)a1;
    }
}

// the primitives, the reconstruction (plain or indicator-gated) and the two face-flux launches of one
// RHS of the FP32 form (Pf: its FP32 primitives)
int launch_rhs_f32(int model, bool learned, const double* Win, float* Pf, void* T, float* F, float* G, const Geo& g,
                   const Eos& e, DevScalars* ds, int slot, const mlp::MmaWeights* mlp, float logit_thr,
                   unsigned long long* flagged, const GateStep& gs, cudaStream_t st) {
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4));
    const dim3 gx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4)), gy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4));
    const MixConst mc{(e.g1 - 1.0) * (e.g2 - 1.0), e.g1 * e.p1 / (e.g1 - 1.0), e.g2 * e.p2 / (e.g2 - 1.0)};
    k_mp_prim_f32<<<cdiv(g.N, 256), 256, 0, st>>>(Win, Pf, e, mc, g.N);
    const float* P = Pf;
#define MP_LAUNCH_F32(M)                                                                                       \
    do {                                                                                                       \
        if (gs.on)                                                                                             \
            launch_gated_recon<float, M, float>(P, (float*)T, g, e, ds, mlp, logit_thr, flagged, gs, st);      \
        else if (learned)                                                                                      \
            k_mp_recon_learned<float, M, float><<<gr, br, 0, st>>>(P, (float*)T, g, e, ds, mlp, logit_thr,     \
                                                                   flagged);                                   \
        else                                                                                                   \
            k_mp_recon<float, M, float><<<gr, br, 0, st>>>(P, (float*)T, g, e, ds);                            \
        k_mp_faces<float, M, 0><<<gx, br, 0, st>>>((const float*)T, F, g, e, ds, slot);                        \
        k_mp_faces<float, M, 1><<<gy, br, 0, st>>>((const float*)T, G, g, e, ds, slot);                        \
    } while (0)
    if (model == HYPE_MP_DI4) MP_LAUNCH_F32(HYPE_MP_DI4);
    else MP_LAUNCH_F32(HYPE_MP_KAPILA5);
#undef MP_LAUNCH_F32
    return HYPE_OK;
}

// The FP32 form's stage update from its FP32 face fluxes: the divergence of each conserved variable
// in FP32 (the flux differences exact where the two fluxes lie within a factor 2, i.e. in smooth
// flow); the volume-fraction term (a u)' - a u', which cancels, and the stage combination are
// formed in FP64 as k_mp_update does.
// Win, X, Y and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_mp_update_f32(const float* __restrict__ F, const float* __restrict__ G,
                                                       const double* Win, const double* X, const double* Y, double* out,
                                                       Geo g, double r1_h, Stage st, const DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    const int nv = g.nv, ia = nv - 1;
    const long long nfx = (long long)(g.nx + 1) * g.ny, nfy = (long long)g.nx * (g.ny + 1);
    const long long fxl = (long long)j * (g.nx + 1) + i, fyl = (long long)j * g.nx + i;
    const long long cell = (long long)j * g.nx + i;
    const double a = Win[ia * g.N + cell];
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt / st.d;
    const float r1hf = (float)r1_h;
    for (int c = 0; c < nv; ++c) {
        double L;
        if (c == ia) {
            const double fr = F[c * nfx + fxl + 1], fl = F[c * nfx + fxl];
            const double ur = F[(c + 1) * nfx + fxl + 1], ul = F[(c + 1) * nfx + fxl];
            const double gt = G[c * nfy + fyl + g.nx], gb = G[c * nfy + fyl];
            const double vt = G[(c + 1) * nfy + fyl + g.nx], vb = G[(c + 1) * nfy + fyl];
            L = -r1_h * ((fr - a * ur) - (fl - a * ul)) - r1_h * ((gt - a * vt) - (gb - a * vb));
        } else {
            const float dx = F[c * nfx + fxl + 1] - F[c * nfx + fxl];
            const float dy = G[c * nfy + fyl + g.nx] - G[c * nfy + fyl];
            L = (double)(-r1hf * (dx + dy));
        }
        double v;
        if (st.rhs_only) {
            v = L;
        } else {
            v = st.a * X[c * g.N + cell] + cdt * L;
            if (st.b != 0.0) v += st.b * Y[c * g.N + cell];
        }
        out[c * g.N + cell] = v;
    }
}

void launch_update_f32(const float* F, const float* G, const double* Win, const double* X, const double* Y, double* out,
                       const Geo& g, double r1_h, Stage st, const DevScalars* ds, cudaStream_t stream) {
    const dim3 b(32, 8), gr(cdiv(g.nx, 32), cdiv(g.ny, 8));
    k_mp_update_f32<<<gr, b, 0, stream>>>(F, G, Win, X, Y, out, g, r1_h, st, ds);
}

}  // namespace mp2d
}  // namespace hype
