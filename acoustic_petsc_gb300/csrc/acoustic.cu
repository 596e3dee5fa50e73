// acoustic.cu -- the acoustic finite-volume path of HyPE (3d/weno4/plane_wave):
// the wave equation u_tt = c^2 lap u as the first-order system (u, v = u_t),
//   du/dt = v,   dv/dt = c^2 div grad u,
// with cell averages of u reconstructed by CWENO4 (the reference runs its optimal-
// weight limit, gammaHi = 1: the R4 polynomial), the normal gradient of the
// polynomial at the 2x2 Gauss points of every face, the central flux
// c^2 (grad_L + grad_R) . n / 2 (pde.c:12-34), and SSPRK(4,3) with a fixed dt.
//
// Per RHS evaluation (rhs_function.c:12-345):
//   k_ac_ghost   u with 3 ghost layers: periodic wrap, or the adiabatic wall's odd
//                mirror u_ghost = -u (rhs_function.c:43-131);
//   k_ac_recon   per extended cell: the 33-point stencil, CWENO4 / R4 coefficients,
//                the 24 face-normal gradients (evaluate_grad, reconstruction.c:25-34);
//   k_ac_faces   per face: 4 Gauss points of the central flux (:176-287);
//   k_ac_update  RHS (v, (1/h) sum of flux differences) fused with the stage
//                combination (:289-300), plus the point source of 3d/weno4/point_source
//                (rhs_function.c:337-346: Source(t)/h^3 in one cell, u at the receiver).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "euler_df64.cuh"
#include "euler_kernels.cuh"
#include "point_source.cuh"

namespace hype {
namespace acoustic {

using euler::NTR;

struct Geo {
    int nx, ny, nz;
    int bc[6];
    long long N, NE;  // owned cells, extended cells (n+2)^3
    int ex;           // extended x extent
    int gx, gy;       // ghosted extents (n + 6)
    long long GN;     // ghosted cells
};

constexpr int GW = 3;

__device__ __forceinline__ long long ext_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + 1) * (g.ny + 2) + (j + 1)) * (long long)g.ex + (i + 1);
}
__device__ __forceinline__ long long ghost_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + GW) * g.gy + (j + GW)) * g.gx + (i + GW);
}

// the boundary map of one axis: periodic wrap, or the mirror of the adiabatic wall
// (whose ghost value is the negated mirror value)
__device__ __forceinline__ int amap(int i, int n, int blo, int bhi, int* flip) {
    return bmap(i, n, blo == HYPE_BC_PERIODIC ? HYPE_BC_PERIODIC : HYPE_BC_REFLECTIVE,
                bhi == HYPE_BC_PERIODIC ? HYPE_BC_PERIODIC : HYPE_BC_REFLECTIVE, flip);
}

__device__ __forceinline__ void put_g(double* p, double v) { *p = v; }
__device__ __forceinline__ void put_g(df64* p, double v) { *p = df_from_double(v); }

// G: the ghosted u in FP64, or (HYPE_PREC_DF64) as double-float pairs
template <typename GT>
__global__ void __launch_bounds__(128) k_ac_ghost(const double* __restrict__ U, GT* __restrict__ G, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - GW;
    const int j = blockIdx.y - GW, k = blockIdx.z - GW;
    if (i >= g.nx + GW) return;
    int fi = 0, fj = 0, fk = 0;
    const int mi = amap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = amap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const int mk = amap(k, g.nz, g.bc[4], g.bc[5], &fk);
    double v = __ldg(U + ((long long)mk * g.ny + mj) * g.nx + mi);  // component u
    if ((fi + fj + fk) & 1) v = -v;
    put_g(G + ghost_index(g, i, j, k), v);
}

// gradient component D of the 20-term polynomial at (x, y, z), times h
template <int D>
__device__ __forceinline__ double grad_poly(const double* c, double x, double y, double z) {
    constexpr double r1_12 = 1. / 12., r3_20 = 3. / 20.;
    if (D == 0)
        return c[1] + 2.0 * c[4] * x + c[7] * y + c[9] * z + c[10] * (3.0 * x * x - r3_20) + 2.0 * c[13] * x * y +
               c[14] * (y * y - r1_12) + 2.0 * c[17] * x * z + c[18] * (z * z - r1_12) + c[19] * y * z;
    if (D == 1)
        return c[2] + 2.0 * c[5] * y + c[7] * x + c[8] * z + c[11] * (3.0 * y * y - r3_20) + c[13] * (x * x - r1_12) +
               2.0 * c[14] * x * y + 2.0 * c[15] * y * z + c[16] * (z * z - r1_12) + c[19] * x * z;
    return c[3] + 2.0 * c[6] * z + c[8] * y + c[9] * x + c[12] * (3.0 * z * z - r3_20) + c[15] * (y * y - r1_12) +
           2.0 * c[16] * y * z + c[17] * (x * x - r1_12) + 2.0 * c[18] * x * z + c[19] * x * y;
}

// grad_poly<D> at the 8 Gauss points of the two faces normal to D at once.  On a face
// x_D = +-1/2 with tangential coordinates (t1, t2) = +-GPT (t1^2 = t2^2 = GPT^2) the normal
// derivative is A + B1 t1 + B2 t2 + B12 t1 t2 with
//   A   = c_D + 0.6 c_DDD + (c_t1t1D + c_t2t2D)(GPT^2 - 1/12) +- c_DD     (3 x^2 - 3/20 = 0.6, 2x = +-1)
//   B1  = c_Dt1 +- c_DDt1,  B2 = c_Dt2 +- c_DDt2,  B12 = c_xyz,
// about 14 operations per face instead of 4 evaluations of the 10-term gradient.
template <int D>
__device__ __forceinline__ void face_normal_grads(const double* c, double* __restrict__ T, long long NE, long long e) {
    constexpr double gp = euler::GPT, g2 = euler::GPT * euler::GPT, q = euler::GPT * euler::GPT - 1. / 12.;
    // coefficient slots of the 20-term basis (grad_poly above): linear, square, cube of D; the
    // cross x_D t; x_D^2 t; t^2 x_D for both tangential axes
    constexpr int LIN = 1 + D, SQ = 4 + D, CUBE = 10 + D;
    constexpr int X1 = D == 0 ? 7 : D == 1 ? 7 : 9;    // c * x_D * t1
    constexpr int X2 = D == 0 ? 9 : D == 1 ? 8 : 8;    // c * x_D * t2
    constexpr int DD1 = D == 0 ? 13 : D == 1 ? 14 : 18;  // c * x_D^2 * t1 term (derivative 2 x_D t1)
    constexpr int DD2 = D == 0 ? 17 : D == 1 ? 15 : 16;  // c * x_D^2 * t2 term
    constexpr int TT1 = D == 0 ? 14 : D == 1 ? 13 : 17;  // c * (t1^2 - 1/12) x_D
    constexpr int TT2 = D == 0 ? 18 : D == 1 ? 16 : 15;  // c * (t2^2 - 1/12) x_D
    const double E = c[LIN] + 0.6 * c[CUBE] + (c[TT1] + c[TT2]) * q;
    const double w = g2 * c[19];
#pragma unroll
    for (int sn = 0; sn < 2; ++sn) {
        const double A = sn ? E + c[SQ] : E - c[SQ];
        const double u = gp * (sn ? c[X1] + c[DD1] : c[X1] - c[DD1]);
        const double v = gp * (sn ? c[X2] + c[DD2] : c[X2] - c[DD2]);
        const double Ap = A + w, Am = A - w, s = u + v, d = u - v;
        double* Tq = T + (long long)((2 * D + sn) * 4) * NE + e;
        Tq[0 * NE] = Ap - s;  // (t1 -, t2 -)
        Tq[1 * NE] = Am - d;  // (t1 -, t2 +)
        Tq[2 * NE] = Am + d;  // (t1 +, t2 -)
        Tq[3 * NE] = Ap + s;  // (t1 +, t2 +)
    }
}

// T[face][gp][extended cell]: the face-normal gradient (times h) at the 4 Gauss points
// of the 6 faces; Gauss point q = 2 (t1 > 0) + (t2 > 0), (t1, t2) the remaining axes
__global__ void __launch_bounds__(128) k_ac_recon(const double* __restrict__ G, double* __restrict__ T, Geo g, int linear) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > g.nx || j > g.ny) return;
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    if (gi + gj + gk > 1) return;
    const double* p = G + ghost_index(g, i, j, k);
    const int sy = g.gx, sz = g.gx * g.gy;
    double s[33], cf[20];
    s[0] = __ldg(p);
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
        s[euler::S1(0, off)] = __ldg(p + off);
        s[euler::S1(1, off)] = __ldg(p + off * sy);
        s[euler::S1(2, off)] = __ldg(p + off * sz);
    }
#pragma unroll
    for (int sa = 0; sa < 2; ++sa)
#pragma unroll
        for (int sb = 0; sb < 2; ++sb) {
            s[euler::SQ(0, sa, 1, sb)] = __ldg(p + (2 * sa - 1) + (2 * sb - 1) * sy);
            s[euler::SQ(1, sa, 2, sb)] = __ldg(p + (2 * sa - 1) * sy + (2 * sb - 1) * sz);
            s[euler::SQ(0, sa, 2, sb)] = __ldg(p + (2 * sa - 1) + (2 * sb - 1) * sz);
        }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) s[euler::SO(a, b, d)] = __ldg(p + (2 * a - 1) + (2 * b - 1) * sy + (2 * d - 1) * sz);
    euler::cweno4<double>(s, linear != 0, cf);
    const long long e = ext_index(g, i, j, k);
    face_normal_grads<0>(cf, T, g.NE, e);
    face_normal_grads<1>(cf, T, g.NE, e);
    face_normal_grads<2>(cf, T, g.NE, e);
}

// the double-float form: face_normal_grads in pairs of FP32 numbers
template <int D>
__device__ __forceinline__ void face_normal_grads_df(const df64* c, df64* __restrict__ T, long long NE, long long e) {
    constexpr double gp = euler::GPT, g2 = euler::GPT * euler::GPT, q = euler::GPT * euler::GPT - 1. / 12.;
    constexpr int LIN = 1 + D, SQ = 4 + D, CUBE = 10 + D;
    constexpr int X1 = D == 0 ? 7 : D == 1 ? 7 : 9;
    constexpr int X2 = D == 0 ? 9 : D == 1 ? 8 : 8;
    constexpr int DD1 = D == 0 ? 13 : D == 1 ? 14 : 18;
    constexpr int DD2 = D == 0 ? 17 : D == 1 ? 15 : 16;
    constexpr int TT1 = D == 0 ? 14 : D == 1 ? 13 : 17;
    constexpr int TT2 = D == 0 ? 18 : D == 1 ? 16 : 15;
    const df64 E = c[LIN] + (c[CUBE] * dfc(0.6) + (c[TT1] + c[TT2]) * dfc(q));
    const df64 w = c[19] * dfc(g2);
#pragma unroll
    for (int sn = 0; sn < 2; ++sn) {
        const df64 A = sn ? E + c[SQ] : E - c[SQ];
        const df64 u = (sn ? c[X1] + c[DD1] : c[X1] - c[DD1]) * dfc(gp);
        const df64 v = (sn ? c[X2] + c[DD2] : c[X2] - c[DD2]) * dfc(gp);
        const df64 Ap = A + w, Am = A - w, s = u + v, d = u - v;
        df64* Tq = T + (long long)((2 * D + sn) * 4) * NE + e;
        Tq[0 * NE] = Ap - s;
        Tq[1 * NE] = Am - d;
        Tq[2 * NE] = Am + d;
        Tq[3 * NE] = Ap + s;
    }
}

// k_ac_recon in double-float: the R4 / CWENO4 coefficients (euler_df64.cuh) and the 24 face-
// normal gradients, kept as pairs for k_ac_faces_df
__global__ void __launch_bounds__(128, 2) k_ac_recon_df(const df64* __restrict__ G, df64* __restrict__ T, Geo g,
                                                        int linear) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > g.nx || j > g.ny) return;
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    if (gi + gj + gk > 1) return;
    const df64* p = G + ghost_index(g, i, j, k);
    const int sy = g.gx, sz = g.gx * g.gy;
    df64 s[33], cf[20];
    s[0] = p[0];
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
        s[euler::S1(0, off)] = p[off];
        s[euler::S1(1, off)] = p[off * sy];
        s[euler::S1(2, off)] = p[off * sz];
    }
#pragma unroll
    for (int sa = 0; sa < 2; ++sa)
#pragma unroll
        for (int sb = 0; sb < 2; ++sb) {
            s[euler::SQ(0, sa, 1, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sy];
            s[euler::SQ(1, sa, 2, sb)] = p[(2 * sa - 1) * sy + (2 * sb - 1) * sz];
            s[euler::SQ(0, sa, 2, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sz];
        }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) s[euler::SO(a, b, d)] = p[(2 * a - 1) + (2 * b - 1) * sy + (2 * d - 1) * sz];
    euler::cweno4_df(s, linear != 0, cf);
    const long long e = ext_index(g, i, j, k);
    face_normal_grads_df<0>(cf, T, g.NE, e);
    face_normal_grads_df<1>(cf, T, g.NE, e);
    face_normal_grads_df<2>(cf, T, g.NE, e);
}

// k_ac_faces in double-float: 1/8 c^2 sum_q (gL + gR), rounded once to FP64
template <int D>
__global__ void __launch_bounds__(128) k_ac_faces_df(const df64* __restrict__ T, double* __restrict__ F, Geo g,
                                                     double c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    if (i >= fx || j >= fy) return;
    const long long eR = ext_index(g, i, j, k);
    const long long eL = ext_index(g, i - (D == 0), j - (D == 1), k - (D == 2));
    df64 sum = df64{0.0f, 0.0f};
#pragma unroll
    for (int q = 0; q < 4; ++q)
        sum = sum + (T[(long long)((2 * D + 1) * 4 + q) * g.NE + eL] + T[(long long)((2 * D) * 4 + q) * g.NE + eR]);
    F[((long long)k * fy + j) * fx + i] = df_to_double(df_scale(sum * df_from_double(c2), 0.125f));
}

// face flux sum_q w_q c^2 (gL + gR) / 2, w_q = 1/4 (the gradients carry a factor h
// that the divergence's 1/h^2 removes)
template <int D>
__global__ void __launch_bounds__(128) k_ac_faces(const double* __restrict__ T, double* __restrict__ F, Geo g, double c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    if (i >= fx || j >= fy) return;
    const long long eR = ext_index(g, i, j, k);
    const long long eL = ext_index(g, i - (D == 0), j - (D == 1), k - (D == 2));
    double flux = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double gL = T[(long long)((2 * D + 1) * 4 + q) * g.NE + eL];
        const double gR = T[(long long)((2 * D) * 4 + q) * g.NE + eR];
        flux += 0.25 * (0.5 * (c2 * gR + c2 * gL));
    }
    F[((long long)k * fy + j) * fx + i] = flux;
}

struct Stage {
    double a, b, c;  // out = a U + b W + (c dt) L, or (rhs_only) out = L
    int rhs_only;
};

// U, W, out: SoA [2][N]; L = (v, (1/h^2) sum of face-flux differences)
// U, W and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_ac_update(const double* __restrict__ Fx, const double* __restrict__ Fy,
                                                   const double* __restrict__ Fz, const double* U,
                                                   const double* W, double* out, Geo g,
                                                   double r1_h2, Stage st, double dt, SourceArgs src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long cell = ((long long)k * g.ny + j) * g.nx + i;
    const long long ix = ((long long)k * g.ny + j) * (g.nx + 1) + i;
    const long long iy = ((long long)k * (g.ny + 1) + j) * g.nx + i;
    const long long iz = cell;
    double div = r1_h2 * (Fx[ix + 1] - Fx[ix]) + r1_h2 * (Fy[iy + g.nx] - Fy[iy]) +
                 r1_h2 * (Fz[iz + (long long)g.nx * g.ny] - Fz[iz]);
    if (cell == src.src_cell) div += src.src_val;
    if (cell == src.rec_cell) *src.slot = W[cell];  // read before out (which may alias W) is written
    const double L[2] = {W[g.N + cell], div};
    const double cdt = st.c * dt;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        double v;
        if (st.rhs_only) v = L[c];
        else if (st.a != 0.0) v = st.a * U[c * g.N + cell] + st.b * W[c * g.N + cell] + cdt * L[c];
        else v = W[c * g.N + cell] + cdt * L[c];
        out[c * g.N + cell] = v;
    }
}

__global__ void k_ac_aos2soa(const double* __restrict__ a, double* __restrict__ s, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    s[q] = a[2 * q];
    s[N + q] = a[2 * q + 1];
}
__global__ void k_ac_soa2aos(const double* __restrict__ s, double* __restrict__ a, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    a[2 * q] = s[q];
    a[2 * q + 1] = s[N + q];
}

}  // namespace acoustic
}  // namespace hype

using namespace hype;
using namespace hype::acoustic;

struct hype_acoustic {
    hype_acoustic_params p;
    Geo g;
    cudaStream_t stream = nullptr;
    double *U = nullptr, *W = nullptr, *L = nullptr, *S = nullptr, *Gh = nullptr, *T = nullptr;
    double *Fx = nullptr, *Fy = nullptr, *Fz = nullptr, *aos = nullptr;
    PointSource ps;
};

static int ac_rhs(hype_acoustic* a, const double* Win) {
    const Geo& g = a->g;
    if (a->p.precision == HYPE_PREC_DF64) {
        k_ac_ghost<df64><<<dim3(cdiv(g.gx, 128), g.gy, g.nz + 2 * GW), 128, 0, a->stream>>>(Win, (df64*)a->Gh, g);
        k_ac_recon_df<<<dim3(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2), dim3(32, 4), 0, a->stream>>>(
            (const df64*)a->Gh, (df64*)a->T, g, a->p.recon == HYPE_RECON_LINEAR4);
        const double c2 = a->p.c * a->p.c;
        const dim3 bf(32, 4);
        const df64* T = (const df64*)a->T;
        k_ac_faces_df<0><<<dim3(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), bf, 0, a->stream>>>(T, a->Fx, g, c2);
        k_ac_faces_df<1><<<dim3(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz), bf, 0, a->stream>>>(T, a->Fy, g, c2);
        k_ac_faces_df<2><<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1), bf, 0, a->stream>>>(T, a->Fz, g, c2);
        HYPE_LAUNCHED(5);
        return HYPE_OK;
    }
    k_ac_ghost<double><<<dim3(cdiv(g.gx, 128), g.gy, g.nz + 2 * GW), 128, 0, a->stream>>>(Win, a->Gh, g);
    k_ac_recon<<<dim3(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2), dim3(32, 4), 0, a->stream>>>(
        a->Gh, a->T, g, a->p.recon == HYPE_RECON_LINEAR4);
    const double c2 = a->p.c * a->p.c;
    const dim3 bf(32, 4);
    k_ac_faces<0><<<dim3(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), bf, 0, a->stream>>>(a->T, a->Fx, g, c2);
    k_ac_faces<1><<<dim3(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz), bf, 0, a->stream>>>(a->T, a->Fy, g, c2);
    k_ac_faces<2><<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1), bf, 0, a->stream>>>(a->T, a->Fz, g, c2);
    HYPE_LAUNCHED(5);
    return HYPE_OK;
}

// t: the time of this RHS evaluation (the point source's argument)
static int ac_update(hype_acoustic* a, const double* U, const double* W, double* out, Stage st, double dt, double t) {
    const Geo& g = a->g;
    k_ac_update<<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 8), g.nz), dim3(32, 8), 0, a->stream>>>(
        a->Fx, a->Fy, a->Fz, U, W, out, g, 1.0 / (a->p.h * a->p.h), st, dt, source_args(a->ps, t));
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

extern "C" int hype_acoustic_create(const hype_acoustic_params* p, hype_acoustic** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3 || !(p->h > 0) || !(p->c > 0) || !(p->dt > 0)) return HYPE_ERR_ARG;
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] != HYPE_BC_PERIODIC && p->bc[f] != HYPE_BC_ADIABATIC) return HYPE_ERR_ARG;
    for (int d = 0; d < 3; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (p->recon != HYPE_RECON_LINEAR4 && p->recon != HYPE_RECON_CWENO4) return HYPE_ERR_ARG;
    if (p->precision != HYPE_PREC_FP64 && p->precision != HYPE_PREC_DF64) return HYPE_ERR_ARG;
    hype_acoustic* a = new hype_acoustic();
    a->p = *p;
    Geo& g = a->g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    for (int f = 0; f < 6; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny * p->nz;
    g.NE = (long long)(p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    g.ex = p->nx + 2;
    g.gx = p->nx + 2 * GW;
    g.gy = p->ny + 2 * GW;
    g.GN = (long long)g.gx * g.gy * (p->nz + 2 * GW);
    const size_t sN = sizeof(double) * 2 * (size_t)g.N;
    cudaError_t ce = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    double** bufs[] = {&a->U, &a->W, &a->L, &a->S, &a->aos};
    for (auto b : bufs)
        if (ce == cudaSuccess) ce = cudaMalloc((void**)b, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->Gh, sizeof(double) * (size_t)g.GN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->T, sizeof(double) * NTR * (size_t)g.NE);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->Fx, sizeof(double) * (size_t)(p->nx + 1) * p->ny * p->nz);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->Fy, sizeof(double) * (size_t)p->nx * (p->ny + 1) * p->nz);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->Fz, sizeof(double) * (size_t)p->nx * p->ny * (p->nz + 1));
    if (ce != cudaSuccess) {
        set_last_error("hype_acoustic_create", ce);
        hype_acoustic_destroy(a);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = a;
    return HYPE_OK;
}

extern "C" void hype_acoustic_destroy(hype_acoustic* a) {
    if (!a) return;
    if (a->stream) cudaStreamSynchronize(a->stream);
    cudaFree(a->U); cudaFree(a->W); cudaFree(a->L); cudaFree(a->S); cudaFree(a->aos); cudaFree(a->Gh); cudaFree(a->T);
    cudaFree(a->Fx); cudaFree(a->Fy); cudaFree(a->Fz);
    a->ps.release();
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
}

static int ac_h2d(hype_acoustic* a, const double* aos, double* soa) {
    const long long N = a->g.N;
    HYPE_CK(cudaMemcpyAsync(a->aos, aos, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, a->stream));
    k_ac_aos2soa<<<cdiv(N, 256), 256, 0, a->stream>>>(a->aos, soa, N);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int ac_d2h(hype_acoustic* a, const double* soa, double* aos) {
    const long long N = a->g.N;
    k_ac_soa2aos<<<cdiv(N, 256), 256, 0, a->stream>>>(soa, a->aos, N);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, a->aos, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, a->stream));
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" int hype_acoustic_upload(hype_acoustic* a, const double* U_aos) {
    if (!a || !U_aos) return HYPE_ERR_ARG;
    int rc = ac_h2d(a, U_aos, a->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" int hype_acoustic_download(hype_acoustic* a, double* U_aos) {
    if (!a || !U_aos) return HYPE_ERR_ARG;
    return ac_d2h(a, a->U, U_aos);
}

extern "C" int hype_acoustic_rhs_t(hype_acoustic* a, double t, const double* U_aos, double* RHS_aos) {
    if (!a || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc = ac_h2d(a, U_aos, a->S);
    if (rc || (rc = ac_rhs(a, a->S))) return rc;
    if ((rc = ac_update(a, a->S, a->S, a->L, Stage{0.0, 0.0, 0.0, 1}, 0.0, t))) return rc;
    return ac_d2h(a, a->L, RHS_aos);
}

extern "C" int hype_acoustic_rhs(hype_acoustic* a, const double* U_aos, double* RHS_aos) {
    return hype_acoustic_rhs_t(a, 0.0, U_aos, RHS_aos);
}

extern "C" int hype_acoustic_set_point_source(hype_acoustic* a, int isx, int isy, int isz, double f0, int irx, int iry,
                                              int irz, int trace_capacity) {
    if (!a || trace_capacity < 0) return HYPE_ERR_ARG;
    const Geo& g = a->g;
    const bool src = isx >= 0, rec = irx >= 0;
    if (src && (isx >= g.nx || isy < 0 || isy >= g.ny || isz < 0 || isz >= g.nz || !(f0 > 0))) return HYPE_ERR_ARG;
    if (rec && (irx >= g.nx || iry < 0 || iry >= g.ny || irz < 0 || irz >= g.nz)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    PointSource& ps = a->ps;
    ps.release();
    ps = PointSource();
    ps.src_on = src;
    ps.src_cell = src ? ((long long)isz * g.ny + isy) * g.nx + isx : -1;
    ps.f0 = f0;
    ps.scale = 1. / ((a->p.h) * (a->p.h) * (a->p.h));  // r1_h3, rhs_function.c:25
    ps.rec_on = rec;
    ps.rec_cell = rec ? ((long long)irz * g.ny + iry) * g.nx + irx : -1;
    if (rec && trace_capacity > 0) {
        cudaError_t ce = cudaMalloc((void**)&ps.trace, sizeof(double) * (size_t)trace_capacity);
        if (ce != cudaSuccess) {
            set_last_error("hype_acoustic_set_point_source", ce);
            return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
        }
        ps.capacity = trace_capacity;
    }
    return HYPE_OK;
}

extern "C" int hype_acoustic_trace(hype_acoustic* a, double* t, double* u, int max, long long* count) {
    if (!a || max < 0 || ((!t || !u) && max > 0)) return HYPE_ERR_ARG;
    const PointSource& ps = a->ps;
    const int n = (int)(ps.count < ps.capacity ? ps.count : ps.capacity);
    const int m = n < max ? n : max;
    if (m > 0) {
        HYPE_CK(cudaMemcpyAsync(u, ps.trace, sizeof(double) * m, cudaMemcpyDeviceToHost, a->stream));
        for (int q = 0; q < m; ++q) t[q] = ps.times[q];
    }
    HYPE_CK(cudaStreamSynchronize(a->stream));
    if (count) *count = ps.count;
    return HYPE_OK;
}

// SSPRK(4,3) steps of dt from *t_inout; a positive t_final shortens the step that
// would pass it so that the run ends on t_final (TS_EXACTFINALTIME_MATCHSTEP)
// and stops there.  Returns the number of steps taken in *steps_taken.
extern "C" int hype_acoustic_step(hype_acoustic* a, int nsteps, double t_final, double* t_inout, int* steps_taken) {
    if (!a || !t_inout || nsteps < 0) return HYPE_ERR_ARG;
    double t = *t_inout;
    int s = 0;
    const Stage s12{0.0, 1.0, 0.5, 0}, s3{2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0};
    // the stage times of SSP RKS3 with 4 stages (n = 2): c_i = i / (s - n) for i < n (n + 1) / 2,
    // else (i - n) / (s - n), i.e. t + (0, 1/2, 1, 1/2) dt
    auto ct = [](int i) { return (i < 2 * (2 + 1) / 2) ? 1.0 * i / (4 - 2) : (1.0 * i - 2) / (4 - 2); };
    for (; s < nsteps; ++s) {
        if (t_final > 0.0 && t >= t_final) break;
        double dt = a->p.dt;
        if (t_final > 0.0 && t + dt > t_final) dt = t_final - t;
        int rc;
        // u1 = u + dt/2 L(u); u2 = u1 + dt/2 L(u1); u3 = 2/3 u + u2/3 + dt/6 L(u2); u3 + dt/2 L(u3)
        if ((rc = ac_rhs(a, a->U)) || (rc = ac_update(a, a->U, a->U, a->W, s12, dt, t + ct(0) * dt))) return rc;
        if ((rc = ac_rhs(a, a->W)) || (rc = ac_update(a, a->U, a->W, a->W, s12, dt, t + ct(1) * dt))) return rc;
        if ((rc = ac_rhs(a, a->W)) || (rc = ac_update(a, a->U, a->W, a->W, s3, dt, t + ct(2) * dt))) return rc;
        if ((rc = ac_rhs(a, a->W)) || (rc = ac_update(a, a->U, a->W, a->U, s12, dt, t + ct(3) * dt))) return rc;
        t += dt;
    }
    HYPE_CK(cudaStreamSynchronize(a->stream));
    *t_inout = t;
    if (steps_taken) *steps_taken = s;
    return HYPE_OK;
}

extern "C" int hype_acoustic_sync(hype_acoustic* a) {
    if (!a) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" void* hype_acoustic_stream(hype_acoustic* a) { return a ? (void*)a->stream : nullptr; }
