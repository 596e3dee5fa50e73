// pc2d.cu -- the path-conservative 2D scheme of HyPE-2D (2d/HyPE-2D, RHSFunction,
// rhs_function.c:12-610) with its Kapila five-equation model (kapila_5eqn.c):
// Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1), the conservative variables reconstructed
// to order N = 0..3 (Reconstruct / weno2 / weno3 / weno4, reconstruction.c:129-377), the
// admissibility check of PDECheckPAD at the N_node nodes with first order on failure,
// the Rusanov flux plus the Roe-path fluctuation B~(QL, QR)(QR - QL) of riemann.c:13-85
// (3-point Gauss path of PDEmatrixB), the non-conservative product PDENCP integrated over
// the cell, dt = CFL h / (2 s_max), and the program's stepper for N (Euler, SSP RKS2/2,
// RKS3/4, RK104, hype.c:361-382) with the dt of the first RHS kept.
//
// Per RHS evaluation:
//   k_pc_ghost   conservative state with 3 ghost layers (periodic, transmissive copy,
//                reflective mirror negating the normal momentum, components 2 / 3);
//   k_pc_cell<N> per extended cell: reconstruction of the 6 variables, node values and
//                the admissibility check, face traces; per owned cell the volume term;
//   k_pc_faces<D,N> per face: Rusanov flux and path fluctuation at the face's Gauss
//                points (the model's B has one non-zero row, the a1 equation);
//   k_pc_update  the RHS (rhs_function.c:586-597) fused with the stage combination.
// The basis tables are compile-time constants formed as hype.c forms them; terms whose
// table entry is zero are left out (they add signed zeros, which change no value).  The
// file is compiled without FMA contraction: results equal the reference's bit for bit.
#include <cuda_runtime.h>
#include <string.h>

#include "mphase2d_kernels.cuh"

namespace hype {
namespace pc2d {

constexpr int KV = 6;
constexpr int GW = 3;
constexpr double RHO_FLOOR = 1.0e-14, PRS_FLOOR = 1.0e-12, SMALL = 1.0e-12;

struct Geo {
    int nx, ny;
    int bc[4];
    long long N, NE, GN;
    int ex, gx;
};

struct Eos {
    double g1, p1, g2, p2;
};

struct DevScalars {
    unsigned long long smax_bits;
    double dt, t;
    unsigned long long bad, fallback;
};

// ---------------------------------------------------------------- basis tables (hype.c:230-330)
__host__ __device__ constexpr double basis(double x, double y, int n) {
    return n == 0 ? 1.0 : n == 1 ? x : n == 2 ? y : n == 3 ? x * x - 1. / 12. : n == 4 ? y * y - 1. / 12.
         : n == 5 ? x * y : n == 6 ? x * (x * x - 3. / 20.) : n == 7 ? y * (y * y - 3. / 20.)
         : n == 8 ? y * (x * x - 1. / 12.) : n == 9 ? x * (y * y - 1. / 12.) : 0.0;
}
__host__ __device__ constexpr double basis_grad(double x, double y, int n, int d) {
    return d == 0 ? (n == 1 ? 1.0 : n == 3 ? 2.0 * x : n == 5 ? y : n == 6 ? 3.0 * x * x - 3. / 20.
                   : n == 8 ? 2.0 * x * y : n == 9 ? (y * y - 1. / 12.) : 0.0)
                  : (n == 2 ? 1.0 : n == 4 ? 2.0 * y : n == 5 ? x : n == 7 ? 3.0 * y * y - 3. / 20.
                   : n == 8 ? (x * x - 1. / 12.) : n == 9 ? 2.0 * x * y : 0.0);
}
__host__ __device__ constexpr int ndof(int N) { return (N + 1) * (N + 2) / 2; }
__host__ __device__ constexpr int ngf(int N) { return N < 2 ? 1 : 2; }   // Gauss points per face
__host__ __device__ constexpr int ngv(int N) { return N < 2 ? 1 : 4; }   // volume Gauss points
__host__ __device__ constexpr int nnode(int N) { return 4 * ngf(N); }  // admissibility nodes
constexpr double GPT = 0.28867513459481287;
__host__ __device__ constexpr double face_gp(int N, int q) { return N < 2 ? 0.0 : (q == 0 ? -GPT : GPT); }
__host__ __device__ constexpr double face_w(int N) { return N < 2 ? 1.0 : 0.5; }
__host__ __device__ constexpr double vol_x(int N, int q) { return N < 2 ? 0.0 : (q < 2 ? -GPT : GPT); }
__host__ __device__ constexpr double vol_y(int N, int q) { return N < 2 ? 0.0 : ((q & 1) ? GPT : -GPT); }
__host__ __device__ constexpr double vol_w(int N) { return N < 2 ? 1.0 : 0.25; }
__host__ __device__ constexpr double node_x(int N, int q) {
    return N < 2 ? (q == 0 ? 0.5 : q == 1 ? -0.5 : 0.0)
                 : (q < 2 ? 0.5 : q < 4 ? -0.5 : (q == 4 || q == 6) ? -GPT : GPT);
}
__host__ __device__ constexpr double node_y(int N, int q) {
    return N < 2 ? (q == 2 ? 0.5 : q == 3 ? -0.5 : 0.0)
                 : (q < 4 ? ((q & 1) ? GPT : -GPT) : q < 6 ? 0.5 : -0.5);
}
// face f (left, right, bottom, top), Gauss point q: the point's coordinates
__host__ __device__ constexpr double face_x(int N, int f, int q) { return f == 0 ? -0.5 : f == 1 ? 0.5 : face_gp(N, q); }
__host__ __device__ constexpr double face_y(int N, int f, int q) { return f == 2 ? -0.5 : f == 3 ? 0.5 : face_gp(N, q); }

// sum_k c[k] W(k), in k order from 0.0, the zero entries of the table W left out
template <int NDOF, typename W, int K = 0>
__device__ __forceinline__ double tsum(const double* c, double acc, W w) {
    if constexpr (K == NDOF) {
        return acc;
    } else {
        constexpr double v = W::template at<K>();
        if constexpr (v == 0.0) return tsum<NDOF, W, K + 1>(c, acc, w);
        else return tsum<NDOF, W, K + 1>(c, acc + c[K] * v, w);
    }
}
template <int N, int Q>
struct NodeT {
    template <int K> __host__ __device__ static constexpr double at() { return basis(node_x(N, Q), node_y(N, Q), K); }
};
template <int N, int F, int Q>
struct FaceT {
    template <int K> __host__ __device__ static constexpr double at() { return basis(face_x(N, F, Q), face_y(N, F, Q), K); }
};
template <int N, int Q>
struct VolT {
    template <int K> __host__ __device__ static constexpr double at() { return basis(vol_x(N, Q), vol_y(N, Q), K); }
};
template <int N, int Q, int D>
struct VolGT {
    template <int K> __host__ __device__ static constexpr double at() { return basis_grad(vol_x(N, Q), vol_y(N, Q), K, D); }
};

// ---------------------------------------------------------------- reconstruction (reconstruction.c:106-377)
__device__ __forceinline__ double minmod(double a, double b) {
    if (a * b < 0.0) return 0.0;
    return (fabs(a) < fabs(b)) ? a : b;
}
__device__ __forceinline__ double pow4(double a) {
    const double a2 = a * a;
    return a2 * a2;
}
__device__ __forceinline__ void weno3_axis(double u_m2, double u_m1, double u_0, double u_p1, double u_p2, double* c1,
                                           double* c2) {
    const double cw = 100.0, r13_3 = 13. / 3.;
    double u_x[3], u_xx[3], wt[3];
    u_x[0] = -2.0 * u_m1 + 0.5 * u_m2 + 1.5 * u_0; u_xx[0] = 0.5 * (u_m2 - 2.0 * u_m1 + u_0);
    u_x[1] = 0.5 * (u_p1 - u_m1);                  u_xx[1] = 0.5 * (u_m1 - 2.0 * u_0 + u_p1);
    u_x[2] = -1.5 * u_0 + 2.0 * u_p1 - 0.5 * u_p2; u_xx[2] = 0.5 * (u_0 - 2.0 * u_p1 + u_p2);
    wt[0] = 1.0 / (pow4(u_x[0] * u_x[0] + r13_3 * u_xx[0] * u_xx[0] + SMALL));
    wt[1] = cw / (pow4(u_x[1] * u_x[1] + r13_3 * u_xx[1] * u_xx[1] + SMALL));
    wt[2] = 1.0 / (pow4(u_x[2] * u_x[2] + r13_3 * u_xx[2] * u_xx[2] + SMALL));
    const double total = wt[0] + wt[1] + wt[2];
    wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total;
    *c1 = wt[0] * u_x[0] + wt[1] * u_x[1] + wt[2] * u_x[2];
    *c2 = wt[0] * u_xx[0] + wt[1] * u_xx[1] + wt[2] * u_xx[2];
}

// the coefficients of order N from the 13-point stencil (ux, uy: 5 points each, centre at [2])
template <int N>
__device__ __forceinline__ void reconstruct(const double* ux, const double* uy, double upp, double upm, double ump,
                                            double umm, double* c) {
    const double u_0 = ux[2];
    c[0] = u_0;
    if constexpr (N == 1) {
        c[1] = minmod(ux[3] - u_0, u_0 - ux[1]);
        c[2] = minmod(uy[3] - u_0, u_0 - uy[1]);
    } else if constexpr (N == 2) {
        weno3_axis(ux[0], ux[1], u_0, ux[3], ux[4], &c[1], &c[3]);
        weno3_axis(uy[0], uy[1], u_0, uy[3], uy[4], &c[2], &c[4]);
        double u_xy[4], wt[4];
        u_xy[0] = upp - u_0 - c[1] - c[2] - c[3] - c[4];
        u_xy[1] = -upm + u_0 + c[1] - c[2] + c[3] + c[4];
        u_xy[2] = -ump + u_0 - c[1] + c[2] + c[3] + c[4];
        u_xy[3] = umm - u_0 + c[1] + c[2] - c[3] - c[4];
        const double temp = 4.0 * (c[3] * c[3] + c[4] * c[4]);
#pragma unroll
        for (int q = 0; q < 4; ++q) wt[q] = 1.0 / (pow4(temp + u_xy[q] * u_xy[q] + SMALL));
        const double total = wt[0] + wt[1] + wt[2] + wt[3];
        wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total; wt[3] = wt[3] / total;
        c[5] = wt[0] * u_xy[0] + wt[1] * u_xy[1] + wt[2] * u_xy[2] + wt[3] * u_xy[3];
    } else if constexpr (N == 3) {
        mp2d::cweno2d<double>(u_0, ux, uy, upp, upm, ump, umm, c);
    }
}

// ---------------------------------------------------------------- Kapila model (kapila_5eqn.c)
__device__ __forceinline__ void mix(const Eos& e, double a1, double& G, double& P) {
    const double a2 = 1.0 - a1;
    G = 1.0 + ((e.g1 - 1.0) * (e.g2 - 1.0)) / ((e.g2 - 1.0) * a1 + (e.g1 - 1.0) * a2);
    P = ((G - 1.0) / G) * (e.g1 * e.p1 * a1 / (e.g1 - 1.0) + e.g2 * e.p2 * a2 / (e.g2 - 1.0));
}

// PDEFlux (kapila_5eqn.c:66-117)
template <int D>
__device__ __forceinline__ double flux(const Eos& e, const double* Q, double* F, bool& bad) {
    const double a1 = Q[5], a2 = 1.0 - a1;
    double G, P;
    mix(e, a1, G, P);
    const double rho_1 = Q[0] / a1, rho_2 = Q[1] / a2;
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (G - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - G * P;
    constexpr double nx = D == 0 ? 1.0 : 0.0, ny = D == 1 ? 1.0 : 0.0;
    const double un = u * nx + v * ny;
    if (rho < RHO_FLOOR || p + P < PRS_FLOOR) bad = true;
    F[0] = a1 * rho_1 * un;
    F[1] = a2 * rho_2 * un;
    F[2] = rho * u * un + p * nx;
    F[3] = rho * v * un + p * ny;
    F[4] = (E + p) * un;
    F[5] = 0.0;
    return fabs(un) + sqrt(G * (p + P) * irho);
}

// PDECheckPAD (kapila_5eqn.c:248-281)
__device__ __forceinline__ bool pad_ok(const Eos& e, const double* Q) {
    const double phi_1 = Q[5], phi_2 = 1.0 - phi_1;
    const double temp = phi_1 / (e.g1 - 1.0) + phi_2 / (e.g2 - 1.0);
    const double gamma = 1.0 + 1.0 / temp;
    const double pi = (phi_1 * e.g1 * e.p1 / (e.g1 - 1.0) + phi_2 * e.g2 * e.p2 / (e.g2 - 1.0)) / (1.0 + temp);
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - gamma * pi;
    return !(rho < RHO_FLOOR) && !((p + pi) < PRS_FLOOR) && !(phi_1 < 1.0e-4 || phi_1 > 1.0 - 1.0e-4);
}

// PDENCP's a1 row (kapila_5eqn.c:164-199; K is set to zero there)
__device__ __forceinline__ double ncp5(const double* Q, const double* gx, const double* gy) {
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3];
    const double u_x = irho * irho * (gx[2] * rho - Q[2] * (gx[0] + gx[1]));
    const double v_y = irho * irho * (gy[3] * rho - Q[3] * (gy[0] + gy[1]));
    const double K = 0.0;
    return u * gx[5] + v * gy[5] - K * (u_x + v_y);
}

// ---------------------------------------------------------------- kernels
__device__ __forceinline__ long long gidx(const Geo& g, int i, int j) { return (long long)(j + GW) * g.gx + (i + GW); }
__device__ __forceinline__ long long eidx(const Geo& g, int i, int j) { return (long long)(j + 1) * g.ex + (i + 1); }

__global__ void __launch_bounds__(128) k_pc_ghost(const double* __restrict__ U, double* __restrict__ G, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - GW;
    const int j = blockIdx.y - GW;
    if (i >= g.nx + GW) return;
    int fi = 0, fj = 0;
    const int mi = bmap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = bmap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const long long src = (long long)mj * g.nx + mi, dst = gidx(g, i, j);
#pragma unroll
    for (int c = 0; c < KV; ++c) {
        double v = __ldg(U + c * g.N + src);
        if ((c == 2 && fi) || (c == 3 && fj)) v = -v;
        G[c * g.GN + dst] = v;
    }
}

// T[c][f * NGF + q][extended cell]: the face traces; V5[cell]: the a1 row of the volume term
template <int N>
__global__ void __launch_bounds__(128) k_pc_cell(const double* __restrict__ G, double* __restrict__ T,
                                                 double* __restrict__ V5, Geo g, Eos e, double r1_h,
                                                 DevScalars* __restrict__ ds) {
    constexpr int NDOF = ndof(N), NGF = ngf(N), NGV = ngv(N), NN = nnode(N);
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    if (i > g.nx || j > g.ny) return;
    const long long ge = gidx(g, i, j);
    const int sy = g.gx;
    double cf[KV][NDOF];
#pragma unroll
    for (int c = 0; c < KV; ++c) {
        const double* p = G + c * g.GN + ge;
        double ux[5], uy[5];
#pragma unroll
        for (int o = 0; o < 5; ++o) {
            ux[o] = __ldg(p + (o - 2));
            uy[o] = __ldg(p + (o - 2) * sy);
        }
        double tmp[10];
        reconstruct<N>(ux, uy, __ldg(p + 1 + sy), __ldg(p + 1 - sy), __ldg(p - 1 + sy), __ldg(p - 1 - sy), tmp);
#pragma unroll
        for (int k = 0; k < NDOF; ++k) cf[c][k] = tmp[k];
    }
    // admissibility at the nodes (rhs_function.c:338-365)
    bool ok = true;
    auto node = [&](auto qc) {
        constexpr int q = decltype(qc)::value;
        double Qn[KV];
#pragma unroll
        for (int c = 0; c < KV; ++c) Qn[c] = tsum<NDOF>(cf[c], 0.0, NodeT<N, q>{});
        ok = ok && pad_ok(e, Qn);
    };
    node(std::integral_constant<int, 0>{});
    node(std::integral_constant<int, 1>{});
    node(std::integral_constant<int, 2>{});
    node(std::integral_constant<int, 3>{});
    if constexpr (NN == 8) {
        node(std::integral_constant<int, 4>{});
        node(std::integral_constant<int, 5>{});
        node(std::integral_constant<int, 6>{});
        node(std::integral_constant<int, 7>{});
    }
    if (!ok) {  // first order (the minmod slopes the reference forms are zeroed, :352-362)
#pragma unroll
        for (int c = 0; c < KV; ++c) {
            cf[c][0] = __ldg(G + c * g.GN + ge);
#pragma unroll
            for (int k = 1; k < NDOF; ++k) cf[c][k] = 0.0;
        }
        if (i >= 0 && i < g.nx && j >= 0 && j < g.ny) atomicAdd(&ds->fallback, 1ull);
    }
    const long long e_ = eidx(g, i, j);
#pragma unroll
    for (int c = 0; c < KV; ++c) {
        double* t = T + (long long)c * 4 * NGF * g.NE + e_;
        t[(0 * NGF + 0) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 0, 0>{});
        t[(1 * NGF + 0) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 1, 0>{});
        t[(2 * NGF + 0) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 2, 0>{});
        t[(3 * NGF + 0) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 3, 0>{});
        if constexpr (NGF == 2) {
            t[(0 * NGF + 1) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 0, 1>{});
            t[(1 * NGF + 1) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 1, 1>{});
            t[(2 * NGF + 1) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 2, 1>{});
            t[(3 * NGF + 1) * g.NE] = tsum<NDOF>(cf[c], 0.0, FaceT<N, 3, 1>{});
        }
    }
    if (i < 0 || i >= g.nx || j < 0 || j >= g.ny) return;
    // the volume term -sum_q w_q B(Q) grad Q (rhs_function.c:380-410)
    double r5 = 0.0;
    auto vol = [&](auto qc) {
        constexpr int q = decltype(qc)::value;
        double Qg[KV], gx[KV], gy[KV];
#pragma unroll
        for (int c = 0; c < KV; ++c) {
            Qg[c] = tsum<NDOF>(cf[c], 0.0, VolT<N, q>{});
            gx[c] = r1_h * tsum<NDOF>(cf[c], 0.0, VolGT<N, q, 0>{});
            gy[c] = r1_h * tsum<NDOF>(cf[c], 0.0, VolGT<N, q, 1>{});
        }
        r5 += -vol_w(N) * ncp5(Qg, gx, gy);
    };
    vol(std::integral_constant<int, 0>{});
    if constexpr (NGV == 4) {
        vol(std::integral_constant<int, 1>{});
        vol(std::integral_constant<int, 2>{});
        vol(std::integral_constant<int, 3>{});
    }
    V5[(long long)j * g.nx + i] = r5;
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// F[c][face] (6 components) and Dn[face]: the a1 row of the path fluctuation
template <int D, int N>
__global__ void __launch_bounds__(128) k_pc_faces(const double* __restrict__ T, double* __restrict__ F,
                                                  double* __restrict__ Dn, Geo g, Eos e, DevScalars* __restrict__ ds) {
    constexpr int NGF = ngf(N);
    constexpr double wq = face_w(N);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    double smax = 0.0;
    bool bad = false;
    if (i < fx && j < fy) {
        const long long eR = eidx(g, i, j), eL = eidx(g, i - (D == 0), j - (D == 1));
        double fl[KV], d5 = 0.0;
#pragma unroll
        for (int c = 0; c < KV; ++c) fl[c] = 0.0;
#pragma unroll
        for (int q = 0; q < NGF; ++q) {
            double QL[KV], QR[KV], FL[KV], FR[KV];
#pragma unroll
            for (int c = 0; c < KV; ++c) {
                QL[c] = __ldg(T + ((long long)c * 4 * NGF + (2 * D + 1) * NGF + q) * g.NE + eL);
                QR[c] = __ldg(T + ((long long)c * 4 * NGF + (2 * D) * NGF + q) * g.NE + eR);
            }
            // RiemannSolver (riemann.c:52-85): Rusanov flux
            const double sl = flux<D>(e, QL, FL, bad), sr = flux<D>(e, QR, FR, bad);
            const double s = sl < sr ? sr : sl;
            smax = fmax(smax, s);
            // RoeMatrix (riemann.c:13-47): B[5][5] = un along the straight path, 3 Gauss points
            constexpr double s_gp[3] = {0.1127016653792583, 0.5, 0.8872983346207417};
            constexpr double w_gp[3] = {0.2777777777777778, 0.4444444444444444, 0.2777777777777778};
            double b55 = 0.0;
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const double r0 = QL[0] + s_gp[p] * (QR[0] - QL[0]), r1 = QL[1] + s_gp[p] * (QR[1] - QL[1]);
                const double m = QL[2 + D] + s_gp[p] * (QR[2 + D] - QL[2 + D]);
                const double irho = 1.0 / (r0 + r1);
                b55 += w_gp[p] * (irho * m);
            }
#pragma unroll
            for (int c = 0; c < KV; ++c) fl[c] += wq * (0.5 * (FR[c] + FL[c] - s * (QR[c] - QL[c])));
            d5 += wq * (b55 * (QR[5] - QL[5]));
        }
        const long long nf = (long long)fx * fy;
        const long long f = (long long)j * fx + i;
#pragma unroll
        for (int c = 0; c < KV; ++c) F[c * nf + f] = fl[c];
        Dn[f] = d5;
        if (bad) {
            const int ci = i < g.nx ? i : g.nx - 1, cj = j < g.ny ? j : g.ny - 1;
            atomicMin(&ds->bad, (unsigned long long)((long long)cj * g.nx + ci));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    if ((threadIdx.x & 31) == 0 && smax > 0.0) atomic_max_pos(&ds->smax_bits, smax);
}

struct Stage {
    double a, b, c, d;  // out = a X + (c dt / d) L (+ b Y when b != 0); rhs_only: out = L
    int rhs_only;
};

// X, Y and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_pc_update(const double* __restrict__ Fx, const double* __restrict__ Fy,
                                                   const double* __restrict__ Dx, const double* __restrict__ Dy,
                                                   const double* __restrict__ V5, const double* X,
                                                   const double* Y, double* out, Geo g,
                                                   double r1_h, Stage st, const DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    const long long nfx = (long long)(g.nx + 1) * g.ny, nfy = (long long)g.nx * (g.ny + 1);
    const long long ix = (long long)j * (g.nx + 1) + i, iy = (long long)j * g.nx + i, cell = iy;
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt / st.d;
#pragma unroll
    for (int c = 0; c < KV; ++c) {
        const double dfx = Fx[c * nfx + ix + 1] - Fx[c * nfx + ix], dfy = Fy[c * nfy + iy + g.nx] - Fy[c * nfy + iy];
        double L;
        if (c == 5) {
            L = V5[cell] + (-r1_h * (dfx + 0.5 * (Dx[ix + 1] + Dx[ix])) - r1_h * (dfy + 0.5 * (Dy[iy + g.nx] + Dy[iy])));
        } else {
            L = -r1_h * dfx - r1_h * dfy;
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

// dt = CFL h / (2 s_max) (rhs_function.c:602), set from the first RHS of a run
__global__ void k_pc_set_dt(DevScalars* ds, double cfl_h) {
    ds->dt = cfl_h / (2.0 * __longlong_as_double((long long)ds->smax_bits));
}

__global__ void k_pc_reset(DevScalars* ds) {
    ds->smax_bits = 0ull;
    ds->bad = ~0ull;
}

__global__ void k_pc_axpby(const double* __restrict__ X, const double* __restrict__ Y, double* __restrict__ out, double a,
                           double b, long long n) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) out[q] = a * X[q] + b * Y[q];
}

__global__ void k_pc_aos2soa(const double* __restrict__ a, double* __restrict__ s, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * KV) return;
    const long long cell = q / KV;
    s[(q - cell * KV) * N + cell] = a[q];
}
__global__ void k_pc_soa2aos(const double* __restrict__ s, double* __restrict__ a, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * KV) return;
    const long long cell = q / KV;
    a[q] = s[(q - cell * KV) * N + cell];
}

}  // namespace pc2d
}  // namespace hype

using namespace hype;
using namespace hype::pc2d;

struct hype_pc2d {
    hype_pc2d_params p;
    Geo g;
    Eos e;
    cudaStream_t stream = nullptr;
    double *U = nullptr, *W0 = nullptr, *W1 = nullptr, *S = nullptr, *L = nullptr, *G = nullptr, *T = nullptr;
    double *Fx = nullptr, *Fy = nullptr, *Dx = nullptr, *Dy = nullptr, *V5 = nullptr, *aos = nullptr;
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;
};

template <int N>
static void pc_launch(hype_pc2d* m, const double* Win) {
    const Geo& g = m->g;
    const double r1_h = 1. / (m->p.h);
    k_pc_cell<N><<<dim3(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4)), dim3(32, 4), 0, m->stream>>>(m->G, m->T, m->V5, g, m->e,
                                                                                           r1_h, m->ds);
    k_pc_faces<0, N><<<dim3(cdiv(g.nx + 1, 32), cdiv(g.ny, 4)), dim3(32, 4), 0, m->stream>>>(m->T, m->Fx, m->Dx, g, m->e,
                                                                                            m->ds);
    k_pc_faces<1, N><<<dim3(cdiv(g.nx, 32), cdiv(g.ny + 1, 4)), dim3(32, 4), 0, m->stream>>>(m->T, m->Fy, m->Dy, g, m->e,
                                                                                            m->ds);
}

// one RHS evaluation of Win into the flux / fluctuation / volume buffers
static int pc_rhs(hype_pc2d* m, const double* Win) {
    const Geo& g = m->g;
    k_pc_ghost<<<dim3(cdiv(g.gx, 128), g.ny + 2 * GW), 128, 0, m->stream>>>(Win, m->G, g);
    switch (m->p.order) {
        case 0: pc_launch<0>(m, Win); break;
        case 1: pc_launch<1>(m, Win); break;
        case 2: pc_launch<2>(m, Win); break;
        default: pc_launch<3>(m, Win); break;
    }
    HYPE_LAUNCHED(4);
    return HYPE_OK;
}

static int pc_update(hype_pc2d* m, const double* X, const double* Y, double* out, Stage st) {
    const Geo& g = m->g;
    k_pc_update<<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 8)), dim3(32, 8), 0, m->stream>>>(
        m->Fx, m->Fy, m->Dx, m->Dy, m->V5, X, Y, out, g, 1. / (m->p.h), st, m->ds);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

extern "C" int hype_pc2d_create(const hype_pc2d_params* p, hype_pc2d** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || !(p->h > 0) || !(p->cfl > 0) || p->order < 0 || p->order > 3) return HYPE_ERR_ARG;
    for (int f = 0; f < 4; ++f)
        if (p->bc[f] < HYPE_BC_PERIODIC || p->bc[f] > HYPE_BC_TRANSMISSIVE) return HYPE_ERR_ARG;
    for (int d = 0; d < 2; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (!(p->g1 > 1.0) || !(p->g2 > 1.0)) return HYPE_ERR_ARG;
    hype_pc2d* m = new hype_pc2d();
    m->p = *p;
    m->e = Eos{p->g1, p->p1, p->g2, p->p2};
    Geo& g = m->g;
    g.nx = p->nx; g.ny = p->ny;
    for (int f = 0; f < 4; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny;
    g.ex = p->nx + 2;
    g.NE = (long long)g.ex * (p->ny + 2);
    g.gx = p->nx + 2 * GW;
    g.GN = (long long)g.gx * (p->ny + 2 * GW);
    const size_t sN = sizeof(double) * KV * (size_t)g.N;
    const int ngf_ = p->order < 2 ? 1 : 2;
    cudaError_t ce = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    auto al = [&](double** ptr, size_t bytes) {
        if (ce == cudaSuccess) ce = cudaMalloc((void**)ptr, bytes);
    };
    al(&m->U, sN); al(&m->W0, sN); al(&m->W1, sN); al(&m->S, sN); al(&m->L, sN); al(&m->aos, sN);
    al(&m->G, sizeof(double) * KV * (size_t)g.GN);
    al(&m->T, sizeof(double) * KV * 4 * ngf_ * (size_t)g.NE);
    al(&m->Fx, sizeof(double) * KV * (size_t)(g.nx + 1) * g.ny);
    al(&m->Fy, sizeof(double) * KV * (size_t)g.nx * (g.ny + 1));
    al(&m->Dx, sizeof(double) * (size_t)(g.nx + 1) * g.ny);
    al(&m->Dy, sizeof(double) * (size_t)g.nx * (g.ny + 1));
    al(&m->V5, sizeof(double) * (size_t)g.N);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->ds, sizeof(DevScalars));
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&m->hs, sizeof(DevScalars));
    if (ce == cudaSuccess) {
        DevScalars z;
        memset(&z, 0, sizeof(z));
        z.bad = ~0ull;
        ce = cudaMemcpy(m->ds, &z, sizeof(z), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        set_last_error("hype_pc2d_create", ce);
        hype_pc2d_destroy(m);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = m;
    return HYPE_OK;
}

extern "C" void hype_pc2d_destroy(hype_pc2d* m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->U); cudaFree(m->W0); cudaFree(m->W1); cudaFree(m->S); cudaFree(m->L); cudaFree(m->aos); cudaFree(m->G);
    cudaFree(m->T); cudaFree(m->Fx); cudaFree(m->Fy); cudaFree(m->Dx); cudaFree(m->Dy); cudaFree(m->V5); cudaFree(m->ds);
    if (m->hs) cudaFreeHost(m->hs);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

extern "C" int hype_pc2d_get_params(const hype_pc2d* m, hype_pc2d_params* out) {
    if (!m || !out) return HYPE_ERR_ARG;
    *out = m->p;
    return HYPE_OK;
}

static int pc_h2d(hype_pc2d* m, const double* aos, double* soa) {
    const long long N = m->g.N;
    HYPE_CK(cudaMemcpyAsync(m->aos, aos, sizeof(double) * KV * N, cudaMemcpyHostToDevice, m->stream));
    k_pc_aos2soa<<<cdiv(N * KV, 256), 256, 0, m->stream>>>(m->aos, soa, N);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int pc_d2h(hype_pc2d* m, const double* soa, double* aos) {
    const long long N = m->g.N;
    k_pc_soa2aos<<<cdiv(N * KV, 256), 256, 0, m->stream>>>(soa, m->aos, N);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, m->aos, sizeof(double) * KV * N, cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

static int pc_scalars(hype_pc2d* m) {
    HYPE_CK(cudaMemcpyAsync(m->hs, m->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_pc2d_upload(hype_pc2d* m, const double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    int rc = pc_h2d(m, U_aos, m->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_pc2d_download(hype_pc2d* m, double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    return pc_d2h(m, m->U, U_aos);
}

extern "C" int hype_pc2d_rhs(hype_pc2d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out) {
    (void)t;
    if (!m || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc = pc_h2d(m, U_aos, m->S);
    if (rc) return rc;
    k_pc_reset<<<1, 1, 0, m->stream>>>(m->ds);
    HYPE_LAUNCHED(1);
    if ((rc = pc_rhs(m, m->S)) || (rc = pc_update(m, nullptr, nullptr, m->L, Stage{0.0, 0.0, 0.0, 1.0, 1}))) return rc;
    k_pc_set_dt<<<1, 1, 0, m->stream>>>(m->ds, m->p.cfl * m->p.h);
    HYPE_LAUNCHED(1);
    if ((rc = pc_scalars(m))) return rc;
    if (dt_out) *dt_out = m->hs->dt;
    const bool bad = m->hs->bad != ~0ull;
    if ((rc = pc_d2h(m, m->L, RHS_aos))) return rc;
    return bad ? HYPE_ERR_STATE : HYPE_OK;
}

// nsteps of the program's stepper for the order N (hype.c:361-382); *dt_inout <= 0: dt
// from the first RHS of the run (the program keeps it: its monitor does not reset it)
extern "C" int hype_pc2d_step(hype_pc2d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells) {
    if (!m || nsteps < 0 || !t_inout || !dt_inout) return HYPE_ERR_ARG;
    DevScalars init;
    memset(&init, 0, sizeof(init));
    init.t = *t_inout;
    init.dt = *dt_inout;
    init.bad = ~0ull;
    HYPE_CK(cudaMemcpyAsync(m->ds, &init, sizeof(init), cudaMemcpyHostToDevice, m->stream));
    const bool from_rhs = !(*dt_inout > 0);
    const long long n = KV * m->g.N;
    const int N = m->p.order;
    int rc;
    for (int s = 0; s < nsteps; ++s) {
        // the first stage's RHS (at the step's state); the first of the run also sets dt
        if ((rc = pc_rhs(m, m->U))) return rc;
        if (s == 0 && from_rhs) {
            k_pc_set_dt<<<1, 1, 0, m->stream>>>(m->ds, m->p.cfl * m->p.h);
            HYPE_LAUNCHED(1);
        }
        if (N == 0) {  // forward Euler
            if ((rc = pc_update(m, m->U, nullptr, m->U, Stage{1.0, 0.0, 1.0, 1.0, 0}))) return rc;
        } else if (N == 1) {  // SSP RKS2, 2 stages: w = u + dt L(u); u = u/2 + dt/2 L(w) + w/2
            if ((rc = pc_update(m, m->U, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 2 - 1.0, 0}))) return rc;
            if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->U, m->W0, m->U, Stage{1.0 / 2, (2 - 1.0) / 2, 1.0, 2.0, 0})))
                return rc;
        } else if (N == 2) {  // SSP RKS3, 4 stages
            const Stage s2{1.0, 0.0, 1.0, 2.0, 0};
            if ((rc = pc_update(m, m->U, nullptr, m->W0, s2))) return rc;
            if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->W0, nullptr, m->W0, s2))) return rc;
            if ((rc = pc_rhs(m, m->W0)) ||
                (rc = pc_update(m, m->U, m->W0, m->W0,
                                Stage{1.0 * 2 / (2 * 2 - 1.0), (2 - 1.0) / (2 * 2 - 1), 2 - 1.0, 2.0 * (2 * 2 - 1), 0})))
                return rc;
            if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->W0, nullptr, m->U, s2))) return rc;
        } else {  // SSP RK104, low storage
            const Stage s6{1.0, 0.0, 1.0, 6.0, 0};
            if ((rc = pc_update(m, m->U, nullptr, m->W0, s6))) return rc;
            for (int k = 1; k < 5; ++k)
                if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->W0, nullptr, m->W0, s6))) return rc;
            k_pc_axpby<<<cdiv(n, 256), 256, 0, m->stream>>>(m->W0, m->U, m->W1, 9.0 / 25, 1.0 / 25, n);
            k_pc_axpby<<<cdiv(n, 256), 256, 0, m->stream>>>(m->W1, m->W0, m->W0, 15.0, -5.0, n);
            HYPE_LAUNCHED(2);
            for (int k = 5; k < 9; ++k)
                if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->W0, nullptr, m->W0, s6))) return rc;
            if ((rc = pc_rhs(m, m->W0)) || (rc = pc_update(m, m->W0, m->W1, m->U, Stage{3.0 / 5, 1.0, 1.0, 10.0, 0})))
                return rc;
        }
    }
    if ((rc = pc_scalars(m))) return rc;
    double t = *t_inout;
    for (int s = 0; s < nsteps; ++s) t += m->hs->dt;
    *t_inout = t;
    *dt_inout = m->hs->dt;
    if (fallback_cells) *fallback_cells = (long long)m->hs->fallback;
    return m->hs->bad == ~0ull ? HYPE_OK : HYPE_ERR_STATE;
}

extern "C" int hype_pc2d_sync(hype_pc2d* m) {
    if (!m) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" void* hype_pc2d_stream(hype_pc2d* m) { return m ? (void*)m->stream : nullptr; }
