// mphase3d.cu -- the 3D primitive-variable multiphase path of HyPE
// (3d/weno4/Viscous-Multiphase-Fourth-Order, RHSFunctionPrimitive, rhs_function.c:56-570):
// Q = (rho, rho u, rho v, rho w, E, phi) with the mixture EOS of two stiffened gases
// mixed by phi (pde.c:9-45), CWENO4 of the primitive variables, the 33-node
// admissibility check of PDECheckPAD with first order on failure (:284-306), the
// rotated HLLC flux with the normal velocity as a 7th component (pde.c:273-440), the
// non-conservative phi equation d phi/dt = -div(phi u) + phi div u (:507-552), and
// dt = (1/3) CFL h / (s_max + 2 s_visc / h) (:559), s_visc the viscous speed
// (4/3)(phi mu1 + (1 - phi) mu2)/rho of PDEViscFluxPrim (pde.c:101-136).  The program's
// viscous flux itself reads gradients that its weno() never writes; with zero gradients it
// is a signed zero, so no viscous flux is applied here.
//
// Per RHS evaluation:
//   k_m3_ghost   conservative SoA -> primitive with 3 ghost layers (boundary maps per
//                axis: periodic, transmissive copy, reflective mirror with the normal
//                velocity negated, rhs_function.c:98-230);
//   k_m3_recon   per extended cell: CWENO4 of the 6 primitive variables, the 33-node
//                density / pressure check (node values from compile-time monomials),
//                the 24 face traces per variable (or the cell values on failure);
//   k_m3_faces   per face: 4 Gauss points of the rotated HLLC flux (7 components),
//                wave-speed maxima;
//   k_m3_update  RHS with the phi term, fused with the SSP stage combination.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "euler_kernels.cuh"

namespace hype {
namespace mp3d {

using euler::cweno4;
using euler::face_traces;
using euler::NTR;
using euler::S1;
using euler::SO;
using euler::SQ;

constexpr int MV = 6;  // variables
constexpr int MF = 7;  // flux components (6 + the normal velocity of the phi term)
constexpr int GW = 3;
constexpr double RHO_FLOOR = 1.0e-14, PRS_FLOOR = 1.0e-12;

struct Geo {
    int nx, ny, nz;
    int bc[6];
    long long N, NE, GN;
    int ex, ey, gx, gy;
};

struct Eos {
    double g1, p1, g2, p2, mu1, mu2;
};

struct DevScalars {
    unsigned long long smax_bits[6];   // [0..3] stages, [4] RHS-only calls
    unsigned long long smaxv_bits[6];  // viscous speeds, same slots
    double dt, t;
    unsigned long long bad;            // first inadmissible face's cell (ULLONG_MAX: none)
    unsigned long long fallback;       // owned-cell first-order fallbacks
};

// ---------------------------------------------------------------- EOS (pde.c:9-45)
__device__ __forceinline__ double mix_g(const Eos& e, double phi) {
    return 1.0 + (e.g1 - 1.0) * (e.g2 - 1.0) / ((1.0 - phi) * (e.g1 - 1.0) + phi * (e.g2 - 1.0));
}
__device__ __forceinline__ double mix_pinf(const Eos& e, double g, double phi) {
    // with no stiffness in either gas both terms vanish, and so does the product: no divisions
    if (e.p1 == 0.0 && e.p2 == 0.0) return 0.0;
    return ((g - 1.0) / g) * (e.g1 * e.p1 * phi / (e.g1 - 1.0) + e.g2 * e.p2 * (1.0 - phi) / (e.g2 - 1.0));
}
__device__ __forceinline__ void cons2prim(const Eos& e, const double* Q, double* V) {
    const double g = mix_g(e, Q[5]);
    const double P_inf = mix_pinf(e, g, Q[5]);
    const double temp = 1.0 / Q[0];
    V[0] = Q[0];
    V[1] = Q[1] * temp;
    V[2] = Q[2] * temp;
    V[3] = Q[3] * temp;
    V[4] = (g - 1.0) * (Q[4] - 0.5 * temp * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3])) - g * P_inf;
    V[5] = Q[5];
}

// One side of a face: the primitive trace and what PDEConsFluxPrim / PDEPrim2Cons derive
// from it that does not depend on the normal (pde.c:142-202, 27-45): mixture gamma and
// P_inf, total energy, sound speed.  Computed once per trace instead of once per HLLC
// evaluation (the rotated solver makes three).
struct Side {
    double rho, u, v, w, p, phi, E, a, irho;
};

__device__ __forceinline__ Side make_side(const Eos& e, const double* V, bool& bad) {
    Side s;
    s.rho = V[0]; s.u = V[1]; s.v = V[2]; s.w = V[3]; s.p = V[4]; s.phi = V[5];
    const double g = mix_g(e, s.phi);
    const double P_inf = mix_pinf(e, g, s.phi);
    s.E = 0.5 * s.rho * (s.u * s.u + s.v * s.v + s.w * s.w) + (s.p + g * P_inf) / (g - 1.0);
    if (s.rho < RHO_FLOOR || (s.p + P_inf) < PRS_FLOOR) bad = true;
    s.irho = euler::recip(s.rho);
    s.a = sqrt(g * (s.p + P_inf) * s.irho);
    return s;
}

// PDEHLLCRiemannSolver (pde.c:273-379) for a unit normal n, 7 flux components.  The
// reference builds the star-state velocity from (S_star, u.t1, u.t2) in its Miller-Colella
// frame M = [n; t1; t2] and the inverse of M (pde.c:290-323); since M^-1 M u = u, that
// velocity is u + (S_star - u.n) c with c the first column of M^-1, (t1 x t2) / det M.
// The frame's t2z of the first branch (pde.c:302) is not the one of n x t1, so M is not
// orthonormal and c is not n: c is formed from the reference's t1, t2 as they are.
__device__ __forceinline__ double hllc7(const Side& L, const Side& R, double nx, double ny, double nz, double* Flux) {
    const double un_L = L.u * nx + L.v * ny + L.w * nz, un_R = R.u * nx + R.v * ny + R.w * nz;
    const double S_L = fmin(un_R - R.a, un_L - L.a);
    const double S_R = fmax(un_L + L.a, un_R + R.a);
    const double S_star = (R.p - L.p + L.rho * un_L * (S_L - un_L) - R.rho * un_R * (S_R - un_R)) *
                          euler::recip(L.rho * (S_L - un_L) - R.rho * (S_R - un_R));
    // the reference's branch order (pde.c:368-376); with S_L == 0 and S_star >= 0 it leaves
    // the flux unset, here zero
    const int sel = (S_L > 0.0) ? 0 : (S_star >= 0.0 && S_L < 0.0) ? 1 : (S_star < 0.0 && S_R >= 0.0) ? 2
                                : (S_R < 0.0) ? 3 : 4;
    if (sel == 4) {
#pragma unroll
        for (int i = 0; i < MF; ++i) Flux[i] = 0.0;
        return fmax(fabs(un_L) + L.a, fabs(un_R) + R.a);
    }
    const bool left = sel <= 1;
    const Side& K = left ? L : R;
    const double un = left ? un_L : un_R;
    // the side's flux (PDEConsFluxPrim) and, for the star states, S (Q* - Q)
    double F[MF];
    F[0] = K.rho * un;
    F[1] = K.rho * K.u * un + K.p * nx;
    F[2] = K.rho * K.v * un + K.p * ny;
    F[3] = K.rho * K.w * un + K.p * nz;
    F[4] = (K.E + K.p) * un;
    F[5] = K.phi * un;
    F[6] = un;
    if (sel == 1 || sel == 2) {
        // the frame of pde.c:290-312 and the first column of its inverse
        double t1x, t1y, t1z, t2x, t2y, t2z;
        if (fabs(ny + nz) > fabs(ny - nz)) {
            const double il = rsqrt(2.0 * (1.0 + nz * (ny - nx) + nx * ny));
            t1x = (ny + nz) * il; t1y = (nz - nx) * il; t1z = -(nx + ny) * il;
            t2x = (nx * (nz - ny) - ny * ny - nz * nz) * il;
            t2y = (ny * (nx + nz) + nx * nx + nz * nz) * il;
            t2z = (nz * (nx - nz) - nx * nx - ny * ny) * il;
        } else {
            const double il = rsqrt(2.0 * (1.0 - nx * ny - nx * nz - ny * nz));
            t1x = (ny - nz) * il; t1y = (nz - nx) * il; t1z = (nx - ny) * il;
            t2x = (nx * (ny + nz) - ny * ny - nz * nz) * il;
            t2y = (ny * (nx + nz) - nx * nx - nz * nz) * il;
            t2z = (nz * (nx + ny) - nx * nx - ny * ny) * il;
        }
        const double cx = t1y * t2z - t1z * t2y, cy = t1z * t2x - t1x * t2z, cz = t1x * t2y - t1y * t2x;
        const double idet = euler::recip(nx * cx + ny * cy + nz * cz);
        const double S = left ? S_L : S_R;
        const double isd = euler::recip(S - S_star);
        const double q0 = K.rho * (S - un) * isd;
        const double dn = (S_star - un) * idet;
        const double Qs[MV] = {q0, q0 * (K.u + dn * cx), q0 * (K.v + dn * cy), q0 * (K.w + dn * cz),
                               q0 * ((K.E * K.irho) + (S_star - un) * (S_star + K.p * K.irho * euler::recip(S - un))),
                               K.phi * (S - un) * isd};
        const double Q[MV] = {K.rho, K.rho * K.u, K.rho * K.v, K.rho * K.w, K.E, K.phi};
#pragma unroll
        for (int i = 0; i < MV; ++i) F[i] = F[i] + S * (Qs[i] - Q[i]);
        F[6] = un + S * (((S - un) * isd) - 1.0);
    }
#pragma unroll
    for (int i = 0; i < MF; ++i) Flux[i] = F[i];
    return fmax(fabs(un_L) + L.a, fabs(un_R) + R.a);
}

// PDErotHLLCRiemannSolver (pde.c:383-440): HLLC along the velocity-jump direction n1 and
// its two Miller-Colella tangents, weighted by their projections on the face normal
__device__ __forceinline__ double rot_hllc7(const Side& L, const Side& R, double nx, double ny, double nz, double* Flux) {
    const double du = R.u - L.u, dv = R.v - L.v, dw = R.w - L.w;
    const double dq2 = du * du + dv * dv + dw * dw;
    double n1x, n1y, n1z;
    if (dq2 < 1.0E-20) {  // |du| < 1e-10 (pde.c:391)
        n1x = nx; n1y = ny; n1z = nz;
    } else {
        const double idq = rsqrt(dq2);
        n1x = du * idq; n1y = dv * idq; n1z = dw * idq;
    }
    double a1 = n1x * nx + n1y * ny + n1z * nz;
    if (a1 < 0.0) {
        n1x = -n1x; n1y = -n1y; n1z = -n1z; a1 = -a1;
    }
    double t1x, t1y, t1z, t2x, t2y, t2z;
    if (fabs(n1y + n1z) > fabs(n1y - n1z)) {
        const double il = rsqrt(2.0 * (1.0 + n1z * (n1y - n1x) + n1x * n1y));
        t1x = (n1y + n1z) * il; t1y = (n1z - n1x) * il; t1z = -(n1x + n1y) * il;
        t2x = (n1x * (n1z - n1y) - n1y * n1y - n1z * n1z) * il;
        t2y = (n1y * (n1x + n1z) + n1x * n1x + n1z * n1z) * il;
        t2z = (n1z * (n1x - n1y) - n1x * n1x - n1y * n1y) * il;
    } else {
        const double il = rsqrt(2.0 * (1.0 - n1x * n1y - n1x * n1z - n1y * n1z));
        t1x = (n1y - n1z) * il; t1y = (n1z - n1x) * il; t1z = (n1x - n1y) * il;
        t2x = (n1x * (n1y + n1z) - n1y * n1y - n1z * n1z) * il;
        t2y = (n1y * (n1x + n1z) - n1x * n1x - n1z * n1z) * il;
        t2z = (n1z * (n1x + n1y) - n1x * n1x - n1y * n1y) * il;
    }
    double a2 = t1x * nx + t1y * ny + t1z * nz;
    if (a2 < 0.0) {
        t1x = -t1x; t1y = -t1y; t1z = -t1z; a2 = -a2;
    }
    double a3 = t2x * nx + t2y * ny + t2z * nz;
    if (a3 < 0.0) {
        t2x = -t2x; t2y = -t2y; t2z = -t2z; a3 = -a3;
    }
    double F1[MF];
    const double s1 = hllc7(L, R, n1x, n1y, n1z, F1);
#pragma unroll
    for (int c = 0; c < MF; ++c) Flux[c] = a1 * F1[c];
    const double s2 = hllc7(L, R, t1x, t1y, t1z, F1);
#pragma unroll
    for (int c = 0; c < MF; ++c) Flux[c] += a2 * F1[c];
    const double s3 = hllc7(L, R, t2x, t2y, t2z, F1);
#pragma unroll
    for (int c = 0; c < MF; ++c) Flux[c] += a3 * F1[c];
    return fmax(s1, fmax(s2, s3));
}

// ---------------------------------------------------------------- admissibility nodes
// the 33 nodes of hype.h:93-96 (centre, 12 axis points, 8 corners, 12 edge midpoints)
__host__ __device__ constexpr double node(int m, int axis) {
    constexpr double X[33] = {0.0, 0.5, 0.25, -0.25, -0.5, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.0, -0.5, 0.5,
                              0.0, -0.5, 0.5, 0.0, -0.5, 0.5, 0.0, -0.5, 0.5, -0.5, 0.5, -0.5, 0.5, -0.5, 0.5, -0.5};
    constexpr double Y[33] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.25, -0.25, -0.5, 0.0, 0.0, 0.0, 0.0, 0.5, 0.5, 0.5, -0.5,
                              -0.5, -0.5, 0.5, 0.5, 0.5, -0.5, -0.5, -0.5, 0.0, 0.0, 0.0, 0.0, 0.5, 0.5, -0.5, -0.5};
    constexpr double Z[33] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.25, -0.25, -0.5, 0.5, 0.5, 0.5, 0.5,
                              0.5, 0.5, -0.5, -0.5, -0.5, -0.5, -0.5, -0.5, 0.5, 0.5, -0.5, -0.5, 0.0, 0.0, 0.0, 0.0};
    return axis == 0 ? X[m] : axis == 1 ? Y[m] : Z[m];
}

// the basis monomials of evaluate_polynomial (reconstruction.c:12-21)
__host__ __device__ constexpr double mono(int k, double x, double y, double z) {
    constexpr double r1_12 = 1. / 12., r3_20 = 3. / 20.;
    switch (k) {
        case 0: return 1.0;
        case 1: return x;
        case 2: return y;
        case 3: return z;
        case 4: return x * x - r1_12;
        case 5: return y * y - r1_12;
        case 6: return z * z - r1_12;
        case 7: return x * y;
        case 8: return y * z;
        case 9: return z * x;
        case 10: return x * (x * x - r3_20);
        case 11: return y * (y * y - r3_20);
        case 12: return z * (z * z - r3_20);
        case 13: return (x * x - r1_12) * y;
        case 14: return x * (y * y - r1_12);
        case 15: return (y * y - r1_12) * z;
        case 16: return y * (z * z - r1_12);
        case 17: return (x * x - r1_12) * z;
        case 18: return x * (z * z - r1_12);
        default: return x * y * z;
    }
}

// the polynomial at node M, the terms whose monomial vanishes there left out
template <int M, int K = 0>
__device__ __forceinline__ double node_value(const double* c, double acc = 0.0) {
    if constexpr (K == 20) {
        return acc;
    } else {
        constexpr double w = mono(K, node(M, 0), node(M, 1), node(M, 2));
        if constexpr (w == 0.0) return node_value<M, K + 1>(c, acc);
        else return node_value<M, K + 1>(c, fma(c[K], w, acc));
    }
}

// true when some node has rho < floor
template <int M = 0>
__device__ __forceinline__ bool rho_fails(const double* c) {
    if constexpr (M == 33) {
        return false;
    } else {
        return (node_value<M>(c) < RHO_FLOOR) | rho_fails<M + 1>(c);
    }
}

// true when some node has p + P_inf(phi) < floor; phi's coefficients at ph[q * 128]
template <int M = 0>
__device__ __forceinline__ bool prs_fails(const double* cp, const double* ph, const Eos& e, bool stiff) {
    if constexpr (M == 33) {
        return false;
    } else {
        double pinf = 0.0;
        if (stiff) {
            double cphi[20];
#pragma unroll
            for (int q = 0; q < 20; ++q) cphi[q] = ph[q * 128];
            const double phi = node_value<M>(cphi);
            pinf = mix_pinf(e, mix_g(e, phi), phi);
        }
        return (node_value<M>(cp) + pinf < PRS_FLOOR) | prs_fails<M + 1>(cp, ph, e, stiff);
    }
}

// ---------------------------------------------------------------- kernels
__device__ __forceinline__ long long ghost_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + GW) * g.gy + (j + GW)) * g.gx + (i + GW);
}
__device__ __forceinline__ long long ext_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + 1) * g.ey + (j + 1)) * g.ex + (i + 1);
}

__global__ void __launch_bounds__(128) k_m3_ghost(const double* __restrict__ U, double* __restrict__ G, Geo g, Eos e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - GW;
    const int j = blockIdx.y - GW, k = blockIdx.z - GW;
    if (i >= g.nx + GW) return;
    int fi = 0, fj = 0, fk = 0;
    const int mi = bmap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = bmap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const int mk = bmap(k, g.nz, g.bc[4], g.bc[5], &fk);
    const long long src = ((long long)mk * g.ny + mj) * g.nx + mi;
    double Q[MV], V[MV];
#pragma unroll
    for (int c = 0; c < MV; ++c) Q[c] = __ldg(U + c * g.N + src);
    cons2prim(e, Q, V);
    if (fi) V[1] = -V[1];
    if (fj) V[2] = -V[2];
    if (fk) V[3] = -V[3];
    const long long dst = ghost_index(g, i, j, k);
#pragma unroll
    for (int c = 0; c < MV; ++c) G[c * g.GN + dst] = V[c];
}

__device__ __forceinline__ void gather33(const double* __restrict__ p, int sy, int sz, double* s) {
    s[0] = __ldg(p);
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
        s[S1(0, off)] = __ldg(p + off);
        s[S1(1, off)] = __ldg(p + off * sy);
        s[S1(2, off)] = __ldg(p + off * sz);
    }
#pragma unroll
    for (int sa = 0; sa < 2; ++sa)
#pragma unroll
        for (int sb = 0; sb < 2; ++sb) {
            s[SQ(0, sa, 1, sb)] = __ldg(p + (2 * sa - 1) + (2 * sb - 1) * sy);
            s[SQ(1, sa, 2, sb)] = __ldg(p + (2 * sa - 1) * sy + (2 * sb - 1) * sz);
            s[SQ(0, sa, 2, sb)] = __ldg(p + (2 * sa - 1) + (2 * sb - 1) * sz);
        }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) s[SO(a, b, d)] = __ldg(p + (2 * a - 1) + (2 * b - 1) * sy + (2 * d - 1) * sz);
}

__device__ __forceinline__ void store_traces6(double* __restrict__ T, const Geo& g, long long e, int c, const double* cf) {
    double tr[8];
    double* Tc = T + (long long)c * NTR * g.NE + e;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d == 0) face_traces<double, 0>(cf, tr);
        else if (d == 1) face_traces<double, 1>(cf, tr);
        else face_traces<double, 2>(cf, tr);
#pragma unroll
        for (int q = 0; q < 8; ++q) Tc[(long long)(8 * d + q) * g.NE] = tr[q];
    }
}

// T[c][face*4+gp][extended cell]; the cells the faces of owned cells need (at most one
// coordinate outside the grid)
__global__ void __launch_bounds__(128) k_m3_recon(const double* __restrict__ G, double* __restrict__ T, Geo g, Eos e,
                                                  DevScalars* __restrict__ ds) {
    __shared__ double sphi[20 * 128];  // phi's coefficients, [q][thread]
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > g.nx || j > g.ny) return;
    const int outside = (i < 0 || i >= g.nx) + (j < 0 || j >= g.ny) + (k < 0 || k >= g.nz);
    if (outside > 1) return;
    const long long e_ = ext_index(g, i, j, k), ge = ghost_index(g, i, j, k);
    const int sy = g.gx, sz = g.gx * g.gy;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    double* ph = sphi + tid;
    const bool stiff = e.p1 != 0.0 || e.p2 != 0.0;
    bool fail = false;
    {  // density: the node check and its traces
        double s[33], cf[20];
        gather33(G + 0 * g.GN + ge, sy, sz, s);
        cweno4<double>(s, false, cf);
        fail |= rho_fails(cf);
        store_traces6(T, g, e_, 0, cf);
    }
    {  // volume fraction: coefficients kept for the pressure check
        double s[33], cf[20];
        gather33(G + 5 * g.GN + ge, sy, sz, s);
        cweno4<double>(s, false, cf);
        if (stiff) {
#pragma unroll
            for (int q = 0; q < 20; ++q) ph[q * 128] = cf[q];
        }
        store_traces6(T, g, e_, 5, cf);
    }
    {  // pressure
        double s[33], cf[20];
        gather33(G + 4 * g.GN + ge, sy, sz, s);
        cweno4<double>(s, false, cf);
        fail |= prs_fails(cf, ph, e, stiff);
        store_traces6(T, g, e_, 4, cf);
    }
#pragma unroll 1
    for (int c = 1; c < 4; ++c) {
        double s[33], cf[20];
        gather33(G + c * g.GN + ge, sy, sz, s);
        cweno4<double>(s, false, cf);
        store_traces6(T, g, e_, c, cf);
    }
    if (fail) {  // first order: every trace is the cell value (rhs_function.c:302-306)
#pragma unroll 1
        for (int c = 0; c < MV; ++c) {
            const double v = G[c * g.GN + ge];
#pragma unroll
            for (int q = 0; q < NTR; ++q) T[((long long)c * NTR + q) * g.NE + e_] = v;
        }
        if (outside == 0) atomicAdd(&ds->fallback, 1ull);
    }
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// faces normal to D: the low cell's face 2D+1 against the high cell's face 2D
template <int D>
__global__ void __launch_bounds__(128) k_m3_faces(const double* __restrict__ T, double* __restrict__ F, Geo g, Eos e,
                                                  DevScalars* __restrict__ ds, int slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    const bool visc = e.mu1 != 0.0 || e.mu2 != 0.0;
    double smax = 0.0, smaxv = 0.0;
    bool bad = false;
    if (i < fx && j < fy) {
        const long long eR = ext_index(g, i, j, k);
        const long long eL = ext_index(g, i - (D == 0), j - (D == 1), k - (D == 2));
        double acc[MF];
#pragma unroll
        for (int c = 0; c < MF; ++c) acc[c] = 0.0;
#pragma unroll 1
        for (int gp = 0; gp < 4; ++gp) {
            double VL[MV], VR[MV], fc[MF];
#pragma unroll
            for (int c = 0; c < MV; ++c) {
                VL[c] = __ldg(T + ((long long)c * NTR + (2 * D + 1) * 4 + gp) * g.NE + eL);
                VR[c] = __ldg(T + ((long long)c * NTR + (2 * D) * 4 + gp) * g.NE + eR);
            }
            const Side SL = make_side(e, VL, bad), SR = make_side(e, VR, bad);
            const double s = rot_hllc7(SL, SR, D == 0 ? 1.0 : 0.0, D == 1 ? 1.0 : 0.0, D == 2 ? 1.0 : 0.0, fc);
            smax = fmax(smax, s);
            if (visc) {  // PDEViscFluxPrim's speed (4/3) mu / rho on both sides
                const double r4_3 = 4. / 3;
                const double svl = r4_3 * (VL[5] * e.mu1 + (1.0 - VL[5]) * e.mu2) / VL[0];
                const double svr = r4_3 * (VR[5] * e.mu1 + (1.0 - VR[5]) * e.mu2) / VR[0];
                smaxv = fmax(smaxv, fmax(svl, svr));
            }
#pragma unroll
            for (int c = 0; c < MF; ++c) acc[c] += 0.25 * fc[c];
        }
        const long long nf = (long long)fx * fy * (g.nz + (D == 2));
        const long long f = ((long long)k * fy + j) * fx + i;
#pragma unroll
        for (int c = 0; c < MF; ++c) F[c * nf + f] = acc[c];
        if (bad) {
            const int ci = i < g.nx ? i : g.nx - 1, cj = j < g.ny ? j : g.ny - 1, ck = k < g.nz ? k : g.nz - 1;
            atomicMin(&ds->bad, (unsigned long long)(((long long)ck * g.ny + cj) * g.nx + ci));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
        smaxv = fmax(smaxv, __shfl_xor_sync(0xffffffffu, smaxv, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (smax > 0.0) atomic_max_pos(&ds->smax_bits[slot], smax);
        if (smaxv > 0.0) atomic_max_pos(&ds->smaxv_bits[slot], smaxv);
    }
}

struct Stage {
    double a, b, c;  // out = a U + b W + (c dt) L (a = 0: W + (c dt) L); rhs_only: out = L
    int rhs_only;
};

// RHS (rhs_function.c:507-552) and the stage combination; Win: the stage input, whose
// volume fraction multiplies the normal-velocity flux in the phi equation
// Win, U, W and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_m3_update(const double* __restrict__ Fx, const double* __restrict__ Fy,
                                                   const double* __restrict__ Fz, const double* Win,
                                                   const double* U, const double* W,
                                                   double* out, Geo g, double r1_h, Stage st,
                                                   const DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long nfx = (long long)(g.nx + 1) * g.ny * g.nz, nfy = (long long)g.nx * (g.ny + 1) * g.nz,
                    nfz = (long long)g.nx * g.ny * (g.nz + 1);
    const long long ix = ((long long)k * g.ny + j) * (g.nx + 1) + i;
    const long long iy = ((long long)k * (g.ny + 1) + j) * g.nx + i;
    const long long cell = ((long long)k * g.ny + j) * g.nx + i, iz = cell;
    const long long sxy = (long long)g.nx * g.ny;
    const double phi = Win[5 * g.N + cell];
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt;
    double L[MV];
#pragma unroll
    for (int c = 0; c < 5; ++c)
        L[c] = -r1_h * (Fx[c * nfx + ix + 1] - Fx[c * nfx + ix]) - r1_h * (Fy[c * nfy + iy + g.nx] - Fy[c * nfy + iy]) -
               r1_h * (Fz[c * nfz + iz + sxy] - Fz[c * nfz + iz]);
    L[5] = -r1_h * ((Fx[5 * nfx + ix + 1] - phi * Fx[6 * nfx + ix + 1]) - (Fx[5 * nfx + ix] - phi * Fx[6 * nfx + ix])) -
           r1_h * ((Fy[5 * nfy + iy + g.nx] - phi * Fy[6 * nfy + iy + g.nx]) - (Fy[5 * nfy + iy] - phi * Fy[6 * nfy + iy])) -
           r1_h * ((Fz[5 * nfz + iz + sxy] - phi * Fz[6 * nfz + iz + sxy]) - (Fz[5 * nfz + iz] - phi * Fz[6 * nfz + iz]));
#pragma unroll
    for (int c = 0; c < MV; ++c) {
        double v;
        if (st.rhs_only) {
            v = L[c];
        } else {
            v = W[c * g.N + cell] + cdt * L[c];
            if (st.a != 0.0) v = st.a * U[c * g.N + cell] + st.b * W[c * g.N + cell] + cdt * L[c];
        }
        out[c * g.N + cell] = v;
    }
}

// dt = (1/3) CFL h / (s_max + 2 s_visc / h) (rhs_function.c:559)
__host__ __device__ inline double m3_dt(double cfl_h, double r1_h, double smax, double smaxv) {
    return (1.0 / 3.0) * cfl_h / (smax + (r1_h * smaxv) * 2.0);
}

__global__ void k_m3_begin(DevScalars* ds, int dt_mode, int src, int use_src, int reset, double cfl_h, double r1_h) {
    if (use_src && dt_mode != HYPE_DT_FIXED) {
        ds->dt = m3_dt(cfl_h, r1_h, __longlong_as_double((long long)ds->smax_bits[src]),
                       __longlong_as_double((long long)ds->smaxv_bits[src]));
    }
    if (reset)
        for (int s = 0; s < 4; ++s) ds->smax_bits[s] = ds->smaxv_bits[s] = 0ull;
    ds->t += ds->dt;
}

__global__ void k_m3_reset_slot(DevScalars* ds, int slot) {
    ds->smax_bits[slot] = 0ull;
    ds->smaxv_bits[slot] = 0ull;
    ds->bad = ~0ull;
}

__global__ void k_m3_aos2soa(const double* __restrict__ a, double* __restrict__ s, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * MV) return;
    const long long cell = q / MV;
    s[(q - cell * MV) * N + cell] = a[q];
}
__global__ void k_m3_soa2aos(const double* __restrict__ s, double* __restrict__ a, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * MV) return;
    const long long cell = q / MV;
    a[q] = s[(q - cell * MV) * N + cell];
}

}  // namespace mp3d
}  // namespace hype

using namespace hype;
using namespace hype::mp3d;

static inline double bits2d3(unsigned long long b) {
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

struct hype_mp3d {
    hype_mp3d_params p;
    Geo g;
    Eos e;
    cudaStream_t stream = nullptr;
    double *U = nullptr, *W = nullptr, *S = nullptr, *L = nullptr, *G = nullptr, *T = nullptr;
    double *Fx = nullptr, *Fy = nullptr, *Fz = nullptr, *aos = nullptr;
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;
};

static int m3_rhs(hype_mp3d* m, const double* Win, int slot) {
    const Geo& g = m->g;
    k_m3_ghost<<<dim3(cdiv(g.gx, 128), g.gy, g.nz + 2 * GW), 128, 0, m->stream>>>(Win, m->G, g, m->e);
    k_m3_recon<<<dim3(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2), dim3(32, 4), 0, m->stream>>>(m->G, m->T, g,
                                                                                                     m->e, m->ds);
    const dim3 bf(32, 4);
    k_m3_faces<0><<<dim3(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), bf, 0, m->stream>>>(m->T, m->Fx, g, m->e, m->ds, slot);
    k_m3_faces<1><<<dim3(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz), bf, 0, m->stream>>>(m->T, m->Fy, g, m->e, m->ds, slot);
    k_m3_faces<2><<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1), bf, 0, m->stream>>>(m->T, m->Fz, g, m->e, m->ds, slot);
    HYPE_LAUNCHED(5);
    return HYPE_OK;
}

static int m3_update(hype_mp3d* m, const double* Win, const double* U, const double* W, double* out, Stage st) {
    const Geo& g = m->g;
    k_m3_update<<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 8), g.nz), dim3(32, 8), 0, m->stream>>>(
        m->Fx, m->Fy, m->Fz, Win, U, W, out, g, 1.0 / m->p.h, st, m->ds);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

extern "C" int hype_mp3d_create(const hype_mp3d_params* p, hype_mp3d** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3 || !(p->h > 0) || !(p->cfl > 0)) return HYPE_ERR_ARG;
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] < HYPE_BC_PERIODIC || p->bc[f] > HYPE_BC_TRANSMISSIVE) return HYPE_ERR_ARG;
    for (int d = 0; d < 3; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (!(p->g1 > 1.0) || !(p->g2 > 1.0) || !(p->mu1 >= 0.0) || !(p->mu2 >= 0.0)) return HYPE_ERR_ARG;
    if (p->dt_mode < HYPE_DT_MONITOR || p->dt_mode > HYPE_DT_FIXED) return HYPE_ERR_ARG;
    hype_mp3d* m = new hype_mp3d();
    m->p = *p;
    m->e = Eos{p->g1, p->p1, p->g2, p->p2, p->mu1, p->mu2};
    Geo& g = m->g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    for (int f = 0; f < 6; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny * p->nz;
    g.ex = p->nx + 2; g.ey = p->ny + 2;
    g.NE = (long long)g.ex * g.ey * (p->nz + 2);
    g.gx = p->nx + 2 * GW; g.gy = p->ny + 2 * GW;
    g.GN = (long long)g.gx * g.gy * (p->nz + 2 * GW);
    const size_t sN = sizeof(double) * MV * (size_t)g.N;
    cudaError_t ce = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    auto al = [&](double** ptr, size_t bytes) {
        if (ce == cudaSuccess) ce = cudaMalloc((void**)ptr, bytes);
    };
    al(&m->U, sN); al(&m->W, sN); al(&m->S, sN); al(&m->L, sN); al(&m->aos, sN);
    al(&m->G, sizeof(double) * MV * (size_t)g.GN);
    al(&m->T, sizeof(double) * MV * NTR * (size_t)g.NE);
    al(&m->Fx, sizeof(double) * MF * (size_t)(g.nx + 1) * g.ny * g.nz);
    al(&m->Fy, sizeof(double) * MF * (size_t)g.nx * (g.ny + 1) * g.nz);
    al(&m->Fz, sizeof(double) * MF * (size_t)g.nx * g.ny * (g.nz + 1));
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->ds, sizeof(DevScalars));
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&m->hs, sizeof(DevScalars));
    if (ce == cudaSuccess) {
        DevScalars z;
        memset(&z, 0, sizeof(z));
        z.bad = ~0ull;
        ce = cudaMemcpy(m->ds, &z, sizeof(z), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        set_last_error("hype_mp3d_create", ce);
        hype_mp3d_destroy(m);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = m;
    return HYPE_OK;
}

extern "C" void hype_mp3d_destroy(hype_mp3d* m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->U); cudaFree(m->W); cudaFree(m->S); cudaFree(m->L); cudaFree(m->aos); cudaFree(m->G); cudaFree(m->T);
    cudaFree(m->Fx); cudaFree(m->Fy); cudaFree(m->Fz); cudaFree(m->ds);
    if (m->hs) cudaFreeHost(m->hs);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

extern "C" int hype_mp3d_get_params(const hype_mp3d* m, hype_mp3d_params* out) {
    if (!m || !out) return HYPE_ERR_ARG;
    *out = m->p;
    return HYPE_OK;
}

static int m3_h2d(hype_mp3d* m, const double* aos, double* soa) {
    const long long N = m->g.N;
    HYPE_CK(cudaMemcpyAsync(m->aos, aos, sizeof(double) * MV * N, cudaMemcpyHostToDevice, m->stream));
    k_m3_aos2soa<<<cdiv(N * MV, 256), 256, 0, m->stream>>>(m->aos, soa, N);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int m3_d2h(hype_mp3d* m, const double* soa, double* aos) {
    const long long N = m->g.N;
    k_m3_soa2aos<<<cdiv(N * MV, 256), 256, 0, m->stream>>>(soa, m->aos, N);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, m->aos, sizeof(double) * MV * N, cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

static int m3_scalars(hype_mp3d* m) {
    HYPE_CK(cudaMemcpyAsync(m->hs, m->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp3d_upload(hype_mp3d* m, const double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    int rc = m3_h2d(m, U_aos, m->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp3d_download(hype_mp3d* m, double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    return m3_d2h(m, m->U, U_aos);
}

extern "C" int hype_mp3d_rhs(hype_mp3d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out) {
    (void)t;
    if (!m || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc = m3_h2d(m, U_aos, m->S);
    if (rc) return rc;
    k_m3_reset_slot<<<1, 1, 0, m->stream>>>(m->ds, 4);
    HYPE_LAUNCHED(1);
    if ((rc = m3_rhs(m, m->S, 4)) || (rc = m3_update(m, m->S, nullptr, nullptr, m->L, Stage{0.0, 0.0, 0.0, 1})))
        return rc;
    if ((rc = m3_scalars(m))) return rc;
    if (dt_out)
        *dt_out = m3_dt(m->p.cfl * m->p.h, 1.0 / m->p.h, bits2d3(m->hs->smax_bits[4]), bits2d3(m->hs->smaxv_bits[4]));
    const bool bad = m->hs->bad != ~0ull;
    if ((rc = m3_d2h(m, m->L, RHS_aos))) return rc;
    return bad ? HYPE_ERR_STATE : HYPE_OK;
}

extern "C" int hype_mp3d_step(hype_mp3d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells) {
    if (!m || nsteps < 0 || !t_inout || !dt_inout) return HYPE_ERR_ARG;
    const int mode = m->p.dt_mode;
    if (mode == HYPE_DT_FIXED && !(*dt_inout > 0)) return HYPE_ERR_ARG;
    const double cfl_h = m->p.cfl * m->p.h, r1_h = 1.0 / m->p.h;
    DevScalars init;
    memset(&init, 0, sizeof(init));
    init.t = *t_inout;
    init.dt = *dt_inout;
    init.bad = ~0ull;
    HYPE_CK(cudaMemcpyAsync(m->ds, &init, sizeof(init), cudaMemcpyHostToDevice, m->stream));
    const bool first_from_rhs = (mode != HYPE_DT_FIXED) && !(*dt_inout > 0);
    // SSPRK(4,3) (PETSc TSSSP RKS3, 4 stages, hype.c:207-209)
    const Stage s12{0.0, 1.0, 0.5, 0}, s3{2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0};
    int rc;
    for (int s = 0; s < nsteps; ++s) {
        if (s == 0 && first_from_rhs) {
            // the initial RHS call of hype.c:168 is this step's first stage RHS
            if ((rc = m3_rhs(m, m->U, 0))) return rc;
            k_m3_begin<<<1, 1, 0, m->stream>>>(m->ds, mode, 0, 1, 0, cfl_h, r1_h);
            HYPE_LAUNCHED(1);
        } else {
            k_m3_begin<<<1, 1, 0, m->stream>>>(m->ds, mode, 3, mode == HYPE_DT_MONITOR && s > 0, 1, cfl_h, r1_h);
            HYPE_LAUNCHED(1);
            if ((rc = m3_rhs(m, m->U, 0))) return rc;
        }
        if ((rc = m3_update(m, m->U, m->U, m->U, m->W, s12))) return rc;
        if ((rc = m3_rhs(m, m->W, 1)) || (rc = m3_update(m, m->W, m->U, m->W, m->W, s12))) return rc;
        if ((rc = m3_rhs(m, m->W, 2)) || (rc = m3_update(m, m->W, m->U, m->W, m->W, s3))) return rc;
        if ((rc = m3_rhs(m, m->W, 3)) || (rc = m3_update(m, m->W, m->U, m->W, m->U, s12))) return rc;
    }
    if ((rc = m3_scalars(m))) return rc;
    *t_inout = m->hs->t;
    *dt_inout = (nsteps > 0 && mode == HYPE_DT_MONITOR)
                    ? m3_dt(cfl_h, r1_h, bits2d3(m->hs->smax_bits[3]), bits2d3(m->hs->smaxv_bits[3]))
                    : m->hs->dt;
    if (fallback_cells) *fallback_cells = (long long)m->hs->fallback;
    return m->hs->bad == ~0ull ? HYPE_OK : HYPE_ERR_STATE;
}

extern "C" int hype_mp3d_sync(hype_mp3d* m) {
    if (!m) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" void* hype_mp3d_stream(hype_mp3d* m) { return m ? (void*)m->stream : nullptr; }
