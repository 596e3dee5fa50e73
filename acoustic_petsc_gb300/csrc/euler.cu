// euler.cu -- 3D Euler CWENO4 + Rusanov RHS and the SSPRK(4,3) stepper on sm_103a.
//
// Per RK stage three kernels run on the context's stream:
//   recon  : one thread per cell of the extended box [-1,n]^3 that some face of an
//            owned cell needs; ghost values come from the boundary index map
//            (replaces DMGlobalToLocal + the BC sweeps of
//            3d/weno4/Navier-Stokes-3D/rhs_function.c:41-181); writes the 24 face
//            Gauss-point traces of each variable (rhs_function.c:185-274);
//   faces  : one thread per face and direction; four Rusanov solves at the 2x2
//            Gauss points, the weighted flux (rhs_function.c:276-417), the block
//            max of the wave speed (atomicMax on the bit pattern: speeds are >= 0)
//            and the admissibility flag (replaces MPI_Abort, pde.c:56-66);
//   update : flux divergence (rhs_function.c:419-433) fused with the SSP stage
//            combination; dt comes from device memory, so a whole step needs no
//            host round trip.
// State and stage buffers are SoA doubles [c][k][j][i]; traces are stored in the
// arithmetic type R of the reconstruction ([c][face][gp][extended cell]).
#include <cuda_runtime.h>

#include <string.h>

#include <algorithm>
#include <type_traits>

#include <vector>

#include "euler_df64.cuh"
#include "euler_kernels.cuh"
#include "mlp_kernels.cuh"

namespace hype {
namespace euler {

struct Geo {
    int nx, ny, nz;
    int bc[6];
    long long N;   // owned cells
    long long NE;  // extended cells (n+2)^3
    int ex, ey;    // extended x, y extents
    int gx, gy;    // ghosted x, y extents (n + 2 GW): the stage input with its ghost layers
    long long GN;  // ghosted cells per variable
};

// ghost width of the stage-input copy: the reconstruction of the first ghost layer
// (i = -1) reads offsets down to -3
constexpr int GW = 3;

__host__ __device__ __forceinline__ void set_ghost_extents(Geo& g) {
    g.gx = g.nx + 2 * GW;
    g.gy = g.ny + 2 * GW;
    g.GN = (long long)g.gx * g.gy * (g.nz + 2 * GW);
}

__device__ __forceinline__ long long ghost_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + GW) * g.gy + (j + GW)) * g.gx + (i + GW);
}

// device scalars of one context
struct DevScalars {
    unsigned long long smax_bits[6];  // [0..3] stages, [4] RHS-only calls
    double dt;
    double t;
    unsigned long long bad;  // first inadmissible cell (ULLONG_MAX: none)
    long long rhs_evals;
    unsigned long long smaxv_bits[6];  // viscous wave speeds, same slots
};

// viscosity of the Navier-Stokes terms (mu = 0: Euler)
struct Visc {
    double mu, kc, vmax, r1_h;  // viscosity, cv mu gamma / Pr, max(4 mu / 3, gamma mu / Pr), 1 / h
};

__device__ __forceinline__ long long ext_index(const Geo& g, int i, int j, int k) {
    return ((long long)(k + 1) * (g.ny + 2) + (j + 1)) * (long long)g.ex + (i + 1);
}

// boundary maps of the offsets -2..2 of one cell along each direction
struct StencilMap {
    int mi[5], mj[5], mk[5];
    int fi, fj, fk;  // bit o set: offset o-2 is a reflective ghost
};

__device__ __forceinline__ void make_map(const Geo& g, int i, int j, int k, StencilMap& m) {
    m.fi = m.fj = m.fk = 0;
#pragma unroll
    for (int o = 0; o < 5; ++o) {
        int f = 0;
        m.mi[o] = bmap(i + o - 2, g.nx, g.bc[0], g.bc[1], &f);
        m.fi |= f << o;
        f = 0;
        m.mj[o] = bmap(j + o - 2, g.ny, g.bc[2], g.bc[3], &f);
        m.fj |= f << o;
        f = 0;
        m.mk[o] = bmap(k + o - 2, g.nz, g.bc[4], g.bc[5], &f);
        m.fk |= f << o;
    }
}

// one value of variable c at offset (oi, oj, ok) from the state (S = double) or its
// FP32 mirror (S = float); a reflective ghost negates the momentum component normal
// to its wall
template <typename R, typename S>
__device__ __forceinline__ R ldw(const S* __restrict__ Wc, int c, const Geo& g, const StencilMap& m, int oi, int oj,
                                 int ok) {
    S v = __ldg(Wc + ((long long)m.mk[ok + 2] * g.ny + m.mj[oj + 2]) * g.nx + m.mi[oi + 2]);
    const int fm = (c == 1) ? m.fi : (c == 2) ? m.fj : (c == 3) ? m.fk : 0;
    const int o = (c == 1) ? oi : (c == 2) ? oj : ok;
    if (fm && ((fm >> (o + 2)) & 1)) v = -v;
    return (R)v;
}

// the 33-point stencil of variable c (index map of euler_kernels.cuh)
template <typename R, typename S>
__device__ __forceinline__ void gather33(const S* __restrict__ Wc, int c, const Geo& g, const StencilMap& m, R* s) {
    s[0] = ldw<R>(Wc, c, g, m, 0, 0, 0);
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
        s[S1(0, off)] = ldw<R>(Wc, c, g, m, off, 0, 0);
        s[S1(1, off)] = ldw<R>(Wc, c, g, m, 0, off, 0);
        s[S1(2, off)] = ldw<R>(Wc, c, g, m, 0, 0, off);
    }
#pragma unroll
    for (int sa = 0; sa < 2; ++sa)
#pragma unroll
        for (int sb = 0; sb < 2; ++sb) {
            s[SQ(0, sa, 1, sb)] = ldw<R>(Wc, c, g, m, 2 * sa - 1, 2 * sb - 1, 0);
            s[SQ(1, sa, 2, sb)] = ldw<R>(Wc, c, g, m, 0, 2 * sa - 1, 2 * sb - 1);
            s[SQ(0, sa, 2, sb)] = ldw<R>(Wc, c, g, m, 2 * sa - 1, 0, 2 * sb - 1);
        }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int d = 0; d < 2; ++d) s[SO(a, b, d)] = ldw<R>(Wc, c, g, m, 2 * a - 1, 2 * b - 1, 2 * d - 1);
}

// Admissibility of a cell's FP32 traces, decided while they are stored: the density
// (c = 0) and the squared momentum (c = 1..3) of each trace point wait in the thread's
// column of a per-warp shared-memory scratch [2][NTR][32] until the energy (c = 4)
// arrives; the test is pde.c:56-66's floors, p >= 1e-12 as
// (gamma-1)(E rho - |m|^2/2) >= 1e-12 rho.
struct TraceCheck {
    float* col;  // the lane's column: [q * 32] density, [(NTR + q) * 32] |m|^2
    float g1;
    bool ok;
};

// The FP32 admissibility test of one trace point from its density, squared momentum
// |m|^2 (accumulated x, y, z in that order: m2 = mx*mx, then fma(my, my, m2), fma(mz, mz, m2))
// and energy; every operation is an explicitly rounded intrinsic, so the unfused and the fused
// stage kernels take the same decision bit for bit.
__device__ __forceinline__ bool adm_f32(float rho, float m2, float E, float g1) {
    return (rho >= 1.0e-14f) &&
           (__fmul_rn(g1, __fmaf_rn(E, rho, __fmul_rn(-0.5f, m2))) >= __fmul_rn(1.0e-12f, rho));
}

__device__ __forceinline__ void trace_check(TraceCheck* ck, int c, int q, float v) {
    float* r = ck->col + q * 32;
    float* m = ck->col + (NTR + q) * 32;
    if (c == 0) {
        *r = v;
    } else if (c == 1) {
        *m = __fmul_rn(v, v);
    } else if (c < 4) {
        *m = __fmaf_rn(v, v, *m);
    } else {
        ck->ok = ck->ok && adm_f32(*r, *m, v, ck->g1);
    }
}

// the 24 face traces of one variable into the trace array (FP32 traces: and into the
// admissibility check ck when one is given)
template <typename R>
__device__ __forceinline__ void store_traces(R* __restrict__ T, const Geo& g, long long e, int c, const R* cf,
                                             TraceCheck* ck = nullptr) {
    R tr[8];
    R* Tc = T + (long long)c * NTR * g.NE + e;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (d == 0) face_traces<R, 0>(cf, tr);
        else if (d == 1) face_traces<R, 1>(cf, tr);
        else face_traces<R, 2>(cf, tr);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            Tc[(long long)(8 * d + q) * g.NE] = tr[q];
            if (sizeof(R) == sizeof(float) && ck) trace_check(ck, c, 8 * d + q, (float)tr[q]);
        }
    }
}

// density and pressure at the 24 face Gauss-point traces of one cell (what the
// Riemann solver consumes) against the floors of pde.c:56-66
template <typename R>
__device__ __forceinline__ bool traces_admissible(const R* __restrict__ T, const Geo& g, long long e, double gm1) {
    if (sizeof(R) == sizeof(float)) {  // FP32 traces: p >= floor as (E rho - |m|^2/2)(gamma-1) >= floor rho
        const float g1 = (float)gm1;
        for (int q = 0; q < NTR; ++q) {
            const float rho = (float)T[((long long)0 * NTR + q) * g.NE + e];
            const float mx = (float)T[((long long)1 * NTR + q) * g.NE + e];
            const float my = (float)T[((long long)2 * NTR + q) * g.NE + e];
            const float mz = (float)T[((long long)3 * NTR + q) * g.NE + e];
            const float E = (float)T[((long long)4 * NTR + q) * g.NE + e];
            if (!(rho >= 1.0e-14f) || !(g1 * (E * rho - 0.5f * (mx * mx + my * my + mz * mz)) >= 1.0e-12f * rho)) return false;
        }
        return true;
    }
    for (int q = 0; q < NTR; ++q) {
        const double rho = (double)T[((long long)0 * NTR + q) * g.NE + e];
        const double mx = (double)T[((long long)1 * NTR + q) * g.NE + e];
        const double my = (double)T[((long long)2 * NTR + q) * g.NE + e];
        const double mz = (double)T[((long long)3 * NTR + q) * g.NE + e];
        const double E = (double)T[((long long)4 * NTR + q) * g.NE + e];
        const double p = gm1 * (E - 0.5 * (mx * mx + my * my + mz * mz) / rho);
        if (!(rho >= 1.0e-14) || !(p >= 1.0e-12)) return false;
    }
    return true;
}


// Device-side ghost fill (what DMGlobalToLocal does for the reference's DMDA, with
// the boundary treatment of rhs_function.c's ghost loops): the stage input W (owned
// cells, SoA) copied into G with GW ghost layers on every side, each ghost the value
// its per-axis boundary map picks (periodic wrap, reflective mirror, transmissive
// copy) and a reflective ghost's wall-normal momentum negated; G is in the
// reconstruction's precision, so the FP32 form converts each value once per stage.
// One thread per ghosted cell of an x-y plane (flat index over the plane, so no block is left
// mostly idle at the end of a row), one grid row per plane.
constexpr int kGhostThreads = 256;

template <typename R>
__global__ void __launch_bounds__(kGhostThreads) k_ghost(const double* __restrict__ W, R* __restrict__ G, Geo g) {
    const int q = blockIdx.x * kGhostThreads + threadIdx.x;
    if (q >= g.gx * g.gy) return;
    const int i = q % g.gx - GW, j = q / g.gx - GW, k = blockIdx.y - GW;
    int fi = 0, fj = 0, fk = 0;
    const int mi = bmap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = bmap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const int mk = bmap(k, g.nz, g.bc[4], g.bc[5], &fk);
    const long long src = ((long long)mk * g.ny + mj) * g.nx + mi;
    const long long dst = ghost_index(g, i, j, k);
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double v = __ldg(W + (long long)c * g.N + src);
        if ((c == 1 && fi) || (c == 2 && fj) || (c == 3 && fk)) v = -v;
        G[(long long)c * g.GN + dst] = (R)v;
    }
}

inline dim3 ghost_grid(const Geo& g) { return dim3(cdiv((long long)g.gx * g.gy, kGhostThreads), g.nz + 2 * GW); }

// the 33-point stencil (index map of euler_kernels.cuh) of one variable about p = &G[cell]
template <typename R>
__device__ __forceinline__ void gather33g(const R* __restrict__ p, int sy, int sz, R* s) {
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

// first-order traces (all higher coefficients zero): the fallback of
// 3d/weno4/Viscous-Multiphase-Fourth-Order/rhs_function.c:297-305
template <typename R>
__device__ __forceinline__ void store_first_order_g(const R* __restrict__ G, R* __restrict__ T, const Geo& g,
                                                    long long ge, long long e) {
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        const R v = __ldg(G + (long long)c * g.GN + ge);
        R* Tc = T + (long long)c * NTR * g.NE + e;
        for (int q = 0; q < NTR; ++q) Tc[(long long)q * g.NE] = v;
    }
}

// Reconstruction of every owned cell and of the first ghost layer (faces of the
// domain boundary); the FP32 form checks admissibility in dynamic shared memory
// (4 warps x 2 x NTR x 32 floats, launched only with the positivity fallback on).
template <typename R>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 1)
    k_recon(const R* __restrict__ G, R* __restrict__ T, Geo g, int recon, int pad, double gm1,
            unsigned long long* __restrict__ counters, double* __restrict__ C4 = nullptr, double c4_scale = 1.0) {
    extern __shared__ float ck_dyn[];
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > g.nx || j > g.ny) return;
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    if (gi + gj + gk > 1) return;  // edge/corner ghosts feed no face of an owned cell
    const long long e = ext_index(g, i, j, k), ge = ghost_index(g, i, j, k);
    const int sy = g.gx, sz = g.gx * g.gy;
    constexpr bool f32 = sizeof(R) == sizeof(float);
    TraceCheck ck{ck_dyn + threadIdx.y * (2 * NTR * 32) + threadIdx.x, (float)gm1, true};
    TraceCheck* ckp = (f32 && pad) ? &ck : nullptr;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        R s[33], cf[20];
        gather33g<R>(G + (long long)c * g.GN + ge, sy, sz, s);
        if (recon == HYPE_RECON_WENO3) weno3<R>(s, cf);
        else cweno4<R>(s, recon == HYPE_RECON_LINEAR4, cf);
        store_traces<R>(T, g, e, c, cf, ckp);
        if (sizeof(R) == sizeof(double) && C4) {  // the R4 polynomial, whose gradients the viscous fluxes take
            R r4[20];
            if (recon == HYPE_RECON_LINEAR4) {
#pragma unroll
                for (int q = 0; q < 20; ++q) r4[q] = cf[q];
            } else {
                cweno4<R>(s, true, r4);
            }
#pragma unroll
            for (int q = 0; q < 20; ++q) C4[((long long)c * 20 + q) * g.NE + e] = (double)r4[q] * c4_scale;
        }
    }
    if (pad && !(f32 ? ck.ok : traces_admissible<R>(T, g, e, gm1))) {
        store_first_order_g<R>(G, T, g, ge, e);
        if (!gi && !gj && !gk) atomicAdd(&counters[1], 1ull);
    }
}

// HYPE_PREC_DF64: the per-variable reference value r_c of one stage, the stage input's
// value at cell 0 rounded to a 24-bit significand (the deviations u - r_c are formed in
// FP64, the traces r_c + deviation are rounded once in FP64)
__device__ __forceinline__ double df_ref(const double* __restrict__ W, const Geo& g, int c) {
    double r;
    df_round24(__ldg(W + (long long)c * g.N), r);
    return r;
}

// ghost fill as k_ghost, storing the deviation from r_c as a double-float pair
__global__ void __launch_bounds__(128) k_ghost_df(const double* __restrict__ W, df64* __restrict__ G, Geo g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - GW;
    const int j = blockIdx.y - GW, k = blockIdx.z - GW;
    if (i >= g.nx + GW) return;
    int fi = 0, fj = 0, fk = 0;
    const int mi = bmap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = bmap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const int mk = bmap(k, g.nz, g.bc[4], g.bc[5], &fk);
    const long long src = ((long long)mk * g.ny + mj) * g.nx + mi;
    const long long dst = ghost_index(g, i, j, k);
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double v = __ldg(W + (long long)c * g.N + src);
        if ((c == 1 && fi) || (c == 2 && fj) || (c == 3 && fk)) v = -v;
        G[(long long)c * g.GN + dst] = df_from_double(v - df_ref(W, g, c));
    }
}

// The stage's reference state r in double-float (its components are the rounded cell-0
// values, exact FP32 numbers) and the pieces of F(r) the deviation form of the flux uses
struct DfRef {
    df64 rho, m[3], E, u[3], p, H;  // u = m / rho, p = (gamma - 1)(E - m.u / 2), H = E + p
};

__device__ __forceinline__ DfRef df_refstate(const double* __restrict__ W, const Geo& g, df64 gm1) {
    DfRef R;
    double fd;
    R.rho = df64{df_round24(__ldg(W), fd), 0.0f};
#pragma unroll
    for (int i = 0; i < 3; ++i) R.m[i] = df64{df_round24(__ldg(W + (long long)(1 + i) * g.N), fd), 0.0f};
    R.E = df64{df_round24(__ldg(W + 4LL * g.N), fd), 0.0f};
    const df64 ir = df_div(dfc(1.0), R.rho);
#pragma unroll
    for (int i = 0; i < 3; ++i) R.u[i] = R.m[i] * ir;
    R.p = (R.E - df_scale((R.m[0] * R.u[0] + R.m[1] * R.u[1]) + R.m[2] * R.u[2], 0.5f)) * gm1;
    R.H = R.E + R.p;
    return R;
}

// One side of a face in deviation form: for the trace r + d, the flux deviation
// dF = F(r + d) - F(r) along D (PDEConsFlux, Navier-Stokes-3D/pde.c:40-88) built only from
// deviation-sized terms -- du = (d_m - u_r d_rho) / rho, d(m.u) = sum m_r du + d_m u,
// dp = (gamma - 1)(d_E - d(m.u) / 2), dF_m = m_r du_n + d_m u_n (+ dp), dF_E = H_r du_n +
// (d_E + dp) u_n -- and the wave speed |u_n| + sqrt(gamma p / rho); the floors of pde.c:56-66
template <int D>
__device__ __forceinline__ void dev_side(const DfRef& R, const df64* d, df64 gm1, df64 gam, df64* dF, df64& sp,
                                         bool& bad) {
    const df64 rho = R.rho + d[0];
    const df64 ir = df_div(dfc(1.0), rho);
    df64 du[3], u[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        du[i] = (d[1 + i] - R.u[i] * d[0]) * ir;
        u[i] = R.u[i] + du[i];
    }
    const df64 dmu = (R.m[0] * du[0] + d[1] * u[0]) + ((R.m[1] * du[1] + d[2] * u[1]) + (R.m[2] * du[2] + d[3] * u[2]));
    const df64 dp = (d[4] - df_scale(dmu, 0.5f)) * gm1;
    const df64 p = R.p + dp;
    bad |= !(rho.hi >= 1.0e-14f && p.hi >= 1.0e-12f);
    dF[0] = d[1 + D];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const df64 f = R.m[i] * du[D] + d[1 + i] * u[D];
        dF[1 + i] = (i == D) ? f + dp : f;
    }
    dF[4] = R.H * du[D] + (d[4] + dp) * u[D];
    sp = df_abs(u[D]) + df_sqrt(gam * p * ir);
}

// density and pressure of the 24 double-float deviation traces against the floors: an FP32
// estimate from the leading parts settles every point whose density and pressure lie clear
// of the floors by more than its rounding (1e-5 of the magnitudes involved, NaN never
// clear); the rest are decided in double-float
__device__ __forceinline__ bool traces_admissible_df(const df64* __restrict__ T, const Geo& g, long long e,
                                                     const DfRef& R, df64 gm1) {
    for (int q = 0; q < NTR; ++q) {
        df64 d[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) d[c] = T[((long long)c * NTR + q) * g.NE + e];
        const float rf = R.rho.hi + d[0].hi, Ef = R.E.hi + d[4].hi;
        const float mxf = R.m[0].hi + d[1].hi, myf = R.m[1].hi + d[2].hi, mzf = R.m[2].hi + d[3].hi;
        const float m2 = mxf * mxf + myf * myf + mzf * mzf;
        const float kef = 0.5f * m2 / rf;
        const float pf = gm1.hi * (Ef - kef);
        const float tr = 1.0e-5f * (fabsf(R.rho.hi) + fabsf(d[0].hi)) + 1.0e-14f;
        const float tp = 1.0e-5f * gm1.hi * (fabsf(Ef) + fabsf(kef)) + 1.0e-12f;
        if (rf > 1.0e-14f + tr && pf > 1.0e-12f + tp) continue;  // clearly admissible
        if (rf < 1.0e-14f - tr || pf < 1.0e-12f - tp) return false;  // clearly not
        const df64 rho = R.rho + d[0];
        const df64 mx = R.m[0] + d[1], my = R.m[1] + d[2], mz = R.m[2] + d[3];
        const df64 p = ((R.E + d[4]) - df_scale(df_div((mx * mx + my * my) + mz * mz, rho), 0.5f)) * gm1;
        if (!(rho.hi >= 1.0e-14f) || !(p.hi >= 1.0e-12f)) return false;
    }
    return true;
}

// CWENO4 / R4 reconstruction in double-float on the deviations (euler_df64.cuh).  DFT: the
// traces stay double-float deviations for k_faces_df (Rusanov); otherwise they go out as FP64
// values r_c + deviation, the array the FP64 face solvers consume.
// (two blocks per SM: with more warps in flight over this long unrolled body the
// instruction-cache misses cost more than the latency they hide)
template <bool DFT>
__global__ void __launch_bounds__(128, 2)
    k_recon_df(const df64* __restrict__ G, void* __restrict__ Tv, const double* __restrict__ W, Geo g, int recon,
               int pad, double gm1, unsigned long long* __restrict__ counters, df64* __restrict__ C4 = nullptr,
               double c4_scale = 1.0) {
    double* T = (double*)Tv;
    df64* Td = (df64*)Tv;
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    if (i > g.nx || j > g.ny) return;
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    if (gi + gj + gk > 1) return;
    const long long e = ext_index(g, i, j, k), ge = ghost_index(g, i, j, k);
    const int sy = g.gx, sz = g.gx * g.gy;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        df64 s[33], cf[20];
        {
            const df64* p = G + (long long)c * g.GN + ge;
            s[0] = p[0];
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
                s[S1(0, off)] = p[off];
                s[S1(1, off)] = p[off * sy];
                s[S1(2, off)] = p[off * sz];
            }
#pragma unroll
            for (int sa = 0; sa < 2; ++sa)
#pragma unroll
                for (int sb = 0; sb < 2; ++sb) {
                    s[SQ(0, sa, 1, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sy];
                    s[SQ(1, sa, 2, sb)] = p[(2 * sa - 1) * sy + (2 * sb - 1) * sz];
                    s[SQ(0, sa, 2, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sz];
                }
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 2; ++b)
#pragma unroll
                    for (int d = 0; d < 2; ++d) s[SO(a, b, d)] = p[(2 * a - 1) + (2 * b - 1) * sy + (2 * d - 1) * sz];
        }
        cweno4_df(s, recon == HYPE_RECON_LINEAR4, cf);
        if (C4) {  // the R4 polynomial (times 1/h) of the deviations, for the viscous face gradients
            const df64 sc = df_from_double(c4_scale);
            df64 r4[20];
            if (recon == HYPE_RECON_LINEAR4) {
#pragma unroll
                for (int q = 0; q < 20; ++q) r4[q] = cf[q];
            } else {
                cweno4_df(s, true, r4);
            }
#pragma unroll
            for (int q = 1; q < 20; ++q) C4[((long long)c * 20 + q) * g.NE + e] = r4[q] * sc;
        }
        df64 tr[8];
        if constexpr (DFT) {
            df64* Tc = Td + (long long)c * NTR * g.NE + e;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d == 0) face_traces_df<0>(cf, tr);
                else if (d == 1) face_traces_df<1>(cf, tr);
                else face_traces_df<2>(cf, tr);
#pragma unroll
                for (int q = 0; q < 8; ++q) Tc[(long long)(8 * d + q) * g.NE] = tr[q];
            }
        } else {
            const double r = df_ref(W, g, c);
            double* Tc = T + (long long)c * NTR * g.NE + e;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                if (d == 0) face_traces_df<0>(cf, tr);
                else if (d == 1) face_traces_df<1>(cf, tr);
                else face_traces_df<2>(cf, tr);
#pragma unroll
                for (int q = 0; q < 8; ++q) Tc[(long long)(8 * d + q) * g.NE] = r + df_to_double(tr[q]);
            }
        }
    }
    if (!pad) return;
    bool ok;
    if constexpr (DFT) {
        const df64 gm1d = df_from_double(gm1);
        ok = traces_admissible_df(Td, g, e, df_refstate(W, g, gm1d), gm1d);
    } else {
        ok = traces_admissible<double>(T, g, e, gm1);
    }
    if (!ok) {
#pragma unroll 1
        for (int c = 0; c < NV; ++c) {
            const df64 dv = G[(long long)c * g.GN + ge];
            const double v = df_ref(W, g, c) + df_to_double(dv);
            for (int q = 0; q < NTR; ++q) {
                if constexpr (DFT) Td[((long long)c * NTR + q) * g.NE + e] = dv;
                else T[((long long)c * NTR + q) * g.NE + e] = v;
            }
        }
        if (!gi && !gj && !gk) atomicAdd(&counters[1], 1ull);
    }
}


// Indicator-gated reconstruction: the network scores the cell from its three
// directional 5-point stencils; flagged or low-confidence cells take the full
// CWENO4, the others the linear R4 -- unless the linear traces give a density
// or pressure below the floors at any face Gauss point, in which case the cell
// is redone with CWENO4 (positivity fallback).
template <typename R>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 1)
    k_recon_learned(const R* __restrict__ G, R* __restrict__ T, Geo g, const mlp::MmaWeights* __restrict__ wts,
                    float logit_thr, double gm1, int pad, unsigned long long* __restrict__ counters) {
    // per warp: the staged network inputs, later the FP32 admissibility scratch
    static_assert(mlp::ROWS * mlp::RSTRIDE * sizeof(__nv_bfloat16) >= 2 * NTR * 32 * sizeof(float), "scratch");
    __shared__ __align__(16) __nv_bfloat16 rows[4][mlp::ROWS * mlp::RSTRIDE];
    __shared__ float lg[4][mlp::ROWS];
    __shared__ unsigned cnt[2];
    if (threadIdx.x == 0 && threadIdx.y == 0) cnt[0] = cnt[1] = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    bool active = !(i > g.nx || j > g.ny);
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    active = active && (gi + gj + gk <= 1);
    const long long ge = active ? ghost_index(g, i, j, k) : 0;
    const int sy = g.gx, sz = g.gx * g.gy;
    // features of the warp's 32 cells (3 rows each) staged as BF16, scored on the tensor cores
    __nv_bfloat16* my_rows = rows[threadIdx.y] + threadIdx.x * 3 * mlp::RSTRIDE;
    float sc[NV];
    if (active) {
        const float rho = (float)__ldg(G + ge), E = (float)__ldg(G + 4 * g.GN + ge);
#pragma unroll
        for (int c = 0; c < NV; ++c) sc[c] = mlp::var_scale<float>(c, rho, E);
    }
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        float x[mlp::NIN];
        const int st = d == 0 ? 1 : d == 1 ? sy : sz;
        if (active) {
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const R* p = G + (long long)c * g.GN + ge;
                float s5[5];
#pragma unroll
                for (int o = 0; o < 5; ++o) s5[o] = (float)__ldg(p + (o - 2) * st);
                mlp::normalise5(s5, sc[c], x + c * 5);
            }
        }
        mlp::stage_row(my_rows + d * mlp::RSTRIDE, x, active);
    }
    __syncthreads();  // counters cleared, rows staged
    mlp::warp_logits(wts, rows[threadIdx.y], lg[threadIdx.y]);
    __syncwarp();
    const float best = fmaxf(lg[threadIdx.y][threadIdx.x * 3], fmaxf(lg[threadIdx.y][threadIdx.x * 3 + 1],
                                                                       lg[threadIdx.y][threadIdx.x * 3 + 2]));
    if (active) {
        const long long e = ext_index(g, i, j, k);
        constexpr bool f32 = sizeof(R) == sizeof(float);
        TraceCheck ck{reinterpret_cast<float*>(rows[threadIdx.y]) + threadIdx.x, (float)gm1, true};
        bool full = best > logit_thr;
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            ck.ok = true;
#pragma unroll 1
            for (int c = 0; c < NV; ++c) {
                R s[33], cf[20];
                gather33g<R>(G + (long long)c * g.GN + ge, sy, sz, s);
                cweno4<R>(s, !full, cf);
                store_traces<R>(T, g, e, c, cf, f32 ? &ck : nullptr);
            }
            if (f32 ? ck.ok : traces_admissible<R>(T, g, e, gm1)) break;
            if (full) {  // CWENO4 itself inadmissible: first order (when enabled)
                if (pad) {
                    store_first_order_g<R>(G, T, g, ge, e);
                    if (!gi && !gj && !gk) atomicAdd(&cnt[1], 1u);
                }
                break;
            }
            full = true;  // the R4 traces broke positivity: redo the cell with CWENO4
        }
        if (full && !gi && !gj && !gk && best > logit_thr) atomicAdd(&cnt[0], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        if (cnt[0]) atomicAdd(&counters[0], (unsigned long long)cnt[0]);
        if (cnt[1]) atomicAdd(&counters[1], (unsigned long long)cnt[1]);
    }
}

// Indicator-gated reconstruction of the double-float form: the network reads the FP32 leading
// parts of the deviations (its normalised stencils are shift-invariant; the magnitude floors
// take the density and energy as r + deviation), flagged or low-confidence cells take the
// double-float CWENO4 and the others its R4 limit, with the positivity redo of k_recon_learned.
// DFT as for k_recon_df.
template <bool DFT>
__global__ void __launch_bounds__(128, 2)
    k_recon_learned_df(const df64* __restrict__ G, void* __restrict__ Tv, const double* __restrict__ W, Geo g,
                       const mlp::MmaWeights* __restrict__ wts, float logit_thr, double gm1, int pad,
                       unsigned long long* __restrict__ counters) {
    __shared__ __align__(16) __nv_bfloat16 rows[4][mlp::ROWS * mlp::RSTRIDE];
    __shared__ float lg[4][mlp::ROWS];
    __shared__ unsigned cnt[2];
    if (threadIdx.x == 0 && threadIdx.y == 0) cnt[0] = cnt[1] = 0;
    double* T = (double*)Tv;
    df64* Td = (df64*)Tv;
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    bool active = !(i > g.nx || j > g.ny);
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    active = active && (gi + gj + gk <= 1);
    const long long ge = active ? ghost_index(g, i, j, k) : 0;
    const int sy = g.gx, sz = g.gx * g.gy;
    __nv_bfloat16* my_rows = rows[threadIdx.y] + threadIdx.x * 3 * mlp::RSTRIDE;
    float sc[NV];
    if (active) {
        double fd;
        const float rho = df_round24(__ldg(W), fd) + G[ge].hi;
        const float E = df_round24(__ldg(W + 4LL * g.N), fd) + G[4 * g.GN + ge].hi;
#pragma unroll
        for (int c = 0; c < NV; ++c) sc[c] = mlp::var_scale<float>(c, rho, E);
    }
#pragma unroll 1
    for (int d = 0; d < 3; ++d) {
        float x[mlp::NIN];
        const int st = d == 0 ? 1 : d == 1 ? sy : sz;
        if (active) {
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const df64* p = G + (long long)c * g.GN + ge;
                float s5[5];
#pragma unroll
                for (int o = 0; o < 5; ++o) s5[o] = p[(o - 2) * st].hi;
                mlp::normalise5(s5, sc[c], x + c * 5);
            }
        }
        mlp::stage_row(my_rows + d * mlp::RSTRIDE, x, active);
    }
    __syncthreads();
    mlp::warp_logits(wts, rows[threadIdx.y], lg[threadIdx.y]);
    __syncwarp();
    const float best = fmaxf(lg[threadIdx.y][threadIdx.x * 3], fmaxf(lg[threadIdx.y][threadIdx.x * 3 + 1],
                                                                       lg[threadIdx.y][threadIdx.x * 3 + 2]));
    if (active) {
        const long long e = ext_index(g, i, j, k);
        const df64 gm1d = df_from_double(gm1);
        bool full = best > logit_thr;
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
#pragma unroll 1
            for (int c = 0; c < NV; ++c) {
                df64 s[33], cf[20];
                const df64* p = G + (long long)c * g.GN + ge;
                s[0] = p[0];
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    const int off = (o == 0) ? -2 : (o == 1) ? -1 : (o == 2) ? 1 : 2;
                    s[S1(0, off)] = p[off];
                    s[S1(1, off)] = p[off * sy];
                    s[S1(2, off)] = p[off * sz];
                }
#pragma unroll
                for (int sa = 0; sa < 2; ++sa)
#pragma unroll
                    for (int sb = 0; sb < 2; ++sb) {
                        s[SQ(0, sa, 1, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sy];
                        s[SQ(1, sa, 2, sb)] = p[(2 * sa - 1) * sy + (2 * sb - 1) * sz];
                        s[SQ(0, sa, 2, sb)] = p[(2 * sa - 1) + (2 * sb - 1) * sz];
                    }
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 2; ++b)
#pragma unroll
                        for (int dd = 0; dd < 2; ++dd)
                            s[SO(a, b, dd)] = p[(2 * a - 1) + (2 * b - 1) * sy + (2 * dd - 1) * sz];
                cweno4_df(s, !full, cf);
                df64 tr[8];
                const double r = df_ref(W, g, c);
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (d == 0) face_traces_df<0>(cf, tr);
                    else if (d == 1) face_traces_df<1>(cf, tr);
                    else face_traces_df<2>(cf, tr);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const long long at = ((long long)c * NTR + 8 * d + q) * g.NE + e;
                        if constexpr (DFT) Td[at] = tr[q];
                        else T[at] = r + df_to_double(tr[q]);
                    }
                }
            }
            bool ok;
            if constexpr (DFT) ok = traces_admissible_df(Td, g, e, df_refstate(W, g, gm1d), gm1d);
            else ok = traces_admissible<double>(T, g, e, gm1);
            if (ok) break;
            if (full) {  // CWENO4 itself inadmissible: first order (when enabled)
                if (pad) {
#pragma unroll 1
                    for (int c = 0; c < NV; ++c) {
                        const df64 dv = G[(long long)c * g.GN + ge];
                        const double v = df_ref(W, g, c) + df_to_double(dv);
                        for (int q = 0; q < NTR; ++q) {
                            if constexpr (DFT) Td[((long long)c * NTR + q) * g.NE + e] = dv;
                            else T[((long long)c * NTR + q) * g.NE + e] = v;
                        }
                    }
                    if (!gi && !gj && !gk) atomicAdd(&cnt[1], 1u);
                }
                break;
            }
            full = true;  // the R4 traces broke positivity: redo the cell with CWENO4
        }
        if (full && !gi && !gj && !gk && best > logit_thr) atomicAdd(&cnt[0], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        if (cnt[0]) atomicAdd(&counters[0], (unsigned long long)cnt[0]);
        if (cnt[1]) atomicAdd(&counters[1], (unsigned long long)cnt[1]);
    }
}

// Indicator training data: for every stride-th owned cell, the three directional
// normalised stencils (X[s][3][25]) and D[s], the largest change that the nonlinear
// CWENO4 weights make to a face trace relative to the linear R4 polynomial, over the
// 5 variables and 24 traces, in units of the variable's magnitude in the cell (labels:
// D > tau).
__global__ void __launch_bounds__(128) k_features(const double* __restrict__ W, Geo g, long long stride, long long ns,
                                                  float* __restrict__ X, float* __restrict__ D) {
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const long long cell = s * stride;
    const int i = (int)(cell % g.nx), j = (int)((cell / g.nx) % g.ny), k = (int)(cell / ((long long)g.nx * g.ny));
    StencilMap m;
    make_map(g, i, j, k, m);
    const double rho = ldw<double, double>(W, 0, g, m, 0, 0, 0), E = ldw<double, double>(W + 4 * g.N, 4, g, m, 0, 0, 0);
    double dmax = 0.0;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        double st[33], cf[20], cl[20], ta[8], tb[8];
        gather33<double, double>(W + (long long)c * g.N, c, g, m, st);
        cweno4<double>(st, false, cf);
        cweno4<double>(st, true, cl);
        const double scale = mlp::var_scale<double>(c, rho, E) + 1e-30;
        double dd = 0.0;
        face_traces<double, 0>(cf, ta);
        face_traces<double, 0>(cl, tb);
        for (int q = 0; q < 8; ++q) dd = fmax(dd, fabs(ta[q] - tb[q]));
        face_traces<double, 1>(cf, ta);
        face_traces<double, 1>(cl, tb);
        for (int q = 0; q < 8; ++q) dd = fmax(dd, fabs(ta[q] - tb[q]));
        face_traces<double, 2>(cf, ta);
        face_traces<double, 2>(cl, tb);
        for (int q = 0; q < 8; ++q) dd = fmax(dd, fabs(ta[q] - tb[q]));
        dmax = fmax(dmax, dd / scale);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float s5[5] = {(float)st[S1(d, -2)], (float)st[S1(d, -1)], (float)st[0], (float)st[S1(d, 1)],
                                 (float)st[S1(d, 2)]};
            mlp::normalise5(s5, (float)mlp::var_scale<double>(c, rho, E), X + (s * 3 + d) * mlp::NIN + c * 5);
        }
    }
    D[s] = (float)dmax;
}

__device__ __forceinline__ void atomic_max_pos(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

// The viscous fluxes of one face side at its 4 Gauss points, 0.125 F_v each, added to
// av: NS = +1 for the low cell's high face, -1 for the high cell's low face.  The
// traces come from T, the gradients from the cell's R4 coefficients (stored times 1/h).
template <int D, int NS>
__device__ __forceinline__ double visc_side(const double* __restrict__ T, const double* __restrict__ C4, const Geo& g,
                                            long long e, double gamma, const Visc& vp, double* av) {
    FaceGrad fg[NV][3];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        const double* p = C4 + (long long)c * 20 * g.NE + e;
        fg[c][0] = face_grad<D, NS, 0>(p, g.NE);
        fg[c][1] = face_grad<D, NS, 1>(p, g.NE);
        fg[c][2] = face_grad<D, NS, 2>(p, g.NE);
    }
    constexpr int face = 2 * D + (NS > 0 ? 1 : 0);
    double sv = 0.0;
    auto at = [&](auto gpc) {
        constexpr int gp = decltype(gpc)::value;
        double Q[NV], G[NV][3], Fv[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            Q[c] = __ldg(T + ((long long)c * NTR + face * 4 + gp) * g.NE + e);
#pragma unroll
            for (int b = 0; b < 3; ++b) G[c][b] = fg_eval<gp>(fg[c][b]);
        }
        sv = fmax(sv, visc_flux<D>(Q, G, gamma - 1.0, vp.mu, vp.kc, vp.vmax, Fv));
#pragma unroll
        for (int c = 0; c < NV; ++c) av[c] = fma(0.125, Fv[c], av[c]);
    };
    at(std::integral_constant<int, 0>{});
    at(std::integral_constant<int, 1>{});
    at(std::integral_constant<int, 2>{});
    at(std::integral_constant<int, 3>{});
    return sv;
}

// Face fluxes of direction D.  Face index (i,j,k) is the face on the low side of
// cell (i,j,k); along D it runs to n (the high face of the last cell).
// Rusanov faces of the double-float form in deviation form: with F(r) dropped (it is the
// same at every face, so the divergence does not see it), the stored flux is
// 1/2 (dF_L + dF_R) - 1/2 s (d_R - d_L) at each Gauss point, weight 1/4, where s is the
// larger wave speed (pde.c:164-187); every term has the size of the deviations, so the
// 48-bit significand meets the FP64 form's error bars with the face solver on the FP32 pipe.
// one side's share of PDEViscRiemannSolver (Navier-Stokes-3D/pde.c:386-404) in double-float:
// 1/8 F_v at each of the 4 Gauss points of the side's face, from its traces (r + deviation)
// and the R4 gradients of the deviations; returns the largest viscous speed
template <int D, int NS>
__device__ __forceinline__ double visc_side_df(const df64* __restrict__ T, const df64* __restrict__ C4, const Geo& g,
                                               long long e, const DfRef& R, df64 gm1, df64 mu, df64 kc, df64 vmax,
                                               df64* av) {
    FaceGradDf fg[NV][3];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        const df64* p = C4 + (long long)c * 20 * g.NE + e;
        fg[c][0] = face_grad_df<D, NS, 0>(p, g.NE);
        fg[c][1] = face_grad_df<D, NS, 1>(p, g.NE);
        fg[c][2] = face_grad_df<D, NS, 2>(p, g.NE);
    }
    constexpr int face = 2 * D + (NS > 0 ? 1 : 0);
    double sv = 0.0;
    auto at = [&](auto gpc) {
        constexpr int gp = decltype(gpc)::value;
        df64 Q[NV], Gq[NV][3], Fv[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            Q[c] = T[((long long)c * NTR + face * 4 + gp) * g.NE + e];
#pragma unroll
            for (int b = 0; b < 3; ++b) Gq[c][b] = fg_eval_df<gp>(fg[c][b]);
        }
        Q[0] = R.rho + Q[0];
#pragma unroll
        for (int i = 0; i < 3; ++i) Q[1 + i] = R.m[i] + Q[1 + i];
        Q[4] = R.E + Q[4];
        sv = fmax(sv, df_to_double(visc_flux_df<D>(Q, Gq, gm1, mu, kc, vmax, Fv)));
#pragma unroll
        for (int c = 0; c < NV; ++c) av[c] = av[c] + df_scale(Fv[c], 0.125f);
    };
    at(std::integral_constant<int, 0>{});
    at(std::integral_constant<int, 1>{});
    at(std::integral_constant<int, 2>{});
    at(std::integral_constant<int, 3>{});
    return sv;
}

template <int D, bool VISC = false>
__global__ void __launch_bounds__(128) k_faces_df(const df64* __restrict__ T, double* __restrict__ F,
                                                  const double* __restrict__ W, Geo g, double gamma,
                                                  DevScalars* __restrict__ ds, int slot,
                                                  const df64* __restrict__ C4 = nullptr,
                                                  Visc vp = Visc{0.0, 0.0, 0.0, 0.0}) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    double smax = 0.0, smaxv = 0.0;
    bool bad = false;
    if (i < fx && j < fy) {
        const long long eR = ext_index(g, i, j, k);
        const long long eL = ext_index(g, i - (D == 0), j - (D == 1), k - (D == 2));
        const df64 gm1 = df_from_double(gamma - 1.0), gam = df_from_double(gamma);
        const DfRef R = df_refstate(W, g, gm1);
        df64 acc[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = df64{0.0f, 0.0f};
#pragma unroll 1
        for (int gp = 0; gp < 4; ++gp) {
            df64 dL[NV], dR[NV], fL[NV], fR[NV], sL, sR;
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                dL[c] = T[((long long)c * NTR + (2 * D + 1) * 4 + gp) * g.NE + eL];
                dR[c] = T[((long long)c * NTR + (2 * D) * 4 + gp) * g.NE + eR];
            }
            dev_side<D>(R, dL, gm1, gam, fL, sL, bad);
            dev_side<D>(R, dR, gm1, gam, fR, sR, bad);
            const df64 sm = df_lt(sL, sR) ? sR : sL;
            smax = fmax(smax, df_to_double(sm));
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] + df_scale((fL[c] + fR[c]) - sm * (dR[c] - dL[c]), 0.125f);
        }
        if constexpr (VISC) {
            const df64 mu = df_from_double(vp.mu), kc = df_from_double(vp.kc), vmax = df_from_double(vp.vmax);
            smaxv = visc_side_df<D, 1>(T, C4, g, eL, R, gm1, mu, kc, vmax, acc);
            smaxv = fmax(smaxv, visc_side_df<D, -1>(T, C4, g, eR, R, gm1, mu, kc, vmax, acc));
        }
        const long long nf = (long long)fx * fy * (g.nz + (D == 2));
        const long long f = ((long long)k * fy + j) * fx + i;
#pragma unroll
        for (int c = 0; c < NV; ++c) F[c * nf + f] = df_to_double(acc[c]);
        if (bad) {
            const int ci = i < g.nx ? i : g.nx - 1, cj = j < g.ny ? j : g.ny - 1, ck = k < g.nz ? k : g.nz - 1;
            atomicMin(&ds->bad, (unsigned long long)(((long long)ck * g.ny + cj) * g.nx + ci));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    if ((threadIdx.x & 31) == 0 && smax > 0.0) atomic_max_pos(&ds->smax_bits[slot], smax);
    if constexpr (VISC) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) smaxv = fmax(smaxv, __shfl_xor_sync(0xffffffffu, smaxv, o));
        if ((threadIdx.x & 31) == 0 && smaxv > 0.0) atomic_max_pos(&ds->smaxv_bits[slot], smaxv);
    }
}

template <typename R, int D, int FLUX, bool VISC = false>
__global__ void __launch_bounds__(128) k_faces(const R* __restrict__ T, double* __restrict__ F, Geo g, double gamma,
                                               DevScalars* __restrict__ ds, int slot, const double* __restrict__ C4 = nullptr,
                                               Visc vp = Visc{0.0, 0.0, 0.0, 0.0}) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    double smax = 0.0, smaxv = 0.0;
    bool bad = false;
    const bool active = (i < fx && j < fy);
    if (active) {
        const long long eR = ext_index(g, i, j, k);
        const long long eL = ext_index(g, i - (D == 0), j - (D == 1), k - (D == 2));
        R acc[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = R(0);
        const R gm = (R)gamma, gm1 = (R)(gamma - 1.0);
#pragma unroll
        for (int gp = 0; gp < 4; ++gp) {
            R QL[NV], QR[NV], fl[NV];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                QL[c] = T[((long long)c * NTR + (2 * D + 1) * 4 + gp) * g.NE + eL];
                QR[c] = T[((long long)c * NTR + (2 * D) * 4 + gp) * g.NE + eR];
            }
            // Rusanov's 1/2 goes into the Gauss weight 1/4
            const R s = FLUX == HYPE_FLUX_RUSANOV ? rusanov<R, D, false>(QL, QR, gm, gm1, fl, bad)
                                                  : face_solver<R, D, FLUX>(QL, QR, gm, gm1, fl, bad);
            smax = fmax(smax, (double)s);
            const R wq = FLUX == HYPE_FLUX_RUSANOV ? R(0.125) : R(0.25);
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] += wq * fl[c];
        }
        if constexpr (VISC) {
            // PDEViscRiemannSolver (Navier-Stokes-3D/pde.c:386-404): 0.5 (F_v(L) + F_v(R)) at
            // each Gauss point, weight 0.25, added to the inviscid flux (rhs_function.c:310-316)
            double av[NV];
#pragma unroll
            for (int c = 0; c < NV; ++c) av[c] = 0.0;
            smaxv = visc_side<D, 1>((const double*)T, C4, g, eL, gamma, vp, av);
            smaxv = fmax(smaxv, visc_side<D, -1>((const double*)T, C4, g, eR, gamma, vp, av));
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] += (R)av[c];
        }
        const long long nf = (long long)fx * fy * (g.nz + (D == 2));
        const long long f = ((long long)k * fy + j) * fx + i;
#pragma unroll
        for (int c = 0; c < NV; ++c) F[c * nf + f] = (double)acc[c];
        if (bad) {
            const int ci = i < g.nx ? i : g.nx - 1, cj = j < g.ny ? j : g.ny - 1, ck = k < g.nz ? k : g.nz - 1;
            atomicMin(&ds->bad, (unsigned long long)(((long long)ck * g.ny + cj) * g.nx + ci));
        }
    }
    // warp max, one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = fmax(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    if ((threadIdx.x & 31) == 0 && smax > 0.0) atomic_max_pos(&ds->smax_bits[slot], smax);
    if constexpr (VISC) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) smaxv = fmax(smaxv, __shfl_xor_sync(0xffffffffu, smaxv, o));
        if ((threadIdx.x & 31) == 0 && smaxv > 0.0) atomic_max_pos(&ds->smaxv_bits[slot], smaxv);
    }
}

// stage combination: out = a*U + b*W + (c*dt)*L   (L = divergence of the face fluxes)
struct Stage {
    double a, b, c;
    int rhs_only;
};

// The flux divergence of one cell from its six face fluxes, -(1/h)(dx + dy + dz) with
// dx = F(i+1/2) - F(i-1/2) etc., as explicitly rounded operations in a fixed order: the x and y
// part first, then the z difference (the fused stage kernel forms the two parts one plane apart).
__device__ __forceinline__ double div_xy(double dx, double dy, double r1_h) {
    return __fma_rn(-r1_h, dy, __dmul_rn(-r1_h, dx));
}
__device__ __forceinline__ double div_z(double pxy, double dz, double r1_h) { return __fma_rn(-r1_h, dz, pxy); }

// the FP32 form's divergence: its face fluxes are FP32 values, differenced and scaled in FP32
// (neighbouring fluxes lie within a factor 2 of each other in smooth flow, where the FP32
// differences are exact); only the stage combination is FP64
__device__ __forceinline__ float div_xy_f(float dx, float dy, float r1_h) {
    return __fmaf_rn(-r1_h, dy, __fmul_rn(-r1_h, dx));
}
__device__ __forceinline__ float div_z_f(float pxy, float dz, float r1_h) { return __fmaf_rn(-r1_h, dz, pxy); }

// the SSP stage value a U + b W + (c dt) L (b = 1 when a = 0), explicitly rounded
__device__ __forceinline__ double stage_value(const Stage& st, double cdt, double u, double w, double L) {
    if (st.rhs_only) return L;
    if (st.a == 0.0) return __fma_rn(cdt, L, w);
    return __fma_rn(cdt, L, __fma_rn(st.b, w, __dmul_rn(st.a, u)));
}

// U, W and out may be one array (in-place stages), so they carry no __restrict__.
// F32: the face fluxes hold FP32 values (the FP32 form); the divergence is formed in FP32
template <bool F32 = false>
__global__ void __launch_bounds__(256) k_update(const double* __restrict__ Fx, const double* __restrict__ Fy,
                                                const double* __restrict__ Fz, const double* U,
                                                const double* W, double* out, Geo g, double r1_h,
                                                Stage st, const DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= g.nx || j >= g.ny) return;
    const long long nfx = (long long)(g.nx + 1) * g.ny * g.nz, nfy = (long long)g.nx * (g.ny + 1) * g.nz,
                    nfz = (long long)g.nx * g.ny * (g.nz + 1);
    const long long ix = ((long long)k * g.ny + j) * (g.nx + 1) + i;
    const long long iy = ((long long)k * (g.ny + 1) + j) * g.nx + i;
    const long long iz = ((long long)k * g.ny + j) * g.nx + i;
    const long long cell = iz;
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        double L;
        if constexpr (F32) {
            const float r1hf = (float)r1_h;
            const float pxy = div_xy_f((float)Fx[c * nfx + ix + 1] - (float)Fx[c * nfx + ix],
                                       (float)Fy[c * nfy + iy + g.nx] - (float)Fy[c * nfy + iy], r1hf);
            L = df_f2d(div_z_f(pxy, (float)Fz[c * nfz + iz + (long long)g.nx * g.ny] - (float)Fz[c * nfz + iz], r1hf));
        } else {
            const double pxy =
                div_xy(Fx[c * nfx + ix + 1] - Fx[c * nfx + ix], Fy[c * nfy + iy + g.nx] - Fy[c * nfy + iy], r1_h);
            L = div_z(pxy, Fz[c * nfz + iz + (long long)g.nx * g.ny] - Fz[c * nfz + iz], r1_h);
        }
        const double u = (!st.rhs_only && st.a != 0.0) ? U[c * g.N + cell] : 0.0;
        const double w = st.rhs_only ? 0.0 : W[c * g.N + cell];
        out[c * g.N + cell] = stage_value(st, cdt, u, w, L);
    }
}

// ---------------------------------------------------------------- fused FP32 stage
// One pass per RK stage for the FP32 reconstruction + Rusanov flux form: reconstruction of
// every variable, the 24 face traces, the Rusanov solves at the face Gauss points, the flux
// divergence, the wave-speed maximum, the admissibility word and the SSP stage combination,
// with the face traces kept in shared memory (the unfused kernels write 120 traces per cell to
// HBM and read them back: 960 B per cell-stage of FP32 traffic).  It follows the loop
// structure of 3d/weno4/Navier-Stokes-3D/rhs_function.c:183-433 (reconstruct, evaluate the
// face traces, solve per face Gauss point, difference) over tiles instead of the whole box.
//
// Layout: a block is FS_TW warps of 32 lanes.  Lane l of warp w holds cell
// (i0 + l - 1, j0 + w - 1) of an x-y tile: lanes 1..30 and warps 1..FS_TW-2 are the owned
// cells, lane 0 / 31 and warp 0 / FS_TW-1 the one-cell ring whose traces the tile's boundary
// faces need (the ring is reconstructed again by the neighbouring tile: 80 ring cells beside
// the 300 owned ones per plane).  The block marches its tile along z; the +z traces of a plane stay in the
// thread's registers as the -z side of the next plane's z faces, and each cell's divergence
// is completed one plane later, when its +z face flux exists.  Blocks are persistent, one per
// SM (the trace and flux arrays take 188 KB of shared memory), and split the tiles' planes into equal
// contiguous runs: a run re-reconstructs one plane below and one above it.
// Every arithmetic step is the unfused kernels' (cweno4 / weno3, face_traces, rusanov, the
// admissibility test and the divergence use the same device functions and explicit roundings),
// so both paths give bit-identical results.
constexpr int FS_TW = 12;                        // warps per block (at most 168 registers per thread)
constexpr int FS_NT = 32 * FS_TW;                // 384 threads
constexpr int FS_OX = 30, FS_OY = FS_TW - 2;     // owned tile: 30 x 10 cells
constexpr int FS_NQ = NV * NTR;                  // traces per cell
// traces [c][q][thread] and the -y face fluxes [c][thread] (FP32): 192,000 B, which leaves 60 KB of
// the SM's L1 for the stencil gathers
constexpr size_t FS_SMEM = sizeof(float) * (FS_NQ + NV) * FS_NT;

__host__ __device__ inline long long fs_tiles_x(int nx) { return (nx + FS_OX - 1) / FS_OX; }
__host__ __device__ inline long long fs_tiles_y(int ny) { return (ny + FS_OY - 1) / FS_OY; }

// one Rusanov face (weight 1/8 per Gauss point, as k_faces): L side trace q0L.., R side q0R..
// read from the shared trace array (columns tL, tR) or, for the z faces' low side, from registers
__device__ __forceinline__ void fs_face(const float* __restrict__ S, int tL, int tR, int qL, int qR,
                                        const float (*zl)[4], float gm, float gm1, float* Fd, float& smax,
                                        bool& bad, int D) {
    float acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = 0.0f;
#pragma unroll
    for (int gp = 0; gp < 4; ++gp) {
        float QL[NV], QR[NV], fl[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            QL[c] = zl ? zl[c][gp] : S[(c * NTR + qL + gp) * FS_NT + tL];
            QR[c] = S[(c * NTR + qR + gp) * FS_NT + tR];
        }
        float s;
        if (D == 0) s = rusanov<float, 0, false>(QL, QR, gm, gm1, fl, bad);
        else if (D == 1) s = rusanov<float, 1, false>(QL, QR, gm, gm1, fl, bad);
        else s = rusanov<float, 2, false>(QL, QR, gm, gm1, fl, bad);
        smax = fmaxf(smax, s);
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] += 0.125f * fl[c];
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) Fd[c] = acc[c];
}

// a hint that the line holding *a will be read soon (into L2); a must lie inside its array
__device__ __forceinline__ void prefetch_l2(const void* a) { asm volatile("prefetch.global.L2 [%0];" ::"l"(a)); }

__device__ __forceinline__ void fs_bad(DevScalars* ds, const Geo& g, int i, int j, int k) {
    const int ci = i < g.nx ? i : g.nx - 1, cj = j < g.ny ? j : g.ny - 1, ck = k < g.nz ? k : g.nz - 1;
    atomicMin(&ds->bad, (unsigned long long)(((long long)ck * g.ny + cj) * g.nx + ci));
}

// one cell's 24 traces of every variable into its column of the shared array (linear: R4)
__device__ __forceinline__ void fs_recon_cell(float* __restrict__ S, const float* __restrict__ G, const Geo& g,
                                              long long ge, int t, bool linear, bool weno) {
    const int sy = g.gx, sz = g.gx * g.gy;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        float s[33], cf[20], tr[8];
        gather33g<float>(G + (long long)c * g.GN + ge, sy, sz, s);
        if (weno) weno3<float>(s, cf);
        else cweno4<float>(s, linear, cf);
        float* Sc = S + (c * NTR) * FS_NT + t;
        face_traces<float, 0>(cf, tr);
#pragma unroll
        for (int q = 0; q < 8; ++q) Sc[q * FS_NT] = tr[q];
        face_traces<float, 1>(cf, tr);
#pragma unroll
        for (int q = 0; q < 8; ++q) Sc[(8 + q) * FS_NT] = tr[q];
        face_traces<float, 2>(cf, tr);
#pragma unroll
        for (int q = 0; q < 8; ++q) Sc[(16 + q) * FS_NT] = tr[q];
    }
}

// the cell's 24 traces (its own column) against the density / pressure floors
__device__ __forceinline__ bool fs_admissible(const float* __restrict__ S, int t, float gm1) {
    bool ok = true;
#pragma unroll 4
    for (int q = 0; q < NTR; ++q) {
        const float rho = S[(0 * NTR + q) * FS_NT + t];
        float m2 = __fmul_rn(S[(1 * NTR + q) * FS_NT + t], S[(1 * NTR + q) * FS_NT + t]);
        m2 = __fmaf_rn(S[(2 * NTR + q) * FS_NT + t], S[(2 * NTR + q) * FS_NT + t], m2);
        m2 = __fmaf_rn(S[(3 * NTR + q) * FS_NT + t], S[(3 * NTR + q) * FS_NT + t], m2);
        ok = ok && adm_f32(rho, m2, S[(4 * NTR + q) * FS_NT + t], gm1);
    }
    return ok;
}

// The learned gate of the fused FP32 stage, scored ahead of it from the ghosted FP32 copy: one
// byte per extended cell, 1 where the network's largest directional logit exceeds the threshold.
// Scored are the cells the stage reconstructs (the owned cells and the one-cell frame without its
// edges and corners, which keep the zero the array is created with).  The features, their BF16
// rounding and the tensor-core scoring are k_recon_learned's, so the flags are that kernel's
// decisions bit for bit.  Block: 32 x 4 cells of one x-y plane, as k_recon_learned.
__global__ void __launch_bounds__(128) k_gate_f32(const float* __restrict__ G, unsigned char* __restrict__ flag, Geo g,
                                                  const mlp::MmaWeights* __restrict__ wts, float logit_thr) {
    __shared__ __align__(16) __nv_bfloat16 rows[4][mlp::ROWS * mlp::RSTRIDE];
    __shared__ float lg[4][mlp::ROWS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const int k = blockIdx.z - 1;
    const int gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny), gk = (k < 0 || k >= g.nz);
    const bool active = i <= g.nx && j <= g.ny && gi + gj + gk <= 1;
    const long long ge = active ? ghost_index(g, i, j, k) : 0;
    __nv_bfloat16* my_rows = rows[threadIdx.y] + threadIdx.x * 3 * mlp::RSTRIDE;
    const float* Gc = G + ge;  // variable c at Gc[c * GN + offset]
    float sc[NV];
    if (active) {
        const float rho = __ldg(Gc), E = __ldg(Gc + 4 * g.GN);
#pragma unroll
        for (int c = 0; c < NV; ++c) sc[c] = mlp::var_scale<float>(c, rho, E);
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float x[mlp::NIN];
#pragma unroll
        for (int q = 0; q < mlp::NIN; ++q) x[q] = 0.0f;  // the row of an inactive lane is never read
        const int stp = d == 0 ? 1 : d == 1 ? g.gx : g.gx * g.gy;
        if (active) {
            float s5[NV][5];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const float* p = Gc + (long long)c * g.GN;
#pragma unroll
                for (int o = 0; o < 5; ++o) s5[c][o] = __ldg(p + (o - 2) * stp);
            }
#pragma unroll
            for (int c = 0; c < NV; ++c) mlp::normalise5(s5[c], sc[c], x + c * 5);
        }
        mlp::stage_row(my_rows + d * mlp::RSTRIDE, x, true);
    }
    __syncwarp();  // the warp's rows staged
    mlp::warp_logits(wts, rows[threadIdx.y], lg[threadIdx.y]);
    __syncwarp();
    if (active) {
        const float* l3 = lg[threadIdx.y] + threadIdx.x * 3;
        flag[ext_index(g, i, j, k)] = fmaxf(l3[0], fmaxf(l3[1], l3[2])) > logit_thr ? 1 : 0;
    }
}

// The gate's flags widened to each cell's 3 x 3 x 3 neighbourhood (a cell is flagged when any cell
// around it is), for the cells the fused stage reconstructs.  Flags scored on a step's first stage
// and reused by its later stages then still cover a discontinuity that moves by less than a cell
// over the step (the CFL number bounds the wave speed x dt by the cell width).
__global__ void __launch_bounds__(128) k_gate_dilate(const unsigned char* __restrict__ f, unsigned char* __restrict__ o,
                                                     Geo g) {
    const int i = blockIdx.x * 128 + threadIdx.x, j = blockIdx.y, k = blockIdx.z;  // extended coordinates
    if (i >= g.ex) return;
    const int ey = g.ny + 2, ez = g.nz + 2;
    unsigned m = 0;
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk) {
        const int kk = k + dk;
        if (kk < 0 || kk >= ez) continue;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
            const int jj = j + dj;
            if (jj < 0 || jj >= ey) continue;
            const unsigned char* row = f + ((long long)kk * ey + jj) * g.ex;
            m |= __ldg(row + i);
            if (i > 0) m |= __ldg(row + i - 1);
            if (i + 1 < g.ex) m |= __ldg(row + i + 1);
        }
    }
    o[((long long)k * ey + j) * g.ex + i] = (unsigned char)m;
}

// LEARNED: the indicator gate of k_recon_learned, read from the flags k_gate_f32 wrote for this
// stage's input: flagged cells take CWENO4, the others R4, and a cell whose R4 traces break the
// floors is redone with CWENO4 (then first order with the positivity fallback)
template <bool LEARNED>
__global__ void __launch_bounds__(FS_NT, 1)
    k_stage_f32(const float* __restrict__ G, const double* U, const double* W, double* out, Geo g, int recon, int pad,
                double gamma, double r1_h, Stage st, DevScalars* __restrict__ ds, int slot,
                unsigned long long* __restrict__ counters, const unsigned char* __restrict__ gate = nullptr) {
    extern __shared__ float S[];  // traces [c][q][thread], then the -y face fluxes [c][thread]
    float* SFy = S + FS_NQ * FS_NT;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const float gm = (float)gamma, gm1 = (float)(gamma - 1.0);
    const long long tiles_x = fs_tiles_x(g.nx);
    const long long total = tiles_x * fs_tiles_y(g.ny) * g.nz;  // plane-units
    const long long b0 = (long long)blockIdx.x * total / gridDim.x, b1 = (long long)(blockIdx.x + 1) * total / gridDim.x;
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt;
    const float r1h = (float)r1_h;
    float smax = 0.0f;
    unsigned nfall = 0, nflag = 0;
    for (long long pos = b0; pos < b1;) {
        const long long tile = pos / g.nz;
        const int kb = (int)(pos - tile * g.nz);
        const int ke = (int)min((long long)g.nz, kb + (b1 - pos));
        pos += ke - kb;
        const int i0 = (int)(tile % tiles_x) * FS_OX, j0 = (int)(tile / tiles_x) * FS_OY;
        const int i = i0 + lane - 1, j = j0 + w - 1;
        const int ihi = min(i0 + FS_OX, g.nx), jhi = min(j0 + FS_OY, g.ny);  // owned: [i0, ihi) x [j0, jhi)
        const bool own_x = i >= i0 && i < ihi, own_y = j >= j0 && j < jhi;
        const bool ring_x = (i == i0 - 1 || i == ihi), ring_y = (j == j0 - 1 || j == jhi);
        const bool owned = own_x && own_y;
        const bool ring = (ring_x && own_y) || (own_x && ring_y);
        // the gate's flag of the next plane, loaded a plane ahead (cells in [-1, n] along x and y)
        unsigned char fnext = 0;
        if (LEARNED && (owned || ring)) fnext = gate[ext_index(g, i, j, kb - 1)];
        float zp[NV][4];    // +z traces of the previous plane
        float Fzp[NV];      // flux of the previous plane's -z face
        float Pp[NV];       // x/y part of the previous plane's divergence
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            Fzp[c] = Pp[c] = 0.0f;
#pragma unroll
            for (int q = 0; q < 4; ++q) zp[c][q] = 0.0f;
        }
#pragma unroll 1
        for (int k = kb - 1; k <= ke; ++k) {
            const bool edge = (k == kb - 1) || (k == ke);  // only the z traces of owned columns are used
            const bool active = owned || (ring && !edge);
            const long long ge = active ? ghost_index(g, i, j, k) : 0;
            bool full = false;
            if constexpr (LEARNED) {
                full = active && fnext != 0;
                if (full && owned && !edge) ++nflag;
                if ((owned || ring) && k < ke) fnext = gate[ext_index(g, i, j, k + 1)];
            }
            // ---- reconstruction: all 24 traces of each variable into the shared array
            if (active) {
                const bool weno = !LEARNED && recon == HYPE_RECON_WENO3;
                bool linear = LEARNED ? !full : recon == HYPE_RECON_LINEAR4;
                bool ok = true;
                // one copy of the reconstruction in the code: with the gate, R4 traces that break
                // the floors are redone with CWENO4 on a second pass
#pragma unroll 1
                for (int pass = 0; pass < 2; ++pass) {
                    fs_recon_cell(S, G, g, ge, t, linear, weno);
                    ok = (LEARNED || pad) ? fs_admissible(S, t, gm1) : true;
                    if (!LEARNED || ok || !linear) break;
                    linear = false;
                }
                // positivity fallback: first order when the traces still break the floors
                if (!ok && pad) {
#pragma unroll 1
                    for (int c = 0; c < NV; ++c) {
                        const float v = __ldg(G + (long long)c * g.GN + ge);
                        for (int q = 0; q < NTR; ++q) S[(c * NTR + q) * FS_NT + t] = v;
                    }
                    if (owned && !edge) ++nfall;
                }
            }
            __syncthreads();
            // ---- Rusanov fluxes of the owned cells' faces: -x (the ring lane at the high side gives
            // the last cell's +x; the +x flux of every cell comes from its right neighbour lane by a
            // shuffle), -y and +y (each y face is solved by both of its cells: no exchange between
            // warps), -z (low side from registers)
            const bool plane = (k >= kb) && (k < ke);
            // z face first: it completes the previous plane (its stage value), then frees zp
            if (k >= kb && owned) {
                float Fz[NV];
                bool b = false;
                fs_face(S, t, t, 0, 16, zp, gm, gm1, Fz, smax, b, 2);  // L: registers (zl), R: own -z (q 16..19)
                if (b) fs_bad(ds, g, i, j, k);
                if (k > kb) {
                    const long long cell = ((long long)(k - 1) * g.ny + j) * g.nx + i;
#pragma unroll
                    for (int c = 0; c < NV; ++c) {
                        const double L = df_f2d(div_z_f(Pp[c], Fz[c] - Fzp[c], r1h));
                        const double u = (!st.rhs_only && st.a != 0.0) ? U[c * g.N + cell] : 0.0;
                        const double wv = st.rhs_only ? 0.0 : W[c * g.N + cell];
                        out[c * g.N + cell] = stage_value(st, cdt, u, wv, L);
                    }
                }
#pragma unroll
                for (int c = 0; c < NV; ++c) Fzp[c] = Fz[c];
            }
            if (owned && k < ke) {
#pragma unroll
                for (int c = 0; c < NV; ++c)
#pragma unroll
                    for (int q = 0; q < 4; ++q) zp[c][q] = S[(c * NTR + 20 + q) * FS_NT + t];
            }
            // x faces: every lane its -x face (the ring lane at the high side gives the last cell's +x),
            // the +x flux from the right neighbour lane
            float dF[NV];
            {
                float Fxl[NV];
#pragma unroll
                for (int c = 0; c < NV; ++c) Fxl[c] = 0.0f;
                if (plane && own_y && (own_x || i == ihi)) {
                    bool b = false;
                    fs_face(S, t - 1, t, 4, 0, nullptr, gm, gm1, Fxl, smax, b, 0);
                    if (b) fs_bad(ds, g, i, j, k);
                }
#pragma unroll
                for (int c = 0; c < NV; ++c) dF[c] = __shfl_down_sync(0xffffffffu, Fxl[c], 1) - Fxl[c];
            }
            // y faces: each owned cell and the ring row at the high side its -y face, shared through
            // the flux array (the row above gives each owned cell its +y face)
            float Fyl[NV];
            if (plane && own_x && (own_y || j == jhi)) {
                bool b = false;
                fs_face(S, t - 32, t, 12, 8, nullptr, gm, gm1, Fyl, smax, b, 1);
                if (b) fs_bad(ds, g, i, j, k);
#pragma unroll
                for (int c = 0; c < NV; ++c) SFy[c * FS_NT + t] = Fyl[c];
            }
            __syncthreads();  // every trace read (the next plane may overwrite them), -y fluxes written
            if (plane && owned) {
#pragma unroll
                for (int c = 0; c < NV; ++c) Pp[c] = div_xy_f(dF[c], SFy[c * FS_NT + t + 32] - Fyl[c], r1h);
            }
            // the flux array is next written after the next plane's first barrier, when every
            // thread has read it
        }
    }
    if (nfall) atomicAdd(&counters[1], (unsigned long long)nfall);
    if (LEARNED && nflag) atomicAdd(&counters[0], (unsigned long long)nflag);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax = fmaxf(smax, __shfl_xor_sync(0xffffffffu, smax, o));
    if (lane == 0 && smax > 0.0f) atomic_max_pos(&ds->smax_bits[slot], (double)smax);
}

// the stage combination alone, from an RHS already in L (the first stage of a step whose dt
// comes from that stage's own RHS): the same explicitly rounded value as the fused kernel's
__global__ void __launch_bounds__(256) k_stage_combine(const double* U, const double* W, const double* __restrict__ L,
                                                       double* out, long long n, Stage st,
                                                       const DevScalars* __restrict__ ds) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt;
    const double u = (!st.rhs_only && st.a != 0.0) ? U[q] : 0.0;
    const double w = st.rhs_only ? 0.0 : W[q];
    out[q] = stage_value(st, cdt, u, w, L[q]);
}

// dt from the largest wave speed, rounded as each reference program does:
// (1/3) (CFL h) / s_max (3d/weno4/Navier-Stokes-3D/rhs_function.c:438-440) or
// (CFL h) / (3 s_max) (3d/weno3/Euler/rhs_function.c:383)
// and, with viscosity, (1/3) (CFL h) / (s_max + 2 s_visc / h) (Navier-Stokes-3D/rhs_function.c:438)
__host__ __device__ inline double cfl_dt(double cfl_h, double smax, int recon, double smaxv = 0.0, double r1_h = 0.0,
                                         bool visc = false) {
    if (visc) return (1.0 / 3.0) * cfl_h / (smax + (r1_h * smaxv) * 2.0);
    return recon == HYPE_RECON_WENO3 ? cfl_h / (3.0 * smax) : (1.0 / 3.0) * cfl_h / (smax + 0.0);
}

// dt of the coming step and the time update (one thread)
__global__ void k_begin_step(DevScalars* ds, int dt_mode, int src_slot, int use_src, int reset_stages, double cfl_h,
                             int recon, double r1_h, int visc) {
    if (use_src && dt_mode != HYPE_DT_FIXED) {
        const double smax = __longlong_as_double((long long)ds->smax_bits[src_slot]);
        const double smaxv = __longlong_as_double((long long)ds->smaxv_bits[src_slot]);
        ds->dt = cfl_dt(cfl_h, smax, recon, smaxv, r1_h, visc != 0);
    }
    if (reset_stages)
        for (int s = 0; s < 4; ++s) ds->smax_bits[s] = ds->smaxv_bits[s] = 0ull;
    ds->t += ds->dt;
}

// sum |a - b| and sum |b| over n values (two doubles accumulated with atomics)
__global__ void k_l1(const double* __restrict__ a, const double* __restrict__ b, long long n, double* __restrict__ acc) {
    double d = 0.0, r = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        d += fabs(a[q] - b[q]);
        r += fabs(b[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        d += __shfl_xor_sync(0xffffffffu, d, o);
        r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], d);
        atomicAdd(&acc[1], r);
    }
}

__global__ void k_reset_slot(DevScalars* ds, int slot) {
    ds->smax_bits[slot] = 0ull;
    ds->smaxv_bits[slot] = 0ull;
    ds->bad = ~0ull;
}

// AoS [cell][c] <-> SoA [c][cell]
__global__ void k_aos_to_soa(const double* __restrict__ a, double* __restrict__ s, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * NV) return;
    const long long cell = q / NV;
    const int c = (int)(q - cell * NV);
    s[c * N + cell] = a[q];
}
__global__ void k_soa_to_aos(const double* __restrict__ s, double* __restrict__ a, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * NV) return;
    const long long cell = q / NV;
    const int c = (int)(q - cell * NV);
    a[q] = s[c * N + cell];
}

// ---------------------------------------------------------------- monitor diagnostics
// KineticEnergy (3d/weno4/Navier-Stokes-3D/kinetic_energy.c:11-44): sum of
// h^3 (|rho u|^2 / 2 rho); Dissipation (dissipation.c:11-67): sum over cells of
// tau : grad v with central velocity differences and the Stokes stress of viscosity
// mu.  Neighbours across a non-periodic face are the context's ghost values of the
// state.  Deterministic: one partial pair per block, then one block sums the
// partials in a fixed order.
constexpr int kMonThreads = 256;

__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[2 * w] = a;
        sh[2 * w + 1] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = l < (int)(blockDim.x >> 5) ? sh[2 * l] : 0.0;
        b = l < (int)(blockDim.x >> 5) ? sh[2 * l + 1] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
    }
}

__device__ __forceinline__ void vel_at(const double* __restrict__ U, const Geo& g, int i, int j, int k, double* v) {
    int fi = 0, fj = 0, fk = 0;
    const int mi = bmap(i, g.nx, g.bc[0], g.bc[1], &fi);
    const int mj = bmap(j, g.ny, g.bc[2], g.bc[3], &fj);
    const int mk = bmap(k, g.nz, g.bc[4], g.bc[5], &fk);
    const long long q = ((long long)mk * g.ny + mj) * g.nx + mi;
    const double rho = __ldg(U + q);
    v[0] = (fi ? -1.0 : 1.0) * __ldg(U + g.N + q) / rho;
    v[1] = (fj ? -1.0 : 1.0) * __ldg(U + 2 * g.N + q) / rho;
    v[2] = (fk ? -1.0 : 1.0) * __ldg(U + 3 * g.N + q) / rho;
}

__global__ void __launch_bounds__(kMonThreads) k_monitor(const double* __restrict__ U, Geo g, double vol, double r1_2h,
                                                         double mu, double* __restrict__ part) {
    __shared__ double sh[2 * (kMonThreads / 32)];
    double ke = 0.0, dr = 0.0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < g.N; q += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(q % g.nx), j = (int)((q / g.nx) % g.ny), k = (int)(q / ((long long)g.nx * g.ny));
        const double rho = __ldg(U + q), mx = __ldg(U + g.N + q), my = __ldg(U + 2 * g.N + q), mz = __ldg(U + 3 * g.N + q);
        ke += vol * 0.5 * (mx * mx + my * my + mz * mz) / rho;
        double a[3], b[3], vg[3][3];  // vg[a][b]: d(velocity a)/d(x_b)
        vel_at(U, g, i + 1, j, k, a);
        vel_at(U, g, i - 1, j, k, b);
#pragma unroll
        for (int c = 0; c < 3; ++c) vg[c][0] = r1_2h * (a[c] - b[c]);
        vel_at(U, g, i, j + 1, k, a);
        vel_at(U, g, i, j - 1, k, b);
#pragma unroll
        for (int c = 0; c < 3; ++c) vg[c][1] = r1_2h * (a[c] - b[c]);
        vel_at(U, g, i, j, k + 1, a);
        vel_at(U, g, i, j, k - 1, b);
#pragma unroll
        for (int c = 0; c < 3; ++c) vg[c][2] = r1_2h * (a[c] - b[c]);
        const double div_v = -(2.0 / 3.0) * mu * (vg[0][0] + vg[1][1] + vg[2][2]);
        const double txx = div_v + 2.0 * mu * vg[0][0], txy = mu * (vg[0][1] + vg[1][0]), txz = mu * (vg[0][2] + vg[2][0]);
        const double tyy = div_v + 2.0 * mu * vg[1][1], tyz = mu * (vg[1][2] + vg[2][1]), tzz = div_v + 2.0 * mu * vg[2][2];
        dr += (txx * vg[0][0] + txy * vg[0][1] + txz * vg[0][2]) + (txy * vg[1][0] + tyy * vg[1][1] + tyz * vg[1][2]) +
              (txz * vg[2][0] + tyz * vg[2][1] + tzz * vg[2][2]);
    }
    block_sum2(ke, dr, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = ke;
        part[2 * blockIdx.x + 1] = dr;
    }
}

__global__ void __launch_bounds__(kMonThreads) k_monitor_sum(const double* __restrict__ part, int nblk, double* out) {
    __shared__ double sh[2 * (kMonThreads / 32)];
    double ke = 0.0, dr = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        ke += part[2 * b];
        dr += part[2 * b + 1];
    }
    block_sum2(ke, dr, sh);
    if (threadIdx.x == 0) {
        out[0] = ke;
        out[1] = dr;
    }
}

}  // namespace euler
}  // namespace hype

using namespace hype;
using namespace hype::euler;

static inline double bits_to_double(unsigned long long b) {
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

struct hype_euler {
    hype_euler_params p;
    Geo g;
    cudaStream_t stream = nullptr;
    double* U = nullptr;   // resident state (SoA)
    double* W = nullptr;   // stage state
    double* L = nullptr;   // RHS buffer (rhs-only calls)
    double* S = nullptr;   // scratch SoA state for host RHS calls
    void* T = nullptr;     // traces
    double* Fx = nullptr;
    double* Fy = nullptr;
    double* Fz = nullptr;
    double* stage_aos = nullptr;  // device AoS staging
    void* G = nullptr;            // ghosted stage input in the reconstruction's precision
    double* C4 = nullptr;         // viscous runs: R4 coefficients [5][20][ext cells] for the face gradients
    double* mon = nullptr;        // monitor partial sums (2 per block) and the result pair
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;  // pinned host copy
    double* pin = nullptr;     // pinned host staging for AoS transfers
    // learned indicator: BF16 parameters, logit threshold, counters (flagged, positivity fallbacks)
    mlp::MmaWeights* mlp = nullptr;  // packed for the tensor-core inference
    // fused FP32 stage: the gate's flags (one byte per extended cell) and, when the gate is scored
    // once per step, their one-cell widening that the step's stages read
    unsigned char* gate = nullptr;
    unsigned char* gate_wide = nullptr;
    int gate_per_step = 0;
    float logit_thr = 0.0f;
    unsigned long long* mlp_cnt = nullptr;
    // per-kernel event timing inside a timed region (hype_euler_profile)
    bool prof = false;
    // the steady-state step (every step after the first of a call) captured as a CUDA graph,
    // with the launch choices it was captured under and the kernels it launches
    cudaGraphExec_t step_graph = nullptr;
    long long graph_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    long long graph_launches = 0;
    // stage kernels: HYPE_STAGE_AUTO takes the fused FP32 stage where it applies; the unfused
    // kernels' trace and face-flux buffers are allocated when first needed
    int stage_mode = HYPE_STAGE_AUTO;
    int nsm = 1;
    double* acc = nullptr;  // two doubles: k_l1's sums
    std::vector<cudaEvent_t> ev;  // pairs (start, end)
    std::vector<int> ev_kind;     // 0 recon, 1 faces (3 directions), 2 update
    size_t ev_used = 0;
};

static void prof_mark(hype_euler* e, int kind, bool start) {
    if (!e->prof) return;
    if (start) {
        if (e->ev_used + 2 > e->ev.size()) {
            for (int q = 0; q < 64; ++q) {
                cudaEvent_t x;
                cudaEventCreate(&x);
                e->ev.push_back(x);
            }
            e->ev_kind.resize(e->ev.size() / 2);
        }
        e->ev_kind[e->ev_used / 2] = kind;
        cudaEventRecord(e->ev[e->ev_used], e->stream);
    } else {
        cudaEventRecord(e->ev[e->ev_used + 1], e->stream);
        e->ev_used += 2;
    }
}

template <typename R, int FLUX, bool VISC = false>
static void launch_faces_t(const Geo& g, const void* T, double* Fx, double* Fy, double* Fz, double gamma, DevScalars* ds,
                           int slot, cudaStream_t st, const double* C4 = nullptr, Visc vp = Visc{0.0, 0.0, 0.0, 0.0}) {
    const dim3 bf(32, 4);
    const dim3 gx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), gy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz),
        gz(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1);
    k_faces<R, 0, FLUX, VISC><<<gx, bf, 0, st>>>((const R*)T, Fx, g, gamma, ds, slot, C4, vp);
    k_faces<R, 1, FLUX, VISC><<<gy, bf, 0, st>>>((const R*)T, Fy, g, gamma, ds, slot, C4, vp);
    k_faces<R, 2, FLUX, VISC><<<gz, bf, 0, st>>>((const R*)T, Fz, g, gamma, ds, slot, C4, vp);
}

// the three face-flux launches of one RHS, for the context's precision and flux
static void launch_faces(const Geo& g, const void* T, double* Fx, double* Fy, double* Fz, double gamma, DevScalars* ds,
                         int slot, bool f32, int flux, cudaStream_t st) {
    if (f32) {
        if (flux == HYPE_FLUX_HLLC) launch_faces_t<float, HYPE_FLUX_HLLC>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
        else if (flux == HYPE_FLUX_ROTHLLC) launch_faces_t<float, HYPE_FLUX_ROTHLLC>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
        else launch_faces_t<float, HYPE_FLUX_RUSANOV>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
    } else {
        if (flux == HYPE_FLUX_HLLC) launch_faces_t<double, HYPE_FLUX_HLLC>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
        else if (flux == HYPE_FLUX_ROTHLLC) launch_faces_t<double, HYPE_FLUX_ROTHLLC>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
        else launch_faces_t<double, HYPE_FLUX_RUSANOV>(g, T, Fx, Fy, Fz, gamma, ds, slot, st);
    }
}

static int launch_rhs(hype_euler* e, const double* Win, int slot) {
    const Geo& g = e->g;
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2);
    const bool f32 = e->p.precision == HYPE_PREC_FP32;
    const bool df = e->p.precision == HYPE_PREC_DF64;
    const int rec = e->p.recon;
    prof_mark(e, 0, true);
    const dim3 bgh(128), ggh(cdiv(g.gx, 128), g.gy, g.nz + 2 * GW);
    if (f32) k_ghost<float><<<ghost_grid(g), kGhostThreads, 0, e->stream>>>(Win, (float*)e->G, g);
    else if (df) k_ghost_df<<<ggh, bgh, 0, e->stream>>>(Win, (df64*)e->G, g);
    else k_ghost<double><<<ghost_grid(g), kGhostThreads, 0, e->stream>>>(Win, (double*)e->G, g);
    HYPE_LAUNCHED(1);
    const double gm1 = e->p.gamma - 1.0;
    const size_t ck_bytes = (f32 && e->p.positivity) ? sizeof(float) * 4 * 2 * NTR * 32 : 0;
    if (e->p.recon == HYPE_RECON_LEARNED) {
        if (!e->mlp) return HYPE_ERR_ARG;  // hype_euler_set_mlp first
        if (df && e->p.flux == HYPE_FLUX_RUSANOV)
            k_recon_learned_df<true><<<gr, br, 0, e->stream>>>((const df64*)e->G, e->T, Win, g, e->mlp, e->logit_thr, gm1,
                                                               e->p.positivity, e->mlp_cnt);
        else if (df)
            k_recon_learned_df<false><<<gr, br, 0, e->stream>>>((const df64*)e->G, e->T, Win, g, e->mlp, e->logit_thr,
                                                                gm1, e->p.positivity, e->mlp_cnt);
        else if (f32)
            k_recon_learned<float><<<gr, br, 0, e->stream>>>((const float*)e->G, (float*)e->T, g, e->mlp, e->logit_thr, gm1,
                                                             e->p.positivity, e->mlp_cnt);
        else
            k_recon_learned<double><<<gr, br, 0, e->stream>>>((const double*)e->G, (double*)e->T, g, e->mlp, e->logit_thr,
                                                              gm1, e->p.positivity, e->mlp_cnt);
    } else if (df) {
        if (e->p.flux == HYPE_FLUX_RUSANOV)
            k_recon_df<true><<<gr, br, 0, e->stream>>>((const df64*)e->G, e->T, Win, g, rec, e->p.positivity, gm1,
                                                       e->mlp_cnt, (df64*)e->C4, 1.0 / e->p.h);
        else
            k_recon_df<false><<<gr, br, 0, e->stream>>>((const df64*)e->G, e->T, Win, g, rec, e->p.positivity, gm1,
                                                        e->mlp_cnt);
    } else if (f32) {
        k_recon<float><<<gr, br, ck_bytes, e->stream>>>((const float*)e->G, (float*)e->T, g, rec, e->p.positivity, gm1,
                                                        e->mlp_cnt);
    } else {
        k_recon<double><<<gr, br, 0, e->stream>>>((const double*)e->G, (double*)e->T, g, rec, e->p.positivity, gm1,
                                                  e->mlp_cnt, e->C4, 1.0 / e->p.h);
    }
    prof_mark(e, 0, false);
    prof_mark(e, 1, true);
    if (e->C4 && df) {
        // Navier-Stokes in double-float: Rusanov in deviation form plus both sides' viscous fluxes
        const double mu = e->p.mu, gm = e->p.gamma;
        const Visc vp{mu, e->p.cv * mu * gm / e->p.prandtl, std::max((4. / 3.) * mu, gm * mu / e->p.prandtl),
                      1.0 / e->p.h};
        const dim3 bf(32, 4);
        const dim3 fgx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), fgy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz),
            fgz(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1);
        const df64* Td = (const df64*)e->T;
        const df64* C4 = (const df64*)e->C4;
        k_faces_df<0, true><<<fgx, bf, 0, e->stream>>>(Td, e->Fx, Win, g, e->p.gamma, e->ds, slot, C4, vp);
        k_faces_df<1, true><<<fgy, bf, 0, e->stream>>>(Td, e->Fy, Win, g, e->p.gamma, e->ds, slot, C4, vp);
        k_faces_df<2, true><<<fgz, bf, 0, e->stream>>>(Td, e->Fz, Win, g, e->p.gamma, e->ds, slot, C4, vp);
    } else if (e->C4) {
        // Navier-Stokes: the inviscid flux plus the average of both sides' viscous fluxes
        const double mu = e->p.mu, g = e->p.gamma;
        const Visc vp{mu, e->p.cv * mu * g / e->p.prandtl, std::max((4. / 3.) * mu, g * mu / e->p.prandtl), 1.0 / e->p.h};
        const auto lf = e->p.flux == HYPE_FLUX_HLLC      ? launch_faces_t<double, HYPE_FLUX_HLLC, true>
                        : e->p.flux == HYPE_FLUX_ROTHLLC ? launch_faces_t<double, HYPE_FLUX_ROTHLLC, true>
                                                         : launch_faces_t<double, HYPE_FLUX_RUSANOV, true>;
        lf(e->g, e->T, e->Fx, e->Fy, e->Fz, e->p.gamma, e->ds, slot, e->stream, e->C4, vp);
    } else if (df && e->p.flux == HYPE_FLUX_RUSANOV) {
        const dim3 bf(32, 4);
        const dim3 fgx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4), g.nz), fgy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4), g.nz),
            fgz(cdiv(g.nx, 32), cdiv(g.ny, 4), g.nz + 1);
        const df64* Td = (const df64*)e->T;
        k_faces_df<0><<<fgx, bf, 0, e->stream>>>(Td, e->Fx, Win, g, e->p.gamma, e->ds, slot);
        k_faces_df<1><<<fgy, bf, 0, e->stream>>>(Td, e->Fy, Win, g, e->p.gamma, e->ds, slot);
        k_faces_df<2><<<fgz, bf, 0, e->stream>>>(Td, e->Fz, Win, g, e->p.gamma, e->ds, slot);
    } else {
        launch_faces(e->g, e->T, e->Fx, e->Fy, e->Fz, e->p.gamma, e->ds, slot, f32, e->p.flux, e->stream);
    }
    prof_mark(e, 1, false);
    HYPE_LAUNCHED(4);
    return HYPE_OK;
}

static int launch_update(hype_euler* e, const double* U, const double* W, double* out, Stage st) {
    const Geo& g = e->g;
    const dim3 b(32, 8), gr(cdiv(g.nx, 32), cdiv(g.ny, 8), g.nz);
    prof_mark(e, 2, true);
    if (e->p.precision == HYPE_PREC_FP32)
        k_update<true><<<gr, b, 0, e->stream>>>(e->Fx, e->Fy, e->Fz, U, W, out, g, 1.0 / e->p.h, st, e->ds);
    else
        k_update<false><<<gr, b, 0, e->stream>>>(e->Fx, e->Fy, e->Fz, U, W, out, g, 1.0 / e->p.h, st, e->ds);
    prof_mark(e, 2, false);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

// whether the context's current options run the fused FP32 stage kernel
static bool uses_fused(const hype_euler* e) {
    return e->stage_mode == HYPE_STAGE_AUTO && e->p.precision == HYPE_PREC_FP32 && e->p.flux == HYPE_FLUX_RUSANOV &&
           !e->C4 && (e->p.recon == HYPE_RECON_CWENO4 || e->p.recon == HYPE_RECON_LINEAR4 ||
                      e->p.recon == HYPE_RECON_WENO3 || (e->p.recon == HYPE_RECON_LEARNED && e->mlp && e->gate));
}

// the unfused kernels' face traces and face fluxes, allocated on first use (never inside a
// stream capture: every entry point that may launch them calls this first)
static int ensure_unfused(hype_euler* e) {
    if (e->T) return HYPE_OK;
    const Geo& g = e->g;
    const hype_euler_params* p = &e->p;
    const size_t tsz = (p->precision == HYPE_PREC_FP32 ? sizeof(float) : sizeof(double)) * NV * NTR * (size_t)g.NE;
    cudaError_t ce = cudaMalloc(&e->T, tsz);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&e->Fx, sizeof(double) * NV * (size_t)(p->nx + 1) * p->ny * p->nz);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&e->Fy, sizeof(double) * NV * (size_t)p->nx * (p->ny + 1) * p->nz);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&e->Fz, sizeof(double) * NV * (size_t)p->nx * p->ny * (p->nz + 1));
    if (ce != cudaSuccess) {
        cudaFree(e->T); cudaFree(e->Fx); cudaFree(e->Fy); cudaFree(e->Fz);
        e->T = nullptr; e->Fx = e->Fy = e->Fz = nullptr;
        set_last_error("cudaMalloc (face traces)", ce);
        return HYPE_ERR_NOMEM;
    }
    return HYPE_OK;
}

static int prepare(hype_euler* e) { return uses_fused(e) ? HYPE_OK : ensure_unfused(e); }

// One RK stage: out = a U + b W + (c dt) L(Win) (or out = L(Win) for RHS-only calls), with the
// wave-speed maximum into slot.  The fused FP32 stage is the device ghost fill plus one kernel;
// every other form is ghost fill, reconstruction, three face-flux kernels and the update.
static int launch_stage(hype_euler* e, const double* Win, const double* U, const double* W, double* out, Stage st,
                        int slot) {
    if (!uses_fused(e)) {
        int rc = launch_rhs(e, Win, slot);
        if (rc) return rc;
        return launch_update(e, U, W, out, st);
    }
    const Geo& g = e->g;
    prof_mark(e, 0, true);
    k_ghost<float><<<ghost_grid(g), kGhostThreads, 0, e->stream>>>(Win, (float*)e->G, g);
    const bool learned = e->p.recon == HYPE_RECON_LEARNED;
    // the gate's flags for this stage's input; scored once per step, on the first stage's input
    // (slot 0) and for RHS-only calls (slot 4), then widened by a cell for the step's later stages
    const bool score = learned && (!e->gate_per_step || slot == 0 || slot == 4);
    if (score) {
        const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2);
        k_gate_f32<<<gr, br, 0, e->stream>>>((const float*)e->G, e->gate, g, e->mlp, e->logit_thr);
        if (e->gate_per_step)
            k_gate_dilate<<<dim3(cdiv(g.ex, 128), g.ny + 2, g.nz + 2), 128, 0, e->stream>>>(e->gate, e->gate_wide, g);
    }
    prof_mark(e, 0, false);
    prof_mark(e, 1, true);
    const long long units = fs_tiles_x(g.nx) * fs_tiles_y(g.ny) * g.nz;
    const unsigned blocks = (unsigned)std::min<long long>(e->nsm, units);
    if (learned)
        k_stage_f32<true><<<blocks, FS_NT, FS_SMEM, e->stream>>>((const float*)e->G, U, W, out, g, e->p.recon,
                                                                e->p.positivity, e->p.gamma, 1.0 / e->p.h, st, e->ds,
                                                                slot, e->mlp_cnt,
                                                                e->gate_per_step ? e->gate_wide : e->gate);
    else
        k_stage_f32<false><<<blocks, FS_NT, FS_SMEM, e->stream>>>((const float*)e->G, U, W, out, g, e->p.recon,
                                                                 e->p.positivity, e->p.gamma, 1.0 / e->p.h, st, e->ds,
                                                                 slot, e->mlp_cnt);
    prof_mark(e, 1, false);
    HYPE_LAUNCHED(2 + (score ? 1 + (e->gate_per_step ? 1 : 0) : 0));
    return HYPE_OK;
}

// the first stage of a step whose dt comes from that stage's own RHS: RHS into L, dt, then the
// stage combination (fused form) or the update kernel (unfused)
static int launch_first_stage_from_rhs(hype_euler* e, int mode, double cfl_h, Stage s12) {
    int rc;
    if (uses_fused(e)) {
        const Stage rhs{0.0, 0.0, 0.0, 1};
        if ((rc = launch_stage(e, e->U, nullptr, nullptr, e->L, rhs, 0))) return rc;
    } else if ((rc = launch_rhs(e, e->U, 0))) {
        return rc;
    }
    k_begin_step<<<1, 1, 0, e->stream>>>(e->ds, mode, 0, 1, 0, cfl_h, e->p.recon, 1.0 / e->p.h, e->C4 != nullptr);
    HYPE_LAUNCHED(1);
    if (!uses_fused(e)) return launch_update(e, e->U, e->U, e->W, s12);
    const long long n = NV * e->g.N;
    prof_mark(e, 2, true);
    k_stage_combine<<<cdiv(n, 256), 256, 0, e->stream>>>(e->U, e->U, e->L, e->W, n, s12, e->ds);
    prof_mark(e, 2, false);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

extern "C" int hype_euler_create(const hype_euler_params* p, hype_euler** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3 || !(p->h > 0) || !(p->cfl > 0) || !(p->gamma > 1.0)) return HYPE_ERR_ARG;
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] < HYPE_BC_PERIODIC || p->bc[f] > HYPE_BC_TRANSMISSIVE) return HYPE_ERR_ARG;
    for (int d = 0; d < 3; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (p->recon < HYPE_RECON_CWENO4 || p->recon > HYPE_RECON_WENO3) return HYPE_ERR_ARG;
    if (p->precision != HYPE_PREC_FP64 && p->precision != HYPE_PREC_FP32 && p->precision != HYPE_PREC_DF64)
        return HYPE_ERR_ARG;
    // the double-float form covers CWENO4, R4 and the indicator gate between them (no WENO3, no
    // viscous fluxes)
    if (p->precision == HYPE_PREC_DF64 && p->recon == HYPE_RECON_WENO3) return HYPE_ERR_UNSUPPORTED;
    if (p->dt_mode < HYPE_DT_MONITOR || p->dt_mode > HYPE_DT_FIXED) return HYPE_ERR_ARG;
    if (p->flux < HYPE_FLUX_RUSANOV || p->flux > HYPE_FLUX_ROTHLLC) return HYPE_ERR_ARG;
    if (p->positivity != 0 && p->positivity != 1) return HYPE_ERR_ARG;
    // viscosity: FP64 (with the CWENO4 / R4 / WENO3 traces) or the double-float form with the Rusanov
    // flux; the gradients always come from R4
    const bool visc = p->mu != 0.0;
    if (visc && (!(p->mu > 0.0) || !(p->prandtl > 0.0) || !(p->cv > 0.0) || p->precision == HYPE_PREC_FP32 ||
                 p->recon == HYPE_RECON_LEARNED))
        return HYPE_ERR_ARG;
    if (visc && p->precision == HYPE_PREC_DF64 && p->flux != HYPE_FLUX_RUSANOV) return HYPE_ERR_UNSUPPORTED;
    hype_euler* e = new hype_euler();
    e->p = *p;
    Geo& g = e->g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    for (int f = 0; f < 6; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny * p->nz;
    g.NE = (long long)(p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    g.ex = p->nx + 2;
    g.ey = p->ny + 2;
    set_ghost_extents(g);
    const size_t sN = sizeof(double) * NV * (size_t)g.N;
    int rc = HYPE_OK;
    auto fail = [&](int code) {
        hype_euler_destroy(e);
        return code;
    };
    cudaError_t ce;
#define ALLOC(ptr, bytes)                                  \
    ce = cudaMalloc((void**)&(ptr), (bytes));              \
    if (ce != cudaSuccess) {                               \
        set_last_error("cudaMalloc", ce);                  \
        return fail(HYPE_ERR_NOMEM);                       \
    }
    ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        set_last_error("cudaStreamCreate", ce);
        return fail(HYPE_ERR_CUDA);
    }
    ALLOC(e->U, sN);
    ALLOC(e->W, sN);
    ALLOC(e->L, sN);
    ALLOC(e->S, sN);
    ALLOC(e->stage_aos, sN);
    ALLOC(e->acc, 2 * sizeof(double));
    ALLOC(e->ds, sizeof(DevScalars));
    ALLOC(e->mlp_cnt, 2 * sizeof(unsigned long long));
    ALLOC(e->G, (p->precision == HYPE_PREC_FP32 ? sizeof(float) : sizeof(double)) * NV * (size_t)g.GN);
    if (visc) ALLOC(e->C4, sizeof(double) * NV * 20 * (size_t)g.NE);
#undef ALLOC
    {
        int dev = 0;
        ce = cudaGetDevice(&dev);
        if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, dev);
        if (ce == cudaSuccess)
            ce = cudaFuncSetAttribute(k_stage_f32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FS_SMEM);
        if (ce == cudaSuccess)
            ce = cudaFuncSetAttribute(k_stage_f32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FS_SMEM);
        if (ce != cudaSuccess) {
            set_last_error("hype_euler_create (device attributes)", ce);
            return fail(HYPE_ERR_CUDA);
        }
        // the FP32 Rusanov form runs fused (the learned gate too, once its network is set): no trace
        // buffers up front; every other form allocates them now
        const bool fusable = p->precision == HYPE_PREC_FP32 && p->flux == HYPE_FLUX_RUSANOV && !visc;
        if (!fusable && (rc = prepare(e))) return fail(rc);
    }
    ce = cudaMemset(e->mlp_cnt, 0, 2 * sizeof(unsigned long long));
    if (ce != cudaSuccess) {
        set_last_error("cudaMemset", ce);
        return fail(HYPE_ERR_CUDA);
    }
    ce = cudaMallocHost((void**)&e->hs, sizeof(DevScalars));
    if (ce != cudaSuccess) {
        set_last_error("cudaMallocHost", ce);
        return fail(HYPE_ERR_NOMEM);
    }
    DevScalars z;
    memset(&z, 0, sizeof(z));
    z.bad = ~0ull;
    ce = cudaMemcpy(e->ds, &z, sizeof(z), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        set_last_error("cudaMemcpy", ce);
        return fail(HYPE_ERR_CUDA);
    }
    *out = e;
    return rc;
}

extern "C" void hype_euler_destroy(hype_euler* e) {
    if (!e) return;
    if (e->stream) cudaStreamSynchronize(e->stream);
    cudaFree(e->U); cudaFree(e->W); cudaFree(e->L); cudaFree(e->S); cudaFree(e->T);
    cudaFree(e->Fx); cudaFree(e->Fy); cudaFree(e->Fz); cudaFree(e->stage_aos); cudaFree(e->ds); cudaFree(e->G);
    cudaFree(e->mlp); cudaFree(e->gate); cudaFree(e->gate_wide); cudaFree(e->mlp_cnt); cudaFree(e->C4); cudaFree(e->mon); cudaFree(e->acc);
    if (e->hs) cudaFreeHost(e->hs);
    for (auto x : e->ev) cudaEventDestroy(x);
    if (e->step_graph) cudaGraphExecDestroy(e->step_graph);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

static int h2d_aos(hype_euler* e, const double* aos, double* soa) {
    const long long n = e->g.N * NV;
    HYPE_CK(cudaMemcpyAsync(e->stage_aos, aos, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
    k_aos_to_soa<<<cdiv(n, 256), 256, 0, e->stream>>>(e->stage_aos, soa, e->g.N);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int d2h_aos(hype_euler* e, const double* soa, double* aos) {
    const long long n = e->g.N * NV;
    k_soa_to_aos<<<cdiv(n, 256), 256, 0, e->stream>>>(soa, e->stage_aos, e->g.N);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, e->stage_aos, sizeof(double) * n, cudaMemcpyDeviceToHost, e->stream));
    return HYPE_OK;
}

static int read_scalars(hype_euler* e) {
    HYPE_CK(cudaMemcpyAsync(e->hs, e->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return HYPE_OK;
}

static int rhs_core(hype_euler* e, const double* dU, double* dRHS, double* dt_out) {
    int rc;
    if ((rc = prepare(e))) return rc;
    k_reset_slot<<<1, 1, 0, e->stream>>>(e->ds, 4);
    HYPE_LAUNCHED(1);
    Stage st{0.0, 0.0, 0.0, 1};
    if ((rc = launch_stage(e, dU, nullptr, nullptr, dRHS, st, 4))) return rc;
    if ((rc = read_scalars(e))) return rc;
    const double smax = bits_to_double(e->hs->smax_bits[4]);
    const double smaxv = bits_to_double(e->hs->smaxv_bits[4]);
    if (dt_out) *dt_out = cfl_dt(e->p.cfl * e->p.h, smax, e->p.recon, smaxv, 1.0 / e->p.h, e->C4 != nullptr);
    if (e->hs->bad != ~0ull) return HYPE_ERR_STATE;
    return HYPE_OK;
}

extern "C" int hype_euler_rhs(hype_euler* e, double t, const double* U_aos, double* RHS_aos, double* dt_out) {
    (void)t;  // the Euler RHS is autonomous
    if (!e || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc;
    if ((rc = h2d_aos(e, U_aos, e->S))) return rc;
    rc = rhs_core(e, e->S, e->L, dt_out);
    if (rc && rc != HYPE_ERR_STATE) return rc;
    int rc2 = d2h_aos(e, e->L, RHS_aos);
    if (rc2) return rc2;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return rc;
}

extern "C" int hype_euler_rhs_device(hype_euler* e, double t, const double* dU, double* dRHS, double* dt_out) {
    (void)t;
    if (!e || !dU || !dRHS) return HYPE_ERR_ARG;
    return rhs_core(e, dU, dRHS, dt_out);
}

extern "C" int hype_euler_get_params(const hype_euler* e, hype_euler_params* out) {
    if (!e || !out) return HYPE_ERR_ARG;
    *out = e->p;
    return HYPE_OK;
}

extern "C" int hype_euler_upload(hype_euler* e, const double* U_aos) {
    if (!e || !U_aos) return HYPE_ERR_ARG;
    int rc = h2d_aos(e, U_aos, e->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return HYPE_OK;
}

extern "C" int hype_euler_download(hype_euler* e, double* U_aos) {
    if (!e || !U_aos) return HYPE_ERR_ARG;
    int rc = d2h_aos(e, e->U, U_aos);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return HYPE_OK;
}

extern "C" double* hype_euler_state_device(hype_euler* e) { return e ? e->U : nullptr; }

extern "C" int hype_euler_sync(hype_euler* e) {
    if (!e) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return HYPE_OK;
}

// One SSPRK(4,3) step after the first of a call: dt from the previous step (MONITOR) or as
// set, then the four stages (the device scalars carry everything that changes between steps)
static int launch_steady_step(hype_euler* e, int mode, double cfl_h) {
    const Stage s12{0.0, 1.0, 0.5, 0};
    const Stage s3{2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0};
    int rc;
    k_begin_step<<<1, 1, 0, e->stream>>>(e->ds, mode, 3, mode == HYPE_DT_MONITOR, 1, cfl_h, e->p.recon, 1.0 / e->p.h,
                                         e->C4 != nullptr);
    HYPE_LAUNCHED(1);
    if ((rc = launch_stage(e, e->U, e->U, e->U, e->W, s12, 0))) return rc;
    if ((rc = launch_stage(e, e->W, e->U, e->W, e->W, s12, 1))) return rc;
    if ((rc = launch_stage(e, e->W, e->U, e->W, e->W, s3, 2))) return rc;
    return launch_stage(e, e->W, e->U, e->W, e->U, s12, 3);
}

// The steady-state step as a CUDA graph (replayed instead of ~25 launches per step; what
// matters on small grids), recaptured when a launch choice changes; falls back to launching
// (returns false) while profiling or if the capture fails.
static bool steady_step_graph(hype_euler* e, int mode, double cfl_h) {
    if (e->prof) return false;
    long long lt;
    memcpy(&lt, &e->logit_thr, sizeof(float));
    const long long key[8] = {mode, e->p.recon, e->p.flux, e->p.precision,
                              e->p.positivity + 2 * e->stage_mode + 8 * e->gate_per_step,
                              (long long)(size_t)e->mlp, lt, (long long)(cfl_h * 1e15)};
    if (e->step_graph && memcmp(key, e->graph_key, sizeof(key)) == 0) return true;
    if (e->step_graph) {
        cudaGraphExecDestroy(e->step_graph);
        e->step_graph = nullptr;
    }
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const long long l0 = hype_launch_count();
    const int rc = launch_steady_step(e, mode, cfl_h);
    const cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
    const long long nl = hype_launch_count() - l0;
    count_launch(-nl);  // captured, not launched
    if (rc != HYPE_OK || ce != cudaSuccess || !graph) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return false;
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    e->step_graph = exec;
    memcpy(e->graph_key, key, sizeof(key));
    e->graph_launches = nl;
    return true;
}

extern "C" int hype_euler_step(hype_euler* e, int nsteps, double* t_inout, double* dt_inout, hype_status* st) {
    if (!e || nsteps < 0 || !t_inout || !dt_inout) return HYPE_ERR_ARG;
    const int mode = e->p.dt_mode;
    if (mode == HYPE_DT_FIXED && !(*dt_inout > 0)) return HYPE_ERR_ARG;
    const double cfl_h = e->p.cfl * e->p.h;
    int rc;
    if ((rc = prepare(e))) return rc;
    // host-side initial values of t, dt, flags
    DevScalars init;
    memset(&init, 0, sizeof(init));
    init.t = *t_inout;
    init.dt = *dt_inout;
    init.bad = ~0ull;
    HYPE_CK(cudaMemcpyAsync(e->ds, &init, sizeof(init), cudaMemcpyHostToDevice, e->stream));
    const bool first_from_rhs = (mode != HYPE_DT_FIXED) && !(*dt_inout > 0);
    // SSPRK(4,3) (PETSc TSSSP RKS3, 4 stages; Ketcheson 2008):
    //   u1 = u + dt/2 L(u); u2 = u1 + dt/2 L(u1); u3 = 2/3 u + 1/3 u2 + dt/6 L(u2); u4 = u3 + dt/2 L(u3)
    const Stage s12{0.0, 1.0, 0.5, 0};
    const Stage s3{2.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0, 0};
    for (int s = 0; s < nsteps; ++s) {
        if (s == 1 && nsteps > 2 && steady_step_graph(e, mode, cfl_h)) {
            for (; s < nsteps; ++s) {
                HYPE_CK(cudaGraphLaunch(e->step_graph, e->stream));
                count_launch(e->graph_launches);
            }
            break;
        }
        if (s == 0 && first_from_rhs) {
            // the initial RHS call of hype.c:175 is this step's first stage RHS
            if ((rc = launch_first_stage_from_rhs(e, mode, cfl_h, s12))) return rc;
        } else {
            // dt: MONITOR refreshes it from the last stage of the previous step
            const int use_src = (mode == HYPE_DT_MONITOR) && s > 0;
            k_begin_step<<<1, 1, 0, e->stream>>>(e->ds, mode, 3, use_src, 1, cfl_h, e->p.recon, 1.0 / e->p.h,
                                                 e->C4 != nullptr);
            HYPE_LAUNCHED(1);
            if ((rc = launch_stage(e, e->U, e->U, e->U, e->W, s12, 0))) return rc;
        }
        if ((rc = launch_stage(e, e->W, e->U, e->W, e->W, s12, 1))) return rc;
        if ((rc = launch_stage(e, e->W, e->U, e->W, e->W, s3, 2))) return rc;
        if ((rc = launch_stage(e, e->W, e->U, e->W, e->U, s12, 3))) return rc;
    }
    if ((rc = read_scalars(e))) return rc;
    *t_inout = e->hs->t;
    const double smax3 = bits_to_double(e->hs->smax_bits[3]);
    if (nsteps > 0 && mode == HYPE_DT_MONITOR)
        *dt_inout = cfl_dt(cfl_h, smax3, e->p.recon, bits_to_double(e->hs->smaxv_bits[3]), 1.0 / e->p.h,
                           e->C4 != nullptr);
    else
        *dt_inout = e->hs->dt;
    if (st) {
        st->bad_cell = e->hs->bad == ~0ull ? -1 : (long long)e->hs->bad;
        st->smax = smax3;
        st->rhs_evals = 4LL * nsteps;
    }
    return e->hs->bad == ~0ull ? HYPE_OK : HYPE_ERR_STATE;
}

extern "C" void* hype_euler_stream(hype_euler* e) { return e ? (void*)e->stream : nullptr; }

extern "C" int hype_euler_monitor(hype_euler* e, double* ke, double* dissipation) {
    if (!e || !ke || !dissipation) return HYPE_ERR_ARG;
    constexpr int kMaxBlocks = 152 * 8;
    const int nblk = (int)std::min<long long>(kMaxBlocks, (e->g.N + kMonThreads - 1) / kMonThreads);
    if (!e->mon) HYPE_CK(cudaMalloc((void**)&e->mon, sizeof(double) * (2 * kMaxBlocks + 2)));
    const double h = e->p.h;
    k_monitor<<<nblk, kMonThreads, 0, e->stream>>>(e->U, e->g, h * h * h, 0.5 / h, e->p.mu, e->mon);
    k_monitor_sum<<<1, kMonThreads, 0, e->stream>>>(e->mon, nblk, e->mon + 2 * kMaxBlocks);
    HYPE_LAUNCHED(2);
    double r[2];
    HYPE_CK(cudaMemcpyAsync(r, e->mon + 2 * kMaxBlocks, sizeof(r), cudaMemcpyDeviceToHost, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    *ke = r[0];
    *dissipation = r[1];
    return HYPE_OK;
}

extern "C" int hype_euler_set_mlp(hype_euler* e, const float* params, float prob_threshold) {
    if (!e || !params || !(prob_threshold > 0.0f) || !(prob_threshold < 1.0f)) return HYPE_ERR_ARG;
    std::vector<__nv_bfloat16> h(mlp::NPARAM);
    for (int q = 0; q < mlp::NPARAM; ++q) h[q] = __float2bfloat16_rn(params[q]);
    mlp::MmaWeights hw;  // host staging, copied before the stream synchronisation below
    mlp::pack_weights(h.data(), hw);
    if (!e->mlp) HYPE_CK(cudaMalloc((void**)&e->mlp, sizeof(mlp::MmaWeights)));
    if (!e->gate && e->p.precision == HYPE_PREC_FP32) {
        HYPE_CK(cudaMalloc((void**)&e->gate, (size_t)e->g.NE));
        HYPE_CK(cudaMalloc((void**)&e->gate_wide, (size_t)e->g.NE));
        HYPE_CK(cudaMemsetAsync(e->gate, 0, (size_t)e->g.NE, e->stream));
        HYPE_CK(cudaMemsetAsync(e->gate_wide, 0, (size_t)e->g.NE, e->stream));
    }
    HYPE_CK(cudaMemcpyAsync(e->mlp, &hw, sizeof(mlp::MmaWeights), cudaMemcpyHostToDevice, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    e->logit_thr = logf(prob_threshold / (1.0f - prob_threshold));
    return HYPE_OK;
}

extern "C" int hype_euler_set_gate_per_step(hype_euler* e, int per_step) {
    if (!e || (per_step != 0 && per_step != 1)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    e->gate_per_step = per_step;  // part of the step graph's key: the next step recaptures
    return HYPE_OK;
}

extern "C" int hype_euler_gate_flags(hype_euler* e, unsigned char* out, int widened) {
    if (!e || !out || (widened != 0 && widened != 1)) return HYPE_ERR_ARG;
    if (!e->gate) return HYPE_ERR_UNSUPPORTED;
    HYPE_CK(cudaMemcpyAsync(out, widened ? e->gate_wide : e->gate, (size_t)e->g.NE, cudaMemcpyDeviceToHost, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    return HYPE_OK;
}

extern "C" int hype_euler_indicator_stats(hype_euler* e, long long* flagged, long long* positivity_fallbacks, int reset) {
    if (!e) return HYPE_ERR_ARG;
    unsigned long long c[2];
    HYPE_CK(cudaMemcpyAsync(c, e->mlp_cnt, sizeof(c), cudaMemcpyDeviceToHost, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    if (flagged) *flagged = (long long)c[0];
    if (positivity_fallbacks) *positivity_fallbacks = (long long)c[1];
    if (reset) HYPE_CK(cudaMemsetAsync(e->mlp_cnt, 0, sizeof(c), e->stream));
    return HYPE_OK;
}

extern "C" int hype_euler_set_recon(hype_euler* e, int recon) {
    if (!e || recon < HYPE_RECON_CWENO4 || recon > HYPE_RECON_WENO3) return HYPE_ERR_ARG;
    if (e->C4 && recon == HYPE_RECON_LEARNED) return HYPE_ERR_ARG;  // the viscous path keeps the R4 coefficients
    if (e->p.precision == HYPE_PREC_DF64 && recon == HYPE_RECON_WENO3) return HYPE_ERR_UNSUPPORTED;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    e->p.recon = recon;
    return HYPE_OK;
}

extern "C" int hype_euler_sample_features(hype_euler* e, long long stride, float* X, float* D, long long* ns_out) {
    if (!e || stride < 1 || !X || !D) return HYPE_ERR_ARG;
    const long long ns = (e->g.N + stride - 1) / stride;
    float *dX = nullptr, *dD = nullptr;
    cudaError_t ce = cudaMalloc((void**)&dX, sizeof(float) * ns * 3 * mlp::NIN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&dD, sizeof(float) * ns);
    if (ce == cudaSuccess) {
        k_features<<<cdiv(ns, 128), 128, 0, e->stream>>>(e->U, e->g, stride, ns, dX, dD);
        count_launch(1);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(X, dX, sizeof(float) * ns * 3 * mlp::NIN, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(D, dD, sizeof(float) * ns, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    cudaFree(dX);
    cudaFree(dD);
    if (ce != cudaSuccess) {
        set_last_error("hype_euler_sample_features", ce);
        return HYPE_ERR_CUDA;
    }
    if (ns_out) *ns_out = ns;
    return HYPE_OK;
}

extern "C" int hype_euler_set_stage_kernel(hype_euler* e, int mode) {
    if (!e || (mode != HYPE_STAGE_AUTO && mode != HYPE_STAGE_UNFUSED)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    e->stage_mode = mode;
    return prepare(e);
}

extern "C" int hype_euler_profile(hype_euler* e, int enable) {
    if (!e) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    e->prof = enable != 0;
    e->ev_used = 0;
    return HYPE_OK;
}

extern "C" int hype_euler_profile_read(hype_euler* e, double* ms, long long* count) {
    if (!e || !ms || !count) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(e->stream));
    for (int k = 0; k < 3; ++k) {
        ms[k] = 0.0;
        count[k] = 0;
    }
    for (size_t q = 0; q + 1 < e->ev_used + 1 && q < e->ev_used; q += 2) {
        float t = 0.0f;
        HYPE_CK(cudaEventElapsedTime(&t, e->ev[q], e->ev[q + 1]));
        ms[e->ev_kind[q / 2]] += t;
        count[e->ev_kind[q / 2]] += 1;
    }
    return HYPE_OK;
}

// ======================================================================
// Allocation-free RHS evaluation.
//
// Some callers cannot let a plugin allocate device memory: hosts that hand the
// plugin pre-allocated device vectors and own every byte of device memory
// through their own pool, and latency-critical loops where cudaMalloc's
// implicit device-wide synchronisation is not acceptable.  For them,
// hype_euler_rhs_noalloc runs the same three kernels as hype_euler_rhs_device
// with all of their scratch (face traces, face fluxes, the wave-speed and
// admissibility words) in the fixed device array below, which every GPU that
// loads this library holds until the process exits.
namespace hype {
namespace euler {

constexpr long long kNoAllocMaxExt = 18LL * 18 * 18;  // (nx+2)(ny+2)(nz+2) <= 5832, e.g. 16^3 cells
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kNoAllocTraceBytes = align_up(sizeof(double) * NV * NTR * kNoAllocMaxExt);
constexpr size_t kNoAllocFluxBytes = align_up(sizeof(double) * NV * kNoAllocMaxExt);  // one direction
constexpr size_t kNoAllocScalarBytes = align_up(sizeof(DevScalars));
// the reconstruction's two event counters (indicator, positivity fallback): written, never read here
constexpr size_t kNoAllocCounterBytes = align_up(2 * sizeof(unsigned long long));
// ghosted stage input: (nx+6)(ny+6)(nz+6) <= (9/5)^3 (nx+2)(ny+2)(nz+2) for n >= 3
constexpr long long kNoAllocMaxGhost = kNoAllocMaxExt * 729 / 125 + 1;
constexpr size_t kNoAllocGhostBytes = align_up(sizeof(double) * NV * kNoAllocMaxGhost);
constexpr size_t kNoAllocBytes = kNoAllocTraceBytes + 3 * kNoAllocFluxBytes + kNoAllocScalarBytes +
                                 kNoAllocCounterBytes + kNoAllocGhostBytes;  // ~7.7 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

}  // namespace euler
}  // namespace hype

#include <mutex>

static std::mutex g_noalloc_mutex;
static void* g_noalloc_base[128] = {nullptr};

extern "C" long long hype_euler_noalloc_max_ext(void) { return kNoAllocMaxExt; }

extern "C" int hype_euler_rhs_noalloc(const hype_euler_params* p, const double* dU, double* dRHS, double* dt_out,
                                      void* stream) {
    if (!p || !dU || !dRHS) return HYPE_ERR_ARG;
    if (p->nx < 3 || p->ny < 3 || p->nz < 3 || !(p->h > 0) || !(p->cfl > 0) || !(p->gamma > 1.0)) return HYPE_ERR_ARG;
    for (int f = 0; f < 6; ++f)
        if (p->bc[f] < HYPE_BC_PERIODIC || p->bc[f] > HYPE_BC_TRANSMISSIVE) return HYPE_ERR_ARG;
    for (int d = 0; d < 3; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (p->recon != HYPE_RECON_CWENO4 && p->recon != HYPE_RECON_LINEAR4 && p->recon != HYPE_RECON_WENO3) return HYPE_ERR_ARG;
    if (p->precision != HYPE_PREC_FP64 && p->precision != HYPE_PREC_FP32) return HYPE_ERR_ARG;
    if (p->flux < HYPE_FLUX_RUSANOV || p->flux > HYPE_FLUX_ROTHLLC) return HYPE_ERR_ARG;
    if (p->positivity != 0 && p->positivity != 1) return HYPE_ERR_ARG;
    if (p->mu != 0.0) {
        set_last_error("hype_euler_rhs_noalloc: the viscous terms need a context (hype_euler_create)", cudaErrorInvalidValue);
        return HYPE_ERR_UNSUPPORTED;
    }
    const long long ne = (long long)(p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    if (ne > kNoAllocMaxExt) {
        set_last_error("hype_euler_rhs_noalloc: grid exceeds the fixed scratch ((nx+2)(ny+2)(nz+2) > 5832)",
                       cudaErrorInvalidValue);
        return HYPE_ERR_ARG;
    }
    // one-time set-up per device, with that device current: the device address of the
    // scratch array (its name is only a host-side stand-in in host code)
    int dev = 0;
    HYPE_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) return HYPE_ERR_UNSUPPORTED;
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mutex);
        if (!g_noalloc_base[dev]) {
            void* ptr = nullptr;
            cudaError_t ce = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (ce != cudaSuccess) {
                set_last_error("cudaGetSymbolAddress", ce);
                return HYPE_ERR_CUDA;
            }
            g_noalloc_base[dev] = ptr;
        }
        base = (unsigned char*)g_noalloc_base[dev];
    }
    Geo g;
    g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
    for (int f = 0; f < 6; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny * p->nz;
    g.NE = ne;
    g.ex = p->nx + 2;
    g.ey = p->ny + 2;
    set_ghost_extents(g);
    void* T = base;
    double* Fx = (double*)(base + kNoAllocTraceBytes);
    double* Fy = (double*)(base + kNoAllocTraceBytes + kNoAllocFluxBytes);
    double* Fz = (double*)(base + kNoAllocTraceBytes + 2 * kNoAllocFluxBytes);
    DevScalars* ds = (DevScalars*)(base + kNoAllocTraceBytes + 3 * kNoAllocFluxBytes);
    unsigned long long* counters =
        (unsigned long long*)(base + kNoAllocTraceBytes + 3 * kNoAllocFluxBytes + kNoAllocScalarBytes);
    void* G = base + kNoAllocTraceBytes + 3 * kNoAllocFluxBytes + kNoAllocScalarBytes + kNoAllocCounterBytes;
    cudaStream_t s = (cudaStream_t)stream;
    // the scratch keeps the previous call's contents: the wave-speed maximum and the
    // admissibility word must start cleared; traces and fluxes are fully rewritten
    k_reset_slot<<<1, 1, 0, s>>>(ds, 4);
    HYPE_CK(cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), s));
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4), g.nz + 2);
    const int rec = p->recon;
    const int pad = p->positivity;
    if (p->precision == HYPE_PREC_FP32) {
        // the FP32 admissibility check of the positivity fallback keeps its per-warp columns in
        // dynamic shared memory, as in the context path
        const size_t ck_bytes = pad ? sizeof(float) * 4 * 2 * NTR * 32 : 0;
        k_ghost<float><<<ghost_grid(g), kGhostThreads, 0, s>>>(dU, (float*)G, g);
        k_recon<float><<<gr, br, ck_bytes, s>>>((const float*)G, (float*)T, g, rec, pad, p->gamma - 1.0, counters);
    } else {
        k_ghost<double><<<ghost_grid(g), kGhostThreads, 0, s>>>(dU, (double*)G, g);
        k_recon<double><<<gr, br, 0, s>>>((const double*)G, (double*)T, g, rec, pad, p->gamma - 1.0, counters);
    }
    launch_faces(g, T, Fx, Fy, Fz, p->gamma, ds, 4, p->precision == HYPE_PREC_FP32, p->flux, s);
    const Stage st{0.0, 0.0, 0.0, 1};
    const dim3 bu(32, 8), gu(cdiv(g.nx, 32), cdiv(g.ny, 8), g.nz);
    if (p->precision == HYPE_PREC_FP32)
        k_update<true><<<gu, bu, 0, s>>>(Fx, Fy, Fz, nullptr, nullptr, dRHS, g, 1.0 / p->h, st, ds);
    else
        k_update<false><<<gu, bu, 0, s>>>(Fx, Fy, Fz, nullptr, nullptr, dRHS, g, 1.0 / p->h, st, ds);
    HYPE_LAUNCHED(7);
    if (dt_out) {
        unsigned long long w[2];
        HYPE_CK(cudaMemcpyAsync(&w[0], &ds->smax_bits[4], sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        HYPE_CK(cudaMemcpyAsync(&w[1], &ds->bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        HYPE_CK(cudaStreamSynchronize(s));
        *dt_out = cfl_dt(p->cfl * p->h, bits_to_double(w[0]), p->recon);
        if (w[1] != ~0ull) return HYPE_ERR_STATE;
    }
    return HYPE_OK;
}

// One step of the current reconstruction and, from the same state, one full-CWENO4
// step; keeps the first, returns the relative L1 difference of the densities.
extern "C" int hype_euler_shadow_step(hype_euler* e, double* t_inout, double* dt_inout, double* l1_rel) {
    if (!e || !t_inout || !dt_inout || !l1_rel) return HYPE_ERR_ARG;
    const size_t bytes = sizeof(double) * NV * (size_t)e->g.N;
    const int recon = e->p.recon;
    const double t0 = *t_inout, dt0 = *dt_inout;
    HYPE_CK(cudaMemcpyAsync(e->S, e->U, bytes, cudaMemcpyDeviceToDevice, e->stream));
    e->p.recon = HYPE_RECON_CWENO4;
    double t = t0, dt = dt0;
    int rc = hype_euler_step(e, 1, &t, &dt, nullptr);
    e->p.recon = recon;
    if (rc) return rc;
    HYPE_CK(cudaMemcpyAsync(e->L, e->U, sizeof(double) * (size_t)e->g.N, cudaMemcpyDeviceToDevice, e->stream));
    HYPE_CK(cudaMemcpyAsync(e->U, e->S, bytes, cudaMemcpyDeviceToDevice, e->stream));
    *t_inout = t0;
    *dt_inout = dt0;
    if ((rc = hype_euler_step(e, 1, t_inout, dt_inout, nullptr))) return rc;
    double* acc = e->acc;
    HYPE_CK(cudaMemsetAsync(acc, 0, 2 * sizeof(double), e->stream));
    k_l1<<<608, 256, 0, e->stream>>>(e->U, e->L, e->g.N, acc);
    HYPE_LAUNCHED(1);
    double h[2];
    HYPE_CK(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, e->stream));
    HYPE_CK(cudaStreamSynchronize(e->stream));
    *l1_rel = h[0] / h[1];
    return HYPE_OK;
}
