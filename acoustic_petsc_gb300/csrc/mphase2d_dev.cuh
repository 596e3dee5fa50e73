// mphase2d_dev.cuh -- the device side of the 2D multiphase RHS shared by two translation
// units: mphase2d.cu instantiates the FP64 kernels (compiled without FMA contraction, so
// they round as the reference does) and mphase2d_f32.cu the FP32 recon/flux form (compiled
// with contraction, which only the FP32 form may use).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "mlp_kernels.cuh"
#include "mphase2d_kernels.cuh"

namespace hype {
namespace mp2d {

struct Geo {
    int nx, ny, nv;
    int bc[4];
    long long N, NE;  // owned cells, extended cells (nx+2)(ny+2)
};

// out = a*X + b*Y + (c*dt)*L, L the divergence with the volume-fraction term
struct Stage {
    double a, b, c, d;  // c*dt/d: the stage's dt fraction formed as the reference forms dt/r
    int rhs_only;
};

struct DevScalars {
    unsigned long long smax_bits[12];  // per stage (10 max) + RHS-only slot 11
    double dt, t;
    unsigned long long bad;
    unsigned long long fallback;  // owned cells reconstructed with the minmod fallback
};

__device__ __forceinline__ double node_x(int q) {
    return q < 2 ? 0.5 : q < 4 ? -0.5 : (q == 4 || q == 6) ? -0.28867513459481287 : 0.28867513459481287;
}
__device__ __forceinline__ double node_y(int q) {
    return q < 4 ? ((q & 1) ? 0.28867513459481287 : -0.28867513459481287) : (q < 6 ? -0.5 : 0.5);
}
// face f (0 -x, 1 +x, 2 -y, 3 +y), Gauss point q (0: -g, 1: +g)
__device__ __forceinline__ double face_x(int f, int q) {
    const double g = q ? 0.28867513459481287 : -0.28867513459481287;
    return f == 0 ? -0.5 : f == 1 ? 0.5 : g;
}
__device__ __forceinline__ double face_y(int f, int q) {
    const double g = q ? 0.28867513459481287 : -0.28867513459481287;
    return f == 2 ? -0.5 : f == 3 ? 0.5 : g;
}


// boundary maps of the offsets -2..2 of one cell (replaces DMGlobalToLocal + the
// BC sweeps of rhs_function.c:54-170)
struct CellMap {
    int mi[5], mj[5], fi, fj;  // fi/fj bit o: offset o-2 is a reflective ghost
    long long e;               // extended-cell index of the traces
};

__device__ __forceinline__ void cell_map(const Geo& g, int i, int j, CellMap& cm) {
    cm.fi = cm.fj = 0;
#pragma unroll
    for (int o = 0; o < 5; ++o) {
        int f = 0;
        cm.mi[o] = bmap(i + o - 2, g.nx, g.bc[0], g.bc[1], &f);
        cm.fi |= f << o;
        f = 0;
        cm.mj[o] = bmap(j + o - 2, g.ny, g.bc[2], g.bc[3], &f);
        cm.fj |= f << o;
    }
    cm.e = (long long)(j + 1) * (g.nx + 2) + (i + 1);
}

// primitive variable c at offset (oi, oj) of the FP64 primitives or of the FP32 form's FP32 copy
// (PT); a reflective ghost negates the velocity normal to its wall (x: u, y: v)
template <int MODEL, typename PT>
__device__ __forceinline__ PT ldp(const PT* __restrict__ P, const Geo& g, const CellMap& cm, int c, int oi, int oj) {
    constexpr int IU = MODEL == HYPE_MP_DI4 ? 1 : 2;
    PT v = __ldg(P + (long long)c * g.N + (long long)cm.mj[oj + 2] * g.nx + cm.mi[oi + 2]);
    if (c == IU && ((cm.fi >> (oi + 2)) & 1)) v = -v;
    if (c == IU + 1 && ((cm.fj >> (oj + 2)) & 1)) v = -v;
    return v;
}

// one cell: 2D CWENO4 (or its optimal-weight R4 limit) of every primitive variable,
// its 8 face traces; returns whether the 8 admissibility nodes pass (rhs_function.c:173-250)
template <typename R, int MODEL, typename PT>
__device__ __forceinline__ bool mp_cell_recon(const PT* __restrict__ P, R* __restrict__ T, const Geo& g, const Eos& e,
                                              const CellMap& cm, bool linear) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    R VN[8][NV];
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        auto ld = [&](int oi, int oj) -> R { return (R)ldp<MODEL>(P, g, cm, c, oi, oj); };
        R ux[5], uy[5], cf[NDOF];
#pragma unroll
        for (int o = 0; o < 5; ++o) {
            ux[o] = ld(o - 2, 0);
            uy[o] = ld(0, o - 2);
        }
        cweno2d<R>(ux[2], ux, uy, ld(1, 1), ld(1, -1), ld(-1, 1), ld(-1, -1), cf, linear);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            R v = R(0);
#pragma unroll
            for (int k = 0; k < NDOF; ++k) v += cf[k] * R(basis2(node_x(q), node_y(q), k));
            VN[q][c] = v;
        }
        R* Tc = T + (long long)c * 8 * g.NE + cm.e;
#pragma unroll
        for (int f = 0; f < 4; ++f)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                R v = R(0);
#pragma unroll
                for (int k = 0; k < NDOF; ++k) v += cf[k] * R(basis2(face_x(f, q), face_y(f, q), k));
                Tc[(long long)(f * 2 + q) * g.NE] = v;
            }
    }
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 8; ++q) ok = ok && pad_ok<R>(e, VN[q]);
    return ok;
}

// physically inadmissible somewhere in the cell: first order + minmod slopes (rhs_function.c:239-250)
template <typename R, int MODEL, typename PT>
__device__ __forceinline__ void mp_cell_fallback(const PT* __restrict__ P, R* __restrict__ T, const Geo& g,
                                                 const CellMap& cm) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        auto ld = [&](int oi, int oj) -> R { return (R)ldp<MODEL>(P, g, cm, c, oi, oj); };
        const R w0 = ld(0, 0);
        const R sx = minmod<R>(ld(1, 0) - w0, w0 - ld(-1, 0));
        const R sy = minmod<R>(ld(0, 1) - w0, w0 - ld(0, -1));
        R* Tc = T + (long long)c * 8 * g.NE + cm.e;
#pragma unroll
        for (int f = 0; f < 4; ++f)
#pragma unroll
            for (int q = 0; q < 2; ++q) Tc[(long long)(f * 2 + q) * g.NE] = w0 + sx * R(face_x(f, q)) + sy * R(face_y(f, q));
    }
}

// PT: the primitives' type (FP64; the FP32 form reads its FP32 copy)
template <typename R, int MODEL, typename PT = double>
__global__ void __launch_bounds__(128) k_mp_recon(const PT* __restrict__ P, R* __restrict__ T, Geo g, Eos e,
                                                  DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    if (i > g.nx || j > g.ny) return;
    const bool gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny);
    if (gi && gj) return;
    CellMap cm;
    cell_map(g, i, j, cm);
    if (mp_cell_recon<R, MODEL, PT>(P, T, g, e, cm, false)) return;
    if (!gi && !gj) atomicAdd(&ds->fallback, 1ull);
    mp_cell_fallback<R, MODEL, PT>(P, T, g, cm);
}

// Network inputs of one cell along direction d (0: x, 1: y): the normalised 5-point
// stencils of the mixture density, the normal and tangential velocity, the pressure
// and the volume fraction, each against a floor of 1 % of its magnitude in the cell
// (density |rho|, velocities sqrt((|p| + pi)/rho), pressure |p| + pi, volume fraction 1).
// From the FP64 primitives (PT = double) or, in the FP32 form, from its FP32 copy (the mixture
// density and the floor's pi then in FP32).
template <int MODEL, typename PT = double>
__device__ __forceinline__ void mp_features(const PT* __restrict__ P, const Geo& g, const Eos& e, const CellMap& cm,
                                            int d, float* x) {
    constexpr int IU = MODEL == HYPE_MP_DI4 ? 1 : 2;
    constexpr int IP = MODEL == HYPE_MP_DI4 ? 3 : 4;
    constexpr int IA = MODEL == HYPE_MP_DI4 ? 4 : 5;
    float q[5][5];
#pragma unroll
    for (int o = 0; o < 5; ++o) {
        const int oi = d == 0 ? o - 2 : 0, oj = d == 1 ? o - 2 : 0;
        const PT a = ldp<MODEL>(P, g, cm, IA, oi, oj);
        const PT rho = MODEL == HYPE_MP_DI4
                           ? ldp<MODEL>(P, g, cm, 0, oi, oj)
                           : a * ldp<MODEL>(P, g, cm, 0, oi, oj) + (PT(1.0) - a) * ldp<MODEL>(P, g, cm, 1, oi, oj);
        const PT u = ldp<MODEL>(P, g, cm, IU, oi, oj), v = ldp<MODEL>(P, g, cm, IU + 1, oi, oj);
        q[0][o] = (float)rho;
        q[1][o] = (float)(d == 0 ? u : v);
        q[2][o] = (float)(d == 0 ? v : u);
        q[3][o] = (float)ldp<MODEL>(P, g, cm, IP, oi, oj);
        q[4][o] = (float)a;
    }
    float pif;
    if constexpr (sizeof(PT) == sizeof(double)) {
        double gm, pi;
        mix(e, (double)q[4][2], gm, pi);
        pif = (float)pi;
    } else {
        float gm;
        mix_r<float>(e, q[4][2], gm, pif);
    }
    const float srho = fabsf(q[0][2]) + 1e-30f;
    const float sp = fabsf(q[3][2]) + pif;
    const float svel = sqrtf(sp / srho);
    const float sc[5] = {srho, svel, svel, sp, 1.0f};
#pragma unroll
    for (int k = 0; k < 5; ++k) mlp::normalise5(q[k], sc[k], x + 5 * k);
}

// Indicator-gated reconstruction (no counterpart in the reference): the network scores
// each cell from its two directional stencils on the tensor cores; flagged cells take
// the full CWENO4, the others its R4 limit; R4 traces that fail the admissibility
// nodes are redone with CWENO4, and the minmod fallback stays the last resort.
template <typename R, int MODEL, typename PT = double>
__global__ void __launch_bounds__(128) k_mp_recon_learned(const PT* __restrict__ P, R* __restrict__ T, Geo g, Eos e,
                                                          DevScalars* __restrict__ ds,
                                                          const mlp::MmaWeights* __restrict__ wts, float logit_thr,
                                                          unsigned long long* __restrict__ flagged) {
    constexpr int NR = 64;  // 32 cells x 2 directions per warp
    __shared__ __align__(16) __nv_bfloat16 rows[4][NR * mlp::RSTRIDE];
    __shared__ float lg[4][NR];
    __shared__ unsigned cnt;
    if (threadIdx.x == 0 && threadIdx.y == 0) cnt = 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const bool gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny);
    const bool active = !(i > g.nx || j > g.ny) && !(gi && gj);
    CellMap cm;
    if (active) cell_map(g, i, j, cm);
#pragma unroll 1
    for (int d = 0; d < 2; ++d) {
        float x[mlp::NIN];
        if (active) mp_features<MODEL, PT>(P, g, e, cm, d, x);
        mlp::stage_row(rows[threadIdx.y] + (threadIdx.x * 2 + d) * mlp::RSTRIDE, x, active);
    }
    __syncthreads();  // counter cleared, rows staged
    mlp::warp_logits<NR>(wts, rows[threadIdx.y], lg[threadIdx.y]);
    __syncwarp();
    const float best = fmaxf(lg[threadIdx.y][threadIdx.x * 2], lg[threadIdx.y][threadIdx.x * 2 + 1]);
    if (active) {
        bool full = best > logit_thr;
        bool ok = mp_cell_recon<R, MODEL, PT>(P, T, g, e, cm, !full);
        if (!ok && !full) {
            full = true;
            ok = mp_cell_recon<R, MODEL, PT>(P, T, g, e, cm, false);
        }
        if (!ok) {
            if (!gi && !gj) atomicAdd(&ds->fallback, 1ull);
            mp_cell_fallback<R, MODEL, PT>(P, T, g, cm);
        }
        if (full && best > logit_thr && !gi && !gj) atomicAdd(&cnt, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0 && cnt) atomicAdd(flagged, (unsigned long long)cnt);
}

// The gate scored on its own pass (hype_mp2d_set_gate_per_step: a step's first stage): one flag byte
// per extended cell the reconstruction covers (the frame's corners keep the zero the array is created
// with), with k_mp_recon_learned's features and tensor-core scoring
template <int MODEL, typename PT = double>
__global__ void __launch_bounds__(128) k_mp_gate(const PT* __restrict__ P, unsigned char* __restrict__ flag, Geo g,
                                                 Eos e, const mlp::MmaWeights* __restrict__ wts, float logit_thr) {
    constexpr int NR = 64;  // 32 cells x 2 directions per warp
    __shared__ __align__(16) __nv_bfloat16 rows[4][NR * mlp::RSTRIDE];
    __shared__ float lg[4][NR];
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    const bool gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny);
    const bool active = !(i > g.nx || j > g.ny) && !(gi && gj);
    CellMap cm;
    if (active) cell_map(g, i, j, cm);
#pragma unroll 1
    for (int d = 0; d < 2; ++d) {
        float x[mlp::NIN];
        if (active) mp_features<MODEL, PT>(P, g, e, cm, d, x);
        mlp::stage_row(rows[threadIdx.y] + (threadIdx.x * 2 + d) * mlp::RSTRIDE, x, active);
    }
    __syncwarp();  // the warp's rows staged
    mlp::warp_logits<NR>(wts, rows[threadIdx.y], lg[threadIdx.y]);
    __syncwarp();
    if (active) flag[cm.e] = fmaxf(lg[threadIdx.y][threadIdx.x * 2], lg[threadIdx.y][threadIdx.x * 2 + 1]) > logit_thr;
}

// the gate's flags widened to each cell's 3 x 3 neighbourhood over the extended grid: flags scored
// on a step's first stage still cover a discontinuity that moves by less than a cell in the step
static __global__ void __launch_bounds__(128) k_mp_gate_dilate(const unsigned char* __restrict__ f, unsigned char* __restrict__ o,
                                                        Geo g) {
    const int ex = g.nx + 2, ey = g.ny + 2;
    const int i = blockIdx.x * 128 + threadIdx.x, j = blockIdx.y;
    if (i >= ex) return;
    unsigned m = 0;
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
        const int jj = j + dj;
        if (jj < 0 || jj >= ey) continue;
        const unsigned char* row = f + (long long)jj * ex;
        m |= __ldg(row + i);
        if (i > 0) m |= __ldg(row + i - 1);
        if (i + 1 < ex) m |= __ldg(row + i + 1);
    }
    o[(long long)j * ex + i] = (unsigned char)m;
}

// k_mp_recon_learned's reconstruction on flags the gate wrote: flagged cells take CWENO4, the others
// its R4 limit, R4 traces that fail the admissibility nodes are redone with CWENO4, the minmod
// fallback stays the last resort; counts the owned cells the flags send to CWENO4
template <typename R, int MODEL, typename PT = double>
__global__ void __launch_bounds__(128) k_mp_recon_flags(const PT* __restrict__ P, R* __restrict__ T, Geo g, Eos e,
                                                        DevScalars* __restrict__ ds,
                                                        const unsigned char* __restrict__ flags,
                                                        unsigned long long* __restrict__ flagged) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    if (i > g.nx || j > g.ny) return;
    const bool gi = (i < 0 || i >= g.nx), gj = (j < 0 || j >= g.ny);
    if (gi && gj) return;
    CellMap cm;
    cell_map(g, i, j, cm);
    bool full = flags[cm.e] != 0;
    if (full && !gi && !gj) atomicAdd(flagged, 1ull);
    bool ok = mp_cell_recon<R, MODEL, PT>(P, T, g, e, cm, !full);
    if (!ok && !full) ok = mp_cell_recon<R, MODEL, PT>(P, T, g, e, cm, false);
    if (!ok) {
        if (!gi && !gj) atomicAdd(&ds->fallback, 1ull);
        mp_cell_fallback<R, MODEL, PT>(P, T, g, cm);
    }
}

// the gate passes of one RHS when the gate is scored once per step: score (and widen) on the step's
// first stage or an RHS-only call, then every stage reconstructs from the widened flags
struct GateStep {
    bool on;               // hype_mp2d_set_gate_per_step
    bool score;            // this stage scores
    unsigned char* raw;    // the network's flags
    unsigned char* wide;   // their 3 x 3 widening
};

template <typename R, int MODEL, typename PT>
inline void launch_gated_recon(const PT* P, R* T, const Geo& g, const Eos& e, DevScalars* ds,
                               const mlp::MmaWeights* wts, float logit_thr, unsigned long long* flagged,
                               const GateStep& gs, cudaStream_t st) {
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4));
    if (gs.score) {
        k_mp_gate<MODEL, PT><<<gr, br, 0, st>>>(P, gs.raw, g, e, wts, logit_thr);
        k_mp_gate_dilate<<<dim3(cdiv(g.nx + 2, 128), g.ny + 2), 128, 0, st>>>(gs.raw, gs.wide, g);
    }
    k_mp_recon_flags<R, MODEL, PT><<<gr, br, 0, st>>>(P, T, g, e, ds, gs.wide, flagged);
}

// Training data: for every stride-th owned cell its features X[s][3][25] (x, y, and y
// again: the training kernels take three directions and the max over a repeated row
// is the max over the two) and D[s], the largest change that the nonlinear CWENO4
// weights make to one of its 8 face traces relative to the R4 polynomial, over the
// primitive variables, in units of the variable's magnitude in the cell.
template <int MODEL>
__global__ void __launch_bounds__(128) k_mp_features(const double* __restrict__ P, Geo g, Eos e, long long stride,
                                                     long long ns, float* __restrict__ X, float* __restrict__ D) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    constexpr int IU = MODEL == HYPE_MP_DI4 ? 1 : 2;
    constexpr int IP = MODEL == HYPE_MP_DI4 ? 3 : 4;
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const long long cell = s * stride;
    const int i = (int)(cell % g.nx), j = (int)(cell / g.nx);
    CellMap cm;
    cell_map(g, i, j, cm);
    float* xs = X + s * 3 * mlp::NIN;
    mp_features<MODEL>(P, g, e, cm, 0, xs);
    mp_features<MODEL>(P, g, e, cm, 1, xs + mlp::NIN);
    for (int k = 0; k < mlp::NIN; ++k) xs[2 * mlp::NIN + k] = xs[mlp::NIN + k];
    const double a = ldp<MODEL>(P, g, cm, MODEL == HYPE_MP_DI4 ? 4 : 5, 0, 0);
    const double rho = MODEL == HYPE_MP_DI4 ? ldp<MODEL>(P, g, cm, 0, 0, 0)
                                            : a * ldp<MODEL>(P, g, cm, 0, 0, 0) + (1.0 - a) * ldp<MODEL>(P, g, cm, 1, 0, 0);
    double gm, pi;
    mix(e, a, gm, pi);
    const double sp = fabs(ldp<MODEL>(P, g, cm, IP, 0, 0)) + pi;
    const double svel = sqrt(sp / (fabs(rho) + 1e-300));
    double dmax = 0.0;
#pragma unroll 1
    for (int c = 0; c < NV; ++c) {
        auto ld = [&](int oi, int oj) { return ldp<MODEL>(P, g, cm, c, oi, oj); };
        double ux[5], uy[5], cf[NDOF], cl[NDOF];
        for (int o = 0; o < 5; ++o) {
            ux[o] = ld(o - 2, 0);
            uy[o] = ld(0, o - 2);
        }
        cweno2d<double>(ux[2], ux, uy, ld(1, 1), ld(1, -1), ld(-1, 1), ld(-1, -1), cf, false);
        cweno2d<double>(ux[2], ux, uy, ld(1, 1), ld(1, -1), ld(-1, 1), ld(-1, -1), cl, true);
        const double scale = (c == IU || c == IU + 1) ? svel : c == IP ? sp : c == NV - 1 ? 1.0 : fabs(ux[2]) + 1e-300;
        for (int f = 0; f < 4; ++f)
            for (int q = 0; q < 2; ++q) {
                double dv = 0.0;
                for (int k = 0; k < NDOF; ++k) dv += (cf[k] - cl[k]) * basis2(face_x(f, q), face_y(f, q), k);
                dmax = fmax(dmax, fabs(dv) / scale);
            }
    }
    D[s] = (float)dmax;
}

// face fluxes stored in the solver's type (FP64; the FP32 form keeps them in FP32 for its update)
template <typename R, int MODEL, int D>
__global__ void __launch_bounds__(128) k_mp_faces(const R* __restrict__ T, R* __restrict__ F, Geo g, Eos e,
                                                  DevScalars* __restrict__ ds, int slot) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int fx = g.nx + (D == 0), fy = g.ny + (D == 1);
    R smax_r = R(0);  // in the solver's type: the maximum of FP32 speeds is the same taken in FP32
    bool bad = false;
    if (i < fx && j < fy) {
        const long long eR = (long long)(j + 1) * (g.nx + 2) + (i + 1);
        const long long eL = eR - (D == 0 ? 1 : (g.nx + 2));
        R acc[NV + 1];
#pragma unroll
        for (int c = 0; c <= NV; ++c) acc[c] = R(0);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            R VL[NV], VR[NV], fl[MAXV + 1];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                VL[c] = T[((long long)c * 8 + (2 * D + 1) * 2 + q) * g.NE + eL];
                VR[c] = T[((long long)c * 8 + (2 * D) * 2 + q) * g.NE + eR];
            }
            const R s = rot_hllc2<R, MODEL>(e, VL, VR, R(D == 0), R(D == 1), fl, bad);
            smax_r = fmax(smax_r, s);
#pragma unroll
            for (int c = 0; c <= NV; ++c) acc[c] += R(0.5) * fl[c];
        }
        const long long nf = (long long)fx * fy;
        const long long f = (long long)j * fx + i;
#pragma unroll
        for (int c = 0; c <= NV; ++c) F[c * nf + f] = acc[c];
        if (bad) atomicMin(&ds->bad, (unsigned long long)((long long)(j < g.ny ? j : g.ny - 1) * g.nx + (i < g.nx ? i : g.nx - 1)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) smax_r = fmax(smax_r, __shfl_xor_sync(0xffffffffu, smax_r, o));
    const double smax = (double)smax_r;
    if ((threadIdx.x & 31) == 0 && smax > 0.0) atomicMax(&ds->smax_bits[slot], (unsigned long long)__double_as_longlong(smax));
}

}  // namespace mp2d
}  // namespace hype
