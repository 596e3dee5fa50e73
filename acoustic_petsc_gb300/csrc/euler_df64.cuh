// euler_df64.cuh -- the CWENO4 reconstruction of euler_kernels.cuh (cweno4, face_traces) in
// double-float arithmetic (df64.cuh), for the HYPE_PREC_DF64 form of the 3D Euler RHS.
//
// The stencil values arrive as deviations from a per-variable reference value r (the
// stage input's value at cell 0 rounded to a 24-bit significand), so every coefficient but
// the constant one is formed from differences of small numbers, and the 48-bit
// significand is spent on the deviation: the absolute error of a trace is ~2^-48 |u - r|
// plus the final FP64 rounding of r + trace, against ~2^-53 |u| for the FP64 form.  The
// coefficients, smoothness indicators, nonlinear weights and face traces are the same
// mathematics as cweno4 (3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259)
// and face_traces (plane_wave/reconstruction.c:12-21 at the 2x2 Gauss points); the
// weights take the ratio form w_k = g_k (m / s_k)^4 / sum, m = min_k s_k, s_k = IS_k + 1e-12,
// because (1e-12)^4 is below the FP32 exponent range.
#pragma once

#include "df64.cuh"
#include "euler_kernels.cuh"

namespace hype {
namespace euler {

__device__ __forceinline__ df64 df_half(df64 x) { return df_scale(x, 0.5f); }
__device__ __forceinline__ df64 df_quarter(df64 x) { return df_scale(x, 0.25f); }

// 20 CWENO4 (or, linear, R4) coefficients of one variable from its 33-point stencil of
// deviations; cf[0] is the centre deviation
__device__ __forceinline__ void cweno4_df(const df64* __restrict__ s, bool linear, df64* __restrict__ cf) {
    const df64 u0 = s[0];
    df64 d4[3], dd4[3], ddd4[3], c1[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const df64 m2 = s[S1(d, -2)], m1 = s[S1(d, -1)], p1 = s[S1(d, 1)], p2 = s[S1(d, 2)];
        const df64 a = p1 - m1, b = p2 - m2;
        d4[d] = a * dfc(82. / 120.) - b * dfc(11. / 120.);
        dd4[d] = df_half(m1 + p1) - u0;
        ddd4[d] = (b - df_scale(a, 2.0f)) * dfc(1. / 12.);
        c1[d] = df_half(a);
    }
    df64 cx[3], aab[3], abb[3];
#pragma unroll
    for (int P = 0; P < 3; ++P) {
        const int a = P == 1 ? 1 : 0, b = P == 0 ? 1 : 2;
        const df64 mm = s[SQ(a, 0, b, 0)], mp = s[SQ(a, 0, b, 1)], pm = s[SQ(a, 1, b, 0)], pp = s[SQ(a, 1, b, 1)];
        const df64 Pd = pp - mm, Qd = mp - pm;
        cx[P] = df_quarter((mm + pp) - (mp + pm));
        aab[P] = df_quarter(Pd + Qd) - c1[b];
        abb[P] = df_quarter(Pd - Qd) - c1[a];
    }
    const df64 xyz = df_scale((s[SO(1, 1, 1)] - s[SO(0, 0, 0)]) +
                                  ((s[SO(0, 0, 1)] + s[SO(0, 1, 0)] + s[SO(1, 0, 0)]) -
                                   (s[SO(0, 1, 1)] + s[SO(1, 0, 1)] + s[SO(1, 1, 0)])),
                              0.125f);
    cf[0] = u0;
    if (linear) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            cf[CLIN(d)] = d4[d];
            cf[CSQ(d)] = dd4[d];
            cf[CCUBE(d)] = ddd4[d];
        }
        cf[7] = cx[0]; cf[8] = cx[1]; cf[9] = cx[2];
        cf[13] = aab[0]; cf[14] = abb[0]; cf[15] = aab[1]; cf[16] = abb[1]; cf[17] = aab[2]; cf[18] = abb[2]; cf[19] = xyz;
        return;
    }
    df64 c1sq[3], ddsq[3], cxsq[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c1sq[d] = df_sqr(c1[d]);
        ddsq[d] = df_sqr(dd4[d]);
        cxsq[d] = df_sqr(cx[d]);
    }
    const df64 r13_3 = dfc(13. / 3.), r7_6 = dfc(7. / 6.);
    const df64 common = (ddsq[0] + ddsq[1] + ddsq[2]) * r13_3 + (cxsq[0] + cxsq[1] + cxsq[2]) * r7_6;
    // sums as balanced trees: a double-float addition is a chain of ~9 dependent FP32
    // operations, so independent partial sums keep more of them in flight
    const df64 lin = (d4[0] * (d4[0] + ddd4[0] * dfc(0.2)) + d4[1] * (d4[1] + ddd4[1] * dfc(0.2))) +
                     (d4[2] * (d4[2] + ddd4[2] * dfc(0.2)) + common);
    const df64 mixed = ((df_sqr(aab[0]) + df_sqr(abb[0])) + (df_sqr(aab[1]) + df_sqr(abb[1]))) +
                       (df_sqr(aab[2]) + df_sqr(abb[2]));
    const df64 cubic = (df_sqr(ddd4[0]) + df_sqr(ddd4[1])) + df_sqr(ddd4[2]);
    const df64 IS4 = (lin + mixed * dfc(4.7)) + (cubic * dfc(39.06) + df_sqr(xyz) * dfc(61. / 48.));
    const df64 IS0 = (c1sq[0] + c1sq[1] + c1sq[2]) + common;
    df64 sd1[6], sd2[6], sx1[6], sx2[6], IS3[6];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int e1 = (d == 0) ? 1 : 0, e2 = (d == 2) ? 1 : 2;
        const int k1 = (d + e1 == 1) ? 0 : (d + e1 == 3) ? 1 : 2;
        const int k2 = (d + e2 == 1) ? 0 : (d + e2 == 3) ? 1 : 2;
        const df64 p1 = s[S1(d, 1)], p2 = s[S1(d, 2)], m1 = s[S1(d, -1)], m2 = s[S1(d, -2)];
        sd2[2 * d] = df_half(u0 + p2) - p1;
        sd1[2 * d] = (p1 - u0) - sd2[2 * d];
        sx1[2 * d] = df_half(s[SQ(d, 1, e1, 1)] - s[SQ(d, 1, e1, 0)]) - c1[e1];
        sx2[2 * d] = df_half(s[SQ(d, 1, e2, 1)] - s[SQ(d, 1, e2, 0)]) - c1[e2];
        sd2[2 * d + 1] = df_half(m2 + u0) - m1;
        sd1[2 * d + 1] = (u0 - m1) + sd2[2 * d + 1];
        sx1[2 * d + 1] = df_half(s[SQ(d, 0, e1, 0)] - s[SQ(d, 0, e1, 1)]) + c1[e1];
        sx2[2 * d + 1] = df_half(s[SQ(d, 0, e2, 0)] - s[SQ(d, 0, e2, 1)]) + c1[e2];
        const int k3 = 3 - k1 - k2;
        const df64 rest1 = c1sq[e1] + c1sq[e2];
        const df64 rest2 = ddsq[e1] + ddsq[e2];
        const df64 restx = cxsq[k3];
#pragma unroll
        for (int sg = 0; sg < 2; ++sg) {
            const int m = 2 * d + sg;
            const df64 a1 = rest1 + df_sqr(sd1[m]);
            const df64 a2 = rest2 + df_sqr(sd2[m]);
            const df64 a3 = restx + df_sqr(sx1[m]) + df_sqr(sx2[m]);
            IS3[m] = a1 + a2 * r13_3 + a3 * r7_6;
        }
    }
    // weights: gammaHi = gammaLo = 0.85, p = 4, eps = 1e-12, in the ratio form
    df64 q[8];
    q[0] = IS4 + dfc(1.0e-12);
    q[1] = IS0 + dfc(1.0e-12);
#pragma unroll
    for (int m = 0; m < 6; ++m) q[2 + m] = IS3[m] + dfc(1.0e-12);
    df64 mn = q[0];
#pragma unroll
    for (int k = 1; k < 8; ++k) mn = df_min(mn, q[k]);
    df64 w[8];
    const df64 gk[3] = {dfc(0.85), dfc((1.0 - 0.85) * 0.85), dfc((1. / 6.) * (1 - 0.85) * (1 - 0.85))};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const df64 r2 = df_sqr(df_div(mn, q[k]));
        w[k] = df_sqr(r2) * gk[k == 0 ? 0 : k == 1 ? 1 : 2];
    }
    const df64 total = ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7]));
    const df64 rt = df_div(dfc(1.0), total);
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] = w[k] * rt;
    const df64 wr = w[0] * dfc(1.0 / 0.85);
    const df64 o0 = w[1] - wr * gk[1];
    df64 os[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) os[m] = w[2 + m] - wr * gk[2];
    const df64 ox = os[0] + os[1], oy = os[2] + os[3], oz = os[4] + os[5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const df64 okeep = o0 + ((d == 0) ? oy + oz : (d == 1) ? ox + oz : ox + oy);
        cf[CLIN(d)] = (wr * d4[d] + okeep * c1[d]) + (os[2 * d] * sd1[2 * d] + os[2 * d + 1] * sd1[2 * d + 1]);
        cf[CSQ(d)] = (wr + okeep) * dd4[d] + (os[2 * d] * sd2[2 * d] + os[2 * d + 1] * sd2[2 * d + 1]);
    }
    cf[7] = (wr + o0 + oz) * cx[0] + ((os[0] * sx1[0] + os[1] * sx1[1]) + (os[2] * sx1[2] + os[3] * sx1[3]));
    cf[8] = (wr + o0 + ox) * cx[1] + ((os[2] * sx2[2] + os[3] * sx2[3]) + (os[4] * sx2[4] + os[5] * sx2[5]));
    cf[9] = (wr + o0 + oy) * cx[2] + ((os[0] * sx2[0] + os[1] * sx2[1]) + (os[4] * sx1[4] + os[5] * sx1[5]));
#pragma unroll
    for (int d = 0; d < 3; ++d) cf[CCUBE(d)] = wr * ddd4[d];
    cf[13] = wr * aab[0]; cf[14] = wr * abb[0]; cf[15] = wr * aab[1]; cf[16] = wr * abb[1];
    cf[17] = wr * aab[2]; cf[18] = wr * abb[2]; cf[19] = wr * xyz;
}

// the 8 traces of the two faces normal to D (face_traces' even/odd split), deviations
template <int D>
__device__ __forceinline__ void face_traces_df(const df64* __restrict__ c, df64* __restrict__ out) {
    constexpr int T1 = (D == 0) ? 1 : 0;
    constexpr int T2 = (D == 2) ? 1 : 2;
    const df64 E0 = c[0] + c[CSQ(D)] * dfc(X2) + (c[CSQ(T1)] + c[CSQ(T2)]) * dfc(A_);
    const df64 E1 = c[CLIN(T1)] * dfc(GPT) + c[CCUBE(T1)] * dfc(B_) + c[CM(D, T1)] * dfc(X2 * GPT) +
                    c[CM(T2, T1)] * dfc(A_ * GPT);
    const df64 E2 = c[CLIN(T2)] * dfc(GPT) + c[CCUBE(T2)] * dfc(B_) + c[CM(D, T2)] * dfc(X2 * GPT) +
                    c[CM(T1, T2)] * dfc(A_ * GPT);
    const df64 E12 = c[CCROSS(T1, T2)] * dfc(G2);
    const df64 O0 = df_half(c[CLIN(D)]) + c[CCUBE(D)] * dfc(X3) + (c[CM(T1, D)] + c[CM(T2, D)]) * dfc(0.5 * A_);
    const df64 O1 = c[CCROSS(D, T1)] * dfc(0.5 * GPT);
    const df64 O2 = c[CCROSS(D, T2)] * dfc(0.5 * GPT);
    const df64 O12 = c[19] * dfc(0.5 * G2);
#pragma unroll
    for (int sn = 0; sn < 2; ++sn) {
        const df64 A = sn ? E0 + O0 : E0 - O0;
        const df64 B1 = sn ? E1 + O1 : E1 - O1;
        const df64 B2 = sn ? E2 + O2 : E2 - O2;
        const df64 B12 = sn ? E12 + O12 : E12 - O12;
        const df64 am = A - B1, ap = A + B1;
        const df64 bm = B2 - B12, bp = B2 + B12;
        out[4 * sn + 0] = am - bm;
        out[4 * sn + 1] = am + bm;
        out[4 * sn + 2] = ap - bp;
        out[4 * sn + 3] = ap + bp;
    }
}

// ---------------------------------------------------------------- viscous fluxes in double-float
// face_grad / fg_eval / visc_flux of euler_kernels.cuh on pairs: the gradient of the R4
// polynomial (coefficients of the deviations, times 1/h) on a face side as P + Q t1 + R t2 + S t1 t2
struct FaceGradDf {
    df64 p, q, r, s;
};

template <int D, int NS, int EX, int EY, int EZ>
__device__ __forceinline__ void fg_term_df(FaceGradDf& f, df64 c, double k) {
    constexpr int eD = D == 0 ? EX : (D == 1 ? EY : EZ);
    constexpr int e1 = D == 0 ? EY : EX, e2 = D == 2 ? EY : EZ;
    constexpr double n = 0.5 * NS;
    constexpr double nf = eD == 0 ? 1.0 : (eD == 1 ? n : n * n);
    if constexpr (e1 == 2 || e2 == 2) f.p = f.p + c * dfc(k * (nf * G2));
    else if constexpr (e1 == 0 && e2 == 0) f.p = f.p + c * dfc(k * nf);
    else if constexpr (e1 == 1 && e2 == 0) f.q = f.q + c * dfc(k * nf);
    else if constexpr (e1 == 0 && e2 == 1) f.r = f.r + c * dfc(k * nf);
    else f.s = f.s + c * dfc(k * nf);
}

template <int D, int NS, int B>
__device__ __forceinline__ FaceGradDf face_grad_df(const df64* __restrict__ p, long long st) {
    auto C = [&](int q) { return p[q * st]; };
    const df64 z{0.0f, 0.0f};
    FaceGradDf f{z, z, z, z};
    if constexpr (B == 0) {
        fg_term_df<D, NS, 0, 0, 0>(f, C(1), 1.0);
        fg_term_df<D, NS, 1, 0, 0>(f, C(4), 2.0);
        fg_term_df<D, NS, 0, 1, 0>(f, C(7), 1.0);
        fg_term_df<D, NS, 0, 0, 1>(f, C(9), 1.0);
        const df64 c10 = C(10), c14 = C(14), c18 = C(18);
        fg_term_df<D, NS, 2, 0, 0>(f, c10, 3.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c10, -R3_20);
        fg_term_df<D, NS, 1, 1, 0>(f, C(13), 2.0);
        fg_term_df<D, NS, 0, 2, 0>(f, c14, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c14, -R1_12);
        fg_term_df<D, NS, 1, 0, 1>(f, C(17), 2.0);
        fg_term_df<D, NS, 0, 0, 2>(f, c18, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c18, -R1_12);
        fg_term_df<D, NS, 0, 1, 1>(f, C(19), 1.0);
    } else if constexpr (B == 1) {
        fg_term_df<D, NS, 0, 0, 0>(f, C(2), 1.0);
        fg_term_df<D, NS, 0, 1, 0>(f, C(5), 2.0);
        fg_term_df<D, NS, 1, 0, 0>(f, C(7), 1.0);
        fg_term_df<D, NS, 0, 0, 1>(f, C(8), 1.0);
        const df64 c11 = C(11), c13 = C(13), c16 = C(16);
        fg_term_df<D, NS, 0, 2, 0>(f, c11, 3.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c11, -R3_20);
        fg_term_df<D, NS, 2, 0, 0>(f, c13, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c13, -R1_12);
        fg_term_df<D, NS, 1, 1, 0>(f, C(14), 2.0);
        fg_term_df<D, NS, 0, 1, 1>(f, C(15), 2.0);
        fg_term_df<D, NS, 0, 0, 2>(f, c16, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c16, -R1_12);
        fg_term_df<D, NS, 1, 0, 1>(f, C(19), 1.0);
    } else {
        fg_term_df<D, NS, 0, 0, 0>(f, C(3), 1.0);
        fg_term_df<D, NS, 0, 0, 1>(f, C(6), 2.0);
        fg_term_df<D, NS, 0, 1, 0>(f, C(8), 1.0);
        fg_term_df<D, NS, 1, 0, 0>(f, C(9), 1.0);
        const df64 c12 = C(12), c15 = C(15), c17 = C(17);
        fg_term_df<D, NS, 0, 0, 2>(f, c12, 3.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c12, -R3_20);
        fg_term_df<D, NS, 0, 2, 0>(f, c15, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c15, -R1_12);
        fg_term_df<D, NS, 0, 1, 1>(f, C(16), 2.0);
        fg_term_df<D, NS, 2, 0, 0>(f, c17, 1.0);
        fg_term_df<D, NS, 0, 0, 0>(f, c17, -R1_12);
        fg_term_df<D, NS, 1, 0, 1>(f, C(18), 2.0);
        fg_term_df<D, NS, 1, 1, 0>(f, C(19), 1.0);
    }
    return f;
}

template <int GP>
__device__ __forceinline__ df64 fg_eval_df(const FaceGradDf& f) {
    constexpr double s1 = (GP & 2) ? GPT : -GPT, s2 = (GP & 1) ? GPT : -GPT;
    return (f.p + f.q * dfc(s1)) + (f.r * dfc(s2) + f.s * dfc(s1 * s2));
}

// PDEViscFlux (Navier-Stokes-3D/pde.c:90-162) as visc_flux: Q the full state (r + deviation),
// G its gradients; every flux term is a product with a gradient, so the flux has the size of
// the deviations and F(r) = 0; returns vmax / rho
template <int D>
__device__ __forceinline__ df64 visc_flux_df(const df64* Q, const df64 (*G)[3], df64 gm1, df64 mu, df64 kc, df64 vmax,
                                             df64* F) {
    const df64 irho = df_div(dfc(1.0), Q[0]);
    const df64 u = irho * Q[1], v = irho * Q[2], w = irho * Q[3];
    const df64 m2 = (Q[1] * Q[1] + Q[2] * Q[2]) + Q[3] * Q[3];
    const df64 em = Q[4] - m2 * irho;  // E - |m|^2 / rho
    df64 vg[3][3], T[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const df64 rb = G[0][b] * irho;
        vg[0][b] = G[1][b] - u * rb;
        vg[1][b] = G[2][b] - v * rb;
        vg[2][b] = G[3][b] - w * rb;
        // the temperature gradient (times c_v) of pde.c:118-130, regrouped:
        // (gamma - 1)/rho (E_b - u.m_b - rho_b/rho (E - |m|^2 / rho))
        const df64 um = (u * G[1][b] + v * G[2][b]) + w * G[3][b];
        T[b] = ((G[4][b] - um) - rb * em) * (gm1 * irho);
    }
    const df64 div_v = ((vg[0][0] + vg[1][1]) + vg[2][2]) * (mu * dfc(-2.0 / 3.0));
    const df64 tdd = div_v + df_scale(mu * vg[D][D], 2.0f);
    const df64 t0 = D == 0 ? tdd : mu * (vg[0][D] + vg[D][0]);
    const df64 t1 = D == 1 ? tdd : mu * (vg[1][D] + vg[D][1]);
    const df64 t2 = D == 2 ? tdd : mu * (vg[2][D] + vg[D][2]);
    F[0] = df64{0.0f, 0.0f};
    F[1] = -t0;
    F[2] = -t1;
    F[3] = -t2;
    F[4] = -(((u * t0 + v * t1) + w * t2) + kc * T[D]);
    return vmax * irho;
}

}  // namespace euler
}  // namespace hype
