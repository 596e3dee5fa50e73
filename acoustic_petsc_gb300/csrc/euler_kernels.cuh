// euler_kernels.cuh -- device arithmetic of the 3D Euler CWENO4 + Rusanov RHS.
//
// The per-cell mathematics follows the reference:
//   weno()               3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259
//   evaluate_polynomial  3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:12-21
//   PDEConsFlux / LLF    3d/weno4/Navier-Stokes-3D/pde.c:40-88, 164-187
// It is written for the GPU: the 33-point stencil lives in registers, the
// 24 face-Gauss-point traces per variable come from an even/odd split of the
// polynomial at the symmetric Gauss points (about 40 operations per direction
// instead of 8 full 20-term evaluations), and the arithmetic type R is a
// template parameter (double: the FP64 path; float: the FP32 recon/flux form).
#pragma once

#include "df64.cuh"
#include "hype_common.cuh"

namespace hype {
namespace euler {

// 1/x to about 1 ulp of FP32 (one MUFU instruction): the FP32 form's weight ratios and face-solver
// reciprocals, where the correctly rounded division's longer instruction sequence would cost more
// than the form's own rounding; x positive and in the normal range (on the host: the division)
__host__ __device__ __forceinline__ float rcp_fast(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return 1.0f / x;
#endif
}

// 1/x for the FP64 CWENO4 weights, whose magnitudes (products of (IS + 1e-12)^2, sums of their inverse
// squares) lie far outside the FP32 range: x is rebased to [1, 2), the approximate FP32 reciprocal of its
// leading bits is scaled back by 2^(1023 - e) on the integer pipe and refined by two FP64 Newton steps
// (relative error 2^-23, 2^-46, then FP64 rounding: within an ulp of the quotient), four FP64 operations
// against the correctly rounded division's longer sequence.  Biased exponent outside [2, 2044] (zero,
// subnormal, a reciprocal that would be subnormal, infinities, NaN): the division.  On the host: the division.
__host__ __device__ __forceinline__ double recip_wide(double x) {
#ifdef __CUDA_ARCH__
    const unsigned hi = (unsigned)__double2hiint(x);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    if (ex - 2u > 2042u) return 1.0 / x;
    const float mf = __uint_as_float((hi & 0x80000000u) | (127u << 23) | ((hi & 0xFFFFFu) << 3));
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(mf));
    double r = df_f2d(rf);
    r = __hiloint2double(__double2hiint(r) - ((int)ex - 1023) * (1 << 20), __double2loint(r));
    r = fma(r, fma(-x, r, 1.0), r);
    r = fma(r, fma(-x, r, 1.0), r);
    return r;
#else
    return 1.0 / x;
#endif
}

// 1/x for the face solvers: the approximate FP32 reciprocal (rcp.approx, ~1 ulp of FP32)
// of x's leading bits, refined by two Newton steps r <- r + r (1 - x r) in FP64 (the
// relative error squares at each: 2^-23, 2^-46, then FP64 rounding), four FP64 operations
// against the longer correctly rounded division; the bits move between the formats on the
// integer pipe.  x outside [2^-126, 2^126) in magnitude, zero or not finite: the division.
template <typename R>
__device__ __forceinline__ R recip(R x) {
    if (sizeof(R) != sizeof(double)) return (R)rcp_fast((float)x);
    const double xd = (double)x;
    const unsigned hi = (unsigned)__double2hiint(xd);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    if (ex - 897u > 251u) return R(1.0 / xd);
    const float xf = __uint_as_float((hi & 0x80000000u) | ((ex - 896u) << 23) | ((hi & 0xFFFFFu) << 3));
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(xf));
    double r = df_f2d(rf);
    r = fma(r, fma(-xd, r, 1.0), r);
    r = fma(r, fma(-xd, r, 1.0), r);
    return (R)r;
}

constexpr int NV = 5;
constexpr int NTR = 24;  // traces per cell and variable: face (0..5: -x,+x,-y,+y,-z,+z) x Gauss point (0..3)

// 33-point stencil index map: 0 centre; 1 + 4d + {0:-2,1:-1,2:+1,3:+2} along d;
// 13 + 4P + 2 s_lo + s_hi for the diagonal pair P (0: xy, 1: yz, 2: xz; s = 0 for -1, 1 for +1);
// 25 + 4 sx + 2 sy + sz for the body diagonals.
__host__ __device__ constexpr int S1(int d, int off) { return 1 + 4 * d + (off == -2 ? 0 : off == -1 ? 1 : off == 1 ? 2 : 3); }
__host__ __device__ constexpr int pair_of(int a, int b) { return (a + b == 1) ? 0 : (a + b == 3) ? 1 : 2; }
__host__ __device__ constexpr int SQ(int a, int sa, int b, int sb) {
    return a < b ? 13 + 4 * pair_of(a, b) + 2 * sa + sb : 13 + 4 * pair_of(a, b) + 2 * sb + sa;
}
__host__ __device__ constexpr int SO(int sx, int sy, int sz) { return 25 + 4 * sx + 2 * sy + sz; }

// polynomial coefficient indices (evaluate_polynomial term order)
__host__ __device__ constexpr int CLIN(int d) { return 1 + d; }
__host__ __device__ constexpr int CSQ(int d) { return 4 + d; }
__host__ __device__ constexpr int CCUBE(int d) { return 10 + d; }
__host__ __device__ constexpr int CCROSS(int a, int b) { return (a + b == 1) ? 7 : (a + b == 3) ? 8 : 9; }
// coefficient of (a^2 - 1/12) * b
__host__ __device__ constexpr int CM(int a, int b) {
    return (a == 0 && b == 1) ? 13 : (a == 1 && b == 0) ? 14 : (a == 1 && b == 2) ? 15 : (a == 2 && b == 1) ? 16
         : (a == 0 && b == 2) ? 17 : 18;
}

// Gauss point of the 2x2 face rule (hype.h:88-91) and the polynomial's basis
// values there, evaluated as evaluate_polynomial does.
constexpr double GPT = 0.28867513459481287;
constexpr double R1_12 = 1. / 12.;
constexpr double R3_20 = 3. / 20.;
constexpr double A_ = GPT * GPT - R1_12;        // (y^2 - 1/12) at y = +/-GPT
constexpr double B_ = GPT * (GPT * GPT - R3_20); // y (y^2 - 3/20) at y = +GPT
constexpr double X2 = 0.5 * 0.5 - R1_12;        // (x^2 - 1/12) at x = +/-1/2
constexpr double X3 = 0.5 * (0.5 * 0.5 - R3_20); // x (x^2 - 3/20) at x = +1/2
constexpr double G2 = GPT * GPT;

template <typename R>
struct Weights;



// CWENO4 coefficients (20) of one variable from its 33-point stencil.
// linear: the R4 polynomial (the limit in which all nonlinear weights equal the linear ones).
//
// The mathematics is the reference's weno() (3d/weno4/Viscous-Multiphase-Fourth-Order/
// reconstruction.c:38-259); the operation count is cut for the FP64 pipe, which bounds
// this kernel on GB300, with every value still formed in the working precision:
//  * per axis the differences a = u(+1) - u(-1), b = u(+2) - u(-2) and the sum
//    u(-1) + u(+1) serve the R4 first/second/third derivatives (:90-108) and the
//    centred R3 derivatives (:123-140);
//  * per axis pair the corner sums P = pp - mm, Q = mp - pm give the R4 cross term,
//    both mixed third derivatives and the centred R3 cross term (the same value as
//    the R4 one, :94-96 and :133-135);
//  * the squared sums shared by IS_R4 (:110-116) and IS_R3 of the centred stencil
//    (:205-213) are formed once;
//  * CWENO combination (:215-257): P = (w4/g4)(P4 - sum_k g_k P_k) + sum_k w_k P_k is
//    evaluated per coefficient as (w4/g4) c4 + sum_k (w_k - (w4/g4) g_k) c_k, one
//    weighted sum instead of a linear and a nonlinear one.
template <typename R>
__host__ __device__ __forceinline__ void cweno4(const R* __restrict__ s, bool linear, R* __restrict__ cf,
                                                R* wdev = nullptr) {
    const R u0 = s[0];
    const R h = R(0.5), q = R(0.25);
    R d4[3], dd4[3], ddd4[3], c1[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const R m2 = s[S1(d, -2)], m1 = s[S1(d, -1)], p1 = s[S1(d, 1)], p2 = s[S1(d, 2)];
        const R a = p1 - m1, b = p2 - m2;
        d4[d] = R(82. / 120.) * a - R(11. / 120.) * b;  // (11 m2 - 82 m1 + 82 p1 - 11 p2) / 120
        dd4[d] = h * (m1 + p1) - u0;                    // (m1 - 2 u0 + p1) / 2
        ddd4[d] = R(1. / 12.) * b - R(1. / 6.) * a;      // (-m2 + 2 (m1 - p1) + p2) / 12
        c1[d] = h * a;                                  // centred R3 first derivative
    }
#define QV(a, sa, b, sb) s[SQ(a, sa, b, sb)]
    // pairs 0: (x,y), 1: (y,z), 2: (x,z); corners mm, mp, pm, pp (first index: sign along a)
    R cx[3], aab[3], abb[3];
#pragma unroll
    for (int P = 0; P < 3; ++P) {
        const int a = P == 1 ? 1 : 0, b = P == 0 ? 1 : 2;
        const R mm = QV(a, 0, b, 0), mp = QV(a, 0, b, 1), pm = QV(a, 1, b, 0), pp = QV(a, 1, b, 1);
        const R Pd = pp - mm, Qd = mp - pm;
        cx[P] = q * ((mm + pp) - (mp + pm));  // u_ab
        aab[P] = q * (Pd + Qd) - c1[b];       // u_aab = 0.25 (-mm + mp - pm + pp) + 0.5 (u_b- - u_b+)
        abb[P] = q * (Pd - Qd) - c1[a];       // u_abb = 0.5 (u_a- - u_a+) + 0.25 (pp - mm - mp + pm)
    }
#undef QV
    const R xyz = R(0.125) * ((s[SO(1, 1, 1)] - s[SO(0, 0, 0)]) + ((s[SO(0, 0, 1)] + s[SO(0, 1, 0)] + s[SO(1, 0, 0)]) -
                                                                 (s[SO(0, 1, 1)] + s[SO(1, 0, 1)] + s[SO(1, 1, 0)])));
    cf[0] = u0;
    // the cubic part is the R4 one scaled by w4/g4 (1 in the linear limit)
    if (linear) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            cf[CLIN(d)] = d4[d];
            cf[CSQ(d)] = dd4[d];
            cf[CCUBE(d)] = ddd4[d];
        }
        cf[7] = cx[0]; cf[8] = cx[1]; cf[9] = cx[2];
        cf[13] = aab[0]; cf[14] = abb[0]; cf[15] = aab[1]; cf[16] = abb[1]; cf[17] = aab[2]; cf[18] = abb[2]; cf[19] = xyz;
        if (wdev) *wdev = R(0);
        return;
    }
    const R r13_3 = R(13. / 3.), r7_6 = R(7. / 6.);
    R c1sq[3], ddsq[3], cxsq[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c1sq[d] = c1[d] * c1[d];
        ddsq[d] = dd4[d] * dd4[d];
        cxsq[d] = cx[d] * cx[d];
    }
    const R common = r13_3 * (ddsq[0] + ddsq[1] + ddsq[2]) + r7_6 * (cxsq[0] + cxsq[1] + cxsq[2]);
    const R IS4 = d4[0] * (d4[0] + R(0.2) * ddd4[0]) + d4[1] * (d4[1] + R(0.2) * ddd4[1]) + d4[2] * (d4[2] + R(0.2) * ddd4[2]) +
                  common + R(4.7) * (aab[0] * aab[0] + abb[0] * abb[0] + aab[1] * aab[1] + abb[1] * abb[1] + aab[2] * aab[2] + abb[2] * abb[2]) +
                  R(39.06) * (ddd4[0] * ddd4[0] + ddd4[1] * ddd4[1] + ddd4[2] * ddd4[2]) + R(61. / 48.) * xyz * xyz;
    const R IS0 = (c1sq[0] + c1sq[1] + c1sq[2]) + common;
    // one-sided stencils: index 2d (towards +d) and 2d+1 (towards -d): first and second
    // derivative along d and the two cross terms that involve d
    R sd1[6], sd2[6], sx1[6], sx2[6], IS3[6];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int e1 = (d == 0) ? 1 : 0, e2 = (d == 2) ? 1 : 2;
        const int k1 = (d + e1 == 1) ? 0 : (d + e1 == 3) ? 1 : 2;  // cross slot of (d,e1)
        const int k2 = (d + e2 == 1) ? 0 : (d + e2 == 3) ? 1 : 2;  // cross slot of (d,e2)
        const R p1 = s[S1(d, 1)], p2 = s[S1(d, 2)], m1 = s[S1(d, -1)], m2 = s[S1(d, -2)];
        // towards +d: u_d = -1.5 u0 + 2 p1 - 0.5 p2, u_dd = 0.5 (u0 - 2 p1 + p2)
        sd2[2 * d] = h * (u0 + p2) - p1;
        sd1[2 * d] = (p1 - u0) - sd2[2 * d];
        sx1[2 * d] = h * (s[SQ(d, 1, e1, 1)] - s[SQ(d, 1, e1, 0)]) - c1[e1];
        sx2[2 * d] = h * (s[SQ(d, 1, e2, 1)] - s[SQ(d, 1, e2, 0)]) - c1[e2];
        // towards -d: u_d = -2 m1 + 0.5 m2 + 1.5 u0, u_dd = 0.5 (m2 - 2 m1 + u0)
        sd2[2 * d + 1] = h * (m2 + u0) - m1;
        sd1[2 * d + 1] = (u0 - m1) + sd2[2 * d + 1];
        sx1[2 * d + 1] = h * (s[SQ(d, 0, e1, 0)] - s[SQ(d, 0, e1, 1)]) + c1[e1];
        sx2[2 * d + 1] = h * (s[SQ(d, 0, e2, 0)] - s[SQ(d, 0, e2, 1)]) + c1[e2];
        // the unchanged terms are summed directly (no subtraction from the centred sums:
        // IS values near zero must keep their relative accuracy)
        const int k3 = 3 - k1 - k2;
        const R rest1 = c1sq[e1] + c1sq[e2];
        const R rest2 = ddsq[e1] + ddsq[e2];
        const R restx = cxsq[k3];
#pragma unroll
        for (int sg = 0; sg < 2; ++sg) {
            const int m = 2 * d + sg;
            const R a1 = rest1 + sd1[m] * sd1[m];
            const R a2 = rest2 + sd2[m] * sd2[m];
            const R a3 = restx + sx1[m] * sx1[m] + sx2[m] * sx2[m];
            IS3[m] = a1 + r13_3 * a2 + r7_6 * a3;
        }
    }
    // nonlinear weights: gammaHi = gammaLo = 0.85, p = 4, eps = 1e-12
    const R gH = R(0.85), g0 = R((1.0 - 0.85) * 0.85), gs = R((1. / 6.) * (1 - 0.85) * (1 - 0.85));
    R w4, w0, ws[6];
    Weights<R>::compute(IS4, IS0, IS3, gH, g0, gs, w4, w0, ws);
    // 1/gammaHi as a constant: a product, not a division
    const R wr = w4 * R(1.0 / 0.85);
    if (wdev) {  // largest departure of a nonlinear weight from its linear value (indicator labels)
        R d = fmax(fabs(w4 - gH), fabs(w0 - g0));
#pragma unroll
        for (int m = 0; m < 6; ++m) d = fmax(d, fabs(ws[m] - gs));
        *wdev = d;
    }
    // weights of the lower-order stencils' values in the combination: w_k - wr g_k
    const R o0 = w0 - wr * g0;
    R os[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) os[m] = ws[m] - wr * gs;
    const R ox = os[0] + os[1], oy = os[2] + os[3], oz = os[4] + os[5];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        // the centred values of direction d are kept by the centred stencil and by the
        // one-sided stencils of the two other directions
        const R okeep = o0 + ((d == 0) ? oy + oz : (d == 1) ? ox + oz : ox + oy);
        cf[CLIN(d)] = wr * d4[d] + okeep * c1[d] + os[2 * d] * sd1[2 * d] + os[2 * d + 1] * sd1[2 * d + 1];
        cf[CSQ(d)] = (wr + okeep) * dd4[d] + os[2 * d] * sd2[2 * d] + os[2 * d + 1] * sd2[2 * d + 1];
    }
    // cross terms: slot 0 (xy) is modified by the x-sided (via sx1 of d=0) and y-sided (sx1 of d=1) stencils,
    // slot 1 (yz) by y-sided (sx2 of d=1) and z-sided (sx2 of d=2), slot 2 (xz) by x-sided (sx2 of d=0) and z-sided (sx1 of d=2)
    cf[7] = (wr + o0 + oz) * cx[0] + os[0] * sx1[0] + os[1] * sx1[1] + os[2] * sx1[2] + os[3] * sx1[3];
    cf[8] = (wr + o0 + ox) * cx[1] + os[2] * sx2[2] + os[3] * sx2[3] + os[4] * sx2[4] + os[5] * sx2[5];
    cf[9] = (wr + o0 + oy) * cx[2] + os[0] * sx2[0] + os[1] * sx2[1] + os[4] * sx1[4] + os[5] * sx1[5];
#pragma unroll
    for (int d = 0; d < 3; ++d) cf[CCUBE(d)] = wr * ddd4[d];
    cf[13] = wr * aab[0]; cf[14] = wr * abb[0]; cf[15] = wr * aab[1]; cf[16] = wr * abb[1];
    cf[17] = wr * aab[2]; cf[18] = wr * abb[2]; cf[19] = wr * xyz;
}

// w = gamma / (IS + eps)^4, normalised.  FP64: the eight reciprocals 1/(IS + eps)^2
// come from one reciprocal of their product (prefix products, then back-substitution:
// 21 multiplications instead of 7 more reciprocals); a product outside the normal
// range (IS beyond ~1e36) takes the plain reciprocals instead.  Reciprocals by recip_wide
// (within an ulp of the division, on a fraction of its FP64 instructions).
template <>
struct Weights<double> {
    __host__ __device__ __forceinline__ static void compute(double IS4, double IS0, const double* IS3, double gH, double g0, double gs,
                                                   double& w4, double& w0, double* ws) {
        double q[8], P[8], r[8];
        q[0] = IS4 + 1.0e-12;
        q[1] = IS0 + 1.0e-12;
#pragma unroll
        for (int m = 0; m < 6; ++m) q[2 + m] = IS3[m] + 1.0e-12;
#pragma unroll
        for (int k = 0; k < 8; ++k) q[k] *= q[k];
        P[0] = q[0];
#pragma unroll
        for (int k = 1; k < 8; ++k) P[k] = P[k - 1] * q[k];
        if (P[7] > 1.0e-290 && P[7] < 1.0e290) {
            double inv = recip_wide(P[7]);
#pragma unroll
            for (int k = 7; k > 0; --k) {
                r[k] = inv * P[k - 1];
                inv *= q[k];
            }
            r[0] = inv;
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) r[k] = recip_wide(q[k]);
        }
        w4 = gH * (r[0] * r[0]);
        w0 = g0 * (r[1] * r[1]);
        double total = w4 + w0;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            ws[m] = gs * (r[2 + m] * r[2 + m]);
            total += ws[m];
        }
        const double rt = recip_wide(total);
        w4 *= rt;
        w0 *= rt;
#pragma unroll
        for (int m = 0; m < 6; ++m) ws[m] *= rt;
    }
};

// FP32: (1e-12)^4 underflows, so the weights are formed from ratios to the
// smallest (IS + eps), which is the same normalised quantity.
template <>
struct Weights<float> {
    __host__ __device__ __forceinline__ static void compute(float IS4, float IS0, const float* IS3, float gH, float g0, float gs,
                                                   float& w4, float& w0, float* ws) {
        float s4 = IS4 + 1.0e-12f, s0 = IS0 + 1.0e-12f, ss[6];
        float mn = fminf(s4, s0);
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            ss[m] = IS3[m] + 1.0e-12f;
            mn = fminf(mn, ss[m]);
        }
        float r = mn * rcp_fast(s4);
        r *= r;
        w4 = gH * r * r;
        r = mn * rcp_fast(s0);
        r *= r;
        w0 = g0 * r * r;
        float total = w4 + w0;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            r = mn * rcp_fast(ss[m]);
            r *= r;
            ws[m] = gs * r * r;
            total += ws[m];
        }
        const float inv = rcp_fast(total);
        w4 *= inv;
        w0 *= inv;
#pragma unroll
        for (int m = 0; m < 6; ++m) ws[m] *= inv;
    }
};

// Normalised WENO weights w_m = gam_m / (IS_m + eps)^4 / sum, eps = 1e-12.  FP64:
// directly, as 3d/weno3/Euler/reconstruction.c:60-67 does; FP32: from ratios to the
// smallest IS + eps, because (1e-12)^4 underflows.
template <typename R, int M>
__device__ __forceinline__ void weno_weights(const R* IS, const R* gam, R* w) {
    if (sizeof(R) == sizeof(double)) {
        R total = R(0);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            R t = IS[m] + R(1.0e-12);
            t *= t;
            w[m] = gam[m] / (t * t);
            total += w[m];
        }
        const R r = R(1) / total;
#pragma unroll
        for (int m = 0; m < M; ++m) w[m] *= r;
    } else {
        R mn = IS[0] + R(1.0e-12);
#pragma unroll
        for (int m = 1; m < M; ++m) mn = fmin(mn, IS[m] + R(1.0e-12));
        R total = R(0);
#pragma unroll
        for (int m = 0; m < M; ++m) {
            R r = mn / (IS[m] + R(1.0e-12));
            r *= r;
            w[m] = gam[m] * r * r;
            total += w[m];
        }
        const R inv = R(1) / total;
#pragma unroll
        for (int m = 0; m < M; ++m) w[m] *= inv;
    }
}

// Third-order WENO coefficients (the first 10 of the 20-term basis; the cubic ones
// are zero) of one variable from the 25 axis and face-diagonal points of its
// 33-point stencil, following 3d/weno3/Euler/reconstruction.c:29-177: per axis the
// three one-sided/central quadratics with linear weights 1 : 100 : 1 (:54-106),
// then per axis pair the four corner-based cross terms with equal weights (:108-163).
template <typename R>
__device__ __forceinline__ void weno3(const R* __restrict__ s, R* __restrict__ cf) {
    const R u0 = s[0];
    cf[0] = u0;
    const R h = R(0.5), r13_3 = R(13. / 3.);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const R m2 = s[S1(d, -2)], m1 = s[S1(d, -1)], p1 = s[S1(d, 1)], p2 = s[S1(d, 2)];
        R ux[3], uxx[3], IS[3], w[3];
        ux[0] = R(-2.0) * m1 + h * m2 + R(1.5) * u0;
        uxx[0] = h * (m2 - R(2.0) * m1 + u0);
        ux[1] = h * (p1 - m1);
        uxx[1] = h * (m1 - R(2.0) * u0 + p1);
        ux[2] = R(-1.5) * u0 + R(2.0) * p1 - h * p2;
        uxx[2] = h * (u0 - R(2.0) * p1 + p2);
#pragma unroll
        for (int m = 0; m < 3; ++m) IS[m] = ux[m] * ux[m] + r13_3 * uxx[m] * uxx[m];
        const R gam[3] = {R(1), R(100), R(1)};
        weno_weights<R, 3>(IS, gam, w);
        cf[CLIN(d)] = w[0] * ux[0] + w[1] * ux[1] + w[2] * ux[2];
        cf[CSQ(d)] = w[0] * uxx[0] + w[1] * uxx[1] + w[2] * uxx[2];
    }
    // cross terms of the pairs (x,y) -> 7, (y,z) -> 8, (z,x) -> 9
#pragma unroll
    for (int P = 0; P < 3; ++P) {
        const int a = P == 0 ? 0 : P == 1 ? 1 : 2, b = P == 0 ? 1 : P == 1 ? 2 : 0;
        const R pp = s[SQ(a, 1, b, 1)], pm = s[SQ(a, 1, b, 0)], mp = s[SQ(a, 0, b, 1)], mm = s[SQ(a, 0, b, 0)];
        const R ca = cf[CLIN(a)], cb = cf[CLIN(b)], caa = cf[CSQ(a)], cbb = cf[CSQ(b)];
        R u[4], IS[4], w[4];
        u[0] = pp - u0 - ca - cb - caa - cbb;
        u[1] = -pm + u0 + ca - cb + caa + cbb;
        u[2] = -mp + u0 - ca + cb + caa + cbb;
        u[3] = mm - u0 + ca + cb - caa - cbb;
        const R temp = R(4.0) * (caa * caa + cbb * cbb);
#pragma unroll
        for (int m = 0; m < 4; ++m) IS[m] = temp + u[m] * u[m];
        const R gam[4] = {R(1), R(1), R(1), R(1)};
        weno_weights<R, 4>(IS, gam, w);
        cf[7 + P] = w[0] * u[0] + w[1] * u[1] + w[2] * u[2] + w[3] * u[3];
    }
#pragma unroll
    for (int q = 10; q < 20; ++q) cf[q] = R(0);
}

// The 8 traces of the two faces normal to d (4 Gauss points each) from the
// coefficients: even/odd split of the polynomial in the normal coordinate.
// out[0..3]: face -d, out[4..7]: face +d; Gauss point g = 2*(t1>0) + (t2>0)
// with (t1,t2) = (y,z), (x,z), (x,y) for d = x, y, z.
template <typename R, int D>
__device__ __forceinline__ void face_traces(const R* __restrict__ c, R* __restrict__ out) {
    constexpr int T1 = (D == 0) ? 1 : 0;
    constexpr int T2 = (D == 2) ? 1 : 2;
    const R G = R(GPT);
    const R E0 = c[0] + c[CSQ(D)] * R(X2) + (c[CSQ(T1)] + c[CSQ(T2)]) * R(A_);
    const R E1 = c[CLIN(T1)] * G + c[CCUBE(T1)] * R(B_) + c[CM(D, T1)] * R(X2 * GPT) + c[CM(T2, T1)] * R(A_ * GPT);
    const R E2 = c[CLIN(T2)] * G + c[CCUBE(T2)] * R(B_) + c[CM(D, T2)] * R(X2 * GPT) + c[CM(T1, T2)] * R(A_ * GPT);
    const R E12 = c[CCROSS(T1, T2)] * R(G2);
    const R O0 = R(0.5) * c[CLIN(D)] + R(X3) * c[CCUBE(D)] + R(0.5 * A_) * (c[CM(T1, D)] + c[CM(T2, D)]);
    const R O1 = R(0.5 * GPT) * c[CCROSS(D, T1)];
    const R O2 = R(0.5 * GPT) * c[CCROSS(D, T2)];
    const R O12 = R(0.5 * G2) * c[19];
#pragma unroll
    for (int sn = 0; sn < 2; ++sn) {
        const R A = sn ? E0 + O0 : E0 - O0;
        const R B1 = sn ? E1 + O1 : E1 - O1;
        const R B2 = sn ? E2 + O2 : E2 - O2;
        const R B12 = sn ? E12 + O12 : E12 - O12;
        const R am = A - B1, ap = A + B1;     // t1 = -, +
        const R bm = B2 - B12, bp = B2 + B12; // coefficient of s2 for t1 = -, +
        out[4 * sn + 0] = am - bm;
        out[4 * sn + 1] = am + bm;
        out[4 * sn + 2] = ap - bp;
        out[4 * sn + 3] = ap + bp;
    }
}

// Rusanov (LLF) flux across an axis face of normal D; returns the max wave
// speed and flags an inadmissible state (rho < 1e-14 or p < 1e-12).
// HALF = false leaves out the factor 1/2 (the caller folds it into its quadrature weight)
template <typename R, int D, bool HALF = true>
__device__ __forceinline__ R rusanov(const R* QL, const R* QR, R gamma, R gm1, R* F, bool& bad) {
    R FL[NV], FR[NV], sL, sR;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const R* Q = side ? QR : QL;
        R* Fo = side ? FR : FL;
        const R rho = Q[0];
        const R ir = recip(rho);
        const R u = ir * Q[1], v = ir * Q[2], w = ir * Q[3];
        const R E = Q[4];
        // 0.5 rho |u|^2 as 0.5 (m . u); the floors rho >= 1e-14, p >= 1e-12 (a NaN fails both)
        const R p = gm1 * (E - R(0.5) * (Q[1] * u + Q[2] * v + Q[3] * w));
        bad |= !(rho >= R(1.0e-14) && p >= R(1.0e-12));
        const R un = (D == 0) ? u : (D == 1) ? v : w;
        const R mun = Q[1 + D];
        Fo[0] = mun;
        Fo[1] = mun * u + ((D == 0) ? p : R(0));
        Fo[2] = mun * v + ((D == 1) ? p : R(0));
        Fo[3] = mun * w + ((D == 2) ? p : R(0));
        Fo[4] = (E + p) * un;
        // sound speed sqrt(gamma p / rho) as x rsqrt(x): it only scales the dissipation
        // s (QR - QL) and sets dt, where a last-bit difference is immaterial
        const R x = ir * gamma * p;
        const R a = x * rsqrt(x);
        (side ? sR : sL) = fabs(un) + a;
    }
    const R s = sL < sR ? sR : sL;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        const R f = FR[c] + FL[c] - s * (QR[c] - QL[c]);
        F[c] = HALF ? R(0.5) * f : f;
    }
    return s;
}

// ---------------------------------------------------------------- viscous fluxes
// The gradient of a cell's R4 polynomial on one of its faces (normal axis D, side
// NS = +1 for the high face x_D = +1/2, -1 for the low face) is, in the two
// tangential coordinates, g(t1, t2) = P + Q t1 + R t2 + S t1 t2 once the squares
// t1^2 = t2^2 = GPT^2 of the 2x2 Gauss points are folded into P (the gradient of
// evaluate_grad, Navier-Stokes-3D/reconstruction.c:24-35, at the face points of
// rhs_function.c:224-270).  Built once per face side from the coefficients, it costs
// 3 FMAs per Gauss point.  The tangential axes are the two other axes in increasing
// order, as for the traces.
struct FaceGrad {
    double p, q, r, s;
};

// adds c k x^EX y^EY z^EZ to f
template <int D, int NS, int EX, int EY, int EZ>
__device__ __forceinline__ void fg_term(FaceGrad& f, double c, double k) {
    constexpr int eD = D == 0 ? EX : (D == 1 ? EY : EZ);
    constexpr int e1 = D == 0 ? EY : EX, e2 = D == 2 ? EY : EZ;
    constexpr double n = 0.5 * NS;
    constexpr double nf = eD == 0 ? 1.0 : (eD == 1 ? n : n * n);
    if constexpr (e1 == 2 || e2 == 2) f.p = fma(c, k * (nf * G2), f.p);
    else if constexpr (e1 == 0 && e2 == 0) f.p = fma(c, k * nf, f.p);
    else if constexpr (e1 == 1 && e2 == 0) f.q = fma(c, k * nf, f.q);
    else if constexpr (e1 == 0 && e2 == 1) f.r = fma(c, k * nf, f.r);
    else f.s = fma(c, k * nf, f.s);
}

// component B of the gradient of the 20-term polynomial whose coefficient q is at p[q * st]
template <int D, int NS, int B>
__device__ __forceinline__ FaceGrad face_grad(const double* __restrict__ p, long long st) {
    auto C = [&](int q) { return __ldg(p + q * st); };
    FaceGrad f{0.0, 0.0, 0.0, 0.0};
    if constexpr (B == 0) {  // d/dx
        fg_term<D, NS, 0, 0, 0>(f, C(1), 1.0);
        fg_term<D, NS, 1, 0, 0>(f, C(4), 2.0);
        fg_term<D, NS, 0, 1, 0>(f, C(7), 1.0);
        fg_term<D, NS, 0, 0, 1>(f, C(9), 1.0);
        const double c10 = C(10), c14 = C(14), c18 = C(18);
        fg_term<D, NS, 2, 0, 0>(f, c10, 3.0);
        fg_term<D, NS, 0, 0, 0>(f, c10, -R3_20);
        fg_term<D, NS, 1, 1, 0>(f, C(13), 2.0);
        fg_term<D, NS, 0, 2, 0>(f, c14, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c14, -R1_12);
        fg_term<D, NS, 1, 0, 1>(f, C(17), 2.0);
        fg_term<D, NS, 0, 0, 2>(f, c18, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c18, -R1_12);
        fg_term<D, NS, 0, 1, 1>(f, C(19), 1.0);
    } else if constexpr (B == 1) {  // d/dy
        fg_term<D, NS, 0, 0, 0>(f, C(2), 1.0);
        fg_term<D, NS, 0, 1, 0>(f, C(5), 2.0);
        fg_term<D, NS, 1, 0, 0>(f, C(7), 1.0);
        fg_term<D, NS, 0, 0, 1>(f, C(8), 1.0);
        const double c11 = C(11), c13 = C(13), c16 = C(16);
        fg_term<D, NS, 0, 2, 0>(f, c11, 3.0);
        fg_term<D, NS, 0, 0, 0>(f, c11, -R3_20);
        fg_term<D, NS, 2, 0, 0>(f, c13, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c13, -R1_12);
        fg_term<D, NS, 1, 1, 0>(f, C(14), 2.0);
        fg_term<D, NS, 0, 1, 1>(f, C(15), 2.0);
        fg_term<D, NS, 0, 0, 2>(f, c16, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c16, -R1_12);
        fg_term<D, NS, 1, 0, 1>(f, C(19), 1.0);
    } else {  // d/dz
        fg_term<D, NS, 0, 0, 0>(f, C(3), 1.0);
        fg_term<D, NS, 0, 0, 1>(f, C(6), 2.0);
        fg_term<D, NS, 0, 1, 0>(f, C(8), 1.0);
        fg_term<D, NS, 1, 0, 0>(f, C(9), 1.0);
        const double c12 = C(12), c15 = C(15), c17 = C(17);
        fg_term<D, NS, 0, 0, 2>(f, c12, 3.0);
        fg_term<D, NS, 0, 0, 0>(f, c12, -R3_20);
        fg_term<D, NS, 0, 2, 0>(f, c15, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c15, -R1_12);
        fg_term<D, NS, 0, 1, 1>(f, C(16), 2.0);
        fg_term<D, NS, 2, 0, 0>(f, c17, 1.0);
        fg_term<D, NS, 0, 0, 0>(f, c17, -R1_12);
        fg_term<D, NS, 1, 0, 1>(f, C(18), 2.0);
        fg_term<D, NS, 1, 1, 0>(f, C(19), 1.0);
    }
    return f;
}

// the value at Gauss point gp (t1 = -/+GPT for gp & 2, t2 = -/+GPT for gp & 1)
template <int GP>
__device__ __forceinline__ double fg_eval(const FaceGrad& f) {
    constexpr double s1 = (GP & 2) ? GPT : -GPT, s2 = (GP & 1) ? GPT : -GPT;
    return fma(f.s, s1 * s2, fma(f.r, s2, fma(f.q, s1, f.p)));
}

// PDEViscFlux (3d/weno4/Navier-Stokes-3D/pde.c:90-162) across a face of normal axis D:
// Newtonian stress with Stokes' hypothesis and Fourier heat flux k = Cv mu gamma / Pr,
// with the program's velocity gradients u_x = (rho u)_x - u rho_x / rho (:118-130);
// returns the viscous speed max(4 mu / (3 rho), gamma mu / (Pr rho))
template <int D>
__device__ __forceinline__ double visc_flux(const double* Q, const double (*G)[3], double gm1, double mu, double kc,
                                            double vmax, double* F) {
    // kc = cv mu gamma / Pr (heat conductivity), vmax = max(4 mu / 3, gamma mu / Pr); the
    // divisions by rho of the reference's expressions are products with 1/rho here
    const double irho = 1.0 / Q[0];
    const double u = irho * Q[1], v = irho * Q[2], w = irho * Q[3];
    const double rhou = Q[1], rhov = Q[2], rhow = Q[3], e = Q[4];
    const double m2 = rhou * rhou + rhov * rhov + rhow * rhow;
    double vg[3][3], T[3];  // vg[a][b]: d(velocity a)/d(x_b)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const double rb = G[0][b] * irho;
        vg[0][b] = G[1][b] - u * rb;
        vg[1][b] = G[2][b] - v * rb;
        vg[2][b] = G[3][b] - w * rb;
        T[b] = (-gm1 * rb * irho) * (e - 0.5 * m2 * irho) +
               (gm1 * irho) * (G[4][b] - (rhou * G[1][b] + rhov * G[2][b] + rhow * G[3][b]) * irho +
                               0.5 * m2 * rb * irho);
    }
    const double div_v = -(2.0 / 3.0) * mu * (vg[0][0] + vg[1][1] + vg[2][2]);
    const double tdd = div_v + 2.0 * mu * vg[D][D];                  // tau_DD
    const double t0 = D == 0 ? tdd : mu * (vg[0][D] + vg[D][0]);     // tau_xD
    const double t1 = D == 1 ? tdd : mu * (vg[1][D] + vg[D][1]);     // tau_yD
    const double t2 = D == 2 ? tdd : mu * (vg[2][D] + vg[D][2]);     // tau_zD
    F[0] = 0.0;
    F[1] = -t0;
    F[2] = -t1;
    F[3] = -t2;
    F[4] = -(u * t0 + v * t1 + w * t2 + kc * T[D]);
    return vmax * irho;
}

// ---------------------------------------------------------------- HLLC family
// Miller-Colella tangents (pde.c:236-251; 'fixed' = the corrected t2z of pde.c:348).  RT: the
// normal is data (rsqrt); otherwise a compile-time axis, for which 1/sqrt folds to a constant.
template <typename R, bool RT = false>
__device__ __forceinline__ void mc_tangents(R nx, R ny, R nz, bool fixed, R* t1, R* t2) {
    auto inv_sqrt = [](R x) { return RT ? rsqrt(x) : R(1) / sqrt(x); };
    if (fabs(ny + nz) > fabs(ny - nz)) {
        const R iL = inv_sqrt(R(2) * (R(1) + nz * (ny - nx) + nx * ny));
        t1[0] = (ny + nz) * iL; t1[1] = (nz - nx) * iL; t1[2] = -(nx + ny) * iL;
        t2[0] = (nx * (nz - ny) - ny * ny - nz * nz) * iL;
        t2[1] = (ny * (nx + nz) + nx * nx + nz * nz) * iL;
        t2[2] = (fixed ? (nz * (nx - ny) - nx * nx - ny * ny) : (nz * (nx - nz) - nx * nx - ny * ny)) * iL;
    } else {
        const R iL = inv_sqrt(R(2) * (R(1) - nx * ny - nx * nz - ny * nz));
        t1[0] = (ny - nz) * iL; t1[1] = (nz - nx) * iL; t1[2] = (nx - ny) * iL;
        t2[0] = (nx * (ny + nz) - ny * ny - nz * nz) * iL;
        t2[1] = (ny * (nx + nz) - nx * nx - nz * nz) * iL;
        t2[2] = (nz * (nx + ny) - nx * nx - ny * ny) * iL;
    }
}

// PDEHLLCRiemannSolver (pde.c:207-322): star states built in the (n, t1, t2)
// frame and rotated back with the inverse frame matrix
// One side of a face for the HLLC family: what PDEConsFlux derives from the conserved
// trace that does not depend on the normal -- 1/rho, velocity, pressure, sound speed --
// formed once per trace (the rotated solver makes three HLLC evaluations)
template <typename R>
struct HSide {
    R rho, u, v, w, p, E, ir, c;
};

template <typename R>
__device__ __forceinline__ HSide<R> hllc_side(const R* Q, R gamma, R gm1, bool& bad) {
    HSide<R> s;
    s.rho = Q[0];
    s.ir = recip(Q[0]);
    s.u = s.ir * Q[1]; s.v = s.ir * Q[2]; s.w = s.ir * Q[3];
    s.E = Q[4];
    s.p = gm1 * (Q[4] - R(0.5) * Q[0] * (s.u * s.u + s.v * s.v + s.w * s.w));
    bad |= (Q[0] < R(1.0e-14)) || (s.p < R(1.0e-12)) || !(Q[0] == Q[0]);
    s.c = sqrt(s.ir * gamma * s.p);
    return s;
}

// PDEHLLCRiemannSolver (pde.c:207-322) for the unit normal n from the two sides: star states
// built in the (n, t1, t2) frame and rotated back with the inverse frame matrix
template <typename R, bool RT = false>
__device__ __forceinline__ R hllc_sides(const HSide<R>* side, const R* QL, const R* QR, R nx, R ny, R nz, R* Flux) {
    R t1[3], t2[3];
    mc_tangents<R, RT>(nx, ny, nz, false, t1, t2);
    // inverse of the frame matrix [n; t1; t2] by cofactors (pde.c:189-205; constant for an axis normal)
    const R M00 = nx, M01 = ny, M02 = nz, M10 = t1[0], M11 = t1[1], M12 = t1[2], M20 = t2[0], M21 = t2[1], M22 = t2[2];
    const R idet = recip(M00 * (M11 * M22 - M12 * M21) - M01 * (M10 * M22 - M12 * M20) + M02 * (M10 * M21 - M11 * M20));
    const R i00 = (M11 * M22 - M12 * M21) * idet, i01 = -(M01 * M22 - M02 * M21) * idet, i02 = (M01 * M12 - M02 * M11) * idet;
    const R i10 = -(M10 * M22 - M12 * M20) * idet, i11 = (M00 * M22 - M02 * M20) * idet, i12 = -(M00 * M12 - M02 * M10) * idet;
    const R i20 = (M10 * M21 - M11 * M20) * idet, i21 = -(M00 * M21 - M01 * M20) * idet, i22 = (M00 * M11 - M01 * M10) * idet;
    R F[2][NV], un[2], ut1[2], ut2[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const HSide<R>& s = side[k];
        un[k] = nx * s.u + ny * s.v + nz * s.w;
        ut1[k] = s.u * t1[0] + s.v * t1[1] + s.w * t1[2];
        ut2[k] = s.u * t2[0] + s.v * t2[1] + s.w * t2[2];
        const R mun = s.rho * un[k];
        F[k][0] = mun;
        F[k][1] = mun * s.u + nx * s.p;
        F[k][2] = mun * s.v + ny * s.p;
        F[k][3] = mun * s.w + nz * s.p;
        F[k][4] = (s.E + s.p) * un[k];
    }
    const R SL = fmin(un[1] - side[1].c, un[0] - side[0].c);
    const R SR = fmax(un[0] + side[0].c, un[1] + side[1].c);
    const R S[2] = {SL, SR};
    const R Ss = (side[1].p - side[0].p + side[0].rho * un[0] * (SL - un[0]) - side[1].rho * un[1] * (SR - un[1])) *
                 recip(side[0].rho * (SL - un[0]) - side[1].rho * (SR - un[1]));
    R Fs[2][NV];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const R* Q = k ? QR : QL;
        const HSide<R>& s = side[k];
        const R d = S[k] - un[k];
        const R rd = s.rho * d;
        const R q0 = rd * recip(S[k] - Ss);
        R Qs[NV];
        Qs[0] = q0;
        Qs[1] = q0 * (Ss * i00 + ut1[k] * i01 + ut2[k] * i02);
        Qs[2] = q0 * (Ss * i10 + ut1[k] * i11 + ut2[k] * i12);
        Qs[3] = q0 * (Ss * i20 + ut1[k] * i21 + ut2[k] * i22);
        Qs[4] = q0 * (s.E * s.ir + (Ss - un[k]) * (Ss + s.p * recip(rd)));
#pragma unroll
        for (int c = 0; c < NV; ++c) Fs[k][c] = F[k][c] + S[k] * (Qs[c] - Q[c]);
    }
#pragma unroll
    for (int c = 0; c < NV; ++c)
        Flux[c] = (SL > R(0)) ? F[0][c] : (Ss >= R(0)) ? Fs[0][c] : (SR >= R(0)) ? Fs[1][c] : F[1][c];
    const R sl = fabs(un[0]) + side[0].c, sr = fabs(un[1]) + side[1].c;
    return sl < sr ? sr : sl;
}

template <typename R>
__device__ __forceinline__ R hllc(const R* QL, const R* QR, R nx, R ny, R nz, R gamma, R gm1, R* Flux, bool& bad) {
    R t1[3], t2[3];
    mc_tangents<R>(nx, ny, nz, false, t1, t2);
    // inverse of the frame matrix [n; t1; t2] by cofactors (pde.c:189-205; constant for an axis normal)
    const R M00 = nx, M01 = ny, M02 = nz, M10 = t1[0], M11 = t1[1], M12 = t1[2], M20 = t2[0], M21 = t2[1], M22 = t2[2];
    const R idet = R(1) / (M00 * (M11 * M22 - M12 * M21) - M01 * (M10 * M22 - M12 * M20) + M02 * (M10 * M21 - M11 * M20));
    const R i00 = (M11 * M22 - M12 * M21) * idet, i01 = -(M01 * M22 - M02 * M21) * idet, i02 = (M01 * M12 - M02 * M11) * idet;
    const R i10 = -(M10 * M22 - M12 * M20) * idet, i11 = (M00 * M22 - M02 * M20) * idet, i12 = -(M00 * M12 - M02 * M10) * idet;
    const R i20 = (M10 * M21 - M11 * M20) * idet, i21 = -(M00 * M21 - M01 * M20) * idet, i22 = (M00 * M11 - M01 * M10) * idet;
    // per side, once: 1/rho, the velocity, the pressure (PDEConsFlux, pde.c:40-88), the physical
    // flux, the frame velocities and the sound speed (the divisions of pde.c:207-322 become
    // products with a few reciprocals)
    R F[2][NV], un[2], ut1[2], ut2[2], P[2], c[2], ir[2];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const R* Q = side ? QR : QL;
        ir[side] = recip(Q[0]);
        const R u = ir[side] * Q[1], v = ir[side] * Q[2], w = ir[side] * Q[3];
        const R p = gm1 * (Q[4] - R(0.5) * Q[0] * (u * u + v * v + w * w));
        bad |= (Q[0] < R(1.0e-14)) || (p < R(1.0e-12)) || !(Q[0] == Q[0]);
        P[side] = p;
        un[side] = nx * u + ny * v + nz * w;
        ut1[side] = u * t1[0] + v * t1[1] + w * t1[2];
        ut2[side] = u * t2[0] + v * t2[1] + w * t2[2];
        const R mun = Q[0] * un[side];
        F[side][0] = mun;
        F[side][1] = mun * u + nx * p;
        F[side][2] = mun * v + ny * p;
        F[side][3] = mun * w + nz * p;
        F[side][4] = (Q[4] + p) * un[side];
        c[side] = sqrt(ir[side] * gamma * p);
    }
    const R SL = fmin(un[1] - c[1], un[0] - c[0]);
    const R SR = fmax(un[0] + c[0], un[1] + c[1]);
    const R S[2] = {SL, SR};
    const R Ss = (P[1] - P[0] + QL[0] * un[0] * (SL - un[0]) - QR[0] * un[1] * (SR - un[1])) *
                 recip(QL[0] * (SL - un[0]) - QR[0] * (SR - un[1]));
    R Fs[2][NV];
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const R* Q = side ? QR : QL;
        const R d = S[side] - un[side];
        const R rd = Q[0] * d;
        const R q0 = rd * recip(S[side] - Ss);
        R Qs[NV];
        Qs[0] = q0;
        Qs[1] = q0 * (Ss * i00 + ut1[side] * i01 + ut2[side] * i02);
        Qs[2] = q0 * (Ss * i10 + ut1[side] * i11 + ut2[side] * i12);
        Qs[3] = q0 * (Ss * i20 + ut1[side] * i21 + ut2[side] * i22);
        Qs[4] = q0 * (Q[4] * ir[side] + (Ss - un[side]) * (Ss + P[side] * recip(rd)));
#pragma unroll
        for (int k = 0; k < NV; ++k) Fs[side][k] = F[side][k] + S[side] * (Qs[k] - Q[k]);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k)
        Flux[k] = (SL > R(0)) ? F[0][k] : (Ss >= R(0)) ? Fs[0][k] : (SR >= R(0)) ? Fs[1][k] : F[1][k];
    const R sl = fabs(un[0]) + c[0], sr = fabs(un[1]) + c[1];
    return sl < sr ? sr : sl;
}

// PDErotHLLCRiemannSolver (pde.c:324-384): HLLC along the velocity-jump
// direction n1 and its two tangents, weighted by their projections on n
template <typename R>
__device__ __forceinline__ R rot_hllc(const R* QL, const R* QR, R nx, R ny, R nz, R gamma, R gm1, R* Flux, bool& bad) {
    const HSide<R> side[2] = {hllc_side<R>(QL, gamma, gm1, bad), hllc_side<R>(QR, gamma, gm1, bad)};
    const R du = side[1].u - side[0].u, dv = side[1].v - side[0].v, dw = side[1].w - side[0].w;
    const R dq2 = du * du + dv * dv + dw * dw;
    R n1[3];
    if (dq2 < R(1.0E-20)) {  // |du| < 1e-10
        n1[0] = nx; n1[1] = ny; n1[2] = nz;
    } else {
        const R idq = rsqrt(dq2);
        n1[0] = du * idq; n1[1] = dv * idq; n1[2] = dw * idq;
    }
    R a1 = n1[0] * nx + n1[1] * ny + n1[2] * nz;
    if (a1 < R(0)) {
        n1[0] = -n1[0]; n1[1] = -n1[1]; n1[2] = -n1[2];
        a1 = -a1;
    }
    R t1[3], t2[3];
    mc_tangents<R, true>(n1[0], n1[1], n1[2], true, t1, t2);
    R a2 = t1[0] * nx + t1[1] * ny + t1[2] * nz;
    if (a2 < R(0)) {
        t1[0] = -t1[0]; t1[1] = -t1[1]; t1[2] = -t1[2];
        a2 = -a2;
    }
    R a3 = t2[0] * nx + t2[1] * ny + t2[2] * nz;
    if (a3 < R(0)) {
        t2[0] = -t2[0]; t2[1] = -t2[1]; t2[2] = -t2[2];
        a3 = -a3;
    }
    R F1[NV], F2[NV], F3[NV];
    const R s1 = hllc_sides<R, true>(side, QL, QR, n1[0], n1[1], n1[2], F1);
    const R s2 = hllc_sides<R, true>(side, QL, QR, t1[0], t1[1], t1[2], F2);
    const R s3 = hllc_sides<R, true>(side, QL, QR, t2[0], t2[1], t2[2], F3);
#pragma unroll
    for (int k = 0; k < NV; ++k) Flux[k] = a1 * F1[k] + a2 * F2[k] + a3 * F3[k];
    return fmax(s1, fmax(s2, s3));
}

// numerical flux selected by the context (HYPE_FLUX_*) across an axis face of normal D
template <typename R, int D, int FLUX>
__device__ __forceinline__ R face_solver(const R* QL, const R* QR, R gamma, R gm1, R* F, bool& bad) {
    if (FLUX == HYPE_FLUX_RUSANOV) return rusanov<R, D>(QL, QR, gamma, gm1, F, bad);
    const R nx = R(D == 0), ny = R(D == 1), nz = R(D == 2);
    if (FLUX == HYPE_FLUX_HLLC) return hllc<R>(QL, QR, nx, ny, nz, gamma, gm1, F, bad);
    return rot_hllc<R>(QL, QR, nx, ny, nz, gamma, gm1, F, bad);
}

}  // namespace euler
}  // namespace hype
