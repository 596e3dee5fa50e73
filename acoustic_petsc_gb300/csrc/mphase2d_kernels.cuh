// mphase2d_kernels.cuh -- device arithmetic of the 2D multiphase RHS.
//
// Follows the reference's 2D diffuse-interface code:
//   weno() 2D CWENO4        2d/weno4/bubble/reconstruction.c:128-251 (pow4 :123, minmod :106)
//   basis()                 2d/weno4/bubble/reconstruction.c:11-48
//   PDEFluxPrim, PAD check  2d/weno4/bubble/pde.c:62-129
//   HLLC / rotated HLLC     2d/weno4/bubble/pde.c:131-274 (+ interface-velocity component)
// and, for the five-equation model, the mixture EOS of
//   2d/HyPE-2D/kapila_5eqn.c:14-113.
// Arithmetic type R of reconstruction + flux is a template parameter; the EOS
// mixture coefficients are always formed in FP64 (stiffened gas with
// p_inf = 6e8 Pa cancels catastrophically in FP32).
#pragma once

#include "hype_common.cuh"

namespace hype {
namespace mp2d {

constexpr int NDOF = 10;
constexpr int MAXV = 6;

struct Eos {
    int model;  // HYPE_MP_DI4 or HYPE_MP_KAPILA5
    double g1, p1, g2, p2;
    float g1f, p1f, g2f, p2f;  // the same rounded to FP32 (the FP32 form's mixture)
    int stiff_nonneg;          // both gamma > 1 and both stiffnesses >= 0: the mixture's pi >= 0
    float rho_floor_f, p_floor_f;  // 1e-14 and 1e-12 rounded up to FP32: for a float x, (double)x < c iff x < c_f
};

inline float float_at_or_above(double c) {
    float f = (float)c;
    if ((double)f < c) f = nextafterf(f, INFINITY);
    return f;
}

inline Eos make_eos(int model, double g1, double p1, double g2, double p2) {
    return Eos{model, g1, p1, g2, p2, (float)g1, (float)p1, (float)g2, (float)p2,
               (p1 >= 0.0 && p2 >= 0.0 && g1 > 1.0 && g2 > 1.0) ? 1 : 0, float_at_or_above(1.0e-14),
               float_at_or_above(1.0e-12)};
}

// basis of the 10-term polynomial (reconstruction.c:11-48)
__host__ __device__ inline double basis2(double x, double y, int n) {
    switch (n) {
        case 0: return 1.0;
        case 1: return x;
        case 2: return y;
        case 3: return x * x - 1. / 12.;
        case 4: return y * y - 1. / 12.;
        case 5: return x * y;
        case 6: return x * (x * x - 3. / 20.);
        case 7: return y * (y * y - 3. / 20.);
        case 8: return y * (x * x - 1. / 12.);
        case 9: return x * (y * y - 1. / 12.);
        default: return 0.0;
    }
}

template <typename R>
__device__ __forceinline__ R pow4(R a) {
    const R a2 = a * a;
    return a2 * a2;
}

template <typename R>
__device__ __forceinline__ R minmod(R a, R b) {
    if (a * b < R(0)) return R(0);
    return (fabs(a) < fabs(b)) ? a : b;
}

// 2D CWENO4: 13-point stencil (centre, x-2..x+2, y-2..y+2, diagonals) -> 10 coefficients.
// Written operation by operation in the reference's order; the file is compiled
// without FMA contraction, so the FP64 instance rounds exactly like the CPU code
// (the admissibility test downstream is a hard threshold on these values).
template <typename R>
struct Cw2Weights;

template <typename R>
__device__ __forceinline__ void cweno2d(R u0, const R* ux, const R* uy, R upp, R upm, R ump, R umm, R* cf,
                                        bool linear = false) {
    const R u_im2 = ux[0], u_im1 = ux[1], u_ip1 = ux[3], u_ip2 = ux[4];
    const R u_jm2 = uy[0], u_jm1 = uy[1], u_jp1 = uy[3], u_jp2 = uy[4];
    const R u_ip1jp1 = upp, u_ip1jm1 = upm, u_im1jp1 = ump, u_im1jm1 = umm;
    const R r41_60 = R(41. / 60.), r11_120 = R(11. / 120.), r1_6 = R(1. / 6.), r1_12 = R(1. / 12.);
    const R r13_3 = R(13. / 3.), r7_6 = R(7. / 6.);
    const R gH = R(0.85), gL = R(0.85);
    R g3[5];
    g3[0] = (R(1.0) - gH) * gL;
#pragma unroll
    for (int i = 1; i < 5; ++i) g3[i] = R(0.25) * (R(1) - gH) * (R(1) - gL);
    const R xR4 = r41_60 * (-u_im1 + u_ip1) + r11_120 * (u_im2 - u_ip2);
    const R yR4 = r41_60 * (-u_jm1 + u_jp1) + r11_120 * (u_jm2 - u_jp2);
    const R xxR4 = -u0 + R(0.5) * (u_im1 + u_ip1);
    const R yyR4 = -u0 + R(0.5) * (u_jm1 + u_jp1);
    const R xyR4 = R(0.25) * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
    const R xxxR4 = r1_6 * (u_im1 - u_ip1) + r1_12 * (u_ip2 - u_im2);
    const R yyyR4 = r1_6 * (u_jm1 - u_jp1) + r1_12 * (u_jp2 - u_jm2);
    const R xxyR4 = R(0.25) * (-u_im1jm1 + u_im1jp1 - u_ip1jm1 + u_ip1jp1) + R(0.5) * (u_jm1 - u_jp1);
    const R xyyR4 = R(0.5) * (u_im1 - u_ip1) + R(0.25) * (u_ip1jp1 - u_im1jm1 - u_im1jp1 + u_ip1jm1);
    if (linear) {  // the optimal-weight limit: the R4 polynomial itself
        cf[0] = u0;
        cf[1] = xR4; cf[2] = yR4; cf[3] = xxR4; cf[4] = yyR4; cf[5] = xyR4;
        cf[6] = xxxR4; cf[7] = yyyR4; cf[8] = xxyR4; cf[9] = xyyR4;
        return;
    }
    const R IS4 = (xR4 + R(0.1) * xxxR4) * (xR4 + R(0.1) * xxxR4) + r13_3 * (xxR4 * xxR4 + yyR4 * yyR4) +
                  (yR4 + R(0.1) * yyyR4) * (yR4 + R(0.1) * yyyR4) + R(39.05) * (xxxR4 * xxxR4 + yyyR4 * yyyR4) +
                  r7_6 * xyR4 * xyR4 + R(4.7) * (xxyR4 * xxyR4 + xyyR4 * xyyR4);
    R X[5], Y[5], XX[5], YY[5], XY[5];
    X[0] = R(0.5) * (-u_im1 + u_ip1);
    Y[0] = R(0.5) * (-u_jm1 + u_jp1);
    XX[0] = -u0 + R(0.5) * (u_im1 + u_ip1);
    YY[0] = -u0 + R(0.5) * (u_jm1 + u_jp1);
    XY[0] = R(0.25) * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
    X[1] = R(1.5) * u0 - R(2.0) * u_im1 + R(0.5) * u_im2;
    Y[1] = R(0.5) * (-u_jm1 + u_jp1);
    XX[1] = R(0.5) * u0 - u_im1 + R(0.5) * u_im2;
    YY[1] = -u0 + R(0.5) * u_jm1 + R(0.5) * u_jp1;
    XY[1] = R(0.5) * (u_im1jm1 - u_im1jp1 - u_jm1 + u_jp1);
    X[2] = R(-1.5) * u0 + R(2.0) * u_ip1 - R(0.5) * u_ip2;
    Y[2] = R(0.5) * (-u_jm1 + u_jp1);
    XX[2] = R(0.5) * u0 - u_ip1 + R(0.5) * u_ip2;
    YY[2] = -u0 + R(0.5) * u_jm1 + R(0.5) * u_jp1;
    XY[2] = R(0.5) * (-u_ip1jm1 + u_ip1jp1 + u_jm1 - u_jp1);
    X[3] = R(0.5) * (-u_im1 + u_ip1);
    Y[3] = R(1.5) * u0 - R(2.0) * u_jm1 + R(0.5) * u_jm2;
    XX[3] = -u0 + R(0.5) * u_im1 + R(0.5) * u_ip1;
    YY[3] = R(0.5) * u0 - u_jm1 + R(0.5) * u_jm2;
    XY[3] = R(0.5) * (-u_im1 + u_im1jm1 + u_ip1 - u_ip1jm1);
    X[4] = R(0.5) * (-u_im1 + u_ip1);
    Y[4] = R(-1.5) * u0 + R(2.0) * u_jp1 - R(0.5) * u_jp2;
    XX[4] = -u0 + R(0.5) * u_im1 + R(0.5) * u_ip1;
    YY[4] = R(0.5) * u0 - u_jp1 + R(0.5) * u_jp2;
    XY[4] = R(0.5) * (u_im1 - u_im1jp1 - u_ip1 + u_ip1jp1);
    R IS3[5];
#pragma unroll
    for (int i = 0; i < 5; ++i)
        IS3[i] = X[i] * X[i] + Y[i] * Y[i] + r13_3 * (XX[i] * XX[i] + YY[i] * YY[i]) + r7_6 * XY[i] * XY[i];
    R w4, w3[5];
    Cw2Weights<R>::compute(IS4, IS3, gH, g3, w4, w3);
    const R wr = w4 / gH;
    const R* Q[5] = {X, Y, XX, YY, XY};
    const R R4[5] = {xR4, yR4, xxR4, yyR4, xyR4};
    cf[0] = u0;
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        const R* v = Q[q];
        cf[1 + q] = wr * (R4[q] - g3[0] * v[0] - g3[1] * v[1] - g3[2] * v[2] - g3[3] * v[3] - g3[4] * v[4]) + w3[0] * v[0] +
                    w3[1] * v[1] + w3[2] * v[2] + w3[3] * v[3] + w3[4] * v[4];
    }
    cf[6] = wr * xxxR4;
    cf[7] = wr * yyyR4;
    cf[8] = wr * xxyR4;
    cf[9] = wr * xyyR4;
}

// FP64: w = gamma / pow4(IS + eps), normalised by division, as the reference does
template <>
struct Cw2Weights<double> {
    __device__ __forceinline__ static void compute(double IS4, const double* IS3, double gH, const double* g3, double& w4,
                                                   double* w3) {
        w4 = gH / (pow4(IS4 + 1.0e-12));
        double sum = w4;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            w3[i] = g3[i] / (pow4(IS3[i] + 1.0e-12));
            sum += w3[i];
        }
        w4 = w4 / sum;
#pragma unroll
        for (int i = 0; i < 5; ++i) w3[i] = w3[i] / sum;
    }
};

// FP32: (1e-12)^4 underflows; the same normalised weights from ratios to the smallest (IS + eps)
template <>
struct Cw2Weights<float> {
    __device__ __forceinline__ static void compute(float IS4, const float* IS3, float gH, const float* g3, float& w4,
                                                   float* w3) {
        float s4 = IS4 + 1.0e-12f, ss[5];
        float mn = s4;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            ss[i] = IS3[i] + 1.0e-12f;
            mn = fminf(mn, ss[i]);
        }
        w4 = gH * pow4(mn / s4);
        float sum = w4;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            w3[i] = g3[i] * pow4(mn / ss[i]);
            sum += w3[i];
        }
        w4 = w4 / sum;
#pragma unroll
        for (int i = 0; i < 5; ++i) w3[i] = w3[i] / sum;
    }
};

// mixture ratio of specific heats and stiffness (FP64)
__device__ __forceinline__ void mix(const Eos& e, double a, double& g, double& pi) {
    if (e.model == HYPE_MP_DI4) {  // pde.c:11-12, a = phi
        g = 1.0 + (e.g1 - 1.0) * (e.g2 - 1.0) / ((1.0 - a) * (e.g1 - 1.0) + a * (e.g2 - 1.0));
        pi = ((g - 1.0) / g) * (e.g1 * e.p1 * a / (e.g1 - 1.0) + e.g2 * e.p2 * (1.0 - a) / (e.g2 - 1.0));
    } else {  // kapila_5eqn.c:18-19, a = alpha_1
        const double a2 = 1.0 - a;
        g = 1.0 + ((e.g1 - 1.0) * (e.g2 - 1.0)) / ((e.g2 - 1.0) * a + (e.g1 - 1.0) * a2);
        pi = ((g - 1.0) / g) * (e.g1 * e.p1 * a / (e.g1 - 1.0) + e.g2 * e.p2 * a2 / (e.g2 - 1.0));
    }
}

// the mixture in the face solver's arithmetic: FP64 for the FP64 form (mix, the reference's
// rounding); FP32 for the FP32 form, whose solver works on FP32 values of g and pi anyway (every
// term of the mixture rules is positive for gamma > 1 and non-negative stiffnesses: nothing
// cancels, and the FP32 pair is within a few ulp of the rounded FP64 one)
template <typename R>
__device__ __forceinline__ void mix_r(const Eos& e, R a, R& g, R& pi) {
    if constexpr (sizeof(R) == sizeof(double)) {
        double gd, pd;
        mix(e, (double)a, gd, pd);
        g = (R)gd;
        pi = (R)pd;
    } else {
        const float g1 = e.g1f, g2 = e.g2f, p1 = e.p1f, p2 = e.p2f;
        const float a2 = 1.0f - a;
        if (e.model == HYPE_MP_DI4) g = 1.0f + (g1 - 1.0f) * (g2 - 1.0f) / (a2 * (g1 - 1.0f) + a * (g2 - 1.0f));
        else g = 1.0f + ((g1 - 1.0f) * (g2 - 1.0f)) / ((g2 - 1.0f) * a + (g1 - 1.0f) * a2);
        pi = ((g - 1.0f) / g) * (g1 * p1 * a / (g1 - 1.0f) + g2 * p2 * a2 / (g2 - 1.0f));
    }
}

// conserved -> primitive (FP64): DI4 (rho,u,v,p,phi), KAPILA5 (rho1,rho2,u,v,p,a1)
__device__ __forceinline__ void cons2prim(const Eos& e, const double* Q, double* V) {
    double g, pi;
    if (e.model == HYPE_MP_DI4) {
        const double phi = Q[4];
        mix(e, phi, g, pi);
        const double irho = 1.0 / Q[0];
        V[0] = Q[0];
        V[1] = irho * Q[1];
        V[2] = irho * Q[2];
        V[3] = (g - 1.0) * (Q[3] - 0.5 * irho * (Q[1] * Q[1] + Q[2] * Q[2])) - g * pi;
        V[4] = phi;
    } else {
        const double a1 = Q[5];
        mix(e, a1, g, pi);
        const double rho = Q[0] + Q[1];
        const double u = Q[2] / rho, v = Q[3] / rho;
        V[0] = Q[0] / a1;
        V[1] = Q[1] / (1.0 - a1);
        V[2] = u;
        V[3] = v;
        V[4] = (g - 1.0) * (Q[4] - 0.5 * rho * (u * u + v * v)) - g * pi;
        V[5] = a1;
    }
}

// admissibility of a reconstructed primitive state (pde.c:99-129).  The mixture's stiffness pi is
// formed only when the pressure test needs it: with both gases' gamma > 1, non-negative
// stiffnesses and the volume fraction in [0, 1] (outside it the state fails anyway), pi >= 0, so
// p + pi rounds to at least p and p >= 1e-12 passes the test whatever pi is (a NaN p fails
// neither form of the test).
template <typename R>
__device__ __forceinline__ bool pad_ok(const Eos& e, const R* V) {
    double g, pi;
    const bool stiff_nonneg = e.stiff_nonneg != 0;
    if constexpr (sizeof(R) == sizeof(float)) {
        // the same tests on the FP32 values without converting them: for a float x, (double)x < c
        // exactly when x < c rounded up to a float
        const float rho_floor = e.rho_floor_f, p_floor = e.p_floor_f;
        const int ia = e.model == HYPE_MP_DI4 ? 4 : 5, ip = ia - 1;
        const float a = V[ia], p = V[ip];
        if (V[0] < rho_floor || (e.model != HYPE_MP_DI4 && V[1] < rho_floor) || a < 0.0f || a > 1.0f) return false;
        if (stiff_nonneg && !(p < p_floor)) return true;
        mix(e, (double)a, g, pi);
        return !(((double)p + pi) < 1.0e-12);
    }
    if (e.model == HYPE_MP_DI4) {
        const double phi = (double)V[4], p = (double)V[3];
        if ((double)V[0] < 1.0e-14 || phi < 0.0 || phi > 1.0) return false;
        if (stiff_nonneg && !(p < 1.0e-12)) return true;
        mix(e, phi, g, pi);
        return !((p + pi) < 1.0e-12);
    }
    const double a1 = (double)V[5], p = (double)V[4];
    if ((double)V[0] < 1.0e-14 || (double)V[1] < 1.0e-14 || a1 < 0.0 || a1 > 1.0) return false;
    if (stiff_nonneg && !(p < 1.0e-12)) return true;
    mix(e, a1, g, pi);
    return !((p + pi) < 1.0e-12);
}

// conserved state of a primitive state (PDEPrim2Cons, pde.c:24-36; kapila_5eqn.c:44-60); (g, pi) is
// the state's mixture, mix_r(e, V[NV - 1]), formed once per face point by the caller
template <typename R, int MODEL>
__device__ __forceinline__ void prim2cons(const R* V, R g, R pi, R* Q) {
    if (MODEL == HYPE_MP_DI4) {
        const R en = (V[3] + g * pi) / (g - R(1.0));
        const R k = R(0.5) * V[0] * (V[1] * V[1] + V[2] * V[2]);
        Q[0] = V[0]; Q[1] = V[0] * V[1]; Q[2] = V[0] * V[2]; Q[3] = k + en; Q[4] = V[4];
    } else {
        const R a1 = V[5], a2 = R(1.0) - a1;
        const R rho = a1 * V[0] + a2 * V[1];
        Q[0] = a1 * V[0]; Q[1] = a2 * V[1]; Q[2] = rho * V[2]; Q[3] = rho * V[3];
        Q[4] = (V[4] + g * pi) / (g - R(1.0)) + R(0.5) * rho * (V[2] * V[2] + V[3] * V[3]);
        Q[5] = a1;
    }
}

// What one side of a face point gives independently of the normal (pde.c:24-129, HLLC :131-232):
// its conserved state (PDEPrim2Cons), mixture density, sound speed sqrt(g (p + pi) / rho) (the
// same expression in PDEFluxPrim and in the HLLC speeds), HLLC's own energy expression, and the
// admissibility flag of PDEFluxPrim.  The rotated solver makes two HLLC evaluations per face point;
// the reference forms these in each, here once per side: the same expressions, the same values.
template <typename R>
struct Side2 {
    R Q[MAXV];
    R rho, c, Eh;
};

template <typename R, int MODEL>
__device__ __forceinline__ void make_side2(const R* V, R g, R pi, Side2<R>& s, bool& bad) {
    prim2cons<R, MODEL>(V, g, pi, s.Q);
    R u, v, p;
    if (MODEL == HYPE_MP_DI4) {
        s.rho = V[0]; u = V[1]; v = V[2]; p = V[3];
    } else {
        s.rho = V[5] * V[0] + (R(1.0) - V[5]) * V[1];  // a1 r1 + a2 r2
        u = V[2]; v = V[3]; p = V[4];
    }
    bad |= (s.rho < R(1.0e-14)) || ((p + pi) < R(1.0e-12)) || !(s.rho == s.rho);
    s.c = sqrt(g * (p + pi) / s.rho);
    s.Eh = (p + g * pi) / (g - R(1.0)) + R(0.5) * s.rho * u * u + R(0.5) * s.rho * v * v;
}

// physical flux of a primitive state along (nx, ny) and its wave speed (PDEFluxPrim, pde.c:62-97);
// its energy (p + g pi)/(g - 1) + rho |u|^2 / 2 is the conserved energy of the side
template <typename R, int MODEL>
__device__ __forceinline__ R flux_prim(const R* V, const Side2<R>& s, R nx, R ny, R* F) {
    if (MODEL == HYPE_MP_DI4) {
        const R phi = V[4];
        const R rho = V[0], u = V[1], v = V[2], p = V[3];
        const R E = s.Q[3];
        const R un = u * nx + v * ny;
        const R rhoun = rho * un;
        F[0] = rhoun; F[1] = rhoun * u + p * nx; F[2] = rhoun * v + p * ny; F[3] = un * (E + p); F[4] = phi * un;
        return fabs(un) + s.c;
    }
    const R a1 = V[5], a2 = R(1.0) - a1;
    const R r1 = V[0], r2 = V[1], u = V[2], v = V[3], p = V[4];
    const R rho = s.rho;
    const R E = s.Q[4];
    const R un = u * nx + v * ny;
    F[0] = a1 * r1 * un; F[1] = a2 * r2 * un; F[2] = rho * u * un + p * nx; F[3] = rho * v * un + p * ny;
    F[4] = (E + p) * un; F[5] = a1 * un;
    return fabs(un) + s.c;
}

// HLLC with the interface velocity as the last component (HLLCRiemannSolver, pde.c:131-232);
// star partial densities of the five-equation model a_k r_k (S - u_n)/(S - S*).  The reference
// re-forms each side's mixture and EOS quantities in every EOS call; they depend on the side's
// state alone, so the caller forms them once per face point (sides L, R): the same values, a
// fraction of the divisions and square roots
template <typename R, int MODEL>
__device__ __forceinline__ R hllc2(const R* VL, const R* VR, const Side2<R>& sL, const Side2<R>& sR, R nx, R ny,
                                   R* Flux) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    R FL[MAXV + 1], FR[MAXV + 1];
    const R* QL = sL.Q;
    const R* QR = sR.Q;
    const R sl = flux_prim<R, MODEL>(VL, sL, nx, ny, FL);
    const R sr = flux_prim<R, MODEL>(VR, sR, nx, ny, FR);
    R uL, uR, vL, vR, PL, PR;
    if (MODEL == HYPE_MP_DI4) {
        uL = VL[1]; vL = VL[2]; PL = VL[3];
        uR = VR[1]; vR = VR[2]; PR = VR[3];
    } else {
        uL = VL[2]; vL = VL[3]; PL = VL[4];
        uR = VR[2]; vR = VR[3]; PR = VR[4];
    }
    const R rL = sL.rho, rR = sR.rho;
    const R unL = uL * nx + vL * ny, utL = -uL * ny + vL * nx;
    const R unR = uR * nx + vR * ny, utR = -uR * ny + vR * nx;
    const R cL = sL.c, cR = sR.c;
    const R EL = sL.Eh, ER = sR.Eh;
    const R a1 = unR - cR, b1 = unL - cL;
    const R SL = (a1 < b1) ? a1 : b1;
    const R a2 = unL + cL, b2 = unR + cR;
    const R SR = (a2 < b2) ? b2 : a2;
    const R Ss = (PR - PL + rL * unL * (SL - unL) - rR * unR * (SR - unR)) / (rL * (SL - unL) - rR * (SR - unR));
    FL[NV] = unL;
    FR[NV] = unR;
    // only the star state of the selected side is needed
    const int sel = (SL > R(0)) ? 0 : (Ss >= R(0)) ? 1 : (SR >= R(0)) ? 2 : 3;
    if (sel == 0 || sel == 3) {
        const R* Fo = sel == 0 ? FL : FR;
#pragma unroll
        for (int i = 0; i <= NV; ++i) Flux[i] = Fo[i];
    } else {
        const bool left = sel == 1;
        const R Sk = left ? SL : SR, rk = left ? rL : rR, unk = left ? unL : unR, utk = left ? utL : utR;
        const R Pk = left ? PL : PR, Ek = left ? EL : ER;
        const R* Vk = left ? VL : VR;
        const R* Qk = left ? QL : QR;
        const R* Fk = left ? FL : FR;
        R Us[MAXV];
        if (MODEL == HYPE_MP_DI4) {
            Us[0] = rk * (Sk - unk) / (Sk - Ss);
            Us[1] = Us[0] * (Ss * nx - utk * ny);
            Us[2] = Us[0] * (Ss * ny + utk * nx);
            Us[3] = Us[0] * ((Ek / rk) + (Ss - unk) * (Ss + Pk / (rk * (Sk - unk))));
            Us[4] = Vk[4] * (Sk - unk) / (Sk - Ss);
        } else {
            const R f = (Sk - unk) / (Sk - Ss);
            const R rs = rk * f;
            Us[0] = Qk[0] * f;
            Us[1] = Qk[1] * f;
            Us[2] = rs * (Ss * nx - utk * ny);
            Us[3] = rs * (Ss * ny + utk * nx);
            Us[4] = rs * ((Ek / rk) + (Ss - unk) * (Ss + Pk / (rk * (Sk - unk))));
            Us[5] = Vk[5] * f;
        }
#pragma unroll
        for (int i = 0; i < NV; ++i) Flux[i] = Fk[i] + Sk * (Us[i] - Qk[i]);
        Flux[NV] = unk + Sk * (((Sk - unk) / (Sk - Ss)) - R(1.0));
    }
    return (sl < sr) ? sr : sl;
}

// rotated HLLC (pde.c:234-274): HLLC along the velocity-jump direction and its normal
template <typename R, int MODEL>
__device__ __forceinline__ R rot_hllc2(const Eos& e, const R* VL, const R* VR, R nx, R ny, R* Flux, bool& bad) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    constexpr int IU = MODEL == HYPE_MP_DI4 ? 1 : 2;
    const R du = VR[IU] - VL[IU], dv = VR[IU + 1] - VL[IU + 1];
    const R dq = sqrt(du * du + dv * dv);
    R n1x, n1y;
    if (dq < R(1.0E-10)) {
        n1x = nx;
        n1y = ny;
    } else {
        n1x = du / dq;
        n1y = dv / dq;
    }
    R a1 = n1x * nx + n1y * ny;
    if (a1 < R(0)) {
        n1x = -n1x; n1y = -n1y; a1 = -a1;
    }
    R n2x = -n1y, n2y = n1x;
    R a2 = n2x * nx + n2y * ny;
    if (a2 < R(0)) {
        n2x = -n2x; n2y = -n2y; a2 = -a2;
    }
    R gL, piL, gR, piR;  // each side's mixture and EOS quantities, once for both solves
    mix_r<R>(e, VL[NV - 1], gL, piL);
    mix_r<R>(e, VR[NV - 1], gR, piR);
    Side2<R> sL, sR;
    make_side2<R, MODEL>(VL, gL, piL, sL, bad);
    make_side2<R, MODEL>(VR, gR, piR, sR, bad);
    R f1[MAXV + 1], f2[MAXV + 1];
    const R s1 = hllc2<R, MODEL>(VL, VR, sL, sR, n1x, n1y, f1);
    const R s2 = hllc2<R, MODEL>(VL, VR, sL, sR, n2x, n2y, f2);
#pragma unroll
    for (int k = 0; k <= NV; ++k) Flux[k] = a1 * f1[k] + a2 * f2[k];
    return (s1 < s2) ? s2 : s1;
}

}  // namespace mp2d
}  // namespace hype
