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
};

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

// 2D CWENO4: 13-point stencil (centre, x-2..x+2, y-2..y+2, diagonals) -> 10 coefficients
template <typename R>
__device__ __forceinline__ void cweno2d(R u0, const R* ux, const R* uy, R upp, R upm, R ump, R umm, R* cf) {
    const R u_im2 = ux[0], u_im1 = ux[1], u_ip1 = ux[3], u_ip2 = ux[4];
    const R u_jm2 = uy[0], u_jm1 = uy[1], u_jp1 = uy[3], u_jp2 = uy[4];
    const R h = R(0.5), q = R(0.25);
    const R xR4 = R(41. / 60.) * (-u_im1 + u_ip1) + R(11. / 120.) * (u_im2 - u_ip2);
    const R yR4 = R(41. / 60.) * (-u_jm1 + u_jp1) + R(11. / 120.) * (u_jm2 - u_jp2);
    const R xxR4 = -u0 + h * (u_im1 + u_ip1);
    const R yyR4 = -u0 + h * (u_jm1 + u_jp1);
    const R xyR4 = q * (umm - ump - upm + upp);
    const R xxxR4 = R(1. / 6.) * (u_im1 - u_ip1) + R(1. / 12.) * (u_ip2 - u_im2);
    const R yyyR4 = R(1. / 6.) * (u_jm1 - u_jp1) + R(1. / 12.) * (u_jp2 - u_jm2);
    const R xxyR4 = q * (-umm + ump - upm + upp) + h * (u_jm1 - u_jp1);
    const R xyyR4 = h * (u_im1 - u_ip1) + q * (upp - umm - ump + upm);
    const R r13_3 = R(13. / 3.), r7_6 = R(7. / 6.);
    const R a = xR4 + R(0.1) * xxxR4, b = yR4 + R(0.1) * yyyR4;
    const R IS4 = a * a + r13_3 * (xxR4 * xxR4 + yyR4 * yyR4) + b * b + R(39.05) * (xxxR4 * xxxR4 + yyyR4 * yyyR4) +
                  r7_6 * xyR4 * xyR4 + R(4.7) * (xxyR4 * xxyR4 + xyyR4 * xyyR4);
    // R3 stencils: 0 centred, 1 towards -x, 2 towards +x, 3 towards -y, 4 towards +y
    const R cx = h * (-u_im1 + u_ip1), cy = h * (-u_jm1 + u_jp1);
    const R X1 = R(1.5) * u0 - R(2.0) * u_im1 + h * u_im2, XX1 = h * u0 - u_im1 + h * u_im2, XY1 = h * (umm - ump - u_jm1 + u_jp1);
    const R X2 = R(-1.5) * u0 + R(2.0) * u_ip1 - h * u_ip2, XX2 = h * u0 - u_ip1 + h * u_ip2, XY2 = h * (-upm + upp + u_jm1 - u_jp1);
    const R Y3 = R(1.5) * u0 - R(2.0) * u_jm1 + h * u_jm2, YY3 = h * u0 - u_jm1 + h * u_jm2, XY3 = h * (-u_im1 + umm + u_ip1 - upm);
    const R Y4 = R(-1.5) * u0 + R(2.0) * u_jp1 - h * u_jp2, YY4 = h * u0 - u_jp1 + h * u_jp2, XY4 = h * (u_im1 - ump - u_ip1 + upp);
    const R IS0 = cx * cx + cy * cy + r13_3 * (xxR4 * xxR4 + yyR4 * yyR4) + r7_6 * xyR4 * xyR4;
    const R IS1 = X1 * X1 + cy * cy + r13_3 * (XX1 * XX1 + yyR4 * yyR4) + r7_6 * XY1 * XY1;
    const R IS2 = X2 * X2 + cy * cy + r13_3 * (XX2 * XX2 + yyR4 * yyR4) + r7_6 * XY2 * XY2;
    const R IS3 = cx * cx + Y3 * Y3 + r13_3 * (xxR4 * xxR4 + YY3 * YY3) + r7_6 * XY3 * XY3;
    const R IS4b = cx * cx + Y4 * Y4 + r13_3 * (xxR4 * xxR4 + YY4 * YY4) + r7_6 * XY4 * XY4;
    const R gH = R(0.85), g0 = R((1.0 - 0.85) * 0.85), gs = R(0.25 * (1 - 0.85) * (1 - 0.85));
    // w = gamma / (IS + eps)^4, normalised; formed from ratios to the smallest (IS + eps)
    // so that FP32 does not underflow (the same normalised weights)
    R s[6] = {IS4 + R(1e-12), IS0 + R(1e-12), IS1 + R(1e-12), IS2 + R(1e-12), IS3 + R(1e-12), IS4b + R(1e-12)};
    R mn = s[0];
#pragma unroll
    for (int k = 1; k < 6; ++k) mn = fmin(mn, s[k]);
    R w[6];
    const R gam[6] = {gH, g0, gs, gs, gs, gs};
    R tot = R(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        w[k] = gam[k] * pow4(mn / s[k]);
        tot += w[k];
    }
    const R it = R(1) / tot;
#pragma unroll
    for (int k = 0; k < 6; ++k) w[k] *= it;
    const R wr = w[0] / gH;
    const R w0 = w[1], w1 = w[2], w2 = w[3], w3 = w[4], w4 = w[5];
    cf[0] = u0;
    // x derivative: modified by stencils 1, 2
    cf[1] = wr * (xR4 - (g0 + R(2) * gs) * cx - gs * (X1 + X2)) + (w0 + w3 + w4) * cx + w1 * X1 + w2 * X2;
    cf[2] = wr * (yR4 - (g0 + R(2) * gs) * cy - gs * (Y3 + Y4)) + (w0 + w1 + w2) * cy + w3 * Y3 + w4 * Y4;
    cf[3] = wr * (xxR4 - (g0 + R(2) * gs) * xxR4 - gs * (XX1 + XX2)) + (w0 + w3 + w4) * xxR4 + w1 * XX1 + w2 * XX2;
    cf[4] = wr * (yyR4 - (g0 + R(2) * gs) * yyR4 - gs * (YY3 + YY4)) + (w0 + w1 + w2) * yyR4 + w3 * YY3 + w4 * YY4;
    cf[5] = wr * (xyR4 - g0 * xyR4 - gs * (XY1 + XY2 + XY3 + XY4)) + w0 * xyR4 + w1 * XY1 + w2 * XY2 + w3 * XY3 + w4 * XY4;
    cf[6] = wr * xxxR4;
    cf[7] = wr * yyyR4;
    cf[8] = wr * xxyR4;
    cf[9] = wr * xyyR4;
}

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

// admissibility of a reconstructed primitive state (pde.c:99-129)
template <typename R>
__device__ __forceinline__ bool pad_ok(const Eos& e, const R* V) {
    double g, pi;
    if (e.model == HYPE_MP_DI4) {
        const double phi = (double)V[4];
        mix(e, phi, g, pi);
        return !((double)V[0] < 1.0e-14 || ((double)V[3] + pi) < 1.0e-12 || phi < 0.0 || phi > 1.0);
    }
    const double a1 = (double)V[5];
    mix(e, a1, g, pi);
    return !((double)V[0] < 1.0e-14 || (double)V[1] < 1.0e-14 || ((double)V[4] + pi) < 1.0e-12 || a1 < 0.0 || a1 > 1.0);
}

// one side of an HLLC solve: primitive state in the rotated frame
template <typename R>
struct Side {
    R rho, un, ut, p, E, c, a;  // mixture density, normal/tangential velocity, pressure, energy, sound speed, fraction
    R q[MAXV];                  // conserved state
    R f[MAXV + 1];              // physical flux (+ u_n)
};

template <typename R, int MODEL>
__device__ __forceinline__ void make_side(const Eos& e, const R* V, R nx, R ny, Side<R>& s, bool& bad) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    double gd, pid;
    mix(e, (double)V[NV - 1], gd, pid);
    const R g = (R)gd, pi = (R)pid;
    R u, v, p;
    if (MODEL == HYPE_MP_DI4) {
        s.rho = V[0]; u = V[1]; v = V[2]; p = V[3];
    } else {
        s.rho = V[5] * V[0] + (R(1) - V[5]) * V[1]; u = V[2]; v = V[3]; p = V[4];
    }
    s.a = V[NV - 1];
    s.p = p;
    s.un = u * nx + v * ny;
    s.ut = -u * ny + v * nx;
    s.E = (p + g * pi) / (g - R(1)) + R(0.5) * s.rho * (u * u + v * v);
    s.c = sqrt(g * (p + pi) / s.rho);
    bad |= (s.rho < R(1.0e-14)) || ((p + pi) < R(1.0e-12)) || !(s.rho == s.rho);
    if (MODEL == HYPE_MP_DI4) {
        s.q[0] = s.rho; s.q[1] = s.rho * u; s.q[2] = s.rho * v; s.q[3] = s.E; s.q[4] = s.a;
        const R m = s.rho * s.un;
        s.f[0] = m; s.f[1] = m * u + p * nx; s.f[2] = m * v + p * ny; s.f[3] = s.un * (s.E + p); s.f[4] = s.a * s.un;
    } else {
        s.q[0] = V[5] * V[0]; s.q[1] = (R(1) - V[5]) * V[1]; s.q[2] = s.rho * u; s.q[3] = s.rho * v; s.q[4] = s.E; s.q[5] = s.a;
        s.f[0] = s.q[0] * s.un; s.f[1] = s.q[1] * s.un; s.f[2] = s.rho * u * s.un + p * nx; s.f[3] = s.rho * v * s.un + p * ny;
        s.f[4] = (s.E + p) * s.un; s.f[5] = s.a * s.un;
    }
    s.f[NV] = s.un;
}

// HLLC with the interface velocity as the last component (pde.c:131-232)
template <typename R, int MODEL>
__device__ __forceinline__ R hllc2(const Eos& e, const R* VL, const R* VR, R nx, R ny, R* Flux, bool& bad) {
    constexpr int NV = MODEL == HYPE_MP_DI4 ? 5 : 6;
    Side<R> L, Rr;
    make_side<R, MODEL>(e, VL, nx, ny, L, bad);
    make_side<R, MODEL>(e, VR, nx, ny, Rr, bad);
    const R SL = fmin(Rr.un - Rr.c, L.un - L.c);
    const R SR = fmax(L.un + L.c, Rr.un + Rr.c);
    const R Ss = (Rr.p - L.p + L.rho * L.un * (SL - L.un) - Rr.rho * Rr.un * (SR - Rr.un)) /
                 (L.rho * (SL - L.un) - Rr.rho * (SR - Rr.un));
    const R sel = SL > R(0) ? R(0) : (Ss >= R(0) ? R(1) : (SR >= R(0) ? R(2) : R(3)));
    const Side<R>& S = (sel < R(1.5)) ? L : Rr;
    const R Sk = (sel < R(1.5)) ? SL : SR;
    if (sel == R(0) || sel == R(3)) {
#pragma unroll
        for (int k = 0; k <= NV; ++k) Flux[k] = S.f[k];
    } else {
        const R fr = (Sk - S.un) / (Sk - Ss);
        const R rs = S.rho * fr;
        R Us[MAXV];
        if (MODEL == HYPE_MP_DI4) {
            Us[0] = rs;
            Us[1] = rs * (Ss * nx - S.ut * ny);
            Us[2] = rs * (Ss * ny + S.ut * nx);
            Us[3] = rs * ((S.E / S.rho) + (Ss - S.un) * (Ss + S.p / (S.rho * (Sk - S.un))));
            Us[4] = S.a * fr;
        } else {
            Us[0] = S.q[0] * fr;
            Us[1] = S.q[1] * fr;
            Us[2] = rs * (Ss * nx - S.ut * ny);
            Us[3] = rs * (Ss * ny + S.ut * nx);
            Us[4] = rs * ((S.E / S.rho) + (Ss - S.un) * (Ss + S.p / (S.rho * (Sk - S.un))));
            Us[5] = S.a * fr;
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) Flux[k] = S.f[k] + Sk * (Us[k] - S.q[k]);
        Flux[NV] = S.un + Sk * (fr - R(1));
    }
    const R sl = fabs(L.un) + L.c, sr = fabs(Rr.un) + Rr.c;
    return sl < sr ? sr : sl;
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
        n1x = nx; n1y = ny;
    } else {
        n1x = du / dq; n1y = dv / dq;
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
    R f1[MAXV + 1], f2[MAXV + 1];
    const R s1 = hllc2<R, MODEL>(e, VL, VR, n1x, n1y, f1, bad);
    const R s2 = hllc2<R, MODEL>(e, VL, VR, n2x, n2y, f2, bad);
#pragma unroll
    for (int k = 0; k <= NV; ++k) Flux[k] = a1 * f1[k] + a2 * f2[k];
    return s1 < s2 ? s2 : s1;
}

}  // namespace mp2d
}  // namespace hype
