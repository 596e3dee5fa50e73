/*
 * mphase2d_oracle.c -- CPU restatement of the 2D multiphase RHS (the oracle).
 * TEST INFRASTRUCTURE ONLY (tests/, smoke, bench CPU baseline).
 *
 * Model DI4 (diffuse interface, Q = rho, rho u, rho v, E, phi) follows
 * 2d/weno4/bubble and is checked bit for bit against it:
 *   RHSFunction         2d/weno4/bubble/rhs_function.c:12-390 (BC :54-170,
 *                       primitive CWENO4 + 8-node PAD -> minmod :173-275,
 *                       rotated-HLLC fluxes :277-349, divergence + phi term :351-380,
 *                       dt = CFL h / (2 s_max) :385)
 *   weno() 2D CWENO4    2d/weno4/bubble/reconstruction.c:128-251 (pow4 :123, minmod :106)
 *   basis()             2d/weno4/bubble/reconstruction.c:11-48
 *   PDE functions       2d/weno4/bubble/pde.c:9-274
 * Model KAPILA5 (Q = a1 r1, a2 r2, rho u, rho v, E, a1) assembles the
 * five-equation model of 2d/HyPE-2D/kapila_5eqn.c:14-113 (mixture gamma, pi from
 * a1; the K term is zero there, :189) with the same reconstruction, PAD
 * fallback, rotated HLLC (star partial densities a_k r_k (S-u_n)/(S-S*)) and the
 * non-conservative a1 update of the bubble code.  Its parity is pinned only
 * through the shared machinery.
 */
#include "hype_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXV 6
#define NDOF 10

static const double R1_6 = 1. / 6.;
static const double R13_3 = 13. / 3.;
static const double R7_6 = 7. / 6.;
static const double R11_120 = 11. / 120.;
static const double R1_12 = 1. / 12.;
static const double R41_60 = 41. / 60.;
static const double X_GP2[2] = {-0.28867513459481287, 0.28867513459481287};
static const double X_NODE[8] = {0.50000000000000000, 0.50000000000000000, -0.50000000000000000, -0.50000000000000000,
                                 -0.28867513459481287, 0.28867513459481287, -0.28867513459481287, 0.28867513459481287};
static const double Y_NODE[8] = {-0.28867513459481287, 0.28867513459481287, -0.28867513459481287, 0.28867513459481287,
                                 -0.50000000000000000, -0.50000000000000000, 0.50000000000000000, 0.50000000000000000};

static double basis2(double x, double y, int n) {
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

static inline double pow4(double a) {
    double a2 = a * a;
    return a2 * a2;
}

static inline double minmod(double a, double b) {
    if (a * b < 0.0) return 0.0;
    return (fabs(a) < fabs(b)) ? a : b;
}

/* 2D CWENO4 from the 13-point stencil: c, x[-2..2], y[-2..2], diagonals pp,pm,mp,mm */
void orc_cweno4_2d(double u0, const double* ux, const double* uy, double upp, double upm, double ump, double umm,
                   double* coeffs) {
    const double gH = 0.85, gL = 0.85;
    const double u_im2 = ux[0], u_im1 = ux[1], u_ip1 = ux[3], u_ip2 = ux[4];
    const double u_jm2 = uy[0], u_jm1 = uy[1], u_jp1 = uy[3], u_jp2 = uy[4];
    const double u_ip1jp1 = upp, u_ip1jm1 = upm, u_im1jp1 = ump, u_im1jm1 = umm;
    double g3[5];
    g3[0] = (1.0 - gH) * gL;
    for (int i = 1; i < 5; ++i) g3[i] = 0.25 * (1 - gH) * (1 - gL);
    const double xR4 = R41_60 * (-u_im1 + u_ip1) + R11_120 * (u_im2 - u_ip2);
    const double yR4 = R41_60 * (-u_jm1 + u_jp1) + R11_120 * (u_jm2 - u_jp2);
    const double xxR4 = -u0 + 0.5 * (u_im1 + u_ip1);
    const double yyR4 = -u0 + 0.5 * (u_jm1 + u_jp1);
    const double xyR4 = 0.25 * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
    const double xxxR4 = R1_6 * (u_im1 - u_ip1) + R1_12 * (u_ip2 - u_im2);
    const double yyyR4 = R1_6 * (u_jm1 - u_jp1) + R1_12 * (u_jp2 - u_jm2);
    const double xxyR4 = 0.25 * (-u_im1jm1 + u_im1jp1 - u_ip1jm1 + u_ip1jp1) + 0.5 * (u_jm1 - u_jp1);
    const double xyyR4 = 0.5 * (u_im1 - u_ip1) + 0.25 * (u_ip1jp1 - u_im1jm1 - u_im1jp1 + u_ip1jm1);
    const double IS4 = (xR4 + 0.1 * xxxR4) * (xR4 + 0.1 * xxxR4) + R13_3 * (xxR4 * xxR4 + yyR4 * yyR4) +
                       (yR4 + 0.1 * yyyR4) * (yR4 + 0.1 * yyyR4) + 39.05 * (xxxR4 * xxxR4 + yyyR4 * yyyR4) +
                       R7_6 * xyR4 * xyR4 + 4.7 * (xxyR4 * xxyR4 + xyyR4 * xyyR4);
    double w4 = gH / (pow4(IS4 + 1.0e-12));
    double sum = w4;
    double X[5], Y[5], XX[5], YY[5], XY[5];
    X[0] = 0.5 * (-u_im1 + u_ip1);
    Y[0] = 0.5 * (-u_jm1 + u_jp1);
    XX[0] = -u0 + 0.5 * (u_im1 + u_ip1);
    YY[0] = -u0 + 0.5 * (u_jm1 + u_jp1);
    XY[0] = 0.25 * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
    X[1] = 1.5 * u0 - 2.0 * u_im1 + 0.5 * u_im2;
    Y[1] = 0.5 * (-u_jm1 + u_jp1);
    XX[1] = 0.5 * u0 - u_im1 + 0.5 * u_im2;
    YY[1] = -u0 + 0.5 * u_jm1 + 0.5 * u_jp1;
    XY[1] = 0.5 * (u_im1jm1 - u_im1jp1 - u_jm1 + u_jp1);
    X[2] = -1.5 * u0 + 2.0 * u_ip1 - 0.5 * u_ip2;
    Y[2] = 0.5 * (-u_jm1 + u_jp1);
    XX[2] = 0.5 * u0 - u_ip1 + 0.5 * u_ip2;
    YY[2] = -u0 + 0.5 * u_jm1 + 0.5 * u_jp1;
    XY[2] = 0.5 * (-u_ip1jm1 + u_ip1jp1 + u_jm1 - u_jp1);
    X[3] = 0.5 * (-u_im1 + u_ip1);
    Y[3] = 1.5 * u0 - 2.0 * u_jm1 + 0.5 * u_jm2;
    XX[3] = -u0 + 0.5 * u_im1 + 0.5 * u_ip1;
    YY[3] = 0.5 * u0 - u_jm1 + 0.5 * u_jm2;
    XY[3] = 0.5 * (-u_im1 + u_im1jm1 + u_ip1 - u_ip1jm1);
    X[4] = 0.5 * (-u_im1 + u_ip1);
    Y[4] = -1.5 * u0 + 2.0 * u_jp1 - 0.5 * u_jp2;
    XX[4] = -u0 + 0.5 * u_im1 + 0.5 * u_ip1;
    YY[4] = 0.5 * u0 - u_jp1 + 0.5 * u_jp2;
    XY[4] = 0.5 * (u_im1 - u_im1jp1 - u_ip1 + u_ip1jp1);
    double w3[5];
    for (int i = 0; i < 5; ++i) {
        const double IS = X[i] * X[i] + Y[i] * Y[i] + R13_3 * (XX[i] * XX[i] + YY[i] * YY[i]) + R7_6 * XY[i] * XY[i];
        w3[i] = g3[i] / (pow4(IS + 1.0e-12));
        sum += w3[i];
    }
    w4 = w4 / sum;
    for (int i = 0; i < 5; ++i) w3[i] = w3[i] / sum;
    const double wr = w4 / gH;
    const double* Q[5] = {X, Y, XX, YY, XY};
    const double R4[5] = {xR4, yR4, xxR4, yyR4, xyR4};
    coeffs[0] = u0;
    for (int q = 0; q < 5; ++q) {
        const double* v = Q[q];
        coeffs[1 + q] = wr * (R4[q] - g3[0] * v[0] - g3[1] * v[1] - g3[2] * v[2] - g3[3] * v[3] - g3[4] * v[4]) + w3[0] * v[0] +
                        w3[1] * v[1] + w3[2] * v[2] + w3[3] * v[3] + w3[4] * v[4];
    }
    coeffs[6] = wr * xxxR4;
    coeffs[7] = wr * yyyR4;
    coeffs[8] = wr * xxyR4;
    coeffs[9] = wr * xyyR4;
}

/* ------------------------------------------------------------------ EOS / PDE */
typedef struct {
    int model;  /* 0 DI4, 1 KAPILA5 */
    double g1, p1, g2, p2;
} Eos;

/* mixture gamma and stiffness of the DI4 model (pde.c:11-12) */
static inline void di4_mix(const Eos* e, double phi, double* g, double* pinf) {
    *g = 1.0 + (e->g1 - 1.0) * (e->g2 - 1.0) / ((1.0 - phi) * (e->g1 - 1.0) + phi * (e->g2 - 1.0));
    *pinf = ((*g - 1.0) / *g) * (e->g1 * e->p1 * phi / (e->g1 - 1.0) + e->g2 * e->p2 * (1.0 - phi) / (e->g2 - 1.0));
}
/* mixture gamma and stiffness of the Kapila model (kapila_5eqn.c:18-19) */
static inline void k5_mix(const Eos* e, double a1, double* g, double* pi) {
    const double a2 = 1.0 - a1;
    *g = 1.0 + ((e->g1 - 1.0) * (e->g2 - 1.0)) / ((e->g2 - 1.0) * a1 + (e->g1 - 1.0) * a2);
    *pi = ((*g - 1.0) / *g) * (e->g1 * e->p1 * a1 / (e->g1 - 1.0) + e->g2 * e->p2 * a2 / (e->g2 - 1.0));
}

void orc_mp_cons2prim(int model, const double* eos4, const double* Q, double* V) {
    Eos e = {model, eos4[0], eos4[1], eos4[2], eos4[3]};
    double g, pi;
    if (model == 0) {
        const double phi = Q[4];
        di4_mix(&e, phi, &g, &pi);
        const double irho = 1.0 / Q[0];
        V[0] = Q[0];
        V[1] = irho * Q[1];
        V[2] = irho * Q[2];
        V[3] = (g - 1.0) * (Q[3] - 0.5 * irho * (Q[1] * Q[1] + Q[2] * Q[2])) - g * pi;
        V[4] = phi;
    } else {
        const double a1 = Q[5], a2 = 1.0 - a1;
        k5_mix(&e, a1, &g, &pi);
        const double rho = Q[0] + Q[1];
        const double u = Q[2] / rho, v = Q[3] / rho, E = Q[4];
        V[0] = Q[0] / a1;
        V[1] = Q[1] / a2;
        V[2] = u;
        V[3] = v;
        V[4] = (g - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - g * pi;
        V[5] = a1;
    }
}

void orc_mp_prim2cons(int model, const double* eos4, const double* V, double* Q) {
    Eos e = {model, eos4[0], eos4[1], eos4[2], eos4[3]};
    double g, pi;
    if (model == 0) {
        di4_mix(&e, V[4], &g, &pi);
        const double en = (V[3] + g * pi) / (g - 1.0);
        const double k = 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2]);
        Q[0] = V[0];
        Q[1] = V[0] * V[1];
        Q[2] = V[0] * V[2];
        Q[3] = k + en;
        Q[4] = V[4];
    } else {
        const double a1 = V[5], a2 = 1.0 - a1;
        k5_mix(&e, a1, &g, &pi);
        const double rho = a1 * V[0] + a2 * V[1];
        const double E = (V[4] + g * pi) / (g - 1.0) + 0.5 * rho * (V[2] * V[2] + V[3] * V[3]);
        Q[0] = a1 * V[0];
        Q[1] = a2 * V[1];
        Q[2] = rho * V[2];
        Q[3] = rho * V[3];
        Q[4] = E;
        Q[5] = a1;
    }
}

/* physical admissibility of a primitive state (pde.c:99-129 for DI4) */
static int pad_ok(const Eos* e, const double* V) {
    double g, pi;
    if (e->model == 0) {
        const double phi = V[4];
        di4_mix(e, phi, &g, &pi);
        if (V[0] < 1.0e-14) return 0;
        if ((V[3] + pi) < 1.0e-12) return 0;
        if (phi < 0.0 || phi > 1.0) return 0;
        return 1;
    }
    const double a1 = V[5];
    k5_mix(e, a1, &g, &pi);
    if (V[0] < 1.0e-14 || V[1] < 1.0e-14) return 0;
    if ((V[4] + pi) < 1.0e-12) return 0;
    if (a1 < 0.0 || a1 > 1.0) return 0;
    return 1;
}

/* Conservative flux of a primitive state (PDEFluxPrim, pde.c:62-97; Kapila
 * PDEFlux kapila_5eqn.c:66-113 written on primitives); the advected fraction's
 * component is phi*u_n (its non-conservative update uses the extra component). */
static double flux_prim(const Eos* e, const double* V, double nx, double ny, double* F, int* bad) {
    double g, pi;
    if (e->model == 0) {
        const double phi = V[4];
        di4_mix(e, phi, &g, &pi);
        const double rho = V[0], u = V[1], v = V[2], p = V[3];
        const double E = (p + g * pi) / (g - 1.0) + 0.5 * rho * (u * u + v * v);
        const double un = u * nx + v * ny;
        const double rhoun = rho * un;
        if (rho < 1.0e-14 || (p + pi) < 1.0e-12) *bad = 1;
        F[0] = rhoun;
        F[1] = rhoun * u + p * nx;
        F[2] = rhoun * v + p * ny;
        F[3] = un * (E + p);
        F[4] = phi * un;
        return fabs(un) + sqrt(g * (p + pi) / rho);
    }
    const double a1 = V[5], a2 = 1.0 - a1;
    k5_mix(e, a1, &g, &pi);
    const double r1 = V[0], r2 = V[1], u = V[2], v = V[3], p = V[4];
    const double rho = a1 * r1 + a2 * r2;
    const double E = (p + g * pi) / (g - 1.0) + 0.5 * rho * (u * u + v * v);
    const double un = u * nx + v * ny;
    if (rho < 1.0e-14 || (p + pi) < 1.0e-12) *bad = 1;
    F[0] = a1 * r1 * un;
    F[1] = a2 * r2 * un;
    F[2] = rho * u * un + p * nx;
    F[3] = rho * v * un + p * ny;
    F[4] = (E + p) * un;
    F[5] = a1 * un;
    return fabs(un) + sqrt(g * (p + pi) / rho);
}

/* HLLC on primitive states with the interface-velocity component appended
 * (HLLCRiemannSolver, 2d/weno4/bubble/pde.c:131-232); nv = 5 (DI4) or 6. */
static double hllc2(const Eos* e, int nv, const double* VL, const double* VR, double nx, double ny, double* Flux, int* bad) {
    double QL[MAXV], QR[MAXV], FL[MAXV + 1], FR[MAXV + 1];
    const double eos4[4] = {e->g1, e->p1, e->g2, e->p2};
    orc_mp_prim2cons(e->model, eos4, VL, QL);
    orc_mp_prim2cons(e->model, eos4, VR, QR);
    const double sl = flux_prim(e, VL, nx, ny, FL, bad);
    const double sr = flux_prim(e, VR, nx, ny, FR, bad);
    double gL, piL, gR, piR;
    double rL, rR, uL, uR, vL, vR, PL, PR, EL, ER;
    if (e->model == 0) {
        gL = 1.0 + (e->g1 - 1.0) * (e->g2 - 1.0) / ((1.0 - VL[4]) * (e->g1 - 1.0) + VL[4] * (e->g2 - 1.0));
        piL = ((gL - 1.0) / gL) * (e->g1 * e->p1 * VL[4] / (e->g1 - 1.0) + e->g2 * e->p2 * (1.0 - VL[4]) / (e->g2 - 1.0));
        gR = 1.0 + (e->g1 - 1.0) * (e->g2 - 1.0) / ((1.0 - VR[4]) * (e->g1 - 1.0) + VR[4] * (e->g2 - 1.0));
        piR = ((gR - 1.0) / gR) * (e->g1 * e->p1 * VR[4] / (e->g1 - 1.0) + e->g2 * e->p2 * (1.0 - VR[4]) / (e->g2 - 1.0));
        rL = VL[0]; uL = VL[1]; vL = VL[2]; PL = VL[3];
        rR = VR[0]; uR = VR[1]; vR = VR[2]; PR = VR[3];
    } else {
        k5_mix(e, VL[5], &gL, &piL);
        k5_mix(e, VR[5], &gR, &piR);
        rL = VL[5] * VL[0] + (1.0 - VL[5]) * VL[1];
        rR = VR[5] * VR[0] + (1.0 - VR[5]) * VR[1];
        uL = VL[2]; vL = VL[3]; PL = VL[4];
        uR = VR[2]; vR = VR[3]; PR = VR[4];
    }
    const double smax = (sl < sr) ? sr : sl;
    const double unL = uL * nx + vL * ny, utL = -uL * ny + vL * nx;
    const double unR = uR * nx + vR * ny, utR = -uR * ny + vR * nx;
    const double cL = sqrt(gL * (PL + piL) / rL), cR = sqrt(gR * (PR + piR) / rR);
    EL = (PL + gL * piL) / (gL - 1.0) + 0.5 * rL * uL * uL + 0.5 * rL * vL * vL;
    ER = (PR + gR * piR) / (gR - 1.0) + 0.5 * rR * uR * uR + 0.5 * rR * vR * vR;
    const double a1 = unR - cR, b1 = unL - cL;
    const double SL = (a1 < b1) ? a1 : b1;
    const double a2 = unL + cL, b2 = unR + cR;
    const double SR = (a2 < b2) ? b2 : a2;
    const double Ss = (PR - PL + rL * unL * (SL - unL) - rR * unR * (SR - unR)) / (rL * (SL - unL) - rR * (SR - unR));
    FL[nv] = unL;
    FR[nv] = unR;
    double UL[MAXV], UR[MAXV], FLs[MAXV + 1], FRs[MAXV + 1];
    if (e->model == 0) {
        UL[0] = rL * (SL - unL) / (SL - Ss);
        UL[1] = UL[0] * (Ss * nx - utL * ny);
        UL[2] = UL[0] * (Ss * ny + utL * nx);
        UL[3] = UL[0] * ((EL / rL) + (Ss - unL) * (Ss + PL / (rL * (SL - unL))));
        UL[4] = VL[4] * (SL - unL) / (SL - Ss);
        UR[0] = rR * (SR - unR) / (SR - Ss);
        UR[1] = UR[0] * (Ss * nx - utR * ny);
        UR[2] = UR[0] * (Ss * ny + utR * nx);
        UR[3] = UR[0] * ((ER / rR) + (Ss - unR) * (Ss + PR / (rR * (SR - unR))));
        UR[4] = VR[4] * (SR - unR) / (SR - Ss);
    } else {
        const double fL = (SL - unL) / (SL - Ss), fR = (SR - unR) / (SR - Ss);
        const double rsL = rL * fL, rsR = rR * fR;
        UL[0] = QL[0] * fL;
        UL[1] = QL[1] * fL;
        UL[2] = rsL * (Ss * nx - utL * ny);
        UL[3] = rsL * (Ss * ny + utL * nx);
        UL[4] = rsL * ((EL / rL) + (Ss - unL) * (Ss + PL / (rL * (SL - unL))));
        UL[5] = VL[5] * fL;
        UR[0] = QR[0] * fR;
        UR[1] = QR[1] * fR;
        UR[2] = rsR * (Ss * nx - utR * ny);
        UR[3] = rsR * (Ss * ny + utR * nx);
        UR[4] = rsR * ((ER / rR) + (Ss - unR) * (Ss + PR / (rR * (SR - unR))));
        UR[5] = VR[5] * fR;
    }
    for (int i = 0; i < nv; i++) FLs[i] = FL[i] + SL * (UL[i] - QL[i]);
    FLs[nv] = unL + SL * (((SL - unL) / (SL - Ss)) - 1.0);
    for (int i = 0; i < nv; i++) FRs[i] = FR[i] + SR * (UR[i] - QR[i]);
    FRs[nv] = unR + SR * (((SR - unR) / (SR - Ss)) - 1.0);
    for (int i = 0; i <= nv; i++) {
        if (SL > 0.0) Flux[i] = FL[i];
        else if (Ss >= 0.0) Flux[i] = FLs[i];
        else if (SR >= 0.0) Flux[i] = FRs[i];
        else Flux[i] = FR[i];
    }
    return smax;
}

/* rotHLLCRiemannSolver (2d/weno4/bubble/pde.c:234-274) */
static double rot_hllc2(const Eos* e, int nv, const double* VL, const double* VR, double nx, double ny, double* Flux, int* bad) {
    const int iu = (e->model == 0) ? 1 : 2;
    const double du = VR[iu] - VL[iu], dv = VR[iu + 1] - VL[iu + 1];
    const double dq = sqrt(du * du + dv * dv);
    double n1x, n1y;
    if (dq < 1.0E-10) {
        n1x = nx; n1y = ny;
    } else {
        n1x = du / dq; n1y = dv / dq;
    }
    double a1 = (n1x * nx + n1y * ny);
    if (a1 < 0) {
        n1x = -n1x; n1y = -n1y; a1 = -a1;
    }
    double n2x = -n1y, n2y = n1x;
    double a2 = (n2x * nx + n2y * ny);
    if (a2 < 0) {
        n2x = -n2x; n2y = -n2y; a2 = -a2;
    }
    double f1[MAXV + 1], f2[MAXV + 1];
    const double s1 = hllc2(e, nv, VL, VR, n1x, n1y, f1, bad);
    const double s2 = hllc2(e, nv, VL, VR, n2x, n2y, f2, bad);
    for (int i = 0; i <= nv; i++) Flux[i] = a1 * f1[i] + a2 * f2[i];
    return (s1 < s2) ? s2 : s1;
}

/* ------------------------------------------------------------------ RHS */
static inline int bmap1(int i, int n, int blo, int bhi, int* flip) {
    if (i < 0) {
        if (blo == ORC_BC_PERIODIC) return i + n;
        if (blo == ORC_BC_TRANSMISSIVE) return 0;
        *flip = 1;
        return -1 - i;
    }
    if (i >= n) {
        if (bhi == ORC_BC_PERIODIC) return i - n;
        if (bhi == ORC_BC_TRANSMISSIVE) return n - 1;
        *flip = 1;
        return 2 * (n - 1) - i + 1;
    }
    return i;
}

int orc_mp2d_rhs(const orc_mp2d_cfg* g, const double* U, double* RHS, double* smax_out, long* bad_out, long* fallback_out) {
    const int nx = g->nx, ny = g->ny, nv = g->model == 0 ? 5 : 6;
    const Eos e = {g->model, g->g1, g->p1, g->g2, g->p2};
    const double eos4[4] = {g->g1, g->p1, g->g2, g->p2};
    const int iu = (g->model == 0) ? 1 : 2; /* x-velocity slot of the primitive state */
#ifdef _OPENMP
    if (g->nthreads > 0) omp_set_num_threads(g->nthreads);
#endif
    const int gx = nx + 6, gy = ny + 6;
    double* W = (double*)malloc(sizeof(double) * (size_t)gx * gy * nv);
    double* Pc = (double*)malloc(sizeof(double) * (size_t)nx * ny * nv);
    const int tx = nx + 2, ty = ny + 2;
    double* T = (double*)malloc(sizeof(double) * (size_t)tx * ty * nv * 8);
    double* F = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny * (nv + 1));
    double* G = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1) * (nv + 1));
    if (!W || !Pc || !T || !F || !G) return 3;
    /* primitive variables (ComputePrimitiveVariables) then the ghosted primitive array */
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)nx * ny; ++q) orc_mp_cons2prim(g->model, eos4, U + q * nv, Pc + q * nv);
#pragma omp parallel for schedule(static)
    for (int j = -3; j < ny + 3; ++j)
        for (int i = -3; i < nx + 3; ++i) {
            int fx = 0, fy = 0;
            int si = bmap1(i, nx, g->bc[0], g->bc[1], &fx);
            int sj = bmap1(j, ny, g->bc[2], g->bc[3], &fy);
            double* o = W + ((size_t)(j + 3) * gx + (i + 3)) * nv;
            const double* s = Pc + ((size_t)sj * nx + si) * nv;
            for (int c = 0; c < nv; ++c) o[c] = s[c];
            if (fx) o[iu] = -o[iu];
            if (fy) o[iu + 1] = -o[iu + 1];
        }
#define WP(i, j) (W + ((size_t)((j) + 3) * gx + ((i) + 3)) * nv)
    double phiF[4][2][NDOF], phiN[8][NDOF];
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < NDOF; ++k) {
            phiF[0][q][k] = basis2(-0.5, X_GP2[q], k);
            phiF[1][q][k] = basis2(0.5, X_GP2[q], k);
            phiF[2][q][k] = basis2(X_GP2[q], -0.5, k);
            phiF[3][q][k] = basis2(X_GP2[q], 0.5, k);
        }
    for (int q = 0; q < 8; ++q)
        for (int k = 0; k < NDOF; ++k) phiN[q][k] = basis2(X_NODE[q], Y_NODE[q], k);
    long fallback = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : fallback)
    for (int j = -1; j <= ny; ++j)
        for (int i = -1; i <= nx; ++i) {
            if ((i < 0 || i >= nx) && (j < 0 || j >= ny)) continue; /* corners feed no face */
            double sol[NDOF][MAXV], VN[8][MAXV];
            for (int c = 0; c < nv; ++c) {
                double ux[5], uy[5], cf[NDOF];
                for (int o = 0; o < 5; ++o) {
                    ux[o] = WP(i + o - 2, j)[c];
                    uy[o] = WP(i, j + o - 2)[c];
                }
                orc_cweno4_2d(WP(i, j)[c], ux, uy, WP(i + 1, j + 1)[c], WP(i + 1, j - 1)[c], WP(i - 1, j + 1)[c],
                              WP(i - 1, j - 1)[c], cf);
                for (int k = 0; k < NDOF; ++k) sol[k][c] = cf[k];
                for (int q = 0; q < 8; ++q) {
                    VN[q][c] = 0.0;
                    for (int k = 0; k < NDOF; ++k) VN[q][c] += cf[k] * phiN[q][k];
                }
            }
            int ok = 1;
            for (int q = 0; q < 8 && ok; ++q) ok = pad_ok(&e, VN[q]);
            if (!ok) {
                ++fallback;
                for (int c = 0; c < nv; ++c) {
                    const double w0 = WP(i, j)[c];
                    sol[0][c] = w0;
                    sol[1][c] = minmod(WP(i + 1, j)[c] - w0, w0 - WP(i - 1, j)[c]);
                    sol[2][c] = minmod(WP(i, j + 1)[c] - w0, w0 - WP(i, j - 1)[c]);
                    for (int k = 3; k < NDOF; ++k) sol[k][c] = 0.0;
                }
            }
            double* t = T + ((size_t)(j + 1) * tx + (i + 1)) * nv * 8;
            for (int c = 0; c < nv; ++c)
                for (int f = 0; f < 4; ++f)
                    for (int q = 0; q < 2; ++q) {
                        double v = 0.0;
                        for (int k = 0; k < NDOF; ++k) v += sol[k][c] * phiF[f][q][k];
                        t[c * 8 + f * 2 + q] = v;
                    }
        }
#define TP(i, j) (T + ((size_t)((j) + 1) * tx + ((i) + 1)) * nv * 8)
    double smax = 0.0;
    long bad = -1;
    int badx = 0, bady = 0;
#pragma omp parallel for schedule(static) reduction(max : smax) reduction(| : badx)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            double Fl[MAXV + 1];
            double* Fo = F + ((size_t)j * (nx + 1) + i) * (nv + 1);
            for (int c = 0; c <= nv; ++c) Fo[c] = 0.0;
            for (int q = 0; q < 2; ++q) {
                double VL[MAXV], VR[MAXV];
                for (int c = 0; c < nv; ++c) {
                    VL[c] = TP(i - 1, j)[c * 8 + 1 * 2 + q];
                    VR[c] = TP(i, j)[c * 8 + 0 * 2 + q];
                }
                int b = 0;
                double s = rot_hllc2(&e, nv, VL, VR, 1.0, 0.0, Fl, &b);
                badx |= b;
                if (s > smax) smax = s;
                for (int c = 0; c <= nv; ++c) Fo[c] += 0.5 * Fl[c];
            }
        }
#pragma omp parallel for schedule(static) reduction(max : smax) reduction(| : bady)
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i) {
            double Fl[MAXV + 1];
            double* Fo = G + ((size_t)j * nx + i) * (nv + 1);
            for (int c = 0; c <= nv; ++c) Fo[c] = 0.0;
            for (int q = 0; q < 2; ++q) {
                double VL[MAXV], VR[MAXV];
                for (int c = 0; c < nv; ++c) {
                    VL[c] = TP(i, j - 1)[c * 8 + 3 * 2 + q];
                    VR[c] = TP(i, j)[c * 8 + 2 * 2 + q];
                }
                int b = 0;
                double s = rot_hllc2(&e, nv, VL, VR, 0.0, 1.0, Fl, &b);
                bady |= b;
                if (s > smax) smax = s;
                for (int c = 0; c <= nv; ++c) Fo[c] += 0.5 * Fl[c];
            }
        }
    if (badx || bady) bad = 0;
    const double r1_h = 1. / (g->h);
    const int ia = nv - 1; /* advected volume fraction */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            double* r = RHS + ((size_t)j * nx + i) * nv;
            const double* Fl = F + ((size_t)j * (nx + 1) + i) * (nv + 1);
            const double* Fr = Fl + (nv + 1);
            const double* Gl = G + ((size_t)j * nx + i) * (nv + 1);
            const double* Gr = G + ((size_t)(j + 1) * nx + i) * (nv + 1);
            const double a = WP(i, j)[ia];
            for (int c = 0; c < nv; ++c) {
                if (c == ia)
                    r[c] = -r1_h * ((Fr[c] - a * Fr[c + 1]) - (Fl[c] - a * Fl[c + 1])) -
                           r1_h * ((Gr[c] - a * Gr[c + 1]) - (Gl[c] - a * Gl[c + 1]));
                else
                    r[c] = -r1_h * (Fr[c] - Fl[c]) - r1_h * (Gr[c] - Gl[c]);
            }
        }
#undef WP
#undef TP
    free(W); free(Pc); free(T); free(F); free(G);
    if (smax_out) *smax_out = smax;
    if (bad_out) *bad_out = bad;
    if (fallback_out) *fallback_out = fallback;
    return bad >= 0 ? 2 : 0;
}

/* dt = CFL h / (2 s_max) (rhs_function.c:385) */
static inline double mp_dt(const orc_mp2d_cfg* g, double smax) { return (g->cfl * g->h) / (2.0 * smax); }

/* stepper 0: SSPRK(4,3); stepper 1: SSPRK(10,4) (PETSc TSSSP RK104, Ketcheson 2008) */
int orc_mp2d_run(const orc_mp2d_cfg* g, int nsteps, int stepper, int dt_mode, double* U, double* t_inout, double* dt_inout,
                 long* bad) {
    const int nv = g->model == 0 ? 5 : 6;
    const size_t n = (size_t)g->nx * g->ny * nv;
    double* w0 = (double*)malloc(sizeof(double) * n);
    double* w1 = (double*)malloc(sizeof(double) * n);
    double* F = (double*)malloc(sizeof(double) * n);
    double smax = 0.0;
    double t = t_inout ? *t_inout : 0.0;
    long fb = 0;
    int rc = orc_mp2d_rhs(g, U, F, &smax, bad, &fb); /* initial RHS sets dt (hype.c:202-204) */
    double dt = (dt_mode == 2) ? *dt_inout : mp_dt(g, smax);
    for (int s = 0; s < nsteps && !rc; ++s) {
        if (stepper == 0) {
            const double dtr = dt / 2;
            if (s > 0) rc = orc_mp2d_rhs(g, U, F, &smax, bad, &fb);
            if (rc) break;
            for (size_t q = 0; q < n; ++q) w0[q] = U[q] + dtr * F[q];
            if ((rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
            for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dtr * F[q];
            if ((rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
            const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * dt / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
            for (size_t q = 0; q < n; ++q) w0[q] = a3 * U[q] + b3 * F[q] + c3 * w0[q];
            if ((rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
            for (size_t q = 0; q < n; ++q) U[q] = w0[q] + dtr * F[q];
        } else {
            memcpy(w0, U, sizeof(double) * n);
            memcpy(w1, U, sizeof(double) * n);
            int i;
            for (i = 0; i < 5; ++i) {
                if (!(s == 0 && i == 0) && (rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
                for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dt / 6 * F[q];
            }
            if (rc) break;
            for (size_t q = 0; q < n; ++q) w1[q] = 9.0 / 25 * w0[q] + 1.0 / 25 * w1[q];
            for (size_t q = 0; q < n; ++q) w0[q] = 15 * w1[q] + -5 * w0[q];
            for (; i < 9; ++i) {
                if ((rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
                for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dt / 6 * F[q];
            }
            if (rc) break;
            if ((rc = orc_mp2d_rhs(g, w0, F, &smax, bad, &fb))) break;
            for (size_t q = 0; q < n; ++q) w1[q] = 3.0 / 5 * w0[q] + dt / 10 * F[q] + 1 * w1[q];
            memcpy(U, w1, sizeof(double) * n);
        }
        t += dt;
        if (dt_mode == 0) dt = mp_dt(g, smax);
    }
    free(w0); free(w1); free(F);
    if (t_inout) *t_inout = t;
    if (dt_inout) *dt_inout = dt;
    return rc;
}
