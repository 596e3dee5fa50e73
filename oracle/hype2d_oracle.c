/*
 * hype2d_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of the 2D
 * path-conservative RHS of 2d/HyPE-2D with its Kapila five-equation model (the
 * checker the GPU path is compared with; never linked into the product).
 *
 *   RHSFunction            2d/HyPE-2D/rhs_function.c:12-610 (conservative variables)
 *     boundary ghosts      :62-300 (transmissive copy, periodic by the DMDA, reflective
 *                           mirror with the normal momentum negated -- for this model
 *                           components 2 (x) and 3 (y))
 *     reconstruction       :304-330, Reconstruct / weno2 / weno3 / weno4 of
 *                           reconstruction.c:129-377 for the order N = 0..3
 *     admissibility        :338-365 (PDECheckPAD at the N_node nodes; on failure the cell
 *                           is first order -- the minmod slopes it computes are zeroed,
 *                           rhs_function.c:352-362)
 *     traces, volume term  :368-410 (face values from the basis tables; the
 *                           non-conservative product PDENCP integrated over the cell)
 *     fluxes               :414-510 (RiemannSolver: Rusanov flux + the Roe-path
 *                           fluctuation B~(QL, QR) (QR - QL), riemann.c:13-85)
 *     RHS, dt              :514-600 (dt = CFL h / (2 s_max))
 *   Kapila model           kapila_5eqn.c:14-281 (mixture gamma / pi from alpha_1, K = 0)
 *   basis tables           hype.c:230-330
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "hype_oracle.h"

#define KV 6
static const double KP_RHO_FLOOR = 1.0e-14, KP_PRS_FLOOR = 1.0e-12, KP_SMALL = 1.0e-12;

/* ---------------------------------------------------------------- basis (reconstruction.c:11-100) */
static double h2_basis(double x, double y, int n) {
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

static void h2_basis_grad(double x, double y, int n, double* gx, double* gy) {
    switch (n) {
        case 0: *gx = 0.0; *gy = 0.0; break;
        case 1: *gx = 1.0; *gy = 0.0; break;
        case 2: *gx = 0.0; *gy = 1.0; break;
        case 3: *gx = 2.0 * x; *gy = 0.0; break;
        case 4: *gx = 0.0; *gy = 2.0 * y; break;
        case 5: *gx = y; *gy = x; break;
        case 6: *gx = 3.0 * x * x - 3. / 20.; *gy = 0.0; break;
        case 7: *gx = 0.0; *gy = 3.0 * y * y - 3. / 20.; break;
        case 8: *gx = 2.0 * x * y; *gy = (x * x - 1. / 12.); break;
        case 9: *gx = (y * y - 1. / 12.); *gy = 2.0 * x * y; break;
        default: *gx = 0.0; *gy = 0.0;
    }
}

static double h2_minmod(double a, double b) {
    if (a * b < 0.0) return 0.0;
    return (fabs(a) < fabs(b)) ? a : b;
}

static double h2_pow4(double a) {
    const double a2 = a * a;
    return a2 * a2;
}

/* weno2 (reconstruction.c:129-142): minmod slopes */
static void h2_weno2(const double* U_x, const double* U_y, const double* U_xy, double* c) {
    const double u_0 = U_xy[0], u_ip1 = U_x[3], u_jp1 = U_y[3], u_im1 = U_x[1], u_jm1 = U_y[1];
    c[0] = u_0;
    c[1] = h2_minmod(u_ip1 - u_0, u_0 - u_im1);
    c[2] = h2_minmod(u_jp1 - u_0, u_0 - u_jm1);
}

/* weno3 (reconstruction.c:144-221): third order, central weight 100 */
static void h2_weno3_axis(double u_m2, double u_m1, double u_0, double u_p1, double u_p2, double* c1, double* c2) {
    const double cw = 100.0, r13_3 = 13. / 3.;
    double u_x[3], u_xx[3], IS[3], wt[3], total;
    u_x[0] = -2.0 * u_m1 + 0.5 * u_m2 + 1.5 * u_0; u_xx[0] = 0.5 * (u_m2 - 2.0 * u_m1 + u_0);
    u_x[1] = 0.5 * (u_p1 - u_m1);                  u_xx[1] = 0.5 * (u_m1 - 2.0 * u_0 + u_p1);
    u_x[2] = -1.5 * u_0 + 2.0 * u_p1 - 0.5 * u_p2; u_xx[2] = 0.5 * (u_0 - 2.0 * u_p1 + u_p2);
    IS[0] = u_x[0] * u_x[0] + r13_3 * u_xx[0] * u_xx[0]; wt[0] = 1.0 / (h2_pow4(IS[0] + KP_SMALL));
    IS[1] = u_x[1] * u_x[1] + r13_3 * u_xx[1] * u_xx[1]; wt[1] = cw / (h2_pow4(IS[1] + KP_SMALL));
    IS[2] = u_x[2] * u_x[2] + r13_3 * u_xx[2] * u_xx[2]; wt[2] = 1.0 / (h2_pow4(IS[2] + KP_SMALL));
    total = wt[0] + wt[1] + wt[2];
    wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total;
    *c1 = wt[0] * u_x[0] + wt[1] * u_x[1] + wt[2] * u_x[2];
    *c2 = wt[0] * u_xx[0] + wt[1] * u_xx[1] + wt[2] * u_xx[2];
}

static void h2_weno3(const double* U_x, const double* U_y, const double* U_xy, double* c) {
    const double u_0 = U_xy[0];
    const double u_ip1jp1 = U_xy[1], u_ip1jm1 = U_xy[2], u_im1jp1 = U_xy[3], u_im1jm1 = U_xy[4];
    double u_xy[4], IS[4], wt[4], total, temp;
    c[0] = u_0;
    h2_weno3_axis(U_x[0], U_x[1], u_0, U_x[3], U_x[4], &c[1], &c[3]);
    h2_weno3_axis(U_y[0], U_y[1], u_0, U_y[3], U_y[4], &c[2], &c[4]);
    u_xy[0] = u_ip1jp1 - u_0 - c[1] - c[2] - c[3] - c[4];
    u_xy[1] = -u_ip1jm1 + u_0 + c[1] - c[2] + c[3] + c[4];
    u_xy[2] = -u_im1jp1 + u_0 - c[1] + c[2] + c[3] + c[4];
    u_xy[3] = u_im1jm1 - u_0 + c[1] + c[2] - c[3] - c[4];
    temp = 4.0 * (c[3] * c[3] + c[4] * c[4]);
    for (int q = 0; q < 4; ++q) {
        IS[q] = temp + u_xy[q] * u_xy[q];
        wt[q] = 1.0 / (h2_pow4(IS[q] + KP_SMALL));
    }
    total = wt[0] + wt[1] + wt[2] + wt[3];
    wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total; wt[3] = wt[3] / total;
    c[5] = wt[0] * u_xy[0] + wt[1] * u_xy[1] + wt[2] * u_xy[2] + wt[3] * u_xy[3];
}

/* ---------------------------------------------------------------- Kapila model */
static inline void kp_mix(const orc_h2d_cfg* e, double a1, double* G, double* P) {
    const double a2 = 1.0 - a1;
    const double GAMMA = 1.0 + ((e->g1 - 1.0) * (e->g2 - 1.0)) / ((e->g2 - 1.0) * a1 + (e->g1 - 1.0) * a2);
    *G = GAMMA;
    *P = ((GAMMA - 1.0) / GAMMA) * (e->g1 * e->p1 * a1 / (e->g1 - 1.0) + e->g2 * e->p2 * a2 / (e->g2 - 1.0));
}

/* PDEFlux (kapila_5eqn.c:66-117) */
static double kp_flux(const orc_h2d_cfg* e, const double* Q, double nx, double ny, double* F, int* bad) {
    const double a1 = Q[5], a2 = 1.0 - a1;
    double GAMMA, PI;
    kp_mix(e, a1, &GAMMA, &PI);
    const double rho_1 = Q[0] / a1, rho_2 = Q[1] / a2;
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (GAMMA - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - GAMMA * PI;
    const double un = u * nx + v * ny;
    if (rho < KP_RHO_FLOOR) *bad = 1;
    if (p + PI < KP_PRS_FLOOR) *bad = 1;
    F[0] = a1 * rho_1 * un;
    F[1] = a2 * rho_2 * un;
    F[2] = rho * u * un + p * nx;
    F[3] = rho * v * un + p * ny;
    F[4] = (E + p) * un;
    F[5] = 0.0;
    return fabs(un) + sqrt(GAMMA * (p + PI) * irho);
}

/* PDENCP (kapila_5eqn.c:164-199) */
static void kp_ncp(const orc_h2d_cfg* e, const double* Q, const double* gx, const double* gy, double* B) {
    const double a1 = Q[5], a2 = 1.0 - a1;
    double GAMMA, PI;
    kp_mix(e, a1, &GAMMA, &PI);
    const double rho_1 = Q[0] / a1, rho_2 = Q[1] / a2;
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (GAMMA - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - GAMMA * PI;
    const double a_1_sq = e->g1 * (p + e->p1) / rho_1, a_2_sq = e->g2 * (p + e->p2) / rho_2;
    double K = a1 * a2 * (rho_2 * a_2_sq - rho_1 * a_1_sq) / (a1 * rho_2 * a_2_sq + a2 * rho_1 * a_1_sq);
    const double u_x = irho * irho * (gx[2] * rho - Q[2] * (gx[0] + gx[1]));
    const double v_y = irho * irho * (gy[3] * rho - Q[3] * (gy[0] + gy[1]));
    K = 0.0;
    B[0] = 0.0; B[1] = 0.0; B[2] = 0.0; B[3] = 0.0; B[4] = 0.0;
    B[5] = u * gx[5] + v * gy[5] - K * (u_x + v_y);
}

/* PDEmatrixB (kapila_5eqn.c:205-240) */
static void kp_matrix_b(const orc_h2d_cfg* e, const double* Q, double nx, double ny, double B[KV][KV]) {
    const double a1 = Q[5], a2 = 1.0 - a1;
    double GAMMA, PI;
    kp_mix(e, a1, &GAMMA, &PI);
    const double rho_1 = Q[0] / a1, rho_2 = Q[1] / a2;
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (GAMMA - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - GAMMA * PI;
    const double a_1_sq = e->g1 * (p + e->p1) / rho_1, a_2_sq = e->g2 * (p + e->p2) / rho_2;
    double K = a1 * a2 * (rho_2 * a_2_sq - rho_1 * a_1_sq) / (a1 * rho_2 * a_2_sq + a2 * rho_1 * a_1_sq);
    const double un = u * nx + v * ny;
    K = 0.0;
    for (int i = 0; i < KV; ++i)
        for (int j = 0; j < KV; ++j) B[i][j] = 0.0;
    B[5][0] = irho * K * un;
    B[5][1] = irho * K * un;
    B[5][2] = -irho * K * nx;
    B[5][3] = -irho * K * ny;
    B[5][5] = un;
}

/* PDECheckPAD (kapila_5eqn.c:248-281) */
static int kp_pad(const orc_h2d_cfg* e, const double* Q) {
    const double phi_1 = Q[5], phi_2 = 1.0 - phi_1;
    const double temp = phi_1 / (e->g1 - 1.0) + phi_2 / (e->g2 - 1.0);
    const double gamma = 1.0 + 1.0 / temp;
    const double pi = (phi_1 * e->g1 * e->p1 / (e->g1 - 1.0) + phi_2 * e->g2 * e->p2 / (e->g2 - 1.0)) / (1.0 + temp);
    const double rho = Q[0] + Q[1], irho = 1.0 / rho;
    const double u = irho * Q[2], v = irho * Q[3], E = Q[4];
    const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v)) - gamma * pi;
    int pad = 1;
    if (rho < KP_RHO_FLOOR) pad = 0;
    if ((p + pi) < KP_PRS_FLOOR) pad = 0;
    if (phi_1 < 1.0e-4 || phi_1 > 1.0 - 1.0e-4) pad = 0;
    return pad;
}

/* RiemannSolver with RoeMatrix (riemann.c:13-85) */
static double kp_riemann(const orc_h2d_cfg* e, const double* QL, const double* QR, double nx, double ny, double* F,
                         double* D, int* bad) {
    static const double s_gp[3] = {0.1127016653792583, 0.5, 0.8872983346207417};
    static const double w_gp[3] = {0.2777777777777778, 0.4444444444444444, 0.2777777777777778};
    double FL[KV], FR[KV], J[KV], BR[KV][KV], B[KV][KV], Q[KV];
    const double sl = kp_flux(e, QL, nx, ny, FL, bad), sr = kp_flux(e, QR, nx, ny, FR, bad);
    const double s_max = sl < sr ? sr : sl;
    for (int c = 0; c < KV; ++c) {
        J[c] = QR[c] - QL[c];
        F[c] = 0.5 * (FR[c] + FL[c] - s_max * J[c]);
    }
    for (int i = 0; i < KV; ++i)
        for (int j = 0; j < KV; ++j) BR[i][j] = 0.0;
    for (int q = 0; q < 3; ++q) {
        for (int c = 0; c < KV; ++c) Q[c] = QL[c] + s_gp[q] * (QR[c] - QL[c]);
        kp_matrix_b(e, Q, nx, ny, B);
        for (int i = 0; i < KV; ++i)
            for (int j = 0; j < KV; ++j) BR[i][j] += w_gp[q] * B[i][j];
    }
    for (int i = 0; i < KV; ++i) {
        D[i] = 0.0;
        for (int j = 0; j < KV; ++j) D[i] += BR[i][j] * J[j];
    }
    return s_max;
}

/* ---------------------------------------------------------------- RHS */
static int h2_map(int i, int n, int blo, int bhi, int* flip) {
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

int orc_h2d_rhs(const orc_h2d_cfg* e, const double* U, double* RHS, double* dt_out) {
    const int nx = e->nx, ny = e->ny, N = e->N;
    const int nDOF = (N + 1) * (N + 2) / 2, ngf = N < 2 ? 1 : 2, ngv = N < 2 ? 1 : 4, nnode = 4 * ngf;
    const double r1_h = 1. / (e->h);
    const double g = 0.28867513459481287;
    double xgf[2], wgf[2], xgv[4], ygv[4], wgv[4], xn[8], yn[8];
    if (N < 2) {
        xgf[0] = 0.0; wgf[0] = 1.0;
        xgv[0] = 0.0; ygv[0] = 0.0; wgv[0] = 1.0;
        xn[0] = 0.5; yn[0] = 0.0; xn[1] = -0.5; yn[1] = 0.0; xn[2] = 0.0; yn[2] = 0.5; xn[3] = 0.0; yn[3] = -0.5;
    } else {
        xgf[0] = -g; wgf[0] = 0.5; xgf[1] = g; wgf[1] = 0.5;
        xgv[0] = -g; ygv[0] = -g; xgv[1] = -g; ygv[1] = g; xgv[2] = g; ygv[2] = -g; xgv[3] = g; ygv[3] = g;
        wgv[0] = wgv[1] = wgv[2] = wgv[3] = 0.25;
        xn[0] = 0.5; yn[0] = -g; xn[1] = 0.5; yn[1] = g; xn[2] = -0.5; yn[2] = -g; xn[3] = -0.5; yn[3] = g;
        xn[4] = -g; yn[4] = 0.5; xn[5] = g; yn[5] = 0.5; xn[6] = -g; yn[6] = -0.5; xn[7] = g; yn[7] = -0.5;
    }
    double phiF[4][2][10], phiN[8][10], phiV[4][10], gvx[4][10], gvy[4][10];
    for (int q = 0; q < ngf; ++q)
        for (int k = 0; k < nDOF; ++k) {
            const double xf[4] = {-0.5, 0.5, xgf[q], xgf[q]}, yf[4] = {xgf[q], xgf[q], -0.5, 0.5};
            for (int f = 0; f < 4; ++f) phiF[f][q][k] = h2_basis(xf[f], yf[f], k);
        }
    for (int q = 0; q < nnode; ++q)
        for (int k = 0; k < nDOF; ++k) phiN[q][k] = h2_basis(xn[q], yn[q], k);
    for (int q = 0; q < ngv; ++q)
        for (int k = 0; k < nDOF && k < 10; ++k) {
            phiV[q][k] = h2_basis(xgv[q], ygv[q], k);
            h2_basis_grad(xgv[q], ygv[q], k, &gvx[q][k], &gvy[q][k]);
        }
#ifdef _OPENMP
    if (e->nthreads > 0) omp_set_num_threads(e->nthreads);
#endif
    const int gx = nx + 6, gy = ny + 6, ex = nx + 2, ey = ny + 2;
    double* P = (double*)malloc(sizeof(double) * (size_t)gx * gy * KV);
    double* T = (double*)malloc(sizeof(double) * (size_t)ex * ey * KV * 4 * 2);
    double* F = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny * KV);
    double* Dx = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny * KV);
    double* G = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1) * KV);
    double* Ey = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1) * KV);
    if (!P || !T || !F || !Dx || !G || !Ey) return 3;
#define PP(i, j) (P + ((size_t)((j) + 3) * gx + ((i) + 3)) * KV)
#define TT(i, j) (T + ((size_t)((j) + 1) * ex + ((i) + 1)) * KV * 8)
    for (int j = -3; j < ny + 3; ++j)
        for (int i = -3; i < nx + 3; ++i) {
            int fx = 0, fy = 0;
            const int si = h2_map(i, nx, e->bc[0], e->bc[1], &fx), sj = h2_map(j, ny, e->bc[2], e->bc[3], &fy);
            double* o = PP(i, j);
            memcpy(o, U + ((size_t)sj * nx + si) * KV, sizeof(double) * KV);
            if (fx) o[2] = -o[2];
            if (fy) o[3] = -o[3];
        }
    /* per extended cell: reconstruction, admissibility, traces; owned cells: the volume term */
#pragma omp parallel for schedule(static)
    for (int j = -1; j < ny + 1; ++j)
        for (int i = -1; i < nx + 1; ++i) {
            double sol[10][KV], QN[8][KV];
            for (int c = 0; c < KV; ++c) {
                double ux[5], uy[5], uxy[5], cf[10];
                for (int o = -2; o < 3; ++o) {
                    ux[o + 2] = PP(i + o, j)[c];
                    uy[o + 2] = PP(i, j + o)[c];
                }
                uxy[0] = PP(i, j)[c]; uxy[1] = PP(i + 1, j + 1)[c]; uxy[2] = PP(i + 1, j - 1)[c];
                uxy[3] = PP(i - 1, j + 1)[c]; uxy[4] = PP(i - 1, j - 1)[c];
                if (N == 0) cf[0] = uxy[0];
                else if (N == 1) h2_weno2(ux, uy, uxy, cf);
                else if (N == 2) h2_weno3(ux, uy, uxy, cf);
                else orc_cweno4_2d(uxy[0], ux, uy, uxy[1], uxy[2], uxy[3], uxy[4], cf);
                for (int k = 0; k < nDOF; ++k) sol[k][c] = cf[k];
                for (int q = 0; q < nnode; ++q) {
                    QN[q][c] = 0.0;
                    for (int k = 0; k < nDOF; ++k) QN[q][c] += cf[k] * phiN[q][k];
                }
            }
            int pad = 1;
            for (int q = 0; q < nnode && pad; ++q) pad = kp_pad(e, QN[q]);
            if (!pad)
                for (int c = 0; c < KV; ++c) {
                    sol[0][c] = PP(i, j)[c];
                    for (int k = 1; k < nDOF; ++k) sol[k][c] = 0.0;
                }
            double* t = TT(i, j);
            for (int c = 0; c < KV; ++c)
                for (int f = 0; f < 4; ++f)
                    for (int q = 0; q < ngf; ++q) {
                        double value = 0.0;
                        for (int k = 0; k < nDOF; ++k) value += sol[k][c] * phiF[f][q][k];
                        t[(c * 4 + f) * 2 + q] = value;
                    }
            if (i >= 0 && i < nx && j >= 0 && j < ny) {
                double Qg[4][KV], gxv[4][KV], gyv[4][KV];
                for (int c = 0; c < KV; ++c)
                    for (int q = 0; q < ngv; ++q) {
                        double value = 0.0, gxs = 0.0, gys = 0.0;
                        for (int k = 0; k < nDOF; ++k) {
                            value += sol[k][c] * phiV[q][k];
                            gxs += sol[k][c] * gvx[q][k];
                            gys += sol[k][c] * gvy[q][k];
                        }
                        Qg[q][c] = value;
                        gxv[q][c] = r1_h * gxs;
                        gyv[q][c] = r1_h * gys;
                    }
                double* r = RHS + ((size_t)j * nx + i) * KV;
                for (int c = 0; c < KV; ++c) r[c] = 0.0;
                for (int q = 0; q < ngv; ++q) {
                    double B[KV];
                    kp_ncp(e, Qg[q], gxv[q], gyv[q], B);
                    for (int c = 0; c < KV; ++c) r[c] += -wgv[q] * B[c];
                }
            }
        }
    double smax = 0.0;
    int bad = 0;
    for (int d = 0; d < 2; ++d) {
        const int fx = nx + (d == 0), fy = ny + (d == 1);
        double* Fd = d == 0 ? F : G;
        double* Dd = d == 0 ? Dx : Ey;
        const double nxv = d == 0 ? 1.0 : 0.0, nyv = d == 1 ? 1.0 : 0.0;
        double sm = 0.0;
        int bd = 0;
#pragma omp parallel for schedule(static) reduction(max : sm) reduction(| : bd)
        for (int j = 0; j < fy; ++j)
            for (int i = 0; i < fx; ++i) {
                const double* tl = TT(i - (d == 0), j - (d == 1));
                const double* tr = TT(i, j);
                double flux[KV], ncp[KV];
                for (int c = 0; c < KV; ++c) flux[c] = ncp[c] = 0.0;
                for (int q = 0; q < ngf; ++q) {
                    double QL[KV], QR[KV], fc[KV], fl[KV];
                    for (int c = 0; c < KV; ++c) {
                        QL[c] = tl[(c * 4 + 2 * d + 1) * 2 + q];
                        QR[c] = tr[(c * 4 + 2 * d) * 2 + q];
                    }
                    int b = 0;
                    const double s = kp_riemann(e, QL, QR, nxv, nyv, fc, fl, &b);
                    if (s > sm) sm = s;
                    bd |= b;
                    for (int c = 0; c < KV; ++c) {
                        flux[c] += wgf[q] * fc[c];
                        ncp[c] += wgf[q] * fl[c];
                    }
                }
                for (int c = 0; c < KV; ++c) {
                    Fd[((size_t)j * fx + i) * KV + c] = flux[c];
                    Dd[((size_t)j * fx + i) * KV + c] = ncp[c];
                }
            }
        if (sm > smax) smax = sm;
        bad |= bd;
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            double* r = RHS + ((size_t)j * nx + i) * KV;
            const size_t il = ((size_t)j * (nx + 1) + i) * KV, jl = ((size_t)j * nx + i) * KV;
            for (int c = 0; c < KV; ++c)
                r[c] += -r1_h * (F[il + KV + c] - F[il + c] + 0.5 * (Dx[il + KV + c] + Dx[il + c])) -
                        r1_h * (G[jl + (size_t)nx * KV + c] - G[jl + c] + 0.5 * (Ey[jl + (size_t)nx * KV + c] + Ey[jl + c]));
        }
#undef PP
#undef TT
    free(P); free(T); free(F); free(Dx); free(G); free(Ey);
    if (dt_out) *dt_out = (e->cfl * e->h) / (2.0 * smax);
    return bad ? 2 : 0;
}

/* nsteps with the program's stepper for N (hype.c:361-382: Euler, SSP RKS2 / 2 stages,
 * RKS3 / 4 stages, RK104) and the dt of the initial RHS call, kept for every step (the
 * program's monitor leaves TSSetTimeStep commented out) */
int orc_h2d_run(const orc_h2d_cfg* e, int nsteps, double* U, double* t_out, double* dt_out) {
    const size_t n = (size_t)e->nx * e->ny * KV;
    double* w0 = (double*)malloc(sizeof(double) * n);
    double* w1 = (double*)malloc(sizeof(double) * n);
    double* L = (double*)malloc(sizeof(double) * n);
    if (!w0 || !w1 || !L) return 3;
    double dt = 0.0, t = 0.0;
    int rc = orc_h2d_rhs(e, U, L, &dt);
    for (int s = 0; s < nsteps && !rc; ++s) {
        if (e->N == 0) {
            if ((rc = orc_h2d_rhs(e, U, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) U[q] = U[q] + dt * L[q];
        } else if (e->N == 1) {
            memcpy(w0, U, sizeof(double) * n);
            if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dt / (2 - 1.0) * L[q];
            if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) U[q] = 1.0 / 2 * U[q] + dt / 2 * L[q] + (2 - 1.0) / 2 * w0[q];
        } else if (e->N == 2) {
            const double dtr = dt / 2;
            const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * dt / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
            if ((rc = orc_h2d_rhs(e, U, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) w0[q] = U[q] + dtr * L[q];
            if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dtr * L[q];
            if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) w0[q] = a3 * U[q] + b3 * L[q] + c3 * w0[q];
            if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) U[q] = w0[q] + dtr * L[q];
        } else {
            memcpy(w0, U, sizeof(double) * n);
            memcpy(w1, U, sizeof(double) * n);
            int i = 0;
            for (; i < 5; ++i) {
                if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
                for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dt / 6 * L[q];
            }
            if (rc) break;
            for (size_t q = 0; q < n; ++q) w1[q] = 9.0 / 25 * w0[q] + 1.0 / 25 * w1[q];
            for (size_t q = 0; q < n; ++q) w0[q] = 15 * w1[q] + -5 * w0[q];
            for (; i < 9; ++i) {
                if ((rc = orc_h2d_rhs(e, w0, L, NULL))) break;
                for (size_t q = 0; q < n; ++q) w0[q] = w0[q] + dt / 6 * L[q];
            }
            if (rc || (rc = orc_h2d_rhs(e, w0, L, NULL))) break;
            for (size_t q = 0; q < n; ++q) U[q] = 3.0 / 5 * w0[q] + dt / 10 * L[q] + 1 * w1[q];
        }
        t += dt;
    }
    free(w0); free(w1); free(L);
    if (t_out) *t_out = t;
    if (dt_out) *dt_out = dt;
    return rc;
}
