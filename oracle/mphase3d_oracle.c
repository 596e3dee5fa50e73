/*
 * mphase3d_oracle.c -- TEST INFRASTRUCTURE ONLY: CPU restatement of the 3D
 * primitive-variable multiphase RHS of 3d/weno4/Viscous-Multiphase-Fourth-Order
 * (the checker the GPU path is compared with; never linked into the product).
 *
 *   RHSFunctionPrimitive     rhs_function.c:56-570
 *     ComputePrimitiveVariables  :12-49 (PDECons2Prim per cell)
 *     boundary ghosts            :98-230 (transmissive copy, reflective mirror with the
 *                                 normal velocity negated; periodic by the DMDA)
 *     reconstruction + PAD       :234-355 (CWENO4 of each primitive variable, the 33-node
 *                                 admissibility check of PDECheckPAD, first order on failure)
 *     fluxes                     :359-505 (PDErotHLLCRiemannSolver, 7 components, weight
 *                                 w_gp2d = 1/4 per Gauss point)
 *     RHS                        :507-552 (the non-conservative phi equation uses F5 - phi F6)
 *     dt                         :559 (1/3) CFL h / (s_max_c + 2 s_max_v / h)
 *   EOS, fluxes, HLLC, rotated HLLC, PAD   pde.c:9-440
 *
 * The program's viscous fluxes are not defined: weno() never writes u_coeffs, so the
 * gradients it reads (rhs_function.c:317-345) are uninitialised, and the flux weights
 * w_gp2[f] are read for f = 2, 3 past the end of a 2-element array (:402-405).  With
 * zero gradients (the program compiled with zero-initialised automatic variables) the
 * viscous flux is a signed zero and changes nothing; only the viscous speed
 * PDEViscFluxPrim returns, (4/3) mu / rho with mu = phi MU_1 + (1 - phi) MU_2 (pde.c:101-136),
 * enters dt.  That is what is restated here.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "hype_oracle.h"

#define MV 6  /* variables */
#define MF 7  /* flux components: 6 + the normal velocity of the phi term */
#define MTR 24

static const double RHO_FLOOR = 1.0e-14, PRS_FLOOR = 1.0e-12;

/* the 33 admissibility nodes (hype.h:93-96) */
static const double XN[33] = {0.0, 0.5, 0.25, -0.25, -0.5, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.0, -0.5, 0.5,
                              0.0, -0.5, 0.5, 0.0, -0.5, 0.5, 0.0, -0.5, 0.5, -0.5, 0.5, -0.5, 0.5, -0.5, 0.5, -0.5};
static const double YN[33] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.25, -0.25, -0.5, 0.0, 0.0, 0.0, 0.0, 0.5, 0.5, 0.5, -0.5,
                              -0.5, -0.5, 0.5, 0.5, 0.5, -0.5, -0.5, -0.5, 0.0, 0.0, 0.0, 0.0, 0.5, 0.5, -0.5, -0.5};
static const double ZN[33] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.5, 0.25, -0.25, -0.5, 0.5, 0.5, 0.5, 0.5,
                              0.5, 0.5, -0.5, -0.5, -0.5, -0.5, -0.5, -0.5, 0.5, 0.5, -0.5, -0.5, 0.0, 0.0, 0.0, 0.0};
static const double GPX4[4] = {-0.28867513459481287, -0.28867513459481287, 0.28867513459481287, 0.28867513459481287};
static const double GPY4[4] = {-0.28867513459481287, 0.28867513459481287, -0.28867513459481287, 0.28867513459481287};

/* ---------------------------------------------------------------- EOS (pde.c:9-45) */
static inline double mix_g(const orc_mp3d_cfg* e, double phi) {
    return 1.0 + (e->g1 - 1.0) * (e->g2 - 1.0) / ((1.0 - phi) * (e->g1 - 1.0) + phi * (e->g2 - 1.0));
}
static inline double mix_pinf(const orc_mp3d_cfg* e, double g, double phi) {
    return ((g - 1.0) / g) * (e->g1 * e->p1 * phi / (e->g1 - 1.0) + e->g2 * e->p2 * (1.0 - phi) / (e->g2 - 1.0));
}

void orc_mp3d_cons2prim(const orc_mp3d_cfg* e, const double* Q, double* V) {
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

void orc_mp3d_prim2cons(const orc_mp3d_cfg* e, const double* V, double* Q) {
    const double g = mix_g(e, V[5]);
    const double P_inf = mix_pinf(e, g, V[5]);
    const double en = (V[4] + g * P_inf) / (g - 1.0);
    const double k = 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]);
    Q[0] = V[0];
    Q[1] = V[0] * V[1];
    Q[2] = V[0] * V[2];
    Q[3] = V[0] * V[3];
    Q[4] = k + en;
    Q[5] = V[5];
}

/* PDEConsFluxPrim (pde.c:142-202); *bad on inadmissible input */
static double cons_flux_prim(const orc_mp3d_cfg* e, const double* V, double nx, double ny, double nz, double* F, int* bad) {
    const double phi = V[5];
    const double g = mix_g(e, phi);
    const double P_inf = mix_pinf(e, g, phi);
    const double rho = V[0], u = V[1], v = V[2], w = V[3], p = V[4];
    const double en = (V[4] + g * P_inf) / (g - 1.0);
    const double k = 0.5 * rho * (u * u + v * v + w * w);
    const double E = k + en;
    const double un = nx * u + ny * v + nz * w;
    if (rho < RHO_FLOOR) *bad = 1;
    if ((p + P_inf) < PRS_FLOOR) *bad = 1;
    F[0] = rho * un;
    F[1] = rho * u * un + p * nx;
    F[2] = rho * v * un + p * ny;
    F[3] = rho * w * un + p * nz;
    F[4] = (E + p) * un;
    F[5] = phi * un;
    F[6] = 0.0;
    const double a = sqrt(g * (p + P_inf) / rho);
    return fabs(un) + a;
}

static void inv3x3(const double M[3][3], double iM[3][3]) {
    const double t4 = M[0][0] * M[1][1], t6 = M[0][0] * M[1][2], t8 = M[0][1] * M[1][0], t00 = M[0][2] * M[1][0],
                 t01 = M[0][1] * M[2][0], t04 = M[0][2] * M[2][0],
                 t07 = 1.0 / (t4 * M[2][2] - t6 * M[2][1] - t8 * M[2][2] + t00 * M[2][1] + t01 * M[1][2] - t04 * M[1][1]);
    iM[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) * t07;
    iM[0][1] = -(M[0][1] * M[2][2] - M[0][2] * M[2][1]) * t07;
    iM[0][2] = -(-M[0][1] * M[1][2] + M[0][2] * M[1][1]) * t07;
    iM[1][0] = -(M[1][0] * M[2][2] - M[1][2] * M[2][0]) * t07;
    iM[1][1] = (M[0][0] * M[2][2] - t04) * t07;
    iM[1][2] = -(t6 - t00) * t07;
    iM[2][0] = -(-M[1][0] * M[2][1] + M[1][1] * M[2][0]) * t07;
    iM[2][1] = -(M[0][0] * M[2][1] - t01) * t07;
    iM[2][2] = (t4 - t8) * t07;
}

static inline double pmin(double a, double b) { return a < b ? a : b; }
static inline double pmax(double a, double b) { return a < b ? b : a; }

/* PDEHLLCRiemannSolver (pde.c:273-379) */
static double hllc7(const orc_mp3d_cfg* e, const double* VL, const double* VR, double nx, double ny, double nz,
                    double* Flux, int* bad) {
    double QL[MV], QR[MV], QLs[MV], QRs[MV], FL[MF], FR[MF], FLs[MF], FRs[MF], R[3][3], iR[3][3], Local;
    double t1x, t1y, t1z, t2x, t2y, t2z;
    const double rho_L = VL[0], u_L = VL[1], v_L = VL[2], w_L = VL[3], P_L = VL[4];
    const double rho_R = VR[0], u_R = VR[1], v_R = VR[2], w_R = VR[3], P_R = VR[4];
    orc_mp3d_prim2cons(e, VL, QL);
    orc_mp3d_prim2cons(e, VR, QR);
    const double smaxl = cons_flux_prim(e, VL, nx, ny, nz, FL, bad);
    const double smaxr = cons_flux_prim(e, VR, nx, ny, nz, FR, bad);
    if (fabs(ny + nz) > fabs(ny - nz)) {
        Local = sqrt(2.0 * (1.0 + nz * (ny - nx) + nx * ny));
        t1x = (ny + nz) / Local; t1y = (nz - nx) / Local; t1z = -(nx + ny) / Local;
        t2x = (nx * (nz - ny) - ny * ny - nz * nz) / Local;
        t2y = (ny * (nx + nz) + nx * nx + nz * nz) / Local;
        t2z = (nz * (nx - nz) - nx * nx - ny * ny) / Local;
    } else {
        Local = sqrt(2.0 * (1.0 - nx * ny - nx * nz - ny * nz));
        t1x = (ny - nz) / Local; t1y = (nz - nx) / Local; t1z = (nx - ny) / Local;
        t2x = (nx * (ny + nz) - ny * ny - nz * nz) / Local;
        t2y = (ny * (nx + nz) - nx * nx - nz * nz) / Local;
        t2z = (nz * (nx + ny) - nx * nx - ny * ny) / Local;
    }
    R[0][0] = nx; R[0][1] = ny; R[0][2] = nz;
    R[1][0] = t1x; R[1][1] = t1y; R[1][2] = t1z;
    R[2][0] = t2x; R[2][1] = t2y; R[2][2] = t2z;
    inv3x3(R, iR);
    const double un_L = u_L * nx + v_L * ny + w_L * nz, ut1_L = u_L * t1x + v_L * t1y + w_L * t1z,
                 ut2_L = u_L * t2x + v_L * t2y + w_L * t2z;
    const double un_R = u_R * nx + v_R * ny + w_R * nz, ut1_R = u_R * t1x + v_R * t1y + w_R * t1z,
                 ut2_R = u_R * t2x + v_R * t2y + w_R * t2z;
    const double c_L = smaxl - fabs(un_L), c_R = smaxr - fabs(un_R);
    const double E_L = QL[4], E_R = QR[4];
    const double S_L = pmin((un_R - c_R), (un_L - c_L));
    const double S_R = pmax((un_L + c_L), (un_R + c_R));
    const double S_star = (P_R - P_L + rho_L * un_L * (S_L - un_L) - rho_R * un_R * (S_R - un_R)) /
                          (rho_L * (S_L - un_L) - rho_R * (S_R - un_R));
    FL[6] = un_L;
    FR[6] = un_R;
    double un = S_star, ut1 = ut1_L, ut2 = ut2_L;
    QLs[0] = rho_L * (S_L - un_L) / (S_L - S_star);
    QLs[1] = QLs[0] * (un * iR[0][0] + ut1 * iR[0][1] + ut2 * iR[0][2]);
    QLs[2] = QLs[0] * (un * iR[1][0] + ut1 * iR[1][1] + ut2 * iR[1][2]);
    QLs[3] = QLs[0] * (un * iR[2][0] + ut1 * iR[2][1] + ut2 * iR[2][2]);
    QLs[4] = QLs[0] * ((E_L / rho_L) + (S_star - un_L) * (S_star + P_L / (rho_L * (S_L - un_L))));
    QLs[5] = VL[5] * (S_L - un_L) / (S_L - S_star);
    ut1 = ut1_R; ut2 = ut2_R;
    QRs[0] = rho_R * (S_R - un_R) / (S_R - S_star);
    QRs[1] = QRs[0] * (un * iR[0][0] + ut1 * iR[0][1] + ut2 * iR[0][2]);
    QRs[2] = QRs[0] * (un * iR[1][0] + ut1 * iR[1][1] + ut2 * iR[1][2]);
    QRs[3] = QRs[0] * (un * iR[2][0] + ut1 * iR[2][1] + ut2 * iR[2][2]);
    QRs[4] = QRs[0] * ((E_R / rho_R) + (S_star - un_R) * (S_star + P_R / (rho_R * (S_R - un_R))));
    QRs[5] = VR[5] * (S_R - un_R) / (S_R - S_star);
    for (int i = 0; i < 6; i++) FLs[i] = FL[i] + S_L * (QLs[i] - QL[i]);
    FLs[6] = un_L + S_L * (((S_L - un_L) / (S_L - S_star)) - 1.0);
    for (int i = 0; i < 6; i++) FRs[i] = FR[i] + S_R * (QRs[i] - QR[i]);
    FRs[6] = un_R + S_R * (((S_R - un_R) / (S_R - S_star)) - 1.0);
    const double* src = NULL;
    if (S_L > 0.0) src = FL;
    else if ((S_star >= 0.0) && (S_L < 0.0)) src = FLs;
    else if ((S_star < 0.0) && (S_R >= 0.0)) src = FRs;
    else if (S_R < 0.0) src = FR;
    if (src) for (int i = 0; i < MF; i++) Flux[i] = src[i];
    else for (int i = 0; i < MF; i++) Flux[i] = 0.0; /* the reference leaves Flux unset here (S_L == 0) */
    return pmax(smaxl, smaxr);
}

/* PDErotHLLCRiemannSolver (pde.c:383-440) */
double orc_mp3d_rothllc(const orc_mp3d_cfg* e, const double* VL, const double* VR, double nx, double ny, double nz,
                        double* Flux, int* bad) {
    double F1[MF], F2[MF], F3[MF], n1x, n1y, n1z, t1x, t1y, t1z, t2x, t2y, t2z, Local;
    const double u_L = VL[1], v_L = VL[2], w_L = VL[3], u_R = VR[1], v_R = VR[2], w_R = VR[3];
    const double du = u_R - u_L, dv = v_R - v_L, dw = w_R - w_L;
    const double dq = sqrt(du * du + dv * dv + dw * dw);
    if (dq < 1.0E-10) { n1x = nx; n1y = ny; n1z = nz; }
    else { n1x = du / dq; n1y = dv / dq; n1z = dw / dq; }
    double alpha1 = (n1x * nx + n1y * ny + n1z * nz);
    if (alpha1 < 0.0) { n1x = -n1x; n1y = -n1y; n1z = -n1z; alpha1 = -alpha1; }
    if (fabs(n1y + n1z) > fabs(n1y - n1z)) {
        Local = sqrt(2.0 * (1.0 + n1z * (n1y - n1x) + n1x * n1y));
        t1x = (n1y + n1z) / Local; t1y = (n1z - n1x) / Local; t1z = -(n1x + n1y) / Local;
        t2x = (n1x * (n1z - n1y) - n1y * n1y - n1z * n1z) / Local;
        t2y = (n1y * (n1x + n1z) + n1x * n1x + n1z * n1z) / Local;
        t2z = (n1z * (n1x - n1y) - n1x * n1x - n1y * n1y) / Local;
    } else {
        Local = sqrt(2.0 * (1.0 - n1x * n1y - n1x * n1z - n1y * n1z));
        t1x = (n1y - n1z) / Local; t1y = (n1z - n1x) / Local; t1z = (n1x - n1y) / Local;
        t2x = (n1x * (n1y + n1z) - n1y * n1y - n1z * n1z) / Local;
        t2y = (n1y * (n1x + n1z) - n1x * n1x - n1z * n1z) / Local;
        t2z = (n1z * (n1x + n1y) - n1x * n1x - n1y * n1y) / Local;
    }
    double alpha2 = (t1x * nx + t1y * ny + t1z * nz);
    if (alpha2 < 0) { t1x = -t1x; t1y = -t1y; t1z = -t1z; alpha2 = -alpha2; }
    double alpha3 = (t2x * nx + t2y * ny + t2z * nz);
    if (alpha3 < 0) { t2x = -t2x; t2y = -t2y; t2z = -t2z; alpha3 = -alpha3; }
    const double s1 = hllc7(e, VL, VR, n1x, n1y, n1z, F1, bad);
    const double s2 = hllc7(e, VL, VR, t1x, t1y, t1z, F2, bad);
    const double s3 = hllc7(e, VL, VR, t2x, t2y, t2z, F3, bad);
    for (int c = 0; c < MF; ++c) Flux[c] = alpha1 * F1[c] + alpha2 * F2[c] + alpha3 * F3[c];
    return pmax(s1, pmax(s2, s3));
}

/* PDECheckPAD (pde.c:227-252) */
static int check_pad(const orc_mp3d_cfg* e, const double* V) {
    const double phi = V[5];
    const double g = mix_g(e, phi);
    const double P_inf = mix_pinf(e, g, phi);
    int pad = 1;
    if (V[0] < RHO_FLOOR) pad = 0;
    if (V[4] + P_inf < PRS_FLOOR) pad = 0;
    return pad;
}

/* the viscous speed of PDEViscFluxPrim (pde.c:101-136) */
static inline double visc_speed(const orc_mp3d_cfg* e, const double* W) {
    const double r4_3 = 4. / 3;
    const double mu = W[5] * e->mu1 + (1.0 - W[5]) * e->mu2;
    return r4_3 * mu / W[0];
}

static int map1(int i, int n, int blo, int bhi, int* flip) {
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

static long g_mp3d_fallbacks = 0;
long orc_mp3d_fallbacks(int reset) {
    long v = g_mp3d_fallbacks;
    if (reset) g_mp3d_fallbacks = 0;
    return v;
}

int orc_mp3d_rhs(const orc_mp3d_cfg* e, const double* U, double* RHS, double* dt_out, double* smax_out,
                 double* smaxv_out) {
    const int nx = e->nx, ny = e->ny, nz = e->nz;
    const int gx = nx + 6, gy = ny + 6, gz = nz + 6, ex = nx + 2, ey = ny + 2, ez = nz + 2;
    const double r1_h = 1. / (e->h);
#ifdef _OPENMP
    if (e->nthreads > 0) omp_set_num_threads(e->nthreads);
#endif
    /* primitive state with 3 ghost layers (the ghost fill is per axis, so corners
     * compose the three maps) */
    double* W = (double*)malloc(sizeof(double) * (size_t)gx * gy * gz * MV);
    double* T = (double*)malloc(sizeof(double) * (size_t)ex * ey * ez * MV * MTR);
    double* F = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny * nz * MF);
    double* G = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1) * nz * MF);
    double* H = (double*)malloc(sizeof(double) * (size_t)nx * ny * (nz + 1) * MF);
    if (!W || !T || !F || !G || !H) return 3;
#define WP(i, j, k) (W + (((size_t)((k) + 3) * gy + ((j) + 3)) * gx + ((i) + 3)) * MV)
#define TP(i, j, k) (T + (((size_t)((k) + 1) * ey + ((j) + 1)) * ex + ((i) + 1)) * MV * MTR)
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = -3; k < nz + 3; ++k)
        for (int j = -3; j < ny + 3; ++j)
            for (int i = -3; i < nx + 3; ++i) {
                int fx = 0, fy = 0, fz = 0;
                const int si = map1(i, nx, e->bc[0], e->bc[1], &fx);
                const int sj = map1(j, ny, e->bc[2], e->bc[3], &fy);
                const int sk = map1(k, nz, e->bc[4], e->bc[5], &fz);
                double* o = WP(i, j, k);
                orc_mp3d_cons2prim(e, U + (((size_t)sk * ny + sj) * nx + si) * MV, o);
                if (fx) o[1] = -o[1];
                if (fy) o[2] = -o[2];
                if (fz) o[3] = -o[3];
            }
    long fb = 0;
#pragma omp parallel for schedule(dynamic, 1) collapse(2) reduction(+ : fb)
    for (int k = -1; k < nz + 1; ++k)
        for (int j = -1; j < ny + 1; ++j)
            for (int i = -1; i < nx + 1; ++i) {
                double sol[MV][20];
                for (int c = 0; c < MV; ++c) {
                    double wx[5], wy[5], wz[5], wxy[5], wyz[5], wzx[5], wxyz[8];
                    for (int o = -2; o < 3; ++o) {
                        wx[o + 2] = WP(i + o, j, k)[c];
                        wy[o + 2] = WP(i, j + o, k)[c];
                        wz[o + 2] = WP(i, j, k + o)[c];
                    }
                    wxy[0] = WP(i, j, k)[c]; wxy[1] = WP(i + 1, j + 1, k)[c]; wxy[2] = WP(i + 1, j - 1, k)[c];
                    wxy[3] = WP(i - 1, j + 1, k)[c]; wxy[4] = WP(i - 1, j - 1, k)[c];
                    wyz[0] = WP(i, j, k)[c]; wyz[1] = WP(i, j + 1, k + 1)[c]; wyz[2] = WP(i, j + 1, k - 1)[c];
                    wyz[3] = WP(i, j - 1, k + 1)[c]; wyz[4] = WP(i, j - 1, k - 1)[c];
                    wzx[0] = WP(i, j, k)[c]; wzx[1] = WP(i + 1, j, k + 1)[c]; wzx[2] = WP(i - 1, j, k + 1)[c];
                    wzx[3] = WP(i + 1, j, k - 1)[c]; wzx[4] = WP(i - 1, j, k - 1)[c];
                    wxyz[0] = WP(i + 1, j + 1, k + 1)[c]; wxyz[1] = WP(i - 1, j + 1, k + 1)[c];
                    wxyz[2] = WP(i + 1, j - 1, k + 1)[c]; wxyz[3] = WP(i + 1, j + 1, k - 1)[c];
                    wxyz[4] = WP(i - 1, j - 1, k + 1)[c]; wxyz[5] = WP(i - 1, j + 1, k - 1)[c];
                    wxyz[6] = WP(i + 1, j - 1, k - 1)[c]; wxyz[7] = WP(i - 1, j - 1, k - 1)[c];
                    orc_cweno4_ref_args(wx, wy, wz, wxy, wyz, wzx, wxyz, sol[c]);
                }
                int pad = 1;
                for (int m = 0; m < 33 && pad; ++m) {
                    double Vn[MV];
                    for (int c = 0; c < MV; ++c) Vn[c] = orc_eval_poly3(XN[m], YN[m], ZN[m], sol[c]);
                    pad = check_pad(e, Vn);
                }
                if (!pad) {
                    for (int c = 0; c < MV; ++c)
                        for (int l = 1; l < 20; ++l) sol[c][l] = 0.0;
                    if (i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz) ++fb;
                }
                double* t = TP(i, j, k);
                for (int c = 0; c < MV; ++c)
                    for (int f = 0; f < 4; ++f) {
                        t[c * MTR + 0 * 4 + f] = orc_eval_poly3(-0.5, GPX4[f], GPY4[f], sol[c]);
                        t[c * MTR + 1 * 4 + f] = orc_eval_poly3(0.5, GPX4[f], GPY4[f], sol[c]);
                        t[c * MTR + 2 * 4 + f] = orc_eval_poly3(GPX4[f], -0.5, GPY4[f], sol[c]);
                        t[c * MTR + 3 * 4 + f] = orc_eval_poly3(GPX4[f], 0.5, GPY4[f], sol[c]);
                        t[c * MTR + 4 * 4 + f] = orc_eval_poly3(GPX4[f], GPY4[f], -0.5, sol[c]);
                        t[c * MTR + 5 * 4 + f] = orc_eval_poly3(GPX4[f], GPY4[f], 0.5, sol[c]);
                    }
            }
    g_mp3d_fallbacks += fb;
    double smax_c = 0.0, smax_v = 0.0;
    int bad = 0;
    /* faces of direction d: the low cell's face 2d+1 against the high cell's face 2d */
    for (int d = 0; d < 3; ++d) {
        const int fx = nx + (d == 0), fy = ny + (d == 1), fz = nz + (d == 2);
        double* Fd = d == 0 ? F : d == 1 ? G : H;
        const double nxv = d == 0 ? 1.0 : 0.0, nyv = d == 1 ? 1.0 : 0.0, nzv = d == 2 ? 1.0 : 0.0;
        double sc = 0.0, sv = 0.0;
        int bd = 0;
#pragma omp parallel for schedule(static) collapse(2) reduction(max : sc, sv) reduction(| : bd)
        for (int k = 0; k < fz; ++k)
            for (int j = 0; j < fy; ++j)
                for (int i = 0; i < fx; ++i) {
                    const double* tl = TP(i - (d == 0), j - (d == 1), k - (d == 2));
                    const double* tr = TP(i, j, k);
                    double flux[MF];
                    for (int c = 0; c < MF; ++c) flux[c] = 0.0;
                    for (int f = 0; f < 4; ++f) {
                        double VL[MV], VR[MV], fc[MF];
                        for (int c = 0; c < MV; ++c) {
                            VL[c] = tl[c * MTR + (2 * d + 1) * 4 + f];
                            VR[c] = tr[c * MTR + (2 * d) * 4 + f];
                        }
                        int b = 0;
                        const double s_c = orc_mp3d_rothllc(e, VL, VR, nxv, nyv, nzv, fc, &b);
                        if (s_c > sc) sc = s_c;
                        bd |= b;
                        const double svl = visc_speed(e, VL), svr = visc_speed(e, VR);
                        const double s_v = pmax(svl, svr);
                        if (s_v > sv) sv = s_v;
                        for (int c = 0; c < MF; ++c) flux[c] += 0.25 * (fc[c]);
                    }
                    double* o = Fd + (((size_t)k * fy + j) * fx + i) * MF;
                    for (int c = 0; c < MF; ++c) o[c] = flux[c];
                }
        if (sc > smax_c) smax_c = sc;
        if (sv > smax_v) smax_v = sv;
        bad |= bd;
    }
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double* Fl = F + (((size_t)k * ny + j) * (nx + 1) + i) * MF;
                const double* Fr = Fl + MF;
                const double* Gl = G + (((size_t)k * (ny + 1) + j) * nx + i) * MF;
                const double* Gr = Gl + (size_t)nx * MF;
                const double* Hl = H + (((size_t)k * ny + j) * nx + i) * MF;
                const double* Hr = Hl + (size_t)nx * ny * MF;
                const double phi = WP(i, j, k)[5];
                double* r = RHS + (((size_t)k * ny + j) * nx + i) * MV;
                for (int c = 0; c < MV; ++c) {
                    if (c == 5)
                        r[c] = -r1_h * ((Fr[c] - phi * Fr[c + 1]) - (Fl[c] - phi * Fl[c + 1])) -
                               r1_h * ((Gr[c] - phi * Gr[c + 1]) - (Gl[c] - phi * Gl[c + 1])) -
                               r1_h * ((Hr[c] - phi * Hr[c + 1]) - (Hl[c] - phi * Hl[c + 1]));
                    else
                        r[c] = -r1_h * (Fr[c] - Fl[c]) - r1_h * (Gr[c] - Gl[c]) - r1_h * (Hr[c] - Hl[c]);
                }
            }
#undef WP
#undef TP
    free(W); free(T); free(F); free(G); free(H);
    if (dt_out) *dt_out = (1.0 / 3.0) * (e->cfl * e->h) / (smax_c + (r1_h * smax_v) * 2.0);
    if (smax_out) *smax_out = smax_c;
    if (smaxv_out) *smaxv_out = smax_v;
    return bad ? 2 : 0;
}

/* SSP RKS3 / 4 stages (the same stage algebra as orc_euler_run); dt_mode 0: the dt of
 * step n+1 from the last stage RHS of step n, the first from the initial RHS call
 * (hype.c: RHSFunctionPrimitive before TSSolve, MonitorFunction's TSSetTimeStep);
 * dt_mode 2: *dt_inout throughout; dt_mode 3: as 0 with the first step's dt given */
int orc_mp3d_run(const orc_mp3d_cfg* e, int nsteps, int dt_mode, double* U, double* t_inout, double* dt_inout) {
    const size_t n = (size_t)e->nx * e->ny * e->nz * MV;
    double* u1 = (double*)malloc(sizeof(double) * n);
    double* F = (double*)malloc(sizeof(double) * n);
    if (!u1 || !F) return 3;
    double t = t_inout ? *t_inout : 0.0, dt_last = 0.0, dt = 0.0;
    int rc = orc_mp3d_rhs(e, U, F, &dt_last, NULL, NULL);
    if (rc) goto out;
    dt = (dt_mode == 2 || dt_mode == 3) ? *dt_inout : dt_last;
    for (int s = 0; s < nsteps; ++s) {
        if (s > 0 && (rc = orc_mp3d_rhs(e, U, F, NULL, NULL, NULL))) goto out;
        const double dtr = dt / 2;
        for (size_t q = 0; q < n; ++q) u1[q] = U[q] + dtr * F[q];
        if ((rc = orc_mp3d_rhs(e, u1, F, NULL, NULL, NULL))) goto out;
        for (size_t q = 0; q < n; ++q) u1[q] = u1[q] + dtr * F[q];
        if ((rc = orc_mp3d_rhs(e, u1, F, NULL, NULL, NULL))) goto out;
        const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * dt / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
        for (size_t q = 0; q < n; ++q) u1[q] = a3 * U[q] + b3 * F[q] + c3 * u1[q];
        if ((rc = orc_mp3d_rhs(e, u1, F, &dt_last, NULL, NULL))) goto out;
        for (size_t q = 0; q < n; ++q) U[q] = u1[q] + dtr * F[q];
        t += dt;
        if (dt_mode == 0 || dt_mode == 3) dt = dt_last;
    }
out:
    free(u1);
    free(F);
    if (t_inout) *t_inout = t;
    if (dt_inout) *dt_inout = dt;
    return rc;
}
