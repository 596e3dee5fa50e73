/*
 * hype_oracle.c -- CPU restatement of the reference's hot path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  tests/, the smoke check and bench.py's CPU
 * baseline leg use it as the checker; the GPU product never links or calls it.
 *
 * Every arithmetic expression keeps the operation order of the reference line
 * it follows, so that with -ffp-contract=off the restatement reproduces the
 * reference compiled from its own sources bit for bit (checked by
 * tests/test_oracle_vs_reference.py).  The loop structure, data layout and
 * ghost handling are this file's own.
 *
 *   CTCS 2D plane-wave form     2d/ctcs/plane_wave/wave.c:161-203 (update :192, alpha :169)
 *   CTCS point-source form      2d/ctcs/line_source/wave.c:149-173, 3d/ctcs/point_source/wave.c:163-194
 *   Source() wavelet            3d/ctcs/point_source/wave.c:232-238
 *   Euler RHS skeleton          3d/weno4/Navier-Stokes-3D/rhs_function.c:12-443 (viscous terms dropped)
 *   boundary ghost fill         3d/weno4/Navier-Stokes-3D/rhs_function.c:52-181
 *   CWENO4 weno()               3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259
 *   evaluate_polynomial         3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:12-21
 *   PDEConsFlux / LLF           3d/weno4/Navier-Stokes-3D/pde.c:40-88, 164-187
 *   dt = CFL h / (3 s_max)      3d/weno4/Navier-Stokes-3D/rhs_function.c:438-440
 *   SSPRK(4,3) stage algebra    PETSc TSSSP RKS3 with 4 stages (3d/weno4/Navier-Stokes-3D/hype.c:185-187),
 *                               restated from Ketcheson 2008 (see oracle/petsc_shim/petsc_shim.c)
 */
#include "hype_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ====================================================================== CTCS */

static inline double at2(const double* p, int nx, int ny, int i, int j, int bc) {
    if (i < 0 || i >= nx || j < 0 || j >= ny) {
        if (bc == ORC_BC_PERIODIC) {
            i = (i % nx + nx) % nx;
            j = (j % ny + ny) % ny;
        } else {
            return 0.0; /* zero exterior (DM_BOUNDARY_GHOSTED) */
        }
    }
    return p[(long)j * nx + i];
}

/* After a three-buffer rotation, leave (older, newest) in (p_old, p). */
static void rotate_back(double* p_old, double* p, double* a, double* b, size_t bytes) {
    if (b == p_old) {
        memcpy(p, b, bytes);
        memcpy(p_old, a, bytes);
    } else {
        if (a != p_old) memcpy(p_old, a, bytes);
        if (b != p) memcpy(p, b, bytes);
    }
}

int orc_ctcs2d_plane(int nx, int ny, double alpha, int bc, int nsteps, double* p_old, double* p, double* scratch) {
    double* a = p_old;
    double* b = p;
    double* c = scratch;
    const double a2 = alpha * alpha;
    for (int s = 0; s < nsteps; ++s) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double pc = b[(long)j * nx + i];
                double sum = at2(b, nx, ny, i, j + 1, bc) + at2(b, nx, ny, i, j - 1, bc) + at2(b, nx, ny, i + 1, j, bc) +
                             at2(b, nx, ny, i - 1, j, bc) - 4.0 * pc;
                c[(long)j * nx + i] = a2 * sum + 2.0 * pc - a[(long)j * nx + i];
            }
        double* t = a;
        a = b;
        b = c;
        c = t;
    }
    rotate_back(p_old, p, a, b, sizeof(double) * (size_t)nx * ny);
    return 0;
}

static double ricker_src(double t, double f0) {
    double t0 = 4.0 / f0;
    return -2.0 * (t - t0) * f0 * f0 * exp(-1.0 * f0 * f0 * (t - t0) * (t - t0));
}

static inline double at3(const double* p, const orc_ctcs_cfg* g, int i, int j, int k) {
    if (i < 0 || i >= g->nx || j < 0 || j >= g->ny || k < 0 || k >= g->nz) {
        if (g->bc != ORC_BC_PERIODIC) return 0.0;
        i = (i % g->nx + g->nx) % g->nx;
        j = (j % g->ny + g->ny) % g->ny;
        k = (k % g->nz + g->nz) % g->nz;
    }
    return p[((long)k * g->ny + j) * g->nx + i];
}

static inline double d2_2(double m1, double c, double p1, double inv) { return (p1 - 2.0 * c + m1) * inv; }
static inline double d2_4(double m2, double m1, double c, double p1, double p2, double inv) {
    return (-1.0 / 12 * p2 + 4.0 / 3.0 * p1 - 5.0 / 2.0 * c + 4.0 / 3.0 * m1 - 1.0 / 12.0 * m2) * inv;
}

int orc_ctcs_pointsrc(const orc_ctcs_cfg* g, const double* cf, int nsteps, double* p_old, double* p, double* scratch,
                      double* receiver) {
    const long n = (long)g->nx * g->ny * (g->dim == 3 ? g->nz : 1);
    orc_ctcs_cfg G = *g;
    if (G.dim == 2) G.nz = 1;
    double* a = p_old;
    double* b = p;
    double* c = scratch;
    const double ix2 = 1.0 / (g->dx * g->dx), iy2 = 1.0 / (g->dy * g->dy), iz2 = 1.0 / (g->dz * g->dz);
    const double dt = g->dt;
    for (int s = 0; s < nsteps; ++s) {
        const int it = g->it0 + s;
        if (receiver) receiver[s] = b[((long)(g->dim == 3 ? g->rec_k : 0) * G.ny + g->rec_j) * G.nx + g->rec_i];
#pragma omp parallel for schedule(static) collapse(2)
        for (int k = 0; k < G.nz; ++k)
            for (int j = 0; j < G.ny; ++j)
                for (int i = 0; i < G.nx; ++i) {
                    long o = ((long)k * G.ny + j) * G.nx + i;
                    double pc = b[o], lap;
                    if (g->order == 4) {
                        double pxx = d2_4(at3(b, &G, i - 2, j, k), at3(b, &G, i - 1, j, k), pc, at3(b, &G, i + 1, j, k),
                                          at3(b, &G, i + 2, j, k), ix2);
                        double pyy = d2_4(at3(b, &G, i, j - 2, k), at3(b, &G, i, j - 1, k), pc, at3(b, &G, i, j + 1, k),
                                          at3(b, &G, i, j + 2, k), iy2);
                        if (g->dim == 3) {
                            double pzz = d2_4(at3(b, &G, i, j, k - 2), at3(b, &G, i, j, k - 1), pc, at3(b, &G, i, j, k + 1),
                                              at3(b, &G, i, j, k + 2), iz2);
                            lap = pxx + pyy + pzz;
                        } else {
                            lap = pxx + pyy;
                        }
                    } else {
                        double pxx = d2_2(at3(b, &G, i - 1, j, k), pc, at3(b, &G, i + 1, j, k), ix2);
                        double pyy = d2_2(at3(b, &G, i, j - 1, k), pc, at3(b, &G, i, j + 1, k), iy2);
                        if (g->dim == 3) {
                            double pzz = d2_2(at3(b, &G, i, j, k - 1), pc, at3(b, &G, i, j, k + 1), iz2);
                            lap = pxx + pyy + pzz;
                        } else {
                            lap = pxx + pyy;
                        }
                    }
                    double cc = cf ? cf[o] : g->c0;
                    double v = 2.0 * pc - a[o] + cc * cc * dt * dt * lap;
                    if (i == g->src_i && j == g->src_j && (g->dim == 2 || k == g->src_k)) {
                        double vol = (g->dim == 3) ? g->dx * g->dy * g->dz : g->dx * g->dy;
                        v += ricker_src(it * dt, g->f0) / vol * dt * dt;
                    }
                    c[o] = v;
                }
        double* t = a;
        a = b;
        b = c;
        c = t;
    }
    rotate_back(p_old, p, a, b, sizeof(double) * (size_t)n);
    return 0;
}

int orc_ctcs_monopole(const orc_mono_cfg* g, int nsteps, double* p_old, double* p, double* scratch) {
    double* a = p_old;
    double* b = p;
    double* c = scratch;
    const int nx = g->nx, ny = g->ny;
    const double inv = 1.0 / (g->h * g->h);
    const double k2 = g->c0 * g->c0 * g->dt * g->dt;
    const double r2s = 1.0 / (2.0 * g->sigma * g->sigma);
    const double two_pi = 6.283185307179586;
    for (int s = 0; s < nsteps; ++s) {
        const double t = (double)(g->it0 + s) * g->dt;
        const double st = sin(two_pi * g->freq * t);
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j) {
            const double y = g->ymin + j * g->h;
            for (int i = 0; i < nx; ++i) {
                const double x = g->xmin + i * g->h;
                long o = (long)j * nx + i;
                double pc = b[o];
                double pxx = d2_2(at2(b, nx, ny, i - 1, j, ORC_BC_ZERO), pc, at2(b, nx, ny, i + 1, j, ORC_BC_ZERO), inv);
                double pyy = d2_2(at2(b, nx, ny, i, j - 1, ORC_BC_ZERO), pc, at2(b, nx, ny, i, j + 1, ORC_BC_ZERO), inv);
                double dx = x - g->xs, dy = y - g->ys;
                double src = exp(-(dx * dx + dy * dy) * r2s) * st;
                c[o] = 2.0 * pc - a[o] + k2 * (pxx + pyy) + k2 * src;
            }
        }
        double* tt = a;
        a = b;
        b = c;
        c = tt;
    }
    rotate_back(p_old, p, a, b, sizeof(double) * (size_t)nx * ny);
    return 0;
}

/* ============================================================ CWENO4 (3D) */

static const double R1_6 = 1. / 6.;
static const double R1_12 = 1. / 12.;
static const double R3_20 = 3. / 20.;
static const double R1_120 = 1. / 120.;
static const double R13_3 = 13. / 3.;
static const double R7_6 = 7. / 6.;
static const double R61_48 = 61. / 48.;
static const double SMALL = 1.0e-12;

/* Stencil of one cell and one variable, addressed by direction.
 *   c         centre
 *   m2,m1,p1,p2[d]   1D neighbours along d (0=x,1=y,2=z)
 *   q[a][b][sa][sb]  diagonal neighbour at +/-1 along a and b (s: 0 -> -1, 1 -> +1)
 *   o[sx][sy][sz]    body-diagonal neighbour */
typedef struct {
    double c;
    double m2[3], m1[3], p1[3], p2[3];
    double q[3][3][2][2];
    double o[2][2][2];
} Stencil;

/* R4 cross derivative, reference pattern 0.25*(mm - mp - pm + pp) (weno() :94-96) */
static inline double r4_cross(const Stencil* s, int a, int b) {
    return 0.25 * (s->q[a][b][0][0] - s->q[a][b][0][1] - s->q[a][b][1][0] + s->q[a][b][1][1]);
}
/* u_aab (:100,:102,:104): 0.25*(-mm + mp - pm + pp) + 0.5*(u_b-1 - u_b+1) */
static inline double r4_aab(const Stencil* s, int a, int b) {
    return 0.25 * (-s->q[a][b][0][0] + s->q[a][b][0][1] - s->q[a][b][1][0] + s->q[a][b][1][1]) + 0.5 * (s->m1[b] - s->p1[b]);
}
/* u_abb (:101,:103,:105): 0.5*(u_a-1 - u_a+1) + 0.25*(pp - mm - mp + pm) */
static inline double r4_abb(const Stencil* s, int a, int b) {
    return 0.5 * (s->m1[a] - s->p1[a]) + 0.25 * (s->q[a][b][1][1] - s->q[a][b][0][0] - s->q[a][b][0][1] + s->q[a][b][1][0]);
}
/* centred R3 cross derivative (:129-131): 0.25*(pp - pm - mp + mm) */
static inline double r3_cross0(const Stencil* s, int a, int b) {
    return 0.25 * (s->q[a][b][1][1] - s->q[a][b][1][0] - s->q[a][b][0][1] + s->q[a][b][0][0]);
}

/* Quantities of one R3 stencil: d[0..2] first derivatives, dd[0..2] second,
 * x[0..2] cross terms in the order xy, yz, xz. */
typedef struct {
    double d[3], dd[3], x[3];
} R3;

static inline double is3(const R3* r) {
    return (r->d[0] * r->d[0] + r->d[1] * r->d[1] + r->d[2] * r->d[2]) +
           R13_3 * (r->dd[0] * r->dd[0] + r->dd[1] * r->dd[1] + r->dd[2] * r->dd[2]) +
           R7_6 * (r->x[0] * r->x[0] + r->x[1] * r->x[1] + r->x[2] * r->x[2]);
}

/* cross-term slot for a pair of directions: xy -> 0, yz -> 1, xz -> 2 */
static inline int xslot(int a, int b) {
    if ((a == 0 && b == 1) || (a == 1 && b == 0)) return 0;
    if ((a == 1 && b == 2) || (a == 2 && b == 1)) return 1;
    return 2;
}

/* CWENO4 with gammaHi = gammaLo = gam (0.85 in the reference); linear=1 returns
 * the R4 polynomial itself (the optimal-weight limit). */
static void cweno4(const Stencil* s, double gam, int linear, double* coef) {
    const double u0 = s->c;
    double d4[3], dd4[3], ddd4[3];
    for (int d = 0; d < 3; ++d) {
        d4[d] = R1_120 * (11.0 * s->m2[d] - 82.0 * s->m1[d] + 82.0 * s->p1[d] - 11.0 * s->p2[d]);
        dd4[d] = 0.5 * (s->m1[d] - 2.0 * u0 + s->p1[d]);
        ddd4[d] = R1_12 * (-s->m2[d] + 2.0 * (s->m1[d] - s->p1[d]) + s->p2[d]);
    }
    const double xy4 = r4_cross(s, 0, 1), yz4 = r4_cross(s, 1, 2), xz4 = r4_cross(s, 2, 0);
    const double xxy = r4_aab(s, 0, 1), xyy = r4_abb(s, 0, 1);
    const double yyz = r4_aab(s, 1, 2), yzz = r4_abb(s, 1, 2);
    const double xxz = r4_aab(s, 0, 2), xzz = r4_abb(s, 0, 2);
    const double xyz = 0.125 * (s->o[1][1][1] - s->o[0][1][1] - s->o[1][0][1] - s->o[1][1][0] + s->o[0][0][1] +
                                s->o[0][1][0] + s->o[1][0][0] - s->o[0][0][0]);
    if (linear) {
        coef[0] = u0;
        coef[1] = d4[0]; coef[2] = d4[1]; coef[3] = d4[2];
        coef[4] = dd4[0]; coef[5] = dd4[1]; coef[6] = dd4[2];
        coef[7] = xy4; coef[8] = yz4; coef[9] = xz4;
        coef[10] = ddd4[0]; coef[11] = ddd4[1]; coef[12] = ddd4[2];
        coef[13] = xxy; coef[14] = xyy; coef[15] = yyz; coef[16] = yzz; coef[17] = xxz; coef[18] = xzz; coef[19] = xyz;
        return;
    }
    const double IS4 = d4[0] * d4[0] + d4[1] * d4[1] + d4[2] * d4[2] + R13_3 * (dd4[0] * dd4[0] + dd4[1] * dd4[1] + dd4[2] * dd4[2]) +
                       R7_6 * (xy4 * xy4 + yz4 * yz4 + xz4 * xz4) + 0.2 * (d4[0] * ddd4[0] + d4[1] * ddd4[1] + d4[2] * ddd4[2]) +
                       4.7 * (xxy * xxy + xxz * xxz + xyy * xyy + xzz * xzz + yyz * yyz + yzz * yzz) +
                       39.06 * (ddd4[0] * ddd4[0] + ddd4[1] * ddd4[1] + ddd4[2] * ddd4[2]) + R61_48 * xyz * xyz;

    /* the seven R3 stencils: 0 centred, 1+2d one-sided towards +d, 2+2d towards -d */
    R3 r[7];
    for (int d = 0; d < 3; ++d) {
        r[0].d[d] = 0.5 * (s->p1[d] - s->m1[d]);
        r[0].dd[d] = 0.5 * (s->m1[d] - 2.0 * u0 + s->p1[d]);
    }
    r[0].x[0] = r3_cross0(s, 0, 1);
    r[0].x[1] = r3_cross0(s, 1, 2);
    r[0].x[2] = r3_cross0(s, 2, 0);
    for (int d = 0; d < 3; ++d) {
        R3* P = &r[1 + 2 * d];
        R3* M = &r[2 + 2 * d];
        *P = r[0];
        *M = r[0];
        P->d[d] = -1.5 * u0 + 2.0 * s->p1[d] - 0.5 * s->p2[d];
        P->dd[d] = 0.5 * (u0 - 2.0 * s->p1[d] + s->p2[d]);
        M->d[d] = -2.0 * s->m1[d] + 0.5 * s->m2[d] + 1.5 * u0;
        M->dd[d] = 0.5 * (s->m2[d] - 2.0 * s->m1[d] + u0);
        for (int e = 0; e < 3; ++e) {
            if (e == d) continue;
            int k = xslot(d, e);
            P->x[k] = 0.5 * (s->q[d][e][1][1] - s->q[d][e][1][0]) - r[0].d[e];
            M->x[k] = 0.5 * (s->q[d][e][0][0] - s->q[d][e][0][1]) + r[0].d[e];
        }
    }
    double g3[7];
    g3[0] = (1.0 - gam) * gam;
    for (int i = 1; i < 7; ++i) g3[i] = R1_6 * (1 - gam) * (1 - gam);
    double w4 = gam / pow((IS4 + SMALL), 4.0);
    double total = w4;
    double w3[7];
    for (int i = 0; i < 7; ++i) {
        w3[i] = g3[i] / pow((is3(&r[i]) + SMALL), 4.0);
        total += w3[i];
    }
    w4 = w4 / total;
    for (int i = 0; i < 7; ++i) w3[i] = w3[i] / total;
    double l[9] = {0}, nl[9] = {0};
    for (int i = 0; i < 7; ++i) {
        for (int d = 0; d < 3; ++d) {
            l[d] += g3[i] * r[i].d[d];
            nl[d] += w3[i] * r[i].d[d];
        }
        for (int d = 0; d < 3; ++d) {
            l[3 + d] += g3[i] * r[i].dd[d];
            nl[3 + d] += w3[i] * r[i].dd[d];
        }
        for (int d = 0; d < 3; ++d) {
            l[6 + d] += g3[i] * r[i].x[d];
            nl[6 + d] += w3[i] * r[i].x[d];
        }
    }
    const double wr = w4 / gam;
    const double lin4[9] = {d4[0], d4[1], d4[2], dd4[0], dd4[1], dd4[2], xy4, yz4, xz4};
    coef[0] = u0;
    for (int q = 0; q < 9; ++q) coef[1 + q] = wr * (lin4[q] - l[q]) + nl[q];
    coef[10] = wr * ddd4[0];
    coef[11] = wr * ddd4[1];
    coef[12] = wr * ddd4[2];
    coef[13] = wr * xxy;
    coef[14] = wr * xyy;
    coef[15] = wr * yyz;
    coef[16] = wr * yzz;
    coef[17] = wr * xxz;
    coef[18] = wr * xzz;
    coef[19] = wr * xyz;
}

double orc_eval_poly3(double x, double y, double z, const double* c) {
    return c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * (x * x - R1_12) + c[5] * (y * y - R1_12) + c[6] * (z * z - R1_12) +
           c[7] * x * y + c[8] * y * z + c[9] * z * x + c[10] * x * (x * x - R3_20) + c[11] * y * (y * y - R3_20) +
           c[12] * z * (z * z - R3_20) + c[13] * (x * x - R1_12) * y + c[14] * x * (y * y - R1_12) +
           c[15] * (y * y - R1_12) * z + c[16] * y * (z * z - R1_12) + c[17] * (x * x - R1_12) * z +
           c[18] * x * (z * z - R1_12) + c[19] * x * y * z;
}

/* Third-order WENO (3d/weno3/Euler/reconstruction.c:29-177), operation for
 * operation: per axis the quadratics of the left, centred and right stencils with
 * weights 1 : 100 : 1 (:54-106), then per axis pair (xy, yz, zx) four corner-based
 * cross terms with equal weights (:108-163); weights 1/pow(IS + 1e-12, 4). */
static void weno3_axis(double u0, double m2, double m1, double p1, double p2, double* c1, double* c2) {
    double u_x[3], u_xx[3], IS[3], wt[3], total;
    u_x[0] = -2.0 * m1 + 0.5 * m2 + 1.5 * u0; u_xx[0] = 0.5 * (m2 - 2.0 * m1 + u0);
    u_x[1] = 0.5 * (p1 - m1);                 u_xx[1] = 0.5 * (m1 - 2.0 * u0 + p1);
    u_x[2] = -1.5 * u0 + 2.0 * p1 - 0.5 * p2; u_xx[2] = 0.5 * (u0 - 2.0 * p1 + p2);
    for (int i = 0; i < 3; ++i) {
        IS[i] = u_x[i] * u_x[i] + R13_3 * u_xx[i] * u_xx[i];
        wt[i] = 1.0 / pow(IS[i] + 1.0e-12, 4.0);
    }
    wt[1] = 100.0 * wt[1];
    total = wt[0] + wt[1] + wt[2];
    wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total;
    *c1 = wt[0] * u_x[0] + wt[1] * u_x[1] + wt[2] * u_x[2];
    *c2 = wt[0] * u_xx[0] + wt[1] * u_xx[1] + wt[2] * u_xx[2];
}

/* pair (a, b) with a's and b's first/second coefficients; pp = u(a+1, b+1) etc. */
static double weno3_cross(double u0, double pp, double pm, double mp, double mm, double ca, double cb, double caa, double cbb) {
    double u_xy[4], IS[4], wt[4], total;
    u_xy[0] = pp - u0 - ca - cb - caa - cbb;
    u_xy[1] = -pm + u0 + ca - cb + caa + cbb;
    u_xy[2] = -mp + u0 - ca + cb + caa + cbb;
    u_xy[3] = mm - u0 + ca + cb - caa - cbb;
    const double temp = 4.0 * (caa * caa + cbb * cbb);
    for (int i = 0; i < 4; ++i) {
        IS[i] = temp + u_xy[i] * u_xy[i];
        wt[i] = 1.0 / pow(IS[i] + 1.0e-12, 4.0);
    }
    total = wt[0] + wt[1] + wt[2] + wt[3];
    wt[0] = wt[0] / total; wt[1] = wt[1] / total; wt[2] = wt[2] / total; wt[3] = wt[3] / total;
    return wt[0] * u_xy[0] + wt[1] * u_xy[1] + wt[2] * u_xy[2] + wt[3] * u_xy[3];
}

/* coef[0..9] in the basis of 3d/weno3/Euler/reconstruction.c:12-16; coef[10..19] = 0 */
static void weno3(const Stencil* s, double* coef) {
    const double u0 = s->c;
    coef[0] = u0;
    for (int d = 0; d < 3; ++d) weno3_axis(u0, s->m2[d], s->m1[d], s->p1[d], s->p2[d], &coef[1 + d], &coef[4 + d]);
    /* q[a][b][sa][sb]: the point at (a: 2sa-1, b: 2sb-1) */
    coef[7] = weno3_cross(u0, s->q[0][1][1][1], s->q[0][1][1][0], s->q[0][1][0][1], s->q[0][1][0][0], coef[1], coef[2],
                          coef[4], coef[5]);
    coef[8] = weno3_cross(u0, s->q[1][2][1][1], s->q[1][2][1][0], s->q[1][2][0][1], s->q[1][2][0][0], coef[2], coef[3],
                          coef[5], coef[6]);
    coef[9] = weno3_cross(u0, s->q[2][0][1][1], s->q[2][0][1][0], s->q[2][0][0][1], s->q[2][0][0][0], coef[3], coef[1],
                          coef[6], coef[4]);
    for (int q = 10; q < 20; ++q) coef[q] = 0.0;
}

/* evaluate_polynomial of 3d/weno3/Euler/reconstruction.c:12-16 (10 terms, same order) */
static double eval_poly_w3(double x, double y, double z, const double* c) {
    return c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * (x * x - R1_12) + c[5] * (y * y - R1_12) + c[6] * (z * z - R1_12) +
           c[7] * x * y + c[8] * y * z + c[9] * z * x;
}

void orc_cweno4_ref_args(const double* Ux, const double* Uy, const double* Uz, const double* Uxy, const double* Uyz,
                         const double* Uzx, const double* Uxyz, double* coeffs) {
    Stencil s;
    memset(&s, 0, sizeof(s));
    s.c = Uxy[0];
    const double* U1[3] = {Ux, Uy, Uz};
    for (int d = 0; d < 3; ++d) {
        s.m2[d] = U1[d][0]; s.m1[d] = U1[d][1]; s.p1[d] = U1[d][3]; s.p2[d] = U1[d][4];
    }
    /* reference argument layout: [1]=(+a,+b) [2]=(+a,-b) [3]=(-a,+b) [4]=(-a,-b) for the
     * pairs (x,y), (y,z) and, for U_zx, [1]=(+z,+x) [2]=(+z,-x) [3]=(-z,+x) [4]=(-z,-x) */
    const double* U2[3] = {Uxy, Uyz, Uzx};
    const int pa[3] = {0, 1, 2}, pb[3] = {1, 2, 0};
    for (int p = 0; p < 3; ++p) {
        int a = pa[p], b = pb[p];
        double pp = U2[p][1], pm = U2[p][2], mp = U2[p][3], mm = U2[p][4];
        s.q[a][b][1][1] = pp; s.q[a][b][1][0] = pm; s.q[a][b][0][1] = mp; s.q[a][b][0][0] = mm;
        s.q[b][a][1][1] = pp; s.q[b][a][0][1] = pm; s.q[b][a][1][0] = mp; s.q[b][a][0][0] = mm;
    }
    /* U_xyz: (+++),(-++),(+-+),(++-),(--+),(-+-),(+--),(---) */
    const int sx[8] = {1, 0, 1, 1, 0, 0, 1, 0}, sy[8] = {1, 1, 0, 1, 0, 1, 0, 0}, sz[8] = {1, 1, 1, 0, 1, 0, 0, 0};
    for (int q = 0; q < 8; ++q) s.o[sx[q]][sy[q]][sz[q]] = Uxyz[q];
    cweno4(&s, 0.85, 0, coeffs);
}

/* ============================================================ Rusanov flux */

/* PDEConsFlux for an axis normal dir (pde.c:40-88): flux, max wave speed;
 * *bad set when rho < 1e-14 or p < 1e-12. */
static inline double cons_flux(const double* Q, int dir, double gm1, double gamma, double* F, int* bad) {
    const double rho = Q[0];
    const double r1_rho = 1.0 / rho;
    const double u = r1_rho * Q[1], v = r1_rho * Q[2], w = r1_rho * Q[3];
    const double E = Q[4];
    const double p = gm1 * (E - 0.5 * rho * (u * u + v * v + w * w));
    if (rho < 1.0e-14 || p < 1.0e-12) *bad = 1;
    const double un = dir == 0 ? u : (dir == 1 ? v : w);
    /* the reference's n-weighted sums with one unit component keep exactly the
     * product order (rho*u)*v etc. of the term that survives */
    F[0] = rho * un;
    if (dir == 0) {
        F[1] = rho * u * u + p;
        F[2] = rho * u * v;
        F[3] = rho * u * w;
    } else if (dir == 1) {
        F[1] = rho * u * v;
        F[2] = rho * v * v + p;
        F[3] = rho * v * w;
    } else {
        F[1] = rho * u * w;
        F[2] = rho * v * w;
        F[3] = rho * w * w + p;
    }
    F[4] = (E + p) * un;
    const double a = sqrt(r1_rho * gamma * p);
    return fabs(un) + a;
}

double orc_rusanov(const double* QL, const double* QR, int dir, double gamma, double* flux, int* bad) {
    double FL[5], FR[5];
    const double gm1 = gamma - 1.0;
    double sl = cons_flux(QL, dir, gm1, gamma, FL, bad);
    double sr = cons_flux(QR, dir, gm1, gamma, FR, bad);
    double s = (sl < sr) ? sr : sl;
    for (int c = 0; c < 5; ++c) flux[c] = 0.5 * (FR[c] + FL[c] - s * (QR[c] - QL[c]));
    return s;
}

/* ============================================================ HLLC (3D, general normal) */

/* PDEConsFlux with a general unit normal (Navier-Stokes-3D/pde.c:40-88) */
static double cons_flux_n(const double* Q, double nx, double ny, double nz, double gamma, double* F, int* bad) {
    const double rho = Q[0];
    const double r1_rho = 1.0 / rho;
    const double u = r1_rho * Q[1], v = r1_rho * Q[2], w = r1_rho * Q[3];
    const double E = Q[4];
    const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v + w * w));
    if (rho < 1.0e-14 || p < 1.0e-12) *bad = 1;
    F[0] = nx * rho * u + ny * rho * v + nz * rho * w;
    F[1] = nx * (rho * u * u + p) + ny * rho * u * v + nz * rho * u * w;
    F[2] = nx * rho * u * v + ny * (rho * v * v + p) + nz * rho * v * w;
    F[3] = nx * rho * u * w + ny * rho * v * w + nz * (rho * w * w + p);
    F[4] = (E + p) * (nx * u + ny * v + nz * w);
    const double a = sqrt(r1_rho * gamma * p);
    return fabs(u * nx + v * ny + w * nz) + a;
}

/* PDECons2Prim (pde.c:9-18) */
static void cons2prim(const double* Q, double gamma, double* V) {
    const double r1_rho = 1.0 / Q[0];
    V[0] = Q[0];
    V[1] = r1_rho * Q[1];
    V[2] = r1_rho * Q[2];
    V[3] = r1_rho * Q[3];
    V[4] = (gamma - 1.0) * (Q[4] - 0.5 * r1_rho * ((Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3])));
}

/* 3x3 inverse by cofactors (pde.c:189-205) */
static void inv3(const double M[3][3], double iM[3][3]) {
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

/* Miller-Colella tangents of a unit normal; 'fixed' selects the corrected t2z
 * of the rotated solver (pde.c:348) instead of the HLLC one (pde.c:238) */
static void tangents(double nx, double ny, double nz, int fixed, double* t1, double* t2) {
    double L;
    if (fabs(ny + nz) > fabs(ny - nz)) {
        L = sqrt(2.0 * (1.0 + nz * (ny - nx) + nx * ny));
        t1[0] = (ny + nz) / L; t1[1] = (nz - nx) / L; t1[2] = -(nx + ny) / L;
        t2[0] = (nx * (nz - ny) - ny * ny - nz * nz) / L;
        t2[1] = (ny * (nx + nz) + nx * nx + nz * nz) / L;
        t2[2] = fixed ? (nz * (nx - ny) - nx * nx - ny * ny) / L : (nz * (nx - nz) - nx * nx - ny * ny) / L;
    } else {
        L = sqrt(2.0 * (1.0 - nx * ny - nx * nz - ny * nz));
        t1[0] = (ny - nz) / L; t1[1] = (nz - nx) / L; t1[2] = (nx - ny) / L;
        t2[0] = (nx * (ny + nz) - ny * ny - nz * nz) / L;
        t2[1] = (ny * (nx + nz) - nx * nx - nz * nz) / L;
        t2[2] = (nz * (nx + ny) - nx * nx - ny * ny) / L;
    }
}

/* PDEHLLCRiemannSolver (pde.c:207-322) */
double orc_hllc(const double* QL, const double* QR, double nx, double ny, double nz, double gamma, double* Flux, int* bad) {
    double FL[5], FR[5], VL[5], VR[5], t1[3], t2[3], M[3][3], iM[3][3];
    double sl = cons_flux_n(QL, nx, ny, nz, gamma, FL, bad);
    double sr = cons_flux_n(QR, nx, ny, nz, gamma, FR, bad);
    double smax = (sl < sr) ? sr : sl;
    cons2prim(QL, gamma, VL);
    cons2prim(QR, gamma, VR);
    const double rL = VL[0], uL = VL[1], vL = VL[2], wL = VL[3], PL = VL[4];
    const double rR = VR[0], uR = VR[1], vR = VR[2], wR = VR[3], PR = VR[4];
    tangents(nx, ny, nz, 0, t1, t2);
    M[0][0] = nx; M[0][1] = ny; M[0][2] = nz;
    M[1][0] = t1[0]; M[1][1] = t1[1]; M[1][2] = t1[2];
    M[2][0] = t2[0]; M[2][1] = t2[1]; M[2][2] = t2[2];
    inv3(M, iM);
    const double unL = uL * nx + vL * ny + wL * nz, ut1L = uL * t1[0] + vL * t1[1] + wL * t1[2], ut2L = uL * t2[0] + vL * t2[1] + wL * t2[2];
    const double unR = uR * nx + vR * ny + wR * nz, ut1R = uR * t1[0] + vR * t1[1] + wR * t1[2], ut2R = uR * t2[0] + vR * t2[1] + wR * t2[2];
    const double cL = sqrt(gamma * PL / rL), cR = sqrt(gamma * PR / rR);
    const double EL = QL[4], ER = QR[4];
    const double a1 = unR - cR, b1 = unL - cL;
    const double SL = (a1 < b1) ? a1 : b1;
    const double a2 = unL + cL, b2 = unR + cR;
    const double SR = (a2 < b2) ? b2 : a2;
    const double Ss = (PR - PL + rL * unL * (SL - unL) - rR * unR * (SR - unR)) / (rL * (SL - unL) - rR * (SR - unR));
    double QLs[5], QRs[5];
    QLs[0] = rL * (SL - unL) / (SL - Ss);
    QLs[1] = QLs[0] * (Ss * iM[0][0] + ut1L * iM[0][1] + ut2L * iM[0][2]);
    QLs[2] = QLs[0] * (Ss * iM[1][0] + ut1L * iM[1][1] + ut2L * iM[1][2]);
    QLs[3] = QLs[0] * (Ss * iM[2][0] + ut1L * iM[2][1] + ut2L * iM[2][2]);
    QLs[4] = QLs[0] * ((EL / rL) + (Ss - unL) * (Ss + PL / (rL * (SL - unL))));
    QRs[0] = rR * (SR - unR) / (SR - Ss);
    QRs[1] = QRs[0] * (Ss * iM[0][0] + ut1R * iM[0][1] + ut2R * iM[0][2]);
    QRs[2] = QRs[0] * (Ss * iM[1][0] + ut1R * iM[1][1] + ut2R * iM[1][2]);
    QRs[3] = QRs[0] * (Ss * iM[2][0] + ut1R * iM[2][1] + ut2R * iM[2][2]);
    QRs[4] = QRs[0] * ((ER / rR) + (Ss - unR) * (Ss + PR / (rR * (SR - unR))));
    for (int c = 0; c < 5; ++c) {
        const double FLs = FL[c] + SL * (QLs[c] - QL[c]);
        const double FRs = FR[c] + SR * (QRs[c] - QR[c]);
        /* the reference leaves the flux unset when S_L == 0 and S* >= 0; the
         * (continuous) star state is taken there */
        if (SL > 0.0) Flux[c] = FL[c];
        else if (Ss >= 0.0) Flux[c] = FLs;
        else if (SR >= 0.0) Flux[c] = FRs;
        else Flux[c] = FR[c];
    }
    return smax;
}

/* PDErotHLLCRiemannSolver (pde.c:324-384) */
double orc_rothllc(const double* QL, const double* QR, double nx, double ny, double nz, double gamma, double* Flux, int* bad) {
    double irho = 1.0 / QL[0];
    const double uL = irho * QL[1], vL = irho * QL[2], wL = irho * QL[3];
    irho = 1.0 / QR[0];
    const double uR = irho * QR[1], vR = irho * QR[2], wR = irho * QR[3];
    const double du = uR - uL, dv = vR - vL, dw = wR - wL;
    const double dq = sqrt(du * du + dv * dv + dw * dw);
    double n1[3];
    if (dq < 1.0E-10) {
        n1[0] = nx; n1[1] = ny; n1[2] = nz;
    } else {
        n1[0] = du / dq; n1[1] = dv / dq; n1[2] = dw / dq;
    }
    double a1 = (n1[0] * nx + n1[1] * ny + n1[2] * nz);
    if (a1 < 0.0) {
        n1[0] = -n1[0]; n1[1] = -n1[1]; n1[2] = -n1[2];
        a1 = -a1;
    }
    double t1[3], t2[3];
    tangents(n1[0], n1[1], n1[2], 1, t1, t2);
    double a2 = (t1[0] * nx + t1[1] * ny + t1[2] * nz);
    if (a2 < 0) {
        t1[0] = -t1[0]; t1[1] = -t1[1]; t1[2] = -t1[2];
        a2 = -a2;
    }
    double a3 = (t2[0] * nx + t2[1] * ny + t2[2] * nz);
    if (a3 < 0) {
        t2[0] = -t2[0]; t2[1] = -t2[1]; t2[2] = -t2[2];
        a3 = -a3;
    }
    double F1[5], F2[5], F3[5];
    double s1 = orc_hllc(QL, QR, n1[0], n1[1], n1[2], gamma, F1, bad);
    double s2 = orc_hllc(QL, QR, t1[0], t1[1], t1[2], gamma, F2, bad);
    double s3 = orc_hllc(QL, QR, t2[0], t2[1], t2[2], gamma, F3, bad);
    for (int c = 0; c < 5; ++c) Flux[c] = a1 * F1[c] + a2 * F2[c] + a3 * F3[c];
    double m23 = (s2 < s3) ? s3 : s2;
    return (s1 < m23) ? m23 : s1;
}

/* ============================================================ Euler RHS */

#define NV 5
#define NTR 24 /* traces per cell and variable: face f (0..5) x Gauss point g (0..3) -> f*4+g */

static const double GP = 0.28867513459481287;
static const double GPX[4] = {-0.28867513459481287, -0.28867513459481287, 0.28867513459481287, 0.28867513459481287};
static const double GPY[4] = {-0.28867513459481287, 0.28867513459481287, -0.28867513459481287, 0.28867513459481287};

/* boundary map of one index: returns the source index, *flip set for a reflective ghost */
static inline int bmap(int i, int n, int blo, int bhi, int* flip) {
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

typedef struct {
    const orc_euler_cfg* g;
    int gx, gy, gz; /* padded dims (n + 6) */
    double* pad;    /* padded state, ghost width 3, AoS */
} Padded;

static void build_padded(Padded* P, const orc_euler_cfg* g, const double* U) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    P->g = g;
    P->gx = nx + 6; P->gy = ny + 6; P->gz = nz + 6;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = -3; k < nz + 3; ++k)
        for (int j = -3; j < ny + 3; ++j)
            for (int i = -3; i < nx + 3; ++i) {
                int fx = 0, fy = 0, fz = 0;
                int si = bmap(i, nx, g->bc[0], g->bc[1], &fx);
                int sj = bmap(j, ny, g->bc[2], g->bc[3], &fy);
                int sk = bmap(k, nz, g->bc[4], g->bc[5], &fz);
                const double* q = U + (((long)sk * ny + sj) * nx + si) * NV;
                double* o = P->pad + (((long)(k + 3) * P->gy + (j + 3)) * P->gx + (i + 3)) * NV;
                for (int c = 0; c < NV; ++c) o[c] = q[c];
                if (fx) o[1] = -o[1];
                if (fy) o[2] = -o[2];
                if (fz) o[3] = -o[3];
            }
}

static inline const double* padp(const Padded* P, int i, int j, int k) {
    return P->pad + (((long)(k + 3) * P->gy + (j + 3)) * P->gx + (i + 3)) * NV;
}

static void gather(const Padded* P, int i, int j, int k, int c, Stencil* s) {
    s->c = padp(P, i, j, k)[c];
    for (int d = 0; d < 3; ++d) {
        int ex = d == 0, ey = d == 1, ez = d == 2;
        s->m2[d] = padp(P, i - 2 * ex, j - 2 * ey, k - 2 * ez)[c];
        s->m1[d] = padp(P, i - ex, j - ey, k - ez)[c];
        s->p1[d] = padp(P, i + ex, j + ey, k + ez)[c];
        s->p2[d] = padp(P, i + 2 * ex, j + 2 * ey, k + 2 * ez)[c];
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            for (int sa = 0; sa < 2; ++sa)
                for (int sb = 0; sb < 2; ++sb) {
                    int off[3] = {0, 0, 0};
                    off[a] = 2 * sa - 1;
                    off[b] = 2 * sb - 1;
                    s->q[a][b][sa][sb] = padp(P, i + off[0], j + off[1], k + off[2])[c];
                }
        }
    for (int sx = 0; sx < 2; ++sx)
        for (int sy = 0; sy < 2; ++sy)
            for (int sz = 0; sz < 2; ++sz) s->o[sx][sy][sz] = padp(P, i + 2 * sx - 1, j + 2 * sy - 1, k + 2 * sz - 1)[c];
}

/* traces of one cell: tr[c*NTR + f*4 + g], faces 0..5 = -x,+x,-y,+y,-z,+z; with viscosity
 * followed by the gradients of the R4 polynomial at the same points,
 * tr[NV*NTR + (c*NTR + f*4 + g)*3 + d] (evaluate_grad, Navier-Stokes-3D/reconstruction.c:24-35).
 * The Navier-Stokes-3D program itself reconstructs with R4 (recon 1): its weno() has the
 * whole CWENO combination inside a comment (reconstruction.c:159-308) and copies u_coeffs
 * into coeffs (:310-312). */
static void cell_traces_raw(const Padded* P, int i, int j, int k, double gam, int recon, double* tr);
static void ac_eval_grad(const double* c, double x, double y, double z, double h, double* gx, double* gy, double* gz);
static int g_visc = 0;          /* set per RHS call: viscous fluxes on */
static double g_visc_h = 1.0;   /* grid spacing for the gradients */

/* optional first-order fallback (positivity = 1): when a face trace has rho < 1e-14
 * or p < 1e-12 the cell is reconstructed at first order, the rule of
 * 3d/weno4/Viscous-Multiphase-Fourth-Order/rhs_function.c:297-305 applied at the traces */
static int g_positivity = 0;
static long g_fallbacks = 0;

static void cell_traces(const Padded* P, int i, int j, int k, double gam, int recon, double* tr) {
    cell_traces_raw(P, i, j, k, gam, recon, tr);
    if (!g_positivity) return;
    const double gm1 = P->g->gamma - 1.0;
    for (int q = 0; q < NTR; ++q) {
        const double rho = tr[0 * NTR + q], mx = tr[1 * NTR + q], my = tr[2 * NTR + q], mz = tr[3 * NTR + q],
                     E = tr[4 * NTR + q];
        const double p = gm1 * (E - 0.5 * (mx * mx + my * my + mz * mz) / rho);
        if (!(rho >= 1.0e-14) || !(p >= 1.0e-12)) {
            for (int c = 0; c < NV; ++c)
                for (int qq = 0; qq < NTR; ++qq) tr[c * NTR + qq] = padp(P, i, j, k)[c];
            if (i >= 0 && i < P->g->nx && j >= 0 && j < P->g->ny && k >= 0 && k < P->g->nz) {
#pragma omp atomic
                ++g_fallbacks;
            }
            return;
        }
    }
}

static void cell_traces_raw(const Padded* P, int i, int j, int k, double gam, int recon, double* tr) {
    Stencil s;
    double coef[20];
    for (int c = 0; c < NV; ++c) {
        gather(P, i, j, k, c, &s);
        double* t = tr + c * NTR;
        if (recon == 3) {
            weno3(&s, coef);
            for (int g = 0; g < 4; ++g) {
                t[0 * 4 + g] = eval_poly_w3(-0.5, GPX[g], GPY[g], coef);
                t[1 * 4 + g] = eval_poly_w3(0.5, GPX[g], GPY[g], coef);
                t[2 * 4 + g] = eval_poly_w3(GPX[g], -0.5, GPY[g], coef);
                t[3 * 4 + g] = eval_poly_w3(GPX[g], 0.5, GPY[g], coef);
                t[4 * 4 + g] = eval_poly_w3(GPX[g], GPY[g], -0.5, coef);
                t[5 * 4 + g] = eval_poly_w3(GPX[g], GPY[g], 0.5, coef);
            }
            continue;
        }
        cweno4(&s, gam, recon == 1, coef);
        if (g_visc) { /* u_coeffs: the R4 polynomial (Navier-Stokes-3D/reconstruction.c:138-157) */
            double r4[20];
            cweno4(&s, gam, 1, r4);
            double* gr = tr + NV * NTR + (size_t)c * NTR * 3;
            for (int g = 0; g < 4; ++g) {
                ac_eval_grad(r4, -0.5, GPX[g], GPY[g], g_visc_h, &gr[(0 * 4 + g) * 3], &gr[(0 * 4 + g) * 3 + 1], &gr[(0 * 4 + g) * 3 + 2]);
                ac_eval_grad(r4, 0.5, GPX[g], GPY[g], g_visc_h, &gr[(1 * 4 + g) * 3], &gr[(1 * 4 + g) * 3 + 1], &gr[(1 * 4 + g) * 3 + 2]);
                ac_eval_grad(r4, GPX[g], -0.5, GPY[g], g_visc_h, &gr[(2 * 4 + g) * 3], &gr[(2 * 4 + g) * 3 + 1], &gr[(2 * 4 + g) * 3 + 2]);
                ac_eval_grad(r4, GPX[g], 0.5, GPY[g], g_visc_h, &gr[(3 * 4 + g) * 3], &gr[(3 * 4 + g) * 3 + 1], &gr[(3 * 4 + g) * 3 + 2]);
                ac_eval_grad(r4, GPX[g], GPY[g], -0.5, g_visc_h, &gr[(4 * 4 + g) * 3], &gr[(4 * 4 + g) * 3 + 1], &gr[(4 * 4 + g) * 3 + 2]);
                ac_eval_grad(r4, GPX[g], GPY[g], 0.5, g_visc_h, &gr[(5 * 4 + g) * 3], &gr[(5 * 4 + g) * 3 + 1], &gr[(5 * 4 + g) * 3 + 2]);
            }
        }
        for (int g = 0; g < 4; ++g) {
            t[0 * 4 + g] = orc_eval_poly3(-0.5, GPX[g], GPY[g], coef);
            t[1 * 4 + g] = orc_eval_poly3(0.5, GPX[g], GPY[g], coef);
            t[2 * 4 + g] = orc_eval_poly3(GPX[g], -0.5, GPY[g], coef);
            t[3 * 4 + g] = orc_eval_poly3(GPX[g], 0.5, GPY[g], coef);
            t[4 * 4 + g] = orc_eval_poly3(GPX[g], GPY[g], -0.5, coef);
            t[5 * 4 + g] = orc_eval_poly3(GPX[g], GPY[g], 0.5, coef);
        }
    }
    (void)GP;
}

/* PDEViscFlux (Navier-Stokes-3D/pde.c:90-162), operation for operation, including its
 * velocity gradients u_x = rhou_x - u rho_x / rho (:118-130); returns the viscous speed */
static double orc_visc_flux(const double* Q, const double G[NV][3], double nx, double ny, double nz, double gamma,
                            double mu0, double pr, double cv, double* F) {
    double rho, rho2, irho, u, v, w, p, mu, k, rho_x, rhou_x, rhov_x, rhow_x, e_x, rho_y, rhou_y, rhov_y, rhow_y, e_y, rho_z,
        rhou_z, rhov_z, rhow_z, e_z, e;
    double rhou, rhov, rhow;
    double u_x, u_y, u_z, v_x, v_y, v_z, w_x, w_y, w_z, T_x, T_y, T_z, div_v;
    double tau_xx, tau_xy, tau_xz, tau_yz, tau_yy, tau_zz, q_x, q_y, q_z;
    rho = Q[0]; rho2 = Q[0] * Q[0]; irho = 1.0 / Q[0];
    u = irho * Q[1];
    v = irho * Q[2];
    w = irho * Q[3];
    rhou = Q[1];
    rhov = Q[2];
    rhow = Q[3];
    e = Q[4];
    p = (gamma - 1.0) * (e - 0.5 * rho * (u * u + v * v + w * w));
    (void)p;
    mu = mu0;
    k = cv * mu * gamma / pr;
    rho_x = G[0][0]; rho_y = G[0][1]; rho_z = G[0][2];
    rhou_x = G[1][0]; rhou_y = G[1][1]; rhou_z = G[1][2];
    rhov_x = G[2][0]; rhov_y = G[2][1]; rhov_z = G[2][2];
    rhow_x = G[3][0]; rhow_y = G[3][1]; rhow_z = G[3][2];
    e_x = G[4][0]; e_y = G[4][1]; e_z = G[4][2];
    u_x = rhou_x - u * rho_x / rho;
    v_x = rhov_x - v * rho_x / rho;
    w_x = rhow_x - w * rho_x / rho;
    T_x = (-(gamma - 1.0) * rho_x / rho2) * (e - 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rho) +
          ((gamma - 1.0) / rho) * (e_x - (rhou * rhou_x + rhov * rhov_x + rhow * rhow_x) / rho +
                                   0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) * rho_x / rho2);
    u_y = rhou_y - u * rho_y / rho;
    v_y = rhov_y - v * rho_y / rho;
    w_y = rhow_y - w * rho_y / rho;
    T_y = (-(gamma - 1.0) * rho_y / rho2) * (e - 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rho) +
          ((gamma - 1.0) / rho) * (e_y - (rhou * rhou_y + rhov * rhov_y + rhow * rhow_y) / rho +
                                   0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) * rho_y / rho2);
    u_z = rhou_z - u * rho_z / rho;
    v_z = rhov_z - v * rho_z / rho;
    w_z = rhow_z - w * rho_z / rho;
    T_z = (-(gamma - 1.0) * rho_z / rho2) * (e - 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rho) +
          ((gamma - 1.0) / rho) * (e_z - (rhou * rhou_z + rhov * rhov_z + rhow * rhow_z) / rho +
                                   0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) * rho_z / rho2);
    div_v = -(2.0 / 3.0) * mu * (u_x + v_y + w_z);
    tau_xx = div_v + 2.0 * mu * u_x;
    tau_xy = mu * (u_y + v_x);
    tau_xz = mu * (u_z + w_x);
    tau_yy = div_v + 2.0 * mu * v_y;
    tau_yz = mu * (v_z + w_y);
    tau_zz = div_v + 2.0 * mu * w_z;
    q_x = -k * T_x;
    q_y = -k * T_y;
    q_z = -k * T_z;
    F[0] = 0.0;
    F[1] = -(nx * tau_xx + ny * tau_xy + nz * tau_xz);
    F[2] = -(nx * tau_xy + ny * tau_yy + nz * tau_yz);
    F[3] = -(nx * tau_xz + ny * tau_yz + nz * tau_zz);
    F[4] = -(nx * (u * tau_xx + v * tau_xy + w * tau_xz - q_x) + ny * (u * tau_xy + v * tau_yy + w * tau_yz - q_y) +
             nz * (u * tau_xz + v * tau_yz + w * tau_zz - q_z));
    const double a = (4. / 3.) * mu / Q[0], b = gamma * mu / (pr * Q[0]);
    return a > b ? a : b;
}

/* face flux from the left cell's trace set (face fl) and the right cell's (face fr) */
static int g_flux_kind = 0; /* set per RHS call: 0 Rusanov, 1 HLLC, 2 rotated HLLC */
static double g_mu = 0.0, g_pr = 1.0, g_cv = 2.5;

static inline double face_flux(const double* trL, int fl, const double* trR, int fr, int dir, double gamma, double* F, int* bad,
                               double* smax_visc) {
    double smax = 0.0;
    for (int c = 0; c < NV; ++c) F[c] = 0.0;
    for (int g = 0; g < 4; ++g) {
        double QL[NV], QR[NV], fl5[NV];
        for (int c = 0; c < NV; ++c) {
            QL[c] = trL[c * NTR + fl * 4 + g];
            QR[c] = trR[c * NTR + fr * 4 + g];
        }
        double s;
        if (g_flux_kind == 0) {
            s = orc_rusanov(QL, QR, dir, gamma, fl5, bad);
        } else {
            const double nx = dir == 0 ? 1.0 : 0.0, ny = dir == 1 ? 1.0 : 0.0, nz = dir == 2 ? 1.0 : 0.0;
            s = (g_flux_kind == 1) ? orc_hllc(QL, QR, nx, ny, nz, gamma, fl5, bad)
                                   : orc_rothllc(QL, QR, nx, ny, nz, gamma, fl5, bad);
        }
        if (s > smax) smax = s;
        if (g_visc) { /* PDEViscRiemannSolver (pde.c:386-404) and rhs_function.c:310-316 */
            const double nx = dir == 0 ? 1.0 : 0.0, ny = dir == 1 ? 1.0 : 0.0, nz = dir == 2 ? 1.0 : 0.0;
            double GL[NV][3], GR[NV][3], FL[NV], FR[NV], fv[NV];
            for (int c = 0; c < NV; ++c)
                for (int d = 0; d < 3; ++d) {
                    GL[c][d] = trL[NV * NTR + (c * NTR + fl * 4 + g) * 3 + d];
                    GR[c][d] = trR[NV * NTR + (c * NTR + fr * 4 + g) * 3 + d];
                }
            const double sl = orc_visc_flux(QL, GL, nx, ny, nz, gamma, g_mu, g_pr, g_cv, FL);
            const double sr = orc_visc_flux(QR, GR, nx, ny, nz, gamma, g_mu, g_pr, g_cv, FR);
            const double sv = sl > sr ? sl : sr;
            for (int c = 0; c < NV; ++c) fv[c] = 0.5 * (FR[c] + FL[c]);
            if (sv > *smax_visc) *smax_visc = sv;
            for (int c = 0; c < NV; ++c) F[c] += 0.25 * (fl5[c] + fv[c]);
        } else {
            for (int c = 0; c < NV; ++c) F[c] += 0.25 * fl5[c];
        }
    }
    return smax;
}

static double g_last_smax_visc = 0.0;
double orc_euler_last_smax_visc(void) { return g_last_smax_visc; }

int orc_euler_rhs(const orc_euler_cfg* g, const double* U, double* RHS, double* smax_out, long* bad_out) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double gam = 0.85;
    const int recon = g->recon;
    const double r1_h = 1. / (g->h);
    g_flux_kind = g->flux;
    g_positivity = g->positivity;
    g_visc = g->mu > 0.0;
    g_visc_h = g->h;
    g_mu = g->mu;
    g_pr = g->prandtl;
    g_cv = g->cv;
    const size_t REC = (size_t)NV * NTR * (g_visc ? 4 : 1);
#ifdef _OPENMP
    if (g->nthreads > 0) omp_set_num_threads(g->nthreads);
#endif
    Padded P;
    P.pad = (double*)malloc(sizeof(double) * (size_t)(nx + 6) * (ny + 6) * (nz + 6) * NV);
    if (!P.pad) return 3;
    build_padded(&P, g, U);
    /* traces for two planes (k-1, k), cells i,j in [-1, n] */
    const int tx = nx + 2, ty = ny + 2;
    const size_t plane = (size_t)tx * ty * REC;
    double* T[2];
    T[0] = (double*)malloc(sizeof(double) * plane);
    T[1] = (double*)malloc(sizeof(double) * plane);
    /* z fluxes at the face below the current plane, and the previous one */
    double* H[2];
    H[0] = (double*)malloc(sizeof(double) * (size_t)nx * ny * NV);
    H[1] = (double*)malloc(sizeof(double) * (size_t)nx * ny * NV);
    double* F = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny * NV);
    double* G = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1) * NV);
    if (!T[0] || !T[1] || !H[0] || !H[1] || !F || !G) return 3;
    double smax = 0.0, smax_v = 0.0;
    long bad = -1;
#define TR(buf, i, j) ((buf) + ((size_t)((j) + 1) * tx + ((i) + 1)) * REC)
    for (int k = -1; k <= nz; ++k) {
        double* Tk = T[(k + 2) & 1];
        double* Tkm1 = T[(k + 1) & 1];
        const int ghostk = (k < 0 || k >= nz);
        /* reconstruct the cells of plane k that some face of an interior cell needs */
#pragma omp parallel for schedule(dynamic, 1)
        for (int j = -1; j <= ny; ++j) {
            const int ghostj = (j < 0 || j >= ny);
            if (ghostk && ghostj) continue;
            for (int i = -1; i <= nx; ++i) {
                const int ghosti = (i < 0 || i >= nx);
                if (ghosti + ghostj + ghostk > 1) continue;
                cell_traces(&P, i, j, k, gam, recon, TR(Tk, i, j));
            }
        }
        if (k < 0) continue;
        double* Hk = H[k & 1];      /* face k-1/2 */
        double* Hkm1 = H[(k + 1) & 1]; /* face k-3/2 (from the previous plane) */
        double smax_k = 0.0, smaxv_k = 0.0;
        int bad_k = 0;
        /* z faces between plane k-1 and k (for k == nz: the top face of plane nz-1) */
#pragma omp parallel for schedule(static) reduction(max : smax_k, smaxv_k) reduction(| : bad_k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int b = 0;
                double sv = 0.0;
                double s = face_flux(TR(Tkm1, i, j), 5, TR(Tk, i, j), 4, 2, g->gamma, Hk + ((size_t)j * nx + i) * NV, &b, &sv);
                if (s > smax_k) smax_k = s;
                if (sv > smaxv_k) smaxv_k = sv;
                bad_k |= b;
            }
        if (bad_k && bad < 0) bad = (long)k * nx * ny;
        if (smax_k > smax) smax = smax_k;
        if (smaxv_k > smax_v) smax_v = smaxv_k;
        if (k == 0) continue;
        /* plane kk = k-1 is complete: x and y faces, then the divergence */
        const int kk = k - 1;
        double* Tc = Tkm1;
        double smax_p = 0.0, smaxv_p = 0.0;
        int bad_p = 0;
#pragma omp parallel for schedule(static) reduction(max : smax_p, smaxv_p) reduction(| : bad_p)
        for (int j = 0; j < ny; ++j) {
            for (int i = 0; i <= nx; ++i) {
                int b = 0;
                double sv = 0.0;
                double s = face_flux(TR(Tc, i - 1, j), 1, TR(Tc, i, j), 0, 0, g->gamma, F + ((size_t)j * (nx + 1) + i) * NV, &b, &sv);
                if (s > smax_p) smax_p = s;
                if (sv > smaxv_p) smaxv_p = sv;
                bad_p |= b;
            }
        }
#pragma omp parallel for schedule(static) reduction(max : smax_p, smaxv_p) reduction(| : bad_p)
        for (int j = 0; j <= ny; ++j) {
            for (int i = 0; i < nx; ++i) {
                int b = 0;
                double sv = 0.0;
                double s = face_flux(TR(Tc, i, j - 1), 3, TR(Tc, i, j), 2, 1, g->gamma, G + ((size_t)j * nx + i) * NV, &b, &sv);
                if (s > smax_p) smax_p = s;
                if (sv > smaxv_p) smaxv_p = sv;
                bad_p |= b;
            }
        }
        if (bad_p && bad < 0) bad = (long)kk * nx * ny;
        if (smax_p > smax) smax = smax_p;
        if (smaxv_p > smax_v) smax_v = smaxv_p;
#pragma omp parallel for schedule(static)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                double* r = RHS + (((size_t)kk * ny + j) * nx + i) * NV;
                const double* Fl = F + ((size_t)j * (nx + 1) + i) * NV;
                const double* Fr = Fl + NV;
                const double* Gl = G + ((size_t)j * nx + i) * NV;
                const double* Gr = G + ((size_t)(j + 1) * nx + i) * NV;
                const double* Hl = Hkm1 + ((size_t)j * nx + i) * NV;
                const double* Hr = Hk + ((size_t)j * nx + i) * NV;
                for (int c = 0; c < NV; ++c)
                    r[c] = -r1_h * (Fr[c] - Fl[c]) - r1_h * (Gr[c] - Gl[c]) - r1_h * (Hr[c] - Hl[c]);
            }
    }
#undef TR
    free(P.pad);
    free(T[0]); free(T[1]); free(H[0]); free(H[1]); free(F); free(G);
    if (smax_out) *smax_out = smax;
    if (bad_out) *bad_out = bad;
    g_last_smax_visc = smax_v;
    return bad >= 0 ? 2 : 0;
}

/* dt = CFL*h/(3*s_max), rhs_function.c:438 with the viscous speed zero */
/* (1/3)(CFL h)/s_max: 3d/weno4/Navier-Stokes-3D/rhs_function.c:438-440;
 * (CFL h)/(3 s_max): 3d/weno3/Euler/rhs_function.c:383 (the WENO3 program) */
static inline double euler_dt(const orc_euler_cfg* g, double smax) {
    if (g->mu > 0.0) /* rhs_function.c:438 with the viscous speed of the last RHS call */
        return (1.0 / 3.0) * (g->cfl * g->h) / (smax + ((1. / g->h) * g_last_smax_visc) * 2.0);
    return g->recon == 3 ? (g->cfl * g->h) / (3.0 * smax) : (1.0 / 3.0) * (g->cfl * g->h) / (smax + 0.0);
}

int orc_euler_run(const orc_euler_cfg* g, int nsteps, int dt_mode, double* U, double* t_inout, double* dt_inout, long* bad) {
    const size_t n = (size_t)g->nx * g->ny * g->nz * NV;
    double* u1 = (double*)malloc(sizeof(double) * n);
    double* F = (double*)malloc(sizeof(double) * n);
    double smax;
    double t = t_inout ? *t_inout : 0.0;
    double dt = 0.0;
    int rc = 0;
    /* initial RHS call that sets the first dt (hype.c:175-180); its result is
     * also the first stage of the first step (same input) */
    rc = orc_euler_rhs(g, U, F, &smax, bad);
    if (rc) goto out;
    double dt_last = euler_dt(g, smax);
    /* dt_mode 2: the given dt throughout; dt_mode 3: monitor semantics continued from an
     * earlier call (its first step takes the dt that call handed back) */
    dt = (dt_mode == 2 || dt_mode == 3) ? *dt_inout : dt_last;
    for (int s = 0; s < nsteps; ++s) {
        /* stage 1: u1 = u + dt/2 F(u) */
        if (s > 0) rc = orc_euler_rhs(g, U, F, &smax, bad);
        if (rc) goto out;
        const double dtr = dt / 2;
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < n; ++q) u1[q] = U[q] + dtr * F[q];
        /* stage 2: u2 = u1 + dt/2 F(u1)  (kept in u1; U still holds u^n) */
        rc = orc_euler_rhs(g, u1, F, &smax, bad);
        if (rc) goto out;
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < n; ++q) u1[q] = u1[q] + dtr * F[q];
        /* stage 3: u3 = 2/3 u + dt/6 F(u2) + 1/3 u2 */
        rc = orc_euler_rhs(g, u1, F, &smax, bad);
        if (rc) goto out;
        const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * dt / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < n; ++q) u1[q] = a3 * U[q] + b3 * F[q] + c3 * u1[q];
        /* stage 4: u^{n+1} = u3 + dt/2 F(u3) */
        rc = orc_euler_rhs(g, u1, F, &smax, bad);
        if (rc) goto out;
#pragma omp parallel for schedule(static)
        for (size_t q = 0; q < n; ++q) U[q] = u1[q] + dtr * F[q];
        t += dt;
        dt_last = euler_dt(g, smax);
        if (dt_mode == 0 || dt_mode == 3) dt = dt_last;
    }
out:
    free(u1);
    free(F);
    if (t_inout) *t_inout = t;
    if (dt_inout) *dt_inout = dt;
    return rc;
}

long orc_positivity_fallbacks(int reset) {
    long v = g_fallbacks;
    if (reset) g_fallbacks = 0;
    return v;
}

/* ============================================================ acoustic FV (plane_wave)
 * RHSFunction            3d/weno4/plane_wave/rhs_function.c:12-345 (adiabatic ghosts
 *                        :43-131, reconstruction + face gradients :135-214, central
 *                        fluxes :216-287, RHS :289-300)
 * weno() with gammaHi=1  3d/weno4/plane_wave/reconstruction.c:38-259 (all R3 weights
 *                        zero: the coefficients are the R4 ones, bit for bit)
 * evaluate_grad          3d/weno4/plane_wave/reconstruction.c:25-34
 * PDEFlux, RiemannSolver 3d/weno4/plane_wave/pde.c:12-34 */
static void ac_eval_grad(const double* c, double x, double y, double z, double h, double* gx, double* gy, double* gz) {
    *gx = (c[1] + 2.0 * c[4] * x + c[7] * y + c[9] * z + c[10] * (3.0 * x * x - R3_20) + 2.0 * c[13] * x * y +
           c[14] * (y * y - R1_12) + 2.0 * c[17] * x * z + c[18] * (z * z - R1_12) + c[19] * y * z) / h;
    *gy = (c[2] + 2.0 * c[5] * y + c[7] * x + c[8] * z + c[11] * (3.0 * y * y - R3_20) + c[13] * (x * x - R1_12) +
           2.0 * c[14] * x * y + 2.0 * c[15] * y * z + c[16] * (z * z - R1_12) + c[19] * x * z) / h;
    *gz = (c[3] + 2.0 * c[6] * z + c[8] * y + c[9] * x + c[12] * (3.0 * z * z - R3_20) + c[15] * (y * y - R1_12) +
           2.0 * c[16] * y * z + c[17] * (x * x - R1_12) + 2.0 * c[18] * x * z + c[19] * x * y) / h;
}

typedef struct {
    const orc_acoustic_cfg* g;
    int gx, gy;
    double* pad; /* u with 3 ghost layers */
} AcPad;

static inline double acp(const AcPad* P, int i, int j, int k) {
    return P->pad[((size_t)(k + 3) * P->gy + (j + 3)) * P->gx + (i + 3)];
}

static int ac_map(int i, int n, int blo, int bhi, int* flip) {
    if (i < 0) {
        if (blo == 0) return i + n;
        *flip ^= 1;
        return -1 - i;
    }
    if (i >= n) {
        if (bhi == 0) return i - n;
        *flip ^= 1;
        return 2 * n - 1 - i;
    }
    return i;
}

static void ac_build_pad(AcPad* P, const orc_acoustic_cfg* g, const double* U) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    P->g = g;
    P->gx = nx + 6;
    P->gy = ny + 6;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = -3; k < nz + 3; ++k)
        for (int j = -3; j < ny + 3; ++j)
            for (int i = -3; i < nx + 3; ++i) {
                int f = 0;
                const int mi = ac_map(i, nx, g->bc[0], g->bc[1], &f);
                const int mj = ac_map(j, ny, g->bc[2], g->bc[3], &f);
                const int mk = ac_map(k, nz, g->bc[4], g->bc[5], &f);
                const double v = U[(((size_t)mk * ny + mj) * nx + mi) * 2];
                P->pad[((size_t)(k + 3) * P->gy + (j + 3)) * P->gx + (i + 3)] = f ? -v : v;
            }
}

/* the 24 normal gradients of one cell: g[face * 4 + q] (faces -x,+x,-y,+y,-z,+z) */
static void ac_cell_grads(const AcPad* P, int i, int j, int k, double* gn) {
    const orc_acoustic_cfg* g = P->g;
    Stencil s;
    s.c = acp(P, i, j, k);
    for (int d = 0; d < 3; ++d) {
        const int ex = d == 0, ey = d == 1, ez = d == 2;
        s.m2[d] = acp(P, i - 2 * ex, j - 2 * ey, k - 2 * ez);
        s.m1[d] = acp(P, i - ex, j - ey, k - ez);
        s.p1[d] = acp(P, i + ex, j + ey, k + ez);
        s.p2[d] = acp(P, i + 2 * ex, j + 2 * ey, k + 2 * ez);
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            if (a == b) continue;
            for (int sa = 0; sa < 2; ++sa)
                for (int sb = 0; sb < 2; ++sb) {
                    int off[3] = {0, 0, 0};
                    off[a] = 2 * sa - 1;
                    off[b] = 2 * sb - 1;
                    s.q[a][b][sa][sb] = acp(P, i + off[0], j + off[1], k + off[2]);
                }
        }
    for (int sx = 0; sx < 2; ++sx)
        for (int sy = 0; sy < 2; ++sy)
            for (int sz = 0; sz < 2; ++sz) s.o[sx][sy][sz] = acp(P, i + 2 * sx - 1, j + 2 * sy - 1, k + 2 * sz - 1);
    double coef[20], gx, gy, gz;
    cweno4(&s, 0.85, g->recon == 1, coef);
    for (int q = 0; q < 4; ++q) {
        ac_eval_grad(coef, -0.5, GPX[q], GPY[q], g->h, &gx, &gy, &gz); gn[0 * 4 + q] = gx;
        ac_eval_grad(coef, 0.5, GPX[q], GPY[q], g->h, &gx, &gy, &gz);  gn[1 * 4 + q] = gx;
        ac_eval_grad(coef, GPX[q], -0.5, GPY[q], g->h, &gx, &gy, &gz); gn[2 * 4 + q] = gy;
        ac_eval_grad(coef, GPX[q], 0.5, GPY[q], g->h, &gx, &gy, &gz);  gn[3 * 4 + q] = gy;
        ac_eval_grad(coef, GPX[q], GPY[q], -0.5, g->h, &gx, &gy, &gz); gn[4 * 4 + q] = gz;
        ac_eval_grad(coef, GPX[q], GPY[q], 0.5, g->h, &gx, &gy, &gz);  gn[5 * 4 + q] = gz;
    }
}

/* sum_q w_q RiemannSolver: 0.5 (FR + FL), F = c^2 (grad . n); the tangential products
 * of PDEFlux are exact zeros */
static double ac_face_flux(const double* gL, int fl, const double* gR, int fr, double c) {
    double flux = 0.0;
    for (int q = 0; q < 4; ++q) {
        const double FL = c * c * (gL[fl * 4 + q] * 1.0 + 0.0 + 0.0);
        const double FR = c * c * (gR[fr * 4 + q] * 1.0 + 0.0 + 0.0);
        flux += 0.25 * (0.5 * (FR + FL));
    }
    return flux;
}

/* ---------------------------------------------------------------- point source + receiver
 * 3d/weno4/point_source and 2d/weno4/line_source add to the u_t equation of one cell the
 * wavelet Source(t) = -2 (t - t0) f0^2 exp(-f0^2 (t - t0)^2), t0 = 4 / f0 (source.c), scaled by
 * 1/h^3 (3D) or 1/h^2 (2D), at the time t of the RHS call (rhs_function.c:337-340 / :244-246),
 * and print u at a receiver cell at every RHS call (:342-346 / :249-253).  Off by default. */
static int g_src_on = 0, g_src[3] = {0, 0, 0}, g_rec_on = 0, g_rec[3] = {0, 0, 0};
static double g_src_f0 = 100.0, g_src_t = 0.0;
static double* g_tr_t = NULL;
static double* g_tr_p = NULL;
static int g_tr_max = 0, g_tr_n = 0;

void orc_set_point_source(int on, int isx, int isy, int isz, double f0, int rec_on, int irx, int iry, int irz) {
    g_src_on = on; g_src[0] = isx; g_src[1] = isy; g_src[2] = isz; g_src_f0 = f0;
    g_rec_on = rec_on; g_rec[0] = irx; g_rec[1] = iry; g_rec[2] = irz;
}

/* the receiver trace of the following RHS calls goes to (t[q], p[q]), q < max; returns nothing */
void orc_set_trace_buffer(double* t, double* p, int max) {
    g_tr_t = t; g_tr_p = p; g_tr_max = max; g_tr_n = 0;
}
int orc_trace_count(void) { return g_tr_n; }

static double src_wavelet(double t) {
    const double f0 = g_src_f0;
    const double t0 = 4.0 / f0;
    return -2.0 * (t - t0) * f0 * f0 * exp(-1.0 * f0 * f0 * (t - t0) * (t - t0));
}

static void rec_sample(double t, double u) {
    if (g_tr_n < g_tr_max && g_tr_t) {
        g_tr_t[g_tr_n] = t;
        g_tr_p[g_tr_n] = u;
    }
    ++g_tr_n;
}

int orc_acoustic_rhs_at(const orc_acoustic_cfg* g, double t, const double* U, double* RHS) {
    g_src_t = t;
    return orc_acoustic_rhs(g, U, RHS);
}

int orc_acoustic_rhs(const orc_acoustic_cfg* g, const double* U, double* RHS) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
#ifdef _OPENMP
    if (g->nthreads > 0) omp_set_num_threads(g->nthreads);
#endif
    AcPad P;
    P.pad = (double*)malloc(sizeof(double) * (size_t)(nx + 6) * (ny + 6) * (nz + 6));
    const int tx = nx + 2, ty = ny + 2, tz = nz + 2;
    double* GR = (double*)malloc(sizeof(double) * 24 * (size_t)tx * ty * tz);
    if (!P.pad || !GR) return 3;
    ac_build_pad(&P, g, U);
#define ACG(i, j, k) (GR + (((size_t)((k) + 1) * ty + ((j) + 1)) * tx + ((i) + 1)) * 24)
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = -1; k <= nz; ++k)
        for (int j = -1; j <= ny; ++j)
            for (int i = -1; i <= nx; ++i) {
                const int gi = (i < 0 || i >= nx), gj = (j < 0 || j >= ny), gk = (k < 0 || k >= nz);
                if (gi + gj + gk > 1) continue;
                ac_cell_grads(&P, i, j, k, ACG(i, j, k));
            }
    const double r1_h = 1. / g->h;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double Fm = ac_face_flux(ACG(i - 1, j, k), 1, ACG(i, j, k), 0, g->c);
                const double Fp = ac_face_flux(ACG(i, j, k), 1, ACG(i + 1, j, k), 0, g->c);
                const double Gm = ac_face_flux(ACG(i, j - 1, k), 3, ACG(i, j, k), 2, g->c);
                const double Gp = ac_face_flux(ACG(i, j, k), 3, ACG(i, j + 1, k), 2, g->c);
                const double Hm = ac_face_flux(ACG(i, j, k - 1), 5, ACG(i, j, k), 4, g->c);
                const double Hp = ac_face_flux(ACG(i, j, k), 5, ACG(i, j, k + 1), 4, g->c);
                const size_t cell = ((size_t)k * ny + j) * nx + i;
                RHS[cell * 2 + 0] = U[cell * 2 + 1];
                RHS[cell * 2 + 1] = r1_h * (Fp - Fm) + r1_h * (Gp - Gm) + r1_h * (Hp - Hm);
            }
#undef ACG
    if (g_src_on) {
        const double r1_h3 = 1. / ((g->h) * (g->h) * (g->h));
        RHS[(((size_t)g_src[2] * ny + g_src[1]) * nx + g_src[0]) * 2 + 1] += src_wavelet(g_src_t) * r1_h3;
    }
    if (g_rec_on) rec_sample(g_src_t, U[(((size_t)g_rec[2] * ny + g_rec[1]) * nx + g_rec[0]) * 2]);
    free(P.pad);
    free(GR);
    return 0;
}

int orc_acoustic_run(const orc_acoustic_cfg* g, int nsteps, double dt, double t_final, double* U, double* t_inout,
                     int* steps_taken) {
    const size_t n = (size_t)g->nx * g->ny * g->nz * 2;
    double* W = (double*)malloc(sizeof(double) * n);
    double* L = (double*)malloc(sizeof(double) * n);
    if (!W || !L) return 3;
    double t = *t_inout;
    int s = 0;
    for (; s < nsteps; ++s) {
        if (t_final > 0.0 && t >= t_final) break;
        double h = dt;
        if (t_final > 0.0 && t + h > t_final) h = t_final - t;
        /* SSP RKS3, 4 stages (Ketcheson 2008, low-storage form as PETSc's TSSSP;
         * the same operation order as orc_euler_run) */
        const double dtr = h / 2;
        const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * h / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
        /* stage times of PETSc's RKS3 with 4 stages: t + (0, 1/2, 1, 1/2) h */
        orc_acoustic_rhs_at(g, t + 1.0 * 0 / (4 - 2) * h, U, L);
        for (size_t q = 0; q < n; ++q) W[q] = U[q] + dtr * L[q];
        orc_acoustic_rhs_at(g, t + 1.0 * 1 / (4 - 2) * h, W, L);
        for (size_t q = 0; q < n; ++q) W[q] = W[q] + dtr * L[q];
        orc_acoustic_rhs_at(g, t + 1.0 * 2 / (4 - 2) * h, W, L);
        for (size_t q = 0; q < n; ++q) W[q] = a3 * U[q] + b3 * L[q] + c3 * W[q];
        orc_acoustic_rhs_at(g, t + (1.0 * 3 - 2) / (4 - 2) * h, W, L);
        for (size_t q = 0; q < n; ++q) U[q] = W[q] + dtr * L[q];
        t += h;
    }
    free(W);
    free(L);
    *t_inout = t;
    if (steps_taken) *steps_taken = s;
    return 0;
}

static const double AC_XGP5[5] = {0.0000000000000000, -0.2692346550528416, 0.2692346550528416, -0.4530899229693320,
                                  0.4530899229693320};
static const double AC_WGP5[5] = {0.28444444444444444, 0.23931433524968326, 0.23931433524968326, 0.11846344252809456,
                                  0.11846344252809456};

/* cell (i,j,k): the corner x_min + i h of the periodic DMDA's uniform coordinates, and
 * the reference's quadrature offsets l*h*x_gp5[l] (initialize_solution.c:56-58) */
static void ac_project(const orc_acoustic_cfg* g, int i, int j, int k, double t, int exact, double* out) {
    const double h = g->h, pi2 = 2.0 * 3.14159265358979323846;
    const double xc = (g->xmin + 0.5 * h + i * (pi2 / g->nx)) - 0.5 * h;
    const double yc = (g->ymin + 0.5 * h + j * (pi2 / g->ny)) - 0.5 * h;
    const double zc = (g->zmin + 0.5 * h + k * (pi2 / g->nz)) - 0.5 * h;
    const double omega = 1.0 * sqrt(1.0 * 1.0 + 1.0 * 1.0 + 1.0 * 1.0);
    double a0 = 0.0, a1 = 0.0;
    for (int l = 0; l < 5; l++)
        for (int m = 0; m < 5; m++)
            for (int n = 0; n < 5; ++n) {
                const double x = xc + (double)l * h * AC_XGP5[l];
                const double y = yc + (double)m * h * AC_XGP5[m];
                const double z = zc + (double)n * h * AC_XGP5[n];
                const double ph = exact ? 1.0 * x + 1.0 * y + 1.0 * z - omega * t : 1.0 * x + 1.0 * y + 1.0 * z;
                const double w = AC_WGP5[l] * AC_WGP5[m] * AC_WGP5[n];
                a0 += w * sin(ph);
                a1 += w * (-omega * cos(ph));
            }
    out[0] = a0;
    out[1] = a1;
}

void orc_acoustic_plane_wave_ic(const orc_acoustic_cfg* g, double* U) {
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) ac_project(g, i, j, k, 0.0, 0, U + (((size_t)k * g->ny + j) * g->nx + i) * 2);
}

void orc_acoustic_plane_wave_errors(const orc_acoustic_cfg* g, const double* U, double t, double* l2, double* linf) {
    double s2 = 0.0, mx = 0.0;
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                double e[2];
                ac_project(g, i, j, k, t, 1, e);
                const double d = e[0] - U[(((size_t)k * g->ny + j) * g->nx + i) * 2];
                s2 += d * d;
                if (fabs(d) > mx) mx = fabs(d);
            }
    *l2 = sqrt(s2) * pow(g->h, 1.5);
    *linf = mx;
}

/* ============================================================ Taylor-Green vortex (Navier-Stokes-3D)
 * InitialCondition    3d/weno4/Navier-Stokes-3D/initial_condition.c (rho 1, p 100/gamma,
 *                     primitive -> conserved by PDEPrim2Cons, pde.c:24-34)
 * InitializeSolution  initialize_solution.c: 5^3 Gauss sum at the offsets l*h*x_gp5[l]
 *                     from the cell corner, the corner taken from the periodic DMDA's
 *                     uniform coordinates (hype.c:114-116)
 * KineticEnergy       kinetic_energy.c:10-36
 * Dissipation         dissipation.c:10-70 (central differences of the velocity) */
static void tgv_cons(double gamma, double x, double y, double z, double* Q) {
    const double rho_0 = 1.0, p_0 = 100.0 / gamma;
    double V[5];
    V[0] = rho_0;
    V[1] = sin(x) * cos(y) * cos(z);
    V[2] = -cos(x) * sin(y) * cos(z);
    V[3] = 0.0;
    V[4] = p_0 + (rho_0 / 16.0) * (cos(2.0 * z) + 2.0) * (cos(2.0 * x) + cos(2.0 * y) - 2.0);
    const double e = V[4] / (gamma - 1.0);
    const double k = 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2] + V[3] * V[3]);
    Q[0] = V[0];
    Q[1] = V[0] * V[1];
    Q[2] = V[0] * V[2];
    Q[3] = V[0] * V[3];
    Q[4] = k + e;
}

void orc_tgv_ic(const orc_euler_cfg* g, double* U) {
    const double h = g->h;
    /* DMDASetUniformCoordinates(da, x_min + h/2, x_max + h/2, ...) on periodic axes */
    const double x0 = g->xmin + 0.5 * h, y0 = g->ymin + 0.5 * h, z0 = g->zmin + 0.5 * h;
    const double hx = ((g->xmin + g->nx * h + 0.5 * h) - x0) / g->nx;
    const double hy = ((g->ymin + g->ny * h + 0.5 * h) - y0) / g->ny;
    const double hz = ((g->zmin + g->nz * h + 0.5 * h) - z0) / g->nz;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = 0; k < g->nz; ++k)
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const double xc = (x0 + hx * i) - 0.5 * h, yc = (y0 + hy * j) - 0.5 * h, zc = (z0 + hz * k) - 0.5 * h;
                double integral[5] = {0, 0, 0, 0, 0};
                for (int l = 0; l < 5; l++)
                    for (int m = 0; m < 5; m++)
                        for (int n = 0; n < 5; ++n) {
                            double Q0[5];
                            tgv_cons(g->gamma, xc + (double)l * h * AC_XGP5[l], yc + (double)m * h * AC_XGP5[m],
                                     zc + (double)n * h * AC_XGP5[n], Q0);
                            for (int c = 0; c < 5; ++c) integral[c] += AC_WGP5[l] * AC_WGP5[m] * AC_WGP5[n] * Q0[c];
                        }
                double* u = U + (((size_t)k * g->ny + j) * g->nx + i) * 5;
                for (int c = 0; c < 5; ++c) u[c] = integral[c];
            }
}

double orc_kinetic_energy(const orc_euler_cfg* g, const double* U) {
    const double h = g->h, vol = h * h * h;
    double ke = 0.0;
    for (size_t q = 0; q < (size_t)g->nx * g->ny * g->nz; ++q) {
        const double* u = U + q * 5;
        ke += vol * 0.5 * (u[1] * u[1] + u[2] * u[2] + u[3] * u[3]) / u[0];
    }
    return ke;
}

double orc_dissipation(const orc_euler_cfg* g, const double* U) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const double r1_2h = 0.5 / g->h, mu = g->mu;
#define TGV_U(i, j, k, c) U[((((size_t)(((k) + nz) % nz) * ny + (((j) + ny) % ny)) * nx + (((i) + nx) % nx)) * 5) + (c)]
#define VEL(i, j, k, c) (TGV_U(i, j, k, c) / TGV_U(i, j, k, 0))
    double dr = 0.0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const double u_x = r1_2h * (VEL(i + 1, j, k, 1) - VEL(i - 1, j, k, 1));
                const double u_y = r1_2h * (VEL(i, j + 1, k, 1) - VEL(i, j - 1, k, 1));
                const double u_z = r1_2h * (VEL(i, j, k + 1, 1) - VEL(i, j, k - 1, 1));
                const double v_x = r1_2h * (VEL(i + 1, j, k, 2) - VEL(i - 1, j, k, 2));
                const double v_y = r1_2h * (VEL(i, j + 1, k, 2) - VEL(i, j - 1, k, 2));
                const double v_z = r1_2h * (VEL(i, j, k + 1, 2) - VEL(i, j, k - 1, 2));
                const double w_x = r1_2h * (VEL(i + 1, j, k, 3) - VEL(i - 1, j, k, 3));
                const double w_y = r1_2h * (VEL(i, j + 1, k, 3) - VEL(i, j - 1, k, 3));
                const double w_z = r1_2h * (VEL(i, j, k + 1, 3) - VEL(i, j, k - 1, 3));
                const double div_v = -(2.0 / 3.0) * mu * (u_x + v_y + w_z);
                const double tau_xx = div_v + 2.0 * mu * u_x, tau_xy = mu * (u_y + v_x), tau_xz = mu * (u_z + w_x);
                const double tau_yy = div_v + 2.0 * mu * v_y, tau_yz = mu * (v_z + w_y), tau_zz = div_v + 2.0 * mu * w_z;
                dr += (tau_xx * u_x + tau_xy * u_y + tau_xz * u_z) + (tau_xy * v_x + tau_yy * v_y + tau_yz * v_z) +
                      (tau_xz * w_x + tau_yz * w_y + tau_zz * w_z);
            }
#undef VEL
#undef TGV_U
    return dr;
}


/* ============================================================ 2D acoustic FV (standing_wave)
 * RHSFunction              2d/weno4/standing_wave/rhs_function.c:12-258 (adiabatic ghosts
 *                          :46-95, reconstruction + face gradients :97-150, fluxes
 *                          :152-205, RHS :207-216)
 * weno()                   2d/weno4/standing_wave/reconstruction.c:108-125 (the R4 polynomial)
 * basis_grad tables        reconstruction.c:50-100, filled as hype.c:137-166 fills them
 * PDEFlux, LLFRiemannSolver pde.c:12-34
 * SSP RK104                PETSc TSSSP RK104 (Ketcheson 2008), restated in oracle/petsc_shim
 * InitializeSolution, ErrorNorms  initialize_solution.c:10-68, post_process.c:80-152 */
static void sw_basis_grad(double x, double y, int n, double* gx, double* gy) {
    switch (n) {
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

static const double SW_GP2[2] = {-0.28867513459481287, 0.28867513459481287};

/* phi[f][q][k][d]: the basis gradients at Gauss point q of edge f (left, right, bottom, top) */
static void sw_tables(double phi[4][2][10][2]) {
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 10; ++k) {
            sw_basis_grad(-0.5, SW_GP2[q], k, &phi[0][q][k][0], &phi[0][q][k][1]);
            sw_basis_grad(0.5, SW_GP2[q], k, &phi[1][q][k][0], &phi[1][q][k][1]);
            sw_basis_grad(SW_GP2[q], -0.5, k, &phi[2][q][k][0], &phi[2][q][k][1]);
            sw_basis_grad(SW_GP2[q], 0.5, k, &phi[3][q][k][0], &phi[3][q][k][1]);
        }
}

/* u of cell (i, j) with the program's ghost values: periodic wrap, or the wall's odd mirror */
static double sw_u(const orc_sw2d_cfg* g, const double* U, int i, int j) {
    double s = 1.0;
    if (i < 0 || i >= g->nx) {
        if (g->bc[i < 0 ? 0 : 1] == 0) i = (i + g->nx) % g->nx;
        else { i = i < 0 ? -1 - i : 2 * (g->nx - 1) - i + 1; s = -s; }
    }
    if (j < 0 || j >= g->ny) {
        if (g->bc[j < 0 ? 2 : 3] == 0) j = (j + g->ny) % g->ny;
        else { j = j < 0 ? -1 - j : 2 * (g->ny - 1) - j + 1; s = -s; }
    }
    const double v = U[((size_t)j * g->nx + i) * 2];
    return s < 0 ? -v : v;
}

int orc_sw2d_rhs_at(const orc_sw2d_cfg* g, double t, const double* U, double* RHS) {
    g_src_t = t;
    return orc_sw2d_rhs(g, U, RHS);
}

int orc_sw2d_rhs(const orc_sw2d_cfg* g, const double* U, double* RHS) {
    const int nx = g->nx, ny = g->ny, ex = nx + 2;
    const double r1_h = 1. / (g->h);
    static const double r41_60 = 41. / 60., r11_120 = 11. / 120., r1_6 = 1. / 6., r1_12 = 1. / 12.;
    double phi[4][2][10][2];
    sw_tables(phi);
    /* gr[((j+1)*ex + (i+1))*16 + (f*2+q)*2 + d]: the r1_h-scaled gradients */
    double* gr = (double*)malloc(sizeof(double) * (size_t)ex * (ny + 2) * 16);
    double* F = (double*)malloc(sizeof(double) * (size_t)(nx + 1) * ny);
    double* G = (double*)malloc(sizeof(double) * (size_t)nx * (ny + 1));
    if (!gr || !F || !G) return 3;
#pragma omp parallel for schedule(static)
    for (int j = -1; j < ny + 1; ++j)
        for (int i = -1; i < nx + 1; ++i) {
            const double u_0 = sw_u(g, U, i, j);
            const double u_ip1 = sw_u(g, U, i + 1, j), u_jp1 = sw_u(g, U, i, j + 1), u_ip1jp1 = sw_u(g, U, i + 1, j + 1);
            const double u_im1 = sw_u(g, U, i - 1, j), u_jm1 = sw_u(g, U, i, j - 1), u_ip1jm1 = sw_u(g, U, i + 1, j - 1);
            const double u_ip2 = sw_u(g, U, i + 2, j), u_jp2 = sw_u(g, U, i, j + 2), u_im1jp1 = sw_u(g, U, i - 1, j + 1);
            const double u_im2 = sw_u(g, U, i - 2, j), u_jm2 = sw_u(g, U, i, j - 2), u_im1jm1 = sw_u(g, U, i - 1, j - 1);
            double c[10];
            c[0] = u_0;
            c[1] = r41_60 * (-u_im1 + u_ip1) + r11_120 * (u_im2 - u_ip2);
            c[2] = r41_60 * (-u_jm1 + u_jp1) + r11_120 * (u_jm2 - u_jp2);
            c[3] = -u_0 + 0.5 * (u_im1 + u_ip1);
            c[4] = -u_0 + 0.5 * (u_jm1 + u_jp1);
            c[5] = 0.25 * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
            c[6] = r1_6 * (u_im1 - u_ip1) + r1_12 * (u_ip2 - u_im2);
            c[7] = r1_6 * (u_jm1 - u_jp1) + r1_12 * (u_jp2 - u_jm2);
            c[8] = 0.25 * (-u_im1jm1 + u_im1jp1 - u_ip1jm1 + u_ip1jp1) + 0.5 * (u_jm1 - u_jp1);
            c[9] = 0.5 * (u_im1 - u_ip1) + 0.25 * (u_ip1jp1 - u_im1jm1 - u_im1jp1 + u_ip1jm1);
            double* o = gr + ((size_t)(j + 1) * ex + (i + 1)) * 16;
            for (int f = 0; f < 4; ++f)
                for (int q = 0; q < 2; ++q) {
                    double gx = 0.0, gy = 0.0;
                    for (int k = 0; k < 10; ++k) {
                        gx += c[k] * phi[f][q][k][0];
                        gy += c[k] * phi[f][q][k][1];
                    }
                    o[(f * 2 + q) * 2] = r1_h * gx;
                    o[(f * 2 + q) * 2 + 1] = r1_h * gy;
                }
        }
    const double c2 = g->c * g->c;
#define SWG(i, j, f, q, d) gr[((size_t)((j) + 1) * ex + ((i) + 1)) * 16 + ((f) * 2 + (q)) * 2 + (d)]
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx + 1; ++i) {
            double flux = 0.0;
            for (int q = 0; q < 2; ++q) {
                const double FL = c2 * (SWG(i - 1, j, 1, q, 0) * 1.0 + SWG(i - 1, j, 1, q, 1) * 0.0);
                const double FR = c2 * (SWG(i, j, 0, q, 0) * 1.0 + SWG(i, j, 0, q, 1) * 0.0);
                flux += 0.5 * (0.5 * (FR + FL));
            }
            F[(size_t)j * (nx + 1) + i] = flux;
        }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny + 1; ++j)
        for (int i = 0; i < nx; ++i) {
            double flux = 0.0;
            for (int q = 0; q < 2; ++q) {
                const double FL = c2 * (SWG(i, j - 1, 3, q, 0) * 0.0 + SWG(i, j - 1, 3, q, 1) * 1.0);
                const double FR = c2 * (SWG(i, j, 2, q, 0) * 0.0 + SWG(i, j, 2, q, 1) * 1.0);
                flux += 0.5 * (0.5 * (FR + FL));
            }
            G[(size_t)j * nx + i] = flux;
        }
#undef SWG
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const size_t q = (size_t)j * nx + i;
            RHS[q * 2] = U[q * 2 + 1];
            RHS[q * 2 + 1] = r1_h * (F[(size_t)j * (nx + 1) + i + 1] - F[(size_t)j * (nx + 1) + i]) +
                             r1_h * (G[(size_t)(j + 1) * nx + i] - G[(size_t)j * nx + i]);
        }
    if (g_src_on) {
        const double r1_h2 = 1. / ((g->h) * (g->h));
        RHS[((size_t)g_src[1] * nx + g_src[0]) * 2 + 1] += src_wavelet(g_src_t) * r1_h2;
    }
    if (g_rec_on) rec_sample(g_src_t, U[((size_t)g_rec[1] * nx + g_rec[0]) * 2]);
    free(gr);
    free(F);
    free(G);
    return 0;
}

int orc_sw2d_run(const orc_sw2d_cfg* g, int stepper, int nsteps, double dt, double t_final, double* U, double* t_inout,
                 int* steps_taken) {
    const size_t n = (size_t)g->nx * g->ny * 2;
    double* W0 = (double*)malloc(sizeof(double) * n);
    double* W1 = (double*)malloc(sizeof(double) * n);
    double* L = (double*)malloc(sizeof(double) * n);
    if (!W0 || !W1 || !L) return 3;
    double t = *t_inout;
    int s = 0;
    for (; s < nsteps; ++s) {
        if (t_final > 0.0 && t >= t_final) break;
        double h = dt;
        if (t_final > 0.0 && t + h > t_final) h = t_final - t;
        if (stepper == 1) {
            /* SSP RK104, low-storage: five stages of dt/6 on w0, w1 = 9/25 w0 + 1/25 w1,
             * w0 = 15 w1 - 5 w0, four stages of dt/6, u = 3/5 w0 + dt/10 L(w0) + w1 */
            memcpy(W0, U, sizeof(double) * n);
            memcpy(W1, U, sizeof(double) * n);
            static const double cst[10] = {0, 1. / 6, 2. / 6, 3. / 6, 4. / 6, 2. / 6, 3. / 6, 4. / 6, 5. / 6, 1};
            int i = 0;
            for (; i < 5; ++i) {
                g_src_t = t + cst[i] * h;
                orc_sw2d_rhs(g, W0, L);
                for (size_t q = 0; q < n; ++q) W0[q] = W0[q] + h / 6 * L[q];
            }
            for (size_t q = 0; q < n; ++q) W1[q] = 9.0 / 25 * W0[q] + 1.0 / 25 * W1[q];
            for (size_t q = 0; q < n; ++q) W0[q] = 15 * W1[q] + -5 * W0[q];
            for (; i < 9; ++i) {
                g_src_t = t + cst[i] * h;
                orc_sw2d_rhs(g, W0, L);
                for (size_t q = 0; q < n; ++q) W0[q] = W0[q] + h / 6 * L[q];
            }
            g_src_t = t + h;
            orc_sw2d_rhs(g, W0, L);
            for (size_t q = 0; q < n; ++q) U[q] = 3.0 / 5 * W0[q] + h / 10 * L[q] + 1 * W1[q];
        } else {
            const double dtr = h / 2;
            const double a3 = 1.0 * 2 / (2 * 2 - 1.0), b3 = (2 - 1.0) * h / (2 * (2 * 2 - 1)), c3 = (2 - 1.0) / (2 * 2 - 1);
            g_src_t = t + 1.0 * 0 / (4 - 2) * h;
            orc_sw2d_rhs(g, U, L);
            for (size_t q = 0; q < n; ++q) W0[q] = U[q] + dtr * L[q];
            g_src_t = t + 1.0 * 1 / (4 - 2) * h;
            orc_sw2d_rhs(g, W0, L);
            for (size_t q = 0; q < n; ++q) W0[q] = W0[q] + dtr * L[q];
            g_src_t = t + 1.0 * 2 / (4 - 2) * h;
            orc_sw2d_rhs(g, W0, L);
            for (size_t q = 0; q < n; ++q) W0[q] = a3 * U[q] + b3 * L[q] + c3 * W0[q];
            g_src_t = t + (1.0 * 3 - 2) / (4 - 2) * h;
            orc_sw2d_rhs(g, W0, L);
            for (size_t q = 0; q < n; ++q) U[q] = W0[q] + dtr * L[q];
        }
        t += h;
    }
    free(W0);
    free(W1);
    free(L);
    *t_inout = t;
    if (steps_taken) *steps_taken = s;
    return 0;
}

/* the DMDA's cell-centre coordinate of index i on an axis: DMDASetUniformCoordinates over
 * [lo + h/2, hi - h/2], spacing (span)/n periodic, (span)/(n-1) otherwise */
static double sw_coord(double lo, double hi, double h, int n, int periodic, int i) {
    const double a = lo + 0.5 * h, b = hi - 0.5 * h;
    const double hh = periodic ? (b - a) / n : (b - a) / (n - 1);
    return a + i * hh;
}

static void sw_project(const orc_sw2d_cfg* g, int i, int j, double t, int exact, double* out) {
    const double h = g->h;
    const double xc = sw_coord(g->xmin, g->xmax, h, g->nx, g->bc[0] == 0, i);
    const double yc = sw_coord(g->ymin, g->ymax, h, g->ny, g->bc[2] == 0, j);
    const double kx = 2 * 3.14159265358979323846, ky = 2 * 3.14159265358979323846;
    const double omega = g->c * sqrt(kx * kx + ky * ky);
    double a0 = 0.0, a1 = 0.0;
    for (int l = 0; l < 5; l++)
        for (int m = 0; m < 5; m++) {
            const double x = xc + h * AC_XGP5[l], y = yc + h * AC_XGP5[m];
            const double w = AC_WGP5[l] * AC_WGP5[m];
            if (exact) {
                a0 += w * (sin(kx * x) * sin(ky * y) * cos(omega * t));
                a1 += w * (-omega * sin(kx * x) * sin(ky * y) * sin(omega * t));
            } else {
                a0 += w * (sin(kx * x) * sin(ky * y));
                a1 += w * 0.0;
            }
        }
    out[0] = a0;
    out[1] = a1;
}

void orc_sw2d_ic(const orc_sw2d_cfg* g, double* U) {
#pragma omp parallel for schedule(static)
    for (int j = 0; j < g->ny; ++j)
        for (int i = 0; i < g->nx; ++i) sw_project(g, i, j, 0.0, 0, U + ((size_t)j * g->nx + i) * 2);
}

void orc_sw2d_errors(const orc_sw2d_cfg* g, const double* U, double t, double* l2, double* linf) {
    /* U_exact - U over the vector with the u_t entries zeroed in both (post_process.c:118-149) */
    double s2 = 0.0, mx = 0.0;
    for (int j = 0; j < g->ny; ++j)
        for (int i = 0; i < g->nx; ++i) {
            double e[2];
            sw_project(g, i, j, t, 1, e);
            const size_t q = ((size_t)j * g->nx + i) * 2;
            const double d0 = e[0] + -1.0 * U[q], d1 = 0.0 + -1.0 * 0.0;
            s2 += d0 * d0;
            s2 += d1 * d1;
            if (fabs(d0) > mx) mx = fabs(d0);
            if (fabs(d1) > mx) mx = fabs(d1);
        }
    *l2 = sqrt(s2) / ((double)g->nx);
    *linf = mx;
}
