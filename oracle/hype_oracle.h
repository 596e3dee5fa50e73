/*
 * hype_oracle.h -- CPU restatement of the reference's hot path.
 * TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
 * baseline leg of bench.py as the checker.  The GPU product never calls it.
 *
 * Layouts follow the reference's DMDA vectors: AoS doubles [k][j][i][c],
 * x fastest, no ghosts (ghosts are built internally from the boundary codes).
 */
#ifndef HYPE_ORACLE_H
#define HYPE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* boundary codes (shared with include/hype_gpu.h) */
#define ORC_BC_PERIODIC 0
#define ORC_BC_REFLECTIVE 1
#define ORC_BC_TRANSMISSIVE 2
#define ORC_BC_ZERO 3

/* 2D CTCS, reference form of 2d/ctcs/plane_wave/wave.c:192 (5-point, alpha = c dt / h). */
int orc_ctcs2d_plane(int nx, int ny, double alpha, int bc, int nsteps, double* p_old, double* p, double* scratch);

/* 2D/3D CTCS, reference form of 2d/ctcs/line_source/wave.c:155-173 and
 * 3d/ctcs/point_source/wave.c:173-194: 2nd (order=2) or 4th (order=4) order
 * Laplacian, c field (NULL -> constant c0), optional Ricker-type point source
 * (src_i < 0 -> none) with dominant frequency f0, receiver trace out. */
typedef struct {
    int dim, nx, ny, nz, order, bc;
    double dx, dy, dz, dt, c0, f0;
    int src_i, src_j, src_k;
    int rec_i, rec_j, rec_k;
    int it0; /* step counter of the first update (time = it*dt) */
} orc_ctcs_cfg;
int orc_ctcs_pointsrc(const orc_ctcs_cfg* cfg, const double* c, int nsteps, double* p_old, double* p, double* scratch,
                      double* receiver);

/* Gaussian-monopole CTCS (one batched-acoustics instance): 2nd-order form of
 * 2d/ctcs/line_source/wave.c with s(x,t)=exp(-|x-xs|^2/(2 sig^2)) sin(2 pi f t)
 * added as c^2 dt^2 s at node (i,j), x_i = xmin + i h. */
typedef struct {
    int nx, ny;
    double xmin, ymin, h, c0, dt, xs, ys, sigma, freq;
    int it0;
} orc_mono_cfg;
int orc_ctcs_monopole(const orc_mono_cfg* cfg, int nsteps, double* p_old, double* p, double* scratch);

/* 3D Euler RHS: CWENO4 reconstruction + Rusanov flux (see hype_oracle.c for the
 * reference lines followed).  bc[6] = left,right,bottom,top,back,front.
 * Returns 0, or 2 for an inadmissible state (then *bad = first offending
 * linear cell index of the face's right cell). */
typedef struct {
    int nx, ny, nz;
    double xmin, ymin, zmin, h, cfl, gamma;
    int bc[6];
    int recon; /* 0 = CWENO4 (gamma 0.85), 1 = linear R4 (the optimal-weight polynomial),
                  3 = WENO3 (3d/weno3/Euler/reconstruction.c:29-177) */
    int nthreads;
    int flux;  /* 0 = Rusanov (LLF), 1 = HLLC, 2 = rotated HLLC (Navier-Stokes-3D/pde.c:164-384) */
    int positivity; /* 1: first-order fallback of cells with an inadmissible face trace */
    double mu, prandtl, cv; /* mu > 0: viscous fluxes of Navier-Stokes-3D/pde.c:90-162,386-404 */
} orc_euler_cfg;
long orc_positivity_fallbacks(int reset);
int orc_euler_rhs(const orc_euler_cfg* cfg, const double* U, double* RHS, double* smax_out, long* bad);
/* the largest viscous wave speed of the last orc_euler_rhs call (0 without viscosity) */
double orc_euler_last_smax_visc(void);
/* Taylor-Green vortex of 3d/weno4/Navier-Stokes-3D/initial_condition.c projected as its
 * initialize_solution.c does (its 3D Gauss-point offsets), and the diagnostics that its
 * monitor writes to ke.csv: kinetic_energy.c and dissipation.c */
void orc_tgv_ic(const orc_euler_cfg* cfg, double* U);
double orc_kinetic_energy(const orc_euler_cfg* cfg, const double* U);
double orc_dissipation(const orc_euler_cfg* cfg, const double* U);
/* SSPRK(4,3) steps with dt semantics: dt_mode 0 -> dt refreshed each step from
 * the last stage RHS (Navier-Stokes-3D monitor), 1 -> frozen at the initial RHS
 * value, 2 -> *dt_inout for every step, 3 -> as 0, continuing an earlier call: the
 * first step takes *dt_inout (the dt that call handed back).  Returns 0 or the RHS error. */
int orc_euler_run(const orc_euler_cfg* cfg, int nsteps, int dt_mode, double* U, double* t_inout, double* dt_inout, long* bad);

/* Single-cell CWENO4 coefficients from the 33-point stencil in the reference's
 * argument order (U_x[5],U_y[5],U_z[5],U_xy[5],U_yz[5],U_zx[5],U_xyz[8]). */
void orc_cweno4_ref_args(const double* Ux, const double* Uy, const double* Uz, const double* Uxy, const double* Uyz,
                         const double* Uzx, const double* Uxyz, double* coeffs);
double orc_eval_poly3(double x, double y, double z, const double* coeffs);
double orc_rusanov(const double* QL, const double* QR, int dir, double gamma, double* flux, int* bad);
double orc_hllc(const double* QL, const double* QR, double nx, double ny, double nz, double gamma, double* flux, int* bad);
double orc_rothllc(const double* QL, const double* QR, double nx, double ny, double nz, double gamma, double* flux, int* bad);

/* 2D multiphase RHS: model 0 = 4-equation diffuse interface (2d/weno4/bubble),
 * model 1 = Kapila five-equation (2d/HyPE-2D/kapila_5eqn.c) with the same
 * machinery.  AoS [j][i][nv], nv = 5 or 6; bc[4] = left,right,bottom,top;
 * EOS: phase 1 (g1, p1), phase 2 (g2, p2). */
typedef struct {
    int nx, ny;
    double xmin, ymin, h, cfl;
    int bc[4];
    int model;
    double g1, p1, g2, p2;
    int nthreads;
} orc_mp2d_cfg;
int orc_mp2d_rhs(const orc_mp2d_cfg* g, const double* U, double* RHS, double* smax_out, long* bad_out, long* fallback_out);
int orc_mp2d_run(const orc_mp2d_cfg* g, int nsteps, int stepper, int dt_mode, double* U, double* t_inout, double* dt_inout,
                 long* bad);
void orc_mp_cons2prim(int model, const double* eos4, const double* Q, double* V);
void orc_mp_prim2cons(int model, const double* eos4, const double* V, double* Q);
void orc_cweno4_2d(double u0, const double* ux, const double* uy, double upp, double upm, double ump, double umm,
                   double* coeffs);

/* Acoustic FV path of 3d/weno4/plane_wave: state AoS [k][j][i][2] = (u, u_t);
 * bc[6]: 0 periodic, 4 adiabatic (odd mirror of u); recon: 1 = the R4 polynomial
 * (the reference's gammaHi = 1), 0 = CWENO4 with gamma 0.85. */
typedef struct {
    int nx, ny, nz;
    double xmin, ymin, zmin, h, c;
    int bc[6];
    int recon;
    int nthreads;
} orc_acoustic_cfg;
int orc_acoustic_rhs(const orc_acoustic_cfg* g, const double* U, double* RHS);
/* SSP RKS3 / 4 stages with fixed dt from *t_inout; t_final > 0: the step that would
 * pass it is shortened (TS_EXACTFINALTIME_MATCHSTEP) and the run stops there */
int orc_acoustic_run(const orc_acoustic_cfg* g, int nsteps, double dt, double t_final, double* U, double* t_inout,
                     int* steps_taken);
/* the plane wave of 3d/weno4/plane_wave/initial_condition.c (k = (1,1,1)) projected
 * as initialize_solution.c does, and error_norms.c's L2/Linf of u against the exact
 * solution at time t, both with the reference's 3D Gauss-point offsets l*h*x_gp5[l] */
void orc_acoustic_plane_wave_ic(const orc_acoustic_cfg* g, double* U);
void orc_acoustic_plane_wave_errors(const orc_acoustic_cfg* g, const double* U, double t, double* l2, double* linf);

/* 2D acoustic FV program of 2d/weno4/standing_wave: state AoS [j][i][2] = (u, u_t);
 * bc[4]: 0 periodic, 4 adiabatic wall (odd mirror of u); the 2D R4 polynomial (10
 * coefficients), its normal gradients at 2 Gauss points per edge, the averaged flux
 * c^2 grad u . n, RHS (u_t, div). stepper 0: SSP RKS3 / 4 stages, 1: SSP RK104. */
typedef struct {
    int nx, ny;
    double xmin, ymin, xmax, ymax, h, c;
    int bc[4];
} orc_sw2d_cfg;
int orc_sw2d_rhs(const orc_sw2d_cfg* g, const double* U, double* RHS);
int orc_sw2d_run(const orc_sw2d_cfg* g, int stepper, int nsteps, double dt, double t_final, double* U, double* t_inout,
                 int* steps_taken);
/* sin(2 pi x) sin(2 pi y) at the 5x5 Gauss points of the cell-centre coordinates of the
 * program's DMDA (initialize_solution.c), and ErrorNorms (post_process.c) at time t */
void orc_sw2d_ic(const orc_sw2d_cfg* g, double* U);
void orc_sw2d_errors(const orc_sw2d_cfg* g, const double* U, double t, double* l2, double* linf);

/* 3D primitive-variable multiphase RHS of 3d/weno4/Viscous-Multiphase-Fourth-Order
 * (RHSFunctionPrimitive): Q = (rho, rho u, rho v, rho w, E, phi), mixture EOS of two
 * stiffened gases (g1, p1) / (g2, p2) mixed by phi, CWENO4 of the primitive variables,
 * 33-node admissibility check with first-order fallback, rotated HLLC with the
 * non-conservative phi term, and the viscous speed (4/3)(phi mu1 + (1-phi) mu2)/rho in
 * dt (the program's viscous flux itself is not defined, see mphase3d_oracle.c).
 * bc[6]: 0 periodic, 1 reflective, 2 transmissive. */
typedef struct {
    int nx, ny, nz;
    double h, cfl;
    int bc[6];
    double g1, p1, g2, p2, mu1, mu2;
    int nthreads;
} orc_mp3d_cfg;
void orc_mp3d_cons2prim(const orc_mp3d_cfg* e, const double* Q, double* V);
void orc_mp3d_prim2cons(const orc_mp3d_cfg* e, const double* V, double* Q);
double orc_mp3d_rothllc(const orc_mp3d_cfg* e, const double* VL, const double* VR, double nx, double ny, double nz,
                        double* Flux, int* bad);
/* returns 0, or 2 for an inadmissible face state (the reference aborts) */
int orc_mp3d_rhs(const orc_mp3d_cfg* e, const double* U, double* RHS, double* dt_out, double* smax_out,
                 double* smaxv_out);
int orc_mp3d_run(const orc_mp3d_cfg* e, int nsteps, int dt_mode, double* U, double* t_inout, double* dt_inout);
long orc_mp3d_fallbacks(int reset);

/* 2D path-conservative RHS of 2d/HyPE-2D with its Kapila five-equation model:
 * Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1), reconstruction of the conservative
 * variables of order N (0..3), admissibility at the nodes with first order on failure,
 * Rusanov flux + Roe-path fluctuation, the non-conservative volume term, and dt =
 * CFL h / (2 s_max).  bc[4]: 0 periodic, 1 reflective, 2 transmissive. */
typedef struct {
    int N, nx, ny;
    double h, cfl;
    int bc[4];
    double g1, p1, g2, p2;
    int nthreads;
} orc_h2d_cfg;
/* returns 0, or 2 for an inadmissible face state (the reference aborts) */
int orc_h2d_rhs(const orc_h2d_cfg* e, const double* U, double* RHS, double* dt_out);
int orc_h2d_run(const orc_h2d_cfg* e, int nsteps, double* U, double* t_out, double* dt_out);

/* point source + receiver of 3d/weno4/point_source and 2d/weno4/line_source for the
 * acoustic FV paths above (the source cell's u_t equation gains Source(t) / h^dim, the
 * receiver records u at every RHS call); the RHS at time t; the trace buffer */
void orc_set_point_source(int on, int isx, int isy, int isz, double f0, int rec_on, int irx, int iry, int irz);
void orc_set_trace_buffer(double* t, double* p, int max);
int orc_trace_count(void);
int orc_acoustic_rhs_at(const orc_acoustic_cfg* g, double t, const double* U, double* RHS);
int orc_sw2d_rhs_at(const orc_sw2d_cfg* g, double t, const double* U, double* RHS);

/* OpenMP threads the restatement runs with */
int orc_threads(void);

#ifdef __cplusplus
}
#endif
#endif
