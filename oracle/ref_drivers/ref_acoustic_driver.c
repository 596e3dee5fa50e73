/*
 * ref_acoustic_driver.c -- TEST INFRASTRUCTURE: drives the reference's own acoustic
 * finite-volume RHS of 3d/weno4/plane_wave (rhs_function.c:12-345, reconstruction.c,
 * pde.c, array.c, compiled unmodified through the PETSc shim).  The set-up mirrors
 * 3d/weno4/plane_wave/hype.c:96-186: a dof-2 DMDA with box stencil width 3, the
 * gradient-trace and flux scratch, and TSSSP RKS3 with 4 stages, a fixed dt and
 * TS_EXACTFINALTIME_MATCHSTEP.
 */
#include "hype.h"
#include <setjmp.h>

/* bc codes shared with the GPU library: 0 periodic, 4 adiabatic */
static enum bndry_type map_bc(int b) { return b == 4 ? adiabatic : periodic; }

typedef struct {
    AppCtx ctx;
    DM da;
    Vec U, RHS;
    TS ts;
} RefAcoustic;

static void setup(RefAcoustic* R, int nx, int ny, int nz, double h, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->N_x = nx; C->N_y = ny; C->N_z = nz;
    C->h = h;
    C->x_max = nx * h; C->y_max = ny * h; C->z_max = nz * h;
    C->left_boundary = map_bc(bc[0]); C->right_boundary = map_bc(bc[1]);
    C->bottom_boundary = map_bc(bc[2]); C->top_boundary = map_bc(bc[3]);
    C->back_boundary = map_bc(bc[4]); C->front_boundary = map_bc(bc[5]);
    DMBoundaryType bx = C->left_boundary == periodic ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType by = C->bottom_boundary == periodic ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType bz = C->back_boundary == periodic ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMDACreate3d(PETSC_COMM_WORLD, bx, by, bz, DMDA_STENCIL_BOX, nx, ny, nz, PETSC_DECIDE, PETSC_DECIDE, PETSC_DECIDE, nVar,
                 3, NULL, NULL, NULL, &R->da);
    DMSetUp(R->da);
    DMCreateGlobalVector(R->da, &R->U);
    VecDuplicate(R->U, &R->RHS);
    PetscInt xs, ys, zs, xm, ym, zm;
    DMDAGetCorners(R->da, &xs, &ys, &zs, &xm, &ym, &zm);
    C->u_bnd_grad = allocate7d(zm + 2, ym + 2, xm + 2, nVar, 6, N_gp2d, DIM);
    C->F = allocate3d(zm, ym, xm + 1);
    C->G = allocate3d(zm, ym + 1, xm);
    C->H = allocate3d(zm + 1, ym, xm);
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefAcoustic* R) {
    free7d(R->ctx.u_bnd_grad);
    free3d(R->ctx.F); free3d(R->ctx.G); free3d(R->ctx.H);
    VecDestroy(&R->ctx.localU);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

int ref_acoustic_rhs(int nx, int ny, int nz, double h, const int* bc, const double* U_aos, double* RHS_aos) {
    RefAcoustic R;
    setup(&R, nx, ny, nz, h, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
    memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
    teardown(&R);
    return 0;
}

/* up to nsteps steps of dt (t_final > 0: MaxTime with MATCHSTEP, as hype.c:177-178) */
int ref_acoustic_run(int nx, int ny, int nz, double h, const int* bc, int nsteps, double dt, double t_final,
                     double* U_aos, double* t_out) {
    RefAcoustic R;
    setup(&R, nx, ny, nz, h, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    R.ctx.dt = dt;
    TSSetRHSFunction(R.ts, NULL, RHSFunction, &R.ctx);
    TSSetStepNumber(R.ts, 0);
    TSSetTime(R.ts, 0.0);
    TSSetTimeStep(R.ts, dt);
    TSSetMaxTime(R.ts, t_final > 0.0 ? t_final : 1e300);
    TSSetMaxSteps(R.ts, nsteps);
    TSSetExactFinalTime(R.ts, TS_EXACTFINALTIME_MATCHSTEP);
    TSSetType(R.ts, TSSSP);
    TSSSPSetType(R.ts, TSSSPRKS3);
    TSSSPSetNumStages(R.ts, 4);
    TSSolve(R.ts, R.U);
    memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
    if (t_out) *t_out = R.ts->t;
    teardown(&R);
    return 0;
}

#ifdef REF_POINT_SOURCE
#include <unistd.h>
/* 3d/weno4/point_source: the same set-up plus its source and receiver cells (AppCtx
 * isx..irz, hype.c:59-64).  Its RHSFunction appends the receiver to results/p.dat under the
 * working directory (rhs_function.c:342-346), so the run switches to dir (which holds a
 * results/ folder) while it lasts.  initial_rhs: the program's RHSFunction call at the
 * initial time before TSSolve (hype.c:160), which prints one receiver line. */
static void set_points(RefAcoustic* R, const int* src, const int* rec) {
    R->ctx.isx = src[0]; R->ctx.isy = src[1]; R->ctx.isz = src[2];
    R->ctx.irx = rec[0]; R->ctx.iry = rec[1]; R->ctx.irz = rec[2];
}

int ref_psrc3d_rhs(int nx, int ny, int nz, double h, const int* bc, const int* src, const int* rec, double t,
                   const double* U_aos, double* RHS_aos, const char* dir) {
    char old[4096];
    if (!getcwd(old, sizeof old) || chdir(dir)) return 1;
    RefAcoustic R;
    setup(&R, nx, ny, nz, h, bc);
    set_points(&R, src, rec);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    RHSFunction(R.ts, t, R.U, R.RHS, &R.ctx);
    memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
    teardown(&R);
    return chdir(old) ? 1 : 0;
}

int ref_psrc3d_run(int nx, int ny, int nz, double h, const int* bc, const int* src, const int* rec, int initial_rhs,
                   int nsteps, double dt, double t_final, double* U_aos, double* t_out, const char* dir) {
    char old[4096];
    if (!getcwd(old, sizeof old) || chdir(dir)) return 1;
    RefAcoustic R;
    setup(&R, nx, ny, nz, h, bc);
    set_points(&R, src, rec);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    R.ctx.dt = dt;
    if (initial_rhs) RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
    TSSetRHSFunction(R.ts, NULL, RHSFunction, &R.ctx);
    TSSetStepNumber(R.ts, 0);
    TSSetTime(R.ts, 0.0);
    TSSetTimeStep(R.ts, dt);
    TSSetMaxTime(R.ts, t_final > 0.0 ? t_final : 1e300);
    TSSetMaxSteps(R.ts, nsteps);
    TSSetExactFinalTime(R.ts, TS_EXACTFINALTIME_MATCHSTEP);
    TSSetType(R.ts, TSSSP);
    TSSSPSetType(R.ts, TSSSPRKS3);
    TSSSPSetNumStages(R.ts, 4);
    TSSolve(R.ts, R.U);
    memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
    if (t_out) *t_out = R.ts->t;
    teardown(&R);
    return chdir(old) ? 1 : 0;
}
#endif
