/*
 * ref_sw2d_driver.c -- TEST INFRASTRUCTURE: drives the reference's own 2D acoustic
 * finite-volume program 2d/weno4/standing_wave (rhs_function.c, reconstruction.c,
 * pde.c, initialize_solution.c, post_process.c, array.c, compiled unmodified through
 * the PETSc shim).  The set-up mirrors standing_wave/hype.c:30-215: a dof-2 DMDA with
 * box stencil width 3, cell-centre coordinates, the face basis-gradient tables, the
 * gradient and flux scratch, and TSSSP RK104 with a fixed dt and
 * TS_EXACTFINALTIME_MATCHSTEP.
 */
#include "hype.h"

/* bc codes shared with the GPU library: 0 periodic, 4 adiabatic wall */
static enum bndry_type map_bc(int b) { return b == 4 ? adiabatic_wall : periodic; }

typedef struct {
    AppCtx ctx;
    DM da;
    Vec U, RHS;
    TS ts;
} RefSW;

static void setup(RefSW* R, int nx, int ny, double xmin, double ymin, double xmax, double ymax, double h, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->N_x = nx; C->N_y = ny;
    C->h = h;
    C->x_min = xmin; C->y_min = ymin;
    C->x_max = xmax; C->y_max = ymax;
    C->left_boundary = map_bc(bc[0]); C->right_boundary = map_bc(bc[1]);
    C->bottom_boundary = map_bc(bc[2]); C->top_boundary = map_bc(bc[3]);
    DMBoundaryType bx = C->left_boundary == periodic ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType by = C->bottom_boundary == periodic ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMDACreate2d(PETSC_COMM_WORLD, bx, by, DMDA_STENCIL_BOX, nx, ny, PETSC_DECIDE, PETSC_DECIDE, nVar, 3, NULL, NULL,
                 &R->da);
    DMSetUp(R->da);
    DMCreateGlobalVector(R->da, &R->U);
    VecDuplicate(R->U, &R->RHS);
    DMDASetUniformCoordinates(R->da, C->x_min + 0.5 * C->h, C->x_max - 0.5 * C->h, C->y_min + 0.5 * C->h,
                              C->y_max - 0.5 * C->h, 0.0, 0.0);
    PetscInt xs, ys, xm, ym, q, k;
    PetscReal gx, gy;
    DMDAGetCorners(R->da, &xs, &ys, NULL, &xm, &ym, NULL);
    C->u_bnd_grad = allocate5d(ym + 2, xm + 2, 4, N_gp2, DIM);
    C->F = allocate2d(ym, xm + 1);
    C->G = allocate2d(ym + 1, xm);
    C->gradphiFace_x = allocate3d(4, N_gp2, nDOF);
    C->gradphiFace_y = allocate3d(4, N_gp2, nDOF);
    for (q = 0; q < N_gp2; ++q)
        for (k = 0; k < nDOF; ++k) {
            basis_grad(-0.5, x_gp2[q], k, &gx, &gy);
            set_element_3d(C->gradphiFace_x, 0, q, k, gx); set_element_3d(C->gradphiFace_y, 0, q, k, gy);
            basis_grad(0.5, x_gp2[q], k, &gx, &gy);
            set_element_3d(C->gradphiFace_x, 1, q, k, gx); set_element_3d(C->gradphiFace_y, 1, q, k, gy);
            basis_grad(x_gp2[q], -0.5, k, &gx, &gy);
            set_element_3d(C->gradphiFace_x, 2, q, k, gx); set_element_3d(C->gradphiFace_y, 2, q, k, gy);
            basis_grad(x_gp2[q], 0.5, k, &gx, &gy);
            set_element_3d(C->gradphiFace_x, 3, q, k, gx); set_element_3d(C->gradphiFace_y, 3, q, k, gy);
        }
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefSW* R) {
    free5d(R->ctx.u_bnd_grad);
    free2d(R->ctx.F); free2d(R->ctx.G);
    free3d(R->ctx.gradphiFace_x); free3d(R->ctx.gradphiFace_y);
    VecDestroy(&R->ctx.localU);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

int ref_sw2d_rhs(int nx, int ny, double xmin, double ymin, double h, const int* bc, const double* U_aos,
                 double* RHS_aos) {
    RefSW R;
    setup(&R, nx, ny, xmin, ymin, xmin + nx * h, ymin + ny * h, h, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
    memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
    teardown(&R);
    return 0;
}

static void solve(RefSW* R, int stepper, int nsteps, double dt, double t_final) {
    R->ctx.dt = dt;
    TSSetRHSFunction(R->ts, NULL, RHSFunction, &R->ctx);
    TSSetStepNumber(R->ts, 0);
    TSSetTime(R->ts, 0.0);
    TSSetTimeStep(R->ts, dt);
    TSSetMaxTime(R->ts, t_final > 0.0 ? t_final : 1e300);
    TSSetMaxSteps(R->ts, nsteps);
    TSSetExactFinalTime(R->ts, TS_EXACTFINALTIME_MATCHSTEP);
    TSSetType(R->ts, TSSSP);
    if (stepper == 1) {
        TSSSPSetType(R->ts, TSSSPRK104);
    } else {
        TSSSPSetType(R->ts, TSSSPRKS3);
        TSSSPSetNumStages(R->ts, 4);
    }
    TSSolve(R->ts, R->U);
}

/* up to nsteps steps of dt (t_final > 0: MaxTime with MATCHSTEP); stepper 1 = RK104 */
int ref_sw2d_run(int nx, int ny, double xmin, double ymin, double h, const int* bc, int stepper, int nsteps, double dt,
                 double t_final, double* U_aos, double* t_out) {
    RefSW R;
    setup(&R, nx, ny, xmin, ymin, xmin + nx * h, ymin + ny * h, h, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    solve(&R, stepper, nsteps, dt, t_final);
    memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
    if (t_out) *t_out = R.ts->t;
    teardown(&R);
    return 0;
}

#ifdef REF_LINE_SOURCE
#include <unistd.h>
/* 2d/weno4/line_source: the same set-up plus its source and receiver cells (AppCtx isx,
 * isy, irx, iry, hype.c:52-55); its RHSFunction appends the receiver to results/p.dat under
 * the working directory (rhs_function.c:249-253), so the run switches to dir meanwhile. */
int ref_lsrc2d_rhs(int nx, int ny, double h, const int* bc, const int* src, const int* rec, double t,
                   const double* U_aos, double* RHS_aos, const char* dir) {
    char old[4096];
    if (!getcwd(old, sizeof old) || chdir(dir)) return 1;
    RefSW R;
    setup(&R, nx, ny, 0.0, 0.0, nx * h, ny * h, h, bc);
    R.ctx.isx = src[0]; R.ctx.isy = src[1]; R.ctx.irx = rec[0]; R.ctx.iry = rec[1];
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    RHSFunction(R.ts, t, R.U, R.RHS, &R.ctx);
    memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
    teardown(&R);
    return chdir(old) ? 1 : 0;
}

int ref_lsrc2d_run(int nx, int ny, double h, const int* bc, const int* src, const int* rec, int stepper, int nsteps,
                   double dt, double t_final, double* U_aos, double* t_out, const char* dir) {
    char old[4096];
    if (!getcwd(old, sizeof old) || chdir(dir)) return 1;
    RefSW R;
    setup(&R, nx, ny, 0.0, 0.0, nx * h, ny * h, h, bc);
    R.ctx.isx = src[0]; R.ctx.isy = src[1]; R.ctx.irx = rec[0]; R.ctx.iry = rec[1];
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    solve(&R, stepper, nsteps, dt, t_final);
    memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
    if (t_out) *t_out = R.ts->t;
    teardown(&R);
    return chdir(old) ? 1 : 0;
}
#else
/* the program of hype.c at N x N cells: [-1,1]^2, adiabatic walls, CFL 0.5, dt = h CFL / 2,
 * RK104 to FinalTime 1.0, then ErrorNorms (post_process.c); U0/U1 (optional) receive the
 * initial and final states */
int ref_sw2d_program(int N, double* l2, double* linf, double* U0, double* U1) {
    RefSW R;
    const int bc[4] = {4, 4, 4, 4};
    const double h = (1.0 - -1.0) / (PetscReal)N;
    setup(&R, N, N, -1.0, -1.0, 1.0, 1.0, h, bc);
    R.ctx.CFL = 0.5;
    R.ctx.FinalTime = 1.0;
    const double dt = 0.5 * R.ctx.h * R.ctx.CFL / wave_speed;
    InitializeSolution(R.U, R.da, R.ctx);
    if (U0) memcpy(U0, R.U->a, sizeof(double) * (size_t)R.U->n);
    solve(&R, 1, 1 << 30, dt, 1.0);
    if (U1) memcpy(U1, R.U->a, sizeof(double) * (size_t)R.U->n);
    ErrorNorms(R.U, R.da, R.ctx, l2, linf, 1.0);
    teardown(&R);
    return 0;
}
#endif
