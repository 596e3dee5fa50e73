/*
 * ref_euler_driver.c -- TEST INFRASTRUCTURE: drives the reference's own
 * conservative 3D RHS, compiled unmodified through the PETSc shim, for the
 * "3D Euler + CWENO4 + Rusanov + SSPRK(4,3)" configuration.
 *
 * Assembled from reference files (all compiled in place from the reference
 * tree by oracle/Makefile):
 *   RHSFunction          3d/weno4/Navier-Stokes-3D/rhs_function.c:12-443
 *   PDEConsFlux, LLF     3d/weno4/Navier-Stokes-3D/pde.c:40-88,164-187
 *   weno()  (CWENO4)     3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259
 *   evaluate_polynomial  3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:12-21
 *   array.c              3d/weno4/Navier-Stokes-3D/array.c
 * The viscous Riemann solver is replaced at link time by ref_visc_zero()
 * (pure Euler: zero viscous flux, zero viscous wave speed), which turns the
 * Navier-Stokes RHS into the Euler RHS with dt = CFL*h/(3*s_max).
 * The driver mirrors 3d/weno4/Navier-Stokes-3D/hype.c:96-188 (DMDA with box
 * stencil width 3, scratch allocation, the initial RHS call that sets dt, the
 * SSP RKS3 4-stage TS) and the dt update of monitor_function.c:31.
 *
 * Built with -DREF_WENO3 against 3d/weno3/Euler (rhs_function.c:12-387,
 * reconstruction.c:12-177, pde.c:40-106, array.c; set-up of hype.c:96-196) it
 * drives the third-order WENO Euler program instead, which has no viscous terms
 * and no gradient traces; its entry points are then renamed by the Makefile.
 * Built with -DREF_NS3D it keeps the program's own viscous Riemann solver and its own
 * reconstruction.c: the whole Navier-Stokes RHS.
 */
#include "hype.h"
#include <setjmp.h>

#if !defined(REF_WENO3) && !defined(REF_NS3D)
/* Zero viscous flux: replaces PDEViscRiemannSolver (pde.c:386-404). */
PetscReal PDEViscRiemannSolver(const Field* QL, PetscReal grad_QL[nVar][DIM], const Field* QR, PetscReal grad_QR[nVar][DIM],
                               const PetscReal nx, const PetscReal ny, const PetscReal nz, Field* Flux) {
    (void)QL; (void)grad_QL; (void)QR; (void)grad_QR; (void)nx; (void)ny; (void)nz;
    for (int c = 0; c < nVar; ++c) Flux->comp[c] = 0.0;
    return 0.0;
}
#endif

/* bc codes shared with the GPU library: 0 periodic, 1 reflective, 2 transmissive */
static enum bndry_type map_bc(int b) {
    if (b == 1) return reflective;
    if (b == 2) return transmissive;
    return periodic;
}

typedef struct {
    AppCtx ctx;
    DM da;
    Vec U, RHS;
    TS ts;
    int dt_mode;
} RefEuler;

static void setup(RefEuler* R, int nx, int ny, int nz, double xmin, double ymin, double zmin, double h, double cfl, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->x_min = xmin; C->y_min = ymin; C->z_min = zmin;
    C->x_max = xmin + nx * h; C->y_max = ymin + ny * h; C->z_max = zmin + nz * h;
    C->N_x = nx; C->N_y = ny; C->N_z = nz;
    C->CFL = cfl;
    C->h = h;
    C->left_boundary = map_bc(bc[0]); C->right_boundary = map_bc(bc[1]);
    C->bottom_boundary = map_bc(bc[2]); C->top_boundary = map_bc(bc[3]);
    C->back_boundary = map_bc(bc[4]); C->front_boundary = map_bc(bc[5]);
    DMBoundaryType bx = (C->left_boundary == periodic || C->right_boundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType by = (C->bottom_boundary == periodic || C->top_boundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType bz = (C->front_boundary == periodic || C->back_boundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMDACreate3d(PETSC_COMM_WORLD, bx, by, bz, DMDA_STENCIL_BOX, nx, ny, nz, PETSC_DECIDE, PETSC_DECIDE, PETSC_DECIDE, nVar, 3,
                 NULL, NULL, NULL, &R->da);
    DMSetUp(R->da);
    DMCreateGlobalVector(R->da, &R->U);
    VecDuplicate(R->U, &R->RHS);
    PetscInt xs, ys, zs, xm, ym, zm;
    DMDAGetCorners(R->da, &xs, &ys, &zs, &xm, &ym, &zm);
    C->u_bnd = allocate6d(zm + 2, ym + 2, xm + 2, nVar, 6, N_gp2d);
#ifndef REF_WENO3
    C->u_bnd_grad = allocate7d(zm + 2, ym + 2, xm + 2, nVar, 6, N_gp2d, DIM);
#endif
    C->F = allocate4d(zm, ym, xm + 1, nVar);
    C->G = allocate4d(zm, ym + 1, xm, nVar);
    C->H = allocate4d(zm + 1, ym, xm, nVar);
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefEuler* R) {
    free6d(R->ctx.u_bnd);
#ifndef REF_WENO3
    free7d(R->ctx.u_bnd_grad);
#endif
    free4d(R->ctx.F); free4d(R->ctx.G); free4d(R->ctx.H);
    VecDestroy(&R->ctx.localU);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

static PetscErrorCode monitor(TS ts, PetscInt step, PetscReal time, Vec U, void* ctx) {
    (void)step; (void)time; (void)U;
    RefEuler* R = (RefEuler*)ctx;
    if (R->dt_mode == 0) TSSetTimeStep(ts, R->ctx.dt); /* monitor_function.c:31 */
    return 0;
}

/* One RHS evaluation on an AoS [k][j][i][c] state. Returns 0, or 2 when the
 * reference aborted on an inadmissible state. */
int ref_euler_rhs(int nx, int ny, int nz, double xmin, double ymin, double zmin, double h, double cfl, const int* bc,
                  const double* U_aos, double* RHS_aos, double* dt_out) {
    RefEuler R;
    setup(&R, nx, ny, nz, xmin, ymin, zmin, h, cfl, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    jmp_buf jb;
    int rc = 0;
    if (setjmp(jb) == 0) {
        shim_set_abort_jump(&jb);
        RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
        memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
        if (dt_out) *dt_out = R.ctx.dt;
    } else {
        rc = 2;
    }
    shim_set_abort_jump(NULL);
    teardown(&R);
    return rc;
}

/* nsteps of SSP RKS3/4 stages from U (in place), reproducing hype.c's set-up:
 * the initial RHS call fixes the first dt; dt_mode 0 then refreshes dt at the
 * start of every step from the last RHS evaluation (Navier-Stokes-3D monitor),
 * dt_mode 1 keeps the first dt (3d/weno3/Euler has the monitor disabled),
 * dt_mode 2 uses *dt_inout for every step. */
int ref_euler_run(int nx, int ny, int nz, double xmin, double ymin, double zmin, double h, double cfl, const int* bc,
                  int nsteps, int dt_mode, double* U_aos, double* t_out, double* dt_inout) {
    RefEuler R;
    setup(&R, nx, ny, nz, xmin, ymin, zmin, h, cfl, bc);
    R.dt_mode = dt_mode;
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    jmp_buf jb;
    int rc = 0;
    if (setjmp(jb) == 0) {
        shim_set_abort_jump(&jb);
        RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
        TSSetRHSFunction(R.ts, NULL, RHSFunction, &R.ctx);
        TSSetStepNumber(R.ts, 0);
        TSSetTime(R.ts, 0.0);
        if (dt_mode == 2) {
            R.dt_mode = 1;
            TSSetTimeStep(R.ts, *dt_inout);
        } else {
            TSSetTimeStep(R.ts, R.ctx.dt);
        }
        TSMonitorSet(R.ts, monitor, &R, NULL);
        TSSetMaxTime(R.ts, 1e300);
        TSSetMaxSteps(R.ts, nsteps);
        TSSetExactFinalTime(R.ts, TS_EXACTFINALTIME_MATCHSTEP);
        TSSetType(R.ts, TSSSP);
        TSSSPSetType(R.ts, TSSSPRKS3);
        TSSSPSetNumStages(R.ts, 4);
        TSSolve(R.ts, R.U);
        memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
        if (t_out) *t_out = R.ts->t;
        if (dt_inout) *dt_inout = R.ts->dt;
    } else {
        rc = 2;
    }
    shim_set_abort_jump(NULL);
    teardown(&R);
    return rc;
}
