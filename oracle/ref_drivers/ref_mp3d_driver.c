/*
 * ref_mp3d_driver.c -- TEST INFRASTRUCTURE: drives the reference's own 3D
 * primitive-variable multiphase RHS, RHSFunctionPrimitive of
 * 3d/weno4/Viscous-Multiphase-Fourth-Order (rhs_function.c, pde.c, reconstruction.c,
 * array.c compiled unmodified through the PETSc shim, with zero-initialised automatic
 * variables: the program's viscous gradients are never written, see oracle/Makefile).
 * The set-up mirrors that program's hype.c:96-160: a dof-6 DMDA with box stencil width
 * 3, the trace / gradient / flux scratch with 7 flux components, the initial RHS call
 * that sets dt, SSP RKS3 with 4 stages and the dt update of monitor_function.c:19.
 */
#include "hype.h"
#include <setjmp.h>

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
} RefMp3d;

static void setup(RefMp3d* R, int nx, int ny, int nz, double h, double cfl, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->x_max = nx * h; C->y_max = ny * h; C->z_max = nz * h;
    C->N_x = nx; C->N_y = ny; C->N_z = nz;
    C->CFL = cfl;
    C->h = h;
    C->ReconsPrimitive = PETSC_TRUE;
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
    C->u_bnd_grad = allocate7d(zm + 2, ym + 2, xm + 2, nVar, 6, N_gp2d, DIM);
    C->F = allocate4d(zm, ym, xm + 1, nVar + 1);
    C->G = allocate4d(zm, ym + 1, xm, nVar + 1);
    C->H = allocate4d(zm + 1, ym, xm, nVar + 1);
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefMp3d* R) {
    free6d(R->ctx.u_bnd);
    free7d(R->ctx.u_bnd_grad);
    free4d(R->ctx.F); free4d(R->ctx.G); free4d(R->ctx.H);
    VecDestroy(&R->ctx.localU);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

static PetscErrorCode monitor(TS ts, PetscInt step, PetscReal time, Vec U, void* ctx) {
    (void)step; (void)time; (void)U;
    RefMp3d* R = (RefMp3d*)ctx;
    if (R->dt_mode == 0) TSSetTimeStep(ts, R->ctx.dt); /* monitor_function.c:19 */
    return 0;
}

/* one RHS evaluation on an AoS [k][j][i][6] state; 0, or 2 when the program aborted */
int ref_mp3d_rhs(int nx, int ny, int nz, double h, double cfl, const int* bc, const double* U_aos, double* RHS_aos,
                 double* dt_out) {
    RefMp3d R;
    setup(&R, nx, ny, nz, h, cfl, bc);
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    jmp_buf jb;
    int rc = 0;
    if (setjmp(jb) == 0) {
        shim_set_abort_jump(&jb);
        RHSFunctionPrimitive(R.ts, 0.0, R.U, R.RHS, &R.ctx);
        memcpy(RHS_aos, R.RHS->a, sizeof(double) * (size_t)R.U->n);
        if (dt_out) *dt_out = R.ctx.dt;
    } else {
        rc = 2;
    }
    shim_set_abort_jump(NULL);
    teardown(&R);
    return rc;
}

/* nsteps of SSP RKS3/4 stages, the initial RHS call fixing the first dt; dt_mode 0
 * refreshes dt every step from the last RHS call (the program's monitor) */
int ref_mp3d_run(int nx, int ny, int nz, double h, double cfl, const int* bc, int nsteps, int dt_mode, double* U_aos,
                 double* t_out, double* dt_out) {
    RefMp3d R;
    setup(&R, nx, ny, nz, h, cfl, bc);
    R.dt_mode = dt_mode;
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    jmp_buf jb;
    int rc = 0;
    if (setjmp(jb) == 0) {
        shim_set_abort_jump(&jb);
        RHSFunctionPrimitive(R.ts, 0.0, R.U, R.RHS, &R.ctx);
        TSSetRHSFunction(R.ts, NULL, RHSFunctionPrimitive, &R.ctx);
        TSSetStepNumber(R.ts, 0);
        TSSetTime(R.ts, 0.0);
        TSSetTimeStep(R.ts, R.ctx.dt);
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
        if (dt_out) *dt_out = R.ctx.dt;
    } else {
        rc = 2;
    }
    shim_set_abort_jump(NULL);
    teardown(&R);
    return rc;
}
