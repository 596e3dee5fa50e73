/*
 * ref_bubble_driver.c -- TEST INFRASTRUCTURE: drives the reference's 2D
 * diffuse-interface RHS (2d/weno4/bubble/rhs_function.c, reconstruction.c,
 * pde.c, post_process.c, array.c, compiled unmodified through the PETSc shim).
 * Mirrors 2d/weno4/bubble/hype.c:80-210: DMDA with box stencil width 3,
 * primitive vector W, scratch u_bnd/F/G, basis tables phiFace/phiNode, the
 * initial RHS call that fixes dt, TSSSP RK104 and the monitor's dt update.
 * The reference's EOS constants (g1 = 4.4, p1 = 6000, g2 = 1.4, p2 = 0) are
 * compiled into its pde.c.
 */
#include "hype.h"
#include <setjmp.h>

void bubble_collapse(PetscReal, PetscReal, PetscReal*);
void InitialCondition(PetscReal x, PetscReal y, PetscReal* Q0) { bubble_collapse(x, y, Q0); }

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
} RefBub;

static void setup(RefBub* R, int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->x_min = xmin; C->y_min = ymin;
    C->x_max = xmin + nx * h; C->y_max = ymin + ny * h;
    C->N_x = nx; C->N_y = ny;
    C->CFL = cfl;
    C->h = h;
    C->left_boundary = map_bc(bc[0]); C->right_boundary = map_bc(bc[1]);
    C->bottom_boundary = map_bc(bc[2]); C->top_boundary = map_bc(bc[3]);
    DMBoundaryType bx = (C->left_boundary == periodic || C->right_boundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType by = (C->bottom_boundary == periodic || C->top_boundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMDACreate2d(PETSC_COMM_WORLD, bx, by, DMDA_STENCIL_BOX, nx, ny, PETSC_DECIDE, PETSC_DECIDE, nVar, 3, NULL, NULL, &R->da);
    DMSetUp(R->da);
    DMCreateGlobalVector(R->da, &R->U);
    VecDuplicate(R->U, &C->W);
    VecDuplicate(R->U, &R->RHS);
    PetscInt xs, ys, xm, ym;
    DMDAGetCorners(R->da, &xs, &ys, NULL, &xm, &ym, NULL);
    C->u_bnd = allocate5d(ym + 2, xm + 2, nVar, 4, N_gp2);
    C->F = allocate3d(ym, xm + 1, nVar + 1);
    C->G = allocate3d(ym + 1, xm, nVar + 1);
    C->phiFace = allocate3d(4, N_gp2, nDOF);
    C->phiNode = allocate2d(N_node, nDOF);
    for (int q = 0; q < N_gp2; ++q)
        for (int k = 0; k < nDOF; ++k) {
            set_element_3d(C->phiFace, 0, q, k, basis(-0.5, x_gp2[q], k));
            set_element_3d(C->phiFace, 1, q, k, basis(0.5, x_gp2[q], k));
            set_element_3d(C->phiFace, 2, q, k, basis(x_gp2[q], -0.5, k));
            set_element_3d(C->phiFace, 3, q, k, basis(x_gp2[q], 0.5, k));
        }
    for (int q = 0; q < N_node; ++q)
        for (int k = 0; k < nDOF; ++k) set_element_2d(C->phiNode, q, k, basis(x_node[q], y_node[q], k));
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefBub* R) {
    free5d(R->ctx.u_bnd);
    free3d(R->ctx.F); free3d(R->ctx.G); free3d(R->ctx.phiFace); free2d(R->ctx.phiNode);
    VecDestroy(&R->ctx.localU); VecDestroy(&R->ctx.W);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

static PetscErrorCode monitor(TS ts, PetscInt step, PetscReal time, Vec U, void* ctx) {
    (void)step; (void)time; (void)U;
    RefBub* R = (RefBub*)ctx;
    if (R->dt_mode == 0) TSSetTimeStep(ts, R->ctx.dt); /* post_process.c:19 */
    return 0;
}

int ref_bubble_rhs(int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc, const double* U_aos,
                   double* RHS_aos, double* dt_out) {
    RefBub R;
    setup(&R, nx, ny, xmin, ymin, h, cfl, bc);
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

/* nsteps of TSSSP RK104 (hype.c:209-210) with the monitor's dt update */
int ref_bubble_run(int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc, int nsteps, double* U_aos,
                   double* t_out, double* dt_out) {
    RefBub R;
    setup(&R, nx, ny, xmin, ymin, h, cfl, bc);
    R.dt_mode = 0;
    memcpy(R.U->a, U_aos, sizeof(double) * (size_t)R.U->n);
    jmp_buf jb;
    int rc = 0;
    if (setjmp(jb) == 0) {
        shim_set_abort_jump(&jb);
        RHSFunction(R.ts, 0.0, R.U, R.RHS, &R.ctx);
        TSSetRHSFunction(R.ts, NULL, RHSFunction, &R.ctx);
        TSSetStepNumber(R.ts, 0);
        TSSetTime(R.ts, 0.0);
        TSSetTimeStep(R.ts, R.ctx.dt);
        TSMonitorSet(R.ts, monitor, &R, NULL);
        TSSetMaxTime(R.ts, 1e300);
        TSSetMaxSteps(R.ts, nsteps);
        TSSetExactFinalTime(R.ts, TS_EXACTFINALTIME_MATCHSTEP);
        TSSetType(R.ts, TSSSP);
        TSSSPSetType(R.ts, TSSSPRK104);
        TSSolve(R.ts, R.U);
        memcpy(U_aos, R.U->a, sizeof(double) * (size_t)R.U->n);
        if (t_out) *t_out = R.ts->t;
        if (dt_out) *dt_out = R.ts->dt;
    } else {
        rc = 2;
    }
    shim_set_abort_jump(NULL);
    teardown(&R);
    return rc;
}
