/*
 * ref_hype2d_driver.c -- TEST INFRASTRUCTURE: drives the reference's own 2D
 * path-conservative RHS of 2d/HyPE-2D (rhs_function.c, reconstruction.c, riemann.c,
 * kapila_5eqn.c, array.c compiled unmodified through the PETSc shim) with the Kapila
 * five-equation model (-DKAPILA_5EQN; the model's own hype.h also keeps its
 * DIFFUSE_INTERFACE define, which only adds a second momentum reflection at reflective
 * walls, so the fixtures use transmissive and periodic boundaries).  The set-up mirrors
 * 2d/HyPE-2D/hype.c:30-340: order N, quadrature and admissibility nodes, the basis
 * tables, the trace / flux / fluctuation scratch, the initial RHS call that sets dt and
 * the SSP stepper chosen by N (Euler, RKS2/2, RKS3/4, RK104) with the dt kept (the
 * program's monitor leaves TSSetTimeStep commented out, post_process.c:19).
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
} RefH2;

static void setup(RefH2* R, int N, int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc) {
    AppCtx* C = &R->ctx;
    memset(C, 0, sizeof(*C));
    C->N = N;
    C->x_min = xmin; C->y_min = ymin;
    C->x_max = xmin + nx * h; C->y_max = ymin + ny * h;
    C->N_x = nx; C->N_y = ny;
    C->CFL = cfl;
    C->h = h;
    C->LeftBoundary = map_bc(bc[0]); C->RightBoundary = map_bc(bc[1]);
    C->BottomBoundary = map_bc(bc[2]); C->TopBoundary = map_bc(bc[3]);
    C->nDOF = (C->N + 1) * (C->N + 2) / 2;
    if (C->N < 2) { C->Ngp_Face = 1; C->Ngp_Vol = 1; }
    else { C->Ngp_Face = 2; C->Ngp_Vol = 4; }
    C->N_node = 4 * C->Ngp_Face;
    C->xGP_Face = malloc(sizeof(double) * C->Ngp_Face); C->wGP_Face = malloc(sizeof(double) * C->Ngp_Face);
    C->xGP_Vol = malloc(sizeof(double) * C->Ngp_Vol); C->yGP_Vol = malloc(sizeof(double) * C->Ngp_Vol);
    C->wGP_Vol = malloc(sizeof(double) * C->Ngp_Vol);
    C->x_node = malloc(sizeof(double) * C->N_node); C->y_node = malloc(sizeof(double) * C->N_node);
    if (C->N < 2) {
        C->xGP_Face[0] = 0.0; C->wGP_Face[0] = 1.0;
        C->xGP_Vol[0] = 0.0; C->yGP_Vol[0] = 0.0; C->wGP_Vol[0] = 1.0;
        C->x_node[0] = 0.5; C->y_node[0] = 0.0; C->x_node[1] = -0.5; C->y_node[1] = 0.0;
        C->x_node[2] = 0.0; C->y_node[2] = 0.5; C->x_node[3] = 0.0; C->y_node[3] = -0.5;
    } else {
        const double g = 0.28867513459481287;
        C->xGP_Face[0] = -g; C->wGP_Face[0] = 0.5; C->xGP_Face[1] = g; C->wGP_Face[1] = 0.5;
        C->xGP_Vol[0] = -g; C->yGP_Vol[0] = -g; C->wGP_Vol[0] = 0.25;
        C->xGP_Vol[1] = -g; C->yGP_Vol[1] = g; C->wGP_Vol[1] = 0.25;
        C->xGP_Vol[2] = g; C->yGP_Vol[2] = -g; C->wGP_Vol[2] = 0.25;
        C->xGP_Vol[3] = g; C->yGP_Vol[3] = g; C->wGP_Vol[3] = 0.25;
        C->x_node[0] = 0.5; C->y_node[0] = -g; C->x_node[1] = 0.5; C->y_node[1] = g;
        C->x_node[2] = -0.5; C->y_node[2] = -g; C->x_node[3] = -0.5; C->y_node[3] = g;
        C->x_node[4] = -g; C->y_node[4] = 0.5; C->x_node[5] = g; C->y_node[5] = 0.5;
        C->x_node[6] = -g; C->y_node[6] = -0.5; C->x_node[7] = g; C->y_node[7] = -0.5;
    }
    DMBoundaryType bx = (C->LeftBoundary == periodic || C->RightBoundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMBoundaryType by = (C->BottomBoundary == periodic || C->TopBoundary == periodic) ? DM_BOUNDARY_PERIODIC : DM_BOUNDARY_GHOSTED;
    DMDACreate2d(PETSC_COMM_WORLD, bx, by, DMDA_STENCIL_BOX, nx, ny, PETSC_DECIDE, PETSC_DECIDE, nVar, 3, NULL, NULL, &R->da);
    DMSetUp(R->da);
    DMCreateGlobalVector(R->da, &R->U);
    VecDuplicate(R->U, &R->RHS);
    PetscInt xs, ys, xm, ym, q, k;
    PetscReal value, gx, gy;
    DMDAGetCorners(R->da, &xs, &ys, NULL, &xm, &ym, NULL);
    C->u_bnd = allocate5d(ym + 2, xm + 2, nVar, 4, C->Ngp_Face);
    C->F = allocate3d(ym, xm + 1, nVar); C->G = allocate3d(ym + 1, xm, nVar);
    C->D = allocate3d(ym, xm + 1, nVar); C->E = allocate3d(ym + 1, xm, nVar);
    C->phiFace = allocate3d(4, C->Ngp_Face, C->nDOF);
    C->phiNode = allocate2d(C->N_node, C->nDOF);
    C->phiVol = allocate2d(C->Ngp_Vol, C->nDOF);
    C->gradphiVol_x = allocate2d(C->Ngp_Vol, C->nDOF); C->gradphiVol_y = allocate2d(C->Ngp_Vol, C->nDOF);
    C->gradphiFace_x = allocate3d(4, C->Ngp_Face, C->nDOF); C->gradphiFace_y = allocate3d(4, C->Ngp_Face, C->nDOF);
    for (q = 0; q < C->Ngp_Face; ++q)
        for (k = 0; k < C->nDOF; ++k) {
            const double xf[4] = {-0.5, 0.5, C->xGP_Face[q], C->xGP_Face[q]};
            const double yf[4] = {C->xGP_Face[q], C->xGP_Face[q], -0.5, 0.5};
            for (int f = 0; f < 4; ++f) {
                value = basis(xf[f], yf[f], k);
                basis_grad(xf[f], yf[f], k, &gx, &gy);
                set_element_3d(C->phiFace, f, q, k, value);
                set_element_3d(C->gradphiFace_x, f, q, k, gx);
                set_element_3d(C->gradphiFace_y, f, q, k, gy);
            }
        }
    for (q = 0; q < C->N_node; ++q)
        for (k = 0; k < C->nDOF; ++k) set_element_2d(C->phiNode, q, k, basis(C->x_node[q], C->y_node[q], k));
    for (q = 0; q < C->Ngp_Vol; ++q)
        for (k = 0; k < C->nDOF; ++k) {
            set_element_2d(C->phiVol, q, k, basis(C->xGP_Vol[q], C->yGP_Vol[q], k));
            basis_grad(C->xGP_Vol[q], C->yGP_Vol[q], k, &gx, &gy);
            set_element_2d(C->gradphiVol_x, q, k, gx);
            set_element_2d(C->gradphiVol_y, q, k, gy);
        }
    DMCreateLocalVector(R->da, &C->localU);
    TSCreate(PETSC_COMM_SELF, &R->ts);
    TSSetDM(R->ts, R->da);
}

static void teardown(RefH2* R) {
    AppCtx* C = &R->ctx;
    free5d(C->u_bnd);
    free3d(C->F); free3d(C->G); free3d(C->D); free3d(C->E);
    free3d(C->phiFace); free2d(C->phiNode); free2d(C->phiVol); free2d(C->gradphiVol_x); free2d(C->gradphiVol_y);
    free3d(C->gradphiFace_x); free3d(C->gradphiFace_y);
    free(C->xGP_Face); free(C->wGP_Face); free(C->xGP_Vol); free(C->yGP_Vol); free(C->wGP_Vol); free(C->x_node);
    free(C->y_node);
    VecDestroy(&C->localU);
    VecDestroy(&R->U); VecDestroy(&R->RHS);
    TSDestroy(&R->ts);
    DMDestroy(&R->da);
}

/* one RHS evaluation on an AoS [j][i][6] state; 0, or 2 when the program aborted */
int ref_hype2d_rhs(int N, int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc,
                   const double* U_aos, double* RHS_aos, double* dt_out) {
    RefH2 R;
    setup(&R, N, nx, ny, xmin, ymin, h, cfl, bc);
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

/* nsteps with the program's stepper for N and the dt of the initial RHS call */
int ref_hype2d_run(int N, int nx, int ny, double xmin, double ymin, double h, double cfl, const int* bc, int nsteps,
                   double* U_aos, double* t_out, double* dt_out) {
    RefH2 R;
    setup(&R, N, nx, ny, xmin, ymin, h, cfl, bc);
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
        TSSetMaxTime(R.ts, 1e300);
        TSSetMaxSteps(R.ts, nsteps);
        TSSetExactFinalTime(R.ts, TS_EXACTFINALTIME_MATCHSTEP);
        if (N == 0) {
            TSSetType(R.ts, TSEULER);
        } else {
            TSSetType(R.ts, TSSSP);
            if (N == 1) { TSSSPSetType(R.ts, TSSSPRKS2); TSSSPSetNumStages(R.ts, 2); }
            else if (N == 2) { TSSSPSetType(R.ts, TSSSPRKS3); TSSSPSetNumStages(R.ts, 4); }
            else TSSSPSetType(R.ts, TSSSPRK104);
        }
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
