/*
 * ref_ctcs2d_tu.c -- TEST INFRASTRUCTURE: compiles the reference's
 * 2d/ctcs/plane_wave/wave.c in place (its main() renamed) and exposes its
 * CTCS() update (wave.c:161-203) on a caller-chosen grid and boundary type.
 * The reference's own program is periodic; the zero-Dirichlet variant uses a
 * DM_BOUNDARY_GHOSTED grid whose exterior ghosts stay zero
 * (the pattern of 1d/ctcs/source/source.c:83).
 */
#define main ref_plane_wave_main
#include "2d/ctcs/plane_wave/wave.c"
#undef main

/* nsteps leapfrog updates; p_old/p are [ny][nx]; on return p_old/p hold the
 * last two levels (p = newest). zero_bc: 1 -> ghosted zero exterior, 0 -> periodic. */
int ref_ctcs2d_run(int nx, int ny, double h, double c0, double dt, int zero_bc, int nsteps, double* p_old, double* p) {
    DM da;
    DMBoundaryType b = zero_bc ? DM_BOUNDARY_GHOSTED : DM_BOUNDARY_PERIODIC;
    DMDACreate2d(PETSC_COMM_WORLD, b, b, DMDA_STENCIL_STAR, nx, ny, PETSC_DECIDE, PETSC_DECIDE, 1, 1, NULL, NULL, &da);
    DMSetUp(da);
    Vec Pold, Pcurr, Pnew;
    DMCreateGlobalVector(da, &Pold);
    VecDuplicate(Pold, &Pcurr);
    VecDuplicate(Pold, &Pnew);
    memcpy(Pold->a, p_old, sizeof(double) * (size_t)nx * ny);
    memcpy(Pcurr->a, p, sizeof(double) * (size_t)nx * ny);
    AppCtx user;
    memset(&user, 0, sizeof(user));
    user.Nx = nx; user.Ny = ny; user.h = h; user.c0 = c0; user.dt = dt;
    int rc = 0;
    for (int s = 0; s < nsteps && !rc; ++s) {
        rc = CTCS(da, Pold, Pcurr, Pnew, &user);
        VecCopy(Pcurr, Pold); /* wave.c:87-88 */
        VecCopy(Pnew, Pcurr);
    }
    memcpy(p_old, Pold->a, sizeof(double) * (size_t)nx * ny);
    memcpy(p, Pcurr->a, sizeof(double) * (size_t)nx * ny);
    VecDestroy(&Pold); VecDestroy(&Pcurr); VecDestroy(&Pnew);
    DMDestroy(&da);
    return rc;
}
