/*
 * hype_gpu.h -- C ABI of the GB300 (sm_103a) implementation of HyPE's
 * finite-volume right-hand side, its SSP Runge-Kutta stepper and the CTCS
 * leapfrog acoustic update.
 *
 * Plain C types only (no CUDA or torch types), so that the reference's PETSc
 * host code can call it from a thin RHSFunction.  Every entry point returns an
 * int status (HYPE_OK = 0) instead of aborting: the reference calls MPI_Abort on
 * an inadmissible state (3d/weno4/Navier-Stokes-3D/pde.c:56-66); here the call
 * returns HYPE_ERR_STATE and reports the first offending cell.
 *
 * State layout at the boundary is the reference's DMDA layout: AoS doubles
 * [k][j][i][c], x fastest, owned box only (the ghost/boundary fill that
 * DMGlobalToLocal + the BC sweeps do in the reference happens on the device).
 * Entry points named *_device take device pointers in the library's SoA
 * layout [c][k][j][i]; all others take host pointers.
 *
 * Threading: one CUDA stream per context; calls on one context are serialised
 * by the caller (the reference also runs one RHS at a time per AppCtx).
 */
#ifndef HYPE_GPU_H
#define HYPE_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define HYPE_OK 0
#define HYPE_ERR_ARG 1         /* bad argument (sizes, codes, null pointers) */
#define HYPE_ERR_STATE 2       /* inadmissible state: rho < 1e-14 or p < 1e-12 at a face Gauss point */
#define HYPE_ERR_CUDA 3        /* CUDA runtime error (message via hype_last_error) */
#define HYPE_ERR_NOMEM 4       /* device allocation failed */
#define HYPE_ERR_UNSUPPORTED 5 /* option combination not implemented */

/* ------------------------------------------------------------ boundary codes
 * per face: [0]=left(-x) [1]=right(+x) [2]=bottom(-y) [3]=top(+y) [4]=back(-z) [5]=front(+z)
 * (enum bndry_type in 3d/weno4/Navier-Stokes-3D/hype.h:124; ZERO is the
 * DM_BOUNDARY_GHOSTED zero exterior of the CTCS codes, 1d/ctcs/source/source.c:83) */
#define HYPE_BC_PERIODIC 0
#define HYPE_BC_REFLECTIVE 1
#define HYPE_BC_TRANSMISSIVE 2
#define HYPE_BC_ZERO 3
#define HYPE_BC_ADIABATIC 4 /* acoustic wall: the ghost value is the negated mirror value (3d/weno4/plane_wave) */

/* reconstruction */
#define HYPE_RECON_CWENO4 0  /* nonlinear CWENO4, gammaHi=gammaLo=0.85
                                (3d/weno4/Viscous-Multiphase-Fourth-Order/reconstruction.c:38-259) */
#define HYPE_RECON_LINEAR4 1 /* the optimal-weight limit: the 4th-order central polynomial R4 */
#define HYPE_RECON_LEARNED 2 /* no counterpart in the reference: a small network (hype_euler_set_mlp) scores
                                each cell from its normalised 5-point stencils; flagged or low-confidence
                                cells take CWENO4, the others R4, and any cell whose R4 face traces break
                                density/pressure positivity is redone with CWENO4 */
#define HYPE_RECON_WENO3 3   /* third-order WENO: per-direction 3-stencil WENO with central weight 100 and
                                4-stencil WENO cross terms, 10 coefficients
                                (3d/weno3/Euler/reconstruction.c:29-177) */

/* numerical flux across each face Gauss point (3d/weno4/Navier-Stokes-3D/pde.c) */
#define HYPE_FLUX_RUSANOV 0  /* PDELLFRiemannSolver, pde.c:164-187 */
#define HYPE_FLUX_HLLC 1     /* PDEHLLCRiemannSolver, pde.c:207-322 */
#define HYPE_FLUX_ROTHLLC 2  /* PDErotHLLCRiemannSolver, pde.c:324-384 */

/* arithmetic of reconstruction + flux (the state and the RK accumulation are always FP64) */
#define HYPE_PREC_FP64 0
#define HYPE_PREC_FP32 1
/* 3D Euler (CWENO4 / R4): state, flux and stage accumulation in FP64, reconstruction in
 * double-float arithmetic (pairs of FP32 numbers, 48-bit significand, on the FP32 pipe,
 * which issues 64x the FP64 rate on GB300) on deviations from a per-variable reference
 * value; traces rounded once in FP64 */
#define HYPE_PREC_DF64 2

/* dt semantics */
#define HYPE_DT_MONITOR 0 /* dt of step n+1 = CFL h / (3 s_max) of the last stage RHS of step n
                             (3d/weno4/Navier-Stokes-3D/monitor_function.c:31) */
#define HYPE_DT_FROZEN 1  /* dt fixed by the first RHS evaluation (3d/weno3/Euler/hype.c:188) */
#define HYPE_DT_FIXED 2   /* caller's dt */

/* ============================================================ 3D Euler */
typedef struct hype_euler hype_euler;

typedef struct {
    int nx, ny, nz;                /* cells (DMDACreate3d M,N,P) */
    double x_min, y_min, z_min, h; /* uniform spacing (AppCtx.h) */
    double cfl;                    /* AppCtx.CFL */
    double gamma;                  /* ideal-gas ratio (GAMMA, hype.h:39) */
    int bc[6];                     /* HYPE_BC_* per face; PERIODIC must be paired */
    int recon;                     /* HYPE_RECON_* */
    int precision;                 /* HYPE_PREC_* */
    int dt_mode;                   /* HYPE_DT_* */
    int flux;                      /* HYPE_FLUX_* (0 = Rusanov) */
    int positivity;                /* 0: an inadmissible face trace is an error (the reference aborts,
                                      pde.c:56-66); 1: the cell drops to first order, the fallback of
                                      3d/weno4/Viscous-Multiphase-Fourth-Order/rhs_function.c:297-305, checked
                                      at the 24 face Gauss-point traces the flux uses; counted in
                                      hype_euler_indicator_stats */
    /* Navier-Stokes terms (3d/weno4/Navier-Stokes-3D/pde.c:90-162, PDEViscFlux): mu = 0 is the Euler
     * system; mu > 0 adds at every face Gauss point the average of both sides' viscous fluxes, built
     * from the gradients of the cells' R4 polynomials, and the viscous speed enters dt as
     * (1/3) CFL h / (s_max + 2 s_visc / h) (Navier-Stokes-3D/rhs_function.c:438).  FP64 only, not
     * with HYPE_RECON_LEARNED nor hype_euler_rhs_noalloc. */
    double mu;      /* dynamic viscosity (MU_0 = 0.01, Navier-Stokes-3D/hype.h:41) */
    double prandtl; /* Prandtl number (PR = 1.0, hype.h:40); conductivity k = cv mu gamma / prandtl */
    double cv;      /* specific heat at constant volume (C_V = 2.5, hype.h:38) */
} hype_euler_params;

typedef struct {
    long long bad_cell; /* first offending linear cell index (k*ny+j)*nx+i, -1 if none */
    double smax;        /* max wave speed seen by the last RHS evaluation */
    long long rhs_evals;
} hype_status;

/* Create a solver context and its device buffers. */
int hype_euler_create(const hype_euler_params* p, hype_euler** out);
void hype_euler_destroy(hype_euler* e);
/* the parameters the context was created with (recon reflects hype_euler_set_recon) */
int hype_euler_get_params(const hype_euler* e, hype_euler_params* out);

/* Drop-in for RHSFunction(TS ts, PetscReal t, Vec U, Vec RHS, void* ctx)
 * (3d/weno3/Euler/hype.h:291 declaration; body 3d/weno4/Navier-Stokes-3D/rhs_function.c:12-443):
 * U_aos, RHS_aos are host arrays of the DMDA global vectors (VecGetArrayRead / VecGetArray);
 * *dt_out receives the value the reference stores in Ctx->dt (rhs_function.c:438-440). */
int hype_euler_rhs(hype_euler* e, double t, const double* U_aos, double* RHS_aos, double* dt_out);

/* Same on device buffers in SoA layout [5][nz][ny][nx]; dt_out may be NULL. */
int hype_euler_rhs_device(hype_euler* e, double t, const double* dU, double* dRHS, double* dt_out);

/* Resident state: host AoS <-> device. */
int hype_euler_upload(hype_euler* e, const double* U_aos);
int hype_euler_download(hype_euler* e, double* U_aos);
/* Device pointer to the resident SoA state (5*nx*ny*nz doubles). */
double* hype_euler_state_device(hype_euler* e);

/* nsteps of SSPRK(4,3) on the resident state -- replaces TSSolve with
 * TSSSP/TSSSPRKS3/4 stages (3d/weno4/Navier-Stokes-3D/hype.c:185-188).  The
 * whole step (4 fused stages, device-side dt) runs without host round trips;
 * with nsteps > 2 the steps after the first replay one CUDA graph of the step,
 * captured on first use and again after a reconstruction, flux, precision,
 * positivity, indicator or dt-mode change (not while hype_euler_profile is on).
 * *t_inout advances by the dts used; *dt_inout is the dt the next step will use
 * (input for HYPE_DT_FIXED; for the other modes pass the value of a previous
 * call, or <= 0 to start from the RHS of the current state as hype.c does). */
int hype_euler_step(hype_euler* e, int nsteps, double* t_inout, double* dt_inout, hype_status* st);

/* Block until all work of the context is done. */
int hype_euler_sync(hype_euler* e);

/* The context's CUDA stream (a cudaStream_t), for callers that record their own
 * events or order their own work after the solver's. */
void* hype_euler_stream(hype_euler* e);

/* The monitor's diagnostics of the resident state (computed on the device, summed in a
 * fixed order): *ke = KineticEnergy, sum of h^3 |rho u|^2 / (2 rho)
 * (3d/weno4/Navier-Stokes-3D/kinetic_energy.c:11-44), *dissipation = Dissipation, the sum
 * of tau : grad v with central velocity differences and viscosity params.mu
 * (dissipation.c:11-67; neighbours across a non-periodic face are the context's ghost
 * values of this state). */
int hype_euler_monitor(hype_euler* e, double* ke, double* dissipation);

/* Per-kernel timing: while enabled, every kernel the context launches is
 * bracketed by CUDA events on its stream; read returns the summed milliseconds
 * and launch counts of [0] ghost fill + reconstruction (fused stage: ghost fill,
 * and the indicator gate's scoring pass when the gate is on), [1] face fluxes (3
 * directions) or, for the fused stage, the fused stage kernel, [2] divergence +
 * stage update (fused stage: only the combination of a first stage whose dt
 * comes from its own RHS) since the last enable. */
int hype_euler_profile(hype_euler* e, int enable);
int hype_euler_profile_read(hype_euler* e, double* ms, long long* count);

/* Stage kernels.  HYPE_STAGE_AUTO (the default) runs the FP32 reconstruction +
 * Rusanov form (CWENO4, R4 or WENO3, inviscid) as one fused kernel per RK stage
 * after the device ghost fill: face traces stay in shared memory, there is no
 * trace or face-flux buffer, and the results are bit-identical to the unfused
 * kernels.  Every other form, and HYPE_STAGE_UNFUSED, runs ghost fill,
 * reconstruction into a face-trace buffer, three face-flux kernels and the
 * update.  No counterpart in the reference (its RHSFunction is one CPU pass,
 * 3d/weno4/Navier-Stokes-3D/rhs_function.c:183-433). */
#define HYPE_STAGE_AUTO 0
#define HYPE_STAGE_UNFUSED 1
int hype_euler_set_stage_kernel(hype_euler* e, int mode);

/* ---- learned troubled-cell indicator (no counterpart in the reference) ----
 * Network 25 -> 32 -> 32 -> 1 (ReLU), BF16 weights, FP32 accumulation; params are
 * hype_mlp_nparam() FP32 values W1[32][25] b1[32] W2[32][32] b2[32] W3[32] b3. A cell
 * is flagged when the sigmoid of the max of its three directional logits exceeds
 * prob_threshold (a low threshold sends low-confidence cells to CWENO4). */
int hype_euler_set_mlp(hype_euler* e, const float* params, float prob_threshold);
/* switch the reconstruction (HYPE_RECON_*) of an existing context, e.g. for a full-WENO shadow step */
int hype_euler_set_recon(hype_euler* e, int recon);
/* counts of owned cells sent to CWENO4 by the network / by the positivity fallback since the last reset
 * (per RK stage: a cell counts once in every stage that reconstructs it with CWENO4) */
int hype_euler_indicator_stats(hype_euler* e, long long* flagged, long long* positivity_fallbacks, int reset);
/* Fused FP32 stage only (HYPE_PREC_FP32, Rusanov, HYPE_STAGE_AUTO): per_step = 1 scores the
 * network once per step, on the first stage's input (and on every RHS-only call), widens the flags
 * to each cell's 3x3x3 neighbourhood and lets the step's four stages read them; per_step = 0 (the
 * default, and what every other form does) scores every stage's input, bit-identical to the
 * unfused kernels.  A discontinuity moves by less than a cell per step at CFL <= 1, so the
 * widened flags of the step's start cover it in the later stages. */
int hype_euler_set_gate_per_step(hype_euler* e, int per_step);
/* the fused FP32 stage's gate flags of the last scoring, one byte per extended cell
 * ((nx+2)(ny+2)(nz+2), x fastest, cell (i, j, k) at ((k+1)(ny+2) + j+1)(nx+2) + i+1): widened = 0
 * the network's flags, 1 their 3x3x3 widening (per-step scoring only); HYPE_ERR_UNSUPPORTED
 * before the network of an FP32 context is set */
int hype_euler_gate_flags(hype_euler* e, unsigned char* out, int widened);
/* training samples from the resident state: every stride-th owned cell, its three
 * directional normalised stencils X[s][3][25] and D[s], the largest change the CWENO4
 * nonlinear weights make to one of its 24 face traces relative to the linear R4
 * polynomial, in units of |cell value| + 1e-3 (labels: D > threshold). */
int hype_euler_sample_features(hype_euler* e, long long stride, float* X, float* D, long long* ns_out);
/* Shadow step: one step with the context's reconstruction and, from the same state,
 * one full-CWENO4 step; the first result is kept, *l1_rel = sum|rho - rho_full| / sum|rho_full|. */
int hype_euler_shadow_step(hype_euler* e, double* t_inout, double* dt_inout, double* l1_rel);

/* Allocation-free RHS evaluation.  This entry point has no counterpart in the
 * reference.  It serves callers that cannot let the library allocate device
 * memory: a host that owns every byte of device memory through its own pool and
 * hands over pre-allocated device vectors, or a latency-critical loop where
 * cudaMalloc's implicit device-wide synchronisation is not acceptable.  It
 * computes what hype_euler_rhs_device computes (same kernels, same results) on
 * device buffers dU -> dRHS (SoA [5][nz][ny][nx]) for the grid and options in
 * *p, without creating a context and without any cudaMalloc / cudaFree: all
 * scratch (face traces, face fluxes, the wave-speed and admissibility words)
 * lives in one fixed device array of this library, about 7.7 MB, that every GPU
 * which loads the library holds until the process exits.
 *   - Limit: (nx+2)(ny+2)(nz+2) <= 5832 (e.g. 16^3 cells; hype_euler_noalloc_max_ext
 *     returns the bound); larger grids return HYPE_ERR_ARG.
 *   - Options: CWENO4, R4 or WENO3; FP64 or FP32 reconstruction and flux; any flux;
 *     the positivity fallback (p->positivity 0 or 1) as in the context path.  No
 *     viscous terms (p->mu != 0 returns HYPE_ERR_UNSUPPORTED), no double-float form
 *     and no learned indicator (both need per-context state).
 *   - The first call on a device looks up the array's device address (once per
 *     device, with that device current) and keeps it for the life of the process;
 *     make that first call before any stream capture.  cudaDeviceReset (or any
 *     other teardown of the device's primary context) after the first call is not
 *     supported: the kept address would be stale.
 *   - Every call shares the one array: calls that overlap on the GPU (other
 *     streams, other host threads on the same device) race and corrupt each
 *     other's results; serialise them.
 *   - stream: a cudaStream_t, or NULL for the legacy default stream.  When dt_out
 *     is non-NULL the call waits for the stream and stores CFL h / (3 s_max) there
 *     (and returns HYPE_ERR_STATE for an inadmissible state); with dt_out NULL it
 *     returns without waiting. */
int hype_euler_rhs_noalloc(const hype_euler_params* p, const double* dU, double* dRHS, double* dt_out, void* stream);
long long hype_euler_noalloc_max_ext(void);

/* ============================================================ 2D multiphase */
/* models */
#define HYPE_MP_DI4 0     /* 4-equation diffuse interface, Q = (rho, rho u, rho v, E, phi)
                             (2d/weno4/bubble: pde.c, rhs_function.c) */
#define HYPE_MP_KAPILA5 1 /* Kapila five-equation, Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1)
                             (mixture EOS of 2d/HyPE-2D/kapila_5eqn.c:14-113) */
/* steppers */
#define HYPE_STEP_SSPRK43 0  /* TSSSP RKS3, 4 stages */
#define HYPE_STEP_SSPRK104 1 /* TSSSP RK104 (2d/weno4/bubble/hype.c:209-210) */

typedef struct hype_mp2d hype_mp2d;

typedef struct {
    int nx, ny;                 /* cells */
    double x_min, y_min, h, cfl;
    int bc[4];                  /* left, right, bottom, top: HYPE_BC_PERIODIC/REFLECTIVE/TRANSMISSIVE */
    int model;                  /* HYPE_MP_* */
    double g1, p1, g2, p2;      /* stiffened-gas phases: ratio of specific heats, stiffness */
    int stepper;                /* HYPE_STEP_* */
    int precision;              /* HYPE_PREC_*: FP32 = reconstruction + flux in FP32, EOS and state in FP64 */
    int dt_mode;                /* HYPE_DT_* (dt = CFL h / (2 s_max), 2d/weno4/bubble/rhs_function.c:385) */
    int recon;                  /* HYPE_RECON_CWENO4, or HYPE_RECON_LEARNED (hype_mp2d_set_mlp): the network
                                   scores each cell from its x and y stencils; flagged cells take CWENO4, the
                                   others its R4 limit, R4 failing the admissibility nodes is redone with CWENO4 */
} hype_mp2d_params;

int hype_mp2d_create(const hype_mp2d_params* p, hype_mp2d** out);
void hype_mp2d_destroy(hype_mp2d* m);
int hype_mp2d_get_params(const hype_mp2d* m, hype_mp2d_params* out);
/* Drop-in for the 2D RHSFunction (2d/weno4/bubble/rhs_function.c:12): primitive
 * CWENO4 with the 8-node admissibility check and minmod fallback, rotated HLLC,
 * divergence with the non-conservative volume-fraction term; host AoS [j][i][nv]. */
int hype_mp2d_rhs(hype_mp2d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out);
int hype_mp2d_upload(hype_mp2d* m, const double* U_aos);
int hype_mp2d_download(hype_mp2d* m, double* U_aos);
/* nsteps of the chosen SSP stepper on the resident state; *fallback_cells gets the
 * number of owned-cell reconstructions that fell back to minmod (PAD violations). */
int hype_mp2d_step(hype_mp2d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells);
int hype_mp2d_sync(hype_mp2d* m);
void* hype_mp2d_stream(hype_mp2d* m);
/* learned indicator of the 2D models (network layout as hype_mlp_*; inputs: the
 * normalised 5-point stencils of mixture density, normal and tangential velocity,
 * pressure and volume fraction along x and along y) */
int hype_mp2d_set_mlp(hype_mp2d* m, const float* params, float prob_threshold);
int hype_mp2d_set_recon(hype_mp2d* m, int recon);
/* owned-cell reconstructions the network flagged (full CWENO4) since the last reset (with the gate
 * scored once per step: those its widened flags send to CWENO4, counted in every stage) */
int hype_mp2d_indicator_stats(hype_mp2d* m, long long* flagged, int reset);
/* per_step = 1: the gate is scored on each step's first stage (and on RHS-only calls) in its own
 * pass, its flags widened to each cell's 3x3 neighbourhood and read by every stage of the step;
 * per_step = 0 (default): scored inside every stage's reconstruction.  Both precision forms. */
int hype_mp2d_set_gate_per_step(hype_mp2d* m, int per_step);
/* the last flags of the per-step gate, one byte per extended cell ((nx+2)(ny+2), x fastest, cell
 * (i, j) at (j+1)(nx+2) + i+1): widened = 0 the network's, 1 their 3x3 widening;
 * HYPE_ERR_UNSUPPORTED before hype_mp2d_set_mlp */
int hype_mp2d_gate_flags(hype_mp2d* m, unsigned char* out, int widened);
/* training samples from the resident state: every stride-th owned cell, its features
 * X[s][3][25] (x, y, y: the training kernels take three directions) and D[s], the
 * largest change the nonlinear CWENO4 weights make to one of its 8 face traces relative
 * to the R4 polynomial, in units of the variable's magnitude in the cell */
int hype_mp2d_sample_features(hype_mp2d* m, long long stride, float* X, float* D, long long* ns);

/* ============================================================ acoustic finite volume */
/* The acoustic path of 3d/weno4/plane_wave: u_tt = c^2 lap u as (u, v = u_t),
 * du/dt = v, dv/dt = c^2 div grad u; CWENO4 reconstruction of u (the reference runs
 * its optimal-weight limit, gammaHi = 1, reconstruction.c:38-44: HYPE_RECON_LINEAR4),
 * face-normal gradients at the 2x2 face Gauss points (evaluate_grad,
 * reconstruction.c:25-34), central flux c^2 (grad_L + grad_R).n/2 (pde.c:12-34),
 * SSPRK(4,3) with a fixed dt. State: host AoS [k][j][i][2] = (u, v). */
typedef struct hype_acoustic hype_acoustic;

typedef struct {
    int nx, ny, nz;
    double x_min, y_min, z_min, h;
    double c;   /* wave speed */
    double dt;  /* fixed time step (hype.c:56: h CFL / (3 c)) */
    int bc[6];  /* HYPE_BC_PERIODIC or HYPE_BC_ADIABATIC */
    int recon;  /* HYPE_RECON_LINEAR4 (the reference's setting) or HYPE_RECON_CWENO4 */
    int precision; /* HYPE_PREC_FP64, or HYPE_PREC_DF64: reconstruction, gradients and face fluxes in double-float
                      (FP32 pairs), state and stage accumulation in FP64 */
} hype_acoustic_params;

int hype_acoustic_create(const hype_acoustic_params* p, hype_acoustic** out);
void hype_acoustic_destroy(hype_acoustic* a);
int hype_acoustic_upload(hype_acoustic* a, const double* U_aos);
int hype_acoustic_download(hype_acoustic* a, double* U_aos);
/* Drop-in for its RHSFunction (3d/weno4/plane_wave/rhs_function.c:12-345) */
int hype_acoustic_rhs(hype_acoustic* a, const double* U_aos, double* RHS_aos);
/* up to nsteps steps from *t_inout; t_final > 0 shortens the step that would pass it
 * and stops there (TS_EXACTFINALTIME_MATCHSTEP, hype.c:178) */
int hype_acoustic_step(hype_acoustic* a, int nsteps, double t_final, double* t_inout, int* steps_taken);
/* the RHS at time t (the point source's argument; hype_acoustic_rhs is t = 0) */
int hype_acoustic_rhs_t(hype_acoustic* a, double t, const double* U_aos, double* RHS_aos);
/* The point source and receiver of 3d/weno4/point_source (AppCtx isx..irz, hype.c:59-64):
 * from now on every RHS evaluation at time t adds Source(t) / h^3 to the u_t equation of
 * cell (isx, isy, isz), Source(t) = -2 (t - t0) f0^2 exp(-f0^2 (t - t0)^2), t0 = 4 / f0
 * (source.c:11-17, rhs_function.c:337-339; the program's f0 is 100), and records u of cell
 * (irx, iry, irz) with t (rhs_function.c:342-346, which prints them to results/p.dat) into a
 * trace of up to trace_capacity samples.  isx < 0: no source; irx < 0: no receiver.  Calling
 * it again replaces the source and clears the trace. */
int hype_acoustic_set_point_source(hype_acoustic* a, int isx, int isy, int isz, double f0, int irx, int iry, int irz,
                                   int trace_capacity);
/* the receiver trace: t[q], u[q] for q < min(recorded, trace_capacity, max); *count = the RHS
 * evaluations seen since the receiver was set (also those past the capacity) */
int hype_acoustic_trace(hype_acoustic* a, double* t, double* u, int max, long long* count);
int hype_acoustic_sync(hype_acoustic* a);
void* hype_acoustic_stream(hype_acoustic* a);

/* ============================================================ 2D path-conservative (HyPE-2D) */
/* The RHS of 2d/HyPE-2D (RHSFunction, rhs_function.c:12-610) with its Kapila
 * five-equation model (kapila_5eqn.c): Q = (a1 rho1, a2 rho2, rho u, rho v, E, a1), AoS
 * [j][i][6]; the conservative variables reconstructed to order N = 0..3 (reconstruction.c),
 * PDECheckPAD at the admissibility nodes with first order on failure, the Rusanov flux plus
 * the Roe-path fluctuation of riemann.c:13-85, the non-conservative volume term, dt = CFL h /
 * (2 s_max), and the program's stepper for N (Euler, SSP RKS2/2, RKS3/4, RK104,
 * hype.c:361-382).  Results equal the reference program's bit for bit. */
typedef struct hype_pc2d hype_pc2d;

typedef struct {
    int nx, ny;
    double x_min, y_min, h;
    double cfl;
    int bc[4];              /* HYPE_BC_PERIODIC / REFLECTIVE / TRANSMISSIVE: left, right, bottom, top */
    int order;              /* N = 0..3 (Ctx.N, hype.c:32) */
    double g1, p1, g2, p2;  /* phase EOS (GAMMA_1, PI_1, GAMMA_2, PI_2; hype.h:41-44: 1.4, 0, 1.4, 0) */
} hype_pc2d_params;

int hype_pc2d_create(const hype_pc2d_params* p, hype_pc2d** out);
void hype_pc2d_destroy(hype_pc2d* m);
int hype_pc2d_get_params(const hype_pc2d* m, hype_pc2d_params* out);
/* Drop-in for RHSFunction (rhs_function.c:12); *dt_out: the Ctx->dt it sets */
int hype_pc2d_rhs(hype_pc2d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out);
int hype_pc2d_upload(hype_pc2d* m, const double* U_aos);
int hype_pc2d_download(hype_pc2d* m, double* U_aos);
/* nsteps of the program's stepper on the resident state; *dt_inout <= 0: dt from the first
 * RHS, kept for every step as the program keeps it (its monitor does not reset dt);
 * *fallback_cells: owned-cell reconstructions that fell back to first order */
int hype_pc2d_step(hype_pc2d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells);
int hype_pc2d_sync(hype_pc2d* m);
void* hype_pc2d_stream(hype_pc2d* m);

/* ============================================================ 3D multiphase */
/* The primitive-variable multiphase RHS of 3d/weno4/Viscous-Multiphase-Fourth-Order
 * (RHSFunctionPrimitive, rhs_function.c:56-570): Q = (rho, rho u, rho v, rho w, E, phi),
 * AoS [k][j][i][6]; the mixture of two stiffened gases (g, p_inf) mixed by phi
 * (pde.c:9-45); CWENO4 of the primitive variables with the 33-node density / pressure
 * check and first order on failure; rotated HLLC (pde.c:383-440) with the
 * non-conservative phi equation; SSP RKS3/4 stages; dt = (1/3) CFL h / (s_max +
 * 2 s_visc / h) with s_visc = (4/3)(phi mu1 + (1 - phi) mu2)/rho (rhs_function.c:559).
 * The program's viscous flux reads gradients its weno() never writes (zero when its
 * automatic variables start at zero): no viscous flux is applied, only its speed
 * limits dt (mu1 = mu2 = 0 for the inviscid CFL limit). */
typedef struct hype_mp3d hype_mp3d;

typedef struct {
    int nx, ny, nz;
    double x_min, y_min, z_min, h;
    double cfl;
    int bc[6];                  /* HYPE_BC_PERIODIC / REFLECTIVE / TRANSMISSIVE */
    double g1, p1, g2, p2;      /* phase EOS (hype.h:39-42 of the program: 1.4, 0, 1.6, 0) */
    double mu1, mu2;            /* phase viscosities of the dt limit (MU_1 1.4, MU_2 1.6) */
    int dt_mode;                /* HYPE_DT_* */
} hype_mp3d_params;

int hype_mp3d_create(const hype_mp3d_params* p, hype_mp3d** out);
void hype_mp3d_destroy(hype_mp3d* m);
int hype_mp3d_get_params(const hype_mp3d* m, hype_mp3d_params* out);
/* Drop-in for RHSFunctionPrimitive (rhs_function.c:56); *dt_out: the Ctx->dt it sets */
int hype_mp3d_rhs(hype_mp3d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out);
int hype_mp3d_upload(hype_mp3d* m, const double* U_aos);
int hype_mp3d_download(hype_mp3d* m, double* U_aos);
/* nsteps of SSP RKS3/4 stages on the resident state (dt semantics as hype_euler_step);
 * *fallback_cells: owned-cell reconstructions that fell back to first order */
int hype_mp3d_step(hype_mp3d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells);
int hype_mp3d_sync(hype_mp3d* m);
void* hype_mp3d_stream(hype_mp3d* m);

/* ---- 2D acoustic FV: 2d/weno4/standing_wave ----
 * The same system in 2D: state AoS [j][i][2] = (u, u_t); the 2D R4 polynomial of u
 * (weno(), reconstruction.c:108-125), its normal gradient at 2 Gauss points per edge,
 * the averaged flux c^2 grad u . n (pde.c:12-34), RK104 (hype.c:211) or RKS3/4 stages.
 * Results equal the reference program's bit for bit. */
typedef struct hype_acoustic2d hype_acoustic2d;

typedef struct {
    int nx, ny;
    double x_min, y_min, h;
    double c;    /* wave speed (wave_speed, hype.h:38) */
    double dt;   /* fixed time step (hype.c:50: h CFL / (2 c)) */
    int bc[4];   /* HYPE_BC_PERIODIC or HYPE_BC_ADIABATIC: left, right, bottom, top */
    int stepper; /* HYPE_STEP_SSPRK104 (the program's) or HYPE_STEP_SSPRK43 */
} hype_acoustic2d_params;

int hype_acoustic2d_create(const hype_acoustic2d_params* p, hype_acoustic2d** out);
void hype_acoustic2d_destroy(hype_acoustic2d* a);
int hype_acoustic2d_upload(hype_acoustic2d* a, const double* U_aos);
int hype_acoustic2d_download(hype_acoustic2d* a, double* U_aos);
/* Drop-in for its RHSFunction (2d/weno4/standing_wave/rhs_function.c:12-258) */
int hype_acoustic2d_rhs(hype_acoustic2d* a, const double* U_aos, double* RHS_aos);
/* up to nsteps steps from *t_inout; t_final > 0 shortens the step that would pass it
 * and stops there (TS_EXACTFINALTIME_MATCHSTEP, hype.c:208) */
int hype_acoustic2d_step(hype_acoustic2d* a, int nsteps, double t_final, double* t_inout, int* steps_taken);
/* the RHS at time t (hype_acoustic2d_rhs is t = 0) */
int hype_acoustic2d_rhs_t(hype_acoustic2d* a, double t, const double* U_aos, double* RHS_aos);
/* The line source and receiver of 2d/weno4/line_source (AppCtx isx, isy, irx, iry,
 * hype.c:52-55): every RHS evaluation at time t adds Source(t) / h^2 to the u_t equation of
 * cell (isx, isy) (source.c:12-18 with the program's f0 = 65, rhs_function.c:244-246) and
 * records u of cell (irx, iry) with t (rhs_function.c:249-253) into a trace of up to
 * trace_capacity samples; negative isx / irx turn them off; calling it again clears the trace. */
int hype_acoustic2d_set_point_source(hype_acoustic2d* a, int isx, int isy, double f0, int irx, int iry,
                                     int trace_capacity);
int hype_acoustic2d_trace(hype_acoustic2d* a, double* t, double* u, int max, long long* count);
int hype_acoustic2d_sync(hype_acoustic2d* a);
void* hype_acoustic2d_stream(hype_acoustic2d* a);

/* ============================================================ restart and output files */
/* PETSc binary Vec record (what VecView on a binary viewer writes and VecLoad reads:
 * int32 class id 1211214, int32 length, big-endian doubles; the reference's restart1.bin /
 * restart2.bin, 3d/weno3/Euler/monitor_function.c:46-62, read back at hype.c:147-155);
 * block_size > 1 also writes "<path>.info" with -vecload_block_size, as PETSc does for
 * a multi-component DMDA vector. */
int hype_write_petsc_vec(const char* path, const double* v, long long n, int block_size);
int hype_read_petsc_vec(const char* path, double* v, long long n);
/* legacy VTK 2.0 ASCII, STRUCTURED_POINTS on the cell centres, one SCALARS section per
 * component of the interleaved [k][j][i][c] array aos (the reference's sol-*.vtk,
 * hype.c:202-208, is PETSc's ASCII_VTK view of the same DMDA vector) */
int hype_write_vtk(const char* path, const char* title, int nx, int ny, int nz, double x0, double y0, double z0, double h,
                   int ncomp, const char* const* names, const double* aos);
/* the resident state of a context, in the DMDA natural order [k][j][i][c] */
int hype_euler_write_restart(hype_euler* e, const char* path);
int hype_euler_read_restart(hype_euler* e, const char* path);
int hype_euler_write_vtk(hype_euler* e, const char* path);
int hype_mp2d_write_restart(hype_mp2d* m, const char* path);
int hype_mp2d_read_restart(hype_mp2d* m, const char* path);
int hype_mp2d_write_vtk(hype_mp2d* m, const char* path);

/* ============================================================ CTCS acoustics */
/* Drop-in for CTCS(DM, Vec Pold, Vec Pcurr, Vec Pnew, AppCtx*)
 * (2d/ctcs/plane_wave/wave.c:161-203): one leapfrog update
 * pnew = alpha^2 (N + S + E + W - 4 C) + 2 C - pold, alpha = c dt / h, on host
 * arrays [ny][nx]; bc = HYPE_BC_PERIODIC or HYPE_BC_ZERO. */
int hype_ctcs2d_update(int nx, int ny, double alpha, int bc, const double* p_old, const double* p, double* p_new);

typedef struct hype_ctcs hype_ctcs;

typedef struct {
    int dim;            /* 2 or 3 */
    int nx, ny, nz;     /* nodes */
    int form;           /* 0: plane-wave form (2d/ctcs/plane_wave/wave.c:192, 2D, 2nd order)
                           1: point-source form (2d/ctcs/line_source/wave.c:149-173,
                              3d/ctcs/point_source/wave.c:163-194) */
    int order;          /* 2 or 4 (form 1) */
    int bc;             /* HYPE_BC_PERIODIC or HYPE_BC_ZERO */
    double dx, dy, dz, dt, c0;
    double f0;          /* Source() dominant frequency (form 1) */
    int src[3];         /* source node, src[0] < 0: none */
    int rec[3];         /* receiver node, rec[0] < 0: none */
} hype_ctcs_params;

int hype_ctcs_create(const hype_ctcs_params* p, hype_ctcs** out);
void hype_ctcs_destroy(hype_ctcs* c);
/* Set the two time levels (host arrays, x fastest). */
int hype_ctcs_set(hype_ctcs* c, const double* p_old, const double* p);
int hype_ctcs_get(hype_ctcs* c, double* p_old, double* p);
/* nsteps leapfrog updates with pointer rotation (no VecCopy); it0 = step index of
 * the first update (source time it*dt).  When a receiver is set, receiver[s]
 * gets p at the receiver before update s (the reference's p.dat line). */
int hype_ctcs_step(hype_ctcs* c, int nsteps, int it0, double* receiver);
/* device pointers of the newest and previous levels */
double* hype_ctcs_level_device(hype_ctcs* c, int which /* 0 = p, 1 = p_old */);
int hype_ctcs_sync(hype_ctcs* c);

/* ============================================================ batched CTCS */
/* Many independent 2D acoustic instances of uneven size in one persistent
 * launch over a tile work-list.  Each instance: nodes nx x ny on
 * [xmin, xmin+(nx-1)h] x [ymin, ...], zero-Dirichlet exterior, 2nd-order
 * CTCS with a Gaussian monopole s = exp(-|x-xs|^2/(2 sigma^2)) sin(2 pi f t)
 * added as c^2 dt^2 s. */
typedef struct {
    int nx, ny;
    double xmin, ymin, h, c0, dt;
    double xs, ys, sigma, freq;
} hype_mono_instance;

typedef struct hype_batch hype_batch;

int hype_batch_create(int ninst, const hype_mono_instance* inst, hype_batch** out);
void hype_batch_destroy(hype_batch* b);
/* tile shape in nodes, width x height: 32x16, 32x32, 32x64, 64x16, 64x32, 64x64,
 * 128x16, 128x32 or 256x16 (each thread marches the rows of its column);
 * 0 x 0 = autotuned by timing every shape and cached per grid-shape signature */
int hype_batch_set_tile(hype_batch* b, int tile_x, int tile_y);
/* the tile shape in use (after autotuning: the chosen one) */
int hype_batch_get_tile(const hype_batch* b, int* tile_x, int* tile_y);
/* initial levels of instance q (host arrays ny*nx) */
int hype_batch_set(hype_batch* b, int q, const double* p_old, const double* p);
int hype_batch_get(hype_batch* b, int q, double* p_old, double* p);
/* nsteps of every instance; graph=1 replays captured CUDA graphs of 30-step chunks */
int hype_batch_step(hype_batch* b, int nsteps, int graph);
int hype_batch_sync(hype_batch* b);
/* Scheduling (no counterpart in the reference, whose instances are separate runs of
 * 2d/ctcs/line_source/wave.c:98-111): the instances are split by node count into
 * nclasses classes of equal size, smallest first; each class runs on its own stream
 * and its kernels carry a launch priority, the smallest class the highest, so small
 * instances finish early while the larger ones fill the rest of the GPU.  nclasses = 0:
 * as many classes as the device has stream priority levels (at most 8); 1: all
 * instances advance together.  Results do not depend on it. */
int hype_batch_set_classes(hype_batch* b, int nclasses);
/* the number of classes and, when cls is not NULL, each instance's class */
int hype_batch_get_classes(const hype_batch* b, int* nclasses, int* cls);
/* completion time of every instance in the last hype_batch_step call, in seconds from
 * the call's start on the device timeline (CUDA events; an instance completes with its
 * class); waits for the call */
int hype_batch_instance_times(hype_batch* b, double* seconds);

/* ============================================================ indicator training */
int hype_mlp_nparam(void);
/* max-pooled logits of n cells (X[n][3][25]) */
int hype_mlp_score(const float* X, int n, const float* params, float* score);
/* summed BCE loss (positive-class weight) and its gradient over n cells, BF16 forward, FP32 accumulation */
int hype_mlp_grad(const float* X, const float* y, int n, const float* params, float pos_weight, float* grad, double* loss);
/* Adam on seeded shuffled minibatches; params updated in place; mean loss of the last epoch */
int hype_mlp_train(const float* X, const float* y, int n, float* params, int epochs, int batch, float lr, float pos_weight,
                   unsigned seed, double* final_loss);

/* ============================================================ misc */
/* Select the CUDA device that later hype_*_create calls of this thread use. */
int hype_set_device(int device);
int hype_device_count(int* n);
const char* hype_strerror(int code);
/* message of the last CUDA error seen by the library (thread-local) */
const char* hype_last_error(void);
/* number of kernel launches issued by the library so far (process-wide) */
long long hype_launch_count(void);
/* library version string */
const char* hype_version(void);

#ifdef __cplusplus
}
#endif
#endif
