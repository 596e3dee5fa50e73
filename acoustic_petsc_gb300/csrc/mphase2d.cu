// mphase2d.cu -- 2D multiphase finite-volume RHS and SSP steppers on sm_103a.
//
// Per RHS evaluation (2d/weno4/bubble/rhs_function.c:12-390):
//   k_mp_prim   conserved -> primitive (ComputePrimitiveVariables), FP64;
//   k_mp_recon  one thread per cell of [-1,n]^2 that some owned face needs:
//               boundary map of the 13-point primitive stencil (replaces
//               DMGlobalToLocal + the BC sweeps :54-170), 2D CWENO4 per variable,
//               the 8-node admissibility check and the minmod fallback (:220-250),
//               the 4 faces x 2 Gauss-point traces (:252-273);
//   k_mp_faces  rotated HLLC at the two Gauss points of each face with the
//               interface-velocity component (:277-349), wave-speed max, flags;
//   k_mp_update divergence with the non-conservative volume-fraction term
//               (:351-380) fused with the stage combination.
// dt = CFL h / (2 s_max) is formed on the device (:385).
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "mphase2d_dev.cuh"

namespace hype {
namespace mp2d {

int launch_rhs_f32(int model, bool learned, const double* Win, float* Pf, void* T, float* F, float* G, const Geo& g,
                   const Eos& e, DevScalars* ds, int slot, const mlp::MmaWeights* mlp, float logit_thr,
                   unsigned long long* flagged, const GateStep& gs, cudaStream_t st);
void launch_update_f32(const float* F, const float* G, const double* Win, const double* X, const double* Y, double* out,
                       const Geo& g, double r1_h, Stage st, const DevScalars* ds, cudaStream_t stream);

__global__ void k_mp_prim(const double* __restrict__ U, double* __restrict__ P, Eos e, long long N, int nv) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    double Q[MAXV], V[MAXV];
    for (int c = 0; c < nv; ++c) Q[c] = U[c * N + q];
    cons2prim(e, Q, V);
    for (int c = 0; c < nv; ++c) P[c * N + q] = V[c];
}

// Win, X, Y and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_mp_update(const double* __restrict__ F, const double* __restrict__ G,
                                                   const double* Win, const double* X,
                                                   const double* Y, double* out, Geo g,
                                                   double r1_h, Stage st, const DevScalars* __restrict__ ds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    const int nv = g.nv, ia = nv - 1;
    const long long nfx = (long long)(g.nx + 1) * g.ny, nfy = (long long)g.nx * (g.ny + 1);
    const long long fxl = (long long)j * (g.nx + 1) + i, fyl = (long long)j * g.nx + i;
    const long long cell = (long long)j * g.nx + i;
    const double a = Win[ia * g.N + cell];
    const double cdt = st.rhs_only ? 0.0 : st.c * ds->dt / st.d;
    for (int c = 0; c < nv; ++c) {
        double L;
        if (c == ia)
            L = -r1_h * ((F[c * nfx + fxl + 1] - a * F[(c + 1) * nfx + fxl + 1]) - (F[c * nfx + fxl] - a * F[(c + 1) * nfx + fxl])) -
                r1_h * ((G[c * nfy + fyl + g.nx] - a * G[(c + 1) * nfy + fyl + g.nx]) - (G[c * nfy + fyl] - a * G[(c + 1) * nfy + fyl]));
        else
            L = -r1_h * (F[c * nfx + fxl + 1] - F[c * nfx + fxl]) - r1_h * (G[c * nfy + fyl + g.nx] - G[c * nfy + fyl]);
        double v;
        if (st.rhs_only) {
            v = L;
        } else {
            v = st.a * X[c * g.N + cell] + cdt * L;
            if (st.b != 0.0) v += st.b * Y[c * g.N + cell];
        }
        out[c * g.N + cell] = v;
    }
}

__global__ void k_mp_axpby(const double* __restrict__ X, const double* __restrict__ Y, double* __restrict__ out, double a,
                           double b, long long n) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) out[q] = a * X[q] + b * Y[q];
}

__global__ void k_mp_begin(DevScalars* ds, int mode, int src, int use_src, int reset, double cfl_h) {
    if (use_src && mode != HYPE_DT_FIXED) {
        const double smax = __longlong_as_double((long long)ds->smax_bits[src]);
        ds->dt = cfl_h / (2.0 * smax);
    }
    if (reset)
        for (int s = 0; s < 10; ++s) ds->smax_bits[s] = 0ull;
    ds->t += ds->dt;
}

__global__ void k_mp_reset(DevScalars* ds, int slot) {
    ds->smax_bits[slot] = 0ull;
    ds->bad = ~0ull;
}

__global__ void k_aos2soa(const double* __restrict__ a, double* __restrict__ s, long long N, int nv) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * nv) return;
    const long long cell = q / nv;
    s[(q - cell * nv) * N + cell] = a[q];
}
__global__ void k_soa2aos(const double* __restrict__ s, double* __restrict__ a, long long N, int nv) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N * nv) return;
    const long long cell = q / nv;
    a[q] = s[(q - cell * nv) * N + cell];
}

}  // namespace mp2d
}  // namespace hype

using namespace hype;
using namespace hype::mp2d;

static inline double bits2d(unsigned long long b) {
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

struct hype_mp2d {
    hype_mp2d_params p;
    Geo g;
    Eos e;
    cudaStream_t stream = nullptr;
    double *U = nullptr, *W0 = nullptr, *W1 = nullptr, *L = nullptr, *S = nullptr, *P = nullptr;
    float* Pf = nullptr;  // the FP32 form's primitives
    void* T = nullptr;
    double *F = nullptr, *G = nullptr, *stage_aos = nullptr;
    DevScalars* ds = nullptr;
    DevScalars* hs = nullptr;
    // learned indicator: packed network, logit threshold, flagged-cell counter
    mlp::MmaWeights* mlp = nullptr;
    float logit_thr = 0.0f;
    unsigned long long* flagged = nullptr;
    // the gate scored once per step: the network's flags and their 3 x 3 widening, one byte per
    // extended cell (allocated with the network)
    unsigned char *gate = nullptr, *gate_wide = nullptr;
    int gate_per_step = 0;
};

static int mp_rhs(hype_mp2d* m, const double* Win, int slot) {
    const Geo& g = m->g;
    const dim3 br(32, 4), gr(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 4));
    const dim3 gx(cdiv(g.nx + 1, 32), cdiv(g.ny, 4)), gy(cdiv(g.nx, 32), cdiv(g.ny + 1, 4));
    const bool f32 = m->p.precision == HYPE_PREC_FP32;
    const bool learned = m->p.recon == HYPE_RECON_LEARNED;
    if (learned && !m->mlp) return HYPE_ERR_ARG;  // hype_mp2d_set_mlp first
    double* Gf = m->G;
    // gate scored once per step: on the step's first stage (slot 0) and on RHS-only calls (slot 11)
    const bool per_step = learned && m->gate_per_step != 0;
    const GateStep gs{per_step, per_step && (slot == 0 || slot == 11), m->gate, m->gate_wide};
#define MP_LAUNCH(R, M)                                                                                        \
    do {                                                                                                       \
        if (gs.on)                                                                                             \
            launch_gated_recon<R, M, double>(m->P, (R*)m->T, g, m->e, m->ds, m->mlp, m->logit_thr, m->flagged, \
                                             gs, m->stream);                                                   \
        else if (learned)                                                                                      \
            k_mp_recon_learned<R, M><<<gr, br, 0, m->stream>>>(m->P, (R*)m->T, g, m->e, m->ds, m->mlp,         \
                                                               m->logit_thr, m->flagged);                      \
        else                                                                                                   \
            k_mp_recon<R, M><<<gr, br, 0, m->stream>>>(m->P, (R*)m->T, g, m->e, m->ds);                        \
        k_mp_faces<R, M, 0><<<gx, br, 0, m->stream>>>((const R*)m->T, m->F, g, m->e, m->ds, slot);             \
        k_mp_faces<R, M, 1><<<gy, br, 0, m->stream>>>((const R*)m->T, Gf, g, m->e, m->ds, slot);               \
    } while (0)
    if (f32) {  // the FP32 form lives in mphase2d_f32.cu (compiled with FMA contraction)
        launch_rhs_f32(m->e.model, learned, Win, m->Pf, m->T, (float*)m->F, (float*)Gf, g, m->e, m->ds, slot, m->mlp,
                       m->logit_thr, m->flagged, gs, m->stream);
    } else {
        k_mp_prim<<<cdiv(g.N, 256), 256, 0, m->stream>>>(Win, m->P, m->e, g.N, g.nv);
        if (m->e.model == HYPE_MP_DI4) MP_LAUNCH(double, HYPE_MP_DI4);
        else MP_LAUNCH(double, HYPE_MP_KAPILA5);
    }
#undef MP_LAUNCH
    HYPE_LAUNCHED(4 + (gs.score ? 2 : 0));
    return HYPE_OK;
}

static int mp_update(hype_mp2d* m, const double* Win, const double* X, const double* Y, double* out, Stage st) {
    const Geo& g = m->g;
    const dim3 b(32, 8), gr(cdiv(g.nx, 32), cdiv(g.ny, 8));
    if (m->p.precision == HYPE_PREC_FP32)  // FP32 face fluxes (mphase2d_f32.cu)
        launch_update_f32((const float*)m->F, (const float*)m->G, Win, X, Y, out, g, 1.0 / m->p.h, st, m->ds, m->stream);
    else
        k_mp_update<<<gr, b, 0, m->stream>>>(m->F, m->G, Win, X, Y, out, g, 1.0 / m->p.h, st, m->ds);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

extern "C" int hype_mp2d_create(const hype_mp2d_params* p, hype_mp2d** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || !(p->h > 0) || !(p->cfl > 0)) return HYPE_ERR_ARG;
    if (p->model != HYPE_MP_DI4 && p->model != HYPE_MP_KAPILA5) return HYPE_ERR_ARG;
    if (!(p->g1 > 1.0) || !(p->g2 > 1.0) || p->p1 < 0 || p->p2 < 0) return HYPE_ERR_ARG;
    for (int f = 0; f < 4; ++f)
        if (p->bc[f] < HYPE_BC_PERIODIC || p->bc[f] > HYPE_BC_TRANSMISSIVE) return HYPE_ERR_ARG;
    for (int d = 0; d < 2; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (p->stepper != HYPE_STEP_SSPRK43 && p->stepper != HYPE_STEP_SSPRK104) return HYPE_ERR_ARG;
    if (p->precision != HYPE_PREC_FP64 && p->precision != HYPE_PREC_FP32) return HYPE_ERR_ARG;
    if (p->dt_mode < HYPE_DT_MONITOR || p->dt_mode > HYPE_DT_FIXED) return HYPE_ERR_ARG;
    if (p->recon != HYPE_RECON_CWENO4 && p->recon != HYPE_RECON_LEARNED) return HYPE_ERR_ARG;
    hype_mp2d* m = new hype_mp2d();
    m->p = *p;
    Geo& g = m->g;
    g.nx = p->nx; g.ny = p->ny; g.nv = p->model == HYPE_MP_DI4 ? 5 : 6;
    for (int f = 0; f < 4; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny;
    g.NE = (long long)(p->nx + 2) * (p->ny + 2);
    m->e = make_eos(p->model, p->g1, p->p1, p->g2, p->p2);
    const size_t sN = sizeof(double) * g.nv * (size_t)g.N;
    const size_t tsz = (p->precision == HYPE_PREC_FP32 ? 4 : 8) * (size_t)g.nv * 8 * g.NE;
    cudaError_t ce = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    double** bufs[] = {&m->U, &m->W0, &m->W1, &m->L, &m->S, &m->P, &m->stage_aos};
    for (auto b : bufs)
        if (ce == cudaSuccess) ce = cudaMalloc((void**)b, sN);
    if (ce == cudaSuccess) ce = cudaMalloc(&m->T, tsz);
    if (ce == cudaSuccess && p->precision == HYPE_PREC_FP32)
        ce = cudaMalloc((void**)&m->Pf, sizeof(float) * g.nv * (size_t)g.N);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->F, sizeof(double) * (g.nv + 1) * (size_t)(p->nx + 1) * p->ny);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->G, sizeof(double) * (g.nv + 1) * (size_t)p->nx * (p->ny + 1));
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->ds, sizeof(DevScalars));
    if (ce == cudaSuccess) ce = cudaMallocHost((void**)&m->hs, sizeof(DevScalars));
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&m->flagged, sizeof(unsigned long long));
    if (ce == cudaSuccess) ce = cudaMemset(m->flagged, 0, sizeof(unsigned long long));
    if (ce == cudaSuccess) {
        DevScalars z;
        memset(&z, 0, sizeof(z));
        z.bad = ~0ull;
        ce = cudaMemcpy(m->ds, &z, sizeof(z), cudaMemcpyHostToDevice);
    }
    if (ce != cudaSuccess) {
        set_last_error("hype_mp2d_create", ce);
        hype_mp2d_destroy(m);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = m;
    return HYPE_OK;
}

extern "C" void hype_mp2d_destroy(hype_mp2d* m) {
    if (!m) return;
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->U); cudaFree(m->W0); cudaFree(m->W1); cudaFree(m->L); cudaFree(m->S); cudaFree(m->P);
    cudaFree(m->stage_aos); cudaFree(m->T); cudaFree(m->Pf); cudaFree(m->F); cudaFree(m->G); cudaFree(m->ds);
    cudaFree(m->mlp); cudaFree(m->flagged); cudaFree(m->gate); cudaFree(m->gate_wide);
    if (m->hs) cudaFreeHost(m->hs);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
}

static int mp_h2d(hype_mp2d* m, const double* aos, double* soa) {
    const long long n = m->g.N * m->g.nv;
    HYPE_CK(cudaMemcpyAsync(m->stage_aos, aos, sizeof(double) * n, cudaMemcpyHostToDevice, m->stream));
    k_aos2soa<<<cdiv(n, 256), 256, 0, m->stream>>>(m->stage_aos, soa, m->g.N, m->g.nv);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int mp_d2h(hype_mp2d* m, const double* soa, double* aos) {
    const long long n = m->g.N * m->g.nv;
    k_soa2aos<<<cdiv(n, 256), 256, 0, m->stream>>>(soa, m->stage_aos, m->g.N, m->g.nv);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, m->stage_aos, sizeof(double) * n, cudaMemcpyDeviceToHost, m->stream));
    return HYPE_OK;
}

static int mp_scalars(hype_mp2d* m) {
    HYPE_CK(cudaMemcpyAsync(m->hs, m->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp2d_rhs(hype_mp2d* m, double t, const double* U_aos, double* RHS_aos, double* dt_out) {
    (void)t;
    if (!m || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc;
    if ((rc = mp_h2d(m, U_aos, m->S))) return rc;
    k_mp_reset<<<1, 1, 0, m->stream>>>(m->ds, 11);
    HYPE_LAUNCHED(1);
    if ((rc = mp_rhs(m, m->S, 11))) return rc;
    if ((rc = mp_update(m, m->S, nullptr, nullptr, m->L, Stage{0, 0, 0, 1, 1}))) return rc;
    if ((rc = mp_d2h(m, m->L, RHS_aos))) return rc;
    if ((rc = mp_scalars(m))) return rc;
    if (dt_out) *dt_out = (m->p.cfl * m->p.h) / (2.0 * bits2d(m->hs->smax_bits[11]));
    return m->hs->bad == ~0ull ? HYPE_OK : HYPE_ERR_STATE;
}

extern "C" int hype_mp2d_get_params(const hype_mp2d* m, hype_mp2d_params* out) {
    if (!m || !out) return HYPE_ERR_ARG;
    *out = m->p;
    return HYPE_OK;
}

extern "C" int hype_mp2d_upload(hype_mp2d* m, const double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    int rc = mp_h2d(m, U_aos, m->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp2d_download(hype_mp2d* m, double* U_aos) {
    if (!m || !U_aos) return HYPE_ERR_ARG;
    int rc = mp_d2h(m, m->U, U_aos);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" void* hype_mp2d_stream(hype_mp2d* m) { return m ? (void*)m->stream : nullptr; }

extern "C" int hype_mp2d_step(hype_mp2d* m, int nsteps, double* t_inout, double* dt_inout, long long* fallback_cells) {
    if (!m || nsteps < 0 || !t_inout || !dt_inout) return HYPE_ERR_ARG;
    const int mode = m->p.dt_mode;
    if (mode == HYPE_DT_FIXED && !(*dt_inout > 0)) return HYPE_ERR_ARG;
    const double cfl_h = m->p.cfl * m->p.h;
    DevScalars init;
    memset(&init, 0, sizeof(init));
    init.t = *t_inout;
    init.dt = *dt_inout;
    init.bad = ~0ull;
    HYPE_CK(cudaMemcpyAsync(m->ds, &init, sizeof(init), cudaMemcpyHostToDevice, m->stream));
    const bool first_from_rhs = (mode != HYPE_DT_FIXED) && !(*dt_inout > 0);
    const int last = m->p.stepper == HYPE_STEP_SSPRK43 ? 3 : 9;
    int rc;
    for (int s = 0; s < nsteps; ++s) {
        if (s == 0 && first_from_rhs) {
            if ((rc = mp_rhs(m, m->U, 0))) return rc;
            k_mp_begin<<<1, 1, 0, m->stream>>>(m->ds, mode, 0, 1, 0, cfl_h);
        } else {
            k_mp_begin<<<1, 1, 0, m->stream>>>(m->ds, mode, last, mode == HYPE_DT_MONITOR && s > 0, 1, cfl_h);
            HYPE_LAUNCHED(1);
            if ((rc = mp_rhs(m, m->U, 0))) return rc;
        }
        HYPE_LAUNCHED(1);
        if (m->p.stepper == HYPE_STEP_SSPRK43) {
            // SSPRK(4,3): u1 = u + dt/2 L(u); u2 = u1 + dt/2 L(u1); u3 = 2/3 u + 1/3 u2 + dt/6 L(u2); u4 = u3 + dt/2 L(u3)
            if ((rc = mp_update(m, m->U, m->U, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 2.0, 0}))) return rc;
            if ((rc = mp_rhs(m, m->W0, 1)) || (rc = mp_update(m, m->W0, m->W0, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 2.0, 0}))) return rc;
            if ((rc = mp_rhs(m, m->W0, 2)) || (rc = mp_update(m, m->W0, m->U, m->W0, m->W0, Stage{1.0 * 2 / (2 * 2 - 1.0), (2 - 1.0) / (2 * 2 - 1), 2 - 1.0, 2.0 * (2 * 2 - 1), 0})))
                return rc;
            if ((rc = mp_rhs(m, m->W0, 3)) || (rc = mp_update(m, m->W0, m->W0, nullptr, m->U, Stage{1.0, 0.0, 1.0, 2.0, 0}))) return rc;
        } else {
            // SSPRK(10,4) low-storage (Ketcheson 2008): five dt/6 stages, q2 = 9/25 q1 + 1/25 u,
            // q1 = 15 q2 - 5 q1, four dt/6 stages, u = 3/5 q1 + q2 + dt/10 L(q1)
            const long long n = m->g.N * m->g.nv;
            if ((rc = mp_update(m, m->U, m->U, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 6.0, 0}))) return rc;
            for (int k = 1; k < 5; ++k)
                if ((rc = mp_rhs(m, m->W0, k)) || (rc = mp_update(m, m->W0, m->W0, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 6.0, 0})))
                    return rc;
            k_mp_axpby<<<cdiv(n, 256), 256, 0, m->stream>>>(m->W0, m->U, m->W1, 9.0 / 25, 1.0 / 25, n);
            k_mp_axpby<<<cdiv(n, 256), 256, 0, m->stream>>>(m->W1, m->W0, m->W0, 15.0, -5.0, n);
            HYPE_LAUNCHED(2);
            for (int k = 5; k < 9; ++k)
                if ((rc = mp_rhs(m, m->W0, k)) || (rc = mp_update(m, m->W0, m->W0, nullptr, m->W0, Stage{1.0, 0.0, 1.0, 6.0, 0})))
                    return rc;
            if ((rc = mp_rhs(m, m->W0, 9)) || (rc = mp_update(m, m->W0, m->W0, m->W1, m->U, Stage{3.0 / 5, 1.0, 1.0, 10.0, 0})))
                return rc;
        }
    }
    if ((rc = mp_scalars(m))) return rc;
    *t_inout = m->hs->t;
    const double sl = bits2d(m->hs->smax_bits[last]);
    *dt_inout = (nsteps > 0 && mode == HYPE_DT_MONITOR) ? cfl_h / (2.0 * sl) : m->hs->dt;
    if (fallback_cells) *fallback_cells = (long long)m->hs->fallback;
    return m->hs->bad == ~0ull ? HYPE_OK : HYPE_ERR_STATE;
}

extern "C" int hype_mp2d_sync(hype_mp2d* m) {
    if (!m) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

// ------------------------------------------------------------------ learned indicator
extern "C" int hype_mp2d_set_mlp(hype_mp2d* m, const float* params, float prob_threshold) {
    if (!m || !params || !(prob_threshold > 0.0f) || !(prob_threshold < 1.0f)) return HYPE_ERR_ARG;
    std::vector<__nv_bfloat16> h(mlp::NPARAM);
    for (int q = 0; q < mlp::NPARAM; ++q) h[q] = __float2bfloat16_rn(params[q]);
    mlp::MmaWeights hw;  // host staging, copied before the stream synchronisation below
    mlp::pack_weights(h.data(), hw);
    if (!m->mlp) HYPE_CK(cudaMalloc((void**)&m->mlp, sizeof(mlp::MmaWeights)));
    if (!m->gate) {
        HYPE_CK(cudaMalloc((void**)&m->gate, (size_t)m->g.NE));
        HYPE_CK(cudaMalloc((void**)&m->gate_wide, (size_t)m->g.NE));
        HYPE_CK(cudaMemsetAsync(m->gate, 0, (size_t)m->g.NE, m->stream));
        HYPE_CK(cudaMemsetAsync(m->gate_wide, 0, (size_t)m->g.NE, m->stream));
    }
    HYPE_CK(cudaMemcpyAsync(m->mlp, &hw, sizeof(mlp::MmaWeights), cudaMemcpyHostToDevice, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    m->logit_thr = logf(prob_threshold / (1.0f - prob_threshold));
    return HYPE_OK;
}

extern "C" int hype_mp2d_set_recon(hype_mp2d* m, int recon) {
    if (!m || (recon != HYPE_RECON_CWENO4 && recon != HYPE_RECON_LEARNED)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    m->p.recon = recon;
    return HYPE_OK;
}

extern "C" int hype_mp2d_set_gate_per_step(hype_mp2d* m, int per_step) {
    if (!m || (per_step != 0 && per_step != 1)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(m->stream));
    m->gate_per_step = per_step;
    return HYPE_OK;
}

extern "C" int hype_mp2d_gate_flags(hype_mp2d* m, unsigned char* out, int widened) {
    if (!m || !out || (widened != 0 && widened != 1)) return HYPE_ERR_ARG;
    if (!m->gate) return HYPE_ERR_UNSUPPORTED;
    HYPE_CK(cudaMemcpyAsync(out, widened ? m->gate_wide : m->gate, (size_t)m->g.NE, cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp2d_indicator_stats(hype_mp2d* m, long long* flagged, int reset) {
    if (!m) return HYPE_ERR_ARG;
    unsigned long long c = 0;
    HYPE_CK(cudaMemcpyAsync(&c, m->flagged, sizeof(c), cudaMemcpyDeviceToHost, m->stream));
    HYPE_CK(cudaStreamSynchronize(m->stream));
    if (flagged) *flagged = (long long)c;
    if (reset) HYPE_CK(cudaMemsetAsync(m->flagged, 0, sizeof(c), m->stream));
    return HYPE_OK;
}

extern "C" int hype_mp2d_sample_features(hype_mp2d* m, long long stride, float* X, float* D, long long* ns_out) {
    if (!m || stride < 1 || !X || !D) return HYPE_ERR_ARG;
    const Geo& g = m->g;
    const long long ns = (g.N + stride - 1) / stride;
    float *dX = nullptr, *dD = nullptr;
    cudaError_t ce = cudaMalloc((void**)&dX, sizeof(float) * ns * 3 * mlp::NIN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&dD, sizeof(float) * ns);
    if (ce == cudaSuccess) {
        k_mp_prim<<<cdiv(g.N, 256), 256, 0, m->stream>>>(m->U, m->P, m->e, g.N, g.nv);
        if (m->e.model == HYPE_MP_DI4)
            k_mp_features<HYPE_MP_DI4><<<cdiv(ns, 128), 128, 0, m->stream>>>(m->P, g, m->e, stride, ns, dX, dD);
        else
            k_mp_features<HYPE_MP_KAPILA5><<<cdiv(ns, 128), 128, 0, m->stream>>>(m->P, g, m->e, stride, ns, dX, dD);
        HYPE_LAUNCHED(2);
        ce = cudaMemcpyAsync(X, dX, sizeof(float) * ns * 3 * mlp::NIN, cudaMemcpyDeviceToHost, m->stream);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(D, dD, sizeof(float) * ns, cudaMemcpyDeviceToHost, m->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(m->stream);
    }
    cudaFree(dX);
    cudaFree(dD);
    if (ce != cudaSuccess) {
        set_last_error("hype_mp2d_sample_features", ce);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    if (ns_out) *ns_out = ns;
    return HYPE_OK;
}
