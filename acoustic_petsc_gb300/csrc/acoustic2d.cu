// acoustic2d.cu -- the 2D acoustic finite-volume program of HyPE (2d/weno4/standing_wave):
// the wave equation u_tt = c^2 lap u as the first-order system (u, v = u_t),
//   du/dt = v,   dv/dt = c^2 div grad u,
// with the 2D fourth-order central polynomial of u in every cell (weno(),
// reconstruction.c:108-125, 10 coefficients), its normal gradient at the 2 Gauss points
// of each edge from the basis-gradient tables (reconstruction.c:50-100, filled as
// hype.c:137-166 fills them), the averaged flux c^2 (grad_L + grad_R) . n / 2
// (pde.c:12-34), and SSP RK104 or SSP RKS3/4 stages with a fixed dt
// (hype.c:197-213, TS_EXACTFINALTIME_MATCHSTEP).
//
// Per RHS evaluation (rhs_function.c:12-258):
//   k_sw_recon   per extended cell (-1..n on both axes): the 13-point stencil with the
//                program's ghost values (periodic wrap, or the adiabatic wall's odd
//                mirror, :46-95), the 10 coefficients and the 8 edge-normal gradients;
//   k_sw_update  per cell: the 4 edge fluxes from its own and its neighbours'
//                gradients (each edge computed identically by both of its cells), the
//                RHS (v, (1/h)(flux differences)) and the Runge-Kutta stage combination,
//                plus the line source of 2d/weno4/line_source (rhs_function.c:244-253:
//                Source(t)/h^2 in one cell, u at the receiver).
// Operation order follows the reference expression by expression and the file is
// compiled without FMA contraction, so results equal the reference's bit for bit.
#include <cuda_runtime.h>
#include <string.h>

#include "hype_common.cuh"
#include "point_source.cuh"

namespace hype {
namespace acoustic2d {

struct Geo {
    int nx, ny;
    int bc[4];
    long long N, NE;  // cells, extended cells (nx+2)(ny+2)
    int ex;           // nx + 2
};

// basis_grad (reconstruction.c:50-100), the component along axis d
__host__ __device__ constexpr double basis_grad_axis(double x, double y, int n, int d) {
    double gx = 0.0, gy = 0.0;
    switch (n) {
        case 1: gx = 1.0; break;
        case 2: gy = 1.0; break;
        case 3: gx = 2.0 * x; break;
        case 4: gy = 2.0 * y; break;
        case 5: gx = y; gy = x; break;
        case 6: gx = 3.0 * x * x - 3. / 20.; break;
        case 7: gy = 3.0 * y * y - 3. / 20.; break;
        case 8: gx = 2.0 * x * y; gy = (x * x - 1. / 12.); break;
        case 9: gx = (y * y - 1. / 12.); gy = 2.0 * x * y; break;
        default: break;
    }
    return d == 0 ? gx : gy;
}

// the 2-point Gauss abscissae on [-1/2, 1/2] (x_gp2, hype.h:56)
__host__ __device__ constexpr double gp2(int q) { return q == 0 ? -0.28867513459481287 : 0.28867513459481287; }

// the normal component of the basis gradient at Gauss point q of edge f (left, right,
// bottom, top) for basis k, as the program fills its tables (hype.c:137-166)
__host__ __device__ constexpr double tab(int f, int q, int k) {
    return f == 0 ? basis_grad_axis(-0.5, gp2(q), k, 0)
         : f == 1 ? basis_grad_axis(0.5, gp2(q), k, 0)
         : f == 2 ? basis_grad_axis(gp2(q), -0.5, k, 1)
                  : basis_grad_axis(gp2(q), 0.5, k, 1);
}

// sum_k c[k] tab(f, q, k) in the program's order (rhs_function.c:139-146), the terms
// whose table entry is zero left out: they add a signed zero, which changes no value
template <int F, int Q, int K = 0>
__device__ __forceinline__ double edge_grad(const double* c, double acc) {
    if constexpr (K == 10) {
        return acc;
    } else {
        constexpr double w = tab(F, Q, K);
        if constexpr (w == 0.0) return edge_grad<F, Q, K + 1>(c, acc);
        else return edge_grad<F, Q, K + 1>(c, acc + c[K] * w);
    }
}

// the program's ghost value map of one axis: periodic wrap, or the wall mirror (odd in u)
__device__ __forceinline__ int sw_map(int i, int n, int blo, int bhi, double& s) {
    if (i < 0) {
        if (blo == HYPE_BC_PERIODIC) return i + n;
        s = -s;
        return -1 - i;
    }
    if (i >= n) {
        if (bhi == HYPE_BC_PERIODIC) return i - n;
        s = -s;
        return 2 * (n - 1) - i + 1;
    }
    return i;
}

__device__ __forceinline__ double sw_u(const double* __restrict__ u, const Geo& g, int i, int j) {
    double s = 1.0;
    const int mi = sw_map(i, g.nx, g.bc[0], g.bc[1], s);
    const int mj = sw_map(j, g.ny, g.bc[2], g.bc[3], s);
    const double v = __ldg(u + (long long)mj * g.nx + mi);
    return s < 0.0 ? -v : v;
}

// T[(f*2+q)][extended cell]: (1/h) times the normal gradient at Gauss point q of edge f
__global__ void __launch_bounds__(256) k_sw_recon(const double* __restrict__ u, double* __restrict__ T, Geo g,
                                                  double r1_h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x - 1;
    const int j = blockIdx.y * blockDim.y + threadIdx.y - 1;
    if (i > g.nx || j > g.ny) return;
    constexpr double r41_60 = 41. / 60., r11_120 = 11. / 120., r1_6 = 1. / 6., r1_12 = 1. / 12.;
    double u_0, u_ip1, u_jp1, u_ip1jp1, u_im1, u_jm1, u_ip1jm1, u_ip2, u_jp2, u_im1jp1, u_im2, u_jm2, u_im1jm1;
    if (i >= 2 && i < g.nx - 2 && j >= 2 && j < g.ny - 2) {  // no ghost value in the stencil
        const double* p = u + (long long)j * g.nx + i;
        const int sy = g.nx;
        u_0 = __ldg(p);
        u_ip1 = __ldg(p + 1), u_jp1 = __ldg(p + sy), u_ip1jp1 = __ldg(p + sy + 1);
        u_im1 = __ldg(p - 1), u_jm1 = __ldg(p - sy), u_ip1jm1 = __ldg(p - sy + 1);
        u_ip2 = __ldg(p + 2), u_jp2 = __ldg(p + 2 * sy), u_im1jp1 = __ldg(p + sy - 1);
        u_im2 = __ldg(p - 2), u_jm2 = __ldg(p - 2 * sy), u_im1jm1 = __ldg(p - sy - 1);
    } else {
        u_0 = sw_u(u, g, i, j);
        u_ip1 = sw_u(u, g, i + 1, j), u_jp1 = sw_u(u, g, i, j + 1), u_ip1jp1 = sw_u(u, g, i + 1, j + 1);
        u_im1 = sw_u(u, g, i - 1, j), u_jm1 = sw_u(u, g, i, j - 1), u_ip1jm1 = sw_u(u, g, i + 1, j - 1);
        u_ip2 = sw_u(u, g, i + 2, j), u_jp2 = sw_u(u, g, i, j + 2), u_im1jp1 = sw_u(u, g, i - 1, j + 1);
        u_im2 = sw_u(u, g, i - 2, j), u_jm2 = sw_u(u, g, i, j - 2), u_im1jm1 = sw_u(u, g, i - 1, j - 1);
    }
    double c[10];
    c[0] = u_0;
    c[1] = r41_60 * (-u_im1 + u_ip1) + r11_120 * (u_im2 - u_ip2);
    c[2] = r41_60 * (-u_jm1 + u_jp1) + r11_120 * (u_jm2 - u_jp2);
    c[3] = -u_0 + 0.5 * (u_im1 + u_ip1);
    c[4] = -u_0 + 0.5 * (u_jm1 + u_jp1);
    c[5] = 0.25 * (u_im1jm1 - u_im1jp1 - u_ip1jm1 + u_ip1jp1);
    c[6] = r1_6 * (u_im1 - u_ip1) + r1_12 * (u_ip2 - u_im2);
    c[7] = r1_6 * (u_jm1 - u_jp1) + r1_12 * (u_jp2 - u_jm2);
    c[8] = 0.25 * (-u_im1jm1 + u_im1jp1 - u_ip1jm1 + u_ip1jp1) + 0.5 * (u_jm1 - u_jp1);
    c[9] = 0.5 * (u_im1 - u_ip1) + 0.25 * (u_ip1jp1 - u_im1jm1 - u_im1jp1 + u_ip1jm1);
    const long long e = (long long)(j + 1) * g.ex + (i + 1);
    T[0 * g.NE + e] = r1_h * edge_grad<0, 0>(c, 0.0);
    T[1 * g.NE + e] = r1_h * edge_grad<0, 1>(c, 0.0);
    T[2 * g.NE + e] = r1_h * edge_grad<1, 0>(c, 0.0);
    T[3 * g.NE + e] = r1_h * edge_grad<1, 1>(c, 0.0);
    T[4 * g.NE + e] = r1_h * edge_grad<2, 0>(c, 0.0);
    T[5 * g.NE + e] = r1_h * edge_grad<2, 1>(c, 0.0);
    T[6 * g.NE + e] = r1_h * edge_grad<3, 0>(c, 0.0);
    T[7 * g.NE + e] = r1_h * edge_grad<3, 1>(c, 0.0);
}

struct Stage {
    double a, b, c, d;  // out = a X + (c dt / d) L (+ b Y when b != 0); rhs_only: out = L
    int rhs_only;
};

// sum over the edge's 2 Gauss points of 0.5 (0.5 (F_R + F_L)), F = c^2 (grad . n)
__device__ __forceinline__ double sw_edge(double c2, double gL0, double gR0, double gL1, double gR1) {
    double flux = 0.0;
    flux += 0.5 * (0.5 * (c2 * gR0 + c2 * gL0));
    flux += 0.5 * (0.5 * (c2 * gR1 + c2 * gL1));
    return flux;
}

// W: the stage input (v = W[1] is the first RHS component); X, Y: the states the stage
// combines; all SoA [2][ny][nx]
// W, X, Y and out may be one array (in-place stages), so they carry no __restrict__
__global__ void __launch_bounds__(256) k_sw_update(const double* __restrict__ T, const double* W,
                                                   const double* X, const double* Y,
                                                   double* out, Geo g, double c2, double r1_h, Stage st,
                                                   double dt, SourceArgs src) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    const long long cell = (long long)j * g.nx + i;
    const long long e = (long long)(j + 1) * g.ex + (i + 1);
    auto t = [&](int f, int q, long long x) { return __ldg(T + (long long)(f * 2 + q) * g.NE + x); };
    // x edges: the left cell's right-edge gradients (f = 1) and the right cell's left-edge ones (f = 0)
    const double Fl = sw_edge(c2, t(1, 0, e - 1), t(0, 0, e), t(1, 1, e - 1), t(0, 1, e));
    const double Fr = sw_edge(c2, t(1, 0, e), t(0, 0, e + 1), t(1, 1, e), t(0, 1, e + 1));
    // y edges: top edge (f = 3) of the lower cell, bottom edge (f = 2) of the upper one
    const double Gb = sw_edge(c2, t(3, 0, e - g.ex), t(2, 0, e), t(3, 1, e - g.ex), t(2, 1, e));
    const double Gt = sw_edge(c2, t(3, 0, e), t(2, 0, e + g.ex), t(3, 1, e), t(2, 1, e + g.ex));
    double L[2] = {__ldg(W + g.N + cell), r1_h * (Fr - Fl) + r1_h * (Gt - Gb)};
    if (cell == src.src_cell) L[1] += src.src_val;
    if (cell == src.rec_cell) *src.slot = W[cell];  // read before out (which may alias W) is written
    const double cdt = st.rhs_only ? 0.0 : st.c * dt / st.d;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        double v;
        if (st.rhs_only) {
            v = L[c];
        } else {
            v = st.a * X[c * g.N + cell] + cdt * L[c];
            if (st.b != 0.0) v += st.b * Y[c * g.N + cell];
        }
        out[c * g.N + cell] = v;
    }
}

__global__ void k_sw_axpby(const double* __restrict__ X, const double* __restrict__ Y, double* __restrict__ out, double a,
                           double b, long long n) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < n) out[q] = a * X[q] + b * Y[q];
}

__global__ void k_sw_aos2soa(const double* __restrict__ a, double* __restrict__ s, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    s[q] = a[2 * q];
    s[N + q] = a[2 * q + 1];
}
__global__ void k_sw_soa2aos(const double* __restrict__ s, double* __restrict__ a, long long N) {
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= N) return;
    a[2 * q] = s[q];
    a[2 * q + 1] = s[N + q];
}

// the table as the program computes it at run time (hype.c:137-166), for the check that
// the compile-time table used by the kernels is the same, bit for bit
static bool tables_match() {
    const volatile double gp[2] = {gp2(0), gp2(1)};
    for (int q = 0; q < 2; ++q)
        for (int k = 0; k < 10; ++k) {
            const double x[4] = {-0.5, 0.5, gp[q], gp[q]}, y[4] = {gp[q], gp[q], -0.5, 0.5};
            for (int f = 0; f < 4; ++f) {
                const double run = basis_grad_axis(x[f], y[f], k, f < 2 ? 0 : 1);
                const double ct = tab(f, q, k);
                if (memcmp(&run, &ct, sizeof(double)) != 0 && !(run == 0.0 && ct == 0.0)) return false;
            }
        }
    return true;
}

}  // namespace acoustic2d
}  // namespace hype

using namespace hype;
using namespace hype::acoustic2d;

struct hype_acoustic2d {
    hype_acoustic2d_params p;
    Geo g;
    cudaStream_t stream = nullptr;
    double *U = nullptr, *W0 = nullptr, *W1 = nullptr, *S = nullptr, *L = nullptr, *T = nullptr, *aos = nullptr;
    PointSource ps;
};

// t: the time of this RHS evaluation (the line source's argument)
static int sw_rhs_stage(hype_acoustic2d* a, const double* Win, const double* X, const double* Y, double* out, Stage st,
                        double dt, double t) {
    const Geo& g = a->g;
    k_sw_recon<<<dim3(cdiv(g.nx + 2, 32), cdiv(g.ny + 2, 8)), dim3(32, 8), 0, a->stream>>>(Win, a->T, g, 1. / (a->p.h));
    k_sw_update<<<dim3(cdiv(g.nx, 32), cdiv(g.ny, 8)), dim3(32, 8), 0, a->stream>>>(
        a->T, Win, X, Y, out, g, a->p.c * a->p.c, 1. / (a->p.h), st, dt, source_args(a->ps, t));
    HYPE_LAUNCHED(2);
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_create(const hype_acoustic2d_params* p, hype_acoustic2d** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->nx < 3 || p->ny < 3 || !(p->h > 0) || !(p->c > 0) || !(p->dt > 0)) return HYPE_ERR_ARG;
    for (int f = 0; f < 4; ++f)
        if (p->bc[f] != HYPE_BC_PERIODIC && p->bc[f] != HYPE_BC_ADIABATIC) return HYPE_ERR_ARG;
    for (int d = 0; d < 2; ++d)
        if ((p->bc[2 * d] == HYPE_BC_PERIODIC) != (p->bc[2 * d + 1] == HYPE_BC_PERIODIC)) return HYPE_ERR_ARG;
    if (p->stepper != HYPE_STEP_SSPRK43 && p->stepper != HYPE_STEP_SSPRK104) return HYPE_ERR_ARG;
    if (!tables_match()) {
        set_last_error("hype_acoustic2d_create: compile-time basis-gradient table differs from the run-time one",
                       cudaSuccess);
        return HYPE_ERR_UNSUPPORTED;
    }
    hype_acoustic2d* a = new hype_acoustic2d();
    a->p = *p;
    Geo& g = a->g;
    g.nx = p->nx;
    g.ny = p->ny;
    for (int f = 0; f < 4; ++f) g.bc[f] = p->bc[f];
    g.N = (long long)p->nx * p->ny;
    g.ex = p->nx + 2;
    g.NE = (long long)(p->nx + 2) * (p->ny + 2);
    const size_t sN = sizeof(double) * 2 * (size_t)g.N;
    cudaError_t ce = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->U, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->W0, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->W1, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->S, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->L, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->aos, sN);
    if (ce == cudaSuccess) ce = cudaMalloc((void**)&a->T, sizeof(double) * 8 * (size_t)g.NE);
    if (ce != cudaSuccess) {
        set_last_error("hype_acoustic2d_create", ce);
        hype_acoustic2d_destroy(a);
        return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = a;
    return HYPE_OK;
}

extern "C" void hype_acoustic2d_destroy(hype_acoustic2d* a) {
    if (!a) return;
    if (a->stream) cudaStreamSynchronize(a->stream);
    cudaFree(a->U); cudaFree(a->W0); cudaFree(a->W1); cudaFree(a->S); cudaFree(a->L); cudaFree(a->aos); cudaFree(a->T);
    a->ps.release();
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
}

static int sw_h2d(hype_acoustic2d* a, const double* aos, double* soa) {
    const long long N = a->g.N;
    HYPE_CK(cudaMemcpyAsync(a->aos, aos, sizeof(double) * 2 * N, cudaMemcpyHostToDevice, a->stream));
    k_sw_aos2soa<<<cdiv(N, 256), 256, 0, a->stream>>>(a->aos, soa, N);
    HYPE_LAUNCHED(1);
    return HYPE_OK;
}

static int sw_d2h(hype_acoustic2d* a, const double* soa, double* aos) {
    const long long N = a->g.N;
    k_sw_soa2aos<<<cdiv(N, 256), 256, 0, a->stream>>>(soa, a->aos, N);
    HYPE_LAUNCHED(1);
    HYPE_CK(cudaMemcpyAsync(aos, a->aos, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, a->stream));
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_upload(hype_acoustic2d* a, const double* U_aos) {
    if (!a || !U_aos) return HYPE_ERR_ARG;
    int rc = sw_h2d(a, U_aos, a->U);
    if (rc) return rc;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_download(hype_acoustic2d* a, double* U_aos) {
    if (!a || !U_aos) return HYPE_ERR_ARG;
    return sw_d2h(a, a->U, U_aos);
}

extern "C" int hype_acoustic2d_rhs_t(hype_acoustic2d* a, double t, const double* U_aos, double* RHS_aos) {
    if (!a || !U_aos || !RHS_aos) return HYPE_ERR_ARG;
    int rc = sw_h2d(a, U_aos, a->S);
    if (rc || (rc = sw_rhs_stage(a, a->S, a->S, a->S, a->L, Stage{0.0, 0.0, 0.0, 1.0, 1}, 0.0, t))) return rc;
    return sw_d2h(a, a->L, RHS_aos);
}

extern "C" int hype_acoustic2d_rhs(hype_acoustic2d* a, const double* U_aos, double* RHS_aos) {
    return hype_acoustic2d_rhs_t(a, 0.0, U_aos, RHS_aos);
}

extern "C" int hype_acoustic2d_set_point_source(hype_acoustic2d* a, int isx, int isy, double f0, int irx, int iry,
                                                int trace_capacity) {
    if (!a || trace_capacity < 0) return HYPE_ERR_ARG;
    const Geo& g = a->g;
    const bool src = isx >= 0, rec = irx >= 0;
    if (src && (isx >= g.nx || isy < 0 || isy >= g.ny || !(f0 > 0))) return HYPE_ERR_ARG;
    if (rec && (irx >= g.nx || iry < 0 || iry >= g.ny)) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    PointSource& ps = a->ps;
    ps.release();
    ps = PointSource();
    ps.src_on = src;
    ps.src_cell = src ? (long long)isy * g.nx + isx : -1;
    ps.f0 = f0;
    ps.scale = 1. / ((a->p.h) * (a->p.h));  // r1_h2, rhs_function.c:24
    ps.rec_on = rec;
    ps.rec_cell = rec ? (long long)iry * g.nx + irx : -1;
    if (rec && trace_capacity > 0) {
        cudaError_t ce = cudaMalloc((void**)&ps.trace, sizeof(double) * (size_t)trace_capacity);
        if (ce != cudaSuccess) {
            set_last_error("hype_acoustic2d_set_point_source", ce);
            return ce == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
        }
        ps.capacity = trace_capacity;
    }
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_trace(hype_acoustic2d* a, double* t, double* u, int max, long long* count) {
    if (!a || max < 0 || ((!t || !u) && max > 0)) return HYPE_ERR_ARG;
    const PointSource& ps = a->ps;
    const int n = (int)(ps.count < ps.capacity ? ps.count : ps.capacity);
    const int m = n < max ? n : max;
    if (m > 0) {
        HYPE_CK(cudaMemcpyAsync(u, ps.trace, sizeof(double) * m, cudaMemcpyDeviceToHost, a->stream));
        for (int q = 0; q < m; ++q) t[q] = ps.times[q];
    }
    HYPE_CK(cudaStreamSynchronize(a->stream));
    if (count) *count = ps.count;
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_step(hype_acoustic2d* a, int nsteps, double t_final, double* t_inout, int* steps_taken) {
    if (!a || !t_inout || nsteps < 0) return HYPE_ERR_ARG;
    double t = *t_inout;
    int s = 0;
    const long long n2 = 2 * a->g.N;
    for (; s < nsteps; ++s) {
        if (t_final > 0.0 && t >= t_final) break;
        double h = a->p.dt;
        if (t_final > 0.0 && t + h > t_final) h = t_final - t;
        int rc;
        if (a->p.stepper == HYPE_STEP_SSPRK104) {
            // SSP RK104, low storage (Ketcheson 2008): five dt/6 stages on w0 = u, then
            // w1 = 9/25 w0 + 1/25 u, w0 = 15 w1 - 5 w0, four dt/6 stages, u = 3/5 w0 + dt/10 L(w0) + w1
            // stage times t + c_i dt, c = (0, 1, 2, 3, 4, 2, 3, 4, 5, 6) / 6
            static const double c[10] = {0, 1. / 6, 2. / 6, 3. / 6, 4. / 6, 2. / 6, 3. / 6, 4. / 6, 5. / 6, 1};
            const Stage s6{1.0, 0.0, 1.0, 6.0, 0};
            if ((rc = sw_rhs_stage(a, a->U, a->U, nullptr, a->W0, s6, h, t + c[0] * h))) return rc;
            for (int k = 1; k < 5; ++k)
                if ((rc = sw_rhs_stage(a, a->W0, a->W0, nullptr, a->W0, s6, h, t + c[k] * h))) return rc;
            k_sw_axpby<<<cdiv(n2, 256), 256, 0, a->stream>>>(a->W0, a->U, a->W1, 9.0 / 25, 1.0 / 25, n2);
            k_sw_axpby<<<cdiv(n2, 256), 256, 0, a->stream>>>(a->W1, a->W0, a->W0, 15.0, -5.0, n2);
            HYPE_LAUNCHED(2);
            for (int k = 5; k < 9; ++k)
                if ((rc = sw_rhs_stage(a, a->W0, a->W0, nullptr, a->W0, s6, h, t + c[k] * h))) return rc;
            if ((rc = sw_rhs_stage(a, a->W0, a->W0, a->W1, a->U, Stage{3.0 / 5, 1.0, 1.0, 10.0, 0}, h, t + h))) return rc;
        } else {
            // SSP RKS3, 4 stages: u1 = u + dt/2 L(u); u2 = u1 + dt/2 L(u1);
            // u3 = 2/3 u + dt/6 L(u2) + 1/3 u2; u^{n+1} = u3 + dt/2 L(u3)
            // stage times t + (0, 1/2, 1, 1/2) dt (c_i = i/(s-n), or (i-n)/(s-n) past n(n+1)/2)
            const Stage s2{1.0, 0.0, 1.0, 2.0, 0};
            if ((rc = sw_rhs_stage(a, a->U, a->U, nullptr, a->W0, s2, h, t + 1.0 * 0 / (4 - 2) * h))) return rc;
            if ((rc = sw_rhs_stage(a, a->W0, a->W0, nullptr, a->W0, s2, h, t + 1.0 * 1 / (4 - 2) * h))) return rc;
            if ((rc = sw_rhs_stage(a, a->W0, a->U, a->W0, a->W0,
                                   Stage{1.0 * 2 / (2 * 2 - 1.0), (2 - 1.0) / (2 * 2 - 1), 2 - 1.0, 2.0 * (2 * 2 - 1), 0},
                                   h, t + 1.0 * 2 / (4 - 2) * h)))
                return rc;
            if ((rc = sw_rhs_stage(a, a->W0, a->W0, nullptr, a->U, s2, h, t + (1.0 * 3 - 2) / (4 - 2) * h))) return rc;
        }
        t += h;
    }
    HYPE_CK(cudaStreamSynchronize(a->stream));
    *t_inout = t;
    if (steps_taken) *steps_taken = s;
    return HYPE_OK;
}

extern "C" int hype_acoustic2d_sync(hype_acoustic2d* a) {
    if (!a) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(a->stream));
    return HYPE_OK;
}

extern "C" void* hype_acoustic2d_stream(hype_acoustic2d* a) { return a ? (void*)a->stream : nullptr; }
