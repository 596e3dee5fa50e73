// ctcs.cu -- CTCS leapfrog acoustics on sm_103a.
//
// Compiled with -fmad=false: every update keeps the reference's operation order
// without FMA contraction, so results are bit-identical to the CPU restatement
// of the reference (memory-bound kernels: contraction buys nothing here).
//   plane-wave form   2d/ctcs/plane_wave/wave.c:192   pnew = a^2 (N+S+E+W-4C) + 2C - pold
//   point-source form 2d/ctcs/line_source/wave.c:155-173, 3d/ctcs/point_source/wave.c:173-194
//                     pnew = 2p - pold + c^2 dt^2 (pxx+pyy[+pzz]) (+ source at one node)
// Time levels rotate by pointer (the reference's two VecCopy per step,
// 2d/ctcs/line_source/wave.c:104-105, become free), and a chunk of steps is
// captured once as a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "hype_common.cuh"

namespace hype {
namespace ctcs {

struct Grid {
    int dim, nx, ny, nz, bc, order;
    double inv_x2, inv_y2, inv_z2;  // 1/(dx*dx) ...
    double k2;                      // c0*c0*dt*dt
    double a2;                      // (c0*dt/h)^2 of the plane-wave form
    long long src, rec;             // linear node of source / receiver (-1: none)
};

struct DevStep {
    int step;  // index of the update inside the current call
};

__device__ __forceinline__ double at2(const double* __restrict__ p, const Grid& g, int i, int j) {
    if (i < 0 || i >= g.nx || j < 0 || j >= g.ny) {
        if (g.bc != HYPE_BC_PERIODIC) return 0.0;
        i = i < 0 ? i + g.nx : (i >= g.nx ? i - g.nx : i);
        j = j < 0 ? j + g.ny : (j >= g.ny ? j - g.ny : j);
    }
    return p[(long long)j * g.nx + i];
}

__device__ __forceinline__ double at3(const double* __restrict__ p, const Grid& g, int i, int j, int k) {
    if (i < 0 || i >= g.nx || j < 0 || j >= g.ny || k < 0 || k >= g.nz) {
        if (g.bc != HYPE_BC_PERIODIC) return 0.0;
        i = i < 0 ? i + g.nx : (i >= g.nx ? i - g.nx : i);
        j = j < 0 ? j + g.ny : (j >= g.ny ? j - g.ny : j);
        k = k < 0 ? k + g.nz : (k >= g.nz ? k - g.nz : k);
    }
    return p[((long long)k * g.ny + j) * g.nx + i];
}

// plane-wave form, 2D 5-point (wave.c:192)
__global__ void __launch_bounds__(256) k_plane2d(const double* __restrict__ pold, const double* __restrict__ p,
                                                 double* __restrict__ pnew, Grid g) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.nx || j >= g.ny) return;
    const long long o = (long long)j * g.nx + i;
    const double c = p[o];
    const double s = at2(p, g, i, j + 1) + at2(p, g, i, j - 1) + at2(p, g, i + 1, j) + at2(p, g, i - 1, j) - 4.0 * c;
    pnew[o] = g.a2 * s + 2.0 * c - pold[o];
}

__device__ __forceinline__ double d2o2(double m1, double c, double p1, double inv) { return (p1 - 2.0 * c + m1) * inv; }
__device__ __forceinline__ double d2o4(double m2, double m1, double c, double p1, double p2, double inv) {
    return (-1.0 / 12 * p2 + 4.0 / 3.0 * p1 - 5.0 / 2.0 * c + 4.0 / 3.0 * m1 - 1.0 / 12.0 * m2) * inv;
}

// point-source form, 2D/3D, 2nd/4th order; srcv[s] = Source(it*dt)/vol*dt*dt precomputed on the host
template <int DIM, int ORDER>
__global__ void __launch_bounds__(256) k_src(const double* __restrict__ pold, const double* __restrict__ p,
                                             double* __restrict__ pnew, Grid g, const double* __restrict__ srcv,
                                             double* __restrict__ recv, const DevStep* __restrict__ st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = (DIM == 3) ? blockIdx.z : 0;
    if (i >= g.nx || j >= g.ny) return;
    const long long o = ((long long)k * g.ny + j) * g.nx + i;
    const double c = p[o];
    double lap;
    if (ORDER == 4) {
        const double pxx = d2o4(at3(p, g, i - 2, j, k), at3(p, g, i - 1, j, k), c, at3(p, g, i + 1, j, k), at3(p, g, i + 2, j, k), g.inv_x2);
        const double pyy = d2o4(at3(p, g, i, j - 2, k), at3(p, g, i, j - 1, k), c, at3(p, g, i, j + 1, k), at3(p, g, i, j + 2, k), g.inv_y2);
        if (DIM == 3) {
            const double pzz = d2o4(at3(p, g, i, j, k - 2), at3(p, g, i, j, k - 1), c, at3(p, g, i, j, k + 1), at3(p, g, i, j, k + 2), g.inv_z2);
            lap = pxx + pyy + pzz;
        } else {
            lap = pxx + pyy;
        }
    } else {
        const double pxx = d2o2(at3(p, g, i - 1, j, k), c, at3(p, g, i + 1, j, k), g.inv_x2);
        const double pyy = d2o2(at3(p, g, i, j - 1, k), c, at3(p, g, i, j + 1, k), g.inv_y2);
        if (DIM == 3) {
            const double pzz = d2o2(at3(p, g, i, j, k - 1), c, at3(p, g, i, j, k + 1), g.inv_z2);
            lap = pxx + pyy + pzz;
        } else {
            lap = pxx + pyy;
        }
    }
    double v = 2.0 * c - pold[o] + g.k2 * lap;
    if (o == g.src && srcv) v += srcv[st->step];
    if (o == g.rec && recv) recv[st->step] = c;
    pnew[o] = v;
}

__global__ void k_tick(DevStep* st) { st->step += 1; }

}  // namespace ctcs
}  // namespace hype

using namespace hype;
using namespace hype::ctcs;

static Grid make_grid_plane(int nx, int ny, double alpha, int bc) {
    Grid g;
    memset(&g, 0, sizeof(g));
    g.dim = 2; g.nx = nx; g.ny = ny; g.nz = 1; g.bc = bc; g.order = 2;
    g.a2 = alpha * alpha;
    g.src = g.rec = -1;
    return g;
}

extern "C" int hype_ctcs2d_update(int nx, int ny, double alpha, int bc, const double* p_old, const double* p, double* p_new) {
    if (nx < 1 || ny < 1 || !p_old || !p || !p_new) return HYPE_ERR_ARG;
    if (bc != HYPE_BC_PERIODIC && bc != HYPE_BC_ZERO) return HYPE_ERR_ARG;
    const size_t bytes = sizeof(double) * (size_t)nx * ny;
    double* d = nullptr;
    HYPE_CK(cudaMalloc((void**)&d, 3 * bytes));
    int rc = HYPE_OK;
    cudaError_t e;
    do {
        if ((e = cudaMemcpy(d, p_old, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(d + (size_t)nx * ny, p, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        Grid g = make_grid_plane(nx, ny, alpha, bc);
        const dim3 b(32, 8), gr(cdiv(nx, 32), cdiv(ny, 8));
        k_plane2d<<<gr, b>>>(d, d + (size_t)nx * ny, d + 2 * (size_t)nx * ny, g);
        count_launch(1);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        if ((e = cudaMemcpy(p_new, d + 2 * (size_t)nx * ny, bytes, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
    } while (0);
    if (e != cudaSuccess) {
        set_last_error("hype_ctcs2d_update", e);
        rc = HYPE_ERR_CUDA;
    }
    cudaFree(d);
    return rc;
}

struct hype_ctcs {
    hype_ctcs_params p;
    Grid g;
    cudaStream_t stream = nullptr;
    double* lv[3] = {nullptr, nullptr, nullptr};  // rotating levels
    int cur = 1;  // index of p (newest); p_old = cur-1 mod 3
    double* srcv = nullptr;
    double* recv = nullptr;
    int cap = 0;  // capacity of srcv/recv
    DevStep* st = nullptr;
    long long n = 0;
    // graph of a chunk of steps for each rotation phase
    cudaGraphExec_t chunk[3] = {nullptr, nullptr, nullptr};
    int chunk_len = 0;
};

static int ctcs_launch(hype_ctcs* c, int phase) {
    const Grid& g = c->g;
    double* po = c->lv[(phase + 2) % 3];
    double* pc = c->lv[phase];
    double* pn = c->lv[(phase + 1) % 3];
    const dim3 b(32, 8);
    const dim3 gr(cdiv(g.nx, 32), cdiv(g.ny, 8), g.dim == 3 ? g.nz : 1);
    if (c->p.form == 0) {
        k_plane2d<<<gr, b, 0, c->stream>>>(po, pc, pn, g);
        HYPE_LAUNCHED(1);
        return HYPE_OK;
    }
    const bool tick = (g.src >= 0 || g.rec >= 0);
    double* sv = g.src >= 0 ? c->srcv : nullptr;
    double* rv = g.rec >= 0 ? c->recv : nullptr;
    if (g.dim == 2 && g.order == 2) k_src<2, 2><<<gr, b, 0, c->stream>>>(po, pc, pn, g, sv, rv, c->st);
    else if (g.dim == 2) k_src<2, 4><<<gr, b, 0, c->stream>>>(po, pc, pn, g, sv, rv, c->st);
    else if (g.order == 2) k_src<3, 2><<<gr, b, 0, c->stream>>>(po, pc, pn, g, sv, rv, c->st);
    else k_src<3, 4><<<gr, b, 0, c->stream>>>(po, pc, pn, g, sv, rv, c->st);
    HYPE_LAUNCHED(1);
    if (tick) {
        k_tick<<<1, 1, 0, c->stream>>>(c->st);
        HYPE_LAUNCHED(1);
    }
    return HYPE_OK;
}

extern "C" int hype_ctcs_create(const hype_ctcs_params* p, hype_ctcs** out) {
    if (!p || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    if (p->dim != 2 && p->dim != 3) return HYPE_ERR_ARG;
    if (p->nx < 3 || p->ny < 3 || (p->dim == 3 && p->nz < 3)) return HYPE_ERR_ARG;
    if (p->bc != HYPE_BC_PERIODIC && p->bc != HYPE_BC_ZERO) return HYPE_ERR_ARG;
    if (p->form == 0 && p->dim != 2) return HYPE_ERR_UNSUPPORTED;
    if (p->form == 1 && p->order != 2 && p->order != 4) return HYPE_ERR_ARG;
    if (!(p->dt > 0) || !(p->dx > 0) || !(p->dy > 0) || (p->dim == 3 && !(p->dz > 0))) return HYPE_ERR_ARG;
    hype_ctcs* c = new hype_ctcs();
    c->p = *p;
    Grid& g = c->g;
    memset(&g, 0, sizeof(g));
    g.dim = p->dim; g.nx = p->nx; g.ny = p->ny; g.nz = p->dim == 3 ? p->nz : 1;
    g.bc = p->bc; g.order = p->order;
    g.inv_x2 = 1.0 / (p->dx * p->dx);
    g.inv_y2 = 1.0 / (p->dy * p->dy);
    g.inv_z2 = p->dim == 3 ? 1.0 / (p->dz * p->dz) : 0.0;
    g.k2 = p->c0 * p->c0 * p->dt * p->dt;
    const double alpha = p->c0 * p->dt / p->dx;  // wave.c:169
    g.a2 = alpha * alpha;
    auto lin = [&](const int* v) -> long long {
        if (v[0] < 0) return -1;
        if (v[0] >= g.nx || v[1] < 0 || v[1] >= g.ny || (g.dim == 3 && (v[2] < 0 || v[2] >= g.nz))) return -2;
        return ((long long)(g.dim == 3 ? v[2] : 0) * g.ny + v[1]) * g.nx + v[0];
    };
    g.src = p->form == 1 ? lin(p->src) : -1;
    g.rec = p->form == 1 ? lin(p->rec) : -1;
    if (g.src == -2 || g.rec == -2) {
        delete c;
        return HYPE_ERR_ARG;
    }
    c->n = (long long)g.nx * g.ny * g.nz;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMalloc((void**)&c->lv[q], sizeof(double) * c->n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&c->st, sizeof(DevStep));
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMemset(c->lv[q], 0, sizeof(double) * c->n);
    if (e != cudaSuccess) {
        set_last_error("hype_ctcs_create", e);
        hype_ctcs_destroy(c);
        return e == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    *out = c;
    return HYPE_OK;
}

extern "C" void hype_ctcs_destroy(hype_ctcs* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int q = 0; q < 3; ++q) {
        cudaFree(c->lv[q]);
        if (c->chunk[q]) cudaGraphExecDestroy(c->chunk[q]);
    }
    cudaFree(c->srcv);
    cudaFree(c->recv);
    cudaFree(c->st);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" int hype_ctcs_set(hype_ctcs* c, const double* p_old, const double* p) {
    if (!c || !p_old || !p) return HYPE_ERR_ARG;
    c->cur = 1;
    HYPE_CK(cudaMemcpyAsync(c->lv[0], p_old, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
    HYPE_CK(cudaMemcpyAsync(c->lv[1], p, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
    HYPE_CK(cudaStreamSynchronize(c->stream));
    return HYPE_OK;
}

extern "C" int hype_ctcs_get(hype_ctcs* c, double* p_old, double* p) {
    if (!c) return HYPE_ERR_ARG;
    if (p_old) HYPE_CK(cudaMemcpyAsync(p_old, c->lv[(c->cur + 2) % 3], sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
    if (p) HYPE_CK(cudaMemcpyAsync(p, c->lv[c->cur], sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
    HYPE_CK(cudaStreamSynchronize(c->stream));
    return HYPE_OK;
}

extern "C" double* hype_ctcs_level_device(hype_ctcs* c, int which) {
    if (!c) return nullptr;
    return which == 0 ? c->lv[c->cur] : c->lv[(c->cur + 2) % 3];
}

extern "C" int hype_ctcs_sync(hype_ctcs* c) {
    if (!c) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(c->stream));
    return HYPE_OK;
}

// Source(t) of 3d/ctcs/point_source/wave.c:232-238 (and 2d/ctcs/line_source/wave.c:213-219)
static double ricker(double t, double f0) {
    double t0 = 4.0 / f0;
    return -2.0 * (t - t0) * f0 * f0 * exp(-1.0 * f0 * f0 * (t - t0) * (t - t0));
}

static const int kChunk = 30;  // steps per captured graph (a multiple of the 3-level rotation)

static int build_chunk(hype_ctcs* c, int phase) {
    cudaGraph_t graph;
    HYPE_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = HYPE_OK;
    for (int s = 0; s < kChunk && rc == HYPE_OK; ++s) rc = ctcs_launch(c, (phase + s) % 3);
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_last_error("cudaStreamEndCapture", e);
        return HYPE_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&c->chunk[phase], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        set_last_error("cudaGraphInstantiate", e);
        return HYPE_ERR_CUDA;
    }
    return HYPE_OK;
}

extern "C" int hype_ctcs_step(hype_ctcs* c, int nsteps, int it0, double* receiver) {
    if (!c || nsteps < 0) return HYPE_ERR_ARG;
    if (nsteps == 0) return HYPE_OK;
    const Grid& g = c->g;
    if ((g.src >= 0 || g.rec >= 0) && nsteps > c->cap) {
        cudaFree(c->srcv);
        cudaFree(c->recv);
        c->srcv = c->recv = nullptr;
        HYPE_CK(cudaMalloc((void**)&c->srcv, sizeof(double) * nsteps));
        HYPE_CK(cudaMalloc((void**)&c->recv, sizeof(double) * nsteps));
        c->cap = nsteps;
        for (int q = 0; q < 3; ++q)
            if (c->chunk[q]) {
                cudaGraphExecDestroy(c->chunk[q]);
                c->chunk[q] = nullptr;
            }
    }
    if (g.src >= 0) {
        std::vector<double> sv(nsteps);
        const double vol = g.dim == 3 ? c->p.dx * c->p.dy * c->p.dz : c->p.dx * c->p.dy;
        const double dt = c->p.dt;
        for (int s = 0; s < nsteps; ++s) sv[s] = ricker((it0 + s) * dt, c->p.f0) / vol * dt * dt;
        HYPE_CK(cudaMemcpyAsync(c->srcv, sv.data(), sizeof(double) * nsteps, cudaMemcpyHostToDevice, c->stream));
    }
    if (g.src >= 0 || g.rec >= 0) {
        DevStep z{0};
        HYPE_CK(cudaMemcpyAsync(c->st, &z, sizeof(z), cudaMemcpyHostToDevice, c->stream));
        HYPE_CK(cudaStreamSynchronize(c->stream));  // z lives on this stack frame
    }
    int s = 0;
    int rc;
    // whole chunks replay a captured graph; the remainder launches directly
    while (nsteps - s >= kChunk) {
        const int phase = c->cur;
        if (!c->chunk[phase] && (rc = build_chunk(c, phase))) return rc;
        HYPE_CK(cudaGraphLaunch(c->chunk[phase], c->stream));
        count_launch(kChunk * ((g.src >= 0 || g.rec >= 0) ? 2 : 1));
        c->cur = (c->cur + kChunk) % 3;
        s += kChunk;
    }
    for (; s < nsteps; ++s) {
        if ((rc = ctcs_launch(c, c->cur))) return rc;
        c->cur = (c->cur + 1) % 3;
    }
    if (receiver && g.rec >= 0) {
        HYPE_CK(cudaMemcpyAsync(receiver, c->recv, sizeof(double) * nsteps, cudaMemcpyDeviceToHost, c->stream));
        HYPE_CK(cudaStreamSynchronize(c->stream));
    }
    return HYPE_OK;
}
