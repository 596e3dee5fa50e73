// batch.cu -- many independent 2D CTCS acoustic instances of uneven size in
// one persistent launch per step over a tile work-list.
//
// Each instance is the 2nd-order point-source form of
// 2d/ctcs/line_source/wave.c:149-173 on a zero-Dirichlet grid, with the point
// source generalised to a Gaussian monopole s = exp(-|x-xs|^2/(2 sig^2)) sin(2 pi f t)
// added as c^2 dt^2 s.  The Gaussian is separable, so it is stored as two 1-D
// factors per instance (nx + ny doubles) instead of a field or an FP64 exp per
// node per step; sin(2 pi f t) is tabulated per step and instance.
//
// Work-list: (instance, tile origin) items; blocks stride over it, so the
// launch is sized to the GPU (a multiple of the SM count), not to the batch.
// A chunk of steps is captured once as a CUDA graph and replayed; the tile
// shape is chosen by timing candidates and cached per grid-shape signature.
//
// Scheduling: the instances are split by size into classes (equal counts, smallest
// first), each with its own stream, work-list and step counter; the classes' kernels
// carry descending launch priorities, smallest class highest, so the block scheduler
// serves the small instances' steps first and fills the SMs they leave idle with the
// larger classes' tiles.  Every instance's arithmetic is unchanged (the classes touch
// disjoint parts of the level pools), small instances finish early, and the
// completion time of each class is an event on the device timeline.
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <algorithm>
#include <string>
#include <vector>

#include "hype_common.cuh"

namespace hype {
namespace batch {

struct Inst {
    int nx, ny;
    long long off;   // offset of the instance in a level pool
    long long goff;  // offset of its Gaussian factors (gx: nx, then gy: ny)
    double a;        // (c0 dt / h)^2: weight of the neighbours
    double b;        // 2 - 4a: weight of the centre
    double k2;       // c0*c0*dt*dt
};

struct Work {
    int q, i0, j0, pad;
};

// One work item is a tile of TX x (TY R) nodes of one instance; thread (x, y) marches
// the R consecutive rows j0 + y R ... of column i0 + x, carrying the centre and
// north values from row to row (4 loads per node: north, west, east, p^{n-1}).  The
// item's instance record, its x source factor and the step's sin(2 pi f t) are read
// once per item.  On GB300 this update is bound by the FP64 pipe (1/64 of the FP32
// rate), not by HBM, so it is written with 6 FP64 operations per node:
//   p^{n+1} = (2 - 4a) p - p^{n-1} + a ((e + w) + (n + s)) + (k2 sin gx) gy,
// a = (c0 dt/h)^2, the same update as 2p - p^{n-1} + c0^2 dt^2 (lap_h p + s) up to
// rounding.
// the step index is the class's counter (advanced once per graph chunk) plus s_off
template <int TX, int TY, int R>
__global__ void __launch_bounds__(TX* TY) k_batch(const Inst* __restrict__ inst, const Work* __restrict__ work, int nwork,
                                                  const double* __restrict__ pold, const double* __restrict__ p,
                                                  double* __restrict__ pnew, const double* __restrict__ gauss,
                                                  const double* __restrict__ sinv, int ninst, const int* __restrict__ step,
                                                  int s_off) {
    const int s = *step + s_off;
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const Work wk = work[w];
        const Inst I = inst[wk.q];
        const int i = wk.i0 + (int)threadIdx.x, jb = wk.j0 + (int)threadIdx.y * R;
        if (i >= I.nx || jb >= I.ny) continue;
        const double* P = p + I.off;
        const double* PO = pold + I.off;
        double* PN = pnew + I.off;
        const double gxa = (I.k2 * sinv[(long long)s * ninst + wk.q]) * gauss[I.goff + i];
        const double* gy = gauss + I.goff + I.nx;
        long long o = (long long)jb * I.nx + i;
        double sv = jb > 0 ? P[o - I.nx] : 0.0;
        double c = P[o];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int j = jb + r;
            if (j < I.ny) {
                const double nv = j < I.ny - 1 ? P[o + I.nx] : 0.0;
                const double w_ = i > 0 ? P[o - 1] : 0.0;
                const double e_ = i < I.nx - 1 ? P[o + 1] : 0.0;
                const double nb = (e_ + w_) + (nv + sv);
                PN[o] = fma(gxa, gy[j], fma(I.a, nb, fma(I.b, c, -PO[o])));
                sv = c;
                c = nv;
                o += I.nx;
            }
        }
    }
}

__global__ void k_tick(int* step, int inc) { *step += inc; }

constexpr int kMaxClasses = 8;

}  // namespace batch
}  // namespace hype

using namespace hype;
using namespace hype::batch;

struct hype_batch {
    std::vector<hype_mono_instance> hi;
    std::vector<Inst> inst;
    long long pool = 0;  // nodes per level
    cudaStream_t stream = nullptr;
    Inst* d_inst = nullptr;
    double* lv[3] = {nullptr, nullptr, nullptr};
    int cur = 1;
    double* gauss = nullptr;
    double* sinv = nullptr;
    int sin_cap = 0;
    long long it = 0;  // global step counter of the instances (time t = it*dt)
    int* d_step = nullptr;  // one step counter per class
    int tx = 0, ty = 0;     // chosen tile
    // size classes: instance -> class, per class its stream, priority, work-list and graphs
    int ncls = 1;
    std::vector<int> cls;
    cudaStream_t cs[kMaxClasses] = {};
    int prio[kMaxClasses] = {};
    Work* d_work[kMaxClasses] = {};
    int nwork[kMaxClasses] = {};
    int grid[kMaxClasses] = {};
    cudaGraphExec_t chunk[kMaxClasses][3] = {};
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_done[kMaxClasses] = {};
    bool timed = false;  // the events hold the last hype_batch_step call
};

static const int kBatchChunk = 30;

typedef void (*BatchKernel)(const Inst*, const Work*, int, const double*, const double*, double*, const double*,
                            const double*, int, const int*, int);

// tile shapes (width x height in nodes) and their thread blocks: TX x TY threads,
// R rows per thread
struct TileCfg {
    int tx, ty;  // tile in nodes
    BatchKernel k;
    int threads_y;
};
static const TileCfg kTiles[] = {
    {32, 16, k_batch<32, 8, 2>, 8},    {32, 32, k_batch<32, 8, 4>, 8},     {32, 64, k_batch<32, 8, 8>, 8},
    {64, 16, k_batch<64, 4, 4>, 4},    {64, 32, k_batch<64, 4, 8>, 4},     {64, 64, k_batch<64, 4, 16>, 4},
    {128, 16, k_batch<128, 2, 8>, 2},  {128, 32, k_batch<128, 2, 16>, 2}, {256, 16, k_batch<256, 1, 16>, 1},
};

static const TileCfg* pick_tile(int tx, int ty) {
    for (const TileCfg& t : kTiles)
        if (t.tx == tx && t.ty == ty) return &t;
    return nullptr;
}

static void drop_graphs(hype_batch* b) {
    for (int c = 0; c < kMaxClasses; ++c)
        for (int q = 0; q < 3; ++q)
            if (b->chunk[c][q]) {
                cudaGraphExecDestroy(b->chunk[c][q]);
                b->chunk[c][q] = nullptr;
            }
}

static int build_worklist(hype_batch* b, int tx, int ty) {
    const TileCfg* tc = pick_tile(tx, ty);
    if (!tc) return HYPE_ERR_ARG;
    int dev = 0, sms = 0, per_sm = 0;
    HYPE_CK(cudaGetDevice(&dev));
    HYPE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    HYPE_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc->k, tx * tc->threads_y, 0));
    if (per_sm < 1) per_sm = 1;
    for (int c = 0; c < b->ncls; ++c) {
        std::vector<Work> w;
        for (size_t q = 0; q < b->inst.size(); ++q) {
            if (b->cls[q] != c) continue;
            for (int j0 = 0; j0 < b->inst[q].ny; j0 += ty)
                for (int i0 = 0; i0 < b->inst[q].nx; i0 += tx) w.push_back(Work{(int)q, i0, j0, 0});
        }
        cudaFree(b->d_work[c]);
        b->d_work[c] = nullptr;
        b->nwork[c] = (int)w.size();
        if (w.empty()) continue;
        HYPE_CK(cudaMalloc((void**)&b->d_work[c], sizeof(Work) * w.size()));
        HYPE_CK(cudaMemcpy(b->d_work[c], w.data(), sizeof(Work) * w.size(), cudaMemcpyHostToDevice));
        b->grid[c] = (int)std::min<long long>((long long)sms * per_sm, (long long)w.size());
    }
    b->tx = tx;
    b->ty = ty;
    drop_graphs(b);
    return HYPE_OK;
}

// class c's kernel for one step (step index = its counter + s_off), at the class's priority
static int class_launch(hype_batch* b, int c, int phase, int s_off) {
    const TileCfg* tc = pick_tile(b->tx, b->ty);
    const double* po = b->lv[(phase + 2) % 3];
    const double* pc = b->lv[phase];
    double* pn = b->lv[(phase + 1) % 3];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->grid[c]);
    cfg.blockDim = dim3(b->tx, tc->threads_y);
    cfg.stream = b->cs[c];
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributePriority;
    attr.val.priority = b->prio[c];
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    const Inst* di = b->d_inst;
    const Work* dw = b->d_work[c];
    const int nw = b->nwork[c], ni = (int)b->inst.size();
    const double* ga = b->gauss;
    const double* sv = b->sinv;
    const int* st = b->d_step + c;
    HYPE_CK(cudaLaunchKernelEx(&cfg, tc->k, di, dw, nw, po, pc, pn, ga, sv, ni, st, s_off));
    count_launch(1);
    return HYPE_OK;
}

static int class_tick(hype_batch* b, int c, int inc) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(1);
    cfg.stream = b->cs[c];
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributePriority;
    attr.val.priority = b->prio[c];
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    HYPE_CK(cudaLaunchKernelEx(&cfg, k_tick, b->d_step + c, inc));
    count_launch(1);
    return HYPE_OK;
}

// a chunk of kBatchChunk steps of class c starting at level phase, one graph
static int build_chunk(hype_batch* b, int c, int phase) {
    cudaGraph_t g;
    HYPE_CK(cudaStreamBeginCapture(b->cs[c], cudaStreamCaptureModeThreadLocal));
    const long long l0 = hype_launch_count();
    int rc = HYPE_OK;
    for (int s = 0; s < kBatchChunk && rc == HYPE_OK; ++s) rc = class_launch(b, c, (phase + s) % 3, s);
    if (rc == HYPE_OK) rc = class_tick(b, c, kBatchChunk);
    cudaError_t e = cudaStreamEndCapture(b->cs[c], &g);
    count_launch(-(hype_launch_count() - l0));  // captured, not launched
    if (rc) return rc;
    if (e != cudaSuccess) {
        set_last_error("cudaStreamEndCapture", e);
        return HYPE_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&b->chunk[c][phase], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_last_error("cudaGraphInstantiate", e);
        return HYPE_ERR_CUDA;
    }
    return HYPE_OK;
}

// sin(2 pi f t) per step and instance for the next nsteps steps
static int fill_sin(hype_batch* b, int nsteps) {
    const int ni = (int)b->inst.size();
    if (nsteps > b->sin_cap) {
        cudaFree(b->sinv);
        b->sinv = nullptr;
        HYPE_CK(cudaMalloc((void**)&b->sinv, sizeof(double) * (size_t)nsteps * ni));
        b->sin_cap = nsteps;
        drop_graphs(b);
    }
    std::vector<double> h((size_t)nsteps * ni);
    const double two_pi = 6.283185307179586;
    for (int s = 0; s < nsteps; ++s)
        for (int q = 0; q < ni; ++q) {
            const double t = (double)(b->it + s) * b->hi[q].dt;
            h[(size_t)s * ni + q] = sin(two_pi * b->hi[q].freq * t);
        }
    HYPE_CK(cudaMemcpyAsync(b->sinv, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, b->stream));
    HYPE_CK(cudaMemsetAsync(b->d_step, 0, sizeof(int) * kMaxClasses, b->stream));
    HYPE_CK(cudaStreamSynchronize(b->stream));
    return HYPE_OK;
}

// every class advances nsteps: the classes' streams start together after the call's start
// event and the library stream waits for all of them
static int run_steps(hype_batch* b, int nsteps, int graph) {
    int rc;
    if ((rc = fill_sin(b, nsteps))) return rc;
    HYPE_CK(cudaEventRecord(b->ev_start, b->stream));
    for (int c = 0; c < b->ncls; ++c) {
        HYPE_CK(cudaStreamWaitEvent(b->cs[c], b->ev_start, 0));
        if (b->nwork[c] > 0) {
            int s = 0, phase = b->cur;
            if (graph) {
                while (nsteps - s >= kBatchChunk) {
                    if (!b->chunk[c][phase] && (rc = build_chunk(b, c, phase))) return rc;
                    HYPE_CK(cudaGraphLaunch(b->chunk[c][phase], b->cs[c]));
                    count_launch(kBatchChunk + 1);
                    phase = (phase + kBatchChunk) % 3;
                    s += kBatchChunk;
                }
            }
            for (; s < nsteps; ++s) {
                if ((rc = class_launch(b, c, phase, 0))) return rc;
                if ((rc = class_tick(b, c, 1))) return rc;
                phase = (phase + 1) % 3;
            }
        }
        HYPE_CK(cudaEventRecord(b->ev_done[c], b->cs[c]));
        HYPE_CK(cudaStreamWaitEvent(b->stream, b->ev_done[c], 0));
    }
    b->cur = (int)((b->cur + nsteps) % 3);
    b->it += nsteps;
    b->timed = true;
    return HYPE_OK;
}

// instances into nclasses size classes of equal count (ties by index), smallest first;
// class c runs at the c-th highest stream priority the device offers
static int set_classes(hype_batch* b, int nclasses) {
    int least = 0, greatest = 0;
    HYPE_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int levels = least - greatest + 1;
    const int ni = (int)b->inst.size();
    int n = nclasses > 0 ? nclasses : std::min(levels, kMaxClasses);
    n = std::max(1, std::min(std::min(n, kMaxClasses), ni));
    HYPE_CK(cudaStreamSynchronize(b->stream));
    for (int c = 0; c < kMaxClasses; ++c)
        if (b->cs[c]) HYPE_CK(cudaStreamSynchronize(b->cs[c]));
    std::vector<int> order(ni);
    for (int q = 0; q < ni; ++q) order[q] = q;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return (long long)b->inst[x].nx * b->inst[x].ny < (long long)b->inst[y].nx * b->inst[y].ny;
    });
    b->cls.assign(ni, 0);
    for (int r = 0; r < ni; ++r) b->cls[order[r]] = (int)((long long)r * n / ni);
    b->ncls = n;
    for (int c = 0; c < n; ++c) {
        // smallest class: the greatest priority (numerically lowest); the rest spread over the range
        b->prio[c] = n == 1 ? least : greatest + (int)((long long)c * (levels - 1) / (n - 1));
        if (!b->cs[c]) HYPE_CK(cudaStreamCreateWithPriority(&b->cs[c], cudaStreamNonBlocking, b->prio[c]));
        if (!b->ev_done[c]) HYPE_CK(cudaEventCreate(&b->ev_done[c]));
    }
    b->timed = false;
    return b->tx ? build_worklist(b, b->tx, b->ty) : HYPE_OK;
}

// ------------------------------------------------------------------ autotuner
static std::string shape_key(const hype_batch* b) {
    std::vector<std::pair<int, int>> s;
    for (auto& i : b->inst) s.push_back({i.nx, i.ny});
    std::sort(s.begin(), s.end());
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over the sorted shapes
    for (auto& x : s) {
        h = (h ^ (unsigned)x.first) * 1099511628211ull;
        h = (h ^ (unsigned)x.second) * 1099511628211ull;
    }
    char buf[64];
    snprintf(buf, sizeof(buf), "v2-%zu-%016llx", s.size(), h);
    return buf;
}

static std::string cache_path() {
    const char* e = getenv("HYPE_TUNE_CACHE");
    if (e && *e) return e;
    const char* home = getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/hype_gb300_tiles.txt";
}

static bool cache_lookup(const std::string& key, int* tx, int* ty) {
    FILE* f = fopen(cache_path().c_str(), "r");
    if (!f) return false;
    char line[256], k[128];
    int a, c;
    bool found = false;
    while (fgets(line, sizeof(line), f))
        if (sscanf(line, "%127s %d %d", k, &a, &c) == 3 && key == k && pick_tile(a, c)) {
            *tx = a;
            *ty = c;
            found = true;
        }
    fclose(f);
    return found;
}

static void cache_store(const std::string& key, int tx, int ty) {
    const std::string p = cache_path();
    for (size_t q = 1; q < p.size(); ++q)  // create missing parent directories
        if (p[q] == '/') mkdir(p.substr(0, q).c_str(), 0755);
    FILE* f = fopen(p.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s %d %d\n", key.c_str(), tx, ty);
    fclose(f);
}

static int autotune(hype_batch* b) {
    int tx = 0, ty = 0;
    const std::string key = shape_key(b);
    if (cache_lookup(key, &tx, &ty)) return build_worklist(b, tx, ty);
    // save levels and step counter: tuning steps are undone afterwards
    const size_t bytes = sizeof(double) * (size_t)b->pool;
    double* save[3];
    for (int q = 0; q < 3; ++q) {
        HYPE_CK(cudaMalloc((void**)&save[q], bytes));
        HYPE_CK(cudaMemcpy(save[q], b->lv[q], bytes, cudaMemcpyDeviceToDevice));
    }
    const int cur0 = b->cur;
    const long long it0 = b->it;
    cudaEvent_t e0, e1;
    HYPE_CK(cudaEventCreate(&e0));
    HYPE_CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int bx = 32, by = 32;
    int rc = HYPE_OK;
    for (const TileCfg& t : kTiles) {
        if ((rc = build_worklist(b, t.tx, t.ty))) break;
        if ((rc = run_steps(b, 3, 0))) break;  // warm-up
        HYPE_CK(cudaEventRecord(e0, b->stream));
        if ((rc = run_steps(b, 12, 0))) break;
        HYPE_CK(cudaEventRecord(e1, b->stream));
        HYPE_CK(cudaEventSynchronize(e1));
        float ms = 0;
        HYPE_CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            bx = t.tx;
            by = t.ty;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int q = 0; q < 3; ++q) {
        cudaMemcpy(b->lv[q], save[q], bytes, cudaMemcpyDeviceToDevice);
        cudaFree(save[q]);
    }
    b->cur = cur0;
    b->it = it0;
    if (rc) return rc;
    cache_store(key, bx, by);
    return build_worklist(b, bx, by);
}

// ------------------------------------------------------------------ C ABI
extern "C" int hype_batch_create(int ninst, const hype_mono_instance* in, hype_batch** out) {
    if (ninst < 1 || !in || !out) return HYPE_ERR_ARG;
    *out = nullptr;
    hype_batch* b = new hype_batch();
    b->hi.assign(in, in + ninst);
    long long off = 0, goff = 0;
    for (int q = 0; q < ninst; ++q) {
        const hype_mono_instance& m = in[q];
        if (m.nx < 3 || m.ny < 3 || !(m.h > 0) || !(m.dt > 0) || !(m.sigma > 0)) {
            delete b;
            return HYPE_ERR_ARG;
        }
        Inst I;
        I.nx = m.nx;
        I.ny = m.ny;
        I.off = off;
        I.goff = goff;
        I.k2 = m.c0 * m.c0 * m.dt * m.dt;
        I.a = I.k2 / (m.h * m.h);
        I.b = 2.0 - 4.0 * I.a;
        b->inst.push_back(I);
        off += ((long long)m.nx * m.ny + 31) / 32 * 32;  // 256-byte aligned instance starts
        goff += m.nx + m.ny;
    }
    b->pool = off;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMalloc((void**)&b->lv[q], sizeof(double) * off);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = cudaMemset(b->lv[q], 0, sizeof(double) * off);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_inst, sizeof(Inst) * ninst);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_inst, b->inst.data(), sizeof(Inst) * ninst, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->gauss, sizeof(double) * goff);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_step, sizeof(int) * kMaxClasses);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_start);
    if (e == cudaSuccess) {
        // separable Gaussian factors exp(-(x-xs)^2/(2 sig^2)), exp(-(y-ys)^2/(2 sig^2))
        std::vector<double> g(goff);
        for (int q = 0; q < ninst; ++q) {
            const hype_mono_instance& m = in[q];
            const double r2s = 1.0 / (2.0 * m.sigma * m.sigma);
            for (int i = 0; i < m.nx; ++i) {
                const double d = (m.xmin + i * m.h) - m.xs;
                g[b->inst[q].goff + i] = exp(-(d * d) * r2s);
            }
            for (int j = 0; j < m.ny; ++j) {
                const double d = (m.ymin + j * m.h) - m.ys;
                g[b->inst[q].goff + m.nx + j] = exp(-(d * d) * r2s);
            }
        }
        e = cudaMemcpy(b->gauss, g.data(), sizeof(double) * goff, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        set_last_error("hype_batch_create", e);
        hype_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? HYPE_ERR_NOMEM : HYPE_ERR_CUDA;
    }
    int rc = set_classes(b, 0);
    if (rc == HYPE_OK) rc = build_worklist(b, 32, 32);
    if (rc) {
        hype_batch_destroy(b);
        return rc;
    }
    *out = b;
    return HYPE_OK;
}

extern "C" void hype_batch_destroy(hype_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    for (int q = 0; q < 3; ++q) cudaFree(b->lv[q]);
    cudaFree(b->d_inst);
    cudaFree(b->gauss);
    cudaFree(b->sinv);
    cudaFree(b->d_step);
    for (int c = 0; c < kMaxClasses; ++c) {
        if (b->cs[c]) cudaStreamSynchronize(b->cs[c]);
        cudaFree(b->d_work[c]);
        if (b->cs[c]) cudaStreamDestroy(b->cs[c]);
        if (b->ev_done[c]) cudaEventDestroy(b->ev_done[c]);
    }
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int hype_batch_set_tile(hype_batch* b, int tx, int ty) {
    if (!b) return HYPE_ERR_ARG;
    if (tx == 0 && ty == 0) return autotune(b);
    return build_worklist(b, tx, ty);
}

extern "C" int hype_batch_get_tile(const hype_batch* b, int* tx, int* ty) {
    if (!b || !tx || !ty) return HYPE_ERR_ARG;
    *tx = b->tx;
    *ty = b->ty;
    return HYPE_OK;
}

extern "C" int hype_batch_set(hype_batch* b, int q, const double* p_old, const double* p) {
    if (!b || q < 0 || q >= (int)b->inst.size() || !p_old || !p) return HYPE_ERR_ARG;
    const Inst& I = b->inst[q];
    const size_t bytes = sizeof(double) * (size_t)I.nx * I.ny;
    HYPE_CK(cudaMemcpyAsync(b->lv[(b->cur + 2) % 3] + I.off, p_old, bytes, cudaMemcpyHostToDevice, b->stream));
    HYPE_CK(cudaMemcpyAsync(b->lv[b->cur] + I.off, p, bytes, cudaMemcpyHostToDevice, b->stream));
    HYPE_CK(cudaStreamSynchronize(b->stream));
    return HYPE_OK;
}

extern "C" int hype_batch_get(hype_batch* b, int q, double* p_old, double* p) {
    if (!b || q < 0 || q >= (int)b->inst.size()) return HYPE_ERR_ARG;
    const Inst& I = b->inst[q];
    const size_t bytes = sizeof(double) * (size_t)I.nx * I.ny;
    if (p_old) HYPE_CK(cudaMemcpyAsync(p_old, b->lv[(b->cur + 2) % 3] + I.off, bytes, cudaMemcpyDeviceToHost, b->stream));
    if (p) HYPE_CK(cudaMemcpyAsync(p, b->lv[b->cur] + I.off, bytes, cudaMemcpyDeviceToHost, b->stream));
    HYPE_CK(cudaStreamSynchronize(b->stream));
    return HYPE_OK;
}

extern "C" int hype_batch_step(hype_batch* b, int nsteps, int graph) {
    if (!b || nsteps < 0) return HYPE_ERR_ARG;
    return run_steps(b, nsteps, graph);
}

extern "C" int hype_batch_set_classes(hype_batch* b, int nclasses) {
    if (!b || nclasses < 0) return HYPE_ERR_ARG;
    return set_classes(b, nclasses);
}

extern "C" int hype_batch_get_classes(const hype_batch* b, int* nclasses, int* cls) {
    if (!b || !nclasses) return HYPE_ERR_ARG;
    *nclasses = b->ncls;
    if (cls)
        for (size_t q = 0; q < b->cls.size(); ++q) cls[q] = b->cls[q];
    return HYPE_OK;
}

extern "C" int hype_batch_instance_times(hype_batch* b, double* seconds) {
    if (!b || !seconds || !b->timed) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(b->stream));
    double t[kMaxClasses];
    for (int c = 0; c < b->ncls; ++c) {
        float ms = 0.0f;
        HYPE_CK(cudaEventElapsedTime(&ms, b->ev_start, b->ev_done[c]));
        t[c] = 1e-3 * ms;
    }
    for (size_t q = 0; q < b->inst.size(); ++q) seconds[q] = t[b->cls[q]];
    return HYPE_OK;
}

extern "C" int hype_batch_sync(hype_batch* b) {
    if (!b) return HYPE_ERR_ARG;
    HYPE_CK(cudaStreamSynchronize(b->stream));
    return HYPE_OK;
}
