/*
 * petsc_shim.c -- single-rank implementation of the PETSc subset declared in
 * petsc_shim.h.  TEST INFRASTRUCTURE ONLY (see the header for the semantics
 * this restates and where they come from).
 */
#include "petsc_shim.h"

#include <setjmp.h>
#include <time.h>
#include <stdint.h>

int shim_abort_count = 0;
static jmp_buf* shim_abort_jmp = NULL;
static int shim_quiet = -1;

static int quiet(void) {
    if (shim_quiet < 0) {
        const char* q = getenv("HYPE_SHIM_VERBOSE");
        shim_quiet = (q && q[0] == '1') ? 0 : 1;
    }
    return shim_quiet;
}

void shim_set_abort_jump(void* p) { shim_abort_jmp = (jmp_buf*)p; }

int shim_seterr(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[petsc-shim] error: ");
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    return 1;
}

/* ------------------------------------------------------------------ sys */
PetscErrorCode PetscInitialize(int* argc, char*** argv, const char* file, const char* help) {
    (void)argc; (void)argv; (void)file; (void)help;
    return 0;
}
PetscErrorCode PetscFinalize(void) { return 0; }
PetscErrorCode PetscPrintf(MPI_Comm comm, const char* fmt, ...) {
    (void)comm;
    if (quiet()) return 0;
    va_list ap;
    va_start(ap, fmt);
    vprintf(fmt, ap);
    va_end(ap);
    return 0;
}
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE* f, const char* fmt, ...) {
    (void)comm;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(f, fmt, ap);
    va_end(ap);
    return 0;
}
PetscErrorCode PetscTime(PetscLogDouble* t) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    *t = (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
    return 0;
}
PetscErrorCode PetscObjectSetName(PetscObject obj, const char* name) {
    (void)obj; (void)name;
    return 0;
}
MPI_Comm PetscObjectComm(PetscObject obj) { (void)obj; return PETSC_COMM_WORLD; }
int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c;
    size_t sz = (t == MPIU_INT) ? sizeof(int) : sizeof(double);
    if (in != out) memmove(out, in, sz * (size_t)n);
    return 0;
}
int MPI_Abort(MPI_Comm c, int code) {
    (void)c;
    shim_abort_count++;
    if (shim_abort_jmp) longjmp(*shim_abort_jmp, code ? code : 1);
    fprintf(stderr, "[petsc-shim] MPI_Abort(%d)\n", code);
    exit(code ? code : 1);
}

/* ------------------------------------------------------------------ Vec */
static Vec vec_new(DM dm, int local, long n) {
    Vec v = (Vec)calloc(1, sizeof(struct _p_Vec));
    v->dm = dm;
    v->local = local;
    v->n = n;
    v->a = (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    return v;
}

PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec* v) { (void)c; *v = vec_new(NULL, 0, n); return 0; }
PetscErrorCode VecDuplicate(Vec v, Vec* w) { *w = vec_new(v->dm, v->local, v->n); return 0; }
PetscErrorCode VecDestroy(Vec* v) {
    if (!v || !*v) return 0;
    free((*v)->a);
    free((*v)->view);
    free(*v);
    *v = NULL;
    return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar a) {
    for (long i = 0; i < v->n; ++i) v->a[i] = a;
    return 0;
}
PetscErrorCode VecCopy(Vec x, Vec y) {
    if (x != y) memcpy(y->a, x->a, sizeof(double) * (size_t)x->n);
    return 0;
}
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
    for (long i = 0; i < y->n; ++i) y->a[i] = y->a[i] + a * x->a[i];
    return 0;
}
PetscErrorCode VecAYPX(Vec y, PetscScalar b, Vec x) {
    for (long i = 0; i < y->n; ++i) y->a[i] = x->a[i] + b * y->a[i];
    return 0;
}
PetscErrorCode VecAXPBYPCZ(Vec z, PetscScalar a, PetscScalar b, PetscScalar c, Vec x, Vec y) {
    for (long i = 0; i < z->n; ++i) z->a[i] = a * x->a[i] + b * y->a[i] + c * z->a[i];
    return 0;
}
PetscErrorCode VecScale(Vec v, PetscScalar a) {
    for (long i = 0; i < v->n; ++i) v->a[i] *= a;
    return 0;
}
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal* r) {
    double s = 0.0;
    if (t == NORM_INFINITY) {
        for (long i = 0; i < v->n; ++i) if (fabs(v->a[i]) > s) s = fabs(v->a[i]);
    } else if (t == NORM_1) {
        for (long i = 0; i < v->n; ++i) s += fabs(v->a[i]);
    } else {
        for (long i = 0; i < v->n; ++i) s += v->a[i] * v->a[i];
        s = sqrt(s);
    }
    *r = s;
    return 0;
}
PetscErrorCode VecStrideNorm(Vec v, PetscInt s, NormType t, PetscReal* r) {
    int dof = v->dm ? v->dm->dof : 1;
    double acc = 0.0;
    for (long i = s; i < v->n; i += dof) {
        double a = v->a[i];
        if (t == NORM_INFINITY) { if (fabs(a) > acc) acc = fabs(a); }
        else if (t == NORM_1) acc += fabs(a);
        else acc += a * a;
    }
    *r = (t == NORM_2) ? sqrt(acc) : acc;
    return 0;
}
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a) { (void)v; *a = NULL; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar** a) { (void)v; *a = NULL; return 0; }
PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n) { *n = (PetscInt)v->n; return 0; }
PetscErrorCode VecGetSize(Vec v, PetscInt* n) { *n = (PetscInt)v->n; return 0; }

/* ------------------------------------------------------------------ viewers */
struct _p_Viewer {
    FILE* f;
    int binary;
    int mode;
};

static PetscViewer viewer_open(const char* name, int binary, int mode) {
    PetscViewer v = (PetscViewer)calloc(1, sizeof(struct _p_Viewer));
    v->binary = binary;
    v->mode = mode;
    const char* w = getenv("HYPE_SHIM_WRITE_FILES");
    if (binary && w && w[0] == '1') v->f = fopen(name, mode == FILE_MODE_READ ? "rb" : "wb");
    return v;
}
PetscErrorCode PetscViewerVTKOpen(MPI_Comm c, const char* name, PetscFileMode m, PetscViewer* v) {
    (void)c; *v = viewer_open(name, 0, m); return 0;
}
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm c, const char* name, PetscViewer* v) {
    (void)c; *v = viewer_open(name, 0, FILE_MODE_WRITE); return 0;
}
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char* name, PetscFileMode m, PetscViewer* v) {
    (void)c; *v = viewer_open(name, 1, m); return 0;
}
PetscErrorCode PetscViewerPushFormat(PetscViewer v, PetscViewerFormat f) { (void)v; (void)f; return 0; }
PetscErrorCode PetscViewerPopFormat(PetscViewer v) { (void)v; return 0; }
PetscErrorCode PetscViewerDestroy(PetscViewer* v) {
    if (!v || !*v) return 0;
    if ((*v)->f) fclose((*v)->f);
    free(*v);
    *v = NULL;
    return 0;
}
PetscErrorCode DMView(DM da, PetscViewer v) { (void)da; (void)v; return 0; }

/* PETSc binary Vec record: int32 class id 1211214, int32 length, then the
 * entries as big-endian IEEE doubles (PETSc manual, PetscViewerBinaryOpen). */
static void put_be32(FILE* f, int32_t x) {
    unsigned char b[4] = {(unsigned char)(x >> 24), (unsigned char)(x >> 16), (unsigned char)(x >> 8), (unsigned char)x};
    fwrite(b, 1, 4, f);
}
PetscErrorCode VecView(Vec x, PetscViewer v) {
    if (!v || !v->binary || !v->f) return 0;
    put_be32(v->f, 1211214);
    put_be32(v->f, (int32_t)x->n);
    for (long i = 0; i < x->n; ++i) {
        uint64_t u;
        memcpy(&u, &x->a[i], 8);
        unsigned char b[8];
        for (int k = 0; k < 8; ++k) b[k] = (unsigned char)(u >> (56 - 8 * k));
        fwrite(b, 1, 8, v->f);
    }
    return 0;
}
PetscErrorCode VecLoad(Vec x, PetscViewer v) {
    if (!v || !v->binary || !v->f) return 1;
    unsigned char h[8];
    if (fread(h, 1, 8, v->f) != 8) return 1;
    int32_t cid = (int32_t)((h[0] << 24) | (h[1] << 16) | (h[2] << 8) | h[3]);
    int32_t n = (int32_t)((h[4] << 24) | (h[5] << 16) | (h[6] << 8) | h[7]);
    if (cid != 1211214 || n != x->n) return 1;
    for (long i = 0; i < x->n; ++i) {
        unsigned char b[8];
        if (fread(b, 1, 8, v->f) != 8) return 1;
        uint64_t u = 0;
        for (int k = 0; k < 8; ++k) u = (u << 8) | b[k];
        memcpy(&x->a[i], &u, 8);
    }
    return 0;
}

/* ------------------------------------------------------------------ DMDA */
static DM dm_new(int dim, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz, DMDAStencilType st, int M, int N, int P,
                 int dof, int sw) {
    DM d = (DM)calloc(1, sizeof(struct _p_DM));
    d->dim = dim; d->bx = bx; d->by = by; d->bz = bz; d->st = st;
    d->M = M; d->N = N; d->P = P; d->dof = dof; d->sw = sw;
    d->xs = d->ys = d->zs = 0;
    d->xm = M; d->ym = N; d->zm = P;
    int sx = (bx == DM_BOUNDARY_NONE) ? 0 : sw;
    int sy = (dim >= 2 && by != DM_BOUNDARY_NONE) ? sw : 0;
    int sz = (dim >= 3 && bz != DM_BOUNDARY_NONE) ? sw : 0;
    d->gxs = -sx; d->gxm = M + 2 * sx;
    d->gys = -sy; d->gym = N + 2 * sy;
    d->gzs = -sz; d->gzm = P + 2 * sz;
    return d;
}

PetscErrorCode DMDACreate1d(MPI_Comm c, DMBoundaryType bx, PetscInt M, PetscInt dof, PetscInt sw, const PetscInt lx[], DM* da) {
    (void)c; (void)lx;
    *da = dm_new(1, bx, DM_BOUNDARY_NONE, DM_BOUNDARY_NONE, DMDA_STENCIL_STAR, M, 1, 1, dof, sw);
    return 0;
}
PetscErrorCode DMDACreate2d(MPI_Comm c, DMBoundaryType bx, DMBoundaryType by, DMDAStencilType st, PetscInt M, PetscInt N,
                            PetscInt m, PetscInt n, PetscInt dof, PetscInt sw, const PetscInt lx[], const PetscInt ly[], DM* da) {
    (void)c; (void)m; (void)n; (void)lx; (void)ly;
    *da = dm_new(2, bx, by, DM_BOUNDARY_NONE, st, M, N, 1, dof, sw);
    return 0;
}
PetscErrorCode DMDACreate3d(MPI_Comm c, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz, DMDAStencilType st, PetscInt M,
                            PetscInt N, PetscInt P, PetscInt m, PetscInt n, PetscInt p, PetscInt dof, PetscInt sw,
                            const PetscInt lx[], const PetscInt ly[], const PetscInt lz[], DM* da) {
    (void)c; (void)m; (void)n; (void)p; (void)lx; (void)ly; (void)lz;
    *da = dm_new(3, bx, by, bz, st, M, N, P, dof, sw);
    return 0;
}
PetscErrorCode DMSetUp(DM da) { (void)da; return 0; }
PetscErrorCode DMSetFromOptions(DM da) { (void)da; return 0; }
PetscErrorCode DMDestroy(DM* da) {
    if (!da || !*da) return 0;
    for (int i = 0; i < 8; ++i) VecDestroy(&(*da)->localpool[i]);
    VecDestroy(&(*da)->coords);
    if ((*da)->cdm) DMDestroy(&(*da)->cdm);
    free(*da);
    *da = NULL;
    return 0;
}
PetscErrorCode DMDAGetCorners(DM d, PetscInt* xs, PetscInt* ys, PetscInt* zs, PetscInt* xm, PetscInt* ym, PetscInt* zm) {
    if (xs) *xs = d->xs;
    if (ys) *ys = d->ys;
    if (zs) *zs = d->zs;
    if (xm) *xm = d->xm;
    if (ym) *ym = d->ym;
    if (zm) *zm = d->zm;
    return 0;
}
PetscErrorCode DMDAGetGhostCorners(DM d, PetscInt* xs, PetscInt* ys, PetscInt* zs, PetscInt* xm, PetscInt* ym, PetscInt* zm) {
    if (xs) *xs = d->gxs;
    if (ys) *ys = d->gys;
    if (zs) *zs = d->gzs;
    if (xm) *xm = d->gxm;
    if (ym) *ym = d->gym;
    if (zm) *zm = d->gzm;
    return 0;
}
PetscErrorCode DMDAGetInfo(DM d, PetscInt* dim, PetscInt* M, PetscInt* N, PetscInt* P, PetscInt* m, PetscInt* n, PetscInt* p,
                           PetscInt* dof, PetscInt* s, DMBoundaryType* bx, DMBoundaryType* by, DMBoundaryType* bz,
                           DMDAStencilType* st) {
    if (dim) *dim = d->dim;
    if (M) *M = d->M;
    if (N) *N = d->N;
    if (P) *P = d->P;
    if (m) *m = 1;
    if (n) *n = 1;
    if (p) *p = 1;
    if (dof) *dof = d->dof;
    if (s) *s = d->sw;
    if (bx) *bx = d->bx;
    if (by) *by = d->by;
    if (bz) *bz = d->bz;
    if (st) *st = d->st;
    return 0;
}
static long local_len(DM d) { return (long)d->gxm * d->gym * d->gzm * d->dof; }
static long global_len(DM d) { return (long)d->xm * d->ym * d->zm * d->dof; }

PetscErrorCode DMCreateGlobalVector(DM d, Vec* v) { *v = vec_new(d, 0, global_len(d)); return 0; }
PetscErrorCode DMCreateLocalVector(DM d, Vec* v) { *v = vec_new(d, 1, local_len(d)); return 0; }
PetscErrorCode DMGetLocalVector(DM d, Vec* v) {
    for (int i = 0; i < 8; ++i) {
        if (!d->localused[i]) {
            if (!d->localpool[i]) d->localpool[i] = vec_new(d, 1, local_len(d));
            d->localused[i] = 1;
            *v = d->localpool[i];
            return 0;
        }
    }
    return shim_seterr("too many local work vectors\n");
}
PetscErrorCode DMRestoreLocalVector(DM d, Vec* v) {
    for (int i = 0; i < 8; ++i)
        if (d->localpool[i] == *v) d->localused[i] = 0;
    *v = NULL;
    return 0;
}
PetscErrorCode DMGetGlobalVector(DM d, Vec* v) { return DMCreateGlobalVector(d, v); }
PetscErrorCode DMRestoreGlobalVector(DM d, Vec* v) { (void)d; return VecDestroy(v); }

static int wrap(int i, int n, DMBoundaryType b, int* ok) {
    if (i >= 0 && i < n) return i;
    if (b == DM_BOUNDARY_PERIODIC) return ((i % n) + n) % n;
    *ok = 0;
    return 0;
}

PetscErrorCode DMGlobalToLocalBegin(DM d, Vec g, InsertMode mode, Vec l) {
    (void)mode;
    const int dof = d->dof;
    for (int k = d->gzs; k < d->gzs + d->gzm; ++k)
        for (int j = d->gys; j < d->gys + d->gym; ++j)
            for (int i = d->gxs; i < d->gxs + d->gxm; ++i) {
                int ok = 1;
                int gi = wrap(i, d->M, d->bx, &ok);
                int gj = (d->dim >= 2) ? wrap(j, d->N, d->by, &ok) : 0;
                int gk = (d->dim >= 3) ? wrap(k, d->P, d->bz, &ok) : 0;
                if (!ok) continue; /* exterior ghost of a non-periodic boundary: untouched */
                long lo = (((long)(k - d->gzs) * d->gym + (j - d->gys)) * d->gxm + (i - d->gxs)) * dof;
                long go = (((long)gk * d->N + gj) * d->M + gi) * dof;
                memcpy(&l->a[lo], &g->a[go], sizeof(double) * (size_t)dof);
            }
    return 0;
}
PetscErrorCode DMGlobalToLocalEnd(DM d, Vec g, InsertMode mode, Vec l) { (void)d; (void)g; (void)mode; (void)l; return 0; }

PetscErrorCode DMDAVecGetArray(DM d, Vec v, void* array) {
    const int dof = d->dof;
    int X = v->local ? d->gxm : d->xm, Y = v->local ? d->gym : d->ym, Z = v->local ? d->gzm : d->zm;
    int x0 = v->local ? d->gxs : d->xs, y0 = v->local ? d->gys : d->ys, z0 = v->local ? d->gzs : d->zs;
    free(v->view);
    if (d->dim == 1) {
        v->view = NULL;
        *(void**)array = (void*)(v->a - (long)x0 * dof);
        return 0;
    }
    if (d->dim == 2) {
        double** rows = (double**)malloc(sizeof(double*) * (size_t)Y);
        for (int jj = 0; jj < Y; ++jj) rows[jj] = v->a + ((long)jj * X - x0) * dof;
        v->view = rows;
        *(void**)array = (void*)(rows - y0);
        return 0;
    }
    size_t nrows = (size_t)Y * (size_t)Z;
    char* mem = (char*)malloc(sizeof(double*) * nrows + sizeof(double**) * (size_t)Z);
    double** rows = (double**)mem;
    double*** planes = (double***)(mem + sizeof(double*) * nrows);
    for (int kk = 0; kk < Z; ++kk)
        for (int jj = 0; jj < Y; ++jj) rows[(size_t)kk * Y + jj] = v->a + (((long)kk * Y + jj) * X - x0) * dof;
    for (int kk = 0; kk < Z; ++kk) planes[kk] = rows + (size_t)kk * Y - y0;
    v->view = mem;
    *(void**)array = (void*)(planes - z0);
    return 0;
}
PetscErrorCode DMDAVecRestoreArray(DM d, Vec v, void* array) { (void)d; (void)v; *(void**)array = NULL; return 0; }
PetscErrorCode DMDAVecGetArrayRead(DM d, Vec v, void* array) { return DMDAVecGetArray(d, v, array); }
PetscErrorCode DMDAVecRestoreArrayRead(DM d, Vec v, void* array) { return DMDAVecRestoreArray(d, v, array); }

/* uniform coordinates (PETSc manual, DMDASetUniformCoordinates): node i of an axis is
 * x0 + i h with h = (x1 - x0)/M on a periodic axis and (x1 - x0)/(M - 1) otherwise,
 * stored interleaved (dof = dim) in a global vector of a coordinate DMDA */
PetscErrorCode DMDASetUniformCoordinates(DM d, PetscReal x0, PetscReal x1, PetscReal y0, PetscReal y1, PetscReal z0, PetscReal z1) {
    d->cmin[0] = x0; d->cmax[0] = x1;
    d->cmin[1] = y0; d->cmax[1] = y1;
    d->cmin[2] = z0; d->cmax[2] = z1;
    if (d->cdm) DMDestroy(&d->cdm);
    VecDestroy(&d->coords);
    d->cdm = dm_new(d->dim, d->bx, d->by, d->bz, d->st, d->M, d->N, d->P, d->dim, d->sw);
    DMCreateGlobalVector(d->cdm, &d->coords);
    const int n[3] = {d->M, d->N, d->P};
    const DMBoundaryType b[3] = {d->bx, d->by, d->bz};
    double h[3];
    for (int a = 0; a < 3; ++a) {
        const double L = d->cmax[a] - d->cmin[a];
        h[a] = (b[a] == DM_BOUNDARY_PERIODIC) ? L / n[a] : (n[a] > 1 ? L / (n[a] - 1) : 0.0);
    }
    long q = 0;
    for (int k = 0; k < (d->dim >= 3 ? d->P : 1); ++k)
        for (int j = 0; j < (d->dim >= 2 ? d->N : 1); ++j)
            for (int i = 0; i < d->M; ++i) {
                d->coords->a[q++] = d->cmin[0] + i * h[0];
                if (d->dim >= 2) d->coords->a[q++] = d->cmin[1] + j * h[1];
                if (d->dim >= 3) d->coords->a[q++] = d->cmin[2] + k * h[2];
            }
    return 0;
}
PetscErrorCode DMGetCoordinateDM(DM d, DM* cda) { *cda = d->cdm ? d->cdm : d; return 0; }
PetscErrorCode DMGetCoordinates(DM d, Vec* c) { *c = d->coords; return 0; }
PetscErrorCode DMGetCoordinatesLocal(DM d, Vec* c) { *c = d->coords; return 0; }
PetscErrorCode DMDASetFieldName(DM d, PetscInt nf, const char* name) { (void)d; (void)nf; (void)name; return 0; }

/* ------------------------------------------------------------------ TS */
PetscErrorCode TSCreate(MPI_Comm c, TS* ts) {
    (void)c;
    TS t = (TS)calloc(1, sizeof(struct _p_TS));
    t->max_time = 1e300;
    t->max_steps = 2147483647;
    t->nstages = 0;
    strcpy(t->type, "euler");
    strcpy(t->ssptype, "rks2");
    *ts = t;
    return 0;
}
PetscErrorCode TSDestroy(TS* ts) { if (ts && *ts) { free(*ts); *ts = NULL; } return 0; }
PetscErrorCode TSSetProblemType(TS ts, TSProblemType t) { (void)ts; (void)t; return 0; }
PetscErrorCode TSSetDM(TS ts, DM dm) { ts->dm = dm; return 0; }
PetscErrorCode TSGetDM(TS ts, DM* dm) { *dm = ts->dm; return 0; }
PetscErrorCode TSSetRHSFunction(TS ts, Vec r, TSRHSFunctionFn f, void* ctx) { (void)r; ts->rhs = f; ts->rhsctx = ctx; return 0; }
PetscErrorCode TSSetStepNumber(TS ts, PetscInt s) { ts->steps = s; return 0; }
PetscErrorCode TSGetStepNumber(TS ts, PetscInt* s) { *s = ts->steps; return 0; }
PetscErrorCode TSSetTime(TS ts, PetscReal t) { ts->t = t; return 0; }
PetscErrorCode TSGetTime(TS ts, PetscReal* t) { *t = ts->t; return 0; }
PetscErrorCode TSSetTimeStep(TS ts, PetscReal dt) { ts->dt = dt; return 0; }
PetscErrorCode TSGetTimeStep(TS ts, PetscReal* dt) { *dt = ts->dt; return 0; }
PetscErrorCode TSMonitorSet(TS ts, TSMonitorFn f, void* ctx, void* destroy) { (void)destroy; ts->mon = f; ts->monctx = ctx; return 0; }
PetscErrorCode TSSetMaxTime(TS ts, PetscReal t) { ts->max_time = t; return 0; }
PetscErrorCode TSSetMaxSteps(TS ts, PetscInt n) { ts->max_steps = n; return 0; }
PetscErrorCode TSSetDuration(TS ts, PetscInt n, PetscReal t) { ts->max_steps = n; ts->max_time = t; return 0; }
PetscErrorCode TSSetExactFinalTime(TS ts, TSExactFinalTimeOption o) { ts->eft = o; return 0; }
PetscErrorCode TSSetFromOptions(TS ts) { (void)ts; return 0; }
PetscErrorCode TSSetType(TS ts, TSType t) { strncpy(ts->type, t, 15); return 0; }
PetscErrorCode TSSSPSetType(TS ts, TSSSPType t) { strncpy(ts->ssptype, t, 15); return 0; }
PetscErrorCode TSSSPSetNumStages(TS ts, PetscInt n) { ts->nstages = n; return 0; }

static PetscErrorCode rhs(TS ts, PetscReal t, Vec u, Vec f) {
    ts->rhs_calls++;
    return ts->rhs(ts, t, u, f, ts->rhsctx);
}

/* SSPRK(s,3), s = n*n (Ketcheson 2008, low-storage form). */
static PetscErrorCode step_rks3(TS ts, PetscReal t0, PetscReal dt, Vec sol) {
    int s = ts->nstages > 0 ? ts->nstages : 4;
    int n = (int)(sqrt((double)s) + 0.001);
    int r = s - n;
    if (n * n != s) return shim_seterr("RKS3 needs a square number of stages\n");
    Vec w0, w1, F;
    VecDuplicate(sol, &w0); VecDuplicate(sol, &w1); VecDuplicate(sol, &F);
    VecCopy(sol, w0);
    int i = 0;
    PetscErrorCode e = 0;
    for (; i < (n - 1) * (n - 2) / 2; ++i) {
        double c = (i < n * (n + 1) / 2) ? 1.0 * i / (s - n) : (1.0 * i - n) / (s - n);
        if ((e = rhs(ts, t0 + c * dt, w0, F))) goto out;
        VecAXPY(w0, dt / r, F);
    }
    VecCopy(w0, w1);
    for (; i < n * (n + 1) / 2 - 1; ++i) {
        double c = (i < n * (n + 1) / 2) ? 1.0 * i / (s - n) : (1.0 * i - n) / (s - n);
        if ((e = rhs(ts, t0 + c * dt, w0, F))) goto out;
        VecAXPY(w0, dt / r, F);
    }
    {
        double c = (i < n * (n + 1) / 2) ? 1.0 * i / (s - n) : (1.0 * i - n) / (s - n);
        if ((e = rhs(ts, t0 + c * dt, w0, F))) goto out;
        VecAXPBYPCZ(w0, 1.0 * n / (2 * n - 1.0), (n - 1.0) * dt / (r * (2 * n - 1)), (n - 1.0) / (2 * n - 1), w1, F);
        ++i;
    }
    for (; i < s; ++i) {
        double c = (i < n * (n + 1) / 2) ? 1.0 * i / (s - n) : (1.0 * i - n) / (s - n);
        if ((e = rhs(ts, t0 + c * dt, w0, F))) goto out;
        VecAXPY(w0, dt / r, F);
    }
    VecCopy(w0, sol);
out:
    VecDestroy(&w0); VecDestroy(&w1); VecDestroy(&F);
    return e;
}

/* SSPRK(s,2) (Ketcheson 2008): s-1 forward-Euler stages of dt/(s-1), then
 * u_new = 1/s u + (s-1)/s (u_{s-1} + dt/(s-1) F(u_{s-1})). */
static PetscErrorCode step_rks2(TS ts, PetscReal t0, PetscReal dt, Vec sol) {
    int s = ts->nstages > 0 ? ts->nstages : 2;
    Vec w0, F;
    VecDuplicate(sol, &w0); VecDuplicate(sol, &F);
    VecCopy(sol, w0);
    PetscErrorCode e = 0;
    for (int i = 0; i < s - 1; ++i) {
        if ((e = rhs(ts, t0 + dt * (i / (s - 1.0)), w0, F))) goto out;
        VecAXPY(w0, dt / (s - 1.0), F);
    }
    if ((e = rhs(ts, t0 + dt, w0, F))) goto out;
    VecAXPBYPCZ(w0, 1.0 / s, dt / s, (s - 1.0) / s, sol, F);
    VecCopy(w0, sol);
out:
    VecDestroy(&w0); VecDestroy(&F);
    return e;
}

/* SSPRK(10,4) (Ketcheson 2008, low-storage form). */
static PetscErrorCode step_rk104(TS ts, PetscReal t0, PetscReal dt, Vec sol) {
    static const double c[10] = {0, 1. / 6, 2. / 6, 3. / 6, 4. / 6, 2. / 6, 3. / 6, 4. / 6, 5. / 6, 1};
    Vec w0, w1, F;
    VecDuplicate(sol, &w0); VecDuplicate(sol, &w1); VecDuplicate(sol, &F);
    VecCopy(sol, w0);
    VecCopy(sol, w1);
    PetscErrorCode e = 0;
    int i;
    for (i = 0; i < 5; ++i) {
        if ((e = rhs(ts, t0 + c[i] * dt, w0, F))) goto out;
        VecAXPY(w0, dt / 6, F);
    }
    for (long q = 0; q < w1->n; ++q) w1->a[q] = 9.0 / 25 * w0->a[q] + 1.0 / 25 * w1->a[q];
    for (long q = 0; q < w0->n; ++q) w0->a[q] = 15 * w1->a[q] + -5 * w0->a[q];
    for (; i < 9; ++i) {
        if ((e = rhs(ts, t0 + c[i] * dt, w0, F))) goto out;
        VecAXPY(w0, dt / 6, F);
    }
    if ((e = rhs(ts, t0 + dt, w0, F))) goto out;
    VecAXPBYPCZ(w1, 3.0 / 5, dt / 10, 1, w0, F);
    VecCopy(w1, sol);
out:
    VecDestroy(&w0); VecDestroy(&w1); VecDestroy(&F);
    return e;
}

static PetscErrorCode step_euler(TS ts, PetscReal t0, PetscReal dt, Vec sol) {
    Vec F;
    VecDuplicate(sol, &F);
    PetscErrorCode e = rhs(ts, t0, sol, F);
    if (!e) VecAXPY(sol, dt, F);
    VecDestroy(&F);
    return e;
}

PetscErrorCode TSSolve(TS ts, Vec u) {
    PetscErrorCode e;
    if (ts->mon && (e = ts->mon(ts, ts->steps, ts->t, u, ts->monctx))) return e;
    while (ts->steps < ts->max_steps && ts->t < ts->max_time) {
        double dt = ts->dt;
        if (ts->eft == TS_EXACTFINALTIME_MATCHSTEP && ts->t + dt > ts->max_time) dt = ts->max_time - ts->t;
        if (!strcmp(ts->type, "ssp")) {
            if (!strcmp(ts->ssptype, "rks3")) e = step_rks3(ts, ts->t, dt, u);
            else if (!strcmp(ts->ssptype, "rk104")) e = step_rk104(ts, ts->t, dt, u);
            else e = step_rks2(ts, ts->t, dt, u);
        } else {
            e = step_euler(ts, ts->t, dt, u);
        }
        if (e) return e;
        ts->t += dt;
        ts->steps++;
        if (ts->mon && (e = ts->mon(ts, ts->steps, ts->t, u, ts->monctx))) return e;
    }
    return 0;
}
