/*
 * petsc_shim.h -- single-rank stand-in for the subset of the PETSc API that the
 * reference programs call (DMDA structured grids, Vec, TS with the SSP family,
 * viewers, MPI reductions).  TEST INFRASTRUCTURE ONLY: it exists so that the
 * reference's own C sources compile unmodified into the CPU checker under
 * oracle/_ref/.  Nothing in the GPU product links it.
 *
 * Semantics restated from PETSc's public manual pages (no PETSc source is
 * available here, and the reference pins no PETSc version):
 *   - one MPI rank: the owned box is the whole grid (xs=ys=zs=0);
 *   - DMDAVecGetArray returns ghost-offset pointers that accept indices from
 *     the ghost corner (negative for ghosted/periodic boundaries);
 *   - DMGlobalToLocal copies the owned box and, for periodic boundaries, the
 *     wrapped ghost values (box stencil: edges and corners too); exterior
 *     ghosts of DM_BOUNDARY_GHOSTED are left untouched (zero in a fresh
 *     local vector);
 *   - TSSSP RKS3 with s = n*n stages follows Ketcheson (2008), "Highly
 *     efficient strong stability preserving Runge-Kutta methods with low-storage
 *     implementations", SIAM J. Sci. Comput. 30:2113, in PETSc's low-storage
 *     form; RK104 is Ketcheson's SSPRK(10,4) from the same paper.
 */
#ifndef PETSC_SHIM_H
#define PETSC_SHIM_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>

typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef int PetscErrorCode;
typedef double PetscLogDouble;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define PETSC_COMM_WORLD 1
#define PETSC_COMM_SELF 2
#define MPI_COMM_WORLD 1
#define MPIU_REAL 1
#define MPIU_SCALAR 1
#define MPIU_INT 2
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPIU_MIN 1
#define MPIU_MAX 2
#define MPIU_SUM 3
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

#define PETSC_DECIDE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_DETERMINE (-1)
#define PETSC_PI 3.14159265358979323846264338327950288
#define PETSC_SUCCESS 0
#define PETSC_ERR_ARG_OUTOFRANGE 63

#define PetscSqrtReal(a) sqrt(a)
#define PetscAbsReal(a) fabs(a)
#define PetscPowReal(a, b) pow(a, b)
#define PetscExpReal(a) exp(a)
#define PetscSinReal(a) sin(a)
#define PetscCosReal(a) cos(a)
#define PetscTanhReal(a) tanh(a)
#define PetscLogReal(a) log(a)
#define PetscAtanReal(a) atan(a)
#define PetscAtan2Real(a, b) atan2(a, b)
#define PetscSign(a) (((a) >= 0) ? ((a) == 0 ? 0 : 1) : -1)
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscAbsScalar(a) fabs(a)
#define PetscRealPart(a) (a)

#define CHKERRQ(e) do { if (e) return (e); } while (0)
#define CHKERRMPI(e) CHKERRQ(e)
#define PetscCall(e) do { PetscErrorCode e__ = (e); if (e__) return e__; } while (0)
#define PetscFunctionBeginUser do {} while (0)
#define PetscFunctionBegin do {} while (0)
#define PetscFunctionReturn(x) return (x)
#define SETERRQ(comm, code, ...) return (shim_seterr(__VA_ARGS__), 1)
int shim_seterr(const char* fmt, ...);

/* ---- objects ---- */
typedef enum { DM_BOUNDARY_NONE = 0, DM_BOUNDARY_GHOSTED = 1, DM_BOUNDARY_MIRROR = 2, DM_BOUNDARY_PERIODIC = 3 } DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR = 0, DMDA_STENCIL_BOX = 1 } DMDAStencilType;
typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3 } NormType;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE = 1, FILE_MODE_APPEND = 2 } PetscFileMode;
typedef enum { PETSC_VIEWER_DEFAULT = 0, PETSC_VIEWER_ASCII_VTK = 1, PETSC_VIEWER_ASCII_VTK_DEPRECATED = 1 } PetscViewerFormat;
typedef enum { TS_LINEAR = 0, TS_NONLINEAR = 1 } TSProblemType;
typedef enum { TS_EXACTFINALTIME_UNSPECIFIED = 0, TS_EXACTFINALTIME_STEPOVER = 1, TS_EXACTFINALTIME_INTERPOLATE = 2,
               TS_EXACTFINALTIME_MATCHSTEP = 3 } TSExactFinalTimeOption;

typedef struct { PetscScalar x, y; } DMDACoor2d;
typedef struct { PetscScalar x, y, z; } DMDACoor3d;
typedef struct _p_DM* DM;
typedef struct _p_Vec* Vec;
typedef struct _p_TS* TS;
typedef struct _p_Viewer* PetscViewer;
typedef void* PetscObject;
typedef const char* TSType;
typedef const char* TSSSPType;
#define TSSSP "ssp"
#define TSEULER "euler"
#define TSRK "rk"
#define TSSSPRKS2 "rks2"
#define TSSSPRKS3 "rks3"
#define TSSSPRK104 "rk104"

struct _p_DM {
    int dim, dof, sw;
    DMBoundaryType bx, by, bz;
    DMDAStencilType st;
    int M, N, P;                 /* global sizes */
    int xs, ys, zs, xm, ym, zm;  /* owned box */
    int gxs, gys, gzs, gxm, gym, gzm; /* ghost box */
    Vec localpool[8];
    int localused[8];
    Vec coords;
    DM cdm;  /* coordinate DMDA (dof = dim), made by DMDASetUniformCoordinates */
    double cmin[3], cmax[3];
};

struct _p_Vec {
    DM dm;      /* may be NULL for plain vectors */
    int local;  /* 1 when shaped like the ghosted box */
    long n;
    double* a;
    char name[64];
    void* view;  /* pointer-array storage for DMDAVecGetArray */
};

/* ---- sys ---- */
PetscErrorCode PetscInitialize(int* argc, char*** argv, const char* file, const char* help);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscPrintf(MPI_Comm comm, const char* fmt, ...);
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE* f, const char* fmt, ...);
PetscErrorCode PetscTime(PetscLogDouble* t);
PetscErrorCode PetscObjectSetName(PetscObject obj, const char* name);
MPI_Comm PetscObjectComm(PetscObject obj);
int MPI_Comm_rank(MPI_Comm c, int* r);
int MPI_Comm_size(MPI_Comm c, int* s);
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Barrier(MPI_Comm c);
/* The reference aborts on an inadmissible state.  The shim records the abort
 * (so a checker can report it) and, when a jump target is armed, unwinds. */
extern int shim_abort_count;
void shim_set_abort_jump(void* jmp_buf_ptr);

/* ---- DM / DMDA ---- */
PetscErrorCode DMDACreate1d(MPI_Comm c, DMBoundaryType bx, PetscInt M, PetscInt dof, PetscInt sw, const PetscInt lx[], DM* da);
PetscErrorCode DMDACreate2d(MPI_Comm c, DMBoundaryType bx, DMBoundaryType by, DMDAStencilType st, PetscInt M, PetscInt N,
                            PetscInt m, PetscInt n, PetscInt dof, PetscInt sw, const PetscInt lx[], const PetscInt ly[], DM* da);
PetscErrorCode DMDACreate3d(MPI_Comm c, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz, DMDAStencilType st, PetscInt M,
                            PetscInt N, PetscInt P, PetscInt m, PetscInt n, PetscInt p, PetscInt dof, PetscInt sw,
                            const PetscInt lx[], const PetscInt ly[], const PetscInt lz[], DM* da);
PetscErrorCode DMSetUp(DM da);
PetscErrorCode DMSetFromOptions(DM da);
PetscErrorCode DMDestroy(DM* da);
PetscErrorCode DMDAGetCorners(DM da, PetscInt* xs, PetscInt* ys, PetscInt* zs, PetscInt* xm, PetscInt* ym, PetscInt* zm);
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt* xs, PetscInt* ys, PetscInt* zs, PetscInt* xm, PetscInt* ym, PetscInt* zm);
PetscErrorCode DMDAGetInfo(DM da, PetscInt* dim, PetscInt* M, PetscInt* N, PetscInt* P, PetscInt* m, PetscInt* n, PetscInt* p,
                           PetscInt* dof, PetscInt* s, DMBoundaryType* bx, DMBoundaryType* by, DMBoundaryType* bz,
                           DMDAStencilType* st);
PetscErrorCode DMCreateGlobalVector(DM da, Vec* v);
PetscErrorCode DMCreateLocalVector(DM da, Vec* v);
PetscErrorCode DMGetLocalVector(DM da, Vec* v);
PetscErrorCode DMRestoreLocalVector(DM da, Vec* v);
PetscErrorCode DMGetGlobalVector(DM da, Vec* v);
PetscErrorCode DMRestoreGlobalVector(DM da, Vec* v);
PetscErrorCode DMGlobalToLocalBegin(DM da, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM da, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void* array);
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void* array);
PetscErrorCode DMDAVecGetArrayRead(DM da, Vec v, void* array);
PetscErrorCode DMDAVecRestoreArrayRead(DM da, Vec v, void* array);
PetscErrorCode DMDASetUniformCoordinates(DM da, PetscReal x0, PetscReal x1, PetscReal y0, PetscReal y1, PetscReal z0, PetscReal z1);
PetscErrorCode DMGetCoordinateDM(DM da, DM* cda);
PetscErrorCode DMGetCoordinates(DM da, Vec* c);
PetscErrorCode DMGetCoordinatesLocal(DM da, Vec* c);
PetscErrorCode DMDASetFieldName(DM da, PetscInt nf, const char* name);
PetscErrorCode DMView(DM da, PetscViewer v);

/* ---- Vec ---- */
PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec* v);
PetscErrorCode VecDuplicate(Vec v, Vec* w);
PetscErrorCode VecDestroy(Vec* v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecAYPX(Vec y, PetscScalar b, Vec x);
PetscErrorCode VecAXPBYPCZ(Vec z, PetscScalar a, PetscScalar b, PetscScalar c, Vec x, Vec y);
PetscErrorCode VecScale(Vec v, PetscScalar a);
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal* r);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar** a);
PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n);
PetscErrorCode VecGetSize(Vec v, PetscInt* n);
PetscErrorCode VecView(Vec v, PetscViewer vw);
PetscErrorCode VecLoad(Vec v, PetscViewer vw);
PetscErrorCode VecStrideNorm(Vec v, PetscInt s, NormType t, PetscReal* r);

/* ---- viewers (no files are written; the checker never needs them) ---- */
PetscErrorCode PetscViewerVTKOpen(MPI_Comm c, const char* name, PetscFileMode m, PetscViewer* v);
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm c, const char* name, PetscViewer* v);
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char* name, PetscFileMode m, PetscViewer* v);
PetscErrorCode PetscViewerPushFormat(PetscViewer v, PetscViewerFormat f);
PetscErrorCode PetscViewerPopFormat(PetscViewer v);
PetscErrorCode PetscViewerDestroy(PetscViewer* v);

/* ---- TS ---- */
typedef PetscErrorCode (*TSRHSFunctionFn)(TS, PetscReal, Vec, Vec, void*);
typedef PetscErrorCode (*TSMonitorFn)(TS, PetscInt, PetscReal, Vec, void*);
struct _p_TS {
    DM dm;
    TSRHSFunctionFn rhs;
    void* rhsctx;
    TSMonitorFn mon;
    void* monctx;
    PetscReal t, dt, max_time;
    PetscInt steps, max_steps;
    TSExactFinalTimeOption eft;
    char type[16], ssptype[16];
    PetscInt nstages;
    long rhs_calls;
};
PetscErrorCode TSCreate(MPI_Comm c, TS* ts);
PetscErrorCode TSDestroy(TS* ts);
PetscErrorCode TSSetProblemType(TS ts, TSProblemType t);
PetscErrorCode TSSetDM(TS ts, DM dm);
PetscErrorCode TSGetDM(TS ts, DM* dm);
PetscErrorCode TSSetRHSFunction(TS ts, Vec r, TSRHSFunctionFn f, void* ctx);
PetscErrorCode TSSetStepNumber(TS ts, PetscInt s);
PetscErrorCode TSGetStepNumber(TS ts, PetscInt* s);
PetscErrorCode TSSetTime(TS ts, PetscReal t);
PetscErrorCode TSGetTime(TS ts, PetscReal* t);
PetscErrorCode TSSetTimeStep(TS ts, PetscReal dt);
PetscErrorCode TSGetTimeStep(TS ts, PetscReal* dt);
PetscErrorCode TSMonitorSet(TS ts, TSMonitorFn f, void* ctx, void* destroy);
PetscErrorCode TSSetMaxTime(TS ts, PetscReal t);
PetscErrorCode TSSetMaxSteps(TS ts, PetscInt n);
PetscErrorCode TSSetDuration(TS ts, PetscInt n, PetscReal t);
PetscErrorCode TSSetExactFinalTime(TS ts, TSExactFinalTimeOption o);
PetscErrorCode TSSetFromOptions(TS ts);
PetscErrorCode TSSetType(TS ts, TSType t);
PetscErrorCode TSSSPSetType(TS ts, TSSSPType t);
PetscErrorCode TSSSPSetNumStages(TS ts, PetscInt n);
PetscErrorCode TSSolve(TS ts, Vec u);

#endif
