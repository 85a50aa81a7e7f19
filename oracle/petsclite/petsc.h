/*
 * petsclite: a single-rank, sequential stand-in for the subset of the PETSc 3.12
 * C API that se2wave.c (Nicolucas/se2dr_fork) calls.
 *
 * TEST INFRASTRUCTURE ONLY.  It exists so that the reference program can be
 * compiled in place, unmodified, as the oracle (oracle/_ref).  Nothing in the
 * product library includes or links it.
 *
 * Semantics are those of PETSc on one MPI rank:
 *   - Vec: contiguous PetscScalar array; VecSetValues ADD does x[i] += y.
 *   - DMDA 2-D: global == local (no ghost points exist on one rank with
 *     DM_BOUNDARY_NONE); Global<->Local scatters are copies / adds.
 *   - MatSeqDense + KSPPREONLY/PCLU: partial-pivot LU with the operation order
 *     of reference LAPACK dgetf2/dgetrs (reciprocal pivot scaling, column
 *     oriented triangular solves).
 *   - MPI_Allreduce: copy.
 *   - PetscViewerVTK / VecView: no output (file I/O of snapshots is not part of
 *     the checked path).
 */
#ifndef PETSCLITE_PETSC_H
#define PETSCLITE_PETSC_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <limits.h>

typedef int          PetscInt;
typedef int          PetscMPIInt;
typedef double       PetscReal;
typedef double       PetscScalar;
typedef int          PetscErrorCode;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;

/* ---- MPI (single rank) ---- */
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_INT      1
#define MPI_DOUBLE   2
#define MPIU_REAL    MPI_DOUBLE
#define MPI_SUM      1
#define MPI_MIN      2
#define MPI_MAX      3
#define MPIU_SUM     MPI_SUM
#define MPIU_MIN     MPI_MIN
#define MPIU_MAX     MPI_MAX
#define MPI_IN_PLACE ((void*)1)
#define PETSC_COMM_WORLD ((MPI_Comm)0)
#define PETSC_COMM_SELF  ((MPI_Comm)1)
int MPI_Comm_rank(MPI_Comm comm, PetscMPIInt *rank);
int MPI_Comm_size(MPI_Comm comm, PetscMPIInt *size);
int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);

/* ---- constants ---- */
#define PETSC_MAX_PATH_LEN 4096
#define PETSC_DECIDE  (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_PI      3.14159265358979323846264338327950288419716939937510582
#define PETSC_MAX_REAL DBL_MAX
#define PETSC_MIN_REAL (-DBL_MAX)
#define PETSC_MAX_INT  INT_MAX

#define PETSC_ERR_MEM        55
#define PETSC_ERR_SUP        56
#define PETSC_ERR_ARG_WRONG  62
#define PETSC_ERR_FILE_OPEN  65
#define PETSC_ERR_USER       83

/* ---- error handling ---- */
PetscErrorCode PetscLiteError(int line, const char *func, PetscErrorCode n, const char *fmt, ...);
PetscErrorCode PetscLiteTrace(int line, const char *func, PetscErrorCode n);
#define PetscUnlikely(x) (x)
#define PetscFunctionReturn(a) return (a)
#define PetscFunctionBegin
#define CHKERRQ(e) do { if (e) return PetscLiteTrace(__LINE__, __func__, (e)); } while (0)
#define SETERRQ(c, n, s)                 return PetscLiteError(__LINE__, __func__, (n), (s))
#define SETERRQ1(c, n, s, a1)            return PetscLiteError(__LINE__, __func__, (n), (s), (a1))
#define SETERRQ2(c, n, s, a1, a2)        return PetscLiteError(__LINE__, __func__, (n), (s), (a1), (a2))
#define SETERRQ3(c, n, s, a1, a2, a3)    return PetscLiteError(__LINE__, __func__, (n), (s), (a1), (a2), (a3))

/* ---- memory ---- */
PetscErrorCode PetscLiteMalloc(size_t n, void **p);
#define PetscMalloc(a, b)   PetscLiteMalloc((size_t)(a), (void**)(b))
#define PetscMalloc1(n, b)  PetscLiteMalloc((size_t)(n) * sizeof(**(b)), (void**)(b))
#define PetscFree(p)        (free(p), (p) = NULL, 0)
#define PetscMemzero(p, n)  (memset((p), 0, (n)), 0)
#define PetscMemcpy(d, s, n) (memcpy((d), (s), (n)), 0)

/* ---- math ---- */
#define PetscAbsReal(a)  fabs(a)
#define PetscSqrtReal(a) sqrt(a)
#define PetscPowReal(a, b) pow((a), (b))
#define PetscExpReal(a)  exp(a)
#define PetscCosReal(a)  cos(a)
#define PetscAsinReal(a) asin(a)
#define PetscAtanReal(a) atan(a)
#define PetscRealPart(a) (a)
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
PetscErrorCode PetscSortReal(PetscInt n, PetscReal v[]);

/* ---- objects ---- */
struct _p_PetscObject { int classid; char name[256]; };
typedef struct _p_PetscObject *PetscObject;
PetscErrorCode PetscObjectSetName(PetscObject o, const char name[]);

typedef struct _p_DM *DM;
typedef struct _p_Vec *Vec;
typedef struct _p_Mat *Mat;
typedef struct _p_KSP *KSP;
typedef struct _p_PC *PC;
typedef struct _p_PetscViewer *PetscViewer;
typedef struct _p_PetscRandom *PetscRandom;

struct _p_Vec {
  struct _p_PetscObject hdr;
  PetscInt n, bs;
  PetscScalar *array;
};

typedef enum { NOT_SET_VALUES = -1, INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3 } NormType;
typedef enum { DM_BOUNDARY_NONE = 0, DM_BOUNDARY_GHOSTED, DM_BOUNDARY_MIRROR, DM_BOUNDARY_PERIODIC } DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR = 0, DMDA_STENCIL_BOX = 1 } DMDAStencilType;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *PetscRandomType;
#define KSPPREONLY  "preonly"
#define PCLU        "lu"
#define PCNONE      "none"
#define PETSCRAND48 "rand48"

typedef struct { PetscReal x, y; } DMDACoor2d;
typedef struct { PetscReal x, y, z; } DMDACoor3d;
typedef struct {
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;
  PetscInt xs, ys, zs, xm, ym, zm;
  PetscInt gxs, gys, gzs, gxm, gym, gzm;
  DMBoundaryType bx, by, bz;
  DMDAStencilType st;
  DM da;
} DMDALocalInfo;

#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)

/* ---- init / options / printing ---- */
PetscErrorCode PetscInitialize(int *argc, char ***args, const char file[], const char help[]);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscOptionsGetInt(void *opt, const char pre[], const char name[], PetscInt *v, PetscBool *set);
PetscErrorCode PetscOptionsGetReal(void *opt, const char pre[], const char name[], PetscReal *v, PetscBool *set);
PetscErrorCode PetscOptionsGetBool(void *opt, const char pre[], const char name[], PetscBool *v, PetscBool *set);
PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...);
PetscErrorCode PetscSNPrintf(char *buf, size_t len, const char fmt[], ...);
/* petsclite extras (used by the oracle driver only) */
PetscErrorCode PetscLiteOptionsSet(int argc, char **argv);
void           PetscLiteSetQuiet(int quiet);

/* ---- Vec ---- */
PetscErrorCode VecCreate(MPI_Comm comm, Vec *v);
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N);
PetscErrorCode VecSetFromOptions(Vec v);
PetscErrorCode VecDuplicate(Vec x, Vec *y);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecScale(Vec v, PetscScalar a);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecPointwiseDivide(Vec w, Vec x, Vec y);
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *nrm);
PetscErrorCode VecMin(Vec v, PetscInt *idx, PetscReal *val);
PetscErrorCode VecMax(Vec v, PetscInt *idx, PetscReal *val);
PetscErrorCode VecGetSize(Vec v, PetscInt *N);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode m);
PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m);
PetscErrorCode VecSetValueLocal(Vec v, PetscInt i, PetscScalar y, InsertMode m);
PetscErrorCode VecSetValuesLocal(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecStrideScale(Vec v, PetscInt start, PetscScalar a);
PetscErrorCode VecStrideSet(Vec v, PetscInt start, PetscScalar a);
PetscErrorCode VecSetRandom(Vec v, PetscRandom r);
PetscErrorCode VecView(Vec v, PetscViewer viewer);

/* ---- DM / DMDA ---- */
PetscErrorCode DMDACreate2d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMDAStencilType st,
                            PetscInt M, PetscInt N, PetscInt m, PetscInt n, PetscInt dof, PetscInt s,
                            const PetscInt lx[], const PetscInt ly[], DM *da);
PetscErrorCode DMSetUp(DM dm);
PetscErrorCode DMDestroy(DM *dm);
PetscErrorCode DMView(DM dm, PetscViewer v);
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v);
PetscErrorCode DMGetLocalVector(DM dm, Vec *v);
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v);
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode m, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode m, Vec l);
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode m, Vec g);
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode m, Vec g);
PetscErrorCode DMGetCoordinates(DM dm, Vec *c);
PetscErrorCode DMGetCoordinatesLocal(DM dm, Vec *c);
PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm);
PetscErrorCode DMGetBoundingBox(DM dm, PetscReal gmin[], PetscReal gmax[]);
PetscErrorCode DMDASetUniformCoordinates(DM dm, PetscReal x0, PetscReal x1, PetscReal y0, PetscReal y1,
                                         PetscReal z0, PetscReal z1);
PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void *array);
PetscErrorCode DMDAGetGhostCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p);
PetscErrorCode DMDAGetCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p);
PetscErrorCode DMDAGetInfo(DM dm, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m, PetscInt *n,
                           PetscInt *p, PetscInt *dof, PetscInt *s, DMBoundaryType *bx, DMBoundaryType *by,
                           DMBoundaryType *bz, DMDAStencilType *st);
PetscErrorCode DMDAGetOwnershipRanges(DM dm, const PetscInt *lx[], const PetscInt *ly[], const PetscInt *lz[]);
PetscErrorCode DMDAGetLocalInfo(DM dm, DMDALocalInfo *info);
PetscErrorCode DMDASetFieldName(DM dm, PetscInt f, const char name[]);

/* ---- Mat / KSP / PC ---- */
PetscErrorCode MatCreateSeqDense(MPI_Comm comm, PetscInt m, PetscInt n, PetscScalar *data, Mat *A);
PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar v, InsertMode m);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatCreateVecs(Mat A, Vec *right, Vec *left);
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n);
PetscErrorCode MatDestroy(Mat *A);
PetscErrorCode KSPCreate(MPI_Comm comm, KSP *ksp);
PetscErrorCode KSPSetOptionsPrefix(KSP ksp, const char prefix[]);
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat P);
PetscErrorCode KSPSetType(KSP ksp, KSPType t);
PetscErrorCode KSPGetPC(KSP ksp, PC *pc);
PetscErrorCode PCSetType(PC pc, PCType t);
PetscErrorCode KSPSetFromOptions(KSP ksp);
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x);
PetscErrorCode KSPComputeEigenvaluesExplicitly(KSP ksp, PetscInt n, PetscReal r[], PetscReal c[]);
PetscErrorCode KSPDestroy(KSP *ksp);

/* ---- viewers / random ---- */
PetscErrorCode PetscViewerVTKOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *v);
PetscErrorCode PetscViewerDestroy(PetscViewer *v);
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r);
PetscErrorCode PetscRandomSetType(PetscRandom r, PetscRandomType t);
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar lo, PetscScalar hi);
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed);
PetscErrorCode PetscRandomSeed(PetscRandom r);
PetscErrorCode PetscRandomDestroy(PetscRandom *r);

#endif
