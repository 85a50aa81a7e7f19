/*
 * petsclite implementation.  TEST INFRASTRUCTURE ONLY (see petsc.h).
 *
 * Built with -ffp-contract=off so that no multiply-add is fused: the reference
 * build (makefile:4, "-g -O2" on x86-64) emits no FMA, and the oracle must give
 * the same bits on x86-64 and aarch64.
 */
#include "petsc.h"
#include <stdarg.h>

static void translate_fmt(const char *in, char *out, size_t len);

/* ------------------------------------------------------------------ */
/* errors                                                              */
/* ------------------------------------------------------------------ */
static int lite_quiet = 0;
void PetscLiteSetQuiet(int q) { lite_quiet = q; }

PetscErrorCode PetscLiteError(int line, const char *func, PetscErrorCode n, const char *fmt, ...)
{
  char buf[2048];
  va_list ap;
  translate_fmt(fmt, buf, sizeof(buf));
  fprintf(stderr, "[petsclite] error %d in %s() line %d: ", (int)n, func, line);
  va_start(ap, fmt);
  vfprintf(stderr, buf, ap);
  va_end(ap);
  fprintf(stderr, "\n");
  return n;
}

PetscErrorCode PetscLiteTrace(int line, const char *func, PetscErrorCode n)
{
  fprintf(stderr, "[petsclite]   from %s() line %d\n", func, line);
  return n;
}

PetscErrorCode PetscLiteMalloc(size_t n, void **p)
{
  *p = malloc(n ? n : 1);
  if (!*p) return PetscLiteError(__LINE__, __func__, PETSC_ERR_MEM, "out of memory (%zu bytes)", n);
  return 0;
}

static int cmp_real(const void *a, const void *b)
{
  double x = *(const double*)a, y = *(const double*)b;
  return (x < y) ? -1 : (x > y) ? 1 : 0;
}
PetscErrorCode PetscSortReal(PetscInt n, PetscReal v[]) { qsort(v, (size_t)n, sizeof(PetscReal), cmp_real); return 0; }

PetscErrorCode PetscObjectSetName(PetscObject o, const char name[])
{
  if (o) { strncpy(o->name, name, sizeof(o->name) - 1); o->name[sizeof(o->name) - 1] = 0; }
  return 0;
}

/* ------------------------------------------------------------------ */
/* MPI, one rank                                                       */
/* ------------------------------------------------------------------ */
int MPI_Comm_rank(MPI_Comm comm, PetscMPIInt *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, PetscMPIInt *size) { (void)comm; *size = 1; return 0; }
int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
  (void)op; (void)comm;
  if (in == MPI_IN_PLACE) return 0;
  memcpy(out, in, (size_t)count * (t == MPI_INT ? sizeof(int) : sizeof(double)));
  return 0;
}

/* ------------------------------------------------------------------ */
/* options database                                                    */
/* ------------------------------------------------------------------ */
static int    opt_argc = 0;
static char **opt_argv = NULL;

PetscErrorCode PetscLiteOptionsSet(int argc, char **argv) { opt_argc = argc; opt_argv = argv; return 0; }

PetscErrorCode PetscInitialize(int *argc, char ***args, const char file[], const char help[])
{
  (void)file; (void)help;
  if (argc && args) PetscLiteOptionsSet(*argc, *args);
  return 0;
}
PetscErrorCode PetscFinalize(void) { return 0; }

/* last occurrence wins, as in PETSc's options database */
static const char *opt_find(const char name[], int *found)
{
  int i;
  *found = 0;
  for (i = opt_argc - 1; i >= 1; i--) {
    if (opt_argv[i] && strcmp(opt_argv[i], name) == 0) {
      *found = 1;
      if (i + 1 < opt_argc) {
        const char *v = opt_argv[i + 1];
        /* a following token is a value unless it is another option name */
        if (v[0] != '-' || (v[1] >= '0' && v[1] <= '9') || v[1] == '.') return v;
      }
      return NULL;
    }
  }
  return NULL;
}

PetscErrorCode PetscOptionsGetInt(void *o, const char pre[], const char name[], PetscInt *v, PetscBool *set)
{
  int found; const char *s = opt_find(name, &found);
  (void)o; (void)pre;
  if (set) *set = PETSC_FALSE;
  if (!found) return 0;
  if (!s) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_USER, "option %s needs an integer value", name);
  *v = (PetscInt)strtol(s, NULL, 10);
  if (set) *set = PETSC_TRUE;
  return 0;
}

PetscErrorCode PetscOptionsGetReal(void *o, const char pre[], const char name[], PetscReal *v, PetscBool *set)
{
  int found; const char *s = opt_find(name, &found);
  (void)o; (void)pre;
  if (set) *set = PETSC_FALSE;
  if (!found) return 0;
  if (!s) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_USER, "option %s needs a real value", name);
  *v = strtod(s, NULL);
  if (set) *set = PETSC_TRUE;
  return 0;
}

PetscErrorCode PetscOptionsGetBool(void *o, const char pre[], const char name[], PetscBool *v, PetscBool *set)
{
  int found; const char *s = opt_find(name, &found);
  (void)o; (void)pre;
  if (set) *set = PETSC_FALSE;
  if (!found) return 0;
  *v = PETSC_TRUE;
  if (s) {
    if (!strcmp(s, "0") || !strcasecmp(s, "false") || !strcasecmp(s, "no")) *v = PETSC_FALSE;
  }
  if (set) *set = PETSC_TRUE;
  return 0;
}

/* translate PETSc's %D conversion (PetscInt), with any flags/width, to %d */
static void translate_fmt(const char *in, char *out, size_t len)
{
  size_t i = 0, j = 0;
  while (in[i] && j < len - 2) {
    if (in[i] == '%' && in[i + 1] != '%') {
      size_t k = i + 1;
      while (in[k] && strchr("-+ #0123456789.", in[k])) k++;
      if (in[k] == 'D') {
        while (i < k && j < len - 2) out[j++] = in[i++];
        out[j++] = 'd';
        i = k + 1;
        continue;
      }
    }
    out[j++] = in[i++];
  }
  out[j] = 0;
}

PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...)
{
  char buf[4096];
  va_list ap;
  (void)comm;
  if (lite_quiet) return 0;
  translate_fmt(fmt, buf, sizeof(buf));
  va_start(ap, fmt);
  vprintf(buf, ap);
  va_end(ap);
  return 0;
}

PetscErrorCode PetscSNPrintf(char *str, size_t len, const char fmt[], ...)
{
  char buf[4096];
  va_list ap;
  translate_fmt(fmt, buf, sizeof(buf));
  va_start(ap, fmt);
  vsnprintf(str, len, buf, ap);
  va_end(ap);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Vec                                                                 */
/* ------------------------------------------------------------------ */
static Vec vec_new(PetscInt n, PetscInt bs)
{
  Vec v = (Vec)calloc(1, sizeof(struct _p_Vec));
  v->n = n;
  v->bs = bs;
  v->array = (PetscScalar*)calloc((size_t)(n > 0 ? n : 1), sizeof(PetscScalar));
  return v;
}

PetscErrorCode VecCreate(MPI_Comm comm, Vec *v)
{
  (void)comm;
  *v = (Vec)calloc(1, sizeof(struct _p_Vec));
  (*v)->bs = 1;
  return 0;
}
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N) { v->n = (n >= 0) ? n : N; return 0; }
PetscErrorCode VecSetFromOptions(Vec v)
{
  if (!v->array) v->array = (PetscScalar*)calloc((size_t)(v->n > 0 ? v->n : 1), sizeof(PetscScalar));
  return 0;
}
PetscErrorCode VecDuplicate(Vec x, Vec *y) { *y = vec_new(x->n, x->bs); return 0; }
PetscErrorCode VecDestroy(Vec *v)
{
  if (!v || !*v) return 0;
  free((*v)->array);
  free(*v);
  *v = NULL;
  return 0;
}
PetscErrorCode VecZeroEntries(Vec v) { memset(v->array, 0, sizeof(PetscScalar) * (size_t)v->n); return 0; }
PetscErrorCode VecSet(Vec v, PetscScalar a) { PetscInt i; for (i = 0; i < v->n; i++) v->array[i] = a; return 0; }
PetscErrorCode VecScale(Vec v, PetscScalar a) { PetscInt i; for (i = 0; i < v->n; i++) v->array[i] *= a; return 0; }

/* y <- y + a*x (BLAS daxpy semantics; PETSc returns early for a == 0) */
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x)
{
  PetscInt i;
  PetscScalar *yy = y->array;
  const PetscScalar *xx = x->array;
  if (a == 0.0) return 0;
  for (i = 0; i < y->n; i++) yy[i] = yy[i] + a * xx[i];
  return 0;
}

PetscErrorCode VecPointwiseDivide(Vec w, Vec x, Vec y)
{
  PetscInt i;
  for (i = 0; i < w->n; i++) w->array[i] = x->array[i] / y->array[i];
  return 0;
}

/* PETSc VecNorm_Seq NORM_2: sqrt(BLASdot(x,x)) */
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *nrm)
{
  PetscInt i;
  double s = 0.0;
  if (t == NORM_2 || t == NORM_FROBENIUS) {
    for (i = 0; i < v->n; i++) s = s + v->array[i] * v->array[i];
    *nrm = sqrt(s);
  } else if (t == NORM_1) {
    for (i = 0; i < v->n; i++) s = s + fabs(v->array[i]);
    *nrm = s;
  } else {
    for (i = 0; i < v->n; i++) if (fabs(v->array[i]) > s) s = fabs(v->array[i]);
    *nrm = s;
  }
  return 0;
}

PetscErrorCode VecMin(Vec v, PetscInt *idx, PetscReal *val)
{
  PetscInt i, j = -1;
  double m = PETSC_MAX_REAL;
  for (i = 0; i < v->n; i++) if (v->array[i] < m) { m = v->array[i]; j = i; }
  if (idx) *idx = j;
  *val = m;
  return 0;
}

PetscErrorCode VecMax(Vec v, PetscInt *idx, PetscReal *val)
{
  PetscInt i, j = -1;
  double m = PETSC_MIN_REAL;
  for (i = 0; i < v->n; i++) if (v->array[i] > m) { m = v->array[i]; j = i; }
  if (idx) *idx = j;
  *val = m;
  return 0;
}

PetscErrorCode VecGetSize(Vec v, PetscInt *N) { *N = v->n; return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->array; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { (void)v; if (a) *a = NULL; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) { *a = v->array; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a) { (void)v; if (a) *a = NULL; return 0; }

PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m)
{
  PetscInt i;
  for (i = 0; i < n; i++) {
    if (idx[i] < 0) continue;
    if (idx[i] >= v->n) SETERRQ2(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONG, "index %D out of range (%D)", idx[i], v->n);
    if (m == ADD_VALUES) v->array[idx[i]] += y[i];
    else v->array[idx[i]] = y[i];
  }
  return 0;
}
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode m) { return VecSetValues(v, 1, &i, &y, m); }
/* one rank, no ghosts: the local-to-global map is the identity */
PetscErrorCode VecSetValuesLocal(Vec v, PetscInt n, const PetscInt idx[], const PetscScalar y[], InsertMode m)
{
  return VecSetValues(v, n, idx, y, m);
}
PetscErrorCode VecSetValueLocal(Vec v, PetscInt i, PetscScalar y, InsertMode m) { return VecSetValues(v, 1, &i, &y, m); }
PetscErrorCode VecAssemblyBegin(Vec v) { (void)v; return 0; }
PetscErrorCode VecAssemblyEnd(Vec v) { (void)v; return 0; }

PetscErrorCode VecStrideScale(Vec v, PetscInt start, PetscScalar a)
{
  PetscInt i;
  for (i = start; i < v->n; i += v->bs) v->array[i] *= a;
  return 0;
}
PetscErrorCode VecStrideSet(Vec v, PetscInt start, PetscScalar a)
{
  PetscInt i;
  for (i = start; i < v->n; i += v->bs) v->array[i] = a;
  return 0;
}

/* ------------------------------------------------------------------ */
/* random (PETSCRAND48)                                                */
/* ------------------------------------------------------------------ */
struct _p_PetscRandom { struct _p_PetscObject hdr; unsigned long seed; double low, width; int iset; };
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r)
{
  (void)comm;
  *r = (PetscRandom)calloc(1, sizeof(struct _p_PetscRandom));
  (*r)->width = 1.0;
  return 0;
}
PetscErrorCode PetscRandomSetType(PetscRandom r, PetscRandomType t) { (void)r; (void)t; return 0; }
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar lo, PetscScalar hi)
{
  r->low = lo; r->width = hi - lo; r->iset = 1;
  return 0;
}
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed) { r->seed = seed; return 0; }
PetscErrorCode PetscRandomSeed(PetscRandom r) { srand48((long)r->seed); return 0; }
PetscErrorCode PetscRandomDestroy(PetscRandom *r) { if (r && *r) { free(*r); *r = NULL; } return 0; }
PetscErrorCode VecSetRandom(Vec v, PetscRandom r)
{
  PetscInt i;
  for (i = 0; i < v->n; i++) {
    if (r->iset) v->array[i] = r->width * drand48() + r->low;
    else v->array[i] = drand48();
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* viewers: snapshots are not produced by the oracle                   */
/* ------------------------------------------------------------------ */
struct _p_PetscViewer { struct _p_PetscObject hdr; };
PetscErrorCode PetscViewerVTKOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *v)
{
  (void)comm; (void)mode;
  *v = (PetscViewer)calloc(1, sizeof(struct _p_PetscViewer));
  PetscObjectSetName((PetscObject)*v, name);
  return 0;
}
PetscErrorCode PetscViewerDestroy(PetscViewer *v) { if (v && *v) { free(*v); *v = NULL; } return 0; }
PetscErrorCode VecView(Vec v, PetscViewer viewer) { (void)v; (void)viewer; return 0; }

/* ------------------------------------------------------------------ */
/* DMDA, 2-D, one rank                                                 */
/* ------------------------------------------------------------------ */
#define LITE_POOL 8
struct _p_DM {
  struct _p_PetscObject hdr;
  PetscInt M, N, dof, s;
  PetscInt lx[1], ly[1];
  Vec coords;
  DM cdm;
  Vec pool[LITE_POOL];
  int pool_used[LITE_POOL];
  PetscScalar **rows; /* DMDAVecGetArray row table */
};

PetscErrorCode DMDACreate2d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMDAStencilType st,
                            PetscInt M, PetscInt N, PetscInt m, PetscInt n, PetscInt dof, PetscInt s,
                            const PetscInt lx[], const PetscInt ly[], DM *da)
{
  DM d;
  (void)comm; (void)bx; (void)by; (void)st; (void)lx; (void)ly;
  if ((m != PETSC_DECIDE && m != 1) || (n != PETSC_DECIDE && n != 1))
    SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "petsclite supports one rank only");
  d = (DM)calloc(1, sizeof(struct _p_DM));
  d->M = M; d->N = N; d->dof = dof; d->s = s;
  d->lx[0] = M; d->ly[0] = N;
  *da = d;
  return 0;
}
PetscErrorCode DMSetUp(DM dm) { (void)dm; return 0; }
PetscErrorCode DMView(DM dm, PetscViewer v) { (void)dm; (void)v; return 0; }
PetscErrorCode DMDestroy(DM *dm)
{
  int i;
  DM d;
  if (!dm || !*dm) return 0;
  d = *dm;
  for (i = 0; i < LITE_POOL; i++) VecDestroy(&d->pool[i]);
  VecDestroy(&d->coords);
  if (d->cdm) DMDestroy(&d->cdm);
  free(d->rows);
  free(d);
  *dm = NULL;
  return 0;
}
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v) { *v = vec_new(dm->M * dm->N * dm->dof, dm->dof); return 0; }

/* PETSc caches local work vectors; their contents on checkout are unspecified */
PetscErrorCode DMGetLocalVector(DM dm, Vec *v)
{
  int i;
  for (i = 0; i < LITE_POOL; i++) {
    if (!dm->pool_used[i]) {
      if (!dm->pool[i]) dm->pool[i] = vec_new(dm->M * dm->N * dm->dof, dm->dof);
      dm->pool_used[i] = 1;
      *v = dm->pool[i];
      return 0;
    }
  }
  SETERRQ(PETSC_COMM_SELF, PETSC_ERR_MEM, "local vector pool exhausted");
}
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v)
{
  int i;
  for (i = 0; i < LITE_POOL; i++) if (dm->pool[i] == *v) { dm->pool_used[i] = 0; *v = NULL; return 0; }
  SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONG, "vector was not checked out of this DM");
}

static PetscErrorCode scatter(Vec from, InsertMode m, Vec to)
{
  PetscInt i;
  if (from->n != to->n) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONG, "size mismatch in scatter");
  if (from == to) return 0;
  if (m == ADD_VALUES) { for (i = 0; i < to->n; i++) to->array[i] += from->array[i]; }
  else memcpy(to->array, from->array, sizeof(PetscScalar) * (size_t)to->n);
  return 0;
}
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode m, Vec l) { (void)dm; return scatter(g, m, l); }
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode m, Vec l) { (void)dm; (void)g; (void)m; (void)l; return 0; }
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode m, Vec g) { (void)dm; return scatter(l, m, g); }
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode m, Vec g) { (void)dm; (void)l; (void)m; (void)g; return 0; }

PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm)
{
  if (!dm->cdm) {
    PetscErrorCode ierr = DMDACreate2d(PETSC_COMM_SELF, DM_BOUNDARY_NONE, DM_BOUNDARY_NONE, DMDA_STENCIL_BOX,
                                       dm->M, dm->N, 1, 1, 2, 1, NULL, NULL, &dm->cdm);
    CHKERRQ(ierr);
  }
  *cdm = dm->cdm;
  return 0;
}
/* one rank: the ghosted (local) coordinate vector is the global one */
PetscErrorCode DMGetCoordinates(DM dm, Vec *c) { *c = dm->coords; return 0; }
PetscErrorCode DMGetCoordinatesLocal(DM dm, Vec *c) { *c = dm->coords; return 0; }

PetscErrorCode DMDASetUniformCoordinates(DM dm, PetscReal x0, PetscReal x1, PetscReal y0, PetscReal y1,
                                         PetscReal z0, PetscReal z1)
{
  PetscInt i, j;
  PetscReal hx, hy;
  (void)z0; (void)z1;
  if (!dm->coords) dm->coords = vec_new(dm->M * dm->N * 2, 2);
  hx = (dm->M > 1) ? (x1 - x0) / (dm->M - 1) : 0.0;
  hy = (dm->N > 1) ? (y1 - y0) / (dm->N - 1) : 0.0;
  for (j = 0; j < dm->N; j++) {
    for (i = 0; i < dm->M; i++) {
      dm->coords->array[2 * (i + j * dm->M) + 0] = x0 + i * hx;
      dm->coords->array[2 * (i + j * dm->M) + 1] = y0 + j * hy;
    }
  }
  return 0;
}

PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void *array)
{
  PetscInt j;
  free(dm->rows);
  dm->rows = (PetscScalar**)malloc(sizeof(PetscScalar*) * (size_t)dm->N);
  for (j = 0; j < dm->N; j++) dm->rows[j] = v->array + (size_t)j * dm->M * dm->dof;
  *(PetscScalar***)array = dm->rows;
  return 0;
}
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void *array) { (void)dm; (void)v; *(PetscScalar***)array = NULL; return 0; }

PetscErrorCode DMGetBoundingBox(DM dm, PetscReal gmin[], PetscReal gmax[])
{
  PetscInt i, j;
  Vec c = dm->coords;
  for (j = 0; j < 2; j++) { gmin[j] = PETSC_MAX_REAL; gmax[j] = PETSC_MIN_REAL; }
  for (i = 0; i < c->n; i += 2) {
    for (j = 0; j < 2; j++) {
      gmin[j] = PetscMin(gmin[j], c->array[i + j]);
      gmax[j] = PetscMax(gmax[j], c->array[i + j]);
    }
  }
  return 0;
}

PetscErrorCode DMDAGetGhostCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p)
{
  if (x) *x = 0;
  if (y) *y = 0;
  if (z) *z = 0;
  if (m) *m = dm->M;
  if (n) *n = dm->N;
  if (p) *p = 1;
  return 0;
}
PetscErrorCode DMDAGetCorners(DM dm, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p)
{
  return DMDAGetGhostCorners(dm, x, y, z, m, n, p);
}
PetscErrorCode DMDAGetInfo(DM dm, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m, PetscInt *n,
                           PetscInt *p, PetscInt *dof, PetscInt *s, DMBoundaryType *bx, DMBoundaryType *by,
                           DMBoundaryType *bz, DMDAStencilType *st)
{
  if (dim) *dim = 2;
  if (M) *M = dm->M;
  if (N) *N = dm->N;
  if (P) *P = 1;
  if (m) *m = 1;
  if (n) *n = 1;
  if (p) *p = 1;
  if (dof) *dof = dm->dof;
  if (s) *s = dm->s;
  if (bx) *bx = DM_BOUNDARY_NONE;
  if (by) *by = DM_BOUNDARY_NONE;
  if (bz) *bz = DM_BOUNDARY_NONE;
  if (st) *st = DMDA_STENCIL_BOX;
  return 0;
}
PetscErrorCode DMDAGetOwnershipRanges(DM dm, const PetscInt *lx[], const PetscInt *ly[], const PetscInt *lz[])
{
  if (lx) *lx = dm->lx;
  if (ly) *ly = dm->ly;
  if (lz) *lz = NULL;
  return 0;
}
PetscErrorCode DMDAGetLocalInfo(DM dm, DMDALocalInfo *info)
{
  memset(info, 0, sizeof(*info));
  info->dim = 2; info->dof = dm->dof; info->sw = dm->s;
  info->mx = dm->M; info->my = dm->N; info->mz = 1;
  info->xm = dm->M; info->ym = dm->N; info->zm = 1;
  info->gxm = dm->M; info->gym = dm->N; info->gzm = 1;
  info->da = dm;
  return 0;
}
PetscErrorCode DMDASetFieldName(DM dm, PetscInt f, const char name[]) { (void)dm; (void)f; (void)name; return 0; }

/* ------------------------------------------------------------------ */
/* dense Mat + KSPPREONLY/PCLU                                         */
/* ------------------------------------------------------------------ */
struct _p_Mat { struct _p_PetscObject hdr; PetscInt m, n; PetscScalar *v; /* column major */ };
struct _p_PC  { struct _p_PetscObject hdr; int type; /* 0 none, 1 lu */ };
struct _p_KSP { struct _p_PetscObject hdr; Mat A; struct _p_PC pc; PetscScalar *lu; PetscInt *piv; int factored; };

PetscErrorCode MatCreateSeqDense(MPI_Comm comm, PetscInt m, PetscInt n, PetscScalar *data, Mat *A)
{
  (void)comm;
  *A = (Mat)calloc(1, sizeof(struct _p_Mat));
  (*A)->m = m; (*A)->n = n;
  (*A)->v = (PetscScalar*)calloc((size_t)(m * n), sizeof(PetscScalar));
  if (data) memcpy((*A)->v, data, sizeof(PetscScalar) * (size_t)(m * n));
  return 0;
}
PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar v, InsertMode m)
{
  if (m == ADD_VALUES) A->v[i + j * A->m] += v;
  else A->v[i + j * A->m] = v;
  return 0;
}
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatCreateVecs(Mat A, Vec *right, Vec *left)
{
  if (right) *right = vec_new(A->n, 1);
  if (left) *left = vec_new(A->m, 1);
  return 0;
}
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n) { if (m) *m = A->m; if (n) *n = A->n; return 0; }
PetscErrorCode MatDestroy(Mat *A) { if (A && *A) { free((*A)->v); free(*A); *A = NULL; } return 0; }

PetscErrorCode KSPCreate(MPI_Comm comm, KSP *ksp) { (void)comm; *ksp = (KSP)calloc(1, sizeof(struct _p_KSP)); return 0; }
PetscErrorCode KSPSetOptionsPrefix(KSP ksp, const char prefix[]) { (void)ksp; (void)prefix; return 0; }
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat P) { (void)P; ksp->A = A; ksp->factored = 0; return 0; }
PetscErrorCode KSPSetType(KSP ksp, KSPType t)
{
  (void)ksp;
  if (strcmp(t, KSPPREONLY)) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_SUP, "KSP type %s not available", t);
  return 0;
}
PetscErrorCode KSPGetPC(KSP ksp, PC *pc) { *pc = &ksp->pc; return 0; }
PetscErrorCode PCSetType(PC pc, PCType t)
{
  if (!strcmp(t, PCLU)) pc->type = 1;
  else if (!strcmp(t, PCNONE)) pc->type = 0;
  else SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_SUP, "PC type %s not available", t);
  return 0;
}
PetscErrorCode KSPSetFromOptions(KSP ksp) { (void)ksp; return 0; }

/* LU with partial pivoting in the operation order of reference LAPACK
   dgetf2/dgetrf2: pivot = first max |a|, column scaled by the reciprocal of the
   pivot, rank-1 updates a_ij <- a_ij - l_ik*u_kj in ascending k. */
static PetscErrorCode lite_getrf(PetscInt n, PetscScalar *a, PetscInt *piv)
{
  PetscInt i, j, k, jp;
  for (j = 0; j < n; j++) {
    double amax = -1.0;
    jp = j;
    for (i = j; i < n; i++) if (fabs(a[i + j * n]) > amax) { amax = fabs(a[i + j * n]); jp = i; }
    piv[j] = jp;
    if (a[jp + j * n] == 0.0) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_USER, "zero pivot in LU at column %D", j);
    if (jp != j) {
      for (k = 0; k < n; k++) { double t = a[j + k * n]; a[j + k * n] = a[jp + k * n]; a[jp + k * n] = t; }
    }
    if (fabs(a[j + j * n]) >= DBL_MIN) {
      double r = 1.0 / a[j + j * n];
      for (i = j + 1; i < n; i++) a[i + j * n] *= r;
    } else {
      for (i = j + 1; i < n; i++) a[i + j * n] = a[i + j * n] / a[j + j * n];
    }
    for (k = j + 1; k < n; k++) {
      double t = -a[j + k * n];
      for (i = j + 1; i < n; i++) a[i + k * n] = a[i + k * n] + a[i + j * n] * t;
    }
  }
  return 0;
}

/* dgetrs('N'): dlaswp, then column-oriented unit-lower and upper solves (dtrsm) */
static void lite_getrs(PetscInt n, const PetscScalar *a, const PetscInt *piv, PetscScalar *b)
{
  PetscInt i, k;
  for (i = 0; i < n; i++) if (piv[i] != i) { double t = b[i]; b[i] = b[piv[i]]; b[piv[i]] = t; }
  for (k = 0; k < n; k++) {
    if (b[k] != 0.0) for (i = k + 1; i < n; i++) b[i] = b[i] - b[k] * a[i + k * n];
  }
  for (k = n - 1; k >= 0; k--) {
    if (b[k] != 0.0) {
      b[k] = b[k] / a[k + k * n];
      for (i = 0; i < k; i++) b[i] = b[i] - b[k] * a[i + k * n];
    }
  }
}

PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x)
{
  PetscInt n;
  PetscErrorCode ierr;
  if (!ksp->A) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONG, "KSPSetOperators not called");
  n = ksp->A->n;
  memcpy(x->array, b->array, sizeof(PetscScalar) * (size_t)n);
  if (ksp->pc.type == 0) return 0;
  if (!ksp->factored) {
    free(ksp->lu); free(ksp->piv);
    ksp->lu = (PetscScalar*)malloc(sizeof(PetscScalar) * (size_t)(n * n));
    ksp->piv = (PetscInt*)malloc(sizeof(PetscInt) * (size_t)n);
    memcpy(ksp->lu, ksp->A->v, sizeof(PetscScalar) * (size_t)(n * n));
    ierr = lite_getrf(n, ksp->lu, ksp->piv); CHKERRQ(ierr);
    ksp->factored = 1;
  }
  lite_getrs(n, ksp->lu, ksp->piv, x->array);
  return 0;
}
PetscErrorCode KSPComputeEigenvaluesExplicitly(KSP ksp, PetscInt n, PetscReal r[], PetscReal c[])
{
  (void)ksp; (void)n; (void)r; (void)c;
  SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "KSPComputeEigenvaluesExplicitly is not available in petsclite");
}
PetscErrorCode KSPDestroy(KSP *ksp)
{
  if (ksp && *ksp) { free((*ksp)->lu); free((*ksp)->piv); free(*ksp); *ksp = NULL; }
  return 0;
}
