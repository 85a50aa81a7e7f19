/*
 * ref_driver: runs the UNMODIFIED reference se2wave.c (compiled in place from
 * its own source tree against oracle/petsclite) on parameterised problems.
 *
 * TEST INFRASTRUCTURE ONLY: it produces golden vectors for tests/golden and a
 * cross-check of the oracle port.  Nothing in the product links it.
 *
 * Modes
 *   ref_driver demo  [options]            the reference's own main() (se2wave.c:4916-4951)
 *   ref_driver run   spec.txt outdir [options]
 *       a parameterised copy of the driver loop of se2wave_demo()
 *       (se2wave.c:4541-4807) calling the reference's own functions; writes
 *       binary FP64 dumps of the setup, receiver traces and final fields.
 *   ref_driver force spec.txt u.bin outdir [options]
 *       F = AssembleLinearForm_ElastoDynamics2d(u)  (se2wave.c:1285-1429)
 *   ref_driver stf   ricker|gaussian|yoffe a b c t0 dt n outfile
 *       the reference's STF evaluators (se2wave.c:3500-3822) on a time grid
 *
 * Receiver values are captured from the reference's own fprintf calls inside
 * RecordUVA_MultipleStations_NearestGLL_MPI (se2wave.c:2908-2962) and, with
 * the spec key "irec x y", RecordUV_interp (2445-2581) at full double
 * precision (the .dat text keeps only 9 significant digits).
 */
#include <petsc.h>
#include <petsctime.h>
#include <petscksp.h>
#include <petscdm.h>
#include <petscdmda.h>
#include <stdarg.h>

/* ---- fprintf capture ---------------------------------------------- */
/* two capture buffers: [0] the multi-station recorder, [1] RecordUV_interp */
static int     cap_on = 0, cap_sel = 0;
static double *cap_buf[2] = {NULL, NULL};
static size_t  cap_n[2] = {0, 0}, cap_cap[2] = {0, 0};

static void cap_push(double v)
{
  const int b = cap_sel;
  if (cap_n[b] == cap_cap[b]) {
    cap_cap[b] = cap_cap[b] ? 2 * cap_cap[b] : 4096;
    cap_buf[b] = (double*)realloc(cap_buf[b], cap_cap[b] * sizeof(double));
  }
  cap_buf[b][cap_n[b]++] = v;
}

int se2lite_fprintf(FILE *fp, const char *fmt, ...)
{
  va_list ap, aq;
  int r;
  va_start(ap, fmt);
  va_copy(aq, ap);
  r = vfprintf(fp, fmt, ap);
  va_end(ap);
  if (cap_on && fmt[0] != '#') {
    const char *c = fmt;
    while ((c = strchr(c, '%')) != NULL) {
      c++;
      if (*c == '%') { c++; continue; }
      while (*c && strchr("-+ #0123456789.l", *c)) c++;
      if (*c == 'e' || *c == 'f' || *c == 'g' || *c == 'E') cap_push(va_arg(aq, double));
      else if (*c == 'd' || *c == 'i') (void)va_arg(aq, int);
      else if (*c == 's') (void)va_arg(aq, char*);
      if (*c) c++;
    }
  }
  va_end(aq);
  return r;
}

#define fprintf se2lite_fprintf
#define main se2wave_reference_main
#include "se2wave.c"
#undef main
#undef fprintf

/* ---- problem spec --------------------------------------------------- */
#define MAXS 64
#define MAXR 4096
typedef struct {
  int mx, my, p;
  double scale[2], shift[2];
  double vp, vs, rho;
  char cell_file[1024];
  double cfl, dt, tmax;
  int nt;
  int nsrc;
  double src_xy[2 * MAXS], src_m[4 * MAXS];
  int stf_type[MAXS];          /* 0 ricker(t0,f0,amp) 1 gaussian(t0,omega,amp) 2 yoffe(tau_s,tau_r,dmax) */
  double stf_par[3 * MAXS];
  int nrec;
  double rec_xy[2 * MAXR];
  int perturb;
  double dvp, dvs, drho;
  int irec;                    /* one interpolating receiver (RecordUV_interp keeps one per process) */
  double irec_xy[2];
} Spec;

static int read_spec(const char *fname, Spec *sp)
{
  FILE *f = fopen(fname, "r");
  char key[128];
  int ns = 0, nr = 0;
  if (!f) { perror(fname); return 1; }
  memset(sp, 0, sizeof(*sp));
  sp->scale[0] = sp->scale[1] = 1.0;
  sp->cfl = 0.5; sp->nt = -1; sp->tmax = 0.4;
  while (fscanf(f, "%127s", key) == 1) {
    if (key[0] == '#') { int ch; while ((ch = fgetc(f)) != '\n' && ch != EOF) {} continue; }
    if (!strcmp(key, "mx")) fscanf(f, "%d", &sp->mx);
    else if (!strcmp(key, "my")) fscanf(f, "%d", &sp->my);
    else if (!strcmp(key, "p")) fscanf(f, "%d", &sp->p);
    else if (!strcmp(key, "scale")) fscanf(f, "%lf %lf", &sp->scale[0], &sp->scale[1]);
    else if (!strcmp(key, "shift")) fscanf(f, "%lf %lf", &sp->shift[0], &sp->shift[1]);
    else if (!strcmp(key, "vp")) fscanf(f, "%lf", &sp->vp);
    else if (!strcmp(key, "vs")) fscanf(f, "%lf", &sp->vs);
    else if (!strcmp(key, "rho")) fscanf(f, "%lf", &sp->rho);
    else if (!strcmp(key, "cell_file")) fscanf(f, "%1023s", sp->cell_file);
    else if (!strcmp(key, "cfl")) fscanf(f, "%lf", &sp->cfl);
    else if (!strcmp(key, "irec")) { sp->irec = 1; fscanf(f, "%lf %lf", &sp->irec_xy[0], &sp->irec_xy[1]); }
    else if (!strcmp(key, "perturb")) { sp->perturb = 1; fscanf(f, "%lf %lf %lf", &sp->dvp, &sp->dvs, &sp->drho); }
    else if (!strcmp(key, "dt")) fscanf(f, "%lf", &sp->dt);
    else if (!strcmp(key, "tmax")) fscanf(f, "%lf", &sp->tmax);
    else if (!strcmp(key, "nt")) fscanf(f, "%d", &sp->nt);
    else if (!strcmp(key, "src")) {
      char t[32];
      fscanf(f, "%lf %lf %lf %lf %lf %lf %31s %lf %lf %lf", &sp->src_xy[2 * ns], &sp->src_xy[2 * ns + 1],
             &sp->src_m[4 * ns], &sp->src_m[4 * ns + 1], &sp->src_m[4 * ns + 2], &sp->src_m[4 * ns + 3], t,
             &sp->stf_par[3 * ns], &sp->stf_par[3 * ns + 1], &sp->stf_par[3 * ns + 2]);
      sp->stf_type[ns] = !strcmp(t, "ricker") ? 0 : !strcmp(t, "gaussian") ? 1 : 2;
      ns++;
    } else if (!strcmp(key, "rec")) {
      fscanf(f, "%lf %lf", &sp->rec_xy[2 * nr], &sp->rec_xy[2 * nr + 1]);
      nr++;
    } else { fprintf(stderr, "unknown spec key %s\n", key); fclose(f); return 1; }
  }
  sp->nsrc = ns; sp->nrec = nr;
  fclose(f);
  return 0;
}

static int dump(const char *dir, const char *name, const void *p, size_t bytes)
{
  char path[2048];
  FILE *f;
  snprintf(path, sizeof(path), "%s/%s", dir, name);
  f = fopen(path, "wb");
  if (!f) { perror(path); return 1; }
  fwrite(p, 1, bytes, f);
  fclose(f);
  return 0;
}

static PetscErrorCode setup_ctx(const Spec *sp, SpecFECtx *_ctx)
{
  SpecFECtx ctx;
  PetscErrorCode ierr;
  ierr = SpecFECtxCreate(&ctx); CHKERRQ(ierr);
  ierr = SpecFECtxCreateMesh(ctx, 2, sp->mx, sp->my, PETSC_DECIDE, sp->p, 2); CHKERRQ(ierr);
  {
    PetscReal scale[2], shift[2];
    scale[0] = sp->scale[0]; scale[1] = sp->scale[1];
    shift[0] = sp->shift[0]; shift[1] = sp->shift[1];
    ierr = SpecFECtxScaleMeshCoords(ctx, scale, shift); CHKERRQ(ierr);
  }
  if (sp->cell_file[0]) {
    /* per-cell (vp, vs, rho): the conversion of se2wave.c:1165-1166 applied cell by cell */
    FILE *f = fopen(sp->cell_file, "rb");
    double *buf = (double*)malloc(sizeof(double) * 3 * (size_t)ctx->ne);
    PetscInt e;
    if (!f) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_FILE_OPEN, "cannot open %s", sp->cell_file);
    if (fread(buf, sizeof(double), 3 * (size_t)ctx->ne, f) != 3 * (size_t)ctx->ne) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_USER, "short cell file");
    fclose(f);
    for (e = 0; e < ctx->ne; e++) {
      PetscReal vp = buf[e], vs = buf[ctx->ne + e], rho = buf[2 * ctx->ne + e], mu, lambda;
      mu = vs * vs * rho;
      lambda = vp * vp * rho - 2.0 * mu;
      ctx->cell_data[e].lambda = lambda;
      ctx->cell_data[e].mu = mu;
      ctx->cell_data[e].rho = rho;
    }
    free(buf);
  } else if (sp->perturb) {
    ierr = SpecFECtxSetPerturbedMaterialProperties_Velocity(ctx, sp->vp, sp->dvp, sp->vs, sp->dvs, sp->rho, sp->drho); CHKERRQ(ierr);
  } else {
    ierr = SpecFECtxSetConstantMaterialProperties_Velocity(ctx, sp->vp, sp->vs, sp->rho); CHKERRQ(ierr);
  }
  *_ctx = ctx;
  return 0;
}

static PetscErrorCode dump_setup(SpecFECtx ctx, const char *outdir)
{
  PetscErrorCode ierr;
  PetscReal **D1;
  PetscInt nb, i, q;
  const PetscReal *LA_c;
  Vec coor;
  double *tab;
  dump(outdir, "xi.bin", ctx->xi1d, sizeof(double) * ctx->npe_1d);
  dump(outdir, "w1d.bin", ctx->w1d, sizeof(double) * ctx->npe_1d);
  dump(outdir, "w.bin", ctx->w, sizeof(double) * ctx->npe);
  ierr = TabulateBasisDerivatives1d_CLEGENDRE(ctx->npe_1d, ctx->xi1d, ctx->basisorder, &nb, &D1); CHKERRQ(ierr);
  tab = (double*)malloc(sizeof(double) * ctx->npe * ctx->npe);
  for (q = 0; q < ctx->npe_1d; q++) for (i = 0; i < nb; i++) tab[q * nb + i] = D1[q][i];
  dump(outdir, "D.bin", tab, sizeof(double) * nb * nb);
  for (q = 0; q < ctx->npe_1d; q++) free(D1[q]);
  free(D1);
  for (q = 0; q < ctx->npe; q++) for (i = 0; i < ctx->npe; i++) tab[q * ctx->npe + i] = ctx->dN_dxi[q][i];
  dump(outdir, "dN_dxi.bin", tab, sizeof(double) * ctx->npe * ctx->npe);
  for (q = 0; q < ctx->npe; q++) for (i = 0; i < ctx->npe; i++) tab[q * ctx->npe + i] = ctx->dN_deta[q][i];
  dump(outdir, "dN_deta.bin", tab, sizeof(double) * ctx->npe * ctx->npe);
  free(tab);
  ierr = DMGetCoordinates(ctx->dm, &coor); CHKERRQ(ierr);
  ierr = VecGetArrayRead(coor, &LA_c); CHKERRQ(ierr);
  dump(outdir, "coords.bin", LA_c, sizeof(double) * 2 * ctx->nx_g * ctx->ny_g);
  ierr = VecRestoreArrayRead(coor, &LA_c); CHKERRQ(ierr);
  {
    double *cd = (double*)malloc(sizeof(double) * 3 * ctx->ne);
    PetscInt e;
    for (e = 0; e < ctx->ne; e++) { cd[e] = ctx->cell_data[e].lambda; cd[ctx->ne + e] = ctx->cell_data[e].mu; cd[2 * ctx->ne + e] = ctx->cell_data[e].rho; }
    dump(outdir, "cell_lmr.bin", cd, sizeof(double) * 3 * ctx->ne);
    free(cd);
  }
  return 0;
}

static PetscErrorCode create_stf(const Spec *sp, int s, SeismicSTF *stf)
{
  PetscErrorCode ierr;
  const double *a = &sp->stf_par[3 * s];
  if (sp->stf_type[s] == 0) { ierr = SeismicSTFCreate_Ricker(a[0], a[1], a[2], stf); CHKERRQ(ierr); }
  else if (sp->stf_type[s] == 1) { ierr = SeismicSTFCreate_Gaussian(a[0], a[1], a[2], stf); CHKERRQ(ierr); }
  else { ierr = SeismicSTFCreate_TriRegYoffe(a[0], a[1], a[2], stf); CHKERRQ(ierr); }
  return 0;
}

/* copy of the se2wave_demo() set-up and time loop (se2wave.c:4594-4775) with the
   hard-coded physics replaced by the spec; every call is the reference's own. */
static PetscErrorCode run(const Spec *sp, const char *outdir)
{
  PetscErrorCode ierr;
  SpecFECtx ctx;
  Vec u, v, a, f, g, Md;
  SeismicSource *src;
  SeismicSTF *stf;
  PetscReal time, dt, time_max;
  PetscInt k, nt, s, nsteps = 0;
  PetscReal nrm, max, min;
  PetscBool ignore_receiver_output = PETSC_FALSE;
  FILE *flog;
  char path[2048];

  ierr = PetscOptionsGetBool(NULL, NULL, "-ignore_receiver_output", &ignore_receiver_output, NULL); CHKERRQ(ierr);
  ierr = setup_ctx(sp, &ctx); CHKERRQ(ierr);
  ierr = dump_setup(ctx, outdir); CHKERRQ(ierr);

  ierr = DMCreateGlobalVector(ctx->dm, &u); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &v); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &a); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &f); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &g); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &Md); CHKERRQ(ierr);
  ierr = VecZeroEntries(u); CHKERRQ(ierr);
  ierr = AssembleBilinearForm_Mass2d(ctx, Md); CHKERRQ(ierr);
  dump(outdir, "mass.bin", Md->array, sizeof(double) * Md->n);

  ierr = PetscMalloc1(sp->nsrc, &src); CHKERRQ(ierr);
  ierr = PetscMalloc1(sp->nsrc, &stf); CHKERRQ(ierr);
  for (s = 0; s < sp->nsrc; s++) {
    PetscReal coor[2], moment[4];
    coor[0] = sp->src_xy[2 * s]; coor[1] = sp->src_xy[2 * s + 1];
    moment[0] = sp->src_m[4 * s]; moment[1] = sp->src_m[4 * s + 1];
    moment[2] = sp->src_m[4 * s + 2]; moment[3] = sp->src_m[4 * s + 3];
    ierr = SeismicSourceCreate(ctx, SOURCE_TYPE_MOMENT, SOURCE_IMPL_NEAREST_QPOINT, coor, moment, &src[s]); CHKERRQ(ierr);
  }
  for (s = 0; s < sp->nsrc; s++) { ierr = SeismicSourceSetup(src[s]); CHKERRQ(ierr); }
  {
    /* source representation: element index, closest GLL, 2*npe element values */
    double *sv = (double*)calloc((size_t)(sp->nsrc * 2 * ctx->npe + 1), sizeof(double));
    int *si = (int*)calloc((size_t)(2 * sp->nsrc + 1), sizeof(int));
    for (s = 0; s < sp->nsrc; s++) {
      PointwiseContext *pw = (PointwiseContext*)src[s]->data;
      memcpy(&sv[s * 2 * ctx->npe], pw->element_values, sizeof(double) * 2 * ctx->npe);
      si[2 * s] = src[s]->element_index;
      si[2 * s + 1] = src[s]->closest_gll;
    }
    dump(outdir, "src_values.bin", sv, sizeof(double) * sp->nsrc * 2 * ctx->npe);
    dump(outdir, "src_index.bin", si, sizeof(int) * 2 * sp->nsrc);
    free(sv); free(si);
  }
  ierr = SeismicSourceEvaluate(0.0, sp->nsrc, src, NULL, g); CHKERRQ(ierr);
  dump(outdir, "g_unit.bin", g->array, sizeof(double) * g->n);
  for (s = 0; s < sp->nsrc; s++) { ierr = create_stf(sp, s, &stf[s]); CHKERRQ(ierr); }

  time = 0.0;
  time_max = sp->tmax;
  ierr = ElastoDynamicsComputeTimeStep_2d(ctx, &dt); CHKERRQ(ierr);
  dump(outdir, "dt_cfl.bin", &dt, sizeof(double));
  dt = dt * sp->cfl;
  if (sp->dt > 0.0) dt = sp->dt;
  nt = (PetscInt)(time_max / dt) + 4;
  if (sp->nt >= 0) nt = sp->nt;

  snprintf(path, sizeof(path), "%s/norms.txt", outdir);
  flog = fopen(path, "w");
  cap_on = 1;
  for (k = 1; k <= nt; k++) {
    time = time + dt;
    ierr = VecAXPY(u, dt, v); CHKERRQ(ierr);
    ierr = VecAXPY(u, 0.5 * dt * dt, a); CHKERRQ(ierr);
    ierr = VecAXPY(v, 0.5 * dt, a); CHKERRQ(ierr);
    ierr = SeismicSourceEvaluate(time, sp->nsrc, src, stf, g); CHKERRQ(ierr);
    ierr = AssembleLinearForm_ElastoDynamics2d(ctx, u, f); CHKERRQ(ierr);
    ierr = VecAXPY(f, 1.0, g); CHKERRQ(ierr);
    ierr = VecPointwiseDivide(a, f, Md); CHKERRQ(ierr);
    ierr = VecAXPY(v, 0.5 * dt, a); CHKERRQ(ierr);
    nsteps = k;
    if (k % 100 == 0 && flog) {
      double r[6];
      VecNorm(u, NORM_2, &nrm); VecMin(u, 0, &min); VecMax(u, 0, &max);
      r[0] = max; r[1] = min; r[2] = nrm;
      VecNorm(v, NORM_2, &nrm); VecMin(v, 0, &min); VecMax(v, 0, &max);
      r[3] = max; r[4] = min; r[5] = nrm;
      fprintf(flog, "%d %.17g %.17g %.17g %.17g %.17g %.17g\n", (int)k, r[0], r[1], r[2], r[3], r[4], r[5]);
    }
    if (!ignore_receiver_output && sp->nrec > 0) {
      ierr = RecordUVA_MultipleStations_NearestGLL(ctx, time, sp->nrec, (PetscReal*)sp->rec_xy, u, v, a); CHKERRQ(ierr);
    }
    if (sp->irec) {
      PetscReal xr[2];
      xr[0] = sp->irec_xy[0]; xr[1] = sp->irec_xy[1];
      cap_sel = 1;
      ierr = RecordUV_interp(ctx, time, xr, u, v); CHKERRQ(ierr);
      cap_sel = 0;
    }
    if (time >= time_max) break;
  }
  cap_on = 0;
  if (flog) fclose(flog);
  {
    double meta[4];
    meta[0] = dt; meta[1] = time; meta[2] = (double)nsteps; meta[3] = (double)nt;
    dump(outdir, "run_meta.bin", meta, sizeof(meta));
  }
  dump(outdir, "trace_capture.bin", cap_buf[0], sizeof(double) * cap_n[0]);
  if (sp->irec) dump(outdir, "interp_capture.bin", cap_buf[1], sizeof(double) * cap_n[1]);
  dump(outdir, "u.bin", u->array, sizeof(double) * u->n);
  dump(outdir, "v.bin", v->array, sizeof(double) * v->n);
  dump(outdir, "a.bin", a->array, sizeof(double) * a->n);
  return 0;
}

static PetscErrorCode force(const Spec *sp, const char *ufile, const char *outdir)
{
  PetscErrorCode ierr;
  SpecFECtx ctx;
  Vec u, f;
  FILE *fu;
  ierr = setup_ctx(sp, &ctx); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &u); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &f); CHKERRQ(ierr);
  fu = fopen(ufile, "rb");
  if (!fu) SETERRQ1(PETSC_COMM_SELF, PETSC_ERR_FILE_OPEN, "cannot open %s", ufile);
  if (fread(u->array, sizeof(double), (size_t)u->n, fu) != (size_t)u->n) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_USER, "short u file");
  fclose(fu);
  ierr = AssembleLinearForm_ElastoDynamics2d(ctx, u, f); CHKERRQ(ierr);
  dump(outdir, "force.bin", f->array, sizeof(double) * f->n);
  return 0;
}

/* assembled source vector of the spec's first source by one of the reference's
   alternative implementations (ElastoDynamicsSourceSetup's switch, 2244-2263) */
static PetscErrorCode srcvec(const Spec *sp, int impl, const char *outdir)
{
  PetscErrorCode ierr;
  SpecFECtx ctx;
  Vec g;
  PetscReal xs[2], m[4];
  int i;
  ierr = setup_ctx(sp, &ctx); CHKERRQ(ierr);
  ierr = DMCreateGlobalVector(ctx->dm, &g); CHKERRQ(ierr);
  xs[0] = sp->src_xy[0]; xs[1] = sp->src_xy[1];
  for (i = 0; i < 4; i++) m[i] = sp->src_m[i];
  if (impl == 0) { ierr = AssembleLinearForm_ElastoDynamicsMomentDirac2d(ctx, 1, xs, m, g); CHKERRQ(ierr); }
  else if (impl == 2) { ierr = AssembleLinearForm_ElastoDynamicsMomentDirac2d_Kernel_CSpline(ctx, 1, xs, m, g); CHKERRQ(ierr); }
  else if (impl == 3) { ierr = AssembleLinearForm_ElastoDynamicsMomentDirac2d_P0(ctx, 1, xs, m, g); CHKERRQ(ierr); }
  else SETERRQ(PETSC_COMM_SELF, PETSC_ERR_USER, "implementation 0, 2 or 3");
  dump(outdir, "g.bin", g->array, sizeof(double) * g->n);
  return 0;
}

static PetscErrorCode stf_table(int argc, char **argv)
{
  SeismicSTF stf;
  PetscErrorCode ierr;
  double a = atof(argv[3]), b = atof(argv[4]), c = atof(argv[5]);
  double t0 = atof(argv[6]), dt = atof(argv[7]), time;
  int n = atoi(argv[8]), k;
  double *out = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  (void)argc;
  if (!strcmp(argv[2], "ricker")) { ierr = SeismicSTFCreate_Ricker(a, b, c, &stf); CHKERRQ(ierr); }
  else if (!strcmp(argv[2], "gaussian")) { ierr = SeismicSTFCreate_Gaussian(a, b, c, &stf); CHKERRQ(ierr); }
  else { ierr = SeismicSTFCreate_TriRegYoffe(a, b, c, &stf); CHKERRQ(ierr); }
  time = t0;
  for (k = 0; k < n; k++) {
    double val;
    ierr = SeismicSTFEvaluate(stf, time, &val); CHKERRQ(ierr);
    out[2 * k] = time; out[2 * k + 1] = val;
    time = time + dt;
  }
  {
    FILE *f = fopen(argv[9], "wb");
    fwrite(out, sizeof(double), 2 * (size_t)n, f);
    fclose(f);
  }
  free(out);
  ierr = SeismicSTFDestroy(&stf); CHKERRQ(ierr);
  return 0;
}

int main(int argc, char **argv)
{
  Spec sp;
  if (argc < 2) {
    fprintf(stderr, "usage: %s demo|run|force|stf ...\n", argv[0]);
    return 1;
  }
  if (!strcmp(argv[1], "demo")) {
    argv[1] = argv[0];
    return se2wave_reference_main(argc - 1, argv + 1);
  }
  if (!strcmp(argv[1], "run") && argc >= 4) {
    PetscLiteOptionsSet(argc - 3, argv + 3);
    if (read_spec(argv[2], &sp)) return 1;
    return run(&sp, argv[3]) ? 2 : 0;
  }
  if (!strcmp(argv[1], "force") && argc >= 5) {
    PetscLiteOptionsSet(argc - 4, argv + 4);
    if (read_spec(argv[2], &sp)) return 1;
    return force(&sp, argv[3], argv[4]) ? 2 : 0;
  }
  if (!strcmp(argv[1], "stf") && argc >= 10) return stf_table(argc, argv) ? 2 : 0;
  if (!strcmp(argv[1], "srcvec") && argc >= 5) {
    PetscLiteOptionsSet(argc - 4, argv + 4);
    if (read_spec(argv[2], &sp)) return 1;
    return srcvec(&sp, atoi(argv[3]), argv[4]) ? 2 : 0;
  }
  fprintf(stderr, "bad arguments\n");
  return 1;
}
