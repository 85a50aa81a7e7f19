/*
 * se2wave_gpu -- drop-in for the se2wave executable (Nicolucas/se2dr_fork) with
 * the time loop on one GB300.
 *
 * Same command line as the reference (main, se2wave.c:4916-4951, and
 * se2wave_demo, 4541-4807): -mx -my -bdegree -tmax -dt -nt -of
 * -ignore_receiver_output -use_nearest_internal_gll -verify_stf [-stf_ricker |
 * -stf_yoffe -stf.yoffe.tau_s -stf.yoffe.tau_r -stf.yoffe.d_max].  With no other
 * options it runs the reference demo's physics and prints the same lines and
 * writes the same closestqpsource-receiverCP-uva-*.dat / .mpimeta files.
 *
 * Additions (defaults reproduce the demo): -precision fp64|fp32_df|fp32_kahan|fp32
 * (fp64 is bit-identical to the reference), -cfl (0.5), -Lx -Ly (2000),
 * -x0 -y0 (-1000), -vp -vs -rho, -cells file (per-cell vp,vs,rho doubles),
 * -problem demo|explosion64|grf2048, -rec_file (x y per line), -block (steps per
 * device batch, default 100), -interp_receiver x,y (the interpolating receiver of
 * RecordUV_interp, se2wave.c:2445-2581: its file and stdout line).
 *
 * The host set-up (libse2host) runs in FP64 on the CPU; the loop runs in
 * libse2gpu through its C-ABI.  There is no CPU fallback.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "se2gpu.h"
#include "se2host.h"

static int g_argc;
static char **g_argv;

static const char *opt_val(const char *name, int *found)
{
  int i;
  *found = 0;
  for (i = g_argc - 1; i >= 1; i--) {
    if (!strcmp(g_argv[i], name)) {
      *found = 1;
      if (i + 1 < g_argc) {
        const char *v = g_argv[i + 1];
        if (v[0] != '-' || (v[1] >= '0' && v[1] <= '9') || v[1] == '.') return v;
      }
      return NULL;
    }
  }
  return NULL;
}
static int opt_int(const char *name, int *v)
{
  int f; const char *s = opt_val(name, &f);
  if (f && s) { *v = (int)strtol(s, NULL, 10); return 1; }
  return 0;
}
static int opt_real(const char *name, double *v)
{
  int f; const char *s = opt_val(name, &f);
  if (f && s) { *v = strtod(s, NULL); return 1; }
  return 0;
}
static int opt_bool(const char *name, int def)
{
  int f; const char *s = opt_val(name, &f);
  if (!f) return def;
  if (s && (!strcmp(s, "0") || !strcasecmp(s, "false") || !strcasecmp(s, "no"))) return 0;
  return 1;
}
static const char *opt_str(const char *name, const char *def)
{
  int f; const char *s = opt_val(name, &f);
  return (f && s) ? s : def;
}

#define CHECK(call)                                                            \
  do {                                                                         \
    int rc_ = (call);                                                          \
    if (rc_ < 0) { fprintf(stderr, "[se2wave_gpu] error: %s\n", errmsg(h)); return 1; } \
  } while (0)
static const char *errmsg(se2gpu_solver *h) { return h ? se2gpu_last_error(h) : se2gpu_create_error(); }

/* test_SeismicSTF (se2wave.c:4809-4914): tabulate an STF to a log file */
static int verify_stf(void)
{
  int is_ricker = opt_bool("-stf_ricker", 0), is_yoffe = opt_bool("-stf_yoffe", 0), type;
  double par[3], time = 0.0, tmax = 2.0, dt = 1.0e-6;
  const char *fname;
  FILE *fp;
  long k;
  if (!is_ricker && !is_yoffe) { fprintf(stderr, "No STF implementation specified. Use one of { -stf_ricker , -stf_yoffe }\n"); return 1; }
  if (is_ricker) {
    double t0 = 0.15, freq = 12.0, amp = 1.0;
    opt_real("-stf.ricker.t0", &t0); opt_real("-stf.ricker.freq", &freq); opt_real("-stf.ricker.amp", &amp);
    /* the reference builds the Ricker STF from the literals (0.15, 12, 1) and only prints the options */
    par[0] = 0.15; par[1] = 12.0; par[2] = 1.0; type = SE2_STF_RICKER;
    fname = "SeismicSTF_Ricker.log";
    fp = fopen(fname, "w");
    if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname); return 1; }
    fprintf(fp, "# --------------------------------\n# SeismicSTF\n#   Parameters\n#     type  \"Ricker\"\n");
    fprintf(fp, "#     t0    %+1.12e (sec)\n#     freq  %+1.12e (Hz)\n#     amp   %+1.12e\n", t0, freq, amp);
    fprintf(fp, "# --------------------------------\n");
  }
  if (is_yoffe) {
    double tau_S = 0.15, tau_R = 1.0, D_max = 1.1, v;
    opt_real("-stf.yoffe.tau_s", &tau_S); opt_real("-stf.yoffe.tau_r", &tau_R); opt_real("-stf.yoffe.d_max", &D_max);
    par[0] = tau_S; par[1] = tau_R; par[2] = D_max; type = SE2_STF_YOFFE;
    if (se2_stf_eval(type, par, 1.0e30, &v)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
    fname = "SeismicSTF_Yoffe.log";
    fp = fopen(fname, "w");
    if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname); return 1; }
    fprintf(fp, "# --------------------------------\n# SeismicSTF\n#   Parameters\n#     type  \"Yoffe\"\n");
    fprintf(fp, "#     tau_S %+1.12e\n#     tau_R %+1.12e\n#     D_max %+1.12e\n", tau_S, tau_R, D_max);
    fprintf(fp, "# --------------------------------\n");
  }
  opt_real("-tmax", &tmax);
  printf("[se2wave] Requested time period: %1.4e\n", tmax);
  opt_real("-dt", &dt);
  printf("[se2wave] Using time step size: %1.4e\n", dt);
  for (k = 0;; k++) {
    double v;
    if (se2_stf_eval(type, par, time, &v)) { fprintf(stderr, "%s\n", se2_host_last_error()); fclose(fp); return 1; }
    fprintf(fp, "%+1.6e %+1.12e\n", time, v);
    time = time + dt;
    if (time >= tmax) break;
  }
  printf("[step %9ld] time = %1.4e : dt = %1.4e \n", k, time, dt);
  fclose(fp);
  return 0;
}

static double *read_doubles(const char *fname, long n)
{
  FILE *f = fopen(fname, "rb");
  double *b;
  if (!f) return NULL;
  b = (double*)malloc(sizeof(double) * (size_t)n);
  if (fread(b, sizeof(double), (size_t)n, f) != (size_t)n) { free(b); b = NULL; }
  fclose(f);
  return b;
}

int main(int argc, char **argv)
{
  int mx = 8, my, p = 2, nt_opt = -1, of = 5000, block = 100, r, s, ignore_rec, precision, dump_ic, ckpt_every = 0;
  const char *restart;
  int sp_src_impl = -1, src_impl_raw = -1, ninterp = 0, nrec_all;
  double sp_sm_h = 0.0, interp_xy[2] = {0.0, 0.0};
  char fname_interp[512];
  double dvp = 0.0, dvs = 0.0, drho = 0.0;
  int perturb;
  double tmax = 0.4, dt_opt = 0.0, cfl = 0.5, Lx = 2000.0, Ly, x0 = -1000.0, y0, vp = 4746.3670317412243,
         vs = 2740.2554625435928, rho = 1000.0;
  const char *problem, *prec_s, *rec_file, *cells;
  se2_spec sp;
  se2_setup *su = NULL;
  se2gpu_problem pr;
  se2gpu_solver *h = NULL;
  double src_xy[8], src_m[16], stf_par[12], *rec_xy = NULL, *cell = NULL;
  int stf_type[4], nsrc, nrec;
  char fname[512], meta[512], fname_vts[512];
  FILE *fp;
  long k, nsteps;
  double time = 0.0;

  g_argc = argc; g_argv = argv;
  opt_int("-mx", &mx);
  my = mx;
  opt_int("-my", &my);
  if (opt_bool("-verify_stf", 0)) return verify_stf();

  ignore_rec = opt_bool("-ignore_receiver_output", 0);
  dump_ic = opt_bool("-dump_ic_src", 0);
  opt_int("-bdegree", &p);
  problem = opt_str("-problem", "demo");
  prec_s = opt_str("-precision", "fp64");
  precision = !strcmp(prec_s, "fp64") ? SE2GPU_FP64 : !strcmp(prec_s, "fp32_df") ? SE2GPU_FP32_DF
            : !strcmp(prec_s, "fp32_kahan") ? SE2GPU_FP32_KAHAN
            : !strcmp(prec_s, "fp32") ? SE2GPU_FP32 : -1;
  if (precision < 0) { fprintf(stderr, "unknown -precision %s\n", prec_s); return 1; }

  /* physics: the demo's (se2wave.c:4575-4697) unless a preset or option replaces it */
  nsrc = 2;
  src_xy[0] = 0.1; src_xy[1] = 100.1;
  src_m[0] = 1000.0; src_m[1] = 0.0; src_m[2] = 0.0; src_m[3] = 1000.0;
  src_xy[2] = 400.1; src_xy[3] = 400.1;
  src_m[4] = 0.0; src_m[5] = -1000.0; src_m[6] = 1000.0; src_m[7] = 0.0;
  stf_type[0] = stf_type[1] = SE2_STF_RICKER;
  stf_par[0] = 0.15; stf_par[1] = 12.0; stf_par[2] = 1.0;
  stf_par[3] = 0.25; stf_par[4] = 4.0; stf_par[5] = 1.0;
  nrec = 3;
  rec_xy = (double*)malloc(sizeof(double) * 6);
  rec_xy[0] = 100.0; rec_xy[1] = 200.0; rec_xy[2] = 150.0; rec_xy[3] = 200.0; rec_xy[4] = 180.0; rec_xy[5] = 200.0;
  if (!strcmp(problem, "explosion64") || !strcmp(problem, "grf2048")) {
    int grf = !strcmp(problem, "grf2048");
    nsrc = 1;
    src_xy[0] = 0.0; src_xy[1] = 0.0;
    src_m[0] = 1e15; src_m[1] = 0.0; src_m[2] = 0.0; src_m[3] = 1e15;
    stf_par[0] = 0.15; stf_par[1] = grf ? 8.0 : 10.0; stf_par[2] = 1.0;
    vp = grf ? 5000.0 : 6000.0; vs = grf ? 5000.0 / 1.73 : 3464.0; rho = 2700.0;
    cfl = 0.2;
    if (grf) {
      Lx = 20000.0; x0 = -10000.0;
      nrec = 64;
      free(rec_xy);
      rec_xy = (double*)malloc(sizeof(double) * 2 * nrec);
      for (r = 0; r < nrec; r++) { rec_xy[2 * r] = -8000.0 + 16000.0 * r / 63.0; rec_xy[2 * r + 1] = 2500.0; }
    } else {
      nrec = 1;
      rec_xy[0] = 500.0; rec_xy[1] = 500.0;
    }
  }
  Ly = Lx; y0 = x0;
  opt_real("-Lx", &Lx); opt_real("-Ly", &Ly); opt_real("-x0", &x0); opt_real("-y0", &y0);
  opt_real("-vp", &vp); opt_real("-vs", &vs); opt_real("-rho", &rho); opt_real("-cfl", &cfl);
  /* -dvp -dvs -drho: per-cell materials from SpecFECtxSetPerturbedMaterialProperties_Velocity */
  perturb = opt_real("-dvp", &dvp) | opt_real("-dvs", &dvs) | opt_real("-drho", &drho);
  opt_real("-tmax", &tmax);
  rec_file = opt_str("-rec_file", NULL);
  if (rec_file) {
    FILE *rf = fopen(rec_file, "r");
    double x, y;
    if (!rf) { fprintf(stderr, "cannot open %s\n", rec_file); return 1; }
    nrec = 0;
    free(rec_xy);
    rec_xy = NULL;
    while (fscanf(rf, "%lf %lf", &x, &y) == 2) {
      rec_xy = (double*)realloc(rec_xy, sizeof(double) * 2 * (nrec + 1));
      rec_xy[2 * nrec] = x; rec_xy[2 * nrec + 1] = y;
      nrec++;
    }
    fclose(rf);
  }
  cells = opt_str("-cells", NULL);
  if (cells) {
    cell = read_doubles(cells, 3L * mx * my);
    if (!cell) { fprintf(stderr, "cannot read %ld doubles from %s\n", 3L * mx * my, cells); return 1; }
  } else if (!strcmp(problem, "grf2048")) {
    cell = (double*)malloc(sizeof(double) * 3 * (size_t)mx * my);
    if (se2_gaussian_random_field(mx, my, 5000.0, 0.1, 8.0, 2048ULL, cell)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
    for (k = 0; k < (long)mx * my; k++) { cell[(long)mx * my + k] = cell[k] / 1.73; cell[2L * mx * my + k] = 2700.0; }
  }

  memset(&sp, 0, sizeof(sp));
  sp.mx = mx; sp.my = my; sp.p = p;
  sp.scale[0] = Lx; sp.scale[1] = Ly; sp.shift[0] = x0; sp.shift[1] = y0;
  if (cell) { sp.cell_vp = cell; sp.cell_vs = cell + (long)mx * my; sp.cell_rho = cell + 2L * mx * my; }
  sp.vp = vp; sp.vs = vs; sp.rho = rho;
  sp.cfl = cfl; sp.tmax = tmax; sp.nt = -1; sp.dt = 0.0;
  if (opt_real("-dt", &dt_opt)) sp.dt = dt_opt;
  if (opt_int("-nt", &nt_opt)) sp.nt = nt_opt;
  opt_int("-of", &of);
  if (of < 1) { fprintf(stderr, "-of must be at least 1\n"); return 1; }
  opt_int("-block", &block);
  opt_int("-checkpoint_every", &ckpt_every);
  {
    int impl = -1;
    double h = 0.0;
    if (opt_int("-source_impl", &impl)) {  /* ElastoDynamicsSetSourceImplementation (2202-2230) */
      const char *nm[4] = {"pointwise evaluation", "closest internal basis", "cspline kernel", "P0"};
      if (impl < 0 || impl > 3) { fprintf(stderr, "-source_impl: valid choices are 0,1,2,3\n"); return 1; }
      printf("  [source implementation]: processed from command line args\n");
      printf("  [source implementation]: %s\n", nm[impl]);
      sp_src_impl = (impl == 1) ? -1 : impl;   /* 1 = the nearest interior GLL point, the default path */
      src_impl_raw = impl;
    }
    if (opt_real("-sm_h", &h)) sp_sm_h = h;
  }
  restart = opt_str("-restart", NULL);
  {
    const char *ir = opt_str("-interp_receiver", NULL);
    if (ir) {
      if (sscanf(ir, "%lf,%lf", &interp_xy[0], &interp_xy[1]) != 2) { fprintf(stderr, "-interp_receiver: expected x,y\n"); return 1; }
      ninterp = 1;
    }
  }
  if (block < 1) block = 1;
  sp.nearest_internal_gll = opt_bool("-use_nearest_internal_gll", 1);
  sp.nsrc = nsrc; sp.src_xy = src_xy; sp.src_m = src_m; sp.stf_type = stf_type; sp.stf_par = stf_par;
  sp.nrec = nrec; sp.rec_xy = rec_xy;
  if (!cell && perturb) { sp.perturb = 1; sp.dvp = dvp; sp.dvs = dvs; sp.drho = drho; }
  sp.src_impl = sp_src_impl;
  sp.sm_h = sp_sm_h;
  sp.ninterp = ninterp; sp.interp_xy = interp_xy;

  if (!cell && perturb) {  /* se2wave.c:1228-1230 */
    printf("  [material]     Vp0 = %1.8e : delta = %+1.8e\n", vp, dvp);
    printf("  [material]     Vs0 = %1.8e : delta = %+1.8e\n", vs, dvs);
    printf("  [material]    rho0 = %1.8e : delta = %+1.8e\n", rho, drho);
  } else if (!cell) {
    double mu = vs * vs * rho, lambda = vp * vp * rho - 2.0 * mu;
    printf("  [material]     Vp = %1.8e\n", vp);
    printf("  [material]     Vs = %1.8e\n", vs);
    printf("  [material] lambda = %1.8e\n", lambda);
    printf("  [material]     mu = %1.8e\n", mu);
    printf("  [material]    rho = %1.8e\n", rho);
  }
  if (se2_setup_create(&sp, &su)) { fprintf(stderr, "[se2wave_gpu] set-up error: %s\n", se2_host_last_error()); return 1; }
  for (s = 0; s < nsrc && sp.src_impl < 0; s++) {  /* the demo prints each moment, then SeismicSourceCreate's lines (4626-4652) */
    int g = su->src_gll[s], e = su->src_elem[s], gi = g % su->n1, gj = g / su->n1;
    printf("Moment: [ %+1.2e , %+1.2e ; %+1.2e , %+1.2e ]\n", src_m[4 * s], src_m[4 * s + 1], src_m[4 * s + 2], src_m[4 * s + 3]);
    printf("[SeismicSource] source (%+1.4e,%+1.4e) --> element %d | rank 0\n", src_xy[2 * s], src_xy[2 * s + 1], e);
    printf("[SeismicSource] source --> closest_gll %d xi: (%+1.4e,%+1.4e) [%d,%d] \n", g, su->xi[gi], su->xi[gj], gi, gj);
    printf("[SeismicSource] source --> closest_gll %d x:  (%+1.4e,%+1.4e)\n", g,
           su->xnode[(e % mx) * p + gi], su->ynode[(e / mx) * p + gj]);
  }
  printf("[se2wave] Requested time period: %1.4e\n", tmax);
  printf("[se2wave] Using time step size: %1.4e\n", su->dt);
  printf("[se2wave] Estimated number of time steps: %ld\n", su->nt);

  if (dump_ic) {  /* initial displacement (zero), se2wave.c:4606-4610 */
    double *u0 = (double*)calloc((size_t)su->nnodes * 2, sizeof(double));
    const char *nm[1] = {"disp"};
    const double *vv[1] = {u0};
    if (se2_write_vts(su, "uva.vts", 1, nm, vv)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
    free(u0);
  }

  memset(&pr, 0, sizeof(pr));
  pr.mx = mx; pr.my = my; pr.p = p; pr.dt = su->dt;
  pr.D = su->D; pr.wq = su->wq; pr.w1d = su->w1d; pr.J00 = su->J00; pr.J11 = su->J11; pr.iJ00 = su->iJ00; pr.iJ11 = su->iJ11;
  pr.lambda = su->lambda; pr.mu = su->mu; pr.mass = su->mass;
  pr.nsrc = su->nsrc; pr.src_elem = su->src_elem; pr.src_vals = su->src_vals;
  pr.nrec = ignore_rec ? 0 : su->nrec; pr.rec_node = su->rec_node; pr.rec_elem = su->rec_elem; pr.rec_gll = su->rec_gll;
  if (block > 100) block = 100 * (block / 100);
  CHECK(se2gpu_create(&pr, precision, block + 1, &h));

  /* receiver files: header of RecordUVA_MultipleStations_NearestGLL_MPI (2808-2882) */
  snprintf(fname, sizeof(fname), "closestqpsource-receiverCP-uva-%dx%d-p%d-rank%d.dat", mx, my, p, 0);
  snprintf(meta, sizeof(meta), "closestqpsource-receiverCP-uva-%dx%d-p%d.mpimeta", mx, my, p);
  nrec_all = ignore_rec ? 0 : su->nrec;   /* the stations, then the interpolating receiver's element nodes */
  {  /* RecordUV_interp's file name by source implementation (2458-2476) */
    const char *kind[5] = {"defaultsource", "deltasource", "closestqpsource", "csplinesource", "p0source"};
    snprintf(fname_interp, sizeof(fname_interp), "%s-receiver-%dx%d-p%d.dat", kind[src_impl_raw + 1], mx, my, p);
  }
  if (!ignore_rec && ninterp > 0 && !restart) {  /* its header (2478-2491) */
    fp = fopen(fname_interp, "w");
    if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname_interp); return 1; }
    fprintf(fp, "# SpecFECtx meta data\n");
    fprintf(fp, "#   mx %d : my %d : basis order %d\n", mx, my, p);
    fprintf(fp, "#   source implementation %d\n", src_impl_raw);
    fprintf(fp, "# Receiver meta data\n");
    fprintf(fp, "#   + receiver location: x,y %+1.8e %+1.8e\n", interp_xy[0], interp_xy[1]);
    fprintf(fp, "#   + records displ/velo at requested receiver location through interpolating the FE solution\n");
    fprintf(fp, "# Time series header\n");
    fprintf(fp, "#   time ux uy vx vy\n");
    fclose(fp);
  }
  if (!ignore_rec && nrec > 0 && !restart) {
    fp = fopen(fname, "w");
    if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname); return 1; }
    fprintf(fp, "# SpecFECtx meta data\n");
    fprintf(fp, "#   mx %d : my %d : basis order %d\n", mx, my, p);
    fprintf(fp, "# Receiver meta data\n");
    fprintf(fp, "#   + number receiver locations: %d\n", nrec);
    fprintf(fp, "#   + number receiver locations <local>: %d\n", nrec);
    fprintf(fp, "#   + takes displ/velo/accel from basis nearest to requested receiver location\n");
    for (r = 0; r < nrec; r++) {
      int n = su->rec_node[r];
      fprintf(fp, "#   + receiver location [%d]: x,y %+1.8e %+1.8e\n", r, rec_xy[2 * r], rec_xy[2 * r + 1]);
      fprintf(fp, "#   +   mapped to nearest node --> %+1.8e %+1.8e\n", su->xnode[n % su->nx_g], su->ynode[n / su->nx_g]);
    }
    fprintf(fp, "# Time series header <field>(<column index>)\n");
    fprintf(fp, "#   time(1)\n");
    for (r = 0; r < nrec; r++) {
      int off = 1 + r * 7;
      fprintf(fp, "#     ux(%d) uy(%d) vx(%d) vy(%d) ax(%d) ay(%d) curl(v) (%d)-> station [%d]\n", off + 1, off + 2, off + 3,
              off + 4, off + 5, off + 6, off + 7, r);
    }
    fclose(fp);
    fp = fopen(meta, "w");
    if (fp) {
      fprintf(fp, "# SpecFECtx parallel/MPI meta data\n");
      fprintf(fp, "#   mx %d : my %d : basis order %d\n", mx, my, p);
      fprintf(fp, "# Receiver meta data\n");
      fprintf(fp, "#   + number receiver locations: %d\n", nrec);
      for (r = 0; r < nrec; r++) fprintf(fp, "#   + receiver [%d]: mapped to MPI rank %d\n", r, 0);
      fclose(fp);
    }
  }

  /* the time loop (4722-4775) in device batches that end on the 100-step log lines */
  nsteps = su->nsteps;
  k = 0;
  if (restart) {  /* resume: step count, time and the device state of a checkpoint file */
    FILE *cf = fopen(restart, "rb");
    char magic[8];
    long bytes = 0;
    void *blob;
    if (!cf || fread(magic, 1, 8, cf) != 8 || memcmp(magic, "SE2RUN01", 8) || fread(&k, sizeof(long), 1, cf) != 1 ||
        fread(&time, sizeof(double), 1, cf) != 1 || fread(&bytes, sizeof(long), 1, cf) != 1 || bytes <= 0) {
      fprintf(stderr, "cannot read checkpoint %s\n", restart);
      return 1;
    }
    blob = malloc((size_t)bytes);
    if (fread(blob, 1, (size_t)bytes, cf) != (size_t)bytes) { fprintf(stderr, "truncated checkpoint %s\n", restart); return 1; }
    fclose(cf);
    CHECK(se2gpu_checkpoint_load(h, blob, bytes));
    free(blob);
  }
  {
    double *stf = (double*)malloc(sizeof(double) * (size_t)block * (nsrc > 0 ? nsrc : 1));
    double *times = (double*)malloc(sizeof(double) * (size_t)block);
    double *rows = (double*)malloc(sizeof(double) * (size_t)(block + 1) * 7 * (nrec_all > 0 ? nrec_all : 1));
    double *irows = (double*)malloc(sizeof(double) * (size_t)(block + 1) * 7 * (ninterp > 0 ? ninterp : 1));
    double nrm[6];
    double *fu = (double*)malloc(sizeof(double) * 2 * (size_t)su->nnodes);
    double *fv = (double*)malloc(sizeof(double) * 2 * (size_t)su->nnodes);
    const char *vnames[2] = {"disp", "velo"};
    const double *vvecs[2] = {fu, fv};
    if (!ignore_rec && ninterp > 0 && k == 0)   /* printed by RecordUV_interp's first call (2543) */
      printf("# receiver location: x,y %+1.8e %+1.8e -- interpolated coordinate --> %+1.8e %+1.8e\n", interp_xy[0],
             interp_xy[1], su->interp_xri[0], su->interp_xri[1]);
    for (; k < nsteps;) {
      long n = block - (k % block);
      long j;
      int nr = 0;
      if (n > of - (k % of)) n = of - (k % of);   /* end blocks on snapshot steps */
      if (ckpt_every > 0 && n > ckpt_every - (k % ckpt_every)) n = ckpt_every - (k % ckpt_every);
      if (k + n > nsteps) n = nsteps - k;
      if (se2_stf_block(su, &time, n, times, stf)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
      CHECK(se2gpu_advance(h, (int)n, stf));
      k += n;
      if (k % 100 == 0) {
        printf("[step %9ld] time = %1.4e : dt = %1.4e \n", k, time, su->dt);
        CHECK(se2gpu_norms(h, nrm));
        printf("  [displacement] max = %+1.4e : min = %+1.4e : l2 = %+1.4e \n", nrm[0], nrm[1], nrm[2]);
        printf("  [velocity]     max = %+1.4e : min = %+1.4e : l2 = %+1.4e \n", nrm[3], nrm[4], nrm[5]);
      }
      if (nrec_all > 0) CHECK(nr = se2gpu_traces(h, rows, block + 1));
      if (!ignore_rec && ninterp > 0) {  /* time ux uy vx vy (2571) */
        if (se2_interp_rows(su, nr, rows, irows)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
        fp = fopen(fname_interp, "a");
        if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname_interp); return 1; }
        for (j = 0; j < nr; j++)
          fprintf(fp, "%1.4e %+1.8e %+1.8e %+1.8e %+1.8e\n", times[j], irows[7 * j], irows[7 * j + 1], irows[7 * j + 2],
                  irows[7 * j + 3]);
        fclose(fp);
      }
      if (!ignore_rec && nrec > 0) {
        fp = fopen(fname, "a");
        if (!fp) { fprintf(stderr, "Failed to open file \"%s\"\n", fname); return 1; }
        for (j = 0; j < nr; j++) {
          fprintf(fp, "%1.4e", times[j]);
          for (r = 0; r < nrec; r++) {
            const double *o = &rows[(size_t)j * 7 * nrec_all + 7 * r];
            fprintf(fp, " %+1.8e %+1.8e %+1.8e %+1.8e %+1.8e %+1.8e", o[0], o[1], o[2], o[3], o[4], o[5]);
            fprintf(fp, " %+1.8e", o[6]);
          }
          fprintf(fp, "\n");
        }
        fclose(fp);
      }
      if (ckpt_every > 0 && k % ckpt_every == 0 && k < nsteps) {  /* checkpoint after the block's rows are out */
        long bytes = se2gpu_checkpoint_size(h);
        void *blob = malloc((size_t)bytes);
        char cname[64];
        FILE *cf;
        CHECK(se2gpu_checkpoint_save(h, blob, bytes));
        snprintf(cname, sizeof(cname), "checkpoint-%06ld.bin", k);
        cf = fopen(cname, "wb");
        if (!cf || fwrite("SE2RUN01", 1, 8, cf) != 8 || fwrite(&k, sizeof(long), 1, cf) != 1 ||
            fwrite(&time, sizeof(double), 1, cf) != 1 || fwrite(&bytes, sizeof(long), 1, cf) != 1 ||
            fwrite(blob, 1, (size_t)bytes, cf) != (size_t)bytes || fclose(cf) != 0) {
          fprintf(stderr, "cannot write %s\n", cname);
          return 1;
        }
        free(blob);
      }
      if (k % of == 0) {  /* se2wave.c:4764-4770 */
        snprintf(fname_vts, sizeof(fname_vts), "step-%.4ld.vts", k);
        CHECK(se2gpu_get_fields(h, fu, fv, NULL));
        if (se2_write_vts(su, fname_vts, 2, vnames, vvecs)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
      }
    }
    /* after the loop the reference prints k: the breaking step, or nt+1 when the loop ran out */
    printf("[step %9ld] time = %1.4e : dt = %1.4e \n", (time >= su->tmax) ? k : k + 1, time, su->dt);
    CHECK(se2gpu_norms(h, nrm));
    printf("  [displacement] max = %+1.4e : min = %+1.4e : l2 = %+1.4e \n", nrm[0], nrm[1], nrm[2]);
    printf("  [velocity]     max = %+1.4e : min = %+1.4e : l2 = %+1.4e \n", nrm[3], nrm[4], nrm[5]);
    /* last snapshot (se2wave.c:4785-4789), named with the same k */
    snprintf(fname_vts, sizeof(fname_vts), "step-%.4ld.vts", (time >= su->tmax) ? k : k + 1);
    CHECK(se2gpu_get_fields(h, fu, fv, NULL));
    if (se2_write_vts(su, fname_vts, 2, vnames, vvecs)) { fprintf(stderr, "%s\n", se2_host_last_error()); return 1; }
    free(stf); free(times); free(rows); free(irows); free(fu); free(fv);
  }
  se2gpu_destroy(h);
  se2_setup_destroy(su);
  free(rec_xy); free(cell);
  return 0;
}
