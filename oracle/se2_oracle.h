/*
 * se2_oracle: CPU restatement of se2wave's explicit SEM time loop
 * (Nicolucas/se2dr_fork, se2wave.c).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity reference for the GPU library and
 * the timed CPU baseline; the product never links or calls it.  It follows the
 * reference operation for operation (dense O(npe^2) element loop, per-element
 * derivative re-tabulation, ascending-element scatter-add, PETSc Vec semantics)
 * so its results match the reference compiled in place (oracle/_ref) bit for bit
 * and its speed stands for the reference's.
 */
#ifndef SE2_ORACLE_H
#define SE2_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int mx, my, p;                 /* elements in x, y; polynomial degree (-bdegree) */
  double scale[2], shift[2];     /* [0,1]^2 mesh scaled then shifted (se2wave.c:781-823) */
  const double *cell_vp, *cell_vs, *cell_rho; /* per cell (ne each) or NULL for constants */
  double vp, vs, rho;
  double cfl;                    /* factor on the CFL step (the demo uses 0.5, se2wave.c:4709) */
  double dt;                     /* > 0: -dt override */
  double tmax;                   /* -tmax */
  int nt;                        /* >= 0: -nt override, else (int)(tmax/dt)+4 */
  int nearest_internal_gll;      /* -use_nearest_internal_gll (default 1) */
  int nsrc;
  const double *src_xy;          /* nsrc*2 */
  const double *src_m;           /* nsrc*4 moment tensor [M00 M01 M10 M11] */
  const int *stf_type;           /* 0 Ricker(t0,f0,amp) 1 Gaussian(t0,omega,amp) 2 Yoffe(tau_S,tau_R,D_max) */
  const double *stf_par;         /* nsrc*3 */
  int nrec;
  const double *rec_xy;          /* nrec*2 */
  int perturb;                   /* SpecFECtxSetPerturbedMaterialProperties_Velocity (1177-1236) */
  double dvp, dvs, drho;
} se2o_spec;

typedef struct se2o_ctx se2o_ctx;

/* setup (mesh, basis, materials, mass, sources, receivers, dt); 0 on success */
int  se2o_create(const se2o_spec *sp, se2o_ctx **ctx);
void se2o_destroy(se2o_ctx *ctx);
const char *se2o_last_error(void);

/* ints[0..5] = nx_g, ny_g, npe_1d, nsteps planned, nrec, nsrc; dbls[0..2] = dt, dt_cfl, tmax */
int se2o_info(const se2o_ctx *ctx, int *ints, double *dbls);

/* setup arrays: "xi","w1d","w","D","dN_dxi","dN_deta","coords","mass","cell_lmr",
   "src_values","src_index"(as doubles),"rec_index"(nid,eid,gll as doubles) */
int se2o_get(const se2o_ctx *ctx, const char *name, double *out, long n);

/* advance up to nsteps (stops early when time >= tmax, like se2wave.c:4772);
   traces (may be NULL): per step [time, (ux uy vx vy ax ay curl) * nrec];
   norms (may be NULL): per step k%100==0: [k, umax umin ul2 vmax vmin vl2];
   returns the number of steps taken, < 0 on error */
long se2o_run(se2o_ctx *ctx, long nsteps, double *traces, double *norms, long max_norm_rows);

/* state access (2*nodes doubles each, interleaved [node][comp]) */
int se2o_get_state(const se2o_ctx *ctx, double *u, double *v, double *a);
int se2o_set_state(se2o_ctx *ctx, const double *u, const double *v, const double *a, double time);

/* F = AssembleLinearForm_ElastoDynamics2d(u) (se2wave.c:1285-1429) */
int se2o_force(se2o_ctx *ctx, const double *u, double *F);

/* source-time function values on a time grid t0 + k*dt accumulated as time = time + dt */
int se2o_stf(int type, const double par[3], double t0, double dt, long n, double *out);

/* CPU baseline: nthreads independent solves of the same spec, nsteps each after
   warmup steps; returns wall seconds of the timed steps (max over threads) */
double se2o_bench(const se2o_spec *sp, int nthreads, long warmup, long nsteps, int record);

#ifdef __cplusplus
}
#endif
#endif
