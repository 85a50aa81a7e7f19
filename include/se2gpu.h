/*
 * se2gpu.h -- C-ABI of the GB300 (sm_103a) SEM time-loop library, libse2gpu.so.
 *
 * Drop-in boundary for the hot path of Nicolucas/se2dr_fork se2wave.c.  The
 * reference has no plugin or FFI layer: its boundary is the C function
 *   PetscErrorCode AssembleLinearForm_ElastoDynamics2d(SpecFECtx c, Vec u, Vec F)   (se2wave.c:1285)
 * plus the Vec operations of the time loop (se2wave.c:4722-4775) that surround
 * it.  This header replaces them:
 *
 *   se2gpu_assemble_linear_form   <- AssembleLinearForm_ElastoDynamics2d           (se2wave.c:1285-1429)
 *   se2gpu_advance                <- one pass of the loop body per step:
 *                                    VecAXPY x3 (4726-4730), SeismicSourceEvaluate (4733, 3470-3497),
 *                                    AssembleLinearForm_ElastoDynamics2d (4736), VecAXPY(f,1,g) (4739),
 *                                    VecPointwiseDivide (4742), VecAXPY (4745), and the per-step
 *                                    receiver sampling of RecordUVA_MultipleStations_NearestGLL_MPI
 *                                    (2886-2981)
 *   se2gpu_norms                  <- VecNorm/VecMin/VecMax of u and v (4747-4755)
 *   se2gpu_set_fields/get_fields  <- the u, v, a Vecs (DMCreateGlobalVector, 4594-4596)
 *
 * Conventions (mirroring PetscErrorCode): every call returns 0 on success and a
 * negative code on error; se2gpu_last_error() returns the handle's message.  No
 * exception crosses the ABI.  The library owns all device memory; the caller
 * owns host arrays.  One host thread per handle.  Vectors are interleaved
 * [node][component] with node = i + j*(p*mx+1), exactly the reference's Vec
 * layout, so fields move between the two unchanged.
 */
#ifndef SE2GPU_H
#define SE2GPU_H
#ifdef __cplusplus
extern "C" {
#endif

/* precision modes */
#define SE2GPU_FP64        64  /* FP64, reference operation order, no fused multiply-add: bit-identical to the CPU reference */
#define SE2GPU_FP32_KAHAN  33  /* FP32 arithmetic, Kahan-compensated u and v updates */
#define SE2GPU_FP32        32  /* FP32 arithmetic, plain updates */
#define SE2GPU_FP32_DF     34  /* two-float arithmetic: every value of a step (displacement differences, gradients,
                                  stresses, forces, 1/M, the updates) carried as an unevaluated sum of two
                                  floats, about 48 significant bits, on the FP32 pipe; state stored as in
                                  SE2GPU_FP32_KAHAN, whose accelerations and curl(v) traces carry the FP32
                                  force evaluation's rounding (1e-4 to 1e-3 relative L2 of FP64) */

/* error codes */
#define SE2GPU_OK            0
#define SE2GPU_ERR_ARG      -1  /* invalid argument */
#define SE2GPU_ERR_CUDA     -2  /* CUDA runtime error */
#define SE2GPU_ERR_NOMEM    -3  /* device allocation failed */
#define SE2GPU_ERR_STATE    -4  /* call not valid in the handle's state */
#define SE2GPU_ERR_NUMERIC  -5  /* non-finite value detected */

/* The discrete problem, produced by the FP64 host set-up (se2host.h).  All
   pointers are host memory, read during se2gpu_create only. */
typedef struct se2gpu_problem {
  int mx, my, p;             /* elements in x and y, polynomial degree 1..8 */
  double dt;                 /* time step */
  const double *D;           /* (p+1)^2: D[q*(p+1)+i] = dN_i/dxi at GLL point q */
  const double *wq;          /* (p+1)^2: tensor GLL weights w[i+j*(p+1)] */
  const double *w1d;         /* p+1: 1-D GLL weights (wq[i+j*(p+1)] = w1d[i]*w1d[j]) */
  const double *J00, *J11;   /* mx, my: element half-widths */
  const double *iJ00, *iJ11; /* mx, my: their reciprocals */
  const double *lambda, *mu; /* mx*my cell Lame parameters */
  const double *mass;        /* (p*mx+1)*(p*my+1) lumped mass per node */
  int nsrc;
  const int *src_elem;       /* nsrc owning elements */
  const double *src_vals;    /* nsrc*2*(p+1)^2 element values, [2*k + component] */
  int nrec;
  const int *rec_node;       /* nrec nearest GLL node */
  const int *rec_elem;       /* nrec owning element */
  const int *rec_gll;        /* nrec element-local GLL index of that node */
} se2gpu_problem;

typedef struct se2gpu_solver se2gpu_solver;

/* Allocate and upload a problem.  trace_capacity = receiver rows buffered on
   the device between se2gpu_traces calls.  The fields start at zero. */
int  se2gpu_create(const se2gpu_problem *prob, int precision, int trace_capacity, se2gpu_solver **out);
void se2gpu_destroy(se2gpu_solver *h);
const char *se2gpu_last_error(const se2gpu_solver *h);
/* message of the last se2gpu_create failure in this thread (no handle exists then) */
const char *se2gpu_create_error(void);

/* Launch on this CUDA stream (a cudaStream_t; NULL = the handle's own stream). */
int se2gpu_set_stream(se2gpu_solver *h, void *stream);
int se2gpu_synchronize(se2gpu_solver *h);

/* Self-test of failure detection (no counterpart in the reference).  Every wait of
   the FP32 step kernels on their tile copies is bounded: on expiry the kernel raises
   the handle's error flag and returns, and the next call that checks the flag
   fails with SE2GPU_ERR_CUDA.  This call runs that same bounded wait, with a limit
   of 256 polls, on an mbarrier that nothing arrives at, on the handle's stream.  It
   returns what se2gpu_synchronize would then return: SE2GPU_ERR_CUDA with the
   bounded-wait message, or 0 if the flag was not raised.  *seconds (if not NULL)
   receives the wait's duration on the device clock.  The flag stays raised, as
   after a real expiry: destroy the handle afterwards.  No copy is in flight and
   nothing faults, so the CUDA context and other handles stay usable. */
int se2gpu_selftest_wait_expiry(se2gpu_solver *h, double *seconds);

/* Fields as FP64 host arrays of 2*nnodes (any may be NULL). */
int se2gpu_set_fields(se2gpu_solver *h, const double *u, const double *v, const double *a);
int se2gpu_get_fields(se2gpu_solver *h, double *u, double *v, double *a);

/* Advance nsteps steps.  stf[k*nsrc + s] is source s's source-time function at
   the time of step k (the host evaluates the STF objects, as the reference does
   per step).  One receiver row per step is buffered on the device; the call
   fails with SE2GPU_ERR_STATE when the trace buffer would overflow. */
int se2gpu_advance(se2gpu_solver *h, int nsteps, const double *stf);

/* Copy up to max_rows buffered receiver rows (oldest first) into out[row][7*nrec]
   = (ux uy vx vy ax ay curl(v)) per receiver, FP64, and empty the buffer.
   Returns the number of rows copied (>= 0) or an error code. */
int se2gpu_traces(se2gpu_solver *h, double *out, int max_rows);

/* out[6] = max, min, l2 of u then of v (VecMax/VecMin/VecNorm NORM_2). */
int se2gpu_norms(se2gpu_solver *h, double out[6]);

/* F = AssembleLinearForm_ElastoDynamics2d(u): internal force of the
   displacement u (2*nnodes FP64 host arrays).  Does not touch the fields. */
int se2gpu_assemble_linear_form(se2gpu_solver *h, const double *u, double *F);

/* Same on device arrays of the handle's precision (double or float, 2*nnodes),
   launched on the handle's stream, no synchronisation. */
int se2gpu_assemble_linear_form_device(se2gpu_solver *h, const void *u_dev, void *F_dev);

/* Introspection: ints[0..8] = nx_g, ny_g, p, precision, nsrc, nrec, kernel
   launches so far, buffered trace rows, device row pitch (nodes). */
int se2gpu_info(const se2gpu_solver *h, long *ints);

/* Device pointers of the current state.  FP64: u, v, a in the reference's
   packed layout.  FP32 modes hold the leapfrog state in rows of `pitch` nodes
   (float2 per node): u = displacement of the next step, v = half-step velocity
   (v_k + dt/2 a_k), a = acceleration of the last step. */
int se2gpu_device_fields(const se2gpu_solver *h, void **u, void **v, void **a);

/* Tile configurations of the step kernel (elements per tile edge, threads per
   CTA) available for the handle's degree and precision, for the autotuner;
   returns how many exist.  se2gpu_set_tile_config selects one; se2gpu_tile_config
   returns the selected one (a new handle starts with the configuration measured
   fastest for its degree on GB300 in the plain and Kahan modes, 0 in the two-float
   and FP64 modes). */
int se2gpu_tile_configs(const se2gpu_solver *h, int *edge, int *threads, int max_configs);
int se2gpu_set_tile_config(se2gpu_solver *h, int config);
int se2gpu_tile_config(const se2gpu_solver *h);
/* One configuration in full (no counterpart in the reference): info = {elements per
   tile edge, threads per CTA, owned-box buffers (2: the next tile's w arrives a tile
   ahead; 1: during the tile's element phases; 0: FP64), resident CTAs per SM on the
   current device (0: FP64)}.  Two configurations may share edge and threads. */
int se2gpu_tile_config_info(const se2gpu_solver *h, int config, int info[4]);

/* ---- Checkpoint / resume (no counterpart in the reference, which restarts from
   t = 0).  The checkpoint holds the handle's whole evolving state: the fields
   in the handle's precision (FP32 modes: leapfrog state with its Kahan terms),
   the acceleration of the last step, and the pending receiver row, so a run
   resumed from it is bit-identical to the uninterrupted run.  Buffered trace
   rows are not part of it: fetch them with se2gpu_traces first (saving with
   rows buffered fails with SE2GPU_ERR_STATE).  Load into a handle created
   from the same problem and precision (checked against the header). */
long se2gpu_checkpoint_size(const se2gpu_solver *h);
int  se2gpu_checkpoint_save(se2gpu_solver *h, void *buf, long bytes);
int  se2gpu_checkpoint_load(se2gpu_solver *h, const void *buf, long bytes);

/* ---- Batched ensemble.  No counterpart in the reference, which runs one shot
   per process (se2wave.c main): many independent problems ("shots") of any
   mesh size and degree advanced in lock-step on one GPU, FP32 precisions only.
   Each step is one persistent launch per degree present, over a flattened
   (shot, tile) work list; each block of `block` steps is captured once as a
   CUDA graph and replayed.  Every shot advances exactly as an se2gpu_solver of
   the same problem and precision would (bit-identical fields and traces). */
typedef struct se2gpu_ensemble se2gpu_ensemble;

int  se2gpu_ensemble_create(const se2gpu_problem *shots, int nshots, int precision, int block, se2gpu_ensemble **out);
void se2gpu_ensemble_destroy(se2gpu_ensemble *e);
/* message of the handle's last failure; with NULL, of the last create failure in this thread */
const char *se2gpu_ensemble_last_error(const se2gpu_ensemble *e);
int se2gpu_ensemble_set_stream(se2gpu_ensemble *e, void *stream);
/* graphs on (default) or plain launches */
int se2gpu_ensemble_set_graphs(se2gpu_ensemble *e, int enable);
/* tile configuration (se2gpu_tile_configs numbering) of all shots of degree p;
   se2gpu_ensemble_tile_config returns the current one */
int se2gpu_ensemble_set_tile_config(se2gpu_ensemble *e, int p, int config);
int se2gpu_ensemble_tile_config(const se2gpu_ensemble *e, int p);

/* Advance every shot nsteps steps.  Shot-major layouts, shot s's block at the
   prefix sum of the earlier shots' counts:
     stf    [shot][nsteps][nsrc_s]        source-time function values per step
     traces [shot][nsteps][nrec_s][7]     receiver rows (ux uy vx vy ax ay curl(v)), FP64;
                                          NULL = do not return them
   Returns when the traces are in `traces`. */
int se2gpu_ensemble_advance(se2gpu_ensemble *e, int nsteps, const double *stf, double *traces);
/* Enqueue nsteps steps with the STF values already staged on the device and
   without returning receiver rows; no synchronisation (device-resident timing). */
int se2gpu_ensemble_enqueue(se2gpu_ensemble *e, int nsteps);
int se2gpu_ensemble_synchronize(se2gpu_ensemble *e);

/* One shot's fields as FP64 host arrays of 2*nnodes (as se2gpu_get/set_fields). */
int se2gpu_ensemble_get_fields(se2gpu_ensemble *e, int shot, double *u, double *v, double *a);
int se2gpu_ensemble_set_fields(se2gpu_ensemble *e, int shot, const double *u, const double *v, const double *a);

/* ints[0..8] = shots, degree groups, block, kernel launches so far, graph
   replays, total nodes, total sources, total receivers, (shot, tile) items. */
int se2gpu_ensemble_info(const se2gpu_ensemble *e, long *ints);

/* ---- Norms without device allocation.  No counterpart in the reference (its
   VecMax/VecMin/VecNorm log lines come from PETSc on host vectors).
   out[6] = max, min, l2 of u then of v (as se2gpu_norms) for n FP64 values of
   caller-owned device vectors u_dev, v_dev, computed on `stream` (a
   cudaStream_t; NULL = the legacy default stream); returns after the result is
   in `out`.  Allocates nothing: the per-block partials use a fixed static device
   array of SE2GPU_NOALLOC_MAX_BLOCKS x 6 doubles (192 KiB), so n may not exceed
   SE2GPU_NOALLOC_MAX_VALUES (larger n is rejected with SE2GPU_ERR_ARG).  The
   first call on each device looks up that array's address and should come
   before any stream capture; the address is kept until the process exits, so
   the device must not be reset (cudaDeviceReset) while the library is loaded.
   Calls that overlap in time share the array and race.  A NaN or Inf in u or v
   makes an l2 norm non-finite and fails the call with SE2GPU_ERR_NUMERIC, as
   se2gpu_norms does.  On failure se2gpu_last_error(NULL) gives the message. */
#define SE2GPU_NOALLOC_CHUNK 65536L
#define SE2GPU_NOALLOC_MAX_BLOCKS 4096
#define SE2GPU_NOALLOC_MAX_VALUES (SE2GPU_NOALLOC_CHUNK * SE2GPU_NOALLOC_MAX_BLOCKS)
int se2gpu_norms_device_noalloc(const double *u_dev, const double *v_dev, long n, void *stream, double out[6]);

/* ---- Arithmetic-pipe peak of the current device (no counterpart in the reference): the
   roofline denominator of the kernels that HBM does not bound.  Measured with CUDA events
   on independent dependency chains (4 CTAs of 256 threads per SM).  kind 0: FP64
   separately rounded multiply + add (the operations of the FP64 step kernel, which
   follows the reference's operation order and fuses nothing); 1: FP64 fused
   multiply-add; 2: FP32 separately rounded multiply + add; 3: FP32 fused multiply-add.
   *ops_per_second counts arithmetic operations (a fused multiply-add counts two). */
int se2gpu_pipe_peak(int kind, double *ops_per_second);

#ifdef __cplusplus
}
#endif
#endif
