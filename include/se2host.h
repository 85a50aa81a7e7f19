/*
 * se2host.h -- FP64 host set-up for the GB300 SEM time loop (C-ABI).
 *
 * The host side of se2wave stays in C: everything here runs once per problem on
 * the CPU in double precision and produces the small tables and per-node arrays
 * that the device library (se2gpu.h) consumes.  Each function states the
 * reference routine of Nicolucas/se2dr_fork se2wave.c it replaces; values are
 * identical to the reference's bit for bit (same operation order, no fused
 * multiply-add).
 *
 * Error convention (mirrors PetscErrorCode): 0 = success, < 0 = error, message
 * available from se2_host_last_error() (thread-local).
 */
#ifndef SE2HOST_H
#define SE2HOST_H
#ifdef __cplusplus
extern "C" {
#endif

#define SE2_STF_RICKER   0   /* (t0, f0, amp)          se2wave.c:3500-3545 */
#define SE2_STF_GAUSSIAN 1   /* (t0, omega, amp)       se2wave.c:3548-3590 */
#define SE2_STF_YOFFE    2   /* (tau_S, tau_R, D_max)  se2wave.c:3592-3822 */

/* Problem specification: what se2wave_demo (se2wave.c:4541-4807) hard-codes or
   reads from -mx -my -bdegree -tmax -dt -nt. */
typedef struct se2_spec {
  int mx, my, p;                 /* -mx -my -bdegree */
  double scale[2], shift[2];     /* [0,1]^2 scaled then shifted (SpecFECtxScaleMeshCoords, 781-823) */
  const double *cell_vp, *cell_vs, *cell_rho; /* per cell, mx*my each, or NULL for the constants */
  double vp, vs, rho;            /* SpecFECtxSetConstantMaterialProperties_Velocity (1161-1175) */
  double cfl;                    /* factor on the CFL step; the demo uses 0.5 (4709) */
  double dt;                     /* > 0: -dt */
  double tmax;                   /* -tmax */
  int nt;                        /* >= 0: -nt, else (int)(tmax/dt)+4 (4714) */
  int nearest_internal_gll;      /* -use_nearest_internal_gll (3125) */
  int nsrc;
  const double *src_xy;          /* nsrc*2 */
  const double *src_m;           /* nsrc*4: [M00 M01 M10 M11] */
  const int *stf_type;           /* nsrc: SE2_STF_* */
  const double *stf_par;         /* nsrc*3 */
  int nrec;
  const double *rec_xy;          /* nrec*2 */
  /* perturb != 0 (and no cell arrays): SpecFECtxSetPerturbedMaterialProperties_Velocity
     (1177-1236): per cell, uniform in [vp - dvp, vp + dvp] etc. from PETSc's RAND48
     (drand48 seeded 1, 2, 3 for vp, vs, rho) */
  int perturb;
  double dvp, dvs, drho;
  /* source representation: < 0 SeismicSourceCreate's nearest GLL point (the demo's); 0 pointwise,
     2 cubic-spline kernel of radius sm_h (<= 0: the reference's default), 3 P0
     (ElastoDynamicsSetSourceImplementation / -source_impl, 2202-2266) */
  int src_impl;
  double sm_h;
  /* interpolating receivers (RecordUV_interp, se2wave.c:2445-2581): displacement, velocity
     and acceleration at the exact points, from the Lagrange interpolant of their element */
  int ninterp;
  const double *interp_xy;       /* ninterp*2 */
} se2_spec;

/* Everything the device needs, FP64, owned by the library. */
typedef struct se2_setup {
  int mx, my, p, n1, npe, nx_g, ny_g;
  long nnodes;
  double *xi;        /* n1 GLL nodes, ascending (CreateGLLCoordsWeights 103-209) */
  double *w1d;       /* n1 GLL weights in the reference's order */
  double *wq;        /* npe tensor weights w[i+j*n1] = w1d[i]*w1d[j] (861-865) */
  double *D;         /* n1*n1: D[q*n1+i] = dN_i/dxi at xi_q (TabulateBasisDerivatives1d_CLEGENDRE 387-523) */
  double *xnode;     /* nx_g node x-coordinates (the mesh is a tensor product, 739-823) */
  double *ynode;     /* ny_g node y-coordinates */
  double *J00, *J11; /* mx, my: half element widths 0.5*dx (1245-1251) */
  double *iJ00, *iJ11; /* 1.0/J00, 1.0/J11 (1270-1271) */
  double *lambda, *mu, *rho; /* mx*my cell data (29-33) */
  double *mass;      /* nnodes lumped mass, ascending-element sum (AssembleBilinearForm_Mass2d 1431-1498) */
  double gmin[2], gmax[2];   /* DMGetBoundingBox */
  double dt_cfl;     /* ElastoDynamicsComputeTimeStep_2d (2276-2349) */
  double dt, tmax;
  long nt;           /* step bound */
  long nsteps;       /* steps the loop of se2wave.c:4722-4775 takes (stops when time >= tmax) */
  int nsrc;
  int *src_elem, *src_gll;   /* owning element, closest interior GLL (2995-3243) */
  double *src_vals;  /* nsrc*2*npe element values [2*k+c] (SeismicSourceSetup_Moment_Pointwise 3367-3429) */
  int *stf_type;
  double *stf_par;
  int nrec;
  double *rec_xy;
  int *rec_node, *rec_elem, *rec_gll; /* nearest GLL node (RecordUVA_MultipleStations_NearestGLL_MPI 2700-2810) */
  /* source entries: nsrc entries (element + element values + STF), each belonging to one of the
     nsrc_phys sources of the spec (src_owner); one entry per source unless src_impl >= 0 */
  int nsrc_phys;
  int *src_owner;
  /* receiver list = the nrec_sta nearest-GLL stations of the spec, then, for each of the
     ninterp interpolating receivers, the (p+1)^2 nodes k of its element interp_elem[i]
     (entry nrec_sta + i*npe + k, gll index k); nrec = nrec_sta + ninterp*npe.
     interp_N[i*npe + k] = N_k at the receiver, interp_xri = the interpolated coordinate */
  int nrec_sta;
  int ninterp;
  double *interp_xy;
  int *interp_elem;
  double *interp_N, *interp_xri;
} se2_setup;

const char *se2_host_last_error(void);

/* Full set-up (replaces SpecFECtxCreateMesh + ScaleMeshCoords + material +
   AssembleBilinearForm_Mass2d + SeismicSourceCreate/Setup + receiver location +
   ElastoDynamicsComputeTimeStep_2d). */
int  se2_setup_create(const se2_spec *spec, se2_setup **out);
void se2_setup_destroy(se2_setup *s);

/* CreateGLLCoordsWeights (se2wave.c:103-209): xi ascending, w in the reference's order */
int se2_gll(int p, double *xi, double *w);
/* TabulateBasis1d_CLEGENDRE (253-385): N[k*(p+1)+i] = N_i(x_k) */
int se2_basis_1d(int p, int npoints, const double *x, double *N);
/* TabulateBasisDerivatives1d_CLEGENDRE (387-523): dN[k*(p+1)+i] = dN_i/dxi(x_k) */
int se2_basis_deriv_1d(int p, int npoints, const double *x, double *dN);

/* Interpolating receiver (RecordUV_interp, se2wave.c:2445-2581): the containing element
   ei = (int)((x - gmin.x)/dx), ej likewise with dx = (gmax - gmin)/mx (2494-2500), the
   reference coordinates xi = 2(x - x0)/dx - 1 (2518-2519) and the tensor weights
   N[i + j*(p+1)] = N_i(xi)*N_j(eta) of TabulateBasis1d_CLEGENDRE (2522-2531).  *eid =
   ei + ej*mx; xri = sum_k N_k * (node coordinates) (2535-2541), the coordinate the reference
   prints.  Points outside [gmin, gmax) are rejected (the reference does not check; at
   x = gmax its element index runs past the mesh). */
int se2_interp_receiver(const se2_setup *s, const double xy[2], int *eid, double *N, double xri[2]);
/* Values at the interpolating receivers from receiver rows of the device library
   (rows[j][7*nrec], the se2gpu_traces layout over the setup's receiver list):
   out[j][7*i + c] = sum_k N_k rows[j][7*(nrec_sta + i*npe + k) + c], k ascending as the
   reference sums (2561-2569); c = ux uy vx vy ax ay curl(v).  The element's interpolant is
   in Q_p, as is its curl, so the curl of the interpolant at the point is exact too. */
int se2_interp_rows(const se2_setup *s, long nrows, const double *rows, double *out);

/* Source-time function values (SeismicSTFEvaluate 3458-3466 with the Ricker,
   Gaussian and Yoffe evaluators).  For steps k = 1..n after time `*time`, the
   time is advanced as time = time + dt (se2wave.c:4724) and times[k-1] and
   stf[(k-1)*nsrc + s] are written; *time is left at the last step's time. */
int se2_stf_block(const se2_setup *s, double *time, long n, double *times, double *stf);
/* one STF at one time */
int se2_stf_eval(int type, const double par[3], double time, double *value);

/* Seeded Gaussian random field on the mx*my cell grid (row-major, x fastest):
   mean*(1 + rel_std*z), z ~ N(0,1) white noise (splitmix64 + Box-Muller)
   smoothed by a separable Gaussian of std corr_cells (periodic), renormalised
   to unit variance and clipped to +-3. */
int se2_gaussian_random_field(int mx, int my, double mean, double rel_std, double corr_cells,
                              unsigned long long seed, double *out);

/* Seeded shot draws (splitmix64 stream per (seed, index)).  Kinds:
   SE2_SHOT_ENSEMBLE  mx, my ~ U{32..512}, p in {3,4,6}, 32 receivers, 5000 steps,
                      source anywhere in the central 80 %;
   SE2_SHOT_TRAINING  128 x 128, p = 4, 16 surface receivers, 4096 steps, source in the lower half;
   SE2_SHOT_OOD       as TRAINING with Vp up to 7500 m/s and two inclusions.
   Elements are 31.25 m squares, the domain is [0, Lx] x [0, Ly].  Materials: two
   layers split at interface_y plus elliptical inclusions, each rock with
   Vp ~ U[3000, 6000] (7500 OOD), Vp/Vs ~ U[1.6, 1.9], rho ~ U[2000, 3000];
   moment tensor entries Mxx, Mxy = Myx, Myy ~ N(0, 1e15); Ricker f0 ~ U[5, 20] Hz,
   t0 = 1.5 / f0. */
enum { SE2_SHOT_ENSEMBLE = 0, SE2_SHOT_TRAINING = 1, SE2_SHOT_OOD = 2 };
typedef struct se2_shot_draw {
  int mx, my, p, nrec;
  long nsteps;
  double h, Lx, Ly;
  double interface_y;
  double lower[3], upper[3];    /* (vp, vs, rho) below / above the interface */
  int ninc;
  double inc[2][8];             /* centre x, y, semi-axes a, b, rotation, vp, vs, rho */
  double src_xy[2];
  double moment[4];             /* Mxx, Mxy, Myx, Myy */
  double f0, t0;
} se2_shot_draw;
int se2_shot_draw_params(unsigned long long seed, long index, int kind, se2_shot_draw *out);
/* the drawn materials on the mx*my cell grid (row-major, x fastest), at cell centres */
int se2_shot_materials(const se2_shot_draw *d, double *vp, double *vs, double *rho);

/* Snapshot of nodal fields (the VecView to a PetscViewerVTK of se2wave.c:4606-4610,
   4764-4770, 4785-4789): a VTK XML StructuredGrid file over the GLL nodes
   (points x, y, 0), one Float64 scalar array per component named <name>_x and
   <name>_y (the Vec names and DMDA field names of the reference), raw appended
   data with UInt64 size headers.  vecs[v] are interleaved [node][component]. */
int se2_write_vts(const se2_setup *s, const char *path, int nvec, const char *const *names, const double *const *vecs);

/* Assembled source vector g (2*nnodes, interleaved) of one moment source M = [M00 M01 M10 M11]
   at xy, in one of the reference's alternative representations (ElastoDynamicsSourceSetup,
   2232-2266): 0 pointwise at the exact reference coordinates (1716-1923), 2 cubic-spline
   smoothed Dirac with radius kernel_h (<= 0: the reference's default; -sm_h, 1925-2057),
   3 P0 cell average (2059-2200). */
int se2_source_vector(const se2_setup *s, int impl, double kernel_h, const double xy[2], const double M[4], double *g);

#ifdef __cplusplus
}
#endif
#endif
