/*
 * se2_oracle.c -- CPU restatement of se2wave.c (Nicolucas/se2dr_fork).
 *
 * TEST INFRASTRUCTURE ONLY (the parity reference of the tests and the timed CPU
 * baseline).  Every function cites the reference lines it restates.  Floating-point expressions
 * keep the reference's association and operand order; the file is compiled with
 * -ffp-contract=off so no multiply-add is fused.  PETSc semantics on one rank:
 * VecAXPY y = y + a*x (returns early for a == 0), VecPointwiseDivide w = x/y,
 * VecSetValues ADD x[i] += y, DMGlobalToLocal / DMLocalToGlobal ADD = copy / add,
 * PCLU = partial-pivot LU in reference-LAPACK order (dgetf2 + dgetrs).
 */
#include "se2_oracle.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <pthread.h>
#include <time.h>

#define O_PI 3.14159265358979323846264338327950288419716939937510582

static __thread char errbuf[512];
const char *se2o_last_error(void) { return errbuf; }
#define FAIL(...) do { snprintf(errbuf, sizeof(errbuf), __VA_ARGS__); return -1; } while (0)

struct se2o_ctx {
  int mx, my, p, n1, npe, ne, nx_g, ny_g, nnodes, ndof;
  double *xi, *w1d, *w;           /* GLL nodes (ascending), weights (reference order), tensor weights */
  double *dN_dxi, *dN_deta;       /* [npe][npe] reference tensor-product tables */
  double *dN_dx, *dN_dy;          /* [npe][npe] per-element scratch (se2wave.c:1254-1279) */
  int *element;                   /* [ne][npe] */
  double *coords;                 /* [nnodes][2] */
  double *lam, *mu, *rho;         /* [ne] */
  double *u, *v, *a, *f, *g, *Md; /* global vectors [ndof] */
  double *ul, *fl, *lu, *lv, *la; /* local work vectors (one rank: same layout) */
  double elcoords[2 * 81], ux[81], uy[81], fe[2 * 81];
  int eldofs[2 * 81];
  /* sources */
  int nsrc;
  int *src_elem, *src_gll;
  double *src_vals;               /* [nsrc][2npe] */
  int *src_dofs;                  /* [nsrc][2npe] */
  int *stf_type;
  double *stf_par;
  /* receivers */
  int nrec;
  double *rec_xy;
  int *rec_nid, *rec_eid, *rec_gll;
  /* time */
  double dt, dt_cfl, tmax, time;
  long nt, k;
};

/* ------------------------------------------------------------------ */
/* CreateGLLCoordsWeights, se2wave.c:103-209                           */
/* xi returned ascending (flipped, 185-191); w keeps the Newton order  */
/* ------------------------------------------------------------------ */
static int gll(int N, double *xi_out, double *w_out)
{
  int N1 = N + 1, i, k;
  double *xold = (double*)malloc(sizeof(double) * N1);
  double *x = (double*)malloc(sizeof(double) * N1);
  double *P = (double*)calloc((size_t)(N1 * N1), sizeof(double));
  double eps, res;
  for (i = 0; i < N1; i++) x[i] = cos(O_PI * i / (double)N);
  for (i = 0; i < N1; i++) xold[i] = 2.0;
  res = 1.0;
  eps = 1.0e-12;
  while (res > eps) {
    for (i = 0; i < N1; i++) xold[i] = x[i];
    for (i = 0; i < N1; i++) { P[i + 0 * N1] = 1.0; P[i + 1 * N1] = x[i]; }
    for (i = 0; i < N1; i++) {
      for (k = 1; k < N; k++) {
        P[i + (k + 1) * N1] = ((2.0 * (k + 1) - 1.0) * x[i] * P[i + k * N1] - (k + 1.0 - 1.0) * P[i + (k - 1) * N1]) / (double)(k + 1.0);
      }
    }
    for (i = 0; i < N1; i++) {
      x[i] = xold[i] - (x[i] * P[i + (N1 - 1) * N1] - P[i + (N - 1) * N1]) / (N1 * P[i + (N1 - 1) * N1]);
    }
    res = 0.0;
    for (i = 0; i < N1; i++) res += (x[i] - xold[i]) * (x[i] - xold[i]);
    res = sqrt(res);
  }
  for (i = 0; i < N1; i++) {
    double pp = P[i + (N1 - 1) * N1];
    if (w_out) w_out[i] = 2.0 / (N * N1 * pp * pp);
  }
  for (i = 0; i < N1 / 2; i++) { double t = x[i]; x[i] = x[N1 - 1 - i]; x[N1 - 1 - i] = t; }
  if (xi_out) memcpy(xi_out, x, sizeof(double) * N1);
  free(xold); free(x); free(P);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Vandermonde coefficients: PCLU on MatSeqDense (se2wave.c:278-334)   */
/* reference-LAPACK dgetf2/dgetrs operation order                      */
/* ------------------------------------------------------------------ */
static int vandermonde_coeffs(int order, double *coeff /* [n][n]: coeff[k*n+i] */)
{
  int n = order + 1, i, j, k, jp;
  double *xl = (double*)malloc(sizeof(double) * n);
  double *A = (double*)malloc(sizeof(double) * n * n); /* column major */
  int *piv = (int*)malloc(sizeof(int) * n);
  double *b = (double*)malloc(sizeof(double) * n);
  gll(order, xl, NULL);
  for (k = 0; k < n; k++) for (i = 0; i < n; i++) A[k + i * n] = pow(xl[k], (double)i);
  for (j = 0; j < n; j++) {
    double amax = -1.0;
    jp = j;
    for (i = j; i < n; i++) if (fabs(A[i + j * n]) > amax) { amax = fabs(A[i + j * n]); jp = i; }
    piv[j] = jp;
    if (A[jp + j * n] == 0.0) { free(xl); free(A); free(piv); free(b); FAIL("singular Vandermonde matrix"); }
    if (jp != j) for (k = 0; k < n; k++) { double t = A[j + k * n]; A[j + k * n] = A[jp + k * n]; A[jp + k * n] = t; }
    if (fabs(A[j + j * n]) >= DBL_MIN) { double r = 1.0 / A[j + j * n]; for (i = j + 1; i < n; i++) A[i + j * n] *= r; }
    else for (i = j + 1; i < n; i++) A[i + j * n] = A[i + j * n] / A[j + j * n];
    for (k = j + 1; k < n; k++) {
      double t = -A[j + k * n];
      for (i = j + 1; i < n; i++) A[i + k * n] = A[i + k * n] + A[i + j * n] * t;
    }
  }
  for (k = 0; k < n; k++) {
    int c;
    for (i = 0; i < n; i++) b[i] = (i == k) ? 1.0 : 0.0;
    for (i = 0; i < n; i++) if (piv[i] != i) { double t = b[i]; b[i] = b[piv[i]]; b[piv[i]] = t; }
    for (c = 0; c < n; c++) if (b[c] != 0.0) for (i = c + 1; i < n; i++) b[i] = b[i] - b[c] * A[i + c * n];
    for (c = n - 1; c >= 0; c--) {
      if (b[c] != 0.0) {
        b[c] = b[c] / A[c + c * n];
        for (i = 0; i < c; i++) b[i] = b[i] - b[c] * A[i + c * n];
      }
    }
    for (i = 0; i < n; i++) coeff[k * n + i] = b[i];
  }
  free(xl); free(A); free(piv); free(b);
  return 0;
}

/* TabulateBasis1d_CLEGENDRE (se2wave.c:253-385), out[p*n+i] = N_i(xi_p) */
static int basis1d(int npoints, const double *xi, int order, double *out)
{
  int n = order + 1, p, i, j;
  double *coeff = (double*)malloc(sizeof(double) * n * n), *mono = (double*)malloc(sizeof(double) * n);
  if (vandermonde_coeffs(order, coeff)) { free(coeff); free(mono); return -1; }
  for (p = 0; p < npoints; p++) {
    for (i = 0; i < n; i++) mono[i] = pow((double)xi[p], (double)i);
    for (i = 0; i < n; i++) {
      double s = 0.0;
      for (j = 0; j < n; j++) s += coeff[i * n + j] * mono[j];
      if (fabs(s) < 1.0e-12) s = 0.0;
      out[p * n + i] = s;
    }
  }
  free(coeff); free(mono);
  return 0;
}

/* TabulateBasisDerivatives1d_CLEGENDRE (se2wave.c:387-523), out[p*n+i] = dN_i/dxi(xi_p) */
static int dbasis1d(int npoints, const double *xi, int order, double *out)
{
  int n = order + 1, p, i, j;
  double *coeff = (double*)malloc(sizeof(double) * n * n), *mono = (double*)malloc(sizeof(double) * n);
  if (vandermonde_coeffs(order, coeff)) { free(coeff); free(mono); return -1; }
  for (p = 0; p < npoints; p++) {
    for (i = 0; i < n; i++) mono[i] = (i == 0) ? 0.0 : ((double)i) * pow((double)xi[p], (double)(i - 1));
    for (i = 0; i < n; i++) {
      double s = 0.0;
      for (j = 0; j < n; j++) s += coeff[i * n + j] * mono[j];
      if (fabs(s) < 1.0e-12) s = 0.0;
      out[p * n + i] = s;
    }
  }
  free(coeff); free(mono);
  return 0;
}

/* ------------------------------------------------------------------ */
/* geometry, se2wave.c:1238-1279                                       */
/* ------------------------------------------------------------------ */
static void el_geometry(int npe, const double *elc, int n1, double *detJ)
{
  double dx = elc[2 * (n1 - 1) + 0] - elc[2 * 0 + 0];
  double dy = elc[2 * (npe - 1) + 1] - elc[2 * 0 + 1];
  double J00 = 0.5 * dx, J11 = 0.5 * dy;
  *detJ = J00 * J11;
}

static void el_derivatives(int nqp, int npe, const double *elc, int n1, const double *dN_dxi, const double *dN_deta,
                           double *dN_dx, double *dN_dy)
{
  int k, q;
  double dx = elc[2 * (n1 - 1) + 0] - elc[2 * 0 + 0];
  double dy = elc[2 * (npe - 1) + 1] - elc[2 * 0 + 1];
  double J00 = 0.5 * dx, J11 = 0.5 * dy, iJ00, iJ11;
  for (q = 0; q < nqp; q++) {
    iJ00 = 1.0 / J00;
    iJ11 = 1.0 / J11;
    for (k = 0; k < npe; k++) {
      dN_dx[q * npe + k] = iJ00 * dN_dxi[q * npe + k];
      dN_dy[q * npe + k] = iJ11 * dN_deta[q * npe + k];
    }
  }
}

static void bounding_box(const se2o_ctx *c, double gmin[2], double gmax[2])
{
  int i, j;
  gmin[0] = gmin[1] = DBL_MAX;
  gmax[0] = gmax[1] = -DBL_MAX;
  for (i = 0; i < c->nnodes; i++) {
    for (j = 0; j < 2; j++) {
      double x = c->coords[2 * i + j];
      gmin[j] = (gmin[j] < x) ? gmin[j] : x;
      gmax[j] = (gmax[j] < x) ? x : gmax[j];
    }
  }
}

/* ------------------------------------------------------------------ */
/* STFs, se2wave.c:3500-3822                                           */
/* ------------------------------------------------------------------ */
static int yoffe_C1(const double *y, double time, double *C1)
{
  double t1, t2, t3, t4, t5, tau_R2, tau_R = y[1];
  tau_R2 = tau_R * tau_R;
  t1 = 0.5 * time + 0.25 * tau_R;
  t2 = time * (tau_R - time);
  t3 = (time - tau_R) * tau_R;
  t4 = time / tau_R;
  if (fabs(time) < 0.0) t5 = 1.0e12; else t5 = (tau_R - time) / time;
  if (t2 < 0.0 || t4 < 0.0 || t5 < 0.0) FAIL("reg_yoffe_compute_C1: negative argument");
  *C1 = t1 * sqrt(t2) + t3 * asin(sqrt(t4)) - 0.75 * tau_R2 * atan(sqrt(t5));
  return 0;
}
static int yoffe_C3(const double *y, double time, double *C3)
{
  double t1, t2, t3, t4, t5, tau_R2, tau_S = y[0], tau_R = y[1];
  tau_R2 = tau_R * tau_R;
  t1 = tau_S - time - 0.5 * tau_R;
  t2 = (time - tau_S) * (tau_R - time + tau_S);
  t3 = tau_R * (2.0 * tau_R - 2.0 * time + 2.0 * tau_S);
  t4 = (time - tau_S) / tau_R;
  if (fabs(time - tau_S) < 0.0) t5 = 1.0e12; else t5 = (tau_R - time + tau_S) / (time - tau_S);
  if (t2 < 0.0 || t4 < 0.0 || t5 < 0.0) FAIL("reg_yoffe_compute_C3: negative argument");
  *C3 = t1 * sqrt(t2) + t3 * asin(sqrt(t4)) + 1.5 * tau_R2 * atan(sqrt(t5));
  return 0;
}
static int yoffe_C4(const double *y, double time, double *C4)
{
  double t1, t2, t3, t4, t5, tau_R2, tau_S = y[0], tau_R = y[1];
  tau_R2 = tau_R * tau_R;
  t1 = -tau_S + 0.5 * time + 0.25 * tau_R;
  t2 = (time - 2.0 * tau_S) * (tau_R - time + 2.0 * tau_S);
  t3 = tau_R * (-tau_R + time - 2.0 * tau_S);
  t4 = (time - 2.0 * tau_S) / tau_R;
  if (fabs(time - 2.0 * tau_S) < 0.0) t5 = 1.0e12; else t5 = (tau_R - time + 2.0 * tau_S) / (time - 2.0 * tau_S);
  if (t2 < 0.0 || t4 < 0.0 || t5 < 0.0) FAIL("reg_yoffe_compute_C4: negative argument");
  *C4 = t1 * sqrt(t2) + t3 * asin(sqrt(t4)) - 0.75 * tau_R2 * atan(sqrt(t5));
  return 0;
}

static int stf_eval(int type, const double *par, double time, double *psi)
{
  if (type == 0) { /* Ricker, se2wave.c:3504-3516 */
    double arg, arg2, a, b;
    arg = O_PI * par[1] * (time - par[0]);
    arg2 = arg * arg;
    a = 1.0 - 2.0 * arg2;
    b = exp(-arg2);
    *psi = par[2] * a * b;
    return 0;
  }
  if (type == 1) { /* Gaussian, se2wave.c:3552-3561 */
    double arg = par[1] * par[1] * (time - par[0]) * (time - par[0]) * 0.5;
    *psi = par[2] * exp(-arg);
    return 0;
  }
  if (type == 2) { /* triangle-regularised Yoffe, se2wave.c:3683-3822 */
    double tau_S = par[0], tau_R = par[1];
    double K = 2.0 / (O_PI * tau_R * tau_S * tau_S);
    double C1 = 0, C2 = 0, C3 = 0, C4 = 0, C5 = 0, C6 = 0, tau_R2, phi;
    if (time >= (tau_R + 2.0 * tau_S)) { *psi = 0.0; return 0; }
    tau_R2 = tau_R * tau_R;
    if (tau_R > 2.0 * tau_S) { /* mode 1, 3683-3732 */
      if ((time >= 0.0) && (time < tau_S)) {
        if (yoffe_C1(par, time, &C1)) return -1;
        C2 = (3.0 / 8.0) * O_PI * tau_R2;
        phi = C1 + C2;
      } else if ((time >= tau_S) && (time < 2.0 * tau_S)) {
        if (yoffe_C1(par, time, &C1)) return -1;
        C2 = (3.0 / 8.0) * O_PI * tau_R2;
        if (yoffe_C3(par, time, &C3)) return -1;
        phi = C1 - C2 + C3;
      } else if ((time >= 2.0 * tau_S) && (time < tau_R)) {
        if (yoffe_C1(par, time, &C1) || yoffe_C3(par, time, &C3) || yoffe_C4(par, time, &C4)) return -1;
        phi = C1 + C3 + C4;
      } else if ((time >= tau_R) && (time < (tau_R + tau_S))) {
        if (yoffe_C3(par, time, &C3) || yoffe_C4(par, time, &C4)) return -1;
        C5 = 0.5 * O_PI * tau_R * (time - tau_R);
        phi = C5 + C3 + C4;
      } else if ((time >= (tau_R + tau_S)) && (time < (tau_R + 2.0 * tau_S))) {
        if (yoffe_C4(par, time, &C4)) return -1;
        C6 = 0.5 * O_PI * tau_R * (2.0 * tau_S - time + tau_R);
        phi = C4 + C6;
      } else phi = 0.0;
    } else if ((tau_S < tau_R) && (tau_R < 2.0 * tau_S)) { /* mode 2, 3735-3784 */
      if ((time >= 0.0) && (time < tau_S)) {
        if (yoffe_C1(par, time, &C1)) return -1;
        C2 = (3.0 / 8.0) * O_PI * tau_R2;
        phi = C1 + C2;
      } else if ((time >= tau_S) && (time < tau_R)) {
        if (yoffe_C1(par, time, &C1)) return -1;
        C2 = (3.0 / 8.0) * O_PI * tau_R2;
        if (yoffe_C3(par, time, &C3)) return -1;
        phi = C1 - C2 + C3;
      } else if ((time >= tau_R) && (time < 2.0 * tau_S)) {
        C2 = (3.0 / 8.0) * O_PI * tau_R2;
        if (yoffe_C3(par, time, &C3)) return -1;
        C5 = 0.5 * O_PI * tau_R * (time - tau_R);
        phi = C5 + C3 - C2;
      } else if ((time >= 2.0 * tau_S) && (time < (tau_R + tau_S))) {
        if (yoffe_C3(par, time, &C3) || yoffe_C4(par, time, &C4)) return -1;
        C5 = 0.5 * O_PI * tau_R * (time - tau_R);
        phi = C5 + C3 + C4;
      } else if ((time >= (tau_R + tau_S)) && (time < (tau_R + 2.0 * tau_S))) {
        if (yoffe_C4(par, time, &C4)) return -1;
        C6 = 0.5 * O_PI * tau_R * (2.0 * tau_S - time + tau_R);
        phi = C4 + C6;
      } else phi = 0.0;
    } else FAIL("Invalid values for tau_S (%+1.4e) and tau_R(%+1.4e) provided", tau_S, tau_R);
    *psi = K * phi;
    return 0;
  }
  FAIL("unknown STF type %d", type);
}

int se2o_stf(int type, const double par[3], double t0, double dt, long n, double *out)
{
  long k;
  double time = t0;
  if (type == 2 && !((par[1] > 2.0 * par[0]) || ((par[0] < par[1]) && (par[1] < 2.0 * par[0]))))
    FAIL("Invalid values for tau_S (%+1.4e) and tau_R(%+1.4e) provided", par[0], par[1]);
  for (k = 0; k < n; k++) {
    if (stf_eval(type, par, time, &out[k])) return -1;
    time = time + dt;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* set-up                                                              */
/* ------------------------------------------------------------------ */
void se2o_destroy(se2o_ctx *c)
{
  if (!c) return;
  free(c->xi); free(c->w1d); free(c->w); free(c->dN_dxi); free(c->dN_deta); free(c->dN_dx); free(c->dN_dy);
  free(c->element); free(c->coords); free(c->lam); free(c->mu); free(c->rho);
  free(c->u); free(c->v); free(c->a); free(c->f); free(c->g); free(c->Md);
  free(c->ul); free(c->fl); free(c->lu); free(c->lv); free(c->la);
  free(c->src_elem); free(c->src_gll); free(c->src_vals); free(c->src_dofs); free(c->stf_type); free(c->stf_par);
  free(c->rec_xy); free(c->rec_nid); free(c->rec_eid); free(c->rec_gll);
  free(c);
}

/* SeismicSourceCreate (se2wave.c:2995-3243) + SeismicSourceSetup_Moment_Pointwise (3310-3429),
   moment source, SOURCE_IMPL_NEAREST_QPOINT */
static int setup_source(se2o_ctx *c, int s, const double coor[2], const double m[4], int nearest_internal)
{
  double gmin[2], gmax[2], gmin_d[2], gmax_d[2], dx, dy;
  int ii, jj, e, i, ni, nj, min_qp = -1, qi, qj, n1 = c->n1, npe = c->npe;
  const int *elnidx;
  double sep2, sep2_min = DBL_MAX, xi[2];
  double *dphi_xi, *Ni_xi, *dphi_eta, *Ni_eta, *dNdxi, *dNdeta, *dNdx, *dNdy, elc[2 * 81];

  bounding_box(c, gmin, gmax);
  dx = (gmax[0] - gmin[0]) / ((double)c->mx);
  dy = (gmax[1] - gmin[1]) / ((double)c->my);
  if (coor[0] < gmin[0]) FAIL("Source x-coordinate (%+1.4e) < min(domain).x (%+1.4e)", coor[0], gmin[0]);
  if (coor[1] < gmin[1]) FAIL("Source y-coordinate (%+1.4e) < min(domain).y (%+1.4e)", coor[1], gmin[1]);
  if (coor[0] > gmax[0]) FAIL("Source x-coordinate (%+1.4e) > max(domain).x (%+1.4e)", coor[0], gmax[0]);
  if (coor[1] > gmax[1]) FAIL("Source y-coordinate (%+1.4e) > max(domain).y (%+1.4e)", coor[1], gmax[1]);
  /* SpecFECtxGetLocalBoundingBox (915-937) on one rank: first and last node */
  gmin_d[0] = c->coords[0]; gmin_d[1] = c->coords[1];
  gmax_d[0] = c->coords[2 * (c->nnodes - 1)]; gmax_d[1] = c->coords[2 * (c->nnodes - 1) + 1];
  if (coor[0] < gmin_d[0] || coor[1] < gmin_d[1] || coor[0] > gmax_d[0] || coor[1] > gmax_d[1])
    FAIL("A source was defined but no rank claimed it");
  ii = (int)((coor[0] - gmin_d[0]) / dx);
  jj = (int)((coor[1] - gmin_d[1]) / dy);
  if (ii == c->mx) ii--;
  if (jj == c->my) jj--;
  if (ii < 0 || jj < 0 || ii >= c->mx || jj >= c->my) FAIL("A source was defined but no rank claimed it");
  e = ii + jj * c->mx;
  if (c->p == 1 && nearest_internal)
    FAIL("Cannot use basis degree = 1 and approximate the source location based on nearest cell interior GLL point. "
         "You must provide the command line option -use_nearest_internal_gll false");
  elnidx = &c->element[npe * e];
  for (i = 0; i < npe; i++) { elc[2 * i] = c->coords[2 * elnidx[i]]; elc[2 * i + 1] = c->coords[2 * elnidx[i] + 1]; }
  {
    int lo = nearest_internal ? 1 : 0, hi = nearest_internal ? n1 - 1 : n1;
    for (nj = lo; nj < hi; nj++) {
      for (ni = lo; ni < hi; ni++) {
        int nid = ni + nj * n1;
        sep2 = (elc[2 * nid] - coor[0]) * (elc[2 * nid] - coor[0]) + (elc[2 * nid + 1] - coor[1]) * (elc[2 * nid + 1] - coor[1]);
        if (sep2 < sep2_min) { sep2_min = sep2; min_qp = nid; }
      }
    }
  }
  if (min_qp < 0) FAIL("Failed to identify a closest quadrature point");
  c->src_elem[s] = e;
  c->src_gll[s] = min_qp;
  qj = min_qp / n1;
  qi = min_qp - qj * n1;
  xi[0] = c->xi[qi];
  xi[1] = c->xi[qj];
  for (i = 0; i < npe; i++) { c->src_dofs[s * 2 * npe + 2 * i] = 2 * elnidx[i]; c->src_dofs[s * 2 * npe + 2 * i + 1] = 2 * elnidx[i] + 1; }
  /* TabulateBasisDerivativesAtPointTensorProduct2d (605-690) */
  dphi_xi = (double*)malloc(sizeof(double) * n1); Ni_xi = (double*)malloc(sizeof(double) * n1);
  dphi_eta = (double*)malloc(sizeof(double) * n1); Ni_eta = (double*)malloc(sizeof(double) * n1);
  dNdxi = (double*)malloc(sizeof(double) * npe); dNdeta = (double*)malloc(sizeof(double) * npe);
  dNdx = (double*)malloc(sizeof(double) * npe); dNdy = (double*)malloc(sizeof(double) * npe);
  if (dbasis1d(1, &xi[0], c->p, dphi_xi) || basis1d(1, &xi[0], c->p, Ni_xi) ||
      dbasis1d(1, &xi[1], c->p, dphi_eta) || basis1d(1, &xi[1], c->p, Ni_eta)) return -1;
  {
    int k = 0, a, b;
    for (b = 0; b < n1; b++) for (a = 0; a < n1; a++) {
      dNdxi[k] = dphi_xi[a] * Ni_eta[b];
      dNdeta[k] = Ni_xi[a] * dphi_eta[b];
      k++;
    }
  }
  el_derivatives(1, npe, elc, n1, dNdxi, dNdeta, dNdx, dNdy);
  for (i = 0; i < npe; i++) {
    c->src_vals[s * 2 * npe + 2 * i] = (m[0] * dNdx[i] + m[1] * dNdy[i]);
    c->src_vals[s * 2 * npe + 2 * i + 1] = (m[2] * dNdx[i] + m[3] * dNdy[i]);
  }
  free(dphi_xi); free(Ni_xi); free(dphi_eta); free(Ni_eta); free(dNdxi); free(dNdeta); free(dNdx); free(dNdy);
  return 0;
}

/* receiver location, first call of RecordUVA_MultipleStations_NearestGLL_MPI (se2wave.c:2700-2810) */
static int setup_receiver(se2o_ctx *c, int r)
{
  double gmin[2], gmax[2], gmin_d[2], gmax_d[2], dx, dy, sep2, sep2min;
  double xr = c->rec_xy[2 * r], yr = c->rec_xy[2 * r + 1];
  int ei, ej, eid, n, nid = -1, gllid = -1;
  const int *elbasis;
  bounding_box(c, gmin, gmax);
  gmin_d[0] = c->coords[0]; gmin_d[1] = c->coords[1];
  gmax_d[0] = c->coords[2 * (c->nnodes - 1)]; gmax_d[1] = c->coords[2 * (c->nnodes - 1) + 1];
  if (xr < gmin[0]) FAIL("Receiver %d, x-coordinate (%+1.4e) < min(domain).x (%+1.4e)", r, xr, gmin[0]);
  if (yr < gmin[1]) FAIL("Receiver %d, y-coordinate (%+1.4e) < min(domain).y (%+1.4e)", r, yr, gmin[1]);
  if (xr > gmax[0]) FAIL("Receiver %d, x-coordinate (%+1.4e) > max(domain).x (%+1.4e)", r, xr, gmax[0]);
  if (yr > gmax[1]) FAIL("Receiver %d, y-coordinate (%+1.4e) > max(domain).y (%+1.4e)", r, yr, gmax[1]);
  if (xr < gmin_d[0] || yr < gmin_d[1] || xr > gmax_d[0] || yr > gmax_d[1]) FAIL("A receiver was defined but no rank claimed it");
  dx = (gmax[0] - gmin[0]) / ((double)c->mx);
  ei = (int)((xr - gmin_d[0]) / dx);
  if (ei == c->mx) ei--;
  dy = (gmax[1] - gmin[1]) / ((double)c->my);
  ej = (int)((yr - gmin_d[1]) / dy);
  if (ej == c->my) ej--;
  if (ei < 0 || ej < 0 || ei > c->mx || ej > c->my) FAIL("A receiver was defined but no rank claimed it");
  eid = ei + ej * c->mx;
  elbasis = &c->element[c->npe * eid];
  sep2min = 1.0e32;
  for (n = 0; n < c->npe; n++) {
    sep2 = (xr - c->coords[2 * elbasis[n]]) * (xr - c->coords[2 * elbasis[n]]);
    sep2 += (yr - c->coords[2 * elbasis[n] + 1]) * (yr - c->coords[2 * elbasis[n] + 1]);
    if (sep2 < sep2min) { nid = elbasis[n]; gllid = n; sep2min = sep2; }
  }
  c->rec_nid[r] = nid; c->rec_eid[r] = eid; c->rec_gll[r] = gllid;
  return 0;
}

int se2o_create(const se2o_spec *sp, se2o_ctx **out)
{
  se2o_ctx *c;
  int i, j, ei, ej, e, q, n1, npe;
  double *D1;
  *out = NULL;
  if (sp->p < 1 || sp->p > 8) FAIL("bdegree must be in 1..8");
  if (sp->mx < 1 || sp->my < 1) FAIL("mx, my must be >= 1");
  c = (se2o_ctx*)calloc(1, sizeof(se2o_ctx));
  c->mx = sp->mx; c->my = sp->my; c->p = sp->p;
  n1 = c->n1 = sp->p + 1;
  npe = c->npe = n1 * n1;
  c->ne = sp->mx * sp->my;
  c->nx_g = sp->p * sp->mx + 1;
  c->ny_g = sp->p * sp->my + 1;
  c->nnodes = c->nx_g * c->ny_g;
  c->ndof = 2 * c->nnodes;

  /* SpecFECtxCreateMesh_SEQ (825-884) */
  c->xi = (double*)malloc(sizeof(double) * n1);
  c->w1d = (double*)malloc(sizeof(double) * n1);
  gll(sp->p, c->xi, c->w1d);
  c->w = (double*)malloc(sizeof(double) * npe);
  for (j = 0; j < n1; j++) for (i = 0; i < n1; i++) c->w[i + j * n1] = c->w1d[i] * c->w1d[j];
  /* TabulateBasisDerivativesTensorProduct2d (525-603) */
  D1 = (double*)malloc(sizeof(double) * npe);
  {
    double *xq = (double*)malloc(sizeof(double) * n1);
    gll(sp->p, xq, NULL);
    if (dbasis1d(n1, xq, sp->p, D1)) { free(xq); free(D1); se2o_destroy(c); return -1; }
    free(xq);
  }
  c->dN_dxi = (double*)malloc(sizeof(double) * npe * npe);
  c->dN_deta = (double*)malloc(sizeof(double) * npe * npe);
  c->dN_dx = (double*)malloc(sizeof(double) * npe * npe);
  c->dN_dy = (double*)malloc(sizeof(double) * npe * npe);
  {
    int qi, qj, k, qpoint = 0;
    for (qj = 0; qj < n1; qj++) for (qi = 0; qi < n1; qi++) {
      k = 0;
      for (j = 0; j < n1; j++) for (i = 0; i < n1; i++) {
        double phi_xi = (qi == i) ? 1.0 : 0.0, phi_eta = (qj == j) ? 1.0 : 0.0;
        c->dN_dxi[qpoint * npe + k] = D1[qi * n1 + i] * phi_eta;
        c->dN_deta[qpoint * npe + k] = phi_xi * D1[qj * n1 + j];
        k++;
      }
      qpoint++;
    }
  }
  free(D1);
  /* SpecFECtxCreateENMap2d_SEQ (706-736) */
  c->element = (int*)malloc(sizeof(int) * (size_t)c->ne * npe);
  for (ej = 0, e = 0; ej < c->my; ej++) for (ei = 0; ei < c->mx; ei++, e++) {
    int ni0 = ei * (n1 - 1), nj0 = ej * (n1 - 1);
    for (j = 0; j < n1; j++) for (i = 0; i < n1; i++) c->element[(size_t)npe * e + i + j * n1] = (ni0 + i) + (nj0 + j) * c->nx_g;
  }
  /* SpecFECtxCreateMeshCoords2d_SEQ (739-779): later elements overwrite shared nodes */
  c->coords = (double*)calloc((size_t)c->ndof, sizeof(double));
  {
    double dx = 1.0 / ((double)c->mx), dy = 1.0 / ((double)c->my), x0, y0;
    for (ej = 0; ej < c->my; ej++) for (ei = 0; ei < c->mx; ei++) {
      int ni0 = ei * (n1 - 1), nj0 = ej * (n1 - 1);
      x0 = 0.0 + ei * dx;
      y0 = 0.0 + ej * dy;
      for (j = 0; j < n1; j++) for (i = 0; i < n1; i++) {
        size_t nid = (size_t)(ni0 + i) + (size_t)(nj0 + j) * c->nx_g;
        c->coords[2 * nid + 0] = 0.5 * (c->xi[i] + 1.0) * dx + x0;
        c->coords[2 * nid + 1] = 0.5 * (c->xi[j] + 1.0) * dy + y0;
      }
    }
  }
  /* SpecFECtxScaleMeshCoords (781-823): VecStrideScale, then VecAXPY(coor,1.0,ss) per component */
  for (i = 0; i < c->nnodes; i++) { c->coords[2 * i] *= sp->scale[0]; c->coords[2 * i + 1] *= sp->scale[1]; }
  for (i = 0; i < c->nnodes; i++) { c->coords[2 * i] = c->coords[2 * i] + 1.0 * sp->shift[0]; c->coords[2 * i + 1] = c->coords[2 * i + 1] + 1.0 * 0.0; }
  for (i = 0; i < c->nnodes; i++) { c->coords[2 * i] = c->coords[2 * i] + 1.0 * 0.0; c->coords[2 * i + 1] = c->coords[2 * i + 1] + 1.0 * sp->shift[1]; }
  /* materials (1161-1175) */
  c->lam = (double*)malloc(sizeof(double) * c->ne);
  c->mu = (double*)malloc(sizeof(double) * c->ne);
  c->rho = (double*)malloc(sizeof(double) * c->ne);
  {
    /* perturbed (1177-1236): VecSetRandom of three Vecs with RAND48 seeded 1, 2, 3 */
    double *pv = NULL;
    if (!sp->cell_vp && sp->perturb) {
      const double base[3] = {sp->vp, sp->vs, sp->rho}, del[3] = {sp->dvp, sp->dvs, sp->drho};
      int f;
      pv = (double*)malloc(sizeof(double) * 3 * (size_t)c->ne);
      for (f = 0; f < 3; f++) {
        double low = base[f] - del[f], width = (base[f] + del[f]) - low;
        unsigned long long x = ((unsigned long long)(unsigned int)(f + 1) << 16) | 0x330EULL;
        for (e = 0; e < c->ne; e++) {
          x = (0x5DEECE66DULL * x + 0xBULL) & 0xFFFFFFFFFFFFULL;
          pv[f * c->ne + e] = width * ((double)x / 281474976710656.0) + low;
        }
      }
    }
    for (e = 0; e < c->ne; e++) {
      double vp = pv ? pv[e] : sp->cell_vp ? sp->cell_vp[e] : sp->vp;
      double vs = pv ? pv[c->ne + e] : sp->cell_vs ? sp->cell_vs[e] : sp->vs;
      double rho = pv ? pv[2 * c->ne + e] : sp->cell_rho ? sp->cell_rho[e] : sp->rho;
      double mu = vs * vs * rho;
      double lambda = vp * vp * rho - 2.0 * mu;
      c->lam[e] = lambda; c->mu[e] = mu; c->rho[e] = rho;
    }
    free(pv);
  }
  /* vectors */
  c->u = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->v = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->a = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->f = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->g = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->Md = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->ul = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->fl = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->lu = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->lv = (double*)calloc((size_t)c->ndof, sizeof(double));
  c->la = (double*)calloc((size_t)c->ndof, sizeof(double));
  /* AssembleBilinearForm_Mass2d (1431-1498) */
  for (e = 0; e < c->ne; e++) {
    const int *elnidx = &c->element[(size_t)npe * e];
    double detJ;
    for (i = 0; i < npe; i++) { c->elcoords[2 * i] = c->coords[2 * elnidx[i]]; c->elcoords[2 * i + 1] = c->coords[2 * elnidx[i] + 1]; }
    el_geometry(npe, c->elcoords, n1, &detJ);
    for (q = 0; q < npe; q++) {
      double fac = detJ * c->w[q];
      double Me_ii = fac * (c->rho[e]);
      c->Md[2 * elnidx[q]] += Me_ii;
      c->Md[2 * elnidx[q] + 1] += Me_ii;
    }
  }
  /* sources */
  c->nsrc = sp->nsrc;
  c->src_elem = (int*)calloc((size_t)(sp->nsrc + 1), sizeof(int));
  c->src_gll = (int*)calloc((size_t)(sp->nsrc + 1), sizeof(int));
  c->src_vals = (double*)calloc((size_t)(sp->nsrc * 2 * npe + 1), sizeof(double));
  c->src_dofs = (int*)calloc((size_t)(sp->nsrc * 2 * npe + 1), sizeof(int));
  c->stf_type = (int*)calloc((size_t)(sp->nsrc + 1), sizeof(int));
  c->stf_par = (double*)calloc((size_t)(3 * sp->nsrc + 1), sizeof(double));
  for (i = 0; i < sp->nsrc; i++) {
    if (setup_source(c, i, &sp->src_xy[2 * i], &sp->src_m[4 * i], sp->nearest_internal_gll)) { se2o_destroy(c); return -1; }
    c->stf_type[i] = sp->stf_type[i];
    memcpy(&c->stf_par[3 * i], &sp->stf_par[3 * i], 3 * sizeof(double));
    if (sp->stf_type[i] == 2) {
      double tS = sp->stf_par[3 * i], tR = sp->stf_par[3 * i + 1];
      if (!((tR > 2.0 * tS) || ((tS < tR) && (tR < 2.0 * tS)))) { se2o_destroy(c); FAIL("Invalid values for tau_S (%+1.4e) and tau_R(%+1.4e) provided", tS, tR); }
    }
  }
  /* receivers */
  c->nrec = sp->nrec;
  c->rec_xy = (double*)calloc((size_t)(2 * sp->nrec + 1), sizeof(double));
  c->rec_nid = (int*)calloc((size_t)(sp->nrec + 1), sizeof(int));
  c->rec_eid = (int*)calloc((size_t)(sp->nrec + 1), sizeof(int));
  c->rec_gll = (int*)calloc((size_t)(sp->nrec + 1), sizeof(int));
  if (sp->nrec) memcpy(c->rec_xy, sp->rec_xy, sizeof(double) * 2 * sp->nrec);
  for (i = 0; i < sp->nrec; i++) if (setup_receiver(c, i)) { se2o_destroy(c); return -1; }
  /* ElastoDynamicsComputeTimeStep_2d (2276-2349) */
  {
    double gmin[2], gmax[2], dx, dy, min_el_r, sep2min, dt_min = DBL_MAX, polynomial_fac;
    int n;
    bounding_box(c, gmin, gmax);
    dx = (gmax[0] - gmin[0]) / ((double)c->mx);
    dy = (gmax[1] - gmin[1]) / ((double)c->my);
    min_el_r = dx;
    min_el_r = (min_el_r < dy) ? min_el_r : dy;
    sep2min = 1.0e32;
    for (n = 0; n < n1 - 1; n++) { double s2 = fabs(c->xi[n + 1] - c->xi[n]); if (s2 < sep2min) sep2min = s2; }
    polynomial_fac = 1.0;
    min_el_r = min_el_r * (sep2min / 2.0);
    for (e = 0; e < c->ne; e++) {
      double max_el_Vp = -DBL_MAX, value;
      for (q = 0; q < npe; q++) {
        double Vp = sqrt((c->lam[e] + 2.0 * c->mu[e]) / c->rho[e]);
        max_el_Vp = (max_el_Vp < Vp) ? Vp : max_el_Vp;
      }
      value = polynomial_fac * 1.0 * min_el_r / max_el_Vp;
      dt_min = (dt_min < value) ? dt_min : value;
    }
    c->dt_cfl = dt_min;
  }
  c->dt = c->dt_cfl * sp->cfl;
  if (sp->dt > 0.0) c->dt = sp->dt;
  c->tmax = sp->tmax;
  {
    /* (PetscInt)(tmax/dt)+4, saturated where the reference's conversion would overflow */
    double q = c->tmax / c->dt;
    c->nt = (q < 2147483000.0) ? (long)(int)q + 4 : 2147483647L;
  }
  if (sp->nt >= 0) c->nt = sp->nt;
  c->time = 0.0;
  c->k = 0;
  *out = c;
  return 0;
}

int se2o_info(const se2o_ctx *c, int *ints, double *dbls)
{
  long k, n = 0;
  double t = 0.0;
  for (k = 1; k <= c->nt; k++) { t = t + c->dt; n = k; if (t >= c->tmax) break; }
  ints[0] = c->nx_g; ints[1] = c->ny_g; ints[2] = c->n1; ints[3] = (int)n; ints[4] = c->nrec; ints[5] = c->nsrc;
  dbls[0] = c->dt; dbls[1] = c->dt_cfl; dbls[2] = c->tmax;
  return 0;
}

int se2o_get(const se2o_ctx *c, const char *name, double *out, long n)
{
  long i, need = 0;
  if (!strcmp(name, "xi")) { need = c->n1; if (n >= need) memcpy(out, c->xi, sizeof(double) * need); }
  else if (!strcmp(name, "w1d")) { need = c->n1; if (n >= need) memcpy(out, c->w1d, sizeof(double) * need); }
  else if (!strcmp(name, "w")) { need = c->npe; if (n >= need) memcpy(out, c->w, sizeof(double) * need); }
  else if (!strcmp(name, "D")) {
    need = c->n1 * c->n1;
    /* row q of the 1-D derivative matrix is dN_dxi at q=(qi,0) restricted to k=(i,0) */
    if (n >= need) for (i = 0; i < need; i++) out[i] = c->dN_dxi[(i / c->n1) * c->npe + (i % c->n1)];
  }
  else if (!strcmp(name, "dN_dxi")) { need = (long)c->npe * c->npe; if (n >= need) memcpy(out, c->dN_dxi, sizeof(double) * need); }
  else if (!strcmp(name, "dN_deta")) { need = (long)c->npe * c->npe; if (n >= need) memcpy(out, c->dN_deta, sizeof(double) * need); }
  else if (!strcmp(name, "coords")) { need = c->ndof; if (n >= need) memcpy(out, c->coords, sizeof(double) * need); }
  else if (!strcmp(name, "mass")) { need = c->ndof; if (n >= need) memcpy(out, c->Md, sizeof(double) * need); }
  else if (!strcmp(name, "cell_lmr")) {
    need = 3L * c->ne;
    if (n >= need) for (i = 0; i < c->ne; i++) { out[i] = c->lam[i]; out[c->ne + i] = c->mu[i]; out[2 * c->ne + i] = c->rho[i]; }
  }
  else if (!strcmp(name, "src_values")) { need = (long)c->nsrc * 2 * c->npe; if (n >= need) memcpy(out, c->src_vals, sizeof(double) * need); }
  else if (!strcmp(name, "src_index")) {
    need = 2L * c->nsrc;
    if (n >= need) for (i = 0; i < c->nsrc; i++) { out[2 * i] = c->src_elem[i]; out[2 * i + 1] = c->src_gll[i]; }
  }
  else if (!strcmp(name, "rec_index")) {
    need = 3L * c->nrec;
    if (n >= need) for (i = 0; i < c->nrec; i++) { out[3 * i] = c->rec_nid[i]; out[3 * i + 1] = c->rec_eid[i]; out[3 * i + 2] = c->rec_gll[i]; }
  }
  else FAIL("unknown array %s", name);
  if (n < need) FAIL("buffer too small for %s: need %ld", name, need);
  return 0;
}

int se2o_get_state(const se2o_ctx *c, double *u, double *v, double *a)
{
  if (u) memcpy(u, c->u, sizeof(double) * c->ndof);
  if (v) memcpy(v, c->v, sizeof(double) * c->ndof);
  if (a) memcpy(a, c->a, sizeof(double) * c->ndof);
  return 0;
}

int se2o_set_state(se2o_ctx *c, const double *u, const double *v, const double *a, double time)
{
  if (u) memcpy(c->u, u, sizeof(double) * c->ndof);
  if (v) memcpy(c->v, v, sizeof(double) * c->ndof);
  if (a) memcpy(c->a, a, sizeof(double) * c->ndof);
  c->time = time;
  return 0;
}

/* ------------------------------------------------------------------ */
/* AssembleLinearForm_ElastoDynamics2d, se2wave.c:1285-1429            */
/* ------------------------------------------------------------------ */
static void assemble_linear_form(se2o_ctx *c, const double *u, double *F)
{
  int e, q, i;
  const int npe = c->npe, n1 = c->n1;
  double *fe = c->fe, *ux = c->ux, *uy = c->uy, *elc = c->elcoords;
  int *eldofs = c->eldofs;
  memset(F, 0, sizeof(double) * c->ndof);                   /* VecZeroEntries(F) */
  memcpy(c->ul, u, sizeof(double) * c->ndof);               /* DMGlobalToLocal(u -> ul) */
  memset(c->fl, 0, sizeof(double) * c->ndof);               /* VecZeroEntries(fl) */
  for (e = 0; e < c->ne; e++) {
    const int *elnidx = &c->element[(size_t)npe * e];
    double detJ, e0, e1, e2, c11, c12, c21, c22, c33, lambda_qp, mu_qp, sxx, syy, sxy;
    for (i = 0; i < npe; i++) { eldofs[2 * i] = 2 * elnidx[i]; eldofs[2 * i + 1] = 2 * elnidx[i] + 1; }
    for (i = 0; i < npe; i++) { elc[2 * i] = c->coords[2 * elnidx[i]]; elc[2 * i + 1] = c->coords[2 * elnidx[i] + 1]; }
    for (i = 0; i < npe; i++) { ux[i] = c->ul[2 * elnidx[i]]; uy[i] = c->ul[2 * elnidx[i] + 1]; }
    el_geometry(npe, elc, n1, &detJ);
    el_derivatives(npe, npe, elc, n1, c->dN_dxi, c->dN_deta, c->dN_dx, c->dN_dy);
    memset(fe, 0, sizeof(double) * 2 * npe);
    for (q = 0; q < npe; q++) {
      const double *dNidx = &c->dN_dx[q * npe], *dNidy = &c->dN_dy[q * npe];
      double fac;
      e0 = e1 = e2 = 0.0;
      for (i = 0; i < npe; i++) {
        e0 += dNidx[i] * ux[i];
        e1 += dNidy[i] * uy[i];
        e2 += (dNidx[i] * uy[i] + dNidy[i] * ux[i]);
      }
      lambda_qp = c->lam[e];
      mu_qp = c->mu[e];
      c11 = 2.0 * mu_qp + lambda_qp;
      c12 = lambda_qp;
      c21 = lambda_qp;
      c22 = 2.0 * mu_qp + lambda_qp;
      c33 = mu_qp;
      sxx = c11 * e0 + c12 * e1;
      syy = c21 * e0 + c22 * e1;
      sxy = c33 * e2;
      fac = detJ * c->w[q];
      for (i = 0; i < npe; i++) {
        fe[2 * i] += -fac * (dNidx[i] * sxx + dNidy[i] * sxy);
        fe[2 * i + 1] += -fac * (dNidy[i] * syy + dNidx[i] * sxy);
      }
    }
    for (i = 0; i < 2 * npe; i++) c->fl[eldofs[i]] += fe[i];  /* VecSetValues(fl, ADD) */
  }
  for (i = 0; i < c->ndof; i++) F[i] += c->fl[i];          /* DMLocalToGlobal(fl -> F, ADD) */
}

int se2o_force(se2o_ctx *c, const double *u, double *F)
{
  assemble_linear_form(c, u, F);
  return 0;
}

/* SeismicSourceEvaluate (3470-3497) + SeismicSourceAddValues_Pointwise (3277-3293) */
static int source_evaluate(se2o_ctx *c, double time, double *g)
{
  int s, k;
  memset(g, 0, sizeof(double) * c->ndof);
  for (s = 0; s < c->nsrc; s++) {
    double value;
    if (stf_eval(c->stf_type[s], &c->stf_par[3 * s], time, &value)) return -1;
    for (k = 0; k < 2 * c->npe; k++) {
      double b = value * c->src_vals[s * 2 * c->npe + k];
      g[c->src_dofs[s * 2 * c->npe + k]] += b;
    }
  }
  return 0;
}

/* per-step part of RecordUVA_MultipleStations_NearestGLL_MPI (2886-2981) */
static void record(se2o_ctx *c, double time, double *row)
{
  int r, k;
  memcpy(c->lu, c->u, sizeof(double) * c->ndof);   /* DMGlobalToLocal x3 */
  memcpy(c->lv, c->v, sizeof(double) * c->ndof);
  memcpy(c->la, c->a, sizeof(double) * c->ndof);
  if (!row) return;
  row[0] = time;
  for (r = 0; r < c->nrec; r++) {
    int nid = c->rec_nid[r], eidx = c->rec_eid[r], gll_ = c->rec_gll[r];
    double elc[2 * 81], vel[2 * 81], gx[81], gy[81], dvxdy, dvydx;
    double *o = &row[1 + 7 * r];
    o[0] = c->lu[2 * nid]; o[1] = c->lu[2 * nid + 1];
    o[2] = c->lv[2 * nid]; o[3] = c->lv[2 * nid + 1];
    o[4] = c->la[2 * nid]; o[5] = c->la[2 * nid + 1];
    for (k = 0; k < c->npe; k++) {
      int b = c->element[(size_t)c->npe * eidx + k];
      elc[2 * k] = c->coords[2 * b]; elc[2 * k + 1] = c->coords[2 * b + 1];
      vel[2 * k] = c->lv[2 * b]; vel[2 * k + 1] = c->lv[2 * b + 1];
    }
    el_derivatives(1, c->npe, elc, c->n1, &c->dN_dxi[gll_ * c->npe], &c->dN_deta[gll_ * c->npe], gx, gy);
    dvxdy = 0.0;
    dvydx = 0.0;
    for (k = 0; k < c->npe; k++) {
      double vx = vel[2 * k], vy = vel[2 * k + 1];
      dvxdy += gy[k] * vx;
      dvydx += gx[k] * vy;
    }
    o[6] = dvydx - dvxdy;
  }
}

static void axpy(long n, double *y, double a, const double *x)
{
  long i;
  if (a == 0.0) return;
  for (i = 0; i < n; i++) y[i] = y[i] + a * x[i];
}

static void norms(const se2o_ctx *c, double *r)
{
  long i;
  const double *vecs[2] = { c->u, c->v };
  int t;
  for (t = 0; t < 2; t++) {
    double mx = -DBL_MAX, mn = DBL_MAX, s = 0.0;
    for (i = 0; i < c->ndof; i++) {
      double x = vecs[t][i];
      if (x > mx) mx = x;
      if (x < mn) mn = x;
      s = s + x * x;
    }
    r[3 * t] = mx; r[3 * t + 1] = mn; r[3 * t + 2] = sqrt(s);
  }
}

/* the time loop of se2wave_demo, se2wave.c:4722-4775 */
long se2o_run(se2o_ctx *c, long nsteps, double *traces, double *nrm, long max_norm_rows)
{
  long taken = 0, nrows = 0;
  const long width = 1 + 7L * c->nrec;
  const double dt = c->dt;
  while (taken < nsteps && c->k < c->nt) {
    long i;
    c->k++;
    c->time = c->time + dt;
    axpy(c->ndof, c->u, dt, c->v);
    axpy(c->ndof, c->u, 0.5 * dt * dt, c->a);
    axpy(c->ndof, c->v, 0.5 * dt, c->a);
    if (source_evaluate(c, c->time, c->g)) return -1;
    assemble_linear_form(c, c->u, c->f);
    axpy(c->ndof, c->f, 1.0, c->g);
    for (i = 0; i < c->ndof; i++) c->a[i] = c->f[i] / c->Md[i];
    axpy(c->ndof, c->v, 0.5 * dt, c->a);
    if (nrm && (c->k % 100 == 0) && nrows < max_norm_rows) {
      nrm[7 * nrows] = (double)c->k;
      norms(c, &nrm[7 * nrows + 1]);
      nrows++;
    }
    if (c->nrec > 0) record(c, c->time, traces ? &traces[taken * width] : NULL);
    taken++;
    if (c->time >= c->tmax) { c->k = c->nt; break; }
  }
  return taken;
}

/* ------------------------------------------------------------------ */
/* CPU baseline: independent solves on host threads                    */
/* ------------------------------------------------------------------ */
typedef struct {
  const se2o_spec *sp;
  long warmup, nsteps;
  int record;
  pthread_barrier_t *bar;
  double seconds;
  int err;
} bench_arg;

static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void *bench_thread(void *p)
{
  bench_arg *b = (bench_arg*)p;
  se2o_ctx *c = NULL;
  double *tr = NULL, t0;
  b->err = se2o_create(b->sp, &c);
  if (!b->err) {
    c->nt = b->warmup + b->nsteps + 1;
    c->tmax = DBL_MAX;
    if (b->record && c->nrec) tr = (double*)malloc(sizeof(double) * (size_t)(1 + 7 * c->nrec) * (size_t)(b->warmup + b->nsteps + 1));
    se2o_run(c, b->warmup, tr, NULL, 0);
  }
  pthread_barrier_wait(b->bar);
  t0 = now_s();
  if (!b->err) se2o_run(c, b->nsteps, tr, NULL, 0);
  b->seconds = now_s() - t0;
  pthread_barrier_wait(b->bar);
  free(tr);
  se2o_destroy(c);
  return NULL;
}

double se2o_bench(const se2o_spec *sp, int nthreads, long warmup, long nsteps, int record)
{
  pthread_t *th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
  bench_arg *args = (bench_arg*)calloc((size_t)nthreads, sizeof(bench_arg));
  pthread_barrier_t bar;
  double mx = 0.0;
  int t, err = 0;
  pthread_barrier_init(&bar, NULL, (unsigned)nthreads);
  for (t = 0; t < nthreads; t++) {
    args[t].sp = sp; args[t].warmup = warmup; args[t].nsteps = nsteps; args[t].record = record; args[t].bar = &bar;
    pthread_create(&th[t], NULL, bench_thread, &args[t]);
  }
  for (t = 0; t < nthreads; t++) {
    pthread_join(th[t], NULL);
    if (args[t].seconds > mx) mx = args[t].seconds;
    if (args[t].err) err = 1;
  }
  pthread_barrier_destroy(&bar);
  free(th); free(args);
  return err ? -1.0 : mx;
}
