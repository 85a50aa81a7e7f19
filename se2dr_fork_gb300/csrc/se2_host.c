/*
 * se2_host.c -- FP64 host set-up for the GB300 SEM time loop (see include/se2host.h).
 *
 * Runs once per problem on the CPU.  The mesh of se2wave is a structured tensor
 * product, so instead of the reference's element-to-node map and interleaved
 * coordinate vector this keeps one coordinate per node column (xnode) and per
 * node row (ynode) and derives every index; the numbers produced are the
 * reference's bit for bit.  Compiled with -ffp-contract=off: no expression here
 * may be fused into a multiply-add, because the reference's x86-64 -O2 build
 * rounds every product and sum separately.
 */
#include "se2host.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define SE2_PI 3.14159265358979323846264338327950288419716939937510582

static __thread char g_err[512];
const char *se2_host_last_error(void) { return g_err; }
#define SE2_FAIL(...) do { snprintf(g_err, sizeof(g_err), __VA_ARGS__); return -1; } while (0)

static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

/* ------------------------------------------------------------------ */
/* GLL nodes and weights: Newton iteration on P_N from the Chebyshev-  */
/* Gauss-Lobatto points (se2wave.c:103-209).                           */
/* ------------------------------------------------------------------ */
int se2_gll(int N, double *xi, double *w)
{
  const int n1 = N + 1;
  double *x, *x_prev, *L;
  double res = 1.0;
  int i, k;
  if (N < 1 || N > 16) SE2_FAIL("polynomial degree %d out of range", N);
  x = (double*)xcalloc((size_t)n1, sizeof(double));
  x_prev = (double*)xcalloc((size_t)n1, sizeof(double));
  L = (double*)xcalloc((size_t)(n1 * n1), sizeof(double)); /* L[i + k*n1] = P_k(x_i) */
  for (i = 0; i < n1; i++) x[i] = cos(SE2_PI * i / (double)N);
  while (res > 1.0e-12) {
    for (i = 0; i < n1; i++) x_prev[i] = x[i];
    for (i = 0; i < n1; i++) { L[i] = 1.0; L[i + n1] = x[i]; }
    for (i = 0; i < n1; i++)
      for (k = 1; k < N; k++)
        L[i + (k + 1) * n1] = ((2.0 * (k + 1) - 1.0) * x[i] * L[i + k * n1] - (k + 1.0 - 1.0) * L[i + (k - 1) * n1]) / (double)(k + 1.0);
    for (i = 0; i < n1; i++)
      x[i] = x_prev[i] - (x[i] * L[i + (n1 - 1) * n1] - L[i + (N - 1) * n1]) / (n1 * L[i + (n1 - 1) * n1]);
    res = 0.0;
    for (i = 0; i < n1; i++) res += (x[i] - x_prev[i]) * (x[i] - x_prev[i]);
    res = sqrt(res);
  }
  if (w)
    for (i = 0; i < n1; i++) { double pn = L[i + (n1 - 1) * n1]; w[i] = 2.0 / (N * n1 * pn * pn); }
  if (xi)
    for (i = 0; i < n1; i++) xi[i] = x[n1 - 1 - i];  /* ascending: the iteration runs from +1 to -1 */
  free(x); free(x_prev); free(L);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Lagrange basis through the GLL nodes in monomial form: the columns  */
/* of the inverse Vandermonde matrix, from a partial-pivot LU with the */
/* operation order of reference LAPACK dgetf2/dgetrs (the PCLU solve   */
/* of se2wave.c:278-334).  coef[b*n + j] multiplies x^j in N_b.        */
/* ------------------------------------------------------------------ */
static int lagrange_monomial_coefs(int p, double *coef)
{
  const int n = p + 1;
  double nodes[17], LU[17 * 17], rhs[17];
  int piv[17], r, c, k;
  if (se2_gll(p, nodes, NULL)) return -1;
  for (r = 0; r < n; r++)
    for (c = 0; c < n; c++) LU[r + c * n] = pow(nodes[r], (double)c);    /* column-major V[r][c] = x_r^c */
  for (c = 0; c < n; c++) {                                               /* factor column c */
    int pr = c;
    double big = -1.0;
    for (r = c; r < n; r++) if (fabs(LU[r + c * n]) > big) { big = fabs(LU[r + c * n]); pr = r; }
    piv[c] = pr;
    if (LU[pr + c * n] == 0.0) SE2_FAIL("singular Vandermonde matrix (degree %d)", p);
    if (pr != c)
      for (k = 0; k < n; k++) { double t = LU[c + k * n]; LU[c + k * n] = LU[pr + k * n]; LU[pr + k * n] = t; }
    if (fabs(LU[c + c * n]) >= DBL_MIN) {
      const double inv = 1.0 / LU[c + c * n];
      for (r = c + 1; r < n; r++) LU[r + c * n] *= inv;
    } else {
      for (r = c + 1; r < n; r++) LU[r + c * n] = LU[r + c * n] / LU[c + c * n];
    }
    for (k = c + 1; k < n; k++) {
      const double m = -LU[c + k * n];
      for (r = c + 1; r < n; r++) LU[r + k * n] = LU[r + k * n] + LU[r + c * n] * m;
    }
  }
  for (k = 0; k < n; k++) {                                               /* solve V coef_k = e_k */
    for (r = 0; r < n; r++) rhs[r] = (r == k) ? 1.0 : 0.0;
    for (r = 0; r < n; r++) if (piv[r] != r) { double t = rhs[r]; rhs[r] = rhs[piv[r]]; rhs[piv[r]] = t; }
    for (c = 0; c < n; c++)
      if (rhs[c] != 0.0) for (r = c + 1; r < n; r++) rhs[r] = rhs[r] - rhs[c] * LU[r + c * n];
    for (c = n - 1; c >= 0; c--)
      if (rhs[c] != 0.0) {
        rhs[c] = rhs[c] / LU[c + c * n];
        for (r = 0; r < c; r++) rhs[r] = rhs[r] - rhs[c] * LU[r + c * n];
      }
    for (r = 0; r < n; r++) coef[k * n + r] = rhs[r];
  }
  return 0;
}

/* evaluate the basis (deriv = 0) or its derivative (deriv = 1) at points;
   entries below 1e-12 in magnitude are set to zero (se2wave.c:360-362, 494-496) */
static int basis_eval(int p, int npts, const double *x, int deriv, double *out)
{
  const int n = p + 1;
  double coef[17 * 17], mono[17];
  int k, b, j;
  if (p < 1 || p > 16) SE2_FAIL("polynomial degree %d out of range", p);
  if (lagrange_monomial_coefs(p, coef)) return -1;
  for (k = 0; k < npts; k++) {
    for (j = 0; j < n; j++) {
      if (!deriv) mono[j] = pow((double)x[k], (double)j);
      else mono[j] = (j == 0) ? 0.0 : ((double)j) * pow((double)x[k], (double)(j - 1));
    }
    for (b = 0; b < n; b++) {
      double s = 0.0;
      for (j = 0; j < n; j++) s += coef[b * n + j] * mono[j];
      out[k * n + b] = (fabs(s) < 1.0e-12) ? 0.0 : s;
    }
  }
  return 0;
}

int se2_basis_1d(int p, int npoints, const double *x, double *N) { return basis_eval(p, npoints, x, 0, N); }
int se2_basis_deriv_1d(int p, int npoints, const double *x, double *dN) { return basis_eval(p, npoints, x, 1, dN); }

/* ------------------------------------------------------------------ */
/* source-time functions                                               */
/* ------------------------------------------------------------------ */
/* Tinti et al. (2005) regularised Yoffe pieces C1, C3, C4 (se2wave.c:3608-3681) */
static int yoffe_piece(int which, double tS, double tR, double t, double *val)
{
  double a, b, c, d, e, tR2 = tR * tR, shift;
  if (which == 1) {
    a = 0.5 * t + 0.25 * tR;
    b = t * (tR - t);
    c = (t - tR) * tR;
    d = t / tR;
    e = (fabs(t) < 0.0) ? 1.0e12 : (tR - t) / t;
  } else if (which == 3) {
    a = tS - t - 0.5 * tR;
    b = (t - tS) * (tR - t + tS);
    c = tR * (2.0 * tR - 2.0 * t + 2.0 * tS);
    d = (t - tS) / tR;
    e = (fabs(t - tS) < 0.0) ? 1.0e12 : (tR - t + tS) / (t - tS);
  } else {
    shift = 2.0 * tS;
    a = -tS + 0.5 * t + 0.25 * tR;
    b = (t - shift) * (tR - t + shift);
    c = tR * (-tR + t - shift);
    d = (t - shift) / tR;
    e = (fabs(t - shift) < 0.0) ? 1.0e12 : (tR - t + shift) / (t - shift);
  }
  if (b < 0.0 || d < 0.0 || e < 0.0) SE2_FAIL("regularised Yoffe: negative argument in C%d at t=%g", which, t);
  if (which == 3) *val = a * sqrt(b) + c * asin(sqrt(d)) + 1.5 * tR2 * atan(sqrt(e));
  else *val = a * sqrt(b) + c * asin(sqrt(d)) - 0.75 * tR2 * atan(sqrt(e));
  return 0;
}

static int yoffe_eval(const double par[3], double t, double *value)
{
  const double tS = par[0], tR = par[1];
  const double K = 2.0 / (SE2_PI * tR * tS * tS);
  double C1 = 0.0, C2, C3 = 0.0, C4 = 0.0, C5, C6, tR2, phi;
  int mode;
  if (tR > 2.0 * tS) mode = 1;
  else if ((tS < tR) && (tR < 2.0 * tS)) mode = 2;
  else SE2_FAIL("Invalid values for tau_S (%+1.4e) and tau_R(%+1.4e) provided", tS, tR);
  if (t >= (tR + 2.0 * tS)) { *value = 0.0; return 0; }
  tR2 = tR * tR;
  C2 = (3.0 / 8.0) * SE2_PI * tR2;
  if ((t >= 0.0) && (t < tS)) {
    if (yoffe_piece(1, tS, tR, t, &C1)) return -1;
    phi = C1 + C2;
  } else if (mode == 1 && (t >= tS) && (t < 2.0 * tS)) {
    if (yoffe_piece(1, tS, tR, t, &C1) || yoffe_piece(3, tS, tR, t, &C3)) return -1;
    phi = C1 - C2 + C3;
  } else if (mode == 1 && (t >= 2.0 * tS) && (t < tR)) {
    if (yoffe_piece(1, tS, tR, t, &C1) || yoffe_piece(3, tS, tR, t, &C3) || yoffe_piece(4, tS, tR, t, &C4)) return -1;
    phi = C1 + C3 + C4;
  } else if (mode == 2 && (t >= tS) && (t < tR)) {
    if (yoffe_piece(1, tS, tR, t, &C1) || yoffe_piece(3, tS, tR, t, &C3)) return -1;
    phi = C1 - C2 + C3;
  } else if (mode == 2 && (t >= tR) && (t < 2.0 * tS)) {
    if (yoffe_piece(3, tS, tR, t, &C3)) return -1;
    C5 = 0.5 * SE2_PI * tR * (t - tR);
    phi = C5 + C3 - C2;
  } else if ((mode == 1 && (t >= tR) && (t < (tR + tS))) || (mode == 2 && (t >= 2.0 * tS) && (t < (tR + tS)))) {
    if (yoffe_piece(3, tS, tR, t, &C3) || yoffe_piece(4, tS, tR, t, &C4)) return -1;
    C5 = 0.5 * SE2_PI * tR * (t - tR);
    phi = C5 + C3 + C4;
  } else if ((t >= (tR + tS)) && (t < (tR + 2.0 * tS))) {
    if (yoffe_piece(4, tS, tR, t, &C4)) return -1;
    C6 = 0.5 * SE2_PI * tR * (2.0 * tS - t + tR);
    phi = C4 + C6;
  } else {
    phi = 0.0;
  }
  *value = K * phi;
  return 0;
}

int se2_stf_eval(int type, const double par[3], double t, double *value)
{
  switch (type) {
    case SE2_STF_RICKER: {  /* amp (1 - 2a^2) e^{-a^2}, a = pi f (t - t0)  (3504-3516) */
      const double arg = SE2_PI * par[1] * (t - par[0]);
      const double arg2 = arg * arg;
      *value = par[2] * (1.0 - 2.0 * arg2) * exp(-arg2);
      return 0;
    }
    case SE2_STF_GAUSSIAN: { /* amp exp(-omega^2 (t-t0)^2 / 2)  (3552-3561) */
      const double arg = par[1] * par[1] * (t - par[0]) * (t - par[0]) * 0.5;
      *value = par[2] * exp(-arg);
      return 0;
    }
    case SE2_STF_YOFFE:
      return yoffe_eval(par, t, value);
    default:
      SE2_FAIL("unknown source-time function type %d", type);
  }
}

int se2_stf_block(const se2_setup *s, double *time, long n, double *times, double *stf)
{
  long k;
  int src;
  double t = *time;
  for (k = 0; k < n; k++) {
    t = t + s->dt;
    if (times) times[k] = t;
    for (src = 0; src < s->nsrc; src++)
      if (se2_stf_eval(s->stf_type[src], &s->stf_par[3 * src], t, &stf[k * s->nsrc + src])) return -1;
  }
  *time = t;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Gaussian random field                                               */
/* ------------------------------------------------------------------ */
static uint64_t splitmix64(uint64_t *st)
{
  uint64_t z = (*st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* POSIX rand48 (drand48 after srand48): X' = (0x5DEECE66D X + 0xB) mod 2^48, value X' / 2^48 */
static uint64_t rand48_seeded(long seed) { return ((uint64_t)(uint32_t)seed << 16) | 0x330EULL; }
static double rand48_next(uint64_t *x)
{
  *x = (0x5DEECE66DULL * *x + 0xBULL) & 0xFFFFFFFFFFFFULL;
  return (double)*x * (1.0 / 281474976710656.0);
}

int se2_gaussian_random_field(int mx, int my, double mean, double rel_std, double corr, unsigned long long seed,
                              double *out)
{
  const long ne = (long)mx * my;
  const int R = (int)ceil(3.0 * corr);
  double *noise, *tmp, *ker, kn = 0.0;
  uint64_t st = (uint64_t)seed;
  long i;
  int x, y, d;
  if (mx < 1 || my < 1 || corr <= 0.0) SE2_FAIL("bad random-field size or correlation length");
  noise = (double*)xcalloc((size_t)ne, sizeof(double));
  tmp = (double*)xcalloc((size_t)ne, sizeof(double));
  ker = (double*)xcalloc((size_t)(2 * R + 1), sizeof(double));
  for (i = 0; i < ne; i += 2) {  /* Box-Muller on 53-bit uniforms in (0,1] */
    double u1 = ((double)(splitmix64(&st) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
    double u2 = ((double)(splitmix64(&st) >> 11)) * (1.0 / 9007199254740992.0);
    double r = sqrt(-2.0 * log(u1));
    noise[i] = r * cos(2.0 * SE2_PI * u2);
    if (i + 1 < ne) noise[i + 1] = r * sin(2.0 * SE2_PI * u2);
  }
  for (d = -R; d <= R; d++) { ker[d + R] = exp(-0.5 * (d / corr) * (d / corr)); kn += ker[d + R] * ker[d + R]; }
  for (y = 0; y < my; y++)
    for (x = 0; x < mx; x++) {
      double s = 0.0;
      for (d = -R; d <= R; d++) s += ker[d + R] * noise[(long)y * mx + (((x + d) % mx) + mx) % mx];
      tmp[(long)y * mx + x] = s;
    }
  for (y = 0; y < my; y++)
    for (x = 0; x < mx; x++) {
      double s = 0.0;
      for (d = -R; d <= R; d++) s += ker[d + R] * tmp[(long)((((y + d) % my) + my) % my) * mx + x];
      out[(long)y * mx + x] = s / kn;   /* unit variance: the 2-D kernel's squared norm is kn^2 */
    }
  for (i = 0; i < ne; i++) {
    double z = out[i];
    z = z > 3.0 ? 3.0 : (z < -3.0 ? -3.0 : z);
    out[i] = mean * (1.0 + rel_std * z);
  }
  free(noise); free(tmp); free(ker);
  return 0;
}

/* ------------------------------------------------------------------ */
/* shot draws: 2-layer + elliptical-inclusion materials, random source */
/* ------------------------------------------------------------------ */
static double unif(uint64_t *st, double a, double b)
{
  return a + (b - a) * ((double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0));
}

static double normal(uint64_t *st)
{
  const double u1 = ((double)(splitmix64(st) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  const double u2 = ((double)(splitmix64(st) >> 11)) * (1.0 / 9007199254740992.0);
  return sqrt(-2.0 * log(u1)) * cos(2.0 * SE2_PI * u2);
}

static void draw_rock(uint64_t *st, double vp_max, double *v)
{
  v[0] = unif(st, 3000.0, vp_max);          /* Vp */
  v[1] = v[0] / unif(st, 1.6, 1.9);         /* Vs from Vp/Vs */
  v[2] = unif(st, 2000.0, 3000.0);          /* rho */
}

int se2_shot_draw_params(unsigned long long seed, long index, int kind, se2_shot_draw *d)
{
  uint64_t st = (uint64_t)seed * 0x9E3779B97F4A7C15ULL ^ ((uint64_t)index + 0x632BE59BD9B4E019ULL) * 0xD1B54A32D192ED03ULL;
  const int degrees[3] = {3, 4, 6};
  int i;
  if (!d) SE2_FAIL("null output");
  if (kind < 0 || kind > 2) SE2_FAIL("unknown shot kind %d", kind);
  memset(d, 0, sizeof(*d));
  splitmix64(&st);
  if (kind == SE2_SHOT_ENSEMBLE) {
    d->mx = 32 + (int)(splitmix64(&st) % 481);   /* U{32..512} */
    d->my = 32 + (int)(splitmix64(&st) % 481);
    d->p = degrees[splitmix64(&st) % 3];
    d->nrec = 32;
    d->nsteps = 5000;
  } else {
    d->mx = d->my = 128;
    d->p = 4;
    d->nrec = 16;
    d->nsteps = 4096;
  }
  d->h = 31.25;                                  /* element size (m): 4 km / 128 */
  d->Lx = d->mx * d->h;
  d->Ly = d->my * d->h;
  {
    const double vp_max = (kind == SE2_SHOT_OOD) ? 7500.0 : 6000.0;
    d->interface_y = unif(&st, 0.3, 0.7) * d->Ly;
    draw_rock(&st, vp_max, d->lower);
    draw_rock(&st, vp_max, d->upper);
    d->ninc = (kind == SE2_SHOT_OOD) ? 2 : 1;
    for (i = 0; i < d->ninc; i++) {
      double *c = d->inc[i];
      const double L = d->Lx < d->Ly ? d->Lx : d->Ly;
      c[0] = unif(&st, 0.2, 0.8) * d->Lx;       /* centre */
      c[1] = unif(&st, 0.2, 0.8) * d->Ly;
      c[2] = unif(&st, 0.05, 0.2) * L;           /* semi-axes */
      c[3] = unif(&st, 0.05, 0.2) * L;
      c[4] = unif(&st, 0.0, SE2_PI);             /* rotation */
      draw_rock(&st, vp_max, c + 5);
    }
  }
  d->src_xy[0] = unif(&st, 0.1, 0.9) * d->Lx;
  d->src_xy[1] = (kind == SE2_SHOT_ENSEMBLE) ? unif(&st, 0.1, 0.9) * d->Ly : unif(&st, 0.1, 0.5) * d->Ly;
  d->moment[0] = 1.0e15 * normal(&st);           /* Mxx, Mxy, Myx, Myy: symmetric */
  d->moment[1] = 1.0e15 * normal(&st);
  d->moment[2] = d->moment[1];
  d->moment[3] = 1.0e15 * normal(&st);
  d->f0 = unif(&st, 5.0, 20.0);
  d->t0 = 1.5 / d->f0;
  return 0;
}

int se2_shot_materials(const se2_shot_draw *d, double *vp, double *vs, double *rho)
{
  int x, y, i;
  if (!d || !vp || !vs || !rho) SE2_FAIL("null argument");
  for (y = 0; y < d->my; y++)
    for (x = 0; x < d->mx; x++) {
      const double cx = (x + 0.5) * d->h, cy = (y + 0.5) * d->h;   /* cell centre */
      const double *v = (cy < d->interface_y) ? d->lower : d->upper;
      const long c = (long)y * d->mx + x;
      for (i = 0; i < d->ninc; i++) {                               /* a later inclusion wins */
        const double *e = d->inc[i];
        const double dx = cx - e[0], dy = cy - e[1], cs = cos(e[4]), sn = sin(e[4]);
        const double u = (cs * dx + sn * dy) / e[2], w = (-sn * dx + cs * dy) / e[3];
        if (u * u + w * w <= 1.0) v = e + 5;
      }
      vp[c] = v[0]; vs[c] = v[1]; rho[c] = v[2];
    }
  return 0;
}

/* ------------------------------------------------------------------ */
/* VTS snapshots (VTK XML StructuredGrid, raw appended Float64)        */
/* ------------------------------------------------------------------ */
int se2_write_vts(const se2_setup *s, const char *path, int nvec, const char *const *names, const double *const *vecs)
{
  FILE *f;
  const long nx = s ? s->nx_g : 0, ny = s ? s->ny_g : 0, n = nx * ny;
  unsigned long long off = 0, nbytes;
  long i, j;
  int v, c;
  if (!s || !path || nvec < 0 || (nvec > 0 && (!names || !vecs))) SE2_FAIL("bad VTS arguments");
  f = fopen(path, "wb");
  if (!f) SE2_FAIL("cannot open %s", path);
  fprintf(f, "<?xml version=\"1.0\"?>\n");
  fprintf(f, "<VTKFile type=\"StructuredGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n");
  fprintf(f, "  <StructuredGrid WholeExtent=\"0 %ld 0 %ld 0 0\">\n", nx - 1, ny - 1);
  fprintf(f, "    <Piece Extent=\"0 %ld 0 %ld 0 0\">\n", nx - 1, ny - 1);
  fprintf(f, "      <Points>\n");
  fprintf(f, "        <DataArray type=\"Float64\" Name=\"Position\" NumberOfComponents=\"3\" format=\"appended\" offset=\"%llu\" />\n", off);
  off += 8ULL + 24ULL * (unsigned long long)n;
  fprintf(f, "      </Points>\n");
  fprintf(f, "      <PointData>\n");
  for (v = 0; v < nvec; v++)
    for (c = 0; c < 2; c++) {
      fprintf(f, "        <DataArray type=\"Float64\" Name=\"%s%s\" NumberOfComponents=\"1\" format=\"appended\" offset=\"%llu\" />\n",
              names[v], c ? "_y" : "_x", off);
      off += 8ULL + 8ULL * (unsigned long long)n;
    }
  fprintf(f, "      </PointData>\n");
  fprintf(f, "    </Piece>\n");
  fprintf(f, "  </StructuredGrid>\n");
  fprintf(f, "  <AppendedData encoding=\"raw\">\n_");
  nbytes = 24ULL * (unsigned long long)n;
  fwrite(&nbytes, 8, 1, f);
  for (j = 0; j < ny; j++)
    for (i = 0; i < nx; i++) {
      const double p[3] = {s->xnode[i], s->ynode[j], 0.0};
      fwrite(p, 8, 3, f);
    }
  nbytes = 8ULL * (unsigned long long)n;
  for (v = 0; v < nvec; v++)
    for (c = 0; c < 2; c++) {
      fwrite(&nbytes, 8, 1, f);
      for (i = 0; i < n; i++) fwrite(&vecs[v][2 * i + c], 8, 1, f);
    }
  fprintf(f, "\n  </AppendedData>\n</VTKFile>\n");
  if (fclose(f) != 0) SE2_FAIL("write error on %s", path);
  return 0;
}

/* ------------------------------------------------------------------ */
/* set-up                                                              */
/* ------------------------------------------------------------------ */
void se2_setup_destroy(se2_setup *s)
{
  if (!s) return;
  free(s->xi); free(s->w1d); free(s->wq); free(s->D); free(s->xnode); free(s->ynode);
  free(s->J00); free(s->J11); free(s->iJ00); free(s->iJ11); free(s->lambda); free(s->mu); free(s->rho);
  free(s->mass); free(s->src_elem); free(s->src_gll); free(s->src_vals); free(s->stf_type); free(s->stf_par);
  free(s->src_owner);
  free(s->rec_xy); free(s->rec_node); free(s->rec_elem); free(s->rec_gll);
  free(s->interp_xy); free(s->interp_elem); free(s->interp_N); free(s->interp_xri);
  free(s);
}

/* node coordinate along one axis: the last element written to a shared node
   wins in SpecFECtxCreateMeshCoords2d_SEQ (757-775), then VecStrideScale and
   VecAXPY(coor, 1.0, shift) (795-813) */
static void axis_coords(int m, int p, const double *xi, double scale, double shift, double *out)
{
  const double h = 1.0 / ((double)m);
  int e, i;
  for (e = 0; e < m; e++) {
    const double x0 = 0.0 + e * h;
    for (i = 0; i <= p; i++) out[e * p + i] = 0.5 * (xi[i] + 1.0) * h + x0;
  }
  for (i = 0; i <= m * p; i++) {
    double x = out[i] * scale;
    out[i] = x + 1.0 * shift;
  }
}

static int locate_source(se2_setup *s, int k, const double c[2], const double M[4], int interior_only)
{
  const int p = s->p, n1 = s->n1, npe = s->npe;
  const double hx = (s->gmax[0] - s->gmin[0]) / ((double)s->mx);
  const double hy = (s->gmax[1] - s->gmin[1]) / ((double)s->my);
  const double x0 = s->xnode[0], y0 = s->ynode[0];
  double best = DBL_MAX, xq[2], dxi[17], Nxi[17], deta[17], Neta[17];
  int ei, ej, a, b, lo, hi, pick = -1;
  if (c[0] < s->gmin[0]) SE2_FAIL("Source x-coordinate (%+1.4e) < min(domain).x (%+1.4e)", c[0], s->gmin[0]);
  if (c[1] < s->gmin[1]) SE2_FAIL("Source y-coordinate (%+1.4e) < min(domain).y (%+1.4e)", c[1], s->gmin[1]);
  if (c[0] > s->gmax[0]) SE2_FAIL("Source x-coordinate (%+1.4e) > max(domain).x (%+1.4e)", c[0], s->gmax[0]);
  if (c[1] > s->gmax[1]) SE2_FAIL("Source y-coordinate (%+1.4e) > max(domain).y (%+1.4e)", c[1], s->gmax[1]);
  if (c[0] > s->xnode[s->nx_g - 1] || c[1] > s->ynode[s->ny_g - 1]) SE2_FAIL("A source was defined but no rank claimed it");
  ei = (int)((c[0] - x0) / hx);
  ej = (int)((c[1] - y0) / hy);
  if (ei == s->mx) ei--;
  if (ej == s->my) ej--;
  if (ei < 0 || ej < 0 || ei >= s->mx || ej >= s->my) SE2_FAIL("A source was defined but no rank claimed it");
  if (p == 1 && interior_only)
    SE2_FAIL("Cannot use basis degree = 1 and approximate the source location based on nearest cell interior GLL point. "
             "You must provide the command line option -use_nearest_internal_gll false");
  lo = interior_only ? 1 : 0;
  hi = interior_only ? n1 - 1 : n1;
  for (b = lo; b < hi; b++)
    for (a = lo; a < hi; a++) {
      const double dx = s->xnode[ei * p + a] - c[0], dy = s->ynode[ej * p + b] - c[1];
      const double d2 = dx * dx + dy * dy;
      if (d2 < best) { best = d2; pick = a + b * n1; }
    }
  if (pick < 0) SE2_FAIL("Failed to identify a closest quadrature point");
  s->src_elem[k] = ei + ej * s->mx;
  s->src_gll[k] = pick;
  /* derivative of the tensor basis at the snapped GLL point (TabulateBasisDerivativesAtPointTensorProduct2d,
     605-690) mapped to x,y with the element Jacobian (ElementEvaluateDerivatives_CellWiseConstant2d) */
  xq[0] = s->xi[pick % n1];
  xq[1] = s->xi[pick / n1];
  if (se2_basis_deriv_1d(p, 1, &xq[0], dxi) || se2_basis_1d(p, 1, &xq[0], Nxi) ||
      se2_basis_deriv_1d(p, 1, &xq[1], deta) || se2_basis_1d(p, 1, &xq[1], Neta)) return -1;
  for (b = 0; b < n1; b++)
    for (a = 0; a < n1; a++) {
      const int q = a + b * n1;
      const double gx = s->iJ00[ei] * (dxi[a] * Neta[b]);
      const double gy = s->iJ11[ej] * (Nxi[a] * deta[b]);
      s->src_vals[(size_t)k * 2 * npe + 2 * q] = (M[0] * gx + M[1] * gy);
      s->src_vals[(size_t)k * 2 * npe + 2 * q + 1] = (M[2] * gx + M[3] * gy);
    }
  return 0;
}

/* ---- alternative moment-source representations (ElastoDynamicsSourceSetup, 2232-2266):
   the assembled source vector g (2 * nnodes, interleaved) of one moment source */
static int source_cell(const se2_setup *s, const double xy[2], int *ii, int *jj, double *dx, double *dy)
{
  *dx = (s->gmax[0] - s->gmin[0]) / ((double)s->mx);
  *dy = (s->gmax[1] - s->gmin[1]) / ((double)s->my);
  *ii = (int)((xy[0] - s->gmin[0]) / *dx);
  *jj = (int)((xy[1] - s->gmin[1]) / *dy);
  if (*ii == s->mx) (*ii)--;
  if (*jj == s->my) (*jj)--;
  if (*ii < 0) SE2_FAIL("source: x < gmin[0]");
  if (*jj < 0) SE2_FAIL("source: y < gmin[1]");
  if (*ii >= s->mx || *jj >= s->my) SE2_FAIL("source outside the domain");
  return 0;
}

/* dN/dx, dN/dy (npe each) at reference point xi of element (ei, ej):
   TabulateBasisDerivativesAtPointTensorProduct2d + ElementEvaluateDerivatives_CellWiseConstant2d */
static int point_derivs(const se2_setup *s, int ei, int ej, const double xi[2], double *gx, double *gy)
{
  const int n1 = s->n1;
  double dxi[17], Nxi[17], deta[17], Neta[17];
  int a, b;
  if (se2_basis_deriv_1d(s->p, 1, &xi[0], dxi) || se2_basis_1d(s->p, 1, &xi[0], Nxi) ||
      se2_basis_deriv_1d(s->p, 1, &xi[1], deta) || se2_basis_1d(s->p, 1, &xi[1], Neta)) return -1;
  for (b = 0; b < n1; b++)
    for (a = 0; a < n1; a++) {
      gx[a + b * n1] = s->iJ00[ei] * (dxi[a] * Neta[b]);
      gy[a + b * n1] = s->iJ11[ej] * (Nxi[a] * deta[b]);
    }
  return 0;
}

int se2_source_vector(const se2_setup *s, int impl, double kernel_h, const double xy[2], const double M[4], double *g)
{
  const int p = s ? s->p : 0, n1 = s ? s->n1 : 0, npe = s ? s->npe : 0;
  double gx[289], gy[289], fe[578];
  int ii, jj, i, q, e;
  double dx, dy;
  if (!s || !xy || !M || !g) SE2_FAIL("null argument");
  memset(g, 0, sizeof(double) * 2 * (size_t)s->nnodes);
  if (impl == 0 || impl == 3) {
    /* 0: pointwise at the source's reference coordinates (1716-1923); 3: P0, the cell centre with
       the cell-averaged weight (2059-2200) */
    double xi[2], detJ;
    if (source_cell(s, xy, &ii, &jj, &dx, &dy)) return -1;
    if (impl == 0) {
      const double cmin0 = s->gmin[0] + ii * dx, cmin1 = s->gmin[1] + jj * dy;
      xi[0] = 2.0 * (xy[0] - cmin0) / dx - 1.0;
      xi[1] = 2.0 * (xy[1] - cmin1) / dy - 1.0;
      if (fabs(xi[0]) < 1.0e-12) xi[0] = 0.0;
      if (fabs(xi[1]) < 1.0e-12) xi[1] = 0.0;
    } else {
      xi[0] = 0.0;
      xi[1] = 0.0;
    }
    if (point_derivs(s, ii, jj, xi, gx, gy)) return -1;
    memset(fe, 0, sizeof(double) * 2 * npe);
    if (impl == 0) {
      for (i = 0; i < npe; i++) {
        fe[2 * i] += (M[0] * gx[i] + M[1] * gy[i]);
        fe[2 * i + 1] += (M[2] * gx[i] + M[3] * gy[i]);
      }
    } else {
      detJ = s->J00[ii] * s->J11[jj];
      for (q = 0; q < npe; q++)
        for (i = 0; i < npe; i++) {
          fe[2 * i] += s->wq[q] * detJ * (M[0] * gx[i] + M[1] * gy[i]) / (dx * dy);
          fe[2 * i + 1] += s->wq[q] * detJ * (M[2] * gx[i] + M[3] * gy[i]) / (dx * dy);
        }
    }
    for (i = 0; i < npe; i++) {
      const long node = (long)(ii * p + i % n1) + (long)(jj * p + i / n1) * s->nx_g;
      g[2 * node] += fe[2 * i];
      g[2 * node + 1] += fe[2 * i + 1];
    }
    return 0;
  }
  if (impl == 2) {
    /* cubic-spline smoothed Dirac over every element (1925-2057) */
    double ds, h;
    dx = (s->gmax[0] - s->gmin[0]) / ((double)s->mx);
    dy = (s->gmax[1] - s->gmin[1]) / ((double)s->my);
    ds = dx;
    if (dy > dx) ds = dy;
    if (kernel_h > 0.0) h = kernel_h;
    else if (p <= 3) h = 1.5 * (0.5 * ds);
    else h = (3.0 / (p - 2.0)) * (0.5 * ds);
    /* basis and derivative tables at the GLL points (TabulateBasisDerivativesTensorProduct2d, 525-603) */
    for (e = 0; e < s->mx * s->my; e++) {
      const int ei = e % s->mx, ej = e / s->mx;
      const double detJ = s->J00[ei] * s->J11[ej];
      memset(fe, 0, sizeof(double) * 2 * npe);
      for (q = 0; q < npe; q++) {
        const int qa = q % n1, qb = q / n1;
        const double xq0 = s->xnode[ei * p + qa], xq1 = s->ynode[ej * p + qb];
        double sep, arg, sd;
        /* dN/dx, dN/dy at GLL point q: the 1-D derivative matrix times exact Kronecker deltas
           (TabulateBasisDerivativesTensorProduct2d, 525-603), scaled by the inverse Jacobian */
        for (i = 0; i < npe; i++) {
          const int ia = i % n1, ib = i / n1;
          gx[i] = s->iJ00[ei] * (s->D[qa * n1 + ia] * ((qb == ib) ? 1.0 : 0.0));
          gy[i] = s->iJ11[ej] * (((qa == ia) ? 1.0 : 0.0) * s->D[qb * n1 + ib]);
        }
        sep = (xq0 - xy[0]) * (xq0 - xy[0]);
        sep += (xq1 - xy[1]) * (xq1 - xy[1]);
        arg = sqrt(sep) / h;
        if (arg < 1.0) sd = 0.25 * (2.0 - arg) * (2.0 - arg) * (2.0 - arg) - (1.0 - arg) * (1.0 - arg) * (1.0 - arg);
        else if (arg < 2.0) sd = 0.25 * (2.0 - arg) * (2.0 - arg) * (2.0 - arg);
        else sd = 0.0;
        sd = 10.0 / (7.0 * SE2_PI) * sd * (1.0 / (h * h));
        for (i = 0; i < npe; i++) {
          fe[2 * i] += s->wq[q] * detJ * (M[0] * gx[i] + M[1] * gy[i]) * sd;
          fe[2 * i + 1] += s->wq[q] * detJ * (M[2] * gx[i] + M[3] * gy[i]) * sd;
        }
      }
      for (i = 0; i < npe; i++) {
        const long node = (long)(ei * p + i % n1) + (long)(ej * p + i / n1) * s->nx_g;
        g[2 * node] += fe[2 * i];
        g[2 * node + 1] += fe[2 * i + 1];
      }
    }
    return 0;
  }
  SE2_FAIL("source implementation %d: use 0 (pointwise), 2 (cubic-spline kernel) or 3 (P0)", impl);
}

static int locate_receiver(se2_setup *s, int r)
{
  const double xr = s->rec_xy[2 * r], yr = s->rec_xy[2 * r + 1];
  const double hx = (s->gmax[0] - s->gmin[0]) / ((double)s->mx);
  const double hy = (s->gmax[1] - s->gmin[1]) / ((double)s->my);
  double best = 1.0e32;
  int ei, ej, a, b, pick = -1;
  if (xr < s->gmin[0]) SE2_FAIL("Receiver %d, x-coordinate (%+1.4e) < min(domain).x (%+1.4e)", r, xr, s->gmin[0]);
  if (yr < s->gmin[1]) SE2_FAIL("Receiver %d, y-coordinate (%+1.4e) < min(domain).y (%+1.4e)", r, yr, s->gmin[1]);
  if (xr > s->gmax[0]) SE2_FAIL("Receiver %d, x-coordinate (%+1.4e) > max(domain).x (%+1.4e)", r, xr, s->gmax[0]);
  if (yr > s->gmax[1]) SE2_FAIL("Receiver %d, y-coordinate (%+1.4e) > max(domain).y (%+1.4e)", r, yr, s->gmax[1]);
  if (xr > s->xnode[s->nx_g - 1] || yr > s->ynode[s->ny_g - 1]) SE2_FAIL("A receiver was defined but no rank claimed it");
  ei = (int)((xr - s->xnode[0]) / hx);
  if (ei == s->mx) ei--;
  ej = (int)((yr - s->ynode[0]) / hy);
  if (ej == s->my) ej--;
  if (ei < 0 || ej < 0 || ei >= s->mx || ej >= s->my) SE2_FAIL("A receiver was defined but no rank claimed it");
  for (b = 0; b < s->n1; b++)
    for (a = 0; a < s->n1; a++) {
      const double dx = xr - s->xnode[ei * s->p + a], dy = yr - s->ynode[ej * s->p + b];
      double d2 = dx * dx;
      d2 += dy * dy;
      if (d2 < best) { best = d2; pick = a + b * s->n1; }
    }
  s->rec_elem[r] = ei + ej * s->mx;
  s->rec_gll[r] = pick;
  s->rec_node[r] = (ei * s->p + pick % s->n1) + (ej * s->p + pick / s->n1) * s->nx_g;
  return 0;
}

int se2_interp_receiver(const se2_setup *s, const double xy[2], int *eid, double *N, double xri[2])
{
  double gmin[2], gmax[2], dx, dy, x0, y0, xi, eta, Ns1[17], Ns2[17], xr0 = 0.0, xr1 = 0.0;
  int ei, ej, i, j, k;
  if (!s || !xy || !eid || !N || !xri) SE2_FAIL("null argument");
  gmin[0] = s->gmin[0]; gmin[1] = s->gmin[1]; gmax[0] = s->gmax[0]; gmax[1] = s->gmax[1];
  if (!(xy[0] >= gmin[0] && xy[0] < gmax[0] && xy[1] >= gmin[1] && xy[1] < gmax[1]))
    SE2_FAIL("interpolating receiver (%+1.8e, %+1.8e) outside [gmin, gmax) of the mesh", xy[0], xy[1]);
  dx = (gmax[0] - gmin[0]) / ((double)s->mx);
  ei = (int)((xy[0] - gmin[0]) / dx);
  dy = (gmax[1] - gmin[1]) / ((double)s->my);
  ej = (int)((xy[1] - gmin[1]) / dy);
  if (ei < 0 || ej < 0 || ei >= s->mx || ej >= s->my)
    SE2_FAIL("interpolating receiver (%+1.8e, %+1.8e): element (%d, %d) outside the mesh", xy[0], xy[1], ei, ej);
  x0 = gmin[0] + ei * dx;
  y0 = gmin[1] + ej * dy;
  xi = 2.0 * (xy[0] - x0) / dx - 1.0;
  eta = 2.0 * (xy[1] - y0) / dy - 1.0;
  if (se2_basis_1d(s->p, 1, &xi, Ns1) || se2_basis_1d(s->p, 1, &eta, Ns2)) return -1;
  k = 0;
  for (j = 0; j < s->n1; j++)
    for (i = 0; i < s->n1; i++) { N[k] = Ns1[i] * Ns2[j]; k++; }
  for (k = 0; k < s->npe; k++) {
    const int gi = ei * s->p + k % s->n1, gj = ej * s->p + k / s->n1;
    xr0 += N[k] * s->xnode[gi];
    xr1 += N[k] * s->ynode[gj];
  }
  *eid = ei + ej * s->mx;
  xri[0] = xr0; xri[1] = xr1;
  return 0;
}

int se2_interp_rows(const se2_setup *s, long nrows, const double *rows, double *out)
{
  long j;
  int i, k, c;
  if (!s || nrows < 0 || (nrows > 0 && s->ninterp > 0 && (!rows || !out))) SE2_FAIL("null argument");
  for (j = 0; j < nrows; j++)
    for (i = 0; i < s->ninterp; i++) {
      const double *Ni = s->interp_N + (size_t)i * s->npe;
      for (c = 0; c < 7; c++) {
        double v = 0.0;
        for (k = 0; k < s->npe; k++) v += Ni[k] * rows[(size_t)j * 7 * s->nrec + 7 * ((size_t)s->nrec_sta + (size_t)i * s->npe + k) + c];
        out[(size_t)j * 7 * s->ninterp + 7 * i + c] = v;
      }
    }
  return 0;
}

int se2_setup_create(const se2_spec *sp, se2_setup **out)
{
  se2_setup *s;
  int i, j, ex, ey;
  long e;
  *out = NULL;
  if (!sp) SE2_FAIL("null spec");
  if (sp->p < 1 || sp->p > 8) SE2_FAIL("-bdegree must be in 1..8 (got %d)", sp->p);
  if (sp->mx < 1 || sp->my < 1) SE2_FAIL("-mx and -my must be positive (got %d, %d)", sp->mx, sp->my);
  if ((long)(sp->p * (long)sp->mx + 1) * (long)(sp->p * (long)sp->my + 1) * 2 >= 2147483647L)
    SE2_FAIL("mesh too large for 32-bit degree-of-freedom indices");
  if (sp->nsrc < 0 || sp->nrec < 0) SE2_FAIL("negative source or receiver count");
  s = (se2_setup*)xcalloc(1, sizeof(se2_setup));
  s->mx = sp->mx; s->my = sp->my; s->p = sp->p;
  s->n1 = sp->p + 1;
  s->npe = s->n1 * s->n1;
  s->nx_g = sp->p * sp->mx + 1;
  s->ny_g = sp->p * sp->my + 1;
  s->nnodes = (long)s->nx_g * s->ny_g;
  s->xi = (double*)xcalloc((size_t)s->n1, sizeof(double));
  s->w1d = (double*)xcalloc((size_t)s->n1, sizeof(double));
  s->wq = (double*)xcalloc((size_t)s->npe, sizeof(double));
  s->D = (double*)xcalloc((size_t)s->npe, sizeof(double));
  if (se2_gll(sp->p, s->xi, s->w1d) || se2_basis_deriv_1d(sp->p, s->n1, s->xi, s->D)) { se2_setup_destroy(s); return -1; }
  for (j = 0; j < s->n1; j++) for (i = 0; i < s->n1; i++) s->wq[i + j * s->n1] = s->w1d[i] * s->w1d[j];

  /* geometry */
  s->xnode = (double*)xcalloc((size_t)s->nx_g, sizeof(double));
  s->ynode = (double*)xcalloc((size_t)s->ny_g, sizeof(double));
  axis_coords(s->mx, s->p, s->xi, sp->scale[0], sp->shift[0], s->xnode);
  axis_coords(s->my, s->p, s->xi, sp->scale[1], sp->shift[1], s->ynode);
  s->gmin[0] = s->gmin[1] = DBL_MAX;
  s->gmax[0] = s->gmax[1] = -DBL_MAX;
  for (i = 0; i < s->nx_g; i++) { if (s->xnode[i] < s->gmin[0]) s->gmin[0] = s->xnode[i]; if (s->gmax[0] < s->xnode[i]) s->gmax[0] = s->xnode[i]; }
  for (i = 0; i < s->ny_g; i++) { if (s->ynode[i] < s->gmin[1]) s->gmin[1] = s->ynode[i]; if (s->gmax[1] < s->ynode[i]) s->gmax[1] = s->ynode[i]; }
  s->J00 = (double*)xcalloc((size_t)s->mx, sizeof(double));
  s->iJ00 = (double*)xcalloc((size_t)s->mx, sizeof(double));
  s->J11 = (double*)xcalloc((size_t)s->my, sizeof(double));
  s->iJ11 = (double*)xcalloc((size_t)s->my, sizeof(double));
  for (ex = 0; ex < s->mx; ex++) { s->J00[ex] = 0.5 * (s->xnode[ex * s->p + s->p] - s->xnode[ex * s->p]); s->iJ00[ex] = 1.0 / s->J00[ex]; }
  for (ey = 0; ey < s->my; ey++) { s->J11[ey] = 0.5 * (s->ynode[ey * s->p + s->p] - s->ynode[ey * s->p]); s->iJ11[ey] = 1.0 / s->J11[ey]; }

  /* materials */
  s->lambda = (double*)xcalloc((size_t)sp->mx * sp->my, sizeof(double));
  s->mu = (double*)xcalloc((size_t)sp->mx * sp->my, sizeof(double));
  s->rho = (double*)xcalloc((size_t)sp->mx * sp->my, sizeof(double));
  if (!sp->cell_vp && sp->perturb) {
    /* se2wave.c:1177-1236: three PETSc RAND48 streams (seeds 1, 2, 3), width * drand48() + low */
    const long ne = (long)sp->mx * sp->my;
    const double x0[3] = {sp->vp, sp->vs, sp->rho}, dx[3] = {sp->dvp, sp->dvs, sp->drho};
    double *pv = (double*)xcalloc((size_t)ne, sizeof(double) * 3);
    int f;
    for (f = 0; f < 3; f++) {
      const double lo = x0[f] - dx[f], width = (x0[f] + dx[f]) - lo;
      uint64_t st = rand48_seeded((long)(f + 1));
      for (e = 0; e < ne; e++) pv[f * ne + e] = width * rand48_next(&st) + lo;
    }
    for (e = 0; e < ne; e++) {
      const double vp = pv[e], vs = pv[ne + e], rho = pv[2 * ne + e];
      if (!(rho > 0.0) || !(vs >= 0.0) || !(vp > 0.0)) { free(pv); se2_setup_destroy(s); SE2_FAIL("cell %ld: non-physical material", e); }
      s->mu[e] = vs * vs * rho;
      s->lambda[e] = vp * vp * rho - 2.0 * s->mu[e];
      s->rho[e] = rho;
    }
    free(pv);
  } else
  for (e = 0; e < (long)sp->mx * sp->my; e++) {
    const double vp = sp->cell_vp ? sp->cell_vp[e] : sp->vp;
    const double vs = sp->cell_vs ? sp->cell_vs[e] : sp->vs;
    const double rho = sp->cell_rho ? sp->cell_rho[e] : sp->rho;
    if (!(rho > 0.0) || !(vs >= 0.0) || !(vp > 0.0)) { se2_setup_destroy(s); SE2_FAIL("cell %ld: non-physical material", e); }
    s->mu[e] = vs * vs * rho;
    s->lambda[e] = vp * vp * rho - 2.0 * s->mu[e];
    s->rho[e] = rho;
  }

  /* lumped mass: element contributions added to each node in ascending element order */
  s->mass = (double*)xcalloc((size_t)s->nnodes, sizeof(double));
  for (ey = 0; ey < s->my; ey++)
    for (ex = 0; ex < s->mx; ex++) {
      const long ec = (long)ex + (long)ey * s->mx;
      const double detJ = s->J00[ex] * s->J11[ey];
      for (j = 0; j < s->n1; j++)
        for (i = 0; i < s->n1; i++) {
          const double fac = detJ * s->wq[i + j * s->n1];
          s->mass[(long)(ex * s->p + i) + (long)(ey * s->p + j) * s->nx_g] += fac * (s->rho[ec]);
        }
    }

  /* sources */
  s->nsrc_phys = sp->nsrc;
  if (sp->src_impl < 0) {
    /* SeismicSourceCreate, SOURCE_IMPL_NEAREST_QPOINT (2995-3243): one entry per source */
    s->nsrc = sp->nsrc;
    s->src_elem = (int*)xcalloc((size_t)sp->nsrc, sizeof(int));
    s->src_gll = (int*)xcalloc((size_t)sp->nsrc, sizeof(int));
    s->src_owner = (int*)xcalloc((size_t)sp->nsrc, sizeof(int));
    s->src_vals = (double*)xcalloc((size_t)sp->nsrc * 2 * s->npe, sizeof(double));
    s->stf_type = (int*)xcalloc((size_t)sp->nsrc, sizeof(int));
    s->stf_par = (double*)xcalloc((size_t)sp->nsrc * 3, sizeof(double));
    for (i = 0; i < sp->nsrc; i++) {
      double dummy;
      if (locate_source(s, i, &sp->src_xy[2 * i], &sp->src_m[4 * i], sp->nearest_internal_gll)) { se2_setup_destroy(s); return -1; }
      s->src_owner[i] = (int)i;
      s->stf_type[i] = sp->stf_type[i];
      memcpy(&s->stf_par[3 * i], &sp->stf_par[3 * i], 3 * sizeof(double));
      if (se2_stf_eval(s->stf_type[i], &s->stf_par[3 * i], 1.0e30, &dummy)) { se2_setup_destroy(s); return -1; }
    }
  } else {
    /* assembled source vectors (ElastoDynamicsSourceSetup, 2232-2266) split into per-element
       entries: every node with a non-zero value belongs to the first element (ascending) that
       holds it, so the entries add up to the vector exactly; each entry carries its source's STF */
    const long nn = s->nnodes;
    double *g = (double*)xcalloc((size_t)nn * 2, sizeof(double));
    char *taken = (char*)xcalloc((size_t)nn, 1);
    long cap = 0, ne = 0, e;
    s->nsrc = 0;
    for (i = 0; i < sp->nsrc; i++) {
      double dummy;
      if (se2_source_vector(s, sp->src_impl, sp->sm_h, &sp->src_xy[2 * i], &sp->src_m[4 * i], g) ||
          se2_stf_eval(sp->stf_type[i], &sp->stf_par[3 * i], 1.0e30, &dummy)) {
        free(g); free(taken); se2_setup_destroy(s); return -1;
      }
      memset(taken, 0, (size_t)nn);
      /* candidate elements: those holding a non-zero node */
      {
        long *cand = NULL, nc = 0, cc = 0;
        for (e = 0; e < (long)s->mx * s->my; e++) {
          const int ei = (int)(e % s->mx), ej = (int)(e / s->mx);
          int a, b, any = 0;
          for (b = 0; b < s->n1 && !any; b++)
            for (a = 0; a < s->n1; a++) {
              const long node = (long)(ei * s->p + a) + (long)(ej * s->p + b) * s->nx_g;
              if (g[2 * node] != 0.0 || g[2 * node + 1] != 0.0) { any = 1; break; }
            }
          if (!any) continue;
          if (nc == cc) { cc = cc ? 2 * cc : 16; cand = (long*)realloc(cand, sizeof(long) * (size_t)cc); }
          cand[nc++] = e;
        }
        /* greedy cover: the element with the most unassigned non-zero nodes first (lowest index on ties) */
        for (;;) {
          long best = -1, k;
          int bestn = 0;
          for (k = 0; k < nc; k++) {
            const int ei = (int)(cand[k] % s->mx), ej = (int)(cand[k] / s->mx);
            int a, b, cnt = 0;
            for (b = 0; b < s->n1; b++)
              for (a = 0; a < s->n1; a++) {
                const long node = (long)(ei * s->p + a) + (long)(ej * s->p + b) * s->nx_g;
                if (!taken[node] && (g[2 * node] != 0.0 || g[2 * node + 1] != 0.0)) cnt++;
              }
            if (cnt > bestn) { bestn = cnt; best = cand[k]; }
          }
          if (best < 0) break;
          e = best;
          {
            const int ei = (int)(e % s->mx), ej = (int)(e / s->mx);
            int a, b;
            if (ne == cap) {
              cap = cap ? 2 * cap : 16;
              s->src_elem = (int*)realloc(s->src_elem, sizeof(int) * (size_t)cap);
              s->src_gll = (int*)realloc(s->src_gll, sizeof(int) * (size_t)cap);
              s->src_owner = (int*)realloc(s->src_owner, sizeof(int) * (size_t)cap);
              s->src_vals = (double*)realloc(s->src_vals, sizeof(double) * 2 * (size_t)s->npe * (size_t)cap);
              s->stf_type = (int*)realloc(s->stf_type, sizeof(int) * (size_t)cap);
              s->stf_par = (double*)realloc(s->stf_par, sizeof(double) * 3 * (size_t)cap);
            }
            s->src_elem[ne] = (int)e;
            s->src_gll[ne] = -1;
            s->src_owner[ne] = (int)i;
            s->stf_type[ne] = sp->stf_type[i];
            memcpy(&s->stf_par[3 * ne], &sp->stf_par[3 * i], 3 * sizeof(double));
            for (b = 0; b < s->n1; b++)
              for (a = 0; a < s->n1; a++) {
                const long node = (long)(ei * s->p + a) + (long)(ej * s->p + b) * s->nx_g;
                double *v = &s->src_vals[(size_t)ne * 2 * s->npe + 2 * (a + b * s->n1)];
                if (!taken[node]) { v[0] = g[2 * node]; v[1] = g[2 * node + 1]; taken[node] = 1; }
                else { v[0] = 0.0; v[1] = 0.0; }
              }
            ne++;
          }
        }
        free(cand);
      }
    }
    s->nsrc = (int)ne;
    free(g); free(taken);
  }

  /* receivers: the nearest-GLL stations, then the element nodes of each interpolating receiver */
  if (sp->ninterp < 0 || (sp->ninterp > 0 && !sp->interp_xy)) { se2_setup_destroy(s); SE2_FAIL("bad interpolating receiver list"); }
  s->nrec_sta = sp->nrec;
  s->ninterp = sp->ninterp;
  s->nrec = sp->nrec + sp->ninterp * s->npe;
  s->rec_xy = (double*)xcalloc((size_t)s->nrec * 2, sizeof(double));
  s->rec_node = (int*)xcalloc((size_t)s->nrec, sizeof(int));
  s->rec_elem = (int*)xcalloc((size_t)s->nrec, sizeof(int));
  s->rec_gll = (int*)xcalloc((size_t)s->nrec, sizeof(int));
  s->interp_xy = (double*)xcalloc((size_t)sp->ninterp * 2, sizeof(double));
  s->interp_elem = (int*)xcalloc((size_t)sp->ninterp, sizeof(int));
  s->interp_N = (double*)xcalloc((size_t)sp->ninterp * s->npe, sizeof(double));
  s->interp_xri = (double*)xcalloc((size_t)sp->ninterp * 2, sizeof(double));
  if (sp->nrec) memcpy(s->rec_xy, sp->rec_xy, sizeof(double) * 2 * sp->nrec);
  for (i = 0; i < sp->nrec; i++) if (locate_receiver(s, i)) { se2_setup_destroy(s); return -1; }
  for (i = 0; i < sp->ninterp; i++) {
    int k, eid;
    s->interp_xy[2 * i] = sp->interp_xy[2 * i]; s->interp_xy[2 * i + 1] = sp->interp_xy[2 * i + 1];
    if (se2_interp_receiver(s, &s->interp_xy[2 * i], &eid, &s->interp_N[(size_t)i * s->npe], &s->interp_xri[2 * i])) {
      se2_setup_destroy(s);
      return -1;
    }
    s->interp_elem[i] = eid;
    for (k = 0; k < s->npe; k++) {
      const int r = sp->nrec + i * s->npe + k;
      const int gi = (eid % s->mx) * s->p + k % s->n1, gj = (eid / s->mx) * s->p + k / s->n1;
      s->rec_elem[r] = eid;
      s->rec_gll[r] = k;
      s->rec_node[r] = gi + gj * s->nx_g;
      s->rec_xy[2 * r] = s->xnode[gi];
      s->rec_xy[2 * r + 1] = s->ynode[gj];
    }
  }

  /* CFL time step: smallest element size times half the smallest GLL gap, over the largest Vp */
  {
    const double hx = (s->gmax[0] - s->gmin[0]) / ((double)s->mx);
    const double hy = (s->gmax[1] - s->gmin[1]) / ((double)s->my);
    double r = hx, gap = 1.0e32, dtmin = DBL_MAX;
    r = (r < hy) ? r : hy;
    for (i = 0; i < s->n1 - 1; i++) { double g = fabs(s->xi[i + 1] - s->xi[i]); if (g < gap) gap = g; }
    r = r * (gap / 2.0);
    for (e = 0; e < (long)s->mx * s->my; e++) {
      const double vpe = sqrt((s->lambda[e] + 2.0 * s->mu[e]) / s->rho[e]);
      const double val = 1.0 * 1.0 * r / vpe;
      dtmin = (dtmin < val) ? dtmin : val;
    }
    s->dt_cfl = dtmin;
  }
  s->dt = s->dt_cfl * sp->cfl;
  if (sp->dt > 0.0) s->dt = sp->dt;
  if (!(s->dt > 0.0)) { se2_setup_destroy(s); SE2_FAIL("non-positive time step"); }
  s->tmax = sp->tmax;
  {
    /* (PetscInt)(tmax/dt) + 4 (se2wave.c:4714); saturate instead of overflowing for huge tmax */
    const double q = s->tmax / s->dt;
    s->nt = (q < 2147483000.0) ? (long)(int)q + 4 : 2147483647L;
  }
  if (sp->nt >= 0) s->nt = sp->nt;
  {
    long k;
    double t = 0.0;
    s->nsteps = 0;
    for (k = 1; k <= s->nt; k++) { t = t + s->dt; s->nsteps = k; if (t >= s->tmax) break; }
  }
  *out = s;
  return 0;
}
