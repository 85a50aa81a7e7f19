// se2gpu_api.cu -- C-ABI of libse2gpu.so (see include/se2gpu.h).
//
// Owns the device memory of one problem: two buffer sets of the fields (the
// step kernel reads one and writes the other), the per-cell and per-axis
// tables, sources, receivers and the device trace buffer.  Every entry point
// validates its arguments on the host and returns a status code; CUDA errors
// are caught after each launch and reported through se2gpu_last_error.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "se2gpu.h"
#include "se2gpu_launch.h"

struct se2gpu_solver {
  int mx, my, p, n1, npe, nx_g, ny_g, precision;
  long nnodes;
  int nsrc, nrec, trace_cap, rows_written;
  bool pending_record;
  double dt;
  int device;
  cudaStream_t stream, own_stream;
  size_t tsize;                  // bytes per scalar (4 or 8)
  void *fields[2][5];            // [buffer][u v a cu cv]
  int cur;
  void *mass, *lam, *mu, *J00, *J11, *iJ00, *iJ11, *D, *wq, *src_vals;
  double *Dd, *iJ00d, *iJ11d, *stf_dev, *traces, *norm_part;
  int stf_cap;
  int *src_elem, *rec_node, *rec_elem, *rec_gll;
  void *scratch_u, *scratch_f;   // assemble_linear_form staging
  long launches;
  int ntx, nty, nblocks;
  char err[512];
};

static thread_local char g_create_err[512];

extern "C" const char *se2gpu_create_error(void) { return g_create_err; }
extern "C" const char *se2gpu_last_error(const se2gpu_solver *h) { return h ? h->err : g_create_err; }

static int fail(se2gpu_solver *h, int code, const char *fmt, ...)
{
  char *buf = h ? h->err : g_create_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, 512, fmt, ap);
  va_end(ap);
  return code;
}

#define CK(h, call)                                                                                     \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) return fail((h), SE2GPU_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                             \
  } while (0)

static int dalloc(se2gpu_solver *h, void **p, size_t bytes)
{
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(h, SE2GPU_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  return 0;
}

// upload an FP64 host array in the handle's compute precision
static int upload(se2gpu_solver *h, void **dst, const double *src, size_t n)
{
  int rc = dalloc(h, dst, n * h->tsize);
  if (rc) return rc;
  if (h->tsize == 8) {
    CK(h, cudaMemcpy(*dst, src, n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (float)src[i];
    CK(h, cudaMemcpy(*dst, tmp.data(), n * 4, cudaMemcpyHostToDevice));
  }
  return 0;
}

static int upload_d(se2gpu_solver *h, double **dst, const double *src, size_t n)
{
  int rc = dalloc(h, (void **)dst, n * 8);
  if (rc) return rc;
  CK(h, cudaMemcpy(*dst, src, n * 8, cudaMemcpyHostToDevice));
  return 0;
}

static int upload_i(se2gpu_solver *h, int **dst, const int *src, size_t n)
{
  int rc = dalloc(h, (void **)dst, n * 4);
  if (rc) return rc;
  if (n) CK(h, cudaMemcpy(*dst, src, n * 4, cudaMemcpyHostToDevice));
  return 0;
}

extern "C" void se2gpu_destroy(se2gpu_solver *h)
{
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int b = 0; b < 2; b++)
    for (int f = 0; f < 5; f++) cudaFree(h->fields[b][f]);
  void *ptrs[] = {h->mass, h->lam, h->mu, h->J00, h->J11, h->iJ00, h->iJ11, h->D, h->wq, h->src_vals,
                  h->Dd, h->iJ00d, h->iJ11d, h->stf_dev, h->traces, h->norm_part, h->src_elem, h->rec_node,
                  h->rec_elem, h->rec_gll, h->scratch_u, h->scratch_f};
  for (void *p : ptrs) cudaFree(p);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  free(h);
}

extern "C" int se2gpu_create(const se2gpu_problem *P, int precision, int trace_capacity, se2gpu_solver **out)
{
  if (!out) return fail(nullptr, SE2GPU_ERR_ARG, "null output handle");
  *out = nullptr;
  if (!P) return fail(nullptr, SE2GPU_ERR_ARG, "null problem");
  if (precision != SE2GPU_FP64 && precision != SE2GPU_FP32 && precision != SE2GPU_FP32_KAHAN)
    return fail(nullptr, SE2GPU_ERR_ARG, "unknown precision %d (use 64, 33 or 32)", precision);
  if (P->p < 1 || P->p > 8) return fail(nullptr, SE2GPU_ERR_ARG, "polynomial degree %d outside 1..8", P->p);
  if (P->mx < 1 || P->my < 1) return fail(nullptr, SE2GPU_ERR_ARG, "mx, my must be positive");
  const long nx_g = (long)P->p * P->mx + 1, ny_g = (long)P->p * P->my + 1;
  if (nx_g * ny_g * 2 >= 2147483647L) return fail(nullptr, SE2GPU_ERR_ARG, "mesh too large for 32-bit node indices");
  if (!(P->dt > 0.0) || !std::isfinite(P->dt)) return fail(nullptr, SE2GPU_ERR_ARG, "time step must be positive and finite");
  if (P->nsrc < 0 || P->nrec < 0 || trace_capacity < 0) return fail(nullptr, SE2GPU_ERR_ARG, "negative count");
  if (!P->D || !P->wq || !P->J00 || !P->J11 || !P->iJ00 || !P->iJ11 || !P->lambda || !P->mu || !P->mass)
    return fail(nullptr, SE2GPU_ERR_ARG, "missing problem table");
  if (P->nsrc && (!P->src_elem || !P->src_vals)) return fail(nullptr, SE2GPU_ERR_ARG, "missing source arrays");
  if (P->nrec && (!P->rec_node || !P->rec_elem || !P->rec_gll)) return fail(nullptr, SE2GPU_ERR_ARG, "missing receiver arrays");
  const int n1 = P->p + 1, npe = n1 * n1;
  const long ne = (long)P->mx * P->my, nnodes = nx_g * ny_g;
  for (int s = 0; s < P->nsrc; s++)
    if (P->src_elem[s] < 0 || P->src_elem[s] >= ne) return fail(nullptr, SE2GPU_ERR_ARG, "source %d: element %d out of range", s, P->src_elem[s]);
  for (int r = 0; r < P->nrec; r++) {
    const int e = P->rec_elem[r], g = P->rec_gll[r];
    if (e < 0 || e >= ne || g < 0 || g >= npe) return fail(nullptr, SE2GPU_ERR_ARG, "receiver %d: element/GLL index out of range", r);
    const long node = ((long)(e % P->mx) * P->p + g % n1) + ((long)(e / P->mx) * P->p + g / n1) * nx_g;
    if (node != P->rec_node[r]) return fail(nullptr, SE2GPU_ERR_ARG, "receiver %d: node %d is not GLL point %d of element %d", r, P->rec_node[r], g, e);
  }
  for (long i = 0; i < nnodes; i++)
    if (!(P->mass[i] > 0.0) || !std::isfinite(P->mass[i])) return fail(nullptr, SE2GPU_ERR_ARG, "mass at node %ld is not positive", i);

  se2gpu_solver *h = (se2gpu_solver *)calloc(1, sizeof(se2gpu_solver));
  h->mx = P->mx; h->my = P->my; h->p = P->p; h->n1 = n1; h->npe = npe;
  h->nx_g = (int)nx_g; h->ny_g = (int)ny_g; h->nnodes = nnodes;
  h->precision = precision; h->nsrc = P->nsrc; h->nrec = P->nrec; h->trace_cap = trace_capacity;
  h->dt = P->dt;
  h->tsize = (precision == SE2GPU_FP64) ? 8 : 4;
  const int te = se2::tile_edge(P->p);
  h->ntx = (P->mx + te - 1) / te;
  h->nty = (P->my + te - 1) / te;
  h->nblocks = h->ntx * h->nty + 1;
  int rc;
#define TRY(x) do { if ((rc = (x)) != 0) { snprintf(g_create_err, sizeof(g_create_err), "%s", h->err); se2gpu_destroy(h); return rc; } } while (0)
  if (cudaGetDevice(&h->device) != cudaSuccess) { cudaGetLastError(); free(h); return fail(nullptr, SE2GPU_ERR_CUDA, "no CUDA device"); }
  {
    cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { free(h); return fail(nullptr, SE2GPU_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
    h->stream = h->own_stream;
  }
  {
    cudaError_t e = (precision == SE2GPU_FP64) ? se2::prepare_f64(P->p) : se2::prepare_f32(P->p, precision == SE2GPU_FP32_KAHAN);
    if (e != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "kernel set-up: %s", cudaGetErrorString(e)); TRY(SE2GPU_ERR_CUDA); }
  }
  const size_t vbytes = (size_t)nnodes * 2 * h->tsize;
  const int nf = (precision == SE2GPU_FP32_KAHAN) ? 5 : 3;
  for (int b = 0; b < 2; b++)
    for (int f = 0; f < nf; f++) {
      TRY(dalloc(h, &h->fields[b][f], vbytes));
      if (cudaMemset(h->fields[b][f], 0, vbytes) != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "cudaMemset failed"); TRY(SE2GPU_ERR_CUDA); }
    }
  // mass: FP64 keeps M (the reference divides); FP32 stores 1/M computed in FP64
  if (precision == SE2GPU_FP64) {
    TRY(upload(h, &h->mass, P->mass, (size_t)nnodes));
  } else {
    std::vector<double> minv((size_t)nnodes);
    for (long i = 0; i < nnodes; i++) minv[i] = 1.0 / P->mass[i];
    TRY(upload(h, &h->mass, minv.data(), (size_t)nnodes));
  }
  TRY(upload(h, &h->lam, P->lambda, (size_t)ne));
  TRY(upload(h, &h->mu, P->mu, (size_t)ne));
  TRY(upload(h, &h->J00, P->J00, (size_t)P->mx));
  TRY(upload(h, &h->J11, P->J11, (size_t)P->my));
  TRY(upload(h, &h->iJ00, P->iJ00, (size_t)P->mx));
  TRY(upload(h, &h->iJ11, P->iJ11, (size_t)P->my));
  TRY(upload(h, &h->D, P->D, (size_t)npe));
  TRY(upload(h, &h->wq, P->wq, (size_t)npe));
  TRY(upload_d(h, &h->Dd, P->D, (size_t)npe));
  TRY(upload_d(h, &h->iJ00d, P->iJ00, (size_t)P->mx));
  TRY(upload_d(h, &h->iJ11d, P->iJ11, (size_t)P->my));
  TRY(upload_i(h, &h->src_elem, P->src_elem, (size_t)P->nsrc));
  if (P->nsrc) TRY(upload(h, &h->src_vals, P->src_vals, (size_t)P->nsrc * 2 * npe));
  TRY(upload_i(h, &h->rec_node, P->rec_node, (size_t)P->nrec));
  TRY(upload_i(h, &h->rec_elem, P->rec_elem, (size_t)P->nrec));
  TRY(upload_i(h, &h->rec_gll, P->rec_gll, (size_t)P->nrec));
  TRY(dalloc(h, (void **)&h->traces, (size_t)trace_capacity * 7 * P->nrec * 8));
  TRY(dalloc(h, (void **)&h->norm_part, 6 * 1024 * 8));
#undef TRY
  *out = h;
  return 0;
}

extern "C" int se2gpu_set_stream(se2gpu_solver *h, void *stream)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return 0;
}

extern "C" int se2gpu_synchronize(se2gpu_solver *h)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

template <typename T>
static se2::StepParams<T> base_params(se2gpu_solver *h)
{
  se2::StepParams<T> prm;
  memset(&prm, 0, sizeof(prm));
  prm.mx = h->mx; prm.my = h->my; prm.nx_g = h->nx_g; prm.ny_g = h->ny_g;
  prm.ntx = h->ntx; prm.nty = h->nty;
  prm.mass = (const T *)h->mass; prm.lam = (const T *)h->lam; prm.mu = (const T *)h->mu;
  prm.J00 = (const T *)h->J00; prm.J11 = (const T *)h->J11; prm.iJ00 = (const T *)h->iJ00; prm.iJ11 = (const T *)h->iJ11;
  prm.D = (const T *)h->D; prm.wq = (const T *)h->wq;
  // coefficients exactly as the reference forms them: dt, 0.5*dt*dt, 0.5*dt
  prm.c_dt = (T)h->dt; prm.c_u = (T)(0.5 * h->dt * h->dt); prm.c_v = (T)(0.5 * h->dt);
  prm.nsrc = h->nsrc; prm.src_elem = h->src_elem; prm.src_vals = (const T *)h->src_vals;
  prm.nrec = h->nrec; prm.rec_node = h->rec_node; prm.rec_elem = h->rec_elem; prm.rec_gll = h->rec_gll;
  prm.Dd = h->Dd; prm.iJ00d = h->iJ00d; prm.iJ11d = h->iJ11d;
  return prm;
}

template <typename T>
static void bind_state(se2gpu_solver *h, se2::StepParams<T> &prm, int in, int outb)
{
  typedef typename se2::Vec2<T>::type T2;
  prm.u_in = (const T2 *)h->fields[in][0]; prm.v_in = (const T2 *)h->fields[in][1]; prm.a_in = (const T2 *)h->fields[in][2];
  prm.cu_in = (const T2 *)h->fields[in][3]; prm.cv_in = (const T2 *)h->fields[in][4];
  prm.u_out = (T2 *)h->fields[outb][0]; prm.v_out = (T2 *)h->fields[outb][1]; prm.a_out = (T2 *)h->fields[outb][2];
  prm.cu_out = (T2 *)h->fields[outb][3]; prm.cv_out = (T2 *)h->fields[outb][4];
}

static cudaError_t launch_step(se2gpu_solver *h, const void *prm, int nblocks)
{
  h->launches++;
  if (h->precision == SE2GPU_FP64)
    return se2::launch_step_f64(h->p, *(const se2::StepParams<double> *)prm, nblocks, h->stream);
  return se2::launch_step_f32(h->p, h->precision == SE2GPU_FP32_KAHAN, *(const se2::StepParams<float> *)prm, nblocks, h->stream);
}

// record the receivers of the current state if a step left its row pending
static int flush_record(se2gpu_solver *h)
{
  if (!h->pending_record) return 0;
  cudaError_t e;
  h->launches++;
  if (h->precision == SE2GPU_FP64) {
    auto prm = base_params<double>(h);
    bind_state(h, prm, h->cur, h->cur);
    prm.record = 1;
    prm.trace_row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
    e = se2::launch_record_f64(h->p, prm, h->stream);
  } else {
    auto prm = base_params<float>(h);
    bind_state(h, prm, h->cur, h->cur);
    prm.record = 1;
    prm.trace_row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
    e = se2::launch_record_f32(h->p, prm, h->stream);
  }
  if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "receiver kernel: %s", cudaGetErrorString(e));
  h->rows_written++;
  h->pending_record = false;
  return 0;
}

template <typename T>
static int advance_t(se2gpu_solver *h, int nsteps)
{
  auto prm = base_params<T>(h);
  prm.mode = 0;
  for (int k = 0; k < nsteps; k++) {
    bind_state(h, prm, h->cur, 1 - h->cur);
    prm.stf = h->stf_dev + (size_t)k * h->nsrc;
    prm.record = h->pending_record ? 1 : 0;
    prm.trace_row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
    cudaError_t e = launch_step(h, &prm, h->nblocks);
    if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "step kernel: %s", cudaGetErrorString(e));
    if (h->pending_record) { h->rows_written++; h->pending_record = false; }
    h->cur = 1 - h->cur;
    if (h->nrec > 0) h->pending_record = true;
  }
  return 0;
}

extern "C" int se2gpu_advance(se2gpu_solver *h, int nsteps, const double *stf)
{
  if (!h) return SE2GPU_ERR_ARG;
  if (nsteps < 0) return fail(h, SE2GPU_ERR_ARG, "negative step count");
  if (nsteps == 0) return 0;
  if (h->nsrc && !stf) return fail(h, SE2GPU_ERR_ARG, "stf values required for %d sources", h->nsrc);
  if (h->nrec && (long)h->rows_written + (h->pending_record ? 1 : 0) + nsteps > h->trace_cap)
    return fail(h, SE2GPU_ERR_STATE, "trace buffer full: %d rows buffered, capacity %d; call se2gpu_traces",
                h->rows_written + (h->pending_record ? 1 : 0), h->trace_cap);
  CK(h, cudaSetDevice(h->device));
  if (h->nsrc) {
    if (nsteps > h->stf_cap) {
      CK(h, cudaStreamSynchronize(h->stream));
      cudaFree(h->stf_dev);
      h->stf_dev = nullptr;
      int rc = dalloc(h, (void **)&h->stf_dev, (size_t)nsteps * h->nsrc * 8);
      if (rc) { h->stf_cap = 0; return rc; }
      h->stf_cap = nsteps;
    }
    // the previous block may still read stf_dev: order the copy on the stream
    CK(h, cudaMemcpyAsync(h->stf_dev, stf, (size_t)nsteps * h->nsrc * 8, cudaMemcpyHostToDevice, h->stream));
  }
  return (h->precision == SE2GPU_FP64) ? advance_t<double>(h, nsteps) : advance_t<float>(h, nsteps);
}

extern "C" int se2gpu_traces(se2gpu_solver *h, double *out, int max_rows)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  int rc = flush_record(h);
  if (rc) return rc;
  if (h->rows_written > max_rows)
    return fail(h, SE2GPU_ERR_ARG, "output holds %d rows but %d are buffered", max_rows, h->rows_written);
  const int rows = h->rows_written;
  if (rows && h->nrec) {
    if (!out) return fail(h, SE2GPU_ERR_ARG, "null output");
    CK(h, cudaMemcpyAsync(out, h->traces, (size_t)rows * 7 * h->nrec * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  CK(h, cudaGetLastError());
  h->rows_written = 0;
  return rows;
}

extern "C" int se2gpu_set_fields(se2gpu_solver *h, const double *u, const double *v, const double *a)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  int rc = flush_record(h);
  if (rc) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  const size_t n = (size_t)h->nnodes * 2;
  const double *src[3] = {u, v, a};
  for (int f = 0; f < 3; f++) {
    if (!src[f]) continue;
    if (h->tsize == 8) {
      CK(h, cudaMemcpy(h->fields[h->cur][f], src[f], n * 8, cudaMemcpyHostToDevice));
    } else {
      std::vector<float> tmp(n);
      for (size_t i = 0; i < n; i++) tmp[i] = (float)src[f][i];
      CK(h, cudaMemcpy(h->fields[h->cur][f], tmp.data(), n * 4, cudaMemcpyHostToDevice));
    }
  }
  if (h->precision == SE2GPU_FP32_KAHAN) {
    CK(h, cudaMemset(h->fields[h->cur][3], 0, n * 4));
    CK(h, cudaMemset(h->fields[h->cur][4], 0, n * 4));
  }
  return 0;
}

extern "C" int se2gpu_get_fields(se2gpu_solver *h, double *u, double *v, double *a)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  CK(h, cudaStreamSynchronize(h->stream));
  const size_t n = (size_t)h->nnodes * 2;
  double *dst[3] = {u, v, a};
  for (int f = 0; f < 3; f++) {
    if (!dst[f]) continue;
    if (h->tsize == 8) {
      CK(h, cudaMemcpy(dst[f], h->fields[h->cur][f], n * 8, cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> tmp(n);
      CK(h, cudaMemcpy(tmp.data(), h->fields[h->cur][f], n * 4, cudaMemcpyDeviceToHost));
      for (size_t i = 0; i < n; i++) dst[f][i] = (double)tmp[i];
    }
  }
  return 0;
}

extern "C" int se2gpu_norms(se2gpu_solver *h, double out[6])
{
  if (!h || !out) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  const long n = h->nnodes * 2;
  const int nb = 1024;
  h->launches++;
  if (h->tsize == 8)
    se2::norms_partial<double><<<nb, 256, 0, h->stream>>>((const double *)h->fields[h->cur][0], (const double *)h->fields[h->cur][1], n, h->norm_part);
  else
    se2::norms_partial<float><<<nb, 256, 0, h->stream>>>((const float *)h->fields[h->cur][0], (const float *)h->fields[h->cur][1], n, h->norm_part);
  CK(h, cudaGetLastError());
  std::vector<double> part(6 * nb);
  CK(h, cudaMemcpyAsync(part.data(), h->norm_part, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  double r[6] = {-1.0e308, 1.0e308, 0.0, -1.0e308, 1.0e308, 0.0};
  for (int b = 0; b < nb; b++) {
    r[0] = std::fmax(r[0], part[6 * b + 0]); r[1] = std::fmin(r[1], part[6 * b + 1]); r[2] += part[6 * b + 2];
    r[3] = std::fmax(r[3], part[6 * b + 3]); r[4] = std::fmin(r[4], part[6 * b + 4]); r[5] += part[6 * b + 5];
  }
  out[0] = r[0]; out[1] = r[1]; out[2] = std::sqrt(r[2]);
  out[3] = r[3]; out[4] = r[4]; out[5] = std::sqrt(r[5]);
  if (!std::isfinite(out[2]) || !std::isfinite(out[5]))
    return fail(h, SE2GPU_ERR_NUMERIC, "non-finite field norm (u l2 = %g, v l2 = %g)", out[2], out[5]);
  return 0;
}

template <typename T>
static int force_t(se2gpu_solver *h, const void *u_dev, void *F_dev)
{
  typedef typename se2::Vec2<T>::type T2;
  auto prm = base_params<T>(h);
  prm.mode = 1;
  prm.u_in = (const T2 *)u_dev;
  prm.f_out = (T2 *)F_dev;
  prm.record = 0;
  cudaError_t e = launch_step(h, &prm, h->nblocks - 1);
  if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "force kernel: %s", cudaGetErrorString(e));
  return 0;
}

extern "C" int se2gpu_assemble_linear_form_device(se2gpu_solver *h, const void *u_dev, void *F_dev)
{
  if (!h || !u_dev || !F_dev) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  return (h->tsize == 8) ? force_t<double>(h, u_dev, F_dev) : force_t<float>(h, u_dev, F_dev);
}

extern "C" int se2gpu_assemble_linear_form(se2gpu_solver *h, const double *u, double *F)
{
  if (!h || !u || !F) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  const size_t n = (size_t)h->nnodes * 2;
  int rc;
  if (!h->scratch_u && (rc = dalloc(h, &h->scratch_u, n * h->tsize))) return rc;
  if (!h->scratch_f && (rc = dalloc(h, &h->scratch_f, n * h->tsize))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  if (h->tsize == 8) {
    CK(h, cudaMemcpy(h->scratch_u, u, n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (float)u[i];
    CK(h, cudaMemcpy(h->scratch_u, tmp.data(), n * 4, cudaMemcpyHostToDevice));
  }
  if ((rc = se2gpu_assemble_linear_form_device(h, h->scratch_u, h->scratch_f))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  if (h->tsize == 8) {
    CK(h, cudaMemcpy(F, h->scratch_f, n * 8, cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> tmp(n);
    CK(h, cudaMemcpy(tmp.data(), h->scratch_f, n * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) F[i] = (double)tmp[i];
  }
  return 0;
}

extern "C" int se2gpu_info(const se2gpu_solver *h, long *ints)
{
  if (!h || !ints) return SE2GPU_ERR_ARG;
  ints[0] = h->nx_g; ints[1] = h->ny_g; ints[2] = h->p; ints[3] = h->precision;
  ints[4] = h->nsrc; ints[5] = h->nrec; ints[6] = h->launches; ints[7] = h->rows_written + (h->pending_record ? 1 : 0);
  return 0;
}

extern "C" int se2gpu_device_fields(const se2gpu_solver *h, void **u, void **v, void **a)
{
  if (!h) return SE2GPU_ERR_ARG;
  if (u) *u = h->fields[h->cur][0];
  if (v) *v = h->fields[h->cur][1];
  if (a) *a = h->fields[h->cur][2];
  return 0;
}
