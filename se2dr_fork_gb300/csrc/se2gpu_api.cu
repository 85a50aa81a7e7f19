// se2gpu_api.cu -- C-ABI of libse2gpu.so (see include/se2gpu.h).
//
// FP64 mode keeps the reference's state (u, v, a) in the reference's packed
// [node][component] layout and runs the tiled reference-order kernel
// (se2gpu_kernels.cuh).  FP32 modes keep the leapfrog state (u, w = half-step
// velocity, Kahan terms) in a padded layout (row pitch a multiple of 16 nodes,
// as the TMA copies require) and run the persistent TMA-pipelined kernel
// (se2gpu_persist.cuh); set/get_fields convert to and from the reference's
// (u, v, a) in FP64 on the host.  Every entry point validates its arguments on
// the host and returns a status code; CUDA errors and the kernels' bounded-wait
// error flag are reported through se2gpu_last_error.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <climits>
#include <memory>
#include <mutex>
#include <thread>
#include <unistd.h>
#include <utility>
#include <vector>

#include "se2gpu.h"
#include "se2gpu_internal.h"
#include "se2gpu_launch.h"
#include "se2gpu_persist_launch.h"


static thread_local char g_create_err[512];

extern "C" const char *se2gpu_create_error(void) { return g_create_err; }
void se2gpu_internal_set_error(const char *msg) { snprintf(g_create_err, sizeof(g_create_err), "%s", msg); }
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

#define CK(h, call)                                                                                              \
  do {                                                                                                           \
    cudaError_t e_ = (call);                                                                                     \
    if (e_ != cudaSuccess) return fail((h), SE2GPU_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                                       __FILE__, __LINE__);                                                      \
  } while (0)

static bool is_f64(const se2gpu_solver *h) { return h->precision == SE2GPU_FP64; }
// FP32 modes that keep compensation terms of u and w (Kahan and two-float)
static bool is_kahan(const se2gpu_solver *h) { return h->precision == SE2GPU_FP32_KAHAN || h->precision == SE2GPU_FP32_DF; }
static bool is_df(const se2gpu_solver *h) { return h->precision == SE2GPU_FP32_DF; }
// the persistent kernel's arithmetic mode
static int pmode(const se2gpu_solver *h)
{
  return is_df(h) ? se2p::MODE_DF : (h->precision == SE2GPU_FP32_KAHAN) ? se2p::MODE_KAHAN : se2p::MODE_PLAIN;
}
// receiver side-buffer floats per element node: (u, v, a), with low parts in the two-float mode
static int rbuf_values(const se2gpu_solver *h) { return is_df(h) ? 12 : 6; }
// the two-float mode keeps the low parts of the last step's a after the high parts
static float2 *pa_lo(const se2gpu_solver *h) { return is_df(h) ? h->pa + (size_t)h->ny_g * h->pitch : nullptr; }

// Device memory of the handles comes from one stream-ordered pool per device whose
// release threshold keeps freed memory for the next handle: a create that follows a
// destroy in the same process maps no new memory, and allocations, frees and the
// zeroing of the state are queued on the handle's stream without host waits.  When the
// pool cannot grow, the memory it holds unused is returned to the device and the
// allocation is tried once more.
static cudaMemPool_t device_pool(int dev)
{
  static std::mutex mu;
  static cudaMemPool_t pools[64];
  static bool made[64];
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!made[dev]) {
    cudaMemPoolProps pr;
    memset(&pr, 0, sizeof(pr));
    pr.allocType = cudaMemAllocationTypePinned;
    pr.location.type = cudaMemLocationTypeDevice;
    pr.location.id = dev;
    if (cudaMemPoolCreate(&pools[dev], &pr) != cudaSuccess) {
      cudaGetLastError();
      pools[dev] = nullptr;
    } else {
      cuuint64_t keep = ~(cuuint64_t)0;
      cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    made[dev] = true;
  }
  return pools[dev];
}

static int dalloc(se2gpu_solver *h, void **p, size_t bytes)
{
  *p = nullptr;
  const size_t n = bytes ? bytes : 16;
  cudaMemPool_t pool = device_pool(h->device);
  cudaError_t e = pool ? cudaMallocFromPoolAsync(p, n, pool, h->stream) : cudaErrorMemoryAllocation;
  if (e != cudaSuccess && pool) {
    cudaGetLastError();
    cudaStreamSynchronize(h->stream);
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(p, n, pool, h->stream);
  }
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(h, SE2GPU_ERR_NOMEM, "device allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
  }
  return 0;
}

// free a handle allocation (null is ignored), ordered on the handle's stream
static void dfree(se2gpu_solver *h, void *p)
{
  if (p) cudaFreeAsync(p, h->stream);
}

static int dzero(se2gpu_solver *h, void **p, size_t bytes)
{
  int rc = dalloc(h, p, bytes);
  if (rc) return rc;
  CK(h, cudaMemsetAsync(*p, 0, bytes ? bytes : 16, h->stream));
  return 0;
}

// fn(begin, end) over [0, n) on up to 16 host threads (at least minchunk items each): the
// per-node host passes over meshes of tens of millions of nodes
template <class F>
static void host_parallel(long n, F fn, long minchunk = 1L << 20)
{
  long nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nt = std::min(nt, (n + minchunk - 1) / minchunk);
  if (nt <= 1) {
    fn(0L, n);
    return;
  }
  std::vector<std::thread> th;
  for (long t = 0; t < nt; t++) th.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
  for (std::thread &x : th) x.join();
}

// 1/M in the padded FP32 layout (padding nodes 0) straight from the caller's FP64 mass,
// for devices that read pageable host memory (cudaDevAttrPageableMemoryAccess).  Double
// division and the conversion to float round as on the host, so the values are the same.
// minv_lo (two-float mode, else null): the remainder 1/M - minv, rounded to float.  *bad
// receives the smallest node whose mass is not positive and finite (it starts at ~0).
// Block (bx, by) takes 1024 padded columns of rows by, by + gridDim.y, ..., four per thread,
// the four host loads issued before any is used so that more of the host link's latency is
// in flight.
__global__ void __launch_bounds__(256) k_minv_from_host(const double *__restrict__ mass, long nx_g, long ny_g,
                                                        int pitch, float *__restrict__ minv,
                                                        float *__restrict__ minv_lo, unsigned long long *bad)
{
  for (long y = blockIdx.y; y < ny_g; y += gridDim.y) {
  const double *row = mass + y * nx_g;
  double m[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const long x = (long)blockIdx.x * 1024 + k * 256 + threadIdx.x;
    m[k] = (x < nx_g) ? row[x] : 1.0;
  }
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const long x = (long)blockIdx.x * 1024 + k * 256 + threadIdx.x;
    if (x >= pitch) continue;
    const long i = y * pitch + x;
    if (!(m[k] > 0.0) || !isfinite(m[k])) atomicMin(bad, (unsigned long long)(y * nx_g + x));
    const double r = (x < nx_g) ? 1.0 / m[k] : 0.0;
    const float h = __double2float_rn(r);
    minv[i] = h;
    if (minv_lo) minv_lo[i] = __double2float_rn(__dsub_rn(r, (double)h));
  }
  }
}

// Bulk transfers between the caller's host arrays and the device, done by kernels that
// read or write the host memory directly when the device can (pageable access): no
// staging copy of whole arrays through pageable memory, and the layout conversion runs
// on the device.  The arithmetic repeats the host paths operation for operation
// (explicit round-to-nearest, nothing fused), so both give the same values.
__global__ void k_copy_f64(double *__restrict__ dst, const double *__restrict__ src, size_t n)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// FP32 leapfrog state (padded rows) -> FP64 (u, v, a) in the reference's node order
// (AL: the low parts of a in the two-float mode, else null)
__global__ void k_fields_to_host(const float2 *__restrict__ U, const float2 *__restrict__ W,
                                 const float2 *__restrict__ CU, const float2 *__restrict__ CW,
                                 const float2 *__restrict__ A, const float2 *__restrict__ AL, long nx_g, long ny_g,
                                 int pitch, double dt, double hdt, double *u, double *v, double *a)
{
  const long nn = nx_g * ny_g;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += (long)gridDim.x * blockDim.x) {
    const long y = i / nx_g, x = i - y * nx_g, k = y * pitch + x;
    const float2 w = W[k], uu = U[k], ac = A[k], al = AL ? AL[k] : make_float2(0.f, 0.f);
    const float2 cw = CW ? CW[k] : make_float2(0.f, 0.f), cu = CU ? CU[k] : make_float2(0.f, 0.f);
    const double w0 = __dsub_rn((double)w.x, (double)cw.x), w1 = __dsub_rn((double)w.y, (double)cw.y);
    const double u0 = __dsub_rn((double)uu.x, (double)cu.x), u1 = __dsub_rn((double)uu.y, (double)cu.y);
    const double a0 = __dadd_rn((double)ac.x, (double)al.x), a1 = __dadd_rn((double)ac.y, (double)al.y);
    if (u) { u[2 * i] = __dsub_rn(u0, __dmul_rn(dt, w0)); u[2 * i + 1] = __dsub_rn(u1, __dmul_rn(dt, w1)); }
    if (v) { v[2 * i] = __dsub_rn(w0, __dmul_rn(hdt, a0)); v[2 * i + 1] = __dsub_rn(w1, __dmul_rn(hdt, a1)); }
    if (a) { a[2 * i] = a0; a[2 * i + 1] = a1; }
  }
}

// FP64 (u, v, a) -> FP32 leapfrog state with its Kahan terms (padding nodes 0)
__global__ void k_fields_from_host(const double *u, const double *v, const double *a, long nx_g, long ny_g,
                                   int pitch, double dt, double hdt, float2 *__restrict__ U, float2 *__restrict__ W,
                                   float2 *__restrict__ CU, float2 *__restrict__ CW, float2 *__restrict__ A,
                                   float2 *__restrict__ AL)
{
  const long np = ny_g * (long)pitch;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < np; k += (long)gridDim.x * blockDim.x) {
    const long y = k / pitch, x = k - y * pitch;
    float2 Wk = make_float2(0.f, 0.f), Uk = Wk, CWk = Wk, CUk = Wk, Ak = Wk, ALk = Wk;
    if (x < nx_g) {
      const long n = y * nx_g + x;
      double wv[2], uv[2];
      for (int c = 0; c < 2; c++) {
        const double uu = u ? u[2 * n + c] : 0.0, vv = v ? v[2 * n + c] : 0.0, aa = a ? a[2 * n + c] : 0.0;
        wv[c] = __dadd_rn(vv, __dmul_rn(hdt, aa));
        uv[c] = __dadd_rn(uu, __dmul_rn(dt, wv[c]));
      }
      Wk = make_float2(__double2float_rn(wv[0]), __double2float_rn(wv[1]));
      Uk = make_float2(__double2float_rn(uv[0]), __double2float_rn(uv[1]));
      CWk = make_float2(__double2float_rn(__dsub_rn((double)Wk.x, wv[0])), __double2float_rn(__dsub_rn((double)Wk.y, wv[1])));
      CUk = make_float2(__double2float_rn(__dsub_rn((double)Uk.x, uv[0])), __double2float_rn(__dsub_rn((double)Uk.y, uv[1])));
      Ak = make_float2(a ? __double2float_rn(a[2 * n]) : 0.f, a ? __double2float_rn(a[2 * n + 1]) : 0.f);
      if (a && AL)
        ALk = make_float2(__double2float_rn(__dsub_rn(a[2 * n], (double)Ak.x)),
                          __double2float_rn(__dsub_rn(a[2 * n + 1], (double)Ak.y)));
    }
    U[k] = Uk; W[k] = Wk; A[k] = Ak;
    if (AL) AL[k] = ALk;
    if (CU) { CU[k] = CUk; CW[k] = CWk; }
  }
}

// Output arrays the device is about to write: fault their pages in on the host threads
// first (one store per page), since a first touch taken through the device is much
// slower.  The stores write zeros into memory that is overwritten next.
static void prefault_output(double *p, size_t n)
{
  if (!p || !n) return;
  const long page = std::max(4096L, sysconf(_SC_PAGESIZE));
  const size_t per = (size_t)page / sizeof(double);
  const long npages = (long)((n + per - 1) / per);
  host_parallel(npages, [&](long i0, long i1) {
    volatile double *q = p;
    for (long i = i0; i < i1; i++) q[(size_t)i * per] = 0.0;
  }, 256);
}

// copy n doubles between host and device through a kernel (pageable access) or cudaMemcpy
static int copy_f64(se2gpu_solver *h, double *dst, const double *src, size_t n, cudaMemcpyKind kind)
{
  if (!n) return 0;
  if (h->pageable) {
    if (kind == cudaMemcpyDeviceToHost) prefault_output(dst, n);
    k_copy_f64<<<4 * h->nsm, 256, 0, h->stream>>>(dst, src, n);
    CK(h, cudaGetLastError());
    CK(h, cudaStreamSynchronize(h->stream));
  } else {
    CK(h, cudaMemcpyAsync(dst, src, n * 8, kind, h->stream));
  }
  return 0;
}

// FP64 host array -> nearest floats (and, with lo, the remainders rounded to float), read
// where it lies by a device that reads pageable host memory
__global__ void k_to_float(const double *__restrict__ src, size_t n, float *__restrict__ dst, float *__restrict__ lo)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    const float f = __double2float_rn(v);
    dst[i] = f;
    if (lo) lo[i] = __double2float_rn(__dsub_rn(v, (double)f));
  }
}

// the constants of each cell as the plain and Kahan step kernels use them, from the
// float tables: (lam detJ, mu detJ, d xi/dx, d eta/dy), detJ = J00 J11, products rounded
__global__ void k_cell_consts(const float *__restrict__ lam, const float *__restrict__ mu, const float *__restrict__ J00,
                              const float *__restrict__ J11, const float *__restrict__ iJ00,
                              const float *__restrict__ iJ11, int mx, long ne, float4 *__restrict__ out)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ne; i += (long)gridDim.x * blockDim.x) {
    const int ex = (int)(i % mx), ey = (int)(i / mx);
    const float detJ = __fmul_rn(J00[ex], J11[ey]);
    out[i] = make_float4(__fmul_rn(lam[i], detJ), __fmul_rn(mu[i], detJ), iJ00[ex], iJ11[ey]);
  }
}

// upload an FP64 host array in the handle's compute precision (two-float mode: the n
// nearest floats followed by the n remainders, rounded to float).  FP32 tables on a
// device that reads pageable host memory are converted by a kernel on the handle's
// stream, which se2gpu_create synchronises once at its end (the caller's arrays stay
// valid until it returns).
static int upload(se2gpu_solver *h, void **dst, const double *src, size_t n)
{
  const size_t nf = is_df(h) ? 2 * n : n;
  int rc = dalloc(h, dst, nf * h->tsize);
  if (rc) return rc;
  if (h->tsize == 8) {
    return copy_f64(h, (double *)*dst, src, n, cudaMemcpyHostToDevice);
  } else if (h->pageable && n) {
    float *d = (float *)*dst;
    k_to_float<<<(int)std::min<size_t>((n + 255) / 256, (size_t)4 * h->nsm), 256, 0, h->stream>>>(
        src, n, d, nf > n ? d + n : nullptr);
    CK(h, cudaGetLastError());
  } else {
    std::vector<float> tmp(nf);
    host_parallel((long)n, [&](long i0, long i1) {
      for (long i = i0; i < i1; i++) tmp[i] = (float)src[i];
      if (nf > n)
        for (long i = i0; i < i1; i++) tmp[n + i] = (float)(src[i] - (double)tmp[i]);
    });
    if (nf) CK(h, cudaMemcpyAsync(*dst, tmp.data(), nf * 4, cudaMemcpyHostToDevice, h->stream));
  }
  return 0;
}

// (cudaMemcpyAsync from pageable host memory returns once the source has been staged)
static int upload_d(se2gpu_solver *h, double **dst, const double *src, size_t n)
{
  int rc = dalloc(h, (void **)dst, n * 8);
  if (rc) return rc;
  if (n) CK(h, cudaMemcpyAsync(*dst, src, n * 8, cudaMemcpyHostToDevice, h->stream));
  return 0;
}

static int upload_i(se2gpu_solver *h, int **dst, const int *src, size_t n)
{
  int rc = dalloc(h, (void **)dst, n * 4);
  if (rc) return rc;
  if (n) CK(h, cudaMemcpyAsync(*dst, src, n * 4, cudaMemcpyHostToDevice, h->stream));
  return 0;
}

extern "C" void se2gpu_destroy(se2gpu_solver *h)
{
  if (!h) return;
  cudaSetDevice(h->device);
  for (cudaEvent_t &ev : h->side_done)   // set-up work of a create that failed part-way
    if (ev) { cudaEventSynchronize(ev); cudaEventDestroy(ev); ev = nullptr; }
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int b = 0; b < 2; b++) {
    for (int f = 0; f < 3; f++) dfree(h, h->f64[b][f]);
    dfree(h, h->pu[b]); dfree(h, h->pw[b]); dfree(h, h->pcu[b]); dfree(h, h->pcw[b]); dfree(h, h->rbuf[b]);
  }
  void *ptrs[] = {h->pa, h->pminv, h->mass_bad, h->err_dev, h->mass, h->lam, h->mu, h->J00, h->J11, h->iJ00, h->iJ11, h->D, h->wq,
                  h->src_vals, h->Dd, h->iJ00d, h->iJ11d, h->stf_dev, h->traces, h->norm_part, h->src_elem,
                  h->rec_node, h->rec_elem, h->rec_gll, h->scratch_u, h->scratch_f, h->tile_src_off,
                  h->tile_src_idx, h->tile_rec_off, h->tile_rec_idx, h->cellc, h->tile_bounds};
  for (void *p : ptrs) dfree(h, p);
  if (h->stream) cudaStreamSynchronize(h->stream);   // the frees are done before the stream goes
  delete h->src_elem_h;
  delete h->rec_elem_h;
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  free(h);
}

// the FP32 leapfrog state of the reference's (u, v, a) at step k:
// w = v + dt/2 a, u' = u + dt w, stored as FP32 value + Kahan residual (true = hi - lo)
static int upload_leapfrog(se2gpu_solver *h, const double *u, const double *v, const double *a)
{
  const size_t np = (size_t)h->ny_g * h->pitch;
  if (h->pageable) {
    const int c = h->cur;
    const bool kahan = is_kahan(h);
    k_fields_from_host<<<4 * h->nsm, 256, 0, h->stream>>>(u, v, a, h->nx_g, h->ny_g, h->pitch, h->dt, 0.5 * h->dt,
                                                          h->pu[c], h->pw[c], kahan ? h->pcu[c] : nullptr,
                                                          kahan ? h->pcw[c] : nullptr, h->pa, pa_lo(h));
    CK(h, cudaGetLastError());
    CK(h, cudaStreamSynchronize(h->stream));
    return 0;
  }
  std::vector<float2> U(np), W(np), CU(np), CW(np), A(np), AL(np, make_float2(0.f, 0.f));
  const double dt = h->dt, hdt = 0.5 * h->dt;
  for (long y = 0; y < h->ny_g; y++)
    for (long x = 0; x < h->nx_g; x++) {
      const size_t n = (size_t)(y * h->nx_g + x), k = (size_t)(y * h->pitch + x);
      double wv[2], uv[2];
      for (int c = 0; c < 2; c++) {
        const double uu = u ? u[2 * n + c] : 0.0, vv = v ? v[2 * n + c] : 0.0, aa = a ? a[2 * n + c] : 0.0;
        wv[c] = vv + hdt * aa;
        uv[c] = uu + dt * wv[c];
      }
      W[k] = make_float2((float)wv[0], (float)wv[1]);
      U[k] = make_float2((float)uv[0], (float)uv[1]);
      CW[k] = make_float2((float)((double)W[k].x - wv[0]), (float)((double)W[k].y - wv[1]));
      CU[k] = make_float2((float)((double)U[k].x - uv[0]), (float)((double)U[k].y - uv[1]));
      A[k] = make_float2(a ? (float)a[2 * n] : 0.f, a ? (float)a[2 * n + 1] : 0.f);
      if (a) AL[k] = make_float2((float)(a[2 * n] - (double)A[k].x), (float)(a[2 * n + 1] - (double)A[k].y));
    }
  const int c = h->cur;
  CK(h, cudaMemcpyAsync(h->pu[c], U.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->pw[c], W.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
  if (is_kahan(h)) {
    CK(h, cudaMemcpyAsync(h->pcu[c], CU.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->pcw[c], CW.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
  }
  CK(h, cudaMemcpyAsync(h->pa, A.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
  if (pa_lo(h)) CK(h, cudaMemcpyAsync(pa_lo(h), AL.data(), np * 8, cudaMemcpyHostToDevice, h->stream));
  return 0;
}

// the step kernel's tensor maps of the per-tile constants (plain and Kahan modes): the
// cell box and the 1/M box, the same for both buffer sets (the two-float mode reads its
// constants with loads and has neither)
static int make_const_maps(se2gpu_solver *h, const se2p::TileShape &ts)
{
  for (int b = 0; b < 2; b++) memset(&h->maps[b][4], 0, 2 * sizeof(CUtensorMap));
  if (pmode(h) == se2p::MODE_DF) return 0;
  int r = se2p::make_map_cells(&h->maps[0][4], h->cellc, h->mx, h->my, ts.cell_box);
  if (!r) r = se2p::make_map_f32(&h->maps[0][5], h->pminv, h->pitch, h->ny_g, h->pitch, ts.minv_w, ts.own_h);
  if (r) return fail(h, SE2GPU_ERR_CUDA, "cuTensorMapEncodeTiled failed for the tile constants (%d)", r);
  h->maps[1][4] = h->maps[0][4];
  h->maps[1][5] = h->maps[0][5];
  return 0;
}

// select one of the persistent kernel's tile configurations: kernel attributes,
// tensor-map boxes, per-tile source/receiver lists and the persistent grid
// (in_create: the handle has run no step yet, so nothing in flight reads the tile lists
// and the host work here overlaps the set-up kernels still reading the caller's arrays)
static int setup_f32_config(se2gpu_solver *h, int config, bool in_create = false)
{
  const bool kahan = is_kahan(h);
  const int mode = pmode(h);
  se2p::TileShape ts;
  if (se2p::config_shape(h->p, config, mode, &ts)) return fail(h, SE2GPU_ERR_ARG, "no tile configuration %d for degree %d", config, h->p);
  if (!in_create) CK(h, cudaStreamSynchronize(h->stream));
  {
    cudaError_t e = se2p::prepare(h->p, config, mode);
    if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "persistent kernel set-up: %s", cudaGetErrorString(e));
  }
  for (int b = 0; b < 2; b++) {
    void *bases[4] = {h->pu[b], kahan ? (void *)h->pcu[b] : (void *)h->pu[b], h->pw[b], kahan ? (void *)h->pcw[b] : (void *)h->pw[b]};
    for (int m = 0; m < 4; m++) {
      const int bw = (m < 2) ? ts.region_w : ts.own_w, bh = (m < 2) ? ts.region_h : ts.own_h;
      const int r = se2p::make_map(&h->maps[b][m], bases[m], h->nx_g, h->ny_g, h->pitch, bw, bh);
      if (r) return fail(h, SE2GPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", r);
    }
  }
  if (h->pminv) {   // (in se2gpu_create the 1/M map follows once 1/M is allocated)
    int r = make_const_maps(h, ts);
    if (r) return r;
  }
  const int te = ts.tex, P = h->p;
  const int ntx = (h->mx + te - 1) / te, nty = (h->my + te - 1) / te, ntiles = ntx * nty;
  // tile lists: a source or receiver element appears in every tile whose owned nodes it touches
  auto build = [&](const std::vector<int> &elems, std::vector<int> &off, std::vector<int> &idx) {
    std::vector<std::vector<int>> per(ntiles);
    for (int q = 0; q < (int)elems.size(); q++) {
      const int ex = elems[q] % h->mx, ey = elems[q] / h->mx;
      for (int ty = std::max(0, (ey - 1) / te); ty <= std::min(nty - 1, (ey + 1) / te); ty++)
        for (int tx = std::max(0, (ex - 1) / te); tx <= std::min(ntx - 1, (ex + 1) / te); tx++) {
          const int X0 = tx * te * P, X1 = std::min((tx + 1) * te, h->mx) * P + (((tx + 1) * te >= h->mx) ? 1 : 0);
          const int Y0 = ty * te * P, Y1 = std::min((ty + 1) * te, h->my) * P + (((ty + 1) * te >= h->my) ? 1 : 0);
          if (ex * P <= X1 - 1 && ex * P + P >= X0 && ey * P <= Y1 - 1 && ey * P + P >= Y0) per[ty * ntx + tx].push_back(q);
        }
    }
    off.assign(ntiles + 1, 0);
    for (int t = 0; t < ntiles; t++) off[t + 1] = off[t] + (int)per[t].size();
    idx.clear();
    for (int t = 0; t < ntiles; t++) idx.insert(idx.end(), per[t].begin(), per[t].end());
  };
  std::vector<int> so, si, ro, ri;
  build(*h->src_elem_h, so, si);
  build(*h->rec_elem_h, ro, ri);
  std::vector<int> tb(4 * (size_t)ntiles);
  for (int t = 0; t < ntiles; t++) {
    tb[4 * (size_t)t] = so[t]; tb[4 * (size_t)t + 1] = so[t + 1];
    tb[4 * (size_t)t + 2] = ro[t]; tb[4 * (size_t)t + 3] = ro[t + 1];
  }
  dfree(h, h->tile_src_off); dfree(h, h->tile_src_idx); dfree(h, h->tile_rec_off); dfree(h, h->tile_rec_idx);
  dfree(h, h->tile_bounds);
  h->tile_src_off = h->tile_src_idx = h->tile_rec_off = h->tile_rec_idx = nullptr;
  h->tile_bounds = nullptr;
  int rc;
  if ((rc = upload_i(h, (int **)&h->tile_bounds, tb.data(), tb.size()))) return rc;
  if ((rc = upload_i(h, &h->tile_src_off, so.data(), so.size()))) return rc;
  if ((rc = upload_i(h, &h->tile_src_idx, si.data(), si.size()))) return rc;
  if ((rc = upload_i(h, &h->tile_rec_off, ro.data(), ro.size()))) return rc;
  if ((rc = upload_i(h, &h->tile_rec_idx, ri.data(), ri.size()))) return rc;
  h->pconfig = config;
  h->pntx = ntx;
  h->pnty = nty;
  h->pgrid = std::min(ntiles, std::max(1, se2p::occupancy(P, config, mode)) * h->nsm);
  return 0;
}

extern "C" int se2gpu_create(const se2gpu_problem *P, int precision, int trace_capacity, se2gpu_solver **out)
{
  if (!out) return fail(nullptr, SE2GPU_ERR_ARG, "null output handle");
  *out = nullptr;
  if (!P) return fail(nullptr, SE2GPU_ERR_ARG, "null problem");
  if (precision != SE2GPU_FP64 && precision != SE2GPU_FP32 && precision != SE2GPU_FP32_KAHAN &&
      precision != SE2GPU_FP32_DF)
    return fail(nullptr, SE2GPU_ERR_ARG, "unknown precision %d (use 64, 34, 33 or 32)", precision);
  if (P->p < 1 || P->p > 8) return fail(nullptr, SE2GPU_ERR_ARG, "polynomial degree %d outside 1..8", P->p);
  if (P->mx < 1 || P->my < 1) return fail(nullptr, SE2GPU_ERR_ARG, "mx, my must be positive");
  const long nx_g = (long)P->p * P->mx + 1, ny_g = (long)P->p * P->my + 1;
  if (nx_g * ny_g * 2 >= 2147483647L) return fail(nullptr, SE2GPU_ERR_ARG, "mesh too large for 32-bit node indices");
  if (!(P->dt > 0.0) || !std::isfinite(P->dt)) return fail(nullptr, SE2GPU_ERR_ARG, "time step must be positive and finite");
  if (P->nsrc < 0 || P->nrec < 0 || trace_capacity < 0) return fail(nullptr, SE2GPU_ERR_ARG, "negative count");
  if (!P->D || !P->wq || !P->w1d || !P->J00 || !P->J11 || !P->iJ00 || !P->iJ11 || !P->lambda || !P->mu || !P->mass)
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
  // where the device reads pageable host memory, the FP32 modes check the mass in the
  // kernel that forms 1/M from it (no host pass over the array); elsewhere the host checks
  int dev0 = 0, pageable0 = 0;
  if (cudaGetDevice(&dev0) != cudaSuccess ||
      cudaDeviceGetAttribute(&pageable0, cudaDevAttrPageableMemoryAccess, dev0) != cudaSuccess) {
    cudaGetLastError();
    pageable0 = 0;
  }
  const bool mass_on_device = (precision != SE2GPU_FP64) && pageable0;
  if (!mass_on_device) {
    std::atomic<long> bad(LONG_MAX);   // the first node whose mass is not positive and finite
    host_parallel(nnodes, [&](long i0, long i1) {
      for (long i = i0; i < i1; i++)
        if (!(P->mass[i] > 0.0) || !std::isfinite(P->mass[i])) {
          long cur = bad.load();
          while (i < cur && !bad.compare_exchange_weak(cur, i)) {}
          break;
        }
    });
    if (bad.load() != LONG_MAX) return fail(nullptr, SE2GPU_ERR_ARG, "mass at node %ld is not positive", bad.load());
  }

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
  cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
  if (cudaDeviceGetAttribute(&h->pageable, cudaDevAttrPageableMemoryAccess, h->device) != cudaSuccess) {
    cudaGetLastError();
    h->pageable = 0;
  }
  {
    cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { free(h); return fail(nullptr, SE2GPU_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e)); }
    h->stream = h->own_stream;
  }
  {
    // the tiled kernels serve FP64 and the FP32 internal-force entry point
    cudaError_t e = (precision == SE2GPU_FP64) ? se2::prepare_f64(P->p) : se2::prepare_f32(P->p);
    if (e != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "kernel set-up: %s", cudaGetErrorString(e)); TRY(SE2GPU_ERR_CUDA); }
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
  TRY(dzero(h, (void **)&h->err_dev, sizeof(int)));

  if (precision == SE2GPU_FP64) {
    const size_t vbytes = (size_t)nnodes * 2 * 8;
    for (int b = 0; b < 2; b++)
      for (int f = 0; f < 3; f++) TRY(dzero(h, &h->f64[b][f], vbytes));
    TRY(upload(h, &h->mass, P->mass, (size_t)nnodes));   // the reference divides by M
  } else {
    const bool kahan = is_kahan(h), df = is_df(h);
    h->pitch = (int)((nx_g + 1 + 15) / 16 * 16);   // >= 1 padding node: paired reads stay in the row
    const size_t np = (size_t)ny_g * h->pitch;
    for (int b = 0; b < 2; b++) {
      TRY(dalloc(h, (void **)&h->pu[b], np * 8));
      TRY(dalloc(h, (void **)&h->pw[b], np * 8));
      if (kahan) { TRY(dalloc(h, (void **)&h->pcu[b], np * 8)); TRY(dalloc(h, (void **)&h->pcw[b], np * 8)); }
      TRY(dzero(h, (void **)&h->rbuf[b], (size_t)P->nrec * npe * rbuf_values(h) * 4));
    }
    TRY(dalloc(h, (void **)&h->pa, np * 8 * (df ? 2 : 1)));   // two-float mode: low parts after the high
    if (!df) {
      TRY(dalloc(h, (void **)&h->cellc, (size_t)ne * sizeof(float4)));
      k_cell_consts<<<(int)std::min<long>((ne + 255) / 256, 8L * h->nsm), 256, 0, h->stream>>>(
          (const float *)h->lam, (const float *)h->mu, (const float *)h->J00, (const float *)h->J11,
          (const float *)h->iJ00, (const float *)h->iJ11, h->mx, ne, h->cellc);
      if (cudaGetLastError() != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "cell constants"); TRY(SE2GPU_ERR_CUDA); }
    }
    // The fields start at zero: the first buffer set and a are cleared.  The second set is
    // written at every mesh node by the first step before anything reads it (the tile copies
    // never read past the mesh), so only its row padding is cleared, to keep checkpoints
    // deterministic.  The clearing and, on a device that reads pageable host memory, the 1/M
    // pass over the caller's mass (the longest part of the set-up: it runs at the host link's
    // rate) run on two side streams, beside the host's tile configuration below; the handle's
    // stream joins them after it, so the configuration's small uploads wait only for the cell
    // tables above.
    if (h->pageable) {
      TRY(dalloc(h, (void **)&h->pminv, np * 4 * (df ? 2 : 1)));
      TRY(dalloc(h, (void **)&h->mass_bad, sizeof(unsigned long long)));
    }
    {
      cudaStream_t side[2] = {nullptr, nullptr};
      cudaEvent_t ev0 = nullptr;
      cudaError_t e = cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming);
      for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        e = cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->side_done[i], cudaEventDisableTiming);
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev0, h->stream);   // the allocations above
      for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaStreamWaitEvent(side[i], ev0, 0);
      float2 *full[5] = {h->pu[0], h->pw[0], kahan ? h->pcu[0] : nullptr, kahan ? h->pcw[0] : nullptr, h->pa};
      for (int f = 0; f < 5 && e == cudaSuccess; f++)
        if (full[f]) e = cudaMemsetAsync(full[f], 0, np * 8 * ((f == 4 && df) ? 2 : 1), side[0]);
      float2 *pad[4] = {h->pu[1], h->pw[1], kahan ? h->pcu[1] : nullptr, kahan ? h->pcw[1] : nullptr};
      for (int f = 0; f < 4 && e == cudaSuccess; f++)
        if (pad[f]) e = cudaMemset2DAsync(pad[f] + nx_g, (size_t)h->pitch * 8, 0, (size_t)(h->pitch - nx_g) * 8, ny_g, side[0]);
      if (h->pageable && e == cudaSuccess) {
        // the device reads the mass where it lies (no staging copy of the whole array)
        e = cudaMemsetAsync(h->mass_bad, 0xff, sizeof(unsigned long long), side[1]);
        if (e == cudaSuccess) {
          k_minv_from_host<<<dim3((h->pitch + 1023) / 1024, (unsigned)std::min(ny_g, 65535L)), 256, 0, side[1]>>>(
              P->mass, nx_g, ny_g, h->pitch, h->pminv, df ? h->pminv + np : nullptr, h->mass_bad);
          e = cudaGetLastError();
        }
      }
      for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventRecord(h->side_done[i], side[i]);
      if (ev0) cudaEventDestroy(ev0);
      for (int i = 0; i < 2; i++)
        if (side[i]) cudaStreamDestroy(side[i]);   // released once its work is done
      if (e != cudaSuccess) {
        cudaGetLastError();
        fail(h, SE2GPU_ERR_CUDA, "clearing the state and 1/M: %s", cudaGetErrorString(e));
        TRY(SE2GPU_ERR_CUDA);
      }
    }
    {
      cudaError_t e = se2p::set_tables(P->p, P->D, P->w1d);
      if (e != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "constant tables: %s", cudaGetErrorString(e)); TRY(SE2GPU_ERR_CUDA); }
      h->src_elem_h = new std::vector<int>(P->src_elem, P->src_elem + P->nsrc);
      h->rec_elem_h = new std::vector<int>(P->rec_elem, P->rec_elem + P->nrec);
      TRY(setup_f32_config(h, df ? 0 : se2p::default_config(P->p), true));
    }
    for (cudaEvent_t &ev : h->side_done) {
      const cudaError_t e = cudaStreamWaitEvent(h->stream, ev, 0);
      cudaEventDestroy(ev);   // (the wait keeps what it needs)
      ev = nullptr;
      if (e != cudaSuccess) { cudaGetLastError(); fail(h, SE2GPU_ERR_CUDA, "joining the set-up streams"); TRY(SE2GPU_ERR_CUDA); }
    }
    if (!h->pageable) {
      // 1/M in the padded FP32 layout (padding nodes 0), row blocks on the host threads;
      // the two-float mode appends the remainders
      const size_t nm = np * (df ? 2 : 1);
      std::unique_ptr<float[]> minv(new float[nm]);
      const int pitch = h->pitch;
      host_parallel(ny_g, [&](long y0, long y1) {
        for (long y = y0; y < y1; y++) {
          float *row = minv.get() + (size_t)y * pitch;
          float *lo = df ? row + np : nullptr;
          const double *m = P->mass + y * nx_g;
          for (long x = 0; x < nx_g; x++) {
            const double r = 1.0 / m[x];
            row[x] = (float)r;
            if (lo) lo[x] = (float)(r - (double)row[x]);
          }
          for (long x = nx_g; x < pitch; x++) {
            row[x] = 0.f;
            if (lo) lo[x] = 0.f;
          }
        }
      });
      TRY(dalloc(h, (void **)&h->pminv, nm * 4));
      if (cudaMemcpyAsync(h->pminv, minv.get(), nm * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) { fail(h, SE2GPU_ERR_CUDA, "upload 1/M"); TRY(SE2GPU_ERR_CUDA); }
    }
    se2p::TileShape ts;
    if (se2p::config_shape(h->p, h->pconfig, pmode(h), &ts)) { fail(h, SE2GPU_ERR_ARG, "tile configuration"); TRY(SE2GPU_ERR_ARG); }
    TRY(make_const_maps(h, ts));
  }
  {
    // one wait for everything queued above (kernels that read the caller's arrays included),
    // then the device's mass check
    unsigned long long bad = ~0ULL;
    cudaError_t e = h->mass_bad ? cudaMemcpyAsync(&bad, h->mass_bad, sizeof(bad), cudaMemcpyDeviceToHost, h->stream)
                                : cudaSuccess;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(h, SE2GPU_ERR_CUDA, "set-up: %s", cudaGetErrorString(e));
      TRY(SE2GPU_ERR_CUDA);
    }
    if (bad != ~0ULL) {
      fail(h, SE2GPU_ERR_ARG, "mass at node %ld is not positive", (long)bad);
      TRY(SE2GPU_ERR_ARG);
    }
  }
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

static int check_err_flag(se2gpu_solver *h)
{
  int flag = 0;
  CK(h, cudaMemcpyAsync(&flag, h->err_dev, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  if (flag) return fail(h, SE2GPU_ERR_CUDA, "a step kernel gave up waiting for its tile copies (bounded wait expired)");
  return 0;
}

extern "C" int se2gpu_synchronize(se2gpu_solver *h)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaStreamSynchronize(h->stream));
  return check_err_flag(h);
}

extern "C" int se2gpu_selftest_wait_expiry(se2gpu_solver *h, double *seconds)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaStreamSynchronize(h->stream));
  unsigned long long *ns_dev = nullptr, ns = 0;
  CK(h, cudaMalloc((void **)&ns_dev, sizeof(ns)));
  cudaError_t e = se2p::launch_wait_expiry_test(h->err_dev, ns_dev, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = cudaMemcpy(&ns, ns_dev, sizeof(ns), cudaMemcpyDeviceToHost);
  cudaFree(ns_dev);
  CK(h, e);
  if (seconds) *seconds = 1e-9 * (double)ns;
  return check_err_flag(h);
}

// ---------------------------------------------------------------- FP64 (tiled, reference order)
static se2::StepParams<double> f64_params(se2gpu_solver *h)
{
  se2::StepParams<double> prm;
  memset(&prm, 0, sizeof(prm));
  prm.mx = h->mx; prm.my = h->my; prm.nx_g = h->nx_g; prm.ny_g = h->ny_g;
  prm.ntx = h->ntx; prm.nty = h->nty;
  prm.mass = (const double *)h->mass; prm.lam = (const double *)h->lam; prm.mu = (const double *)h->mu;
  prm.J00 = (const double *)h->J00; prm.J11 = (const double *)h->J11;
  prm.iJ00 = (const double *)h->iJ00; prm.iJ11 = (const double *)h->iJ11;
  prm.D = (const double *)h->D; prm.wq = (const double *)h->wq;
  // coefficients exactly as the reference forms them: dt, 0.5*dt*dt, 0.5*dt
  prm.c_dt = h->dt; prm.c_u = 0.5 * h->dt * h->dt; prm.c_v = 0.5 * h->dt;
  prm.nsrc = h->nsrc; prm.src_elem = h->src_elem; prm.src_vals = (const double *)h->src_vals;
  prm.nrec = h->nrec; prm.rec_node = h->rec_node; prm.rec_elem = h->rec_elem; prm.rec_gll = h->rec_gll;
  prm.Dd = h->Dd; prm.iJ00d = h->iJ00d; prm.iJ11d = h->iJ11d;
  return prm;
}

static void f64_bind(se2gpu_solver *h, se2::StepParams<double> &prm, int in, int outb)
{
  prm.u_in = (const double2 *)h->f64[in][0]; prm.v_in = (const double2 *)h->f64[in][1]; prm.a_in = (const double2 *)h->f64[in][2];
  prm.u_out = (double2 *)h->f64[outb][0]; prm.v_out = (double2 *)h->f64[outb][1]; prm.a_out = (double2 *)h->f64[outb][2];
}

// ---------------------------------------------------------------- FP32 (persistent leapfrog)
static se2p::Params f32_params(se2gpu_solver *h)
{
  se2p::Params prm;
  memset(&prm, 0, sizeof(prm));
  prm.mx = h->mx; prm.my = h->my; prm.nx_g = h->nx_g; prm.ny_g = h->ny_g; prm.pitch = h->pitch;
  prm.ntx = h->pntx; prm.nty = h->pnty; prm.ntiles = h->pntx * h->pnty;
  prm.minv = h->pminv;
  prm.lam = (const float *)h->lam; prm.mu = (const float *)h->mu;
  prm.J00 = (const float *)h->J00; prm.J11 = (const float *)h->J11;
  prm.iJ00 = (const float *)h->iJ00; prm.iJ11 = (const float *)h->iJ11;
  prm.dt = (float)h->dt; prm.half_dt = (float)(0.5 * h->dt);
  prm.dt_lo = (float)(h->dt - (double)prm.dt); prm.half_dt_lo = (float)(0.5 * h->dt - (double)prm.half_dt);
  prm.nsrc = h->nsrc; prm.src_elem = h->src_elem; prm.src_vals = (const float *)h->src_vals;
  prm.nrec = h->nrec; prm.rec_elem = h->rec_elem; prm.rec_gll = h->rec_gll;
  prm.Dd = h->Dd; prm.iJ00d = h->iJ00d; prm.iJ11d = h->iJ11d;
  prm.err = h->err_dev;
  prm.tile_src_off = h->tile_src_off; prm.tile_src_idx = h->tile_src_idx;
  prm.tile_rec_off = h->tile_rec_off; prm.tile_rec_idx = h->tile_rec_idx;
  prm.cellc = h->cellc; prm.tile_bounds = h->tile_bounds;
  return prm;
}

se2p::Params se2gpu_internal_f32_params(se2gpu_solver *h) { return f32_params(h); }

// record the receivers of the last step if its row is still pending
static int flush_record(se2gpu_solver *h)
{
  if (!h->pending_record) return 0;
  cudaError_t e;
  h->launches++;
  double *row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
  if (is_f64(h)) {
    auto prm = f64_params(h);
    f64_bind(h, prm, h->cur, h->cur);
    prm.record = 1;
    prm.trace_row = row;
    e = se2::launch_record_f64(h->p, prm, h->stream);
  } else {
    auto prm = f32_params(h);
    prm.rbuf_in = h->rbuf[h->rlast];
    prm.record = 1;
    prm.trace_row = row;
    e = se2p::launch_record(h->p, prm, h->stream, is_df(h));
  }
  if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "receiver kernel: %s", cudaGetErrorString(e));
  h->rows_written++;
  h->pending_record = false;
  return 0;
}

static int advance_f64(se2gpu_solver *h, int nsteps)
{
  auto prm = f64_params(h);
  prm.mode = 0;
  for (int k = 0; k < nsteps; k++) {
    f64_bind(h, prm, h->cur, 1 - h->cur);
    prm.stf = h->stf_dev + (size_t)k * h->nsrc;
    prm.record = h->pending_record ? 1 : 0;
    prm.trace_row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
    h->launches++;
    cudaError_t e = se2::launch_step_f64(h->p, prm, h->nblocks, h->stream);
    if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "step kernel: %s", cudaGetErrorString(e));
    if (h->pending_record) { h->rows_written++; h->pending_record = false; }
    h->cur = 1 - h->cur;
    if (h->nrec > 0) h->pending_record = true;
  }
  return 0;
}

static int advance_f32(se2gpu_solver *h, int nsteps)
{
  auto prm = f32_params(h);
  const int mode = pmode(h);
  for (int k = 0; k < nsteps; k++) {
    const int in = h->cur, outb = 1 - h->cur;
    prm.u_out = h->pu[outb]; prm.w_out = h->pw[outb]; prm.cu_out = h->pcu[outb]; prm.cw_out = h->pcw[outb];
    prm.a_out = (k == nsteps - 1) ? h->pa : nullptr;
    prm.stf = h->stf_dev + (size_t)k * h->nsrc;
    prm.rbuf_in = h->rbuf[h->rlast];
    prm.rbuf_out = h->rbuf[1 - h->rlast];
    prm.record = h->pending_record ? 1 : 0;
    prm.trace_row = h->traces + (size_t)h->rows_written * 7 * h->nrec;
    h->launches++;
    cudaError_t e = se2p::launch_step(h->p, h->pconfig, mode, h->maps[in], prm, h->pgrid, h->stream);
    if (e != cudaSuccess) return fail(h, SE2GPU_ERR_CUDA, "step kernel: %s", cudaGetErrorString(e));
    if (h->pending_record) { h->rows_written++; h->pending_record = false; }
    h->cur = outb;
    h->rlast = 1 - h->rlast;
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
      dfree(h, h->stf_dev);
      h->stf_dev = nullptr;
      int rc = dalloc(h, (void **)&h->stf_dev, (size_t)nsteps * h->nsrc * 8);
      if (rc) { h->stf_cap = 0; return rc; }
      h->stf_cap = nsteps;
    }
    // the previous block may still read stf_dev: order the copy on the stream
    CK(h, cudaMemcpyAsync(h->stf_dev, stf, (size_t)nsteps * h->nsrc * 8, cudaMemcpyHostToDevice, h->stream));
  }
  return is_f64(h) ? advance_f64(h, nsteps) : advance_f32(h, nsteps);
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
  if ((rc = check_err_flag(h))) return rc;
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
  if (is_f64(h)) {
    const double *src[3] = {u, v, a};
    for (int f = 0; f < 3; f++)
      if (src[f] && (rc = copy_f64(h, (double *)h->f64[h->cur][f], src[f], n, cudaMemcpyHostToDevice))) return rc;
    return 0;
  }
  // FP32: unspecified fields keep their current values
  if (!u || !v || !a) {
    std::vector<double> cu(n), cv(n), ca(n);
    if ((rc = se2gpu_get_fields(h, cu.data(), cv.data(), ca.data()))) return rc;
    return upload_leapfrog(h, u ? u : cu.data(), v ? v : cv.data(), a ? a : ca.data());
  }
  return upload_leapfrog(h, u, v, a);
}

extern "C" int se2gpu_get_fields(se2gpu_solver *h, double *u, double *v, double *a)
{
  if (!h) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  CK(h, cudaStreamSynchronize(h->stream));
  int rc;
  if ((rc = check_err_flag(h))) return rc;
  const size_t n = (size_t)h->nnodes * 2;
  if (is_f64(h)) {
    double *dst[3] = {u, v, a};
    for (int f = 0; f < 3; f++)
      if (dst[f] && (rc = copy_f64(h, dst[f], (const double *)h->f64[h->cur][f], n, cudaMemcpyDeviceToHost))) return rc;
    return 0;
  }
  if (h->pageable) {
    const int c = h->cur;
    const bool kahan = is_kahan(h);
    prefault_output(u, n);
    prefault_output(v, n);
    prefault_output(a, n);
    k_fields_to_host<<<4 * h->nsm, 256, 0, h->stream>>>(h->pu[c], h->pw[c], kahan ? h->pcu[c] : nullptr,
                                                        kahan ? h->pcw[c] : nullptr, h->pa, pa_lo(h), h->nx_g, h->ny_g, h->pitch,
                                                        h->dt, 0.5 * h->dt, u, v, a);
    CK(h, cudaGetLastError());
    CK(h, cudaStreamSynchronize(h->stream));
    return 0;
  }
  const size_t np = (size_t)h->ny_g * h->pitch;
  std::vector<float2> U(np), W(np), CU(np, make_float2(0.f, 0.f)), CW(np, make_float2(0.f, 0.f)), A(np),
      AL(np, make_float2(0.f, 0.f));
  const int c = h->cur;
  CK(h, cudaMemcpyAsync(U.data(), h->pu[c], np * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaMemcpyAsync(W.data(), h->pw[c], np * 8, cudaMemcpyDeviceToHost, h->stream));
  if (is_kahan(h)) {
    CK(h, cudaMemcpyAsync(CU.data(), h->pcu[c], np * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(CW.data(), h->pcw[c], np * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(h, cudaMemcpyAsync(A.data(), h->pa, np * 8, cudaMemcpyDeviceToHost, h->stream));
  if (pa_lo(h)) CK(h, cudaMemcpyAsync(AL.data(), pa_lo(h), np * 8, cudaMemcpyDeviceToHost, h->stream));
  const double dt = h->dt, hdt = 0.5 * h->dt;
  for (long y = 0; y < h->ny_g; y++)
    for (long x = 0; x < h->nx_g; x++) {
      const size_t nn = (size_t)(y * h->nx_g + x), k = (size_t)(y * h->pitch + x);
      const double w0 = (double)W[k].x - (double)CW[k].x, w1 = (double)W[k].y - (double)CW[k].y;
      const double u0 = (double)U[k].x - (double)CU[k].x, u1 = (double)U[k].y - (double)CU[k].y;
      if (u) { u[2 * nn] = u0 - dt * w0; u[2 * nn + 1] = u1 - dt * w1; }
      const double a0 = (double)A[k].x + (double)AL[k].x, a1 = (double)A[k].y + (double)AL[k].y;
      if (v) { v[2 * nn] = w0 - hdt * a0; v[2 * nn + 1] = w1 - hdt * a1; }
      if (a) { a[2 * nn] = a0; a[2 * nn + 1] = a1; }
    }
  return 0;
}

extern "C" int se2gpu_norms(se2gpu_solver *h, double out[6])
{
  if (!h || !out) return SE2GPU_ERR_ARG;
  CK(h, cudaSetDevice(h->device));
  const int nb = 1024;
  h->launches++;
  if (is_f64(h)) {
    se2::norms_partial<double><<<nb, 256, 0, h->stream>>>((const double *)h->f64[h->cur][0], (const double *)h->f64[h->cur][1],
                                                          h->nnodes * 2, h->norm_part);
    CK(h, cudaGetLastError());
  } else {
    CK(h, se2p::launch_norms(h->pu[h->cur], h->pw[h->cur], is_kahan(h) ? h->pcu[h->cur] : nullptr,
                             is_kahan(h) ? h->pcw[h->cur] : nullptr, h->pa, pa_lo(h), h->nx_g, h->ny_g, h->pitch, h->dt,
                             h->norm_part, nb, h->stream));
  }
  std::vector<double> part(6 * nb);
  CK(h, cudaMemcpyAsync(part.data(), h->norm_part, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  int rc;
  if ((rc = check_err_flag(h))) return rc;
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

// ---------------------------------------------------------------- internal force (packed layout)
template <typename T>
static int force_t(se2gpu_solver *h, const void *u_dev, void *F_dev)
{
  typedef typename se2::Vec2<T>::type T2;
  se2::StepParams<T> prm;
  memset(&prm, 0, sizeof(prm));
  prm.mx = h->mx; prm.my = h->my; prm.nx_g = h->nx_g; prm.ny_g = h->ny_g; prm.ntx = h->ntx; prm.nty = h->nty;
  prm.lam = (const T *)h->lam; prm.mu = (const T *)h->mu; prm.J00 = (const T *)h->J00; prm.J11 = (const T *)h->J11;
  prm.iJ00 = (const T *)h->iJ00; prm.iJ11 = (const T *)h->iJ11; prm.D = (const T *)h->D; prm.wq = (const T *)h->wq;
  prm.mode = 1;
  prm.u_in = (const T2 *)u_dev;
  prm.f_out = (T2 *)F_dev;
  h->launches++;
  cudaError_t e;
  if constexpr (sizeof(T) == 8) e = se2::launch_step_f64(h->p, prm, h->nblocks - 1, h->stream);
  else e = se2::launch_step_f32(h->p, prm, h->nblocks - 1, h->stream);
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
    CK(h, cudaMemcpyAsync(h->scratch_u, u, n * 8, cudaMemcpyHostToDevice, h->stream));
  } else {
    std::vector<float> tmp(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (float)u[i];
    CK(h, cudaMemcpyAsync(h->scratch_u, tmp.data(), n * 4, cudaMemcpyHostToDevice, h->stream));
  }
  if ((rc = se2gpu_assemble_linear_form_device(h, h->scratch_u, h->scratch_f))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  if (h->tsize == 8) {
    CK(h, cudaMemcpyAsync(F, h->scratch_f, n * 8, cudaMemcpyDeviceToHost, h->stream));
  } else {
    std::vector<float> tmp(n);
    CK(h, cudaMemcpyAsync(tmp.data(), h->scratch_f, n * 4, cudaMemcpyDeviceToHost, h->stream));
    for (size_t i = 0; i < n; i++) F[i] = (double)tmp[i];
  }
  return 0;
}

extern "C" int se2gpu_info(const se2gpu_solver *h, long *ints)
{
  if (!h || !ints) return SE2GPU_ERR_ARG;
  ints[0] = h->nx_g; ints[1] = h->ny_g; ints[2] = h->p; ints[3] = h->precision;
  ints[4] = h->nsrc; ints[5] = h->nrec; ints[6] = h->launches; ints[7] = h->rows_written + (h->pending_record ? 1 : 0);
  ints[8] = is_f64(h) ? h->nx_g : h->pitch;
  return 0;
}

extern "C" int se2gpu_device_fields(const se2gpu_solver *h, void **u, void **v, void **a)
{
  if (!h) return SE2GPU_ERR_ARG;
  if (is_f64(h)) {
    if (u) *u = h->f64[h->cur][0];
    if (v) *v = h->f64[h->cur][1];
    if (a) *a = h->f64[h->cur][2];
  } else {
    if (u) *u = h->pu[h->cur];
    if (v) *v = h->pw[h->cur];
    if (a) *a = h->pa;
  }
  return 0;
}

extern "C" int se2gpu_tile_configs(const se2gpu_solver *h, int *edge, int *threads, int max_configs)
{
  if (!h) return SE2GPU_ERR_ARG;
  if (is_f64(h)) {
    if (max_configs > 0 && edge && threads) { edge[0] = se2::tile_edge(h->p); threads[0] = 256; }
    return 1;
  }
  const int n = se2p::num_configs(h->p);
  for (int c = 0; c < n && c < max_configs; c++) {
    se2p::TileShape ts;
    se2p::config_shape(h->p, c, pmode(h), &ts);
    if (edge) edge[c] = ts.tex;
    if (threads) threads[c] = ts.nt;
  }
  return n;
}

extern "C" int se2gpu_tile_config_info(const se2gpu_solver *h, int config, int info[4])
{
  if (!h || !info) return SE2GPU_ERR_ARG;
  if (is_f64(h)) {
    if (config != 0) return SE2GPU_ERR_ARG;
    info[0] = se2::tile_edge(h->p); info[1] = 256; info[2] = 0; info[3] = 0;
    return 0;
  }
  se2p::TileShape ts;
  if (config < 0 || se2p::config_shape(h->p, config, pmode(h), &ts)) return SE2GPU_ERR_ARG;
  info[0] = ts.tex; info[1] = ts.nt; info[2] = ts.owned_buffers;
  // the occupancy query needs the kernel's dynamic shared-memory limit raised first
  if (cudaSetDevice(h->device) != cudaSuccess || se2p::prepare(h->p, config, pmode(h)) != cudaSuccess) {
    cudaGetLastError();
    return SE2GPU_ERR_CUDA;
  }
  info[3] = se2p::occupancy(h->p, config, pmode(h), false);
  return 0;
}

extern "C" int se2gpu_tile_config(const se2gpu_solver *h)
{
  if (!h) return SE2GPU_ERR_ARG;
  return is_f64(h) ? 0 : h->pconfig;
}

extern "C" int se2gpu_set_tile_config(se2gpu_solver *h, int config)
{
  if (!h) return SE2GPU_ERR_ARG;
  if (is_f64(h)) return (config == 0) ? 0 : fail(h, SE2GPU_ERR_ARG, "FP64 mode has a single tile configuration");
  if (config < 0 || config >= se2p::num_configs(h->p)) return fail(h, SE2GPU_ERR_ARG, "tile configuration %d out of range", config);
  CK(h, cudaSetDevice(h->device));
  if (config == h->pconfig) return 0;   // already selected: tables, maps and grid are current
  return setup_f32_config(h, config);
}

// ---------------------------------------------------------------- checkpoint / resume
namespace {
struct CkptHeader {
  char magic[8];               // "SE2CKPT1"
  int precision, mx, my, p, nrec, pitch;
  int pending_record, rlast;
  long nnodes;
};

// the device arrays of the evolving state, in checkpoint order
std::vector<std::pair<void *, size_t>> state_arrays(se2gpu_solver *h)
{
  std::vector<std::pair<void *, size_t>> v;
  if (is_f64(h)) {
    const size_t b = (size_t)h->nnodes * 2 * 8;
    for (int f = 0; f < 3; f++) v.push_back({h->f64[h->cur][f], b});
  } else {
    const size_t b = (size_t)h->ny_g * h->pitch * 8;
    v.push_back({h->pu[h->cur], b});
    v.push_back({h->pw[h->cur], b});
    if (is_kahan(h)) { v.push_back({h->pcu[h->cur], b}); v.push_back({h->pcw[h->cur], b}); }
    v.push_back({h->pa, b * (is_df(h) ? 2 : 1)});
    if (h->nrec) v.push_back({h->rbuf[h->rlast], (size_t)h->nrec * h->npe * rbuf_values(h) * 4});
  }
  return v;
}
}  // namespace

extern "C" long se2gpu_checkpoint_size(const se2gpu_solver *h)
{
  if (!h) return SE2GPU_ERR_ARG;
  long n = (long)sizeof(CkptHeader);
  for (auto &a : state_arrays(const_cast<se2gpu_solver *>(h))) n += (long)a.second;
  return n;
}

extern "C" int se2gpu_checkpoint_save(se2gpu_solver *h, void *buf, long bytes)
{
  if (!h || !buf) return SE2GPU_ERR_ARG;
  if (bytes < se2gpu_checkpoint_size(h)) return fail(h, SE2GPU_ERR_ARG, "checkpoint buffer of %ld bytes, %ld needed", bytes, se2gpu_checkpoint_size(h));
  if (h->rows_written > 0) return fail(h, SE2GPU_ERR_STATE, "%d trace rows are buffered; fetch them with se2gpu_traces before saving", h->rows_written);
  CK(h, cudaSetDevice(h->device));
  CK(h, cudaStreamSynchronize(h->stream));
  int rc;
  if ((rc = check_err_flag(h))) return rc;
  CkptHeader hd;
  memset(&hd, 0, sizeof(hd));
  memcpy(hd.magic, "SE2CKPT1", 8);
  hd.precision = h->precision; hd.mx = h->mx; hd.my = h->my; hd.p = h->p; hd.nrec = h->nrec; hd.pitch = h->pitch;
  hd.pending_record = h->pending_record ? 1 : 0; hd.rlast = h->rlast; hd.nnodes = h->nnodes;
  char *o = static_cast<char *>(buf);
  memcpy(o, &hd, sizeof(hd));
  o += sizeof(hd);
  for (auto &a : state_arrays(h)) {
    CK(h, cudaMemcpyAsync(o, a.first, a.second, cudaMemcpyDeviceToHost, h->stream));
    o += a.second;
  }
  return 0;
}

extern "C" int se2gpu_checkpoint_load(se2gpu_solver *h, const void *buf, long bytes)
{
  if (!h || !buf) return SE2GPU_ERR_ARG;
  if (bytes < (long)sizeof(CkptHeader)) return fail(h, SE2GPU_ERR_ARG, "checkpoint too short");
  CkptHeader hd;
  memcpy(&hd, buf, sizeof(hd));
  if (memcmp(hd.magic, "SE2CKPT1", 8) != 0) return fail(h, SE2GPU_ERR_ARG, "not a checkpoint");
  if (hd.precision != h->precision || hd.mx != h->mx || hd.my != h->my || hd.p != h->p || hd.nrec != h->nrec ||
      hd.pitch != h->pitch || hd.nnodes != h->nnodes)
    return fail(h, SE2GPU_ERR_ARG, "checkpoint of another problem or precision (%dx%d p%d precision %d)", hd.mx, hd.my, hd.p, hd.precision);
  // the size does not depend on the state switched below: reject a truncated buffer
  // before the handle is touched
  if (bytes < se2gpu_checkpoint_size(h)) return fail(h, SE2GPU_ERR_ARG, "checkpoint truncated");
  CK(h, cudaSetDevice(h->device));
  CK(h, cudaStreamSynchronize(h->stream));
  h->rows_written = 0;
  h->pending_record = hd.pending_record != 0;
  if (!is_f64(h)) h->rlast = hd.rlast & 1;
  const char *o = static_cast<const char *>(buf) + sizeof(hd);
  for (auto &a : state_arrays(h)) {
    CK(h, cudaMemcpyAsync(a.first, o, a.second, cudaMemcpyHostToDevice, h->stream));
    o += a.second;
  }
  return 0;
}
