// se2gpu_noalloc.cu -- se2gpu_norms_device_noalloc: the log norms of se2gpu_norms
// (VecMax / VecMin / VecNorm NORM_2 of u and v) on caller-owned FP64 device
// vectors, computed without allocating device memory.
//
// The per-block partials live in a file-scope static __device__ array of fixed
// size (SE2GPU_NOALLOC_MAX_BLOCKS blocks of SE2GPU_NOALLOC_CHUNK values each), so
// the largest accepted vector has SE2GPU_NOALLOC_MAX_VALUES values; longer ones
// are rejected.  Its address is looked up once per device with
// cudaGetSymbolAddress (with that device current).  One launch: every block
// reduces its fixed chunk in a fixed order and writes its partial; the last
// block to finish (a ticket counter, cleared with cudaMemsetAsync before each
// launch) reduces the partials in block order.  The result is therefore
// independent of scheduling.  All calls share the one scratch array per device,
// so calls that overlap in time (other streams or threads) race.  The looked-up
// address is kept for the life of the process: it assumes the device is not
// reset (cudaDeviceReset) while the library is loaded.  As se2gpu_norms does, a
// non-finite l2 norm (a NaN or Inf anywhere in u or v) fails the call with
// SE2GPU_ERR_NUMERIC: fmax/fmin skip NaN, so max and min alone could look finite.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "se2gpu.h"
#include "se2gpu_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr long kChunk = SE2GPU_NOALLOC_CHUNK;
constexpr int kMaxBlocks = SE2GPU_NOALLOC_MAX_BLOCKS;

// partials [kMaxBlocks][6], result [6], ticket (+ padding)
struct Scratch {
  double partial[kMaxBlocks * 6];
  double result[8];
  unsigned int ticket;
};

static __device__ __align__(256) Scratch g_scratch;

int fail(int code, const char *msg)
{
  se2gpu_internal_set_error(msg);   // read back with se2gpu_last_error(NULL)
  return code;
}

__device__ __forceinline__ void combine(double *a, const double *b)
{
  a[0] = fmax(a[0], b[0]); a[1] = fmin(a[1], b[1]); a[2] += b[2];
  a[3] = fmax(a[3], b[3]); a[4] = fmin(a[4], b[4]); a[5] += b[5];
}

// shared-memory tree over the block's threads (fixed order); result in s[0..5][0]
__device__ void block_reduce(double (*s)[kThreads], double *r)
{
  for (int c = 0; c < 6; c++) s[c][threadIdx.x] = r[c];
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      const int t = threadIdx.x;
      s[0][t] = fmax(s[0][t], s[0][t + h]); s[1][t] = fmin(s[1][t], s[1][t + h]); s[2][t] += s[2][t + h];
      s[3][t] = fmax(s[3][t], s[3][t + h]); s[4][t] = fmin(s[4][t], s[4][t + h]); s[5][t] += s[5][t + h];
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) norms_noalloc(const double *u, const double *v, long n, Scratch *sc)
{
  __shared__ double s[6][kThreads];
  __shared__ bool last;
  double r[6] = {-1.0e308, 1.0e308, 0.0, -1.0e308, 1.0e308, 0.0};
  const long b0 = (long)blockIdx.x * kChunk, b1 = (b0 + kChunk < n) ? b0 + kChunk : n;
  for (long i = b0 + threadIdx.x; i < b1; i += kThreads) {
    const double x = u[i], y = v[i];
    r[0] = fmax(r[0], x); r[1] = fmin(r[1], x); r[2] += x * x;
    r[3] = fmax(r[3], y); r[4] = fmin(r[4], y); r[5] += y * y;
  }
  block_reduce(s, r);
  if (threadIdx.x < 6) sc->partial[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(&sc->ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block: partials in block order, thread t takes blocks t, t + 256, ...
  double q[6] = {-1.0e308, 1.0e308, 0.0, -1.0e308, 1.0e308, 0.0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) {
    double p[6];
    for (int c = 0; c < 6; c++) p[c] = __ldcg(&sc->partial[b * 6 + c]);
    combine(q, p);
  }
  block_reduce(s, q);
  if (threadIdx.x < 6) {
    const double x = s[threadIdx.x][0];
    sc->result[threadIdx.x] = (threadIdx.x == 2 || threadIdx.x == 5) ? sqrt(x) : x;
  }
}

// address of this device's scratch, looked up once per device
std::mutex g_mu;
Scratch *g_addr[64];

int scratch_address(Scratch **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(SE2GPU_ERR_CUDA, "no CUDA device");
  }
  if (dev < 0 || dev >= 64) return fail(SE2GPU_ERR_CUDA, "device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      char msg[256];
      snprintf(msg, sizeof(msg), "cudaGetSymbolAddress of the norms scratch: %s", cudaGetErrorString(e));
      return fail(SE2GPU_ERR_CUDA, msg);
    }
    g_addr[dev] = static_cast<Scratch *>(p);
  }
  *out = g_addr[dev];
  return 0;
}

}  // namespace

extern "C" int se2gpu_norms_device_noalloc(const double *u_dev, const double *v_dev, long n, void *stream,
                                           double out[6])
{
  if (!u_dev || !v_dev || !out) return fail(SE2GPU_ERR_ARG, "null argument");
  if (n < 1) return fail(SE2GPU_ERR_ARG, "vector length must be at least 1");
  if (n > SE2GPU_NOALLOC_MAX_VALUES) {
    char msg[256];
    snprintf(msg, sizeof(msg), "vector of %ld values exceeds the scratch limit of %ld values (%d blocks of %ld)", n,
             (long)SE2GPU_NOALLOC_MAX_VALUES, kMaxBlocks, kChunk);
    return fail(SE2GPU_ERR_ARG, msg);
  }
  Scratch *sc = nullptr;
  int rc = scratch_address(&sc);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = (int)((n + kChunk - 1) / kChunk);
  // a non-sticky error left by an earlier, unrelated call of the caller's is not this
  // call's: clear it so that the launch check below reports this launch alone
  (void)cudaGetLastError();
  cudaError_t e = cudaMemsetAsync(&sc->ticket, 0, sizeof(unsigned int), st);   // the ticket must start at zero
  if (e == cudaSuccess) {
    norms_noalloc<<<nb, kThreads, 0, st>>>(u_dev, v_dev, n, sc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, sc->result, 6 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    char msg[256];
    snprintf(msg, sizeof(msg), "norms (no allocation): %s", cudaGetErrorString(e));
    return fail(SE2GPU_ERR_CUDA, msg);
  }
  if (!std::isfinite(out[2]) || !std::isfinite(out[5])) {
    char msg[256];
    snprintf(msg, sizeof(msg), "non-finite field norm (u l2 = %g, v l2 = %g)", out[2], out[5]);
    return fail(SE2GPU_ERR_NUMERIC, msg);
  }
  return 0;
}
