// se2gpu_peaks.cu -- arithmetic-pipe peaks of the current GPU, measured with CUDA events,
// as roofline denominators for the kernels that are not bound by HBM: the FP64 step
// kernel (reference operation order: separately rounded multiplies and adds, no fused
// multiply-add) and the two-float FP32 step kernel (FP32 adds, multiplies and fused
// multiply-adds).  No counterpart in the reference.
//
// Each thread runs 8 independent dependency chains of the measured operation pair for
// a fixed number of iterations; the grid holds 4 CTAs of 256 threads per SM, so every
// scheduler has several warps with independent work.  The result is the number of
// arithmetic instructions per second (a multiply and an add count as two).
#include <cuda_runtime.h>

#include <cstdio>

#include "se2gpu.h"
#include "se2gpu_internal.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

// kind 0: FP64 __dmul_rn + __dadd_rn; 1: FP64 fma; 2: FP32 __fmul_rn + __fadd_rn; 3: FP32 fmaf
template <int KIND>
__global__ void __launch_bounds__(kThreads) pipe_loop(int iters, double seed, double *sink)
{
  double d[kChains];
  float f[kChains];
  const double x = 1.0 + 1e-9 * threadIdx.x, y = seed;
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    d[c] = seed + c;
    f[c] = (float)(seed + c);
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      if (KIND == 0) d[c] = __dadd_rn(__dmul_rn(d[c], x), y);
      if (KIND == 1) d[c] = __fma_rn(d[c], x, y);
      if (KIND == 2) f[c] = __fadd_rn(__fmul_rn(f[c], (float)x), (float)y);
      if (KIND == 3) f[c] = __fmaf_rn(f[c], (float)x, (float)y);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += (KIND < 2) ? d[c] : (double)f[c];
  if (s == 1.2345e300) sink[0] = s;   // keeps the chains live; never true for these inputs
}

template <int KIND>
cudaError_t launch(int blocks, int iters, double *sink, cudaStream_t st)
{
  pipe_loop<KIND><<<blocks, kThreads, 0, st>>>(iters, 1e-3, sink);
  return cudaGetLastError();
}

}  // namespace

extern "C" int se2gpu_pipe_peak(int kind, double *ops_per_second)
{
  if (!ops_per_second || kind < 0 || kind > 3) return SE2GPU_ERR_ARG;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return SE2GPU_ERR_CUDA;
  }
  const int blocks = 4 * nsm;
  const int iters = (kind < 2) ? 2048 : 65536;   // FP64 runs at a small fraction of the FP32 rate
  double *sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&sink, sizeof(double));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best_ms = 0.f;
  auto run = [&](void) -> cudaError_t {
    switch (kind) {
      case 0: return launch<0>(blocks, iters, sink, st);
      case 1: return launch<1>(blocks, iters, sink, st);
      case 2: return launch<2>(blocks, iters, sink, st);
      default: return launch<3>(blocks, iters, sink, st);
    }
  };
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {   // first repetition: warm-up
    e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) e = run();
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best_ms == 0.f || ms < best_ms)) best_ms = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess || best_ms <= 0.f) {
    char msg[256];
    snprintf(msg, sizeof(msg), "pipe peak: %s", cudaGetErrorString(e));
    se2gpu_internal_set_error(msg);
    return SE2GPU_ERR_CUDA;
  }
  const double ops = 2.0 * kChains * (double)iters * kThreads * blocks;   // two instructions per chain step (or one fma = 2 flops)
  *ops_per_second = ops / (1e-3 * best_ms);
  return 0;
}
