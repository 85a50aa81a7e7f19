// se2nn_tc.cuh -- the surrogate network's row GEMMs on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for sm_103a.
//
//   C = act(alpha * A op(B) + beta * Cin + bias)      A: M x K row-major (k contiguous)
//
// Used where the shape allows (se2nn.cu, tc_eligible): one batch, M rows of activations
// (pixels or decoder rows), K and N multiples of 16 with K <= 128, 16 <= N <= 128 --
// the lift, the 1x1 convolutions, the decoder and their data-gradient GEMMs.  The same
// epilogue as gemm_bf16 (scale, in-place accumulation, bias, pre-activation store,
// GELU, FP32 or BF16 output).
//
// One CTA of 256 threads per work unit of 128 rows, persistent over the row tiles:
//  * op(B) (the layer's weights, N x K) is staged once per CTA in shared memory in the
//    canonical K-major layout without swizzle: 8 x 8 core matrices of 128 bytes, the
//    core matrix (row group g, k chunk c) at byte ((g * K/8) + c) * 128;
//  * the A tiles (128 x K) are copied with 16-byte cp.async into the same layout, two
//    stages;
//  * one thread issues K/16 tcgen05.mma (M = 128, N, K = 16, BF16 in, FP32 accumulate)
//    per tile and commits them to the mbarrier of one of two tensor-memory accumulators;
//    shared-memory descriptors: start address, leading byte offset 128 (the next k
//    chunk), stride byte offset K/8 * 128 (the next row group).  The next tile's MMAs
//    run while the current tile's epilogue reads the other accumulator;
//  * eight warps read the accumulator, two per 32 lanes (rows), with tcgen05.ld
//    32x32b.x32, alternate 32-column chunks each, and turn them through a per-warp
//    shared-memory patch so that the epilogue's loads and stores run along rows (4
//    consecutive columns per lane, whole 128-byte row segments per chunk).
// Every mbarrier wait is bounded: on expiry the kernel raises *err, waits (bounded) for
// its own tensor-core operations, frees its tensor memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "se2nn_gemm.cuh"

namespace nnk {

constexpr int TC_M = 128, TC_THREADS = 256, TC_KMAX = 128, TC_NMAX = 128;
constexpr long TC_WAIT_LIMIT = 1L << 18;   // about one second of polls

// shared memory: B [N][K], the A stages [128][K] (canonical layouts), the epilogue
// patches (8 warps x 32 rows x 33 floats), then two barriers and the tensor-memory address.
// Two A stages (a third, copying two tiles ahead, measured no faster).
constexpr int TC_PATCH = 32 * 33;   // 32 rows x 32 columns, padded
__host__ __device__ constexpr int tc_stages(int) { return 2; }
__host__ __device__ constexpr size_t tc_smem_bytes(int N, int K)
{
  return (size_t)N * K * 2 + tc_stages(K) * (size_t)TC_M * K * 2 + (TC_THREADS / 32) * TC_PATCH * 4 + 64;
}
// tensor-memory columns of one CTA (two accumulators of at least 32 columns)
__host__ __device__ constexpr int tc_tmem_cols(int N) { return 2 * ((N <= 32) ? 32 : (N <= 64) ? 64 : 128); }

__device__ __forceinline__ void tc_mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool tc_mbar_try(uint32_t bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool tc_mbar_wait(uint32_t bar, uint32_t parity)
{
  for (long i = 0; i < TC_WAIT_LIMIT; i++)
    if (tc_mbar_try(bar, parity)) return true;
  return false;
}

// shared-memory matrix descriptor: no swizzle, start address, leading / stride byte offsets
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version of the 5th-generation tensor cores
  return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__device__ __forceinline__ uint32_t tc_idesc(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float *v)
{
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float *v)
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// copies of A tile t (rows t*128 ..) into stage sA: 16-byte chunks, consecutive threads on
// consecutive chunks of the canonical layout; rows past M are zero-filled
__device__ __forceinline__ void tc_stage_a(bf16 *sA, const bf16 *A, long lda, int M, int K, int t)
{
  const int KC = K / 8, chunks = TC_M * KC;
  for (int c = threadIdx.x; c < chunks; c += TC_THREADS) {
    const int r = c & 7, kc = (c >> 3) % KC, g = (c >> 3) / KC;
    const long m = (long)t * TC_M + g * 8 + r;
    const bool ok = m < M;
    cp_async16(smem_addr(sA + (size_t)c * 8), ok ? A + m * lda + kc * 8 : A, ok ? 16 : 0);
  }
}

// four values of row m, columns n .. n+3 (n a multiple of 4), through the epilogue
__device__ __forceinline__ void tc_epilogue4(const GemmArgs &g, long m, int n, float *x)
{
  const bool vec_in = g.Cin && (g.ldcin % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.Cin) & (g.cin_f32 ? 15 : 7)) == 0);
  const bool vec_c = (g.ldc % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.C) & (g.c_f32 ? 15 : 7)) == 0);
  const bool vec_aux = g.aux && (g.ldaux % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.aux) & 7) == 0);
#pragma unroll
  for (int i = 0; i < 4; i++) x[i] *= g.alpha;
  if (g.Cin && g.beta != 0.f) {
    const long o = m * g.ldcin + n;
    float c[4];
    if (vec_in && g.cin_f32) {
      const float4 q = *reinterpret_cast<const float4 *>(static_cast<const float *>(g.Cin) + o);
      c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = q.w;
    } else if (vec_in) {
      const uint2 q = *reinterpret_cast<const uint2 *>(static_cast<const bf16 *>(g.Cin) + o);
      const __nv_bfloat162 lo = *reinterpret_cast<const __nv_bfloat162 *>(&q.x), hi = *reinterpret_cast<const __nv_bfloat162 *>(&q.y);
      c[0] = __low2float(lo); c[1] = __high2float(lo); c[2] = __low2float(hi); c[3] = __high2float(hi);
    } else {
#pragma unroll
      for (int i = 0; i < 4; i++)
        c[i] = g.cin_f32 ? static_cast<const float *>(g.Cin)[o + i] : __bfloat162float(static_cast<const bf16 *>(g.Cin)[o + i]);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) x[i] += g.beta * c[i];
  }
  if (g.bias) {
#pragma unroll
    for (int i = 0; i < 4; i++) x[i] += g.bias[n + i];
  }
  if (g.aux) {
    const long o = m * g.ldaux + n;
    if (vec_aux) {
      uint2 q;
      *reinterpret_cast<__nv_bfloat162 *>(&q.x) = __floats2bfloat162_rn(x[0], x[1]);
      *reinterpret_cast<__nv_bfloat162 *>(&q.y) = __floats2bfloat162_rn(x[2], x[3]);
      *reinterpret_cast<uint2 *>(g.aux + o) = q;
    } else {
#pragma unroll
      for (int i = 0; i < 4; i++) g.aux[o + i] = __float2bfloat16(x[i]);
    }
  }
  if (g.act == 1) {
#pragma unroll
    for (int i = 0; i < 4; i++) x[i] = gelu_f(x[i]);
  }
  const long o = m * g.ldc + n;
  if (vec_c && g.c_f32) {
    *reinterpret_cast<float4 *>(static_cast<float *>(g.C) + o) = make_float4(x[0], x[1], x[2], x[3]);
  } else if (vec_c) {
    uint2 q;
    *reinterpret_cast<__nv_bfloat162 *>(&q.x) = __floats2bfloat162_rn(x[0], x[1]);
    *reinterpret_cast<__nv_bfloat162 *>(&q.y) = __floats2bfloat162_rn(x[2], x[3]);
    *reinterpret_cast<uint2 *>(static_cast<bf16 *>(g.C) + o) = q;
  } else {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (g.c_f32) static_cast<float *>(g.C)[o + i] = x[i];
      else static_cast<bf16 *>(g.C)[o + i] = __float2bfloat16(x[i]);
    }
  }
}

__global__ void __launch_bounds__(TC_THREADS, 2) gemm_tc(const GemmArgs g, int *err)
{
  extern __shared__ __align__(1024) unsigned char tsm[];
  const int N = g.N, K = g.K, KC = K / 8;
  bf16 *sB = reinterpret_cast<bf16 *>(tsm);
  const int NS = tc_stages(K);
  bf16 *sA0 = sB + (size_t)N * K;   // stage j at sA0 + j * 128 K
  auto stage = [&](int i) { return sA0 + (size_t)(i % NS) * TC_M * K; };
  float *patch = reinterpret_cast<float *>(sA0 + (size_t)NS * TC_M * K);
  uint64_t *bars = reinterpret_cast<uint64_t *>(patch + (TC_THREADS / 32) * TC_PATCH);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);
  const uint32_t bar[2] = {smem_addr(&bars[0]), smem_addr(&bars[1])};
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncols = tc_tmem_cols(N), acc_cols = ncols / 2;   // two accumulators

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    tc_mbar_init(bar[0], 1);
    tc_mbar_init(bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // op(B) as N x K, K-major canonical, read along the stored rows of B (consecutive
  // threads on consecutive addresses): B[k][n] at B[k*ldb + n] (transB = 0) or B[n*ldb + k]
  for (int e = threadIdx.x; e < N * K; e += TC_THREADS) {
    int n, k;
    if (g.transB) { n = e / K; k = e - n * K; }
    else { k = e / N; n = e - k * N; }
    const bf16 v = g.transB ? g.B[(long)n * g.ldb + k] : g.B[(long)k * g.ldb + n];
    sB[((n >> 3) * KC + (k >> 3)) * 64 + (n & 7) * 8 + (k & 7)] = v;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int ntiles = (g.M + TC_M - 1) / TC_M;
  const int step = gridDim.x;
  const int mine = (blockIdx.x < ntiles) ? (ntiles - 1 - blockIdx.x) / step + 1 : 0;   // tiles of this CTA
  const uint32_t idesc = tc_idesc(TC_M, N);
  const uint32_t lbo = 128, sbo = (uint32_t)KC * 128;
  auto tile_of = [&](int i) { return blockIdx.x + i * step; };
  auto issue = [&](int i) {   // one thread: the MMAs of this CTA's i-th tile into accumulator i & 1
    tc_fence_after();
    const uint32_t a0 = smem_addr(stage(i)), b0 = smem_addr(sB), d = tmem + (uint32_t)((i & 1) * acc_cols);
    for (int ks = 0; ks < K / 16; ks++)
      tc_mma(d, tc_desc(a0 + ks * 256, lbo, sbo), tc_desc(b0 + ks * 256, lbo, sbo), idesc, ks > 0 ? 1u : 0u);
    tc_commit(bar[i & 1]);
  };
  // prologue: tile 0 copied and multiplied; the copies of tiles 1 .. NS-1 in flight (one
  // cp.async group each, empty groups past the CTA's last tile keep the count)
  if (mine > 0) tc_stage_a(stage(0), g.A, g.lda, g.M, K, tile_of(0));
  cp_async_commit();
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic-proxy writes -> tensor-core reads
  __syncthreads();
  if (mine > 0 && threadIdx.x == 0) issue(0);
  for (int j = 1; j < NS; j++) {
    if (j < mine) tc_stage_a(stage(j), g.A, g.lda, g.M, K, tile_of(j));
    cp_async_commit();
  }
  int failed = -1;
  float *pw = patch + warp * TC_PATCH;
  for (int i = 0; i < mine; i++) {
    // tile i+1's copy has landed (the newer NS-2 groups may still be in flight): its MMAs
    // go to the other accumulator
    if (NS == 3) asm volatile("cp.async.wait_group 1;" ::: "memory");
    else asm volatile("cp.async.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (i + 1 < mine && threadIdx.x == 0) issue(i + 1);
    // tile i's MMAs done: its stage is free for tile i+NS's copy, its accumulator readable
    const bool ok = tc_mbar_wait(bar[i & 1], (uint32_t)((i >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      failed = i;
      break;
    }
    tc_fence_after();
    if (i + NS < mine) tc_stage_a(stage(i), g.A, g.lda, g.M, K, tile_of(i + NS));
    cp_async_commit();
    // warps w and w + 4 share tensor-memory lanes 32 (w % 4) .. (the tile's rows), and take
    // alternate 16-column chunks
    const int quarter = warp & 3;
    const long row0 = (long)tile_of(i) * TC_M + quarter * 32;
    const uint32_t acc = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((i & 1) * acc_cols);
    // chunks of 32 columns (16 where N is not a multiple of 32), alternating between the
    // two warps of a lane quarter; a chunk's row segments are then written whole (32
    // floats = one 128-byte line), 4 consecutive columns per lane
    const int CW = (N % 32 == 0) ? 32 : 16, LPR = CW / 4, RPP = 32 / LPR;   // lanes per row, rows per pass
    for (int n0 = (warp >> 2) * CW; n0 < N; n0 += 2 * CW) {
      {
        float v[32];
        if (CW == 32) tc_ld32(acc + (uint32_t)n0, v);
        else tc_ld16(acc + (uint32_t)n0, v);
#pragma unroll
        for (int c = 0; c < 32; c++)
          if (c < CW) pw[lane * 33 + c] = v[c];
      }
      __syncwarp();
      for (int pass = 0; pass < 32 / RPP; pass++) {
        const int r = pass * RPP + lane / LPR, c4 = (lane % LPR) * 4;
        const long m = row0 + r;
        float x[4] = {pw[r * 33 + c4], pw[r * 33 + c4 + 1], pw[r * 33 + c4 + 2], pw[r * 33 + c4 + 3]};
        if (m < g.M) tc_epilogue4(g, m, n0 + c4, x);
      }
      __syncwarp();
    }
    tc_fence_before();
    __syncthreads();   // accumulator i & 1 is free for tile i+2's MMAs
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (failed >= 0 && threadIdx.x == 0) {
    atomicExch(err, 1);
    // (bounded) let the MMAs in flight land before the memory goes: tile `failed`'s and,
    // if issued, the next one's
    tc_mbar_wait(bar[failed & 1], (uint32_t)((failed >> 1) & 1));
    if (failed + 1 < mine) tc_mbar_wait(bar[(failed + 1) & 1], (uint32_t)(((failed + 1) >> 1) & 1));
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

}  // namespace nnk
