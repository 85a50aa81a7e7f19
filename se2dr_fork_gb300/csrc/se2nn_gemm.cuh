// se2nn_gemm.cuh -- strided-batched BF16 GEMM with FP32 accumulation on the
// tensor cores, the one contraction kernel of the surrogate network.
//
//   C[b] = act(alpha * op(A[b]) op(B[b]) + beta * Cin[b] + bias)      b < batch
//
// op(A) is M x K: A[m,k] = A[m*lda + k] (transA = 0) or A[k*lda + m] (transA = 1);
// op(B) is K x N: B[k,n] = B[k*ldb + n] (transB = 0) or B[n*ldb + k] (transB = 1).
// Batch strides may be 0 (an operand shared by every batch).  The epilogue can
// add a per-column bias, store the pre-activation (aux, BF16), apply GELU and
// write C in FP32 or BF16; Cin may alias C (in-place accumulation).
//
// Tiles: 64 x 64 x 32 per CTA, 4 warps of 32 x 32, each warp 2 x 4
// mma.m16n8k16 (bf16 -> f32).  Operands keep their global layout in shared
// memory, filled by a 3-stage pipeline of 16-byte cp.async copies (zero-filled
// at the edges; element copies when the leading dimension or the base is not
// 16-byte aligned); fragments are read with ldmatrix, transposing (.trans) for
// operands whose contiguous dimension is m or n.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace nnk {

typedef __nv_bfloat16 bf16;

struct GemmArgs {
  const bf16 *A, *B;
  long lda, ldb, sA, sB;
  int transA, transB;
  int M, N, K, batch;
  float alpha, beta;
  const void *Cin;       // optional (beta != 0): same type as C unless cin_f32 says otherwise
  long ldcin, sCin;
  int cin_f32;
  const float *bias;     // optional, per column
  int act;               // 0 none, 1 GELU (erf form)
  void *C;
  long ldc, sC;
  int c_f32;
  bf16 *aux;             // optional pre-activation output
  long ldaux, sAux;
};

constexpr int GBM = 64, GBN = 64, GBK = 32, GPAD = 8, GTHREADS = 128, GSTAGES = 3;
// one stage of one operand: [64][32 + 8] (k contiguous) or [32][64 + 8] (m or n contiguous)
constexpr int GSTAGE_ELEMS = (GBM * (GBK + GPAD) > GBK * (GBM + GPAD)) ? GBM * (GBK + GPAD) : GBK * (GBM + GPAD);

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float x)
{
  // d/dx [x Phi(x)] = Phi(x) + x phi(x)
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b)
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t *r, uint32_t addr, bool trans)
{
  if (trans)
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(addr));
  else
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(addr));
}

// 16-byte asynchronous copy global -> shared; bytes < 16 zero-fills the rest (0: nothing is read)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, int bytes)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_stages() { asm volatile("cp.async.wait_group %0;" ::"n"(GSTAGES - 2) : "memory"); }

// Stage the k-tile starting at k0 of one operand, keeping its global layout:
//   k contiguous (kc): tile [ROWS (m or n)][GBK], element (r, k) at X[(r0 + r) * ld + k0 + k];
//   otherwise:         tile [GBK][ROWS],         element (k, r) at X[(k0 + k) * ld + r0 + r].
// vec: 16-byte cp.async copies (ld % 8 == 0, 16-byte aligned base); else plain element copies.
template <int ROWS>
__device__ __forceinline__ void stage_operand(bf16 *sm, const bf16 *X, long ld, bool kc, int r0, int rows, int k0,
                                              int K, bool vec)
{
  const bf16 zero = __float2bfloat16(0.f);
  const int W = kc ? GBK : ROWS;            // tile row length (elements)
  const int H = kc ? ROWS : GBK;            // tile rows
  const int lim_row = kc ? rows - r0 : K - k0;     // valid tile rows
  const int lim_col = kc ? K - k0 : rows - r0;     // valid elements per tile row
  const long grow0 = kc ? r0 : k0, gcol0 = kc ? k0 : r0;
  if (vec) {
    for (int e = threadIdx.x; e < H * W / 8; e += GTHREADS) {
      const int tr = e / (W / 8), tc = (e % (W / 8)) * 8;
      int valid = (tr < lim_row) ? lim_col - tc : 0;
      valid = valid < 0 ? 0 : (valid > 8 ? 8 : valid);
      const bf16 *src = valid ? X + (grow0 + tr) * ld + gcol0 + tc : X;
      cp_async16(smem_addr(sm + tr * (W + GPAD) + tc), src, valid * 2);
    }
  } else {
    for (int e = threadIdx.x; e < H * W; e += GTHREADS) {
      const int tr = e / W, tc = e % W;
      sm[tr * (W + GPAD) + tc] = (tr < lim_row && tc < lim_col) ? X[(grow0 + tr) * ld + gcol0 + tc] : zero;
    }
  }
}

__global__ void __launch_bounds__(GTHREADS) gemm_bf16(const GemmArgs g)
{
  __shared__ __align__(128) bf16 sA[GSTAGES][GSTAGE_ELEMS];
  __shared__ __align__(128) bf16 sB[GSTAGES][GSTAGE_ELEMS];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const bf16 *A = g.A + (long)b * g.sA;
  const bf16 *B = g.B + (long)b * g.sB;
  const bool a_kc = !g.transA, b_kc = g.transB;   // k contiguous in the stored tile
  const bool a_vec = ((g.lda % 8) == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
  const bool b_vec = ((g.ldb % 8) == 0) && ((reinterpret_cast<uintptr_t>(B) & 15) == 0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;

  const int KT = (g.K + GBK - 1) / GBK;
#pragma unroll
  for (int st = 0; st < GSTAGES - 1; st++) {
    if (st < KT) {
      stage_operand<GBM>(sA[st], A, g.lda, a_kc, m0, g.M, st * GBK, g.K, a_vec);
      stage_operand<GBN>(sB[st], B, g.ldb, b_kc, n0, g.N, st * GBK, g.K, b_vec);
    }
    cp_async_commit();
  }
  // ldmatrix row addresses: lane l -> matrix l / 8, row l % 8 of that 8x8 matrix
  const int mat = lane >> 3, mrow = lane & 7;
  for (int kt = 0; kt < KT; kt++) {
    cp_async_wait_stages();
    __syncthreads();
    {
      const int nk = kt + GSTAGES - 1;
      if (nk < KT) {
        stage_operand<GBM>(sA[nk % GSTAGES], A, g.lda, a_kc, m0, g.M, nk * GBK, g.K, a_vec);
        stage_operand<GBN>(sB[nk % GSTAGES], B, g.ldb, b_kc, n0, g.N, nk * GBK, g.K, b_vec);
      }
      cp_async_commit();
    }
    const bf16 *tA = sA[kt % GSTAGES];
    const bf16 *tB = sB[kt % GSTAGES];
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        // matrices: 0 rows m..m+7 / k..k+7, 1 rows m+8.. / k.., 2 rows m.. / k+8.., 3 rows m+8.. / k+8..
        const int mm = wm + i * 16 + (mat & 1) * 8, kq = kk + (mat >> 1) * 8;
        const uint32_t addr = a_kc ? smem_addr(tA + (mm + mrow) * (GBK + GPAD) + kq)
                                   : smem_addr(tA + (kq + mrow) * (GBM + GPAD) + mm);
        ldsm_x4(af[i], addr, !a_kc);
      }
#pragma unroll
      for (int jj = 0; jj < 2; jj++) {
        // matrices: 0 n..n+7 / k..k+7, 1 n.. / k+8.., 2 n+8.. / k.., 3 n+8.. / k+8..
        const int nn = wn + jj * 16 + (mat >> 1) * 8, kq = kk + (mat & 1) * 8;
        const uint32_t addr = b_kc ? smem_addr(tB + (nn + mrow) * (GBK + GPAD) + kq)
                                   : smem_addr(tB + (kq + mrow) * (GBN + GPAD) + nn);
        uint32_t r[4];
        ldsm_x4(r, addr, !b_kc);
        bfr[2 * jj][0] = r[0]; bfr[2 * jj][1] = r[1];
        bfr[2 * jj + 1][0] = r[2]; bfr[2 * jj + 1][1] = r[3];
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");

  // epilogue: accumulator element r of tile (i, j) is (row gid + 8*(r/2), column 2*tig + r%2);
  // the two columns of a row are handled as a pair (one 4- or 8-byte access) when aligned
  const bool c_pair = (((g.ldc | g.sC) & 1) == 0) && ((reinterpret_cast<uintptr_t>(g.C) & (g.c_f32 ? 7 : 3)) == 0);
  const bool in_pair = g.Cin && (((g.ldcin | g.sCin) & 1) == 0) &&
                       ((reinterpret_cast<uintptr_t>(g.Cin) & (g.cin_f32 ? 7 : 3)) == 0);
  const bool aux_pair = g.aux && (((g.ldaux | g.sAux) & 1) == 0) && ((reinterpret_cast<uintptr_t>(g.aux) & 3) == 0);
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int hf = 0; hf < 2; hf++) {
        const int m = m0 + wm + i * 16 + gid + 8 * hf;
        const int n = n0 + wn + j * 8 + tig * 2;
        if (m >= g.M || n >= g.N) continue;
        const bool two = (n + 1 < g.N);
        float v[2] = {g.alpha * acc[i][j][2 * hf], g.alpha * acc[i][j][2 * hf + 1]};
        if (g.Cin && g.beta != 0.f) {
          const long o = (long)b * g.sCin + (long)m * g.ldcin + n;
          if (two && in_pair) {
            if (g.cin_f32) {
              const float2 c = *reinterpret_cast<const float2 *>(static_cast<const float *>(g.Cin) + o);
              v[0] += g.beta * c.x; v[1] += g.beta * c.y;
            } else {
              const __nv_bfloat162 c = *reinterpret_cast<const __nv_bfloat162 *>(static_cast<const bf16 *>(g.Cin) + o);
              v[0] += g.beta * __low2float(c); v[1] += g.beta * __high2float(c);
            }
          } else {
            for (int t = 0; t < (two ? 2 : 1); t++)
              v[t] += g.beta * (g.cin_f32 ? static_cast<const float *>(g.Cin)[o + t]
                                          : __bfloat162float(static_cast<const bf16 *>(g.Cin)[o + t]));
          }
        }
        if (g.bias) { v[0] += g.bias[n]; if (two) v[1] += g.bias[n + 1]; }
        if (g.aux) {
          const long o = (long)b * g.sAux + (long)m * g.ldaux + n;
          if (two && aux_pair) *reinterpret_cast<__nv_bfloat162 *>(g.aux + o) = __floats2bfloat162_rn(v[0], v[1]);
          else for (int t = 0; t < (two ? 2 : 1); t++) g.aux[o + t] = __float2bfloat16(v[t]);
        }
        if (g.act == 1) { v[0] = gelu_f(v[0]); v[1] = gelu_f(v[1]); }
        const long o = (long)b * g.sC + (long)m * g.ldc + n;
        if (two && c_pair) {
          if (g.c_f32) *reinterpret_cast<float2 *>(static_cast<float *>(g.C) + o) = make_float2(v[0], v[1]);
          else *reinterpret_cast<__nv_bfloat162 *>(static_cast<bf16 *>(g.C) + o) = __floats2bfloat162_rn(v[0], v[1]);
        } else {
          for (int t = 0; t < (two ? 2 : 1); t++) {
            if (g.c_f32) static_cast<float *>(g.C)[o + t] = v[t];
            else static_cast<bf16 *>(g.C)[o + t] = __float2bfloat16(v[t]);
          }
        }
      }
}

}  // namespace nnk
