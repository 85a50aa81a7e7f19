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
// mma.m16n8k16 (bf16 -> f32).  Both operands are staged in shared memory
// k-contiguous ([m][k] and [n][k]) whatever their global layout, so a single
// fragment path serves every transpose combination; global loads are 16-byte
// vectors when the contiguous dimension and the pointers allow it.
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

constexpr int GBM = 64, GBN = 64, GBK = 32, GPAD = 8, GTHREADS = 128;

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

// stage a ROWS x GBK tile of a k-contiguous-in-shared operand:
// element (r, k) of the tile is X[(r0 + r) * ld_r + (k0 + k) * ld_k] in global memory,
// with (ld_r, ld_k) = (ld, 1) when k is contiguous, (1, ld) when r is.
template <int ROWS>
__device__ __forceinline__ void stage_tile(bf16 (*s)[GBK + GPAD], const bf16 *X, long ld, bool k_contig, int r0,
                                           int rows, int k0, int K, bool vec_ok)
{
  const bf16 zero = __float2bfloat16(0.f);
  if (k_contig) {
    if (vec_ok) {
      // 8 consecutive k per 16-byte vector: ROWS * GBK / 8 vectors
      for (int e = threadIdx.x; e < ROWS * GBK / 8; e += GTHREADS) {
        const int r = e / (GBK / 8), kk = (e % (GBK / 8)) * 8;
        const int gr = r0 + r, gk = k0 + kk;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr < rows && gk + 7 < K) v = *reinterpret_cast<const uint4 *>(X + (long)gr * ld + gk);
        else if (gr < rows) {
          __align__(16) bf16 t[8];
          for (int i = 0; i < 8; i++) t[i] = (gk + i < K) ? X[(long)gr * ld + gk + i] : zero;
          v = *reinterpret_cast<uint4 *>(t);
        }
        *reinterpret_cast<uint4 *>(&s[r][kk]) = v;
      }
    } else {
      for (int e = threadIdx.x; e < ROWS * GBK; e += GTHREADS) {
        const int r = e / GBK, k = e % GBK;
        const int gr = r0 + r, gk = k0 + k;
        s[r][k] = (gr < rows && gk < K) ? X[(long)gr * ld + gk] : zero;
      }
    }
  } else {
    if (vec_ok) {
      // 8 consecutive rows per 16-byte vector, transposed into shared memory
      for (int e = threadIdx.x; e < ROWS * GBK / 8; e += GTHREADS) {
        const int k = e / (ROWS / 8), rr = (e % (ROWS / 8)) * 8;
        const int gk = k0 + k, gr = r0 + rr;
        __align__(16) bf16 t[8];
        if (gk < K && gr + 7 < rows) {
          *reinterpret_cast<uint4 *>(t) = *reinterpret_cast<const uint4 *>(X + (long)gk * ld + gr);
        } else {
          for (int i = 0; i < 8; i++) t[i] = (gk < K && gr + i < rows) ? X[(long)gk * ld + gr + i] : zero;
        }
        for (int i = 0; i < 8; i++) s[rr + i][k] = t[i];
      }
    } else {
      for (int e = threadIdx.x; e < ROWS * GBK; e += GTHREADS) {
        const int k = e / ROWS, r = e % ROWS;
        const int gr = r0 + r, gk = k0 + k;
        s[r][k] = (gr < rows && gk < K) ? X[(long)gk * ld + gr] : zero;
      }
    }
  }
}

__global__ void __launch_bounds__(GTHREADS) gemm_bf16(const GemmArgs g)
{
  __shared__ __align__(16) bf16 sA[GBM][GBK + GPAD];
  __shared__ __align__(16) bf16 sB[GBN][GBK + GPAD];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const bf16 *A = g.A + (long)b * g.sA;
  const bf16 *B = g.B + (long)b * g.sB;
  // A as rows m: k contiguous unless transposed; B as rows n: k contiguous when transposed
  const bool a_kc = !g.transA, b_kc = g.transB;
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

  for (int k0 = 0; k0 < g.K; k0 += GBK) {
    stage_tile<GBM>(sA, A, g.lda, a_kc, m0, g.M, k0, g.K, a_vec);
    stage_tile<GBN>(sB, B, g.ldb, b_kc, n0, g.N, k0, g.K, b_vec);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int r = wm + i * 16 + gid;
        af[i][0] = *reinterpret_cast<const uint32_t *>(&sA[r][kk + tig * 2]);
        af[i][1] = *reinterpret_cast<const uint32_t *>(&sA[r + 8][kk + tig * 2]);
        af[i][2] = *reinterpret_cast<const uint32_t *>(&sA[r][kk + 8 + tig * 2]);
        af[i][3] = *reinterpret_cast<const uint32_t *>(&sA[r + 8][kk + 8 + tig * 2]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int c = wn + j * 8 + gid;
        bfr[j][0] = *reinterpret_cast<const uint32_t *>(&sB[c][kk + tig * 2]);
        bfr[j][1] = *reinterpret_cast<const uint32_t *>(&sB[c][kk + 8 + tig * 2]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }

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
