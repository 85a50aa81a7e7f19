// se2nn.cu -- the surrogate network runtime (include/se2nn.h): parameter and
// activation buffers, forward and backward passes as sequences of hand-written
// kernels, Adam, data-set gathers.  Every contraction runs through the BF16
// tensor-core GEMM of se2nn_gemm.cuh; everything else is a small elementwise,
// permutation or fixed-order reduction kernel below.  Results do not depend on
// scheduling: reductions are two-stage with fixed partitions, no atomics.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "se2nn.h"
#include "se2nn_gemm.cuh"
#include "se2nn_tc.cuh"

using nnk::bf16;
using nnk::GemmArgs;

namespace {

constexpr int EW = 256;   // threads of the elementwise kernels

inline unsigned nblk(long n, int t = EW) { return (unsigned)((n + t - 1) / t); }

// ------------------------------------------------------------------ kernels
__global__ void k_f32_to_bf16(const float *x, bf16 *y, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

// Wblk[mode] (2w x 2w, rows (part, ci), columns (part', co)) of the complex
// weights W = Wre + i Wim, so that [Zre Zim] Wblk = [Re(Z W) Im(Z W)]
__global__ void k_build_wblk(const float *wre, const float *wim, bf16 *blk, int nmodes, int w)
{
  const long n = (long)nmodes * 4 * w * w;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int w2 = 2 * w;
    const long mode = i / ((long)w2 * w2);
    const int r = (int)((i / w2) % w2), c = (int)(i % w2);
    const int pi = r / w, ci = r % w, po = c / w, co = c % w;
    const long o = (mode * w + ci) * w + co;
    float v;
    if (pi == po) v = wre[o];
    else v = (pi == 0) ? wim[o] : -wim[o];
    blk[i] = __float2bfloat16(v);
  }
}

// gradient of Wre, Wim from the gradient of Wblk
__global__ void k_fold_wblk(const float *dblk, float *dwre, float *dwim, int nmodes, int w)
{
  const long n = (long)nmodes * w * w;
  const int w2 = 2 * w;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long mode = i / ((long)w * w);
    const int ci = (int)((i / w) % w), co = (int)(i % w);
    const float *d = dblk + mode * w2 * w2;
    dwre[i] = d[ci * w2 + co] + d[(w + ci) * w2 + w + co];
    dwim[i] = d[ci * w2 + w + co] - d[(w + ci) * w2 + co];
  }
}

// Z[b][j][part][kx][c]  <->  Zp[(j, kx)][b][part][c]    (dir 0: Z -> Zp, 1: Zp -> Z)
__global__ void k_permute_modes(const bf16 *src, bf16 *dst, int B, int m, int w, int dir)
{
  const int jn = 2 * m;
  const long n = (long)B * jn * 2 * m * w;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    // i indexes Z
    const int c = (int)(i % w);
    const int kx = (int)((i / w) % m);
    const int part = (int)((i / ((long)w * m)) % 2);
    const int j = (int)((i / ((long)w * m * 2)) % jn);
    const int b = (int)(i / ((long)w * m * 2 * jn));
    const long p = (((long)(j * m + kx) * B + b) * 2 + part) * w + c;
    if (dir == 0) dst[p] = src[i];
    else dst[i] = src[p];
  }
}

__global__ void k_gelu_bwd(const bf16 *dpost, const bf16 *pre, bf16 *dpre, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dpre[i] = __float2bfloat16(__bfloat162float(dpost[i]) * nnk::gelu_grad_f(__bfloat162float(pre[i])));
}

// column sums of X[M][N] (bf16): partial[chunk][N] over rows [chunk*rows, ...).  With N <= EW
// the block's threads split into EW / N row lanes per column; each lane sums every
// (EW / N)-th row of the chunk and the lanes are added in lane order (fixed partition).
__global__ void k_colsum_partial(const bf16 *X, long M, int N, long rows, float *partial)
{
  __shared__ float s[EW];
  const long r0 = blockIdx.y * rows, r1 = (r0 + rows < M) ? r0 + rows : M;
  if (N <= EW) {
    const int lanes = EW / N, c = threadIdx.x % N, lane = threadIdx.x / N;
    float v = 0.f;
    if (lane < lanes)
      for (long r = r0 + lane; r < r1; r += lanes) v += __bfloat162float(X[r * N + c]);
    s[threadIdx.x] = v;
    __syncthreads();
    if ((int)threadIdx.x < N) {
      float t = 0.f;
      for (int l = 0; l < lanes; l++) t += s[l * N + threadIdx.x];
      partial[(long)blockIdx.y * N + threadIdx.x] = t;
    }
    return;
  }
  for (int n = threadIdx.x; n < N; n += blockDim.x) {
    float t = 0.f;
    for (long r = r0; r < r1; r++) t += __bfloat162float(X[r * N + n]);
    partial[(long)blockIdx.y * N + n] = t;
  }
}

// out[i] = sum over k < nparts of partial[k][i], in order
__global__ void k_sum_parts(const float *partial, int nparts, long n, float *out)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < nparts; k++) s += partial[(long)k * n + i];
    out[i] = s;
  }
}

// D0[((b*nrec + r)*ny + row)] = H[b][row][rec_x[r]][0:w]: every row of each receiver's column
__global__ void k_decoder_gather(const bf16 *H, const int *rec_x, int B, int nrec, int ny, int nx, int w, bf16 *D0)
{
  const long n = (long)B * nrec * ny * w;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % w);
    const long q = i / w;
    const int row = (int)(q % ny), r = (int)((q / ny) % nrec), b = (int)(q / ((long)ny * nrec));
    D0[i] = H[(((long)b * ny + row) * nx + rec_x[r]) * w + c];
  }
}

// dH[b][row][x][c] = sum over receivers r in column x of dD0[((b*nrec + r)*ny + row)][c]
__global__ void k_decoder_scatter(const bf16 *dD0, const int *rec_x, int B, int nrec, int ny, int nx, int w, bf16 *dH)
{
  const long n = (long)B * ny * nx * w;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % w);
    const long pix = i / w;
    const int x = (int)(pix % nx), row = (int)((pix / nx) % ny), b = (int)(pix / ((long)nx * ny));
    float v = 0.f;
    for (int r = 0; r < nrec; r++)
      if (rec_x[r] == x) v += __bfloat162float(dD0[(((long)b * nrec + r) * ny + row) * w + c]);
    dH[i] = __float2bfloat16(v);
  }
}

// squared-error partial sums (double, per block) and dL/dout = 2 (out - t) / n
__global__ void k_mse(const float *out, const float *target, long n, double *partial, bf16 *dout)
{
  __shared__ double s[EW];
  double acc = 0.0;
  const float scale = 2.0f / (float)n;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float d = out[i] - target[i];
    acc += (double)d * (double)d;
    dout[i] = __float2bfloat16(scale * d);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, long n, float lr, float b1, float b2, float eps,
                       float wd, float c1, float c2)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / c1, vh = vi / c2;
    p[i] = p[i] - lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
  }
}

// network input of sample idx[b]: normalised materials, source blob, coordinates
__global__ void k_build_inputs(const float *mat, const float *src, const int *idx, int B, int ny, int nx, int cin,
                               float inv2s2, bf16 *x)
{
  const long n = (long)B * ny * nx;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int cx = (int)(i % nx), cy = (int)((i / nx) % ny), b = (int)(i / ((long)nx * ny));
    const long s = idx[b];
    // network row cy counts down from the top surface: material row ny - 1 - cy, source row ny - y
    const float *mm = mat + ((s * ny + (ny - 1 - cy)) * nx + cx) * 3;
    const float dx = (cx + 0.5f) - src[2 * s], dy = (cy + 0.5f) - ((float)ny - src[2 * s + 1]);
    float ch[6];
    ch[0] = (mm[0] - 5000.f) * (1.f / 1500.f);   // vp
    ch[1] = (mm[1] - 2800.f) * (1.f / 800.f);    // vs
    ch[2] = (mm[2] - 2500.f) * (1.f / 500.f);    // rho
    ch[3] = __expf(-(dx * dx + dy * dy) * inv2s2);
    ch[4] = (2.f * cx + 1.f) / nx - 1.f;
    ch[5] = (2.f * cy + 1.f) / ny - 1.f;
    bf16 *o = x + i * cin;
    for (int c = 0; c < cin; c++) o[c] = __float2bfloat16(c < 6 ? ch[c] : 0.f);
  }
}

__global__ void k_gather_rows(const float *src, const int *idx, int B, long row, float *dst)
{
  const long n = (long)B * row;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = src[(long)idx[i / row] * row + i % row];
}

}  // namespace

// ------------------------------------------------------------------ the network
struct se2nn {
  se2nn_config c{};
  int npix = 0, w = 0, m = 0, nmodes = 0, L = 0;
  long P = 0;
  // parameter offsets (floats)
  long oW0 = 0, ob0 = 0, oW1 = 0, oc1 = 0, oW2 = 0, oc2 = 0;
  std::vector<long> oWre, oWim, oW, ob;
  float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr;
  long adam_t = 0;
  // BF16 copies of the matrix parameters
  bf16 *W0b = nullptr, *W1b = nullptr, *W2b = nullptr;
  std::vector<bf16 *> Wb, Wblk;
  // DFT matrices (BF16): Ex [2m][nx], My [4m][2ny], Myinv [2ny][4m], Exinv [nx][2m]
  bf16 *Ex = nullptr, *My = nullptr, *Myinv = nullptr, *Exinv = nullptr;
  int *rec_x = nullptr;
  // activations (max batch)
  std::vector<bf16 *> H, Apre, Zp;
  bf16 *S = nullptr, *Xf = nullptr, *Z = nullptr, *Yp = nullptr, *Y = nullptr, *Yy = nullptr, *dZp = nullptr;
  bf16 *D0 = nullptr, *D1pre = nullptr, *D1 = nullptr, *dpred = nullptr;
  bf16 *dHa = nullptr, *dHb = nullptr, *dA = nullptr, *dD1 = nullptr, *dD0 = nullptr;
  float *out = nullptr, *partial = nullptr, *dblk = nullptr;
  double *lpart = nullptr;
  long partial_n = 0;
  int split = 1, nsub = 1;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  char err[512] = {0};
};

namespace {

thread_local char g_nn_create_err[512];

int nfail(se2nn *h, int code, const char *fmt, ...)
{
  char *buf = h ? h->err : g_nn_create_err;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, 512, fmt, ap);
  va_end(ap);
  return code;
}

#define NCK(h, call)                                                                                             \
  do {                                                                                                           \
    cudaError_t e_ = (call);                                                                                     \
    if (e_ != cudaSuccess) return nfail((h), -2, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

template <class T>
int nalloc(se2nn *h, T **p, size_t count)
{
  *p = nullptr;
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, count ? count * sizeof(T) : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nfail(h, -3, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
  }
  h->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return 0;
}

uint64_t mix64(uint64_t *s)
{
  uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

float uniform_pm(uint64_t *s, float a) { return a * (float)(2.0 * ((double)(mix64(s) >> 11) / 9007199254740992.0) - 1.0); }

int upload_bf16(se2nn *h, bf16 *dst, const std::vector<float> &src)
{
  std::vector<bf16> t(src.size());
  for (size_t i = 0; i < src.size(); i++) t[i] = __float2bfloat16(src[i]);
  NCK(h, cudaMemcpy(dst, t.data(), t.size() * sizeof(bf16), cudaMemcpyHostToDevice));
  return 0;
}

// the truncated DFT matrices of the spectral layers (built in double, stored BF16)
int build_dft(se2nn *h)
{
  const int nx = h->c.nx, ny = h->c.ny, m = h->m;
  const double tau = 2.0 * M_PI;
  auto ky_of = [&](int j) { return j < m ? j : ny - 2 * m + j; };
  std::vector<float> ex(2 * m * nx), my(4 * m * 2 * ny), myi(2 * ny * 4 * m), exi(nx * 2 * m);
  for (int kx = 0; kx < m; kx++)
    for (int x = 0; x < nx; x++) {
      const double t = tau * kx * x / nx;
      ex[(0 * m + kx) * nx + x] = (float)cos(t);
      ex[(1 * m + kx) * nx + x] = (float)-sin(t);
      const double wk = (kx == 0 ? 1.0 : 2.0) / ((double)nx * ny);
      exi[x * 2 * m + 0 * m + kx] = (float)(wk * cos(t));
      exi[x * 2 * m + 1 * m + kx] = (float)(-wk * sin(t));
    }
  for (int j = 0; j < 2 * m; j++)
    for (int y = 0; y < ny; y++) {
      const double t = tau * ky_of(j) * y / ny, c = cos(t), s = sin(t);
      // forward: Z = sum_y e^{-i t} Xf
      my[(j * 2 + 0) * 2 * ny + y * 2 + 0] = (float)c;
      my[(j * 2 + 0) * 2 * ny + y * 2 + 1] = (float)s;
      my[(j * 2 + 1) * 2 * ny + y * 2 + 0] = (float)-s;
      my[(j * 2 + 1) * 2 * ny + y * 2 + 1] = (float)c;
      // inverse: Yy = sum_j e^{+i t} Y
      myi[(y * 2 + 0) * 4 * m + j * 2 + 0] = (float)c;
      myi[(y * 2 + 0) * 4 * m + j * 2 + 1] = (float)-s;
      myi[(y * 2 + 1) * 4 * m + j * 2 + 0] = (float)s;
      myi[(y * 2 + 1) * 4 * m + j * 2 + 1] = (float)c;
    }
  int rc;
  if ((rc = nalloc(h, &h->Ex, ex.size())) || (rc = upload_bf16(h, h->Ex, ex))) return rc;
  if ((rc = nalloc(h, &h->My, my.size())) || (rc = upload_bf16(h, h->My, my))) return rc;
  if ((rc = nalloc(h, &h->Myinv, myi.size())) || (rc = upload_bf16(h, h->Myinv, myi))) return rc;
  if ((rc = nalloc(h, &h->Exinv, exi.size())) || (rc = upload_bf16(h, h->Exinv, exi))) return rc;
  return 0;
}

// refresh the BF16 operand copies from the FP32 master parameters
int refresh_bf16(se2nn *h)
{
  const int w = h->w, cin = h->c.cin, hid = h->c.hidden, ns = h->nsub;
  k_f32_to_bf16<<<nblk((long)cin * w), EW, 0, h->stream>>>(h->params + h->oW0, h->W0b, (long)cin * w);
  k_f32_to_bf16<<<nblk((long)w * hid), EW, 0, h->stream>>>(h->params + h->oW1, h->W1b, (long)w * hid);
  k_f32_to_bf16<<<nblk((long)hid * ns), EW, 0, h->stream>>>(h->params + h->oW2, h->W2b, (long)hid * ns);
  for (int l = 0; l < h->L; l++) {
    k_f32_to_bf16<<<nblk((long)w * w), EW, 0, h->stream>>>(h->params + h->oW[l], h->Wb[l], (long)w * w);
    const long nb = (long)h->nmodes * 4 * w * w;
    k_build_wblk<<<nblk(nb), EW, 0, h->stream>>>(h->params + h->oWre[l], h->params + h->oWim[l], h->Wblk[l], h->nmodes, w);
  }
  NCK(h, cudaGetLastError());
  return 0;
}

}  // namespace

namespace {

GemmArgs mk(const bf16 *A, long lda, long sA, int tA, const bf16 *B, long ldb, long sB, int tB, int M, int N, int K,
            int batch, void *C, long ldc, long sC, int c_f32)
{
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.A = A; g.lda = lda; g.sA = sA; g.transA = tA;
  g.B = B; g.ldb = ldb; g.sB = sB; g.transB = tB;
  g.M = M; g.N = N; g.K = K; g.batch = batch;
  g.alpha = 1.f; g.beta = 0.f;
  g.C = C; g.ldc = ldc; g.sC = sC; g.c_f32 = c_f32;
  return g;
}

// ---- the tensor-core (tcgen05) path for the row GEMMs -----------------------------
// 0: every GEMM runs gemm_bf16; 1 (default): qualifying row GEMMs run gemm_tc except those
// with N <= 64 and 32 < K <= 64 (the 1x1 convolutions and their data gradients, where
// the mma.sync kernel measured faster); 2: every qualifying row GEMM runs gemm_tc
std::atomic<int> g_tc_path{1};
std::atomic<long> g_tc_launches{0}, g_mma_launches{0};
__device__ int g_tc_err;

bool tc_eligible(const GemmArgs &g)
{
  return g_tc_path && (g_tc_path == 2 || !(g.N <= 64 && g.K > 32 && g.K <= 64)) && !g.transA && g.batch == 1 && g.M >= nnk::TC_M && g.K % 16 == 0 && g.K >= 16 &&
         g.K <= nnk::TC_KMAX && g.N % 16 == 0 && g.N >= 16 && g.N <= nnk::TC_NMAX && g.lda % 8 == 0 &&
         (reinterpret_cast<uintptr_t>(g.A) & 15) == 0;
}

// per device (the current one at the launch): the error flag's address, the SM count and
// the kernel's shared-memory limit, set up on the first launch on that device
struct TcDevice {
  int *err = nullptr;
  int nsm = 0;
};

cudaError_t launch_gemm_tc(const GemmArgs &g, cudaStream_t st)
{
  static std::mutex mu;
  static TcDevice devs[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  TcDevice d;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!devs[dev].err) {
      int nsm = 0;
      int *err = nullptr;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&err, g_tc_err);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(nnk::gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)nnk::tc_smem_bytes(nnk::TC_NMAX, nnk::TC_KMAX));
      if (e != cudaSuccess) return e;
      devs[dev].nsm = nsm;
      devs[dev].err = err;
    }
    d = devs[dev];
  }
  int *err = d.err;
  const int nsm = d.nsm;
  // resident CTAs per SM: what registers and shared memory allow, capped by the 512
  // tensor-memory columns of an SM (a CTA beyond them would wait in its allocation)
  const size_t smem = nnk::tc_smem_bytes(g.N, g.K);
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, nnk::gemm_tc, nnk::TC_THREADS, smem) != cudaSuccess) {
    cudaGetLastError();
    occ = 1;
  }
  occ = std::max(1, std::min(occ, 512 / nnk::tc_tmem_cols(g.N)));
  const int ntiles = (g.M + nnk::TC_M - 1) / nnk::TC_M;
  const int grid = std::min(ntiles, occ * nsm);
  nnk::gemm_tc<<<grid, nnk::TC_THREADS, smem, st>>>(g, err);
  g_tc_launches++;
  return cudaGetLastError();
}

cudaError_t launch_gemm(const GemmArgs &g, cudaStream_t st)
{
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return cudaSuccess;
  if (tc_eligible(g)) return launch_gemm_tc(g, st);
  g_mma_launches++;
  const unsigned gy = (unsigned)((g.M + nnk::GBM - 1) / nnk::GBM), gx = (unsigned)((g.N + nnk::GBN - 1) / nnk::GBN);
  if (gy > 65535u || g.batch > 65535) return cudaErrorInvalidConfiguration;
  nnk::gemm_bf16<<<dim3(gx, gy, (unsigned)g.batch), nnk::GTHREADS, 0, st>>>(g);
  return cudaGetLastError();
}

#define GEMM(h, g) NCK((h), launch_gemm((g), (h)->stream))

// column sums of X[M][N] (bf16) into out (f32), fixed partition of rows
int colsum(se2nn *h, const bf16 *X, long M, int N, long rows, float *out)
{
  const int chunks = (int)((M + rows - 1) / rows);
  k_colsum_partial<<<dim3(1, chunks), EW, 0, h->stream>>>(X, M, N, rows, h->partial);
  k_sum_parts<<<nblk(N), EW, 0, h->stream>>>(h->partial, chunks, N, out);
  NCK(h, cudaGetLastError());
  return 0;
}

// out (rows x w, f32) = X^T dY over B*npix pixels, split into B*split chunks then summed in order
int weight_grad(se2nn *h, const bf16 *X, int rows, const bf16 *dY, int B, float *out)
{
  const int w = h->w, s = h->split;
  const long kc = h->npix / s;
  GemmArgs g = mk(X, rows, kc * rows, 1, dY, w, kc * w, 0, rows, w, (int)kc, B * s, h->partial, w, (long)rows * w, 1);
  GEMM(h, g);
  k_sum_parts<<<nblk((long)rows * w), EW, 0, h->stream>>>(h->partial, B * s, (long)rows * w, out);
  NCK(h, cudaGetLastError());
  return 0;
}

// out (M x N, f32) = X^T dY for X [K][M], dY [K][N] (bf16, K rows a multiple of chunk), split-K in fixed order
int splitk_grad(se2nn *h, const bf16 *X, int M, const bf16 *dY, int N, long K, long chunk, float *out)
{
  const int parts = (int)(K / chunk);
  GemmArgs g = mk(X, M, chunk * M, 1, dY, N, chunk * N, 0, M, N, (int)chunk, parts, h->partial, N, (long)M * N, 1);
  GEMM(h, g);
  k_sum_parts<<<nblk((long)M * N), EW, 0, h->stream>>>(h->partial, parts, (long)M * N, out);
  NCK(h, cudaGetLastError());
  return 0;
}

// S = spectral convolution of Hin with layer l's weights; the mode-major input is kept in Zp[l]
int spectral_fwd(se2nn *h, int l, const bf16 *Hin, int B, bf16 *Sout)
{
  const int nx = h->c.nx, ny = h->c.ny, m = h->m, w = h->w;
  const long mw = (long)m * w;
  GEMM(h, mk(h->Ex, nx, 0, 0, Hin, w, (long)nx * w, 0, 2 * m, w, nx, B * ny, h->Xf, w, 2L * m * w, 0));
  GEMM(h, mk(h->My, 2 * ny, 0, 0, h->Xf, mw, (long)ny * 2 * mw, 0, 4 * m, (int)mw, 2 * ny, B, h->Z, mw, 4 * m * mw, 0));
  k_permute_modes<<<nblk((long)B * 4 * m * mw), EW, 0, h->stream>>>(h->Z, h->Zp[l], B, m, w, 0);
  GEMM(h, mk(h->Zp[l], 2 * w, (long)B * 2 * w, 0, h->Wblk[l], 2 * w, 4L * w * w, 0, B, 2 * w, 2 * w, h->nmodes, h->Yp,
             2 * w, (long)B * 2 * w, 0));
  k_permute_modes<<<nblk((long)B * 4 * m * mw), EW, 0, h->stream>>>(h->Yp, h->Y, B, m, w, 1);
  GEMM(h, mk(h->Myinv, 4 * m, 0, 0, h->Y, mw, 4 * m * mw, 0, 2 * ny, (int)mw, 4 * m, B, h->Yy, mw, 2L * ny * mw, 0));
  GEMM(h, mk(h->Exinv, 2 * m, 0, 0, h->Yy, w, 2L * m * w, 0, nx, w, 2 * m, B * ny, Sout, w, (long)nx * w, 0));
  return 0;
}

// backward of spectral_fwd: dS -> weight gradients of layer l, dHacc += dHin
int spectral_bwd(se2nn *h, int l, const bf16 *dS, int B, bf16 *dHacc)
{
  const int nx = h->c.nx, ny = h->c.ny, m = h->m, w = h->w;
  const long mw = (long)m * w;
  GEMM(h, mk(h->Exinv, 2 * m, 0, 1, dS, w, (long)nx * w, 0, 2 * m, w, nx, B * ny, h->Yy, w, 2L * m * w, 0));
  GEMM(h, mk(h->Myinv, 4 * m, 0, 1, h->Yy, mw, 2L * ny * mw, 0, 4 * m, (int)mw, 2 * ny, B, h->Y, mw, 4 * m * mw, 0));
  k_permute_modes<<<nblk((long)B * 4 * m * mw), EW, 0, h->stream>>>(h->Y, h->Yp, B, m, w, 0);
  GEMM(h, mk(h->Zp[l], 2 * w, (long)B * 2 * w, 1, h->Yp, 2 * w, (long)B * 2 * w, 0, 2 * w, 2 * w, B, h->nmodes, h->dblk,
             2 * w, 4L * w * w, 1));
  k_fold_wblk<<<nblk((long)h->nmodes * w * w), EW, 0, h->stream>>>(h->dblk, h->grads + h->oWre[l], h->grads + h->oWim[l],
                                                                    h->nmodes, w);
  GEMM(h, mk(h->Yp, 2 * w, (long)B * 2 * w, 0, h->Wblk[l], 2 * w, 4L * w * w, 1, B, 2 * w, 2 * w, h->nmodes, h->dZp,
             2 * w, (long)B * 2 * w, 0));
  k_permute_modes<<<nblk((long)B * 4 * m * mw), EW, 0, h->stream>>>(h->dZp, h->Z, B, m, w, 1);
  GEMM(h, mk(h->My, 2 * ny, 0, 1, h->Z, mw, 4 * m * mw, 0, 2 * ny, (int)mw, 4 * m, B, h->Xf, mw, 2L * ny * mw, 0));
  GemmArgs g = mk(h->Ex, nx, 0, 1, h->Xf, w, 2L * m * w, 0, nx, w, 2 * m, B * ny, dHacc, w, (long)nx * w, 0);
  g.beta = 1.f; g.Cin = dHacc; g.ldcin = w; g.sCin = (long)nx * w;
  GEMM(h, g);
  return 0;
}

int forward(se2nn *h, const bf16 *x, int B, float *out)
{
  const int w = h->w, L = h->L, nrec = h->c.nrec, hid = h->c.hidden;
  const long rows = (long)B * h->npix;
  {
    GemmArgs g = mk(x, h->c.cin, 0, 0, h->W0b, w, 0, 0, (int)rows, w, h->c.cin, 1, h->H[0], w, 0, 0);
    g.bias = h->params + h->ob0;
    GEMM(h, g);
  }
  int rc;
  for (int l = 0; l < L; l++) {
    if ((rc = spectral_fwd(h, l, h->H[l], B, h->S))) return rc;
    GemmArgs g = mk(h->H[l], w, 0, 0, h->Wb[l], w, 0, 0, (int)rows, w, w, 1, h->H[l + 1], w, 0, 0);
    g.beta = 1.f; g.Cin = h->S; g.ldcin = w;
    g.bias = h->params + h->ob[l];
    if (l < L - 1) { g.act = 1; g.aux = h->Apre[l]; g.ldaux = w; }
    GEMM(h, g);
  }
  const bf16 *HL = h->H[L];
  const long drows = (long)B * nrec * h->c.ny;
  k_decoder_gather<<<nblk(drows * w), EW, 0, h->stream>>>(HL, h->rec_x, B, nrec, h->c.ny, h->c.nx, w, h->D0);
  {
    GemmArgs g = mk(h->D0, w, 0, 0, h->W1b, hid, 0, 0, (int)drows, hid, w, 1, h->D1, hid, 0, 0);
    g.bias = h->params + h->oc1; g.act = 1; g.aux = h->D1pre; g.ldaux = hid;
    GEMM(h, g);
  }
  {
    GemmArgs g = mk(h->D1, hid, 0, 0, h->W2b, h->nsub, 0, 0, (int)drows, h->nsub, hid, 1, out, h->nsub, 0, 1);
    g.bias = h->params + h->oc2;
    GEMM(h, g);
  }
  NCK(h, cudaGetLastError());
  return 0;
}

int backward(se2nn *h, const bf16 *x, int B)
{
  const int w = h->w, npix = h->npix, L = h->L, nrec = h->c.nrec, hid = h->c.hidden, ns = h->nsub;
  const long rows = (long)B * npix, drows = (long)B * nrec * h->c.ny;
  int rc;
  // decoder (pointwise MLP over the receivers' columns); drows is a multiple of ny
  if ((rc = splitk_grad(h, h->D1, hid, h->dpred, ns, drows, h->c.ny, h->grads + h->oW2))) return rc;
  if ((rc = colsum(h, h->dpred, drows, ns, 256, h->grads + h->oc2))) return rc;
  GEMM(h, mk(h->dpred, ns, 0, 0, h->W2b, ns, 0, 1, (int)drows, hid, ns, 1, h->dD1, hid, 0, 0));
  k_gelu_bwd<<<nblk(drows * hid), EW, 0, h->stream>>>(h->dD1, h->D1pre, h->dD1, drows * hid);
  if ((rc = splitk_grad(h, h->D0, w, h->dD1, hid, drows, h->c.ny, h->grads + h->oW1))) return rc;
  if ((rc = colsum(h, h->dD1, drows, hid, 256, h->grads + h->oc1))) return rc;
  GEMM(h, mk(h->dD1, hid, 0, 0, h->W1b, hid, 0, 1, (int)drows, w, hid, 1, h->dD0, w, 0, 0));
  k_decoder_scatter<<<nblk(rows * w), EW, 0, h->stream>>>(h->dD0, h->rec_x, B, nrec, h->c.ny, h->c.nx, w, h->dHa);
  // Fourier layers, last to first: dHa holds dL/dH[l+1]
  for (int l = L - 1; l >= 0; l--) {
    const bf16 *dA = h->dHa;
    if (l < L - 1) {
      k_gelu_bwd<<<nblk(rows * w), EW, 0, h->stream>>>(h->dHa, h->Apre[l], h->dA, rows * w);
      dA = h->dA;
    }
    if ((rc = weight_grad(h, h->H[l], w, dA, B, h->grads + h->oW[l]))) return rc;
    if ((rc = colsum(h, dA, rows, w, 1024, h->grads + h->ob[l]))) return rc;
    GEMM(h, mk(dA, w, 0, 0, h->Wb[l], w, 0, 1, (int)rows, w, w, 1, h->dHb, w, 0, 0));
    if ((rc = spectral_bwd(h, l, dA, B, h->dHb))) return rc;
    bf16 *t = h->dHa; h->dHa = h->dHb; h->dHb = t;
  }
  // lift
  if ((rc = weight_grad(h, x, h->c.cin, h->dHa, B, h->grads + h->oW0))) return rc;
  if ((rc = colsum(h, h->dHa, rows, w, 1024, h->grads + h->ob0))) return rc;
  NCK(h, cudaGetLastError());
  return 0;
}

}  // namespace

extern "C" const char *se2nn_last_error(const se2nn *h) { return h ? h->err : g_nn_create_err; }

extern "C" void se2nn_destroy(se2nn *h)
{
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (void *p : h->allocs) cudaFree(p);
  delete h;
}

extern "C" long se2nn_num_params(const se2nn *h) { return h ? h->P : -1; }

extern "C" int se2nn_create(const se2nn_config *cfg, unsigned long long seed, se2nn **out)
{
  if (!out || !cfg) return nfail(nullptr, -1, "null argument");
  *out = nullptr;
  const se2nn_config c = *cfg;
  if (c.ny < 2 || c.nx < 2 || c.cin < 16 || c.cin % 16 || c.width < 16 || c.width % 16 || c.modes < 1 ||
      2 * c.modes > c.ny || 2 * c.modes > c.nx || c.layers < 1 || c.nrec < 1 || c.nout < c.ny || c.nout % c.ny ||
      c.hidden < 16 || c.hidden % 16 || c.max_batch < 1)
    return nfail(nullptr, -1, "invalid network configuration");
  if ((long)c.max_batch * c.ny > 65535 || 2L * c.modes * c.modes > 65535 ||
      ((long)c.max_batch * c.ny * c.nx + 63) / 64 > 65535)
    return nfail(nullptr, -1, "batch too large for the launch grid");
  se2nn *h = new se2nn();
  h->c = c;
  h->npix = c.ny * c.nx; h->w = c.width; h->m = c.modes; h->nmodes = 2 * c.modes * c.modes; h->L = c.layers;
  const int w = h->w, L = h->L, Bm = c.max_batch;
  const long nm = h->nmodes, npix = h->npix;
  // parameter layout
  long o = 0;
  h->oW0 = o; o += (long)c.cin * w;
  h->ob0 = o; o += w;
  for (int l = 0; l < L; l++) {
    h->oWre.push_back(o); o += nm * w * w;
    h->oWim.push_back(o); o += nm * w * w;
    h->oW.push_back(o); o += (long)w * w;
    h->ob.push_back(o); o += w;
  }
  h->nsub = c.nout / c.ny;
  h->oW1 = o; o += (long)w * c.hidden;
  h->oc1 = o; o += c.hidden;
  h->oW2 = o; o += (long)c.hidden * h->nsub;
  h->oc2 = o; o += h->nsub;
  h->P = o;
  h->split = (npix % 8 == 0) ? 8 : (npix % 4 == 0) ? 4 : (npix % 2 == 0) ? 2 : 1;
  int rc = 0;
#define TRY(x) do { if ((rc = (x)) != 0) { snprintf(g_nn_create_err, sizeof(g_nn_create_err), "%s", h->err); se2nn_destroy(h); return rc; } } while (0)
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return nfail(nullptr, -2, "cudaStreamCreate failed");
  }
  TRY(nalloc(h, &h->params, h->P));
  TRY(nalloc(h, &h->grads, h->P));
  TRY(nalloc(h, &h->adam_m, h->P));
  TRY(nalloc(h, &h->adam_v, h->P));
  TRY(nalloc(h, &h->W0b, (size_t)c.cin * w));
  TRY(nalloc(h, &h->W1b, (size_t)w * c.hidden));
  TRY(nalloc(h, &h->W2b, (size_t)c.hidden * h->nsub));
  h->Wb.assign(L, nullptr); h->Wblk.assign(L, nullptr); h->Zp.assign(L, nullptr);
  h->H.assign(L + 1, nullptr); h->Apre.assign(L > 1 ? L - 1 : 0, nullptr);
  for (int l = 0; l < L; l++) {
    TRY(nalloc(h, &h->Wb[l], (size_t)w * w));
    TRY(nalloc(h, &h->Wblk[l], (size_t)nm * 4 * w * w));
    TRY(nalloc(h, &h->Zp[l], (size_t)nm * Bm * 2 * w));
  }
  const size_t act = (size_t)Bm * npix * w;
  for (int l = 0; l <= L; l++) TRY(nalloc(h, &h->H[l], act));
  for (size_t l = 0; l < h->Apre.size(); l++) TRY(nalloc(h, &h->Apre[l], act));
  TRY(nalloc(h, &h->S, act));
  TRY(nalloc(h, &h->dHa, act));
  TRY(nalloc(h, &h->dHb, act));
  TRY(nalloc(h, &h->dA, act));
  TRY(nalloc(h, &h->Xf, (size_t)Bm * c.ny * 2 * h->m * w));
  TRY(nalloc(h, &h->Z, (size_t)Bm * 4 * h->m * h->m * w));
  TRY(nalloc(h, &h->Y, (size_t)Bm * 4 * h->m * h->m * w));
  TRY(nalloc(h, &h->Yy, (size_t)Bm * 2 * c.ny * h->m * w));
  TRY(nalloc(h, &h->Yp, (size_t)nm * Bm * 2 * w));
  TRY(nalloc(h, &h->dZp, (size_t)nm * Bm * 2 * w));
  const size_t drows = (size_t)Bm * c.nrec * c.ny;
  TRY(nalloc(h, &h->D0, drows * w));
  TRY(nalloc(h, &h->dD0, drows * w));
  TRY(nalloc(h, &h->D1pre, drows * c.hidden));
  TRY(nalloc(h, &h->D1, drows * c.hidden));
  TRY(nalloc(h, &h->dD1, drows * c.hidden));
  TRY(nalloc(h, &h->out, drows * h->nsub));
  TRY(nalloc(h, &h->dpred, drows * h->nsub));
  TRY(nalloc(h, &h->dblk, (size_t)nm * 4 * w * w));
  TRY(nalloc(h, &h->lpart, 1024));
  TRY(nalloc(h, &h->rec_x, (size_t)c.nrec));
  {
    const long wg = (long)Bm * h->split * (long)w * std::max(w, c.cin);
    const long cs1 = (((long)Bm * npix + 1023) / 1024) * w;
    const long cs2 = std::max((long)Bm * c.nrec * (long)c.hidden * std::max(w, h->nsub),
                              (((long)drows + 255) / 256) * std::max(h->nsub, c.hidden));
    h->partial_n = std::max(wg, std::max(cs1, cs2));
    TRY(nalloc(h, &h->partial, (size_t)h->partial_n));
  }
  TRY(build_dft(h));
  // initial parameters (seeded)
  {
    std::vector<float> p(h->P, 0.f);
    uint64_t s = seed ^ 0x5EED5EED12345678ULL;
    for (long i = 0; i < (long)c.cin * w; i++) p[h->oW0 + i] = uniform_pm(&s, 1.0f / sqrtf((float)c.cin));
    for (int l = 0; l < L; l++) {
      for (long i = 0; i < nm * w * w; i++) p[h->oWre[l] + i] = uniform_pm(&s, 1.0f / (float)w);
      for (long i = 0; i < nm * w * w; i++) p[h->oWim[l] + i] = uniform_pm(&s, 1.0f / (float)w);
      for (long i = 0; i < (long)w * w; i++) p[h->oW[l] + i] = uniform_pm(&s, 1.0f / sqrtf((float)w));
    }
    for (long i = 0; i < (long)w * c.hidden; i++) p[h->oW1 + i] = uniform_pm(&s, 1.0f / sqrtf((float)w));
    for (long i = 0; i < (long)c.hidden * h->nsub; i++) p[h->oW2 + i] = uniform_pm(&s, 1.0f / sqrtf((float)c.hidden));
    if (cudaMemcpy(h->params, p.data(), h->P * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(h->grads, 0, h->P * 4) != cudaSuccess || cudaMemset(h->adam_m, 0, h->P * 4) != cudaSuccess ||
        cudaMemset(h->adam_v, 0, h->P * 4) != cudaSuccess) {
      nfail(h, -2, "parameter upload failed");
      TRY(-2);
    }
    std::vector<int> rx(c.nrec);
    for (int r = 0; r < c.nrec; r++) rx[r] = (int)(((2 * r + 1) * (long)c.nx) / (2 * c.nrec));
    if (cudaMemcpy(h->rec_x, rx.data(), c.nrec * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
      nfail(h, -2, "receiver upload failed");
      TRY(-2);
    }
  }
  TRY(refresh_bf16(h));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) { nfail(h, -2, "set-up kernels failed"); TRY(-2); }
#undef TRY
  *out = h;
  return 0;
}

extern "C" int se2nn_set_stream(se2nn *h, void *stream)
{
  if (!h) return -1;
  NCK(h, cudaStreamSynchronize(h->stream));
  if (stream) h->stream = static_cast<cudaStream_t>(stream);
  return 0;
}

extern "C" int se2nn_get_params(se2nn *h, float *p)
{
  if (!h || !p) return -1;
  NCK(h, cudaStreamSynchronize(h->stream));
  NCK(h, cudaMemcpy(p, h->params, h->P * 4, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int se2nn_set_params(se2nn *h, const float *p)
{
  if (!h || !p) return -1;
  NCK(h, cudaStreamSynchronize(h->stream));
  NCK(h, cudaMemcpy(h->params, p, h->P * 4, cudaMemcpyHostToDevice));
  int rc = refresh_bf16(h);
  if (rc) return rc;
  NCK(h, cudaStreamSynchronize(h->stream));
  return 0;
}

extern "C" int se2nn_get_grads(se2nn *h, float *g)
{
  if (!h || !g) return -1;
  NCK(h, cudaStreamSynchronize(h->stream));
  NCK(h, cudaMemcpy(g, h->grads, h->P * 4, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int se2nn_set_receivers(se2nn *h, const int *rec_x)
{
  if (!h || !rec_x) return -1;
  for (int r = 0; r < h->c.nrec; r++)
    if (rec_x[r] < 0 || rec_x[r] >= h->c.nx) return nfail(h, -1, "receiver %d: cell %d outside 0..%d", r, rec_x[r], h->c.nx - 1);
  NCK(h, cudaStreamSynchronize(h->stream));
  NCK(h, cudaMemcpy(h->rec_x, rec_x, h->c.nrec * 4, cudaMemcpyHostToDevice));
  return 0;
}

static int check_batch(se2nn *h, int batch)
{
  if (batch < 1 || batch > h->c.max_batch) return nfail(h, -1, "batch %d outside 1..%d", batch, h->c.max_batch);
  return 0;
}

extern "C" int se2nn_forward(se2nn *h, const void *x_dev, int batch, float *out_dev)
{
  if (!h || !x_dev || !out_dev) return -1;
  int rc = check_batch(h, batch);
  if (rc) return rc;
  return forward(h, static_cast<const bf16 *>(x_dev), batch, out_dev);
}

extern "C" int se2nn_loss_grad(se2nn *h, const void *x_dev, int batch, const float *target_dev, double *loss,
                               float *out_dev)
{
  if (!h || !x_dev || !target_dev) return -1;
  int rc = check_batch(h, batch);
  if (rc) return rc;
  const bf16 *x = static_cast<const bf16 *>(x_dev);
  float *out = out_dev ? out_dev : h->out;
  if ((rc = forward(h, x, batch, out))) return rc;
  const long n = (long)batch * h->c.nrec * h->c.nout;
  const int nb = (int)std::min<long>(1024, (n + EW - 1) / EW);
  k_mse<<<nb, EW, 0, h->stream>>>(out, target_dev, n, h->lpart, h->dpred);
  NCK(h, cudaGetLastError());
  if ((rc = backward(h, x, batch))) return rc;
  std::vector<double> part(nb);
  NCK(h, cudaMemcpyAsync(part.data(), h->lpart, nb * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  NCK(h, cudaStreamSynchronize(h->stream));
  double s = 0.0;
  for (int i = 0; i < nb; i++) s += part[i];
  if (loss) *loss = s / (double)n;
  return 0;
}

extern "C" int se2nn_adam_step(se2nn *h, float lr, float beta1, float beta2, float eps, float weight_decay)
{
  if (!h) return -1;
  h->adam_t++;
  const float c1 = 1.f - powf(beta1, (float)h->adam_t), c2 = 1.f - powf(beta2, (float)h->adam_t);
  k_adam<<<nblk(h->P), EW, 0, h->stream>>>(h->params, h->grads, h->adam_m, h->adam_v, h->P, lr, beta1, beta2, eps,
                                            weight_decay, c1, c2);
  NCK(h, cudaGetLastError());
  return refresh_bf16(h);
}

extern "C" int se2nn_build_inputs(se2nn *h, const void *materials_dev, const float *src_dev, const int *idx_dev,
                                  int batch, float sigma_cells, void *x_dev)
{
  if (!h || !materials_dev || !src_dev || !idx_dev || !x_dev || !(sigma_cells > 0.f)) return -1;
  int rc = check_batch(h, batch);
  if (rc) return rc;
  k_build_inputs<<<nblk((long)batch * h->npix), EW, 0, h->stream>>>(
      static_cast<const float *>(materials_dev), src_dev, idx_dev, batch, h->c.ny, h->c.nx, h->c.cin,
      1.0f / (2.0f * sigma_cells * sigma_cells), static_cast<bf16 *>(x_dev));
  NCK(h, cudaGetLastError());
  return 0;
}

extern "C" int se2nn_gather_targets(se2nn *h, const float *targets_dev, const int *idx_dev, int batch, float *out_dev)
{
  if (!h || !targets_dev || !idx_dev || !out_dev) return -1;
  int rc = check_batch(h, batch);
  if (rc) return rc;
  const long row = (long)h->c.nrec * h->c.nout;
  k_gather_rows<<<nblk(batch * row), EW, 0, h->stream>>>(targets_dev, idx_dev, batch, row, out_dev);
  NCK(h, cudaGetLastError());
  return 0;
}

extern "C" int se2nn_set_tensor_path(int mode)
{
  if (mode < 0 || mode > 2) return -1;
  g_tc_path = mode;
  return 0;
}

extern "C" int se2nn_tensor_path_info(long out[3])
{
  if (!out) return -1;
  int flag = 0;   // (the current device's flag)
  if (cudaMemcpyFromSymbol(&flag, g_tc_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return -2;
  }
  out[0] = g_tc_launches.load();
  out[1] = g_mma_launches.load();
  out[2] = flag;
  return 0;
}

extern "C" int se2nn_gemm(const void *A_dev, const void *B_dev, float *C_dev, int M, int N, int K, int batch, long lda,
                          long ldb, long ldc, long sA, long sB, long sC, int transA, int transB, float alpha, float beta,
                          void *stream)
{
  if (!A_dev || !B_dev || !C_dev || M < 1 || N < 1 || K < 1 || batch < 1) return nfail(nullptr, -1, "bad GEMM arguments");
  GemmArgs g = mk(static_cast<const bf16 *>(A_dev), lda, sA, transA, static_cast<const bf16 *>(B_dev), ldb, sB, transB,
                  M, N, K, batch, C_dev, ldc, sC, 1);
  g.alpha = alpha;
  g.beta = beta;
  if (beta != 0.f) { g.Cin = C_dev; g.ldcin = ldc; g.sCin = sC; g.cin_f32 = 1; }
  cudaError_t e = launch_gemm(g, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return nfail(nullptr, -2, "GEMM launch: %s", cudaGetErrorString(e));
  return 0;
}
