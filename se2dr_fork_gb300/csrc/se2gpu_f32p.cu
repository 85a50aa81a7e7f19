// se2gpu_f32p.cu -- persistent TMA-pipelined FP32 kernels (plain / Kahan; the two-float mode is
// in se2gpu_f32df.cu), degrees 1..8, the tile configurations the autotuner chooses from, and
// their host-side helpers (tensor maps, constant tables, norms of the leapfrog state).
#include <cudaTypedefs.h>

#include "se2gpu_persist.cuh"
#include "se2gpu_persist_launch.h"

namespace se2p {

cudaError_t set_tables(int p, const double *D, const double *w1d)
{
  float d[81] = {0}, w[9] = {0};
  const int n1 = p + 1;
  for (int i = 0; i < n1 * n1; i++) d[i] = (float)D[i];
  for (int i = 0; i < n1; i++) w[i] = (float)w1d[i];
  cudaError_t e = cudaMemcpyToSymbol(c_D, d, sizeof(d), sizeof(d) * (p - 1));
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_w, w, sizeof(w), sizeof(w) * (p - 1));
  if (e != cudaSuccess) return e;
  return df_set_tables(p, D, w1d);
}

// ---- one configuration = (degree, elements per tile edge, threads) ----------
struct Entry {
  int p, te, nt, nob;
  size_t smem[2];                 // [kahan]
  size_t bsmem[2];                // batched kernel [kahan]
  const void *fn[2];              // persist_step<...> [kahan]
  const void *bfn[2];             // persist_batch<...> [kahan]
};

template <int P, int TE, int NT, int NOB = owned_buffers(P), int MINB = 0, bool WE = false>
static Entry entry()
{
  constexpr int M0 = MINB ? MINB : min_blocks(Layout<P, TE, false, NOB, false, true>::TOTAL);
  constexpr int M1 = MINB ? MINB : min_blocks(Layout<P, TE, true, NOB, false, true>::TOTAL);
  constexpr int B0 = MINB ? MINB : min_blocks(Layout<P, TE, false, NOB>::BATCH_TOTAL);
  constexpr int B1 = MINB ? MINB : min_blocks(Layout<P, TE, true, NOB>::BATCH_TOTAL);
  Entry e;
  e.p = P; e.te = TE; e.nt = NT; e.nob = NOB;
  e.smem[0] = Layout<P, TE, false, NOB, false, true>::TOTAL;
  e.smem[1] = Layout<P, TE, true, NOB, false, true>::TOTAL;
  e.bsmem[0] = Layout<P, TE, false, NOB>::BATCH_TOTAL;
  e.bsmem[1] = Layout<P, TE, true, NOB>::BATCH_TOTAL;
  e.fn[0] = (const void *)persist_step<P, TE, NT, false, NOB, M0, false, WE>;
  e.fn[1] = (const void *)persist_step<P, TE, NT, true, NOB, M1, false, WE>;
  e.bfn[0] = (const void *)persist_batch<P, TE, NT, false, NOB, B0, WE>;
  e.bfn[1] = (const void *)persist_batch<P, TE, NT, true, NOB, B1, WE>;
  return e;
}

static const Entry *table(int *n)
{
#define SE2P_ENTRY(P, TE, NT, NOB, MINB, WE) entry<P, TE, NT, (NOB) ? (NOB) : owned_buffers(P), MINB, (WE) != 0>(),
  static Entry t[] = {SE2P_CONFIGS(SE2P_ENTRY)};
#undef SE2P_ENTRY
  *n = (int)(sizeof(t) / sizeof(t[0]));
  return t;
}

static const Entry *find(int p, int config)
{
  int n, k = 0;
  const Entry *t = table(&n);
  for (int i = 0; i < n; i++)
    if (t[i].p == p) {
      if (k == config) return &t[i];
      k++;
    }
  return nullptr;
}

// the configuration a handle starts with: per degree the one the autotuner measured
// fastest on GB300 at about 16M nodes (and, at degree 4, at the 2048^2 workload)
int default_config(int p)
{
  static const int best[8] = {2, 0, 2, 1, 2, 0, 2, 1};
  return (p >= 1 && p <= 8 && best[p - 1] < num_configs(p)) ? best[p - 1] : 0;
}

int num_configs(int p)
{
  int n, k = 0;
  const Entry *t = table(&n);
  for (int i = 0; i < n; i++) k += (t[i].p == p);
  return k;
}

int config_shape(int p, int config, int mode, TileShape *s)
{
  const Entry *e = find(p, config);
  if (!e) return -1;
  size_t df_smem = 0;
  if (mode == MODE_DF && !df_kernel(p, config, &df_smem)) return -1;
  s->tex = s->tey = e->te;
  s->nt = e->nt;
  s->region_w = round_up((e->te + 1) * p + 2 + ((p & 1) ? 2 : 0), 2);
  s->region_h = (e->te + 1) * p + 1;
  s->own_w = round_up(e->te * p + 2, 2);
  s->own_h = e->te * p + 1;
  s->cell_box = e->te + 1;
  s->minv_w = round_up(e->te * p + 1 + 4, 4);
  s->owned_buffers = (mode == MODE_DF) ? 1 : e->nob;
  s->smem = (mode == MODE_DF) ? df_smem : e->smem[mode ? 1 : 0];
  return 0;
}

cudaError_t prepare(int p, int config, int mode)
{
  const Entry *e = find(p, config);
  if (!e) return cudaErrorInvalidValue;
  const int k = mode ? 1 : 0;
  size_t df_smem = 0;
  const void *dfn = (mode == MODE_DF) ? df_kernel(p, config, &df_smem) : nullptr;
  if (mode == MODE_DF && !dfn) return cudaErrorInvalidValue;
  const void *fns[2] = {dfn ? dfn : e->fn[k], e->bfn[k]};
  const size_t sizes[2] = {dfn ? df_smem : e->smem[k], e->bsmem[k]};
  for (int i = 0; i < 2; i++) {
    const void *fn = fns[i];
    cudaError_t r = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizes[i]);
    if (r != cudaSuccess) return r;
    r = cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (r != cudaSuccess) return r;
  }
  return cudaSuccess;
}

int occupancy(int p, int config, int mode, bool batch)
{
  const Entry *e = find(p, config);
  int n = 0;
  if (!e) return 1;
  const int k = mode ? 1 : 0;
  const void *fn = (batch ? e->bfn : e->fn)[k];
  size_t smem = (batch ? e->bsmem : e->smem)[k];
  if (mode == MODE_DF && !batch) fn = df_kernel(p, config, &smem);
  if (!fn || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, e->nt, smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n;
}

cudaError_t launch_step(int p, int config, int mode, const CUtensorMap *maps, const Params &prm, int grid,
                        cudaStream_t st)
{
  const Entry *e = find(p, config);
  if (!e) return cudaErrorInvalidValue;
  const void *fn = e->fn[mode ? 1 : 0];
  size_t smem = e->smem[mode ? 1 : 0];
  if (mode == MODE_DF) fn = df_kernel(p, config, &smem);
  if (!fn) return cudaErrorInvalidValue;
  Params pc = prm;
  CUtensorMap m0 = maps[0], m1 = maps[1], m2 = maps[2], m3 = maps[3], m4 = maps[4], m5 = maps[5];
  void *args[] = {&m0, &m1, &m2, &m3, &m4, &m5, &pc};
  return cudaLaunchKernel(fn, dim3(grid), dim3(e->nt), args, smem, st);
}

cudaError_t launch_batch(int p, int config, bool kahan, const BatchArgs &ba, int grid, cudaStream_t st)
{
  const Entry *e = find(p, config);
  if (!e) return cudaErrorInvalidValue;
  BatchArgs a = ba;
  void *args[] = {&a};
  return cudaLaunchKernel(e->bfn[kahan ? 1 : 0], dim3(grid), dim3(e->nt), args, e->bsmem[kahan ? 1 : 0], st);
}

template <int P>
static cudaError_t record_batch_t(const Params *shots, int nshots, int kblk, cudaStream_t st)
{
  persist_record_batch<P><<<nshots, 128, 0, st>>>(shots, nshots, kblk);
  return cudaGetLastError();
}
cudaError_t launch_record_batch(int p, const Params *shots, int nshots, int kblk, cudaStream_t st)
{
  if (nshots <= 0) return cudaSuccess;
  switch (p) {
    case 1: return record_batch_t<1>(shots, nshots, kblk, st); case 2: return record_batch_t<2>(shots, nshots, kblk, st);
    case 3: return record_batch_t<3>(shots, nshots, kblk, st); case 4: return record_batch_t<4>(shots, nshots, kblk, st);
    case 5: return record_batch_t<5>(shots, nshots, kblk, st); case 6: return record_batch_t<6>(shots, nshots, kblk, st);
    case 7: return record_batch_t<7>(shots, nshots, kblk, st); case 8: return record_batch_t<8>(shots, nshots, kblk, st);
    default: return cudaErrorInvalidValue;
  }
}

template <int P>
static cudaError_t record_t(const Params &prm, cudaStream_t st)
{
  persist_record<P><<<1, 128, 0, st>>>(prm);
  return cudaGetLastError();
}
cudaError_t launch_record(int p, const Params &prm, cudaStream_t st, bool df)
{
  if (df) return df_launch_record(p, prm, st);
  switch (p) {
    case 1: return record_t<1>(prm, st); case 2: return record_t<2>(prm, st);
    case 3: return record_t<3>(prm, st); case 4: return record_t<4>(prm, st);
    case 5: return record_t<5>(prm, st); case 6: return record_t<6>(prm, st);
    case 7: return record_t<7>(prm, st); case 8: return record_t<8>(prm, st);
    default: return cudaErrorInvalidValue;
  }
}

// tensor map of one padded float2 field, box (bw, bh) nodes
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int encoder()
{
  if (!g_encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return -1;
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  return 0;
}

int make_map(CUtensorMap *map, void *base, int nx, int ny, int pitch, int bw, int bh)
{
  if (encoder()) return -1;
  cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * 8};
  cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -(int)r - 1000;
}

int make_map_f32(CUtensorMap *map, void *base, int nx, int ny, int pitch, int bw, int bh)
{
  if (encoder()) return -1;
  cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * 4};
  cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -(int)r - 1000;
}

int make_map_cells(CUtensorMap *map, void *base, int mx, int my, int box)
{
  if (encoder()) return -1;
  cuuint64_t dims[3] = {4, (cuuint64_t)mx, (cuuint64_t)my};
  cuuint64_t strides[2] = {16, (cuuint64_t)mx * 16};
  cuuint32_t bx[3] = {4, (cuuint32_t)box, (cuuint32_t)box};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, bx, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -(int)r - 1000;
}

// norms of (u_k, v_k) recovered from the leapfrog state in FP64:
// u_k = (u - cu) - dt (w - cw),  v_k = (w - cw) - dt/2 a_k
__global__ void norms_leapfrog(const float2 *u, const float2 *w, const float2 *cu, const float2 *cw, const float2 *a,
                               const float2 *al, int nx, int ny, int pitch, double dt, double half_dt, double *part)
{
  __shared__ double s[6][256];
  double umax = -1.0e308, umin = 1.0e308, uss = 0.0, vmax = -1.0e308, vmin = 1.0e308, vss = 0.0;
  const long n = (long)nx * ny;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long y = i / nx, x = i - y * nx, k = y * pitch + x;
    const float2 uu = u[k], ww = w[k], aa = a[k], aal = al ? al[k] : make_float2(0.f, 0.f);
    const float2 cuu = cu ? cu[k] : make_float2(0.f, 0.f), cww = cw ? cw[k] : make_float2(0.f, 0.f);
    const double wx = (double)ww.x - (double)cww.x, wy = (double)ww.y - (double)cww.y;
    const double ux = ((double)uu.x - (double)cuu.x) - dt * wx, uy = ((double)uu.y - (double)cuu.y) - dt * wy;
    const double vx = wx - half_dt * ((double)aa.x + (double)aal.x), vy = wy - half_dt * ((double)aa.y + (double)aal.y);
    umax = fmax(umax, fmax(ux, uy)); umin = fmin(umin, fmin(ux, uy)); uss += ux * ux + uy * uy;
    vmax = fmax(vmax, fmax(vx, vy)); vmin = fmin(vmin, fmin(vx, vy)); vss += vx * vx + vy * vy;
  }
  s[0][threadIdx.x] = umax; s[1][threadIdx.x] = umin; s[2][threadIdx.x] = uss;
  s[3][threadIdx.x] = vmax; s[4][threadIdx.x] = vmin; s[5][threadIdx.x] = vss;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      const int t = threadIdx.x;
      s[0][t] = fmax(s[0][t], s[0][t + h]); s[1][t] = fmin(s[1][t], s[1][t + h]); s[2][t] += s[2][t + h];
      s[3][t] = fmax(s[3][t], s[3][t + h]); s[4][t] = fmin(s[4][t], s[4][t + h]); s[5][t] += s[5][t + h];
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

cudaError_t launch_norms(const float2 *u, const float2 *w, const float2 *cu, const float2 *cw, const float2 *a,
                         const float2 *al, int nx, int ny, int pitch, double dt, double *part, int nblocks,
                         cudaStream_t st)
{
  norms_leapfrog<<<nblocks, 256, 0, st>>>(u, w, cu, cw, a, al, nx, ny, pitch, dt, 0.5 * dt, part);
  return cudaGetLastError();
}

// The step kernels' bounded wait and error flag, on an mbarrier that nothing arrives
// at: the wait gives up after EXPIRY_TEST_POLLS polls and the kernel raises the flag,
// as a step kernel does when its tile copies never land.  No copy is in flight, so
// the CTA exits normally.  ns[0] = the wait's duration (globaltimer).
__global__ void wait_expiry_test(int *err, unsigned long long *ns)
{
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  fence_barrier_init();
  unsigned long long t0, t1;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  const bool ok = mbar_wait_bounded<EXPIRY_TEST_POLLS>(b, 0);
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
  if (!ok) atomicExch(err, 1);
  ns[0] = t1 - t0;
}

cudaError_t launch_wait_expiry_test(int *err, unsigned long long *ns, cudaStream_t st)
{
  wait_expiry_test<<<1, 32, 0, st>>>(err, ns);
  return cudaGetLastError();
}

}  // namespace se2p
