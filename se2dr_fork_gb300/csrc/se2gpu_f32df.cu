// se2gpu_f32df.cu -- the persistent step kernel in the two-float mode (every value of a
// step carried as a float pair, about 48 significant bits), degrees 1..8, over the same
// tile configurations as the plain and Kahan modes.  A translation unit of its own:
// the kernels are large and compile in parallel with the others, and this unit's
// constant tables (high and low parts of D and the GLL weights) are set here.
#include "se2gpu_persist.cuh"
#include "se2gpu_persist_launch.h"

namespace se2p {

cudaError_t df_set_tables(int p, const double *D, const double *w1d)
{
  float dh[81] = {0}, dl[81] = {0}, wh[9] = {0}, wl[9] = {0};
  const int n1 = p + 1;
  for (int i = 0; i < n1 * n1; i++) {
    dh[i] = (float)D[i];
    dl[i] = (float)(D[i] - (double)dh[i]);
  }
  for (int i = 0; i < n1; i++) {
    wh[i] = (float)w1d[i];
    wl[i] = (float)(w1d[i] - (double)wh[i]);
  }
  const size_t od = sizeof(dh) * (p - 1), ow = sizeof(wh) * (p - 1);
  cudaError_t e = cudaMemcpyToSymbol(c_D, dh, sizeof(dh), od);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_Dl, dl, sizeof(dl), od);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_w, wh, sizeof(wh), ow);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_wl, wl, sizeof(wl), ow);
  return e;
}

namespace {

struct DfEntry {
  int p, te, nt;
  size_t smem;
  const void *fn;
};

// registers sized for 2 CTAs per SM at most (1 with 384 threads or more): the pairs
// double most live values
template <int P, int TE, int NT, bool WE>
DfEntry df_entry()
{
  typedef Layout<P, TE, true, 1, true> L;
  constexpr int MS = min_blocks(L::TOTAL);
  constexpr int M = (NT >= 384) ? 1 : (MS < 2 ? MS : 2);
  return DfEntry{P, TE, NT, L::TOTAL, (const void *)persist_step<P, TE, NT, true, 1, M, true, WE>};
}

const DfEntry *df_table(int *n)
{
#define SE2P_DF_ENTRY(P, TE, NT, NOB, MINB, WE) df_entry<P, TE, NT, (WE) != 0>(),
  static DfEntry t[] = {SE2P_CONFIGS(SE2P_DF_ENTRY)};
#undef SE2P_DF_ENTRY
  *n = (int)(sizeof(t) / sizeof(t[0]));
  return t;
}

template <int P>
cudaError_t record_t(const Params &prm, cudaStream_t st)
{
  persist_record<P, true><<<1, 128, 0, st>>>(prm);
  return cudaGetLastError();
}

}  // namespace

const void *df_kernel(int p, int config, size_t *smem)
{
  int n, k = 0;
  const DfEntry *t = df_table(&n);
  for (int i = 0; i < n; i++)
    if (t[i].p == p) {
      if (k == config) {
        if (smem) *smem = t[i].smem;
        return t[i].fn;
      }
      k++;
    }
  return nullptr;
}

cudaError_t df_launch_record(int p, const Params &prm, cudaStream_t st)
{
  switch (p) {
    case 1: return record_t<1>(prm, st); case 2: return record_t<2>(prm, st);
    case 3: return record_t<3>(prm, st); case 4: return record_t<4>(prm, st);
    case 5: return record_t<5>(prm, st); case 6: return record_t<6>(prm, st);
    case 7: return record_t<7>(prm, st); case 8: return record_t<8>(prm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace se2p
