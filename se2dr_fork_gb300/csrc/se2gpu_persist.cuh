// se2gpu_persist.cuh -- persistent, TMA-pipelined FP32 step kernel for sm_103a.
//
// FP32 modes advance the same explicit Newmark (beta = 0, gamma = 1/2) scheme as
// se2wave.c:4722-4775, written as kick-drift leapfrog so that a step needs the
// neighbours' displacement only:
//
//   state before step k: u_k, w_k = v_{k-1} + dt/2 a_{k-1}          (half-step velocity)
//   a_k     = M^-1 (K u_k + sum_s stf_s(t_k) g_s)
//   v_k     = w_k + dt/2 a_k                                        (recorded at receivers)
//   w_{k+1} = w_k + dt a_k,   u_{k+1} = u_k + dt w_{k+1}             (Kahan-compensated)
//
// which is algebraically identical to the reference's u += dt v + dt^2/2 a,
// v += dt/2 a, a = f/M, v += dt/2 a.  Per node and step the kernel reads u, w
// (+ compensations cu, cw) and writes them back: 68.5 B/node with Kahan terms.
//
// Execution: a persistent grid (CTAs resident on every SM) walks the tiles.  A
// tile is TE x TE elements; its CTA owns their nodes except the line shared
// with the next tile, and recomputes the one-element halo column/row on its
// left/bottom whose forces reach its boundary nodes.  Thread 0 issues 2-D TMA
// bulk-tensor copies of the next tile's node region (u, cu) and owned nodes
// (w, cw) into the second shared-memory stage, signalled through an mbarrier,
// while all threads compute the current tile.  Every wait is bounded: on
// timeout the CTA records an error code, waits (bounded) for its own copies and
// returns.
//
// Per tile, one thread per (element, line j) -- NT covers every item, so all
// per-item values stay in registers between the three phases:
//   1. along row j: d/dxi at the row's GLL points; along column j: d/deta at
//      the column's points (to shared memory).  Derivatives are taken of the
//      compensated displacement relative to the line's first node,
//      (u_k - u_0) - (cu_k - cu_0): differences of nearby values are exact, so
//      the derivative of a smooth field loses no digits to cancellation;
//   2. Hooke stress at the row's points, scaled by -detJ w_q; the xi part of
//      the weak divergence from registers, the eta fluxes to shared memory;
//   3. the eta part of the divergence for the row's nodes; element forces to
//      shared memory.
// Then one thread per owned node sums the 1, 2 or 4 element contributions in a
// fixed order (deterministic, no atomics), adds the sources and updates.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "se2gpu_persist_params.h"

namespace se2p {

// FP32 derivative matrix and GLL weights per degree, in constant memory so that
// compile-time indices become constant-bank operands (this header is compiled
// into one translation unit only)
__constant__ float c_D[8][81];
__constant__ float c_w[8][9];
// their low parts (FP64 value - FP32 value, rounded to FP32) for the two-float mode
__constant__ float c_Dl[8][81];
__constant__ float c_wl[8][9];

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
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
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
// plain bulk copy (16-byte aligned addresses, a multiple of 16 bytes)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"((uint64_t)src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap *map)
{
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// bounded wait on a tile's copies (LIMIT polls; a smaller limit serves the expiry
// self-test).  A poll of a barrier whose phase does not complete returns after the
// hardware's suspend limit, measured at 3.75 us on GB300, so 2^18 polls give up
// after about one second; copies that land take microseconds.
constexpr long WAIT_LIMIT = 1L << 18;
template <long LIMIT = WAIT_LIMIT>
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
  for (long i = 0; i < LIMIT; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---------------------------------------------------------------- geometry
__host__ __device__ constexpr int round_up(int x, int m) { return (x + m - 1) / m * m; }

template <int P, int TE>
struct Geo {
  static constexpr int N1 = P + 1, NPE = N1 * N1;
  // element stride of the exchange buffers: (p+1)^2 node values plus a pad that spreads
  // the elements a warp touches over the 32 banks (with (p+1)^2 = 16 at p = 3 every
  // element would start on bank 0; pads chosen with a wavefront model of the kernel's
  // accesses)
  static constexpr int XS = NPE + (P == 1 ? 2 : P == 3 ? 3 : P == 6 ? 6 : P == 7 ? 7 : P == 8 ? 8 : 0);
  // the plain and Kahan tile body's exchange buffers: element stride XSK and the stride RS of
  // an element's rows (point (a, b) at a + b RS).  At degree 4 rows of 6 in elements of 37
  // float2: the same wavefront count gives 9-10 % fewer exchange-buffer wavefronts than
  // rows of 5 in elements of 25 for 6x6, 7x7 and 8x8 tiles (the two-float body keeps XS)
  static constexpr int RS = (P == 4) ? 6 : N1;
  static constexpr int XSK = (P == 4) ? 37 : XS;
  static constexpr int NEX = TE + 1, NE = NEX * NEX;      // elements incl. halo
  static constexpr int ITEMS = NE * N1;                   // (element, line) work items
  // warp-aligned mapping: EPW whole elements per warp (their N1 lines in consecutive
  // lanes), NW warps; the element phases then exchange values within a warp only
  static constexpr int EPW = 32 / N1;
  static constexpr int NW = (NE + EPW - 1) / EPW;
  // region box (u, cu): the x start is rounded down to an even node so the copy
  // starts on a 16-byte boundary; one extra column absorbs the shift and two
  // more keep the node phase's paired (16-byte) reads inside the box
  static constexpr int BXW = round_up(NEX * P + 2 + ((P & 1) ? 2 : 0), 2);
  static constexpr int BXH = NEX * P + 1;
  static constexpr int OWM = TE * P + 1;                  // owned nodes per row (max)
  static constexpr int OBW = round_up(OWM + 1, 2);        // owned box (w, cw)
  static constexpr int OBH = OWM;
  static constexpr int PW = OBW / 2;                      // node pairs per owned row
  static constexpr int NPAIR = OWM * PW;
  // 1/M box (floats): the x start rounded down to a multiple of 4 (16 bytes); wide enough
  // for the owned nodes and the paired reads' second node
  static constexpr int MBW = round_up(OWM + 4, 4);
};

__host__ __device__ constexpr size_t al128(size_t x) { return (x + 127) & ~size_t(127); }

// owned-box buffers of the tile configurations that name none: 2 up to degree 3 (the
// next tile's w, cw arrive with its region, a whole tile ahead), 1 above (the current
// tile's arrive during its element phases; the smaller footprint fits 2 CTAs per SM at
// degree 8 instead of 1).  Degree 4 runs fastest with two (its configuration 1).
__host__ __device__ constexpr int owned_buffers(int p) { return p <= 3 ? 2 : 1; }

template <int P, int TE, bool KAHAN, int NOB = owned_buffers(P), bool DF = false, bool AC = false>
struct Layout {
  typedef Geo<P, TE> G;
  static constexpr size_t REG = al128(sizeof(float2) * G::BXW * G::BXH);
  static constexpr size_t OWN = al128(sizeof(float2) * G::OBW * G::OBH);
  // AC: the per-tile constants arrive with the copies too -- the cell constants of the
  // tile's elements (float4 per cell) with the region, 1/M of the owned nodes and the
  // tile's source/receiver bounds (int4) with the owned boxes
  static constexpr size_t CELLB = AC ? al128(sizeof(float4) * G::NEX * G::NEX) : 0;
  static constexpr size_t MINVB = AC ? al128(sizeof(float) * G::MBW * G::OBH) : 0;
  static constexpr size_t BNDB = AC ? 128 : 0;
  // the region boxes (u and cu) are double-buffered: the next tile's arrive while this
  // tile is computed.  The owned boxes (w and cw) are read only by the node phase:
  // NOB = 2 buffers hold this tile's and the next's, NOB = 1 this tile's only.
  static constexpr size_t STAGE = REG * (KAHAN ? 2 : 1) + CELLB;
  static constexpr size_t OWNB = OWN * (KAHAN ? 2 : 1) + MINVB + BNDB;
  // exchange buffer: float2 per point, float4 (two-float x, y) in the two-float mode
  static constexpr size_t XCH = al128(DF ? sizeof(float4) * G::NE * G::XS : sizeof(float2) * G::NE * G::XSK);
  static constexpr size_t MISC = 64;
  static constexpr size_t TOTAL = 2 * STAGE + NOB * OWNB + 2 * XCH + MISC;
  static constexpr size_t BATCH_TOTAL = TOTAL;   // the batched kernel's shot parameters are a kernel parameter
  static constexpr uint32_t TX_REGION =
      (uint32_t)((KAHAN ? 2 : 1) * sizeof(float2) * G::BXW * G::BXH + (AC ? sizeof(float4) * G::NEX * G::NEX : 0));
  static constexpr uint32_t TX_OWNED =
      (uint32_t)((KAHAN ? 2 : 1) * sizeof(float2) * G::OBW * G::OBH + (AC ? sizeof(float) * G::MBW * G::OBH + 16 : 0));
};

// CTAs per SM the register budget is sized for: as many as the shared memory allows (up
// to 3; 228 KB per SM, 1 KB reserved per CTA).  Three CTAs cap small tiles at 65536 /
// (3 NT) registers, which they fit without spilling, and hide more shared-memory latency.
__host__ __device__ constexpr int min_blocks(size_t smem)
{
  return (3 * (smem + 1024) <= 233472) ? 3 : (2 * (smem + 1024) <= 233472) ? 2 : 1;
}

struct TileBox {
  int ex0, ex1, ey0, ey1, EX0, EY0, NEXa, NEYa, X0, Y0, OW, OH, RXa, RYa, OXa;
};

template <int P, int TE>
__device__ __forceinline__ TileBox tile_box(const Params &prm, int tx, int ty)
{
  TileBox b;
  b.ex0 = tx * TE; b.ex1 = min(b.ex0 + TE, prm.mx);
  b.ey0 = ty * TE; b.ey1 = min(b.ey0 + TE, prm.my);
  b.EX0 = max(b.ex0 - 1, 0); b.EY0 = max(b.ey0 - 1, 0);
  b.NEXa = b.ex1 - b.EX0; b.NEYa = b.ey1 - b.EY0;
  b.X0 = b.ex0 * P; b.Y0 = b.ey0 * P;
  b.OW = (b.ex1 - b.ex0) * P + (b.ex1 == prm.mx ? 1 : 0);
  b.OH = (b.ey1 - b.ey0) * P + (b.ey1 == prm.my ? 1 : 0);
  b.RXa = (b.EX0 * P) & ~1;     // region box origin (even x)
  b.RYa = b.EY0 * P;
  b.OXa = b.X0 & ~1;            // owned box origin (even x)
  return b;
}

// TMA copies of tile (tx, ty).  The box origins depend only on the tile coordinates
// (the same formulas as tile_box); boxes reaching past the mesh read the tensor maps'
// zero fill.  issue_region: the u (and cu) region box into a stage; issue_owned: the w
// (and cw) owned box into the owned buffer.  AC: the cell box (tm_c: float4 per cell,
// from the region's first element) after the region, and the 1/M box (tm_m) and the
// tile's bounds (tb) after the owned boxes.
template <int P, int TE, bool KAHAN, bool AC = false>
__device__ __forceinline__ void region_boxes(int tx, int ty, unsigned char *stage, uint32_t bar,
                                             const CUtensorMap *tm_u, const CUtensorMap *tm_cu, const CUtensorMap *tm_c)
{
  typedef Layout<P, TE, KAHAN, 1, false, AC> L;
  const int ex0 = tx * TE, ey0 = ty * TE;
  const int RXa = (max(ex0 - 1, 0) * P) & ~1, RYa = max(ey0 - 1, 0) * P;
  tma_load_2d(smem_u32(stage), tm_u, RXa, RYa, bar);
  if (KAHAN) tma_load_2d(smem_u32(stage + L::REG), tm_cu, RXa, RYa, bar);
  if (AC) tma_load_3d(smem_u32(stage + L::REG * (KAHAN ? 2 : 1)), tm_c, 0, max(ex0 - 1, 0), max(ey0 - 1, 0), bar);
}

// (one arrive per barrier phase, with every byte the phase's copies bring)
template <int P, int TE, bool KAHAN, bool AC = false>
__device__ __forceinline__ void issue_region(int tx, int ty, unsigned char *stage, uint32_t bar,
                                             const CUtensorMap *tm_u, const CUtensorMap *tm_cu,
                                             const CUtensorMap *tm_c = nullptr)
{
  mbar_expect_tx(bar, Layout<P, TE, KAHAN, 1, false, AC>::TX_REGION);
  region_boxes<P, TE, KAHAN, AC>(tx, ty, stage, bar, tm_u, tm_cu, tm_c);
}

template <int P, int TE, bool KAHAN, bool AC = false>
__device__ __forceinline__ void issue_owned_boxes(int tx, int ty, unsigned char *ob, uint32_t bar,
                                                  const CUtensorMap *tm_w, const CUtensorMap *tm_cw,
                                                  const CUtensorMap *tm_m, const int4 *tb)
{
  typedef Layout<P, TE, KAHAN, 1, false, AC> L;
  const int X0 = tx * TE * P, Y0 = ty * TE * P;
  tma_load_2d(smem_u32(ob), tm_w, X0 & ~1, Y0, bar);
  if (KAHAN) tma_load_2d(smem_u32(ob + L::OWN), tm_cw, X0 & ~1, Y0, bar);
  if (AC) {
    tma_load_2d(smem_u32(ob + L::OWN * (KAHAN ? 2 : 1)), tm_m, X0 & ~3, Y0, bar);
    bulk_load(smem_u32(ob + L::OWN * (KAHAN ? 2 : 1) + L::MINVB), tb, 16, bar);
  }
}

// the region and owned boxes of one tile on one barrier (two owned buffers)
template <int P, int TE, bool KAHAN, bool AC = false>
__device__ __forceinline__ void issue_both(int tx, int ty, unsigned char *stage, unsigned char *ob, uint32_t bar,
                                           const CUtensorMap *tm_u, const CUtensorMap *tm_cu,
                                           const CUtensorMap *tm_w, const CUtensorMap *tm_cw,
                                           const CUtensorMap *tm_c = nullptr, const CUtensorMap *tm_m = nullptr,
                                           const int4 *tb = nullptr)
{
  typedef Layout<P, TE, KAHAN, 1, false, AC> L;
  mbar_expect_tx(bar, L::TX_REGION + L::TX_OWNED);
  region_boxes<P, TE, KAHAN, AC>(tx, ty, stage, bar, tm_u, tm_cu, tm_c);
  issue_owned_boxes<P, TE, KAHAN, AC>(tx, ty, ob, bar, tm_w, tm_cw, tm_m, tb);
}

template <int P, int TE, bool KAHAN, bool AC = false>
__device__ __forceinline__ void issue_owned(int tx, int ty, unsigned char *ob, uint32_t bar,
                                            const CUtensorMap *tm_w, const CUtensorMap *tm_cw,
                                            const CUtensorMap *tm_m = nullptr, const int4 *tb = nullptr)
{
  typedef Layout<P, TE, KAHAN, 1, false, AC> L;
  mbar_expect_tx(bar, L::TX_OWNED);
  issue_owned_boxes<P, TE, KAHAN, AC>(tx, ty, ob, bar, tm_w, tm_cw, tm_m, tb);
}

// the P + 1 nodes of an element row from the region box (even P: p is 16-byte aligned)
template <int P>
__device__ __forceinline__ void row_nodes(const float2 *p, float2 (&r)[P + 1])
{
  if constexpr ((P & 1) == 0) {
#pragma unroll
    for (int k = 0; k < P; k += 2) {
      const float4 v = *reinterpret_cast<const float4 *>(p + k);
      r[k] = make_float2(v.x, v.y);
      r[k + 1] = make_float2(v.z, v.w);
    }
    r[P] = p[P];
  } else {
#pragma unroll
    for (int k = 0; k <= P; k++) r[k] = p[k];
  }
}

__device__ __forceinline__ void kahan_add(float &s, float &c, float inc)
{
  const float y = inc - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// receiver rows of the previous step from the side buffer (u, v, a per element node)
// (two-float mode: 12 values per node, the value being high + low)
template <int P, bool DF = false>
__device__ void sample_rows(const Params &prm, const float *rbuf_in, double *trace_row)
{
  constexpr int N1 = P + 1, NPE = N1 * N1, NV = DF ? 12 : 6;
  for (int r = threadIdx.x; r < prm.nrec; r += blockDim.x) {
    const float *rb = rbuf_in + (size_t)r * NPE * NV;
    auto val = [&](int node, int c) { return DF ? (double)rb[node * NV + c] + (double)rb[node * NV + 6 + c] : (double)rb[node * NV + c]; };
    const int g = prm.rec_gll[r], eid = prm.rec_elem[r];
    const int ga = g % N1, gb = g / N1, ex = eid % prm.mx, ey = eid / prm.mx;
    double *o = trace_row + 7 * r;
    for (int c = 0; c < 6; c++) o[c] = val(g, c);
    const double ix = prm.iJ00d[ex], iy = prm.iJ11d[ey];
    double dvxdy = 0.0, dvydx = 0.0;
    for (int k = 0; k < N1; k++) {
      dvxdy += (iy * prm.Dd[gb * N1 + k]) * val(ga + k * N1, 2);
      dvydx += (ix * prm.Dd[ga * N1 + k]) * val(k + gb * N1, 3);
    }
    o[6] = dvydx - dvxdy;
  }
}

// the pointers of one step of a tile's shot: this step's source values, the receiver
// side buffer it writes and the optional a_k output (null: not written)
struct StepPtrs {
  const double *stf;
  float *rbuf_out;
  float2 *a_out;
};

// one tile: prefetch of global values, wait for the tile's copies, the three
// element phases and the node phase.  Returns false when the bounded wait expired.
// WE: the warp-aligned item mapping (every element's lines in one warp), whose element
// phases synchronise within the warp instead of the block.  AC: the tile's constants are
// in shared memory, after its region and owned boxes (see Layout).
template <int P, int TE, int NT, bool KAHAN, bool OWAIT, bool WE = false, bool AC = false>
__device__ __forceinline__ bool tile_body(const Params &prm, const StepPtrs stp, int tx, int ty, const unsigned char *st, uint32_t bar,
                                          uint32_t parity, const unsigned char *ob, uint32_t bar_o, uint32_t par_o,
                                          float2 *X1, float2 *X2, bool valid, int el, int j, int ecx, int ecy, float wj)
{
  typedef Geo<P, TE> G;
  typedef Layout<P, TE, KAHAN, 1, false, AC> L;
  constexpr int N1 = G::N1, NPE = G::NPE, NEX = G::NEX, BXW = G::BXW, OBW = G::OBW, XS = G::XSK, RS = G::RS;
  const float *D = c_D[P - 1];
  const float *W = c_w[P - 1];
  const TileBox b = tile_box<P, TE>(prm, tx, ty);
  const int t = ty * prm.ntx + tx;
  const int xoff = b.EX0 * P - b.RXa;   // region-box column of the first region node
  const bool active = valid && (ecx < b.NEXa) && (ecy < b.NEYa);
  const int ex = b.EX0 + ecx, ey = b.EY0 + ecy;
  // without AC, global loads issued before the wait: the element's constants, the tile's
  // source/receiver bounds and 1/M of this thread's owned nodes.  The barrier after the
  // wait holds every thread until its loads in flight have landed (measured: a sixth of
  // the step at degree 4), so with AC these arrive with the tile's copies instead.
  float4 ccg = make_float4(0.f, 0.f, 0.f, 0.f);
  int4 bnd = make_int4(0, 0, 0, 0);
  if constexpr (!AC) {
    if (active) ccg = prm.cellc[(size_t)ey * prm.mx + ex];
    bnd = prm.tile_bounds[t];
  }
  // node phase granularity: pairs of adjacent nodes (16-byte accesses), or single nodes strided
  // by NT (8-byte accesses, still coalesced) when that lowers the most nodes any thread handles
  constexpr int NOWN = G::OWM * G::OWM;
  constexpr bool SINGLE = ((NOWN + NT - 1) / NT) < 2 * ((G::NPAIR + NT - 1) / NT);
  constexpr int MAXS = SINGLE ? (NOWN + NT - 1) / NT : 1;
  constexpr int MAXP = SINGLE ? 1 : (G::NPAIR + NT - 1) / NT;
  float minv_s[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; k++) {
    minv_s[k] = 0.f;
    if constexpr (SINGLE && !AC) {
      const int o = threadIdx.x + k * NT, oy = o / G::OWM, ox = o - (o / G::OWM) * G::OWM;
      if (o < NOWN && oy < b.OH && ox < b.OW) minv_s[k] = prm.minv[(size_t)(b.Y0 + oy) * prm.pitch + b.X0 + ox];
    }
  }
  float2 minv_pre[MAXP];
#pragma unroll
  for (int k = 0; k < MAXP; k++) {
    if constexpr (SINGLE || AC) { minv_pre[k] = make_float2(0.f, 0.f); continue; }
    const int o = threadIdx.x + k * NT;
    const int oy = o / G::PW, px = o - (o / G::PW) * G::PW;
    const int XA = b.OXa + 2 * px, Y = b.Y0 + oy;
    minv_pre[k] = (o < G::NPAIR && oy < b.OH && XA < b.X0 + b.OW && XA + 1 >= b.X0)
                      ? *reinterpret_cast<const float2 *>(prm.minv + (size_t)Y * prm.pitch + XA)
                      : make_float2(0.f, 0.f);
  }
  const bool ok = mbar_wait_bounded(bar, parity);
  if (__syncthreads_or(!ok)) return false;
  const float2 *rU = reinterpret_cast<const float2 *>(st);
  const float2 *rCU = reinterpret_cast<const float2 *>(st + L::REG);
  const float2 *oW = reinterpret_cast<const float2 *>(ob);
  const float2 *oCW = reinterpret_cast<const float2 *>(ob + L::OWN);

  // ---- 1. derivatives along row j (registers) and column j (to X1) -----
  float2 gxi[N1];
  const int base = (ecy * P) * BXW + ecx * P + xoff;   // region-box index of element node (0,0)
  if (active) {
    {
      // the row's nodes; at even degrees a row starts on a 16-byte boundary (xoff = 0, P and
      // BXW even) and is read as node pairs: 8-byte reads of rows P apart would use only half
      // of the shared-memory banks
      float2 ur[N1], cr[N1];
      row_nodes<P>(rU + base + j * BXW, ur);
      if (KAHAN) row_nodes<P>(rCU + base + j * BXW, cr);
      const float2 u0 = ur[0];
      const float2 c0 = KAHAN ? cr[0] : make_float2(0.f, 0.f);
      float2 d[N1];
#pragma unroll
      for (int k = 1; k < N1; k++) {
        const float2 uk = ur[k];
        d[k].x = uk.x - u0.x; d[k].y = uk.y - u0.y;
        if (KAHAN) {
          const float2 ck = cr[k];
          d[k].x -= (ck.x - c0.x); d[k].y -= (ck.y - c0.y);
        }
      }
#pragma unroll
      for (int q = 0; q < N1; q++) {
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int k = 1; k < N1; k++) { sx = fmaf(D[q * N1 + k], d[k].x, sx); sy = fmaf(D[q * N1 + k], d[k].y, sy); }
        gxi[q] = make_float2(sx, sy);
      }
    }
    {
      const float2 u0 = rU[base + j];
      const float2 c0 = KAHAN ? rCU[base + j] : make_float2(0.f, 0.f);
      float2 d[N1];
#pragma unroll
      for (int k = 1; k < N1; k++) {
        const float2 uk = rU[base + k * BXW + j];
        d[k].x = uk.x - u0.x; d[k].y = uk.y - u0.y;
        if (KAHAN) {
          const float2 ck = rCU[base + k * BXW + j];
          d[k].x -= (ck.x - c0.x); d[k].y -= (ck.y - c0.y);
        }
      }
#pragma unroll
      for (int q = 0; q < N1; q++) {
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int k = 1; k < N1; k++) { sx = fmaf(D[q * N1 + k], d[k].x, sx); sy = fmaf(D[q * N1 + k], d[k].y, sy); }
        X1[el * XS + j + q * RS] = make_float2(sx, sy);   // d/deta at (j, q)
      }
    }
  }
  if constexpr (WE) __syncwarp(); else __syncthreads();

  // ---- 2. stress at the row's points; xi divergence; eta fluxes to X2 ---
  if (active) {
    // the element's (lam detJ, mu detJ, d xi/dx, d eta/dy)
    const float4 cc = AC ? reinterpret_cast<const float4 *>(st + L::REG * (KAHAN ? 2 : 1))[ecy * NEX + ecx] : ccg;
    const float lam = cc.x, mu = cc.y, ix = cc.z, iy = cc.w;
    const float c11 = fmaf(2.f, mu, lam);
    const float nfj = -wj;
    float2 Fxi[N1];
#pragma unroll
    for (int q = 0; q < N1; q++) {
      const float2 ge = X1[el * XS + q + j * RS];   // d/deta at (q, j)
      const float e0 = ix * gxi[q].x, e1 = iy * ge.y, e2 = fmaf(ix, gxi[q].y, iy * ge.x);
      const float nf = nfj * W[q];                   // -detJ w_q w_j
      const float fx_ = ix * nf, fy_ = iy * nf;
      const float sxx = fmaf(c11, e0, lam * e1), syy = fmaf(lam, e0, c11 * e1), sxy = mu * e2;
      Fxi[q] = make_float2(fx_ * sxx, fx_ * sxy);
      X2[el * XS + q + j * RS] = make_float2(fy_ * sxy, fy_ * syy);
    }
    // xi part of the divergence for the row's nodes, to X1 (this thread alone read row j of X1)
#pragma unroll
    for (int a = 0; a < N1; a++) {
      float rx = 0.f, ry = 0.f;
#pragma unroll
      for (int q = 0; q < N1; q++) { rx = fmaf(D[q * N1 + a], Fxi[q].x, rx); ry = fmaf(D[q * N1 + a], Fxi[q].y, ry); }
      X1[el * XS + a + j * RS] = make_float2(rx, ry);
    }
  }
  if constexpr (WE) __syncwarp(); else __syncthreads();

  // ---- 3. eta part of the divergence along column j (its 5 fluxes), added to X1 -----
  if (active) {
    float2 fc[N1];
#pragma unroll
    for (int q = 0; q < N1; q++) fc[q] = X2[el * XS + j + q * RS];
#pragma unroll
    for (int bq = 0; bq < N1; bq++) {
      const float2 r = X1[el * XS + j + bq * RS];
      float cx = r.x, cy = r.y;
#pragma unroll
      for (int q = 0; q < N1; q++) { cx = fmaf(D[q * N1 + bq], fc[q].x, cx); cy = fmaf(D[q * N1 + bq], fc[q].y, cy); }
      X1[el * XS + j + bq * RS] = make_float2(cx, cy);
    }
  }
  if (OWAIT) {
    // the owned w (cw) copies of this tile, issued at its start, have normally landed by now
    const bool ok_o = mbar_wait_bounded(bar_o, par_o);
    if (__syncthreads_or(!ok_o)) return false;
  } else {
    __syncthreads();   // (the owned boxes came with the region, on its barrier)
  }
  // AC: 1/M of the owned nodes (from the column X0 rounded down to a multiple of 4) and
  // the tile's bounds, after the owned boxes
  const float *mbox = reinterpret_cast<const float *>(ob + L::OWN * (KAHAN ? 2 : 1));
  if constexpr (AC) bnd = *reinterpret_cast<const int4 *>(ob + L::OWN * (KAHAN ? 2 : 1) + L::MINVB);
  const int s0 = bnd.x, s1 = bnd.y, r0 = bnd.z, r1 = bnd.w;
  const int MXa = b.X0 & ~3;

  // the node phase's parameters in registers: when prm lives in shared memory (the
  // batched kernel), every store through an output pointer would otherwise force
  // the following parameter reads to be repeated
  float2 *const u_out = prm.u_out, *const w_out = prm.w_out, *const cu_out = prm.cu_out, *const cw_out = prm.cw_out;
  float2 *const a_out = stp.a_out;
  const int pitch = prm.pitch, NXP = prm.mx * P, NYP = prm.my * P;
  const float dt = prm.dt, half_dt = prm.half_dt;
  // ---- owned nodes: ordered element sum, sources, update
  if constexpr (SINGLE) {
#pragma unroll
    for (int k = 0; k < MAXS; k++) {
      const int o = threadIdx.x + k * NT, oy = o / G::OWM, ox = o - (o / G::OWM) * G::OWM;
      if (o >= NOWN || oy >= b.OH || ox >= b.OW) continue;
      const int X = b.X0 + ox, Y = b.Y0 + oy;
      float fx = 0.f, fy = 0.f;
      {
        const int lx = X - b.EX0 * P, ly = Y - b.EY0 * P;
        const int ex = lx / P, ey = ly / P, ix = lx - ex * P, iy = ly - ey * P;
        const bool in_x = X < NXP, in_y = Y < NYP;
        const bool lft = (ix == 0) && (X > 0), bot = (iy == 0) && (Y > 0);
        const int own = (ey * NEX + ex) * XS + ix + iy * RS;
        if (bot && lft) { const float2 fe = X1[own - NEX * XS - XS + P + P * RS]; fx += fe.x; fy += fe.y; }
        if (bot && in_x) { const float2 fe = X1[own - NEX * XS + P * RS]; fx += fe.x; fy += fe.y; }
        if (lft && in_y) { const float2 fe = X1[own - XS + P]; fx += fe.x; fy += fe.y; }
        if (in_x && in_y) { const float2 fe = X1[own]; fx += fe.x; fy += fe.y; }
      }
      for (int q = s0; q < s1; q++) {
        const int sidx = prm.tile_src_idx[q], se = prm.src_elem[sidx], sx = se % prm.mx, sy = se / prm.mx;
        const int a = X - sx * P, bb = Y - sy * P;
        if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
          const float val = (float)stp.stf[sidx];
          const float *sv = prm.src_vals + (size_t)sidx * 2 * NPE + 2 * (a + bb * N1);
          fx = fmaf(val, sv[0], fx); fy = fmaf(val, sv[1], fy);
        }
      }
      const float mv = AC ? mbox[oy * G::MBW + (X - MXa)] : minv_s[k];
      const float2 acc = make_float2(fx * mv, fy * mv);
      const int ri = (Y - b.RYa) * BXW + (X - b.RXa);
      const int oi = oy * OBW + (X - b.OXa);
      float2 u = rU[ri], w = oW[oi];
      float2 cu = KAHAN ? rCU[ri] : make_float2(0.f, 0.f), cw = KAHAN ? oCW[oi] : make_float2(0.f, 0.f);
      for (int q = r0; q < r1; q++) {
        const int r = prm.tile_rec_idx[q], re = prm.rec_elem[r], rx = re % prm.mx, ry = re / prm.mx;
        const int a = X - rx * P, bb = Y - ry * P;
        if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
          float *rb = stp.rbuf_out + ((size_t)r * NPE + a + bb * N1) * 6;
          rb[0] = u.x; rb[1] = u.y; rb[2] = fmaf(half_dt, acc.x, w.x); rb[3] = fmaf(half_dt, acc.y, w.y);
          rb[4] = acc.x; rb[5] = acc.y;
        }
      }
      if (KAHAN) {
        kahan_add(w.x, cw.x, dt * acc.x); kahan_add(w.y, cw.y, dt * acc.y);
        kahan_add(u.x, cu.x, dt * w.x); kahan_add(u.y, cu.y, dt * w.y);
      } else {
        w.x = fmaf(dt, acc.x, w.x); w.y = fmaf(dt, acc.y, w.y);
        u.x = fmaf(dt, w.x, u.x); u.y = fmaf(dt, w.y, u.y);
      }
      const size_t n = (size_t)Y * pitch + X;
      u_out[n] = u;
      w_out[n] = w;
      if (KAHAN) { cu_out[n] = cu; cw_out[n] = cw; }
      if (a_out) a_out[n] = acc;
    }
  }
#pragma unroll
  for (int k = 0; k < MAXP; k++) {
    if constexpr (SINGLE) break;
    const int o = threadIdx.x + k * NT;
    if (o >= G::NPAIR) break;
    const int oy = o / G::PW, px = o - (o / G::PW) * G::PW;
    const int XA = b.OXa + 2 * px, Y = b.Y0 + oy;
    const bool v0 = (oy < b.OH) && (XA >= b.X0) && (XA < b.X0 + b.OW);
    const bool v1 = (oy < b.OH) && (XA + 1 >= b.X0) && (XA + 1 < b.X0 + b.OW);
    if (!v0 && !v1) continue;
    float f[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (!(h ? v1 : v0)) continue;
      const int X = XA + h;
      // the 1, 2 or 4 elements around the node, in ascending element order (diagonal,
      // below, left, own), addressed relative to the node's own element in the region
      const int lx = X - b.EX0 * P, ly = Y - b.EY0 * P;
      const int ex = lx / P, ey = ly / P, ix = lx - ex * P, iy = ly - ey * P;
      const bool in_x = X < NXP, in_y = Y < NYP;
      const bool lft = (ix == 0) && (X > 0), bot = (iy == 0) && (Y > 0);
      const int own = (ey * NEX + ex) * XS + ix + iy * RS;
      if (bot && lft) { const float2 fe = X1[own - NEX * XS - XS + P + P * RS]; f[h][0] += fe.x; f[h][1] += fe.y; }
      if (bot && in_x) { const float2 fe = X1[own - NEX * XS + P * RS]; f[h][0] += fe.x; f[h][1] += fe.y; }
      if (lft && in_y) { const float2 fe = X1[own - XS + P]; f[h][0] += fe.x; f[h][1] += fe.y; }
      if (in_x && in_y) { const float2 fe = X1[own]; f[h][0] += fe.x; f[h][1] += fe.y; }
      for (int q = s0; q < s1; q++) {
        const int sidx = prm.tile_src_idx[q], se = prm.src_elem[sidx], sx = se % prm.mx, sy = se / prm.mx;
        const int a = X - sx * P, bb = Y - sy * P;
        if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
          const float val = (float)stp.stf[sidx];
          const float *sv = prm.src_vals + (size_t)sidx * 2 * NPE + 2 * (a + bb * N1);
          f[h][0] = fmaf(val, sv[0], f[h][0]); f[h][1] = fmaf(val, sv[1], f[h][1]);
        }
      }
    }
    const float2 mv = AC ? *reinterpret_cast<const float2 *>(mbox + oy * G::MBW + (XA - MXa)) : minv_pre[k];
    const float4 acc = make_float4(f[0][0] * mv.x, f[0][1] * mv.x, f[1][0] * mv.y, f[1][1] * mv.y);
    const int ri = (Y - b.RYa) * BXW + (XA - b.RXa);     // even: 16-byte aligned pairs
    const int oi = oy * OBW + (XA - b.OXa);
    float4 u = *reinterpret_cast<const float4 *>(rU + ri);
    float4 w = *reinterpret_cast<const float4 *>(oW + oi);
    float4 cu = KAHAN ? *reinterpret_cast<const float4 *>(rCU + ri) : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 cw = KAHAN ? *reinterpret_cast<const float4 *>(oCW + oi) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (r1 > r0) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!(h ? v1 : v0)) continue;
        const int X = XA + h;
        const float ux = h ? u.z : u.x, uy = h ? u.w : u.y, wx = h ? w.z : w.x, wy = h ? w.w : w.y;
        const float ax = h ? acc.z : acc.x, ay = h ? acc.w : acc.y;
        for (int q = r0; q < r1; q++) {
          const int r = prm.tile_rec_idx[q], re = prm.rec_elem[r], rx = re % prm.mx, ry = re / prm.mx;
          const int a = X - rx * P, bb = Y - ry * P;
          if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
            float *rb = stp.rbuf_out + ((size_t)r * NPE + a + bb * N1) * 6;
            rb[0] = ux; rb[1] = uy; rb[2] = fmaf(half_dt, ax, wx); rb[3] = fmaf(half_dt, ay, wy);
            rb[4] = ax; rb[5] = ay;
          }
        }
      }
    }
    if (KAHAN) {
      kahan_add(w.x, cw.x, dt * acc.x); kahan_add(w.y, cw.y, dt * acc.y);
      kahan_add(w.z, cw.z, dt * acc.z); kahan_add(w.w, cw.w, dt * acc.w);
      kahan_add(u.x, cu.x, dt * w.x); kahan_add(u.y, cu.y, dt * w.y);
      kahan_add(u.z, cu.z, dt * w.z); kahan_add(u.w, cu.w, dt * w.w);
    } else {
      w.x = fmaf(dt, acc.x, w.x); w.y = fmaf(dt, acc.y, w.y);
      w.z = fmaf(dt, acc.z, w.z); w.w = fmaf(dt, acc.w, w.w);
      u.x = fmaf(dt, w.x, u.x); u.y = fmaf(dt, w.y, u.y);
      u.z = fmaf(dt, w.z, u.z); u.w = fmaf(dt, w.w, u.w);
    }
    const size_t n = (size_t)Y * pitch + XA;
    if (v0 && v1) {
      *reinterpret_cast<float4 *>(u_out + n) = u;
      *reinterpret_cast<float4 *>(w_out + n) = w;
      if (KAHAN) { *reinterpret_cast<float4 *>(cu_out + n) = cu; *reinterpret_cast<float4 *>(cw_out + n) = cw; }
      if (a_out) *reinterpret_cast<float4 *>(a_out + n) = acc;
    } else {
      const int h = v0 ? 0 : 1;
      u_out[n + h] = h ? make_float2(u.z, u.w) : make_float2(u.x, u.y);
      w_out[n + h] = h ? make_float2(w.z, w.w) : make_float2(w.x, w.y);
      if (KAHAN) {
        cu_out[n + h] = h ? make_float2(cu.z, cu.w) : make_float2(cu.x, cu.y);
        cw_out[n + h] = h ? make_float2(cw.z, cw.w) : make_float2(cw.x, cw.y);
      }
      if (a_out) a_out[n + h] = h ? make_float2(acc.z, acc.w) : make_float2(acc.x, acc.y);
    }
  }
  __syncthreads();   // stage s, the owned buffer and the exchange buffers are free again
  return true;
}

// ---------------------------------------------------------------- two-float arithmetic
// The two-float mode carries every quantity of a step as an unevaluated sum h + l of
// two floats (about 48 significant bits).  The building blocks are the error-free
// transformations TwoSum (Knuth), FastTwoSum (Dekker) and TwoProduct through a fused
// multiply-add; sums of products are accumulated as in the compensated dot product
// Dot2 of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26, 2005): the running sum in h,
// the errors of every product and addition collected in l, normalised once at the end.
// Every operation is an explicit round-to-nearest intrinsic, so the compiler neither
// fuses nor reorders them.
struct tf {
  float h, l;
};

__device__ __forceinline__ tf tf_two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return tf{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ tf tf_fast_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  return tf{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ tf tf_add(tf a, tf b)
{
  const tf s = tf_two_sum(a.h, b.h);
  return tf_fast_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
// the product as the pair (rounded product, remainder), not renormalised: the remainder
// is within about two units in the last place of the product, and every consumer (another
// product, a sum, a dot-product term) takes a pair in that state at the same accuracy
__device__ __forceinline__ tf tf_mul(tf a, tf b)
{
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return tf{p, e};
}
__device__ __forceinline__ tf tf_neg(tf a) { return tf{-a.h, -a.l}; }
// s += a * x, unnormalised (Dot2 step); finish with tf_norm
__device__ __forceinline__ void tf_dot(tf &s, float ah, float al, tf x)
{
  const float p = __fmul_rn(ah, x.h);
  float e = __fmaf_rn(ah, x.h, -p);
  e = __fmaf_rn(ah, x.l, e);
  e = __fmaf_rn(al, x.h, e);
  const tf t = tf_two_sum(s.h, p);
  s.h = t.h;
  s.l = __fadd_rn(s.l, __fadd_rn(t.l, e));
}
__device__ __forceinline__ tf tf_norm(tf s) { return tf_two_sum(s.h, s.l); }
// a double split into its nearest float and the float nearest the remainder
__device__ __forceinline__ tf tf_from_double(double v)
{
  const float h = __double2float_rn(v);
  return tf{h, __double2float_rn(__dsub_rn(v, (double)h))};
}

// One tile in the two-float mode: the same phases, items and shared-memory traffic
// pattern as tile_body, with every value a two-float pair (exchange buffers hold
// float4 = (x.h, y.h, x.l, y.l)) and the tables' low parts read beside their high
// parts.  The state keeps the Kahan mode's storage (value = hi - c), so fields,
// norms and checkpoints are shared with that mode.
template <int P, int TE, int NT, bool OWAIT, bool WE = false>
__device__ __forceinline__ bool tile_body_df(const Params &prm, const StepPtrs stp, int tx, int ty, const unsigned char *st,
                                             uint32_t bar, uint32_t parity, const unsigned char *ob, uint32_t bar_o,
                                             uint32_t par_o, float4 *X1, float4 *X2, bool valid, int el, int j, int ecx,
                                             int ecy)
{
  typedef Geo<P, TE> G;
  typedef Layout<P, TE, true, 1, true> L;
  constexpr int N1 = G::N1, NPE = G::NPE, NEX = G::NEX, BXW = G::BXW, OBW = G::OBW, XS = G::XS;
  const float *Dh = c_D[P - 1], *Dl = c_Dl[P - 1];
  const TileBox b = tile_box<P, TE>(prm, tx, ty);
  const int t = ty * prm.ntx + tx;
  const int xoff = b.EX0 * P - b.RXa;
  const bool active = valid && (ecx < b.NEXa) && (ecy < b.NEYa);
  const int ex = b.EX0 + ecx, ey = b.EY0 + ecy;
  const size_t ncell = (size_t)prm.mx * prm.my;
  tf lam{0.f, 0.f}, mu{0.f, 0.f}, ix{0.f, 0.f}, iy{0.f, 0.f}, detJ{0.f, 0.f};
  if (active) {
    const size_t cell = (size_t)ey * prm.mx + ex;
    lam = tf{prm.lam[cell], prm.lam[ncell + cell]};
    mu = tf{prm.mu[cell], prm.mu[ncell + cell]};
    ix = tf{prm.iJ00[ex], prm.iJ00[prm.mx + ex]};
    iy = tf{prm.iJ11[ey], prm.iJ11[prm.my + ey]};
    detJ = tf_mul(tf{prm.J00[ex], prm.J00[prm.mx + ex]}, tf{prm.J11[ey], prm.J11[prm.my + ey]});
  }
  const int s0 = prm.tile_src_off[t], s1 = prm.tile_src_off[t + 1];
  const int r0 = prm.tile_rec_off[t], r1 = prm.tile_rec_off[t + 1];
  // node phase: single nodes strided by NT; 1/M (both parts) loaded before the wait
  constexpr int NOWN = G::OWM * G::OWM;
  constexpr int MAXS = (NOWN + NT - 1) / NT;
  const float *minv_lo = prm.minv + (size_t)prm.ny_g * prm.pitch;
  tf minv_s[MAXS];
#pragma unroll
  for (int k = 0; k < MAXS; k++) {
    minv_s[k] = tf{0.f, 0.f};
    const int o = threadIdx.x + k * NT, oy = o / G::OWM, ox = o - (o / G::OWM) * G::OWM;
    if (o < NOWN && oy < b.OH && ox < b.OW) {
      const size_t n = (size_t)(b.Y0 + oy) * prm.pitch + b.X0 + ox;
      minv_s[k] = tf{prm.minv[n], minv_lo[n]};
    }
  }
  const bool ok = mbar_wait_bounded(bar, parity);
  if (__syncthreads_or(!ok)) return false;
  const float2 *rU = reinterpret_cast<const float2 *>(st);
  const float2 *rCU = reinterpret_cast<const float2 *>(st + L::REG);
  const float2 *oW = reinterpret_cast<const float2 *>(ob);
  const float2 *oCW = reinterpret_cast<const float2 *>(ob + L::OWN);

  // ---- 1. derivatives along row j (registers) and column j (to X1), of the
  // displacement relative to the line's first node: (u_k - u_0) + (c_0 - c_k) with the
  // first difference split exactly by TwoSum
  tf gx[N1], gy[N1];
  const int base = (ecy * P) * BXW + ecx * P + xoff;
  if (active) {
#pragma unroll
    for (int dir = 0; dir < 2; dir++) {
      const int stride = dir ? BXW : 1, b0 = dir ? base + j : base + j * BXW;
      const float2 u0 = rU[b0], c0 = rCU[b0];
      tf dx[N1], dy[N1];
#pragma unroll
      for (int k = 1; k < N1; k++) {
        const float2 uk = rU[b0 + k * stride], ck = rCU[b0 + k * stride];
        dx[k] = tf_two_sum(uk.x, -u0.x);
        dx[k].l = __fsub_rn(dx[k].l, __fsub_rn(ck.x, c0.x));
        dy[k] = tf_two_sum(uk.y, -u0.y);
        dy[k].l = __fsub_rn(dy[k].l, __fsub_rn(ck.y, c0.y));
      }
#pragma unroll
      for (int q = 0; q < N1; q++) {
        tf sx{0.f, 0.f}, sy{0.f, 0.f};
#pragma unroll
        for (int k = 1; k < N1; k++) {
          tf_dot(sx, Dh[q * N1 + k], Dl[q * N1 + k], dx[k]);
          tf_dot(sy, Dh[q * N1 + k], Dl[q * N1 + k], dy[k]);
        }
        sx = tf_norm(sx);
        sy = tf_norm(sy);
        if (dir == 0) {
          gx[q] = sx;
          gy[q] = sy;
        } else {
          X1[el * XS + j + q * N1] = make_float4(sx.h, sy.h, sx.l, sy.l);   // d/deta at (j, q)
        }
      }
    }
  }
  if constexpr (WE) __syncwarp(); else __syncthreads();

  // ---- 2. stress at the row's points; xi divergence; eta fluxes to X2 ---
  if (active) {
    const tf c11 = tf_add(tf_add(mu, mu), lam);
    const tf nfj = tf_neg(tf_mul(detJ, tf{c_w[P - 1][j], c_wl[P - 1][j]}));
    tf Fx[N1], Fy[N1];
#pragma unroll
    for (int q = 0; q < N1; q++) {
      const float4 g4 = X1[el * XS + q + j * N1];   // d/deta at (q, j)
      const tf gex{g4.x, g4.z}, gey{g4.y, g4.w};
      const tf e0 = tf_mul(ix, gx[q]), e1 = tf_mul(iy, gey);
      const tf e2 = tf_add(tf_mul(ix, gy[q]), tf_mul(iy, gex));
      const tf nf = tf_mul(nfj, tf{c_w[P - 1][q], c_wl[P - 1][q]});   // -detJ w_q w_j
      const tf fx_ = tf_mul(ix, nf), fy_ = tf_mul(iy, nf);
      const tf sxx = tf_add(tf_mul(c11, e0), tf_mul(lam, e1));
      const tf syy = tf_add(tf_mul(lam, e0), tf_mul(c11, e1));
      const tf sxy = tf_mul(mu, e2);
      Fx[q] = tf_mul(fx_, sxx);
      Fy[q] = tf_mul(fx_, sxy);
      const tf hx = tf_mul(fy_, sxy), hy = tf_mul(fy_, syy);
      X2[el * XS + q + j * N1] = make_float4(hx.h, hy.h, hx.l, hy.l);
    }
    // xi part of the divergence for the row's nodes, to X1 (this thread alone read row j of X1)
#pragma unroll
    for (int a = 0; a < N1; a++) {
      tf rx{0.f, 0.f}, ry{0.f, 0.f};
#pragma unroll
      for (int q = 0; q < N1; q++) {
        tf_dot(rx, Dh[q * N1 + a], Dl[q * N1 + a], Fx[q]);
        tf_dot(ry, Dh[q * N1 + a], Dl[q * N1 + a], Fy[q]);
      }
      rx = tf_norm(rx);
      ry = tf_norm(ry);
      X1[el * XS + a + j * N1] = make_float4(rx.h, ry.h, rx.l, ry.l);
    }
  }
  if constexpr (WE) __syncwarp(); else __syncthreads();

  // ---- 3. eta part of the divergence along column j, added to X1 -----
  if (active) {
    tf fcx[N1], fcy[N1];
#pragma unroll
    for (int q = 0; q < N1; q++) {
      const float4 f4 = X2[el * XS + j + q * N1];
      fcx[q] = tf{f4.x, f4.z};
      fcy[q] = tf{f4.y, f4.w};
    }
#pragma unroll
    for (int bq = 0; bq < N1; bq++) {
      const float4 r = X1[el * XS + j + bq * N1];
      tf cx{r.x, r.z}, cy{r.y, r.w};
#pragma unroll
      for (int q = 0; q < N1; q++) {
        tf_dot(cx, Dh[q * N1 + bq], Dl[q * N1 + bq], fcx[q]);
        tf_dot(cy, Dh[q * N1 + bq], Dl[q * N1 + bq], fcy[q]);
      }
      cx = tf_norm(cx);
      cy = tf_norm(cy);
      X1[el * XS + j + bq * N1] = make_float4(cx.h, cy.h, cx.l, cy.l);
    }
  }
  if (OWAIT) {
    const bool ok_o = mbar_wait_bounded(bar_o, par_o);
    if (__syncthreads_or(!ok_o)) return false;
  } else {
    __syncthreads();
  }

  float2 *const u_out = prm.u_out, *const w_out = prm.w_out, *const cu_out = prm.cu_out, *const cw_out = prm.cw_out;
  float2 *const a_out = stp.a_out;
  const int pitch = prm.pitch, NXP = prm.mx * P, NYP = prm.my * P;
  const tf dt{prm.dt, prm.dt_lo}, hdt{prm.half_dt, prm.half_dt_lo};
  const float *src_lo = prm.src_vals + (size_t)prm.nsrc * 2 * NPE;
  // ---- owned nodes: ordered element sum, sources, update
#pragma unroll
  for (int k = 0; k < MAXS; k++) {
    const int o = threadIdx.x + k * NT, oy = o / G::OWM, ox = o - (o / G::OWM) * G::OWM;
    if (o >= NOWN || oy >= b.OH || ox >= b.OW) continue;
    const int X = b.X0 + ox, Y = b.Y0 + oy;
    tf fx{0.f, 0.f}, fy{0.f, 0.f};
    {
      const int lx = X - b.EX0 * P, ly = Y - b.EY0 * P;
      const int exl = lx / P, eyl = ly / P, ixl = lx - exl * P, iyl = ly - eyl * P;
      const bool in_x = X < NXP, in_y = Y < NYP;
      const bool lft = (ixl == 0) && (X > 0), bot = (iyl == 0) && (Y > 0);
      const int own = (eyl * NEX + exl) * XS + ixl + iyl * N1;
      auto add = [&](const float4 fe) {
        fx = tf_add(fx, tf{fe.x, fe.z});
        fy = tf_add(fy, tf{fe.y, fe.w});
      };
      if (bot && lft) add(X1[own - NEX * XS - XS + P + P * N1]);
      if (bot && in_x) add(X1[own - NEX * XS + P * N1]);
      if (lft && in_y) add(X1[own - XS + P]);
      if (in_x && in_y) add(X1[own]);
    }
    for (int q = s0; q < s1; q++) {
      const int sidx = prm.tile_src_idx[q], se = prm.src_elem[sidx], sx = se % prm.mx, sy = se / prm.mx;
      const int a = X - sx * P, bb = Y - sy * P;
      if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
        const tf val = tf_from_double(stp.stf[sidx]);
        const size_t vi = (size_t)sidx * 2 * NPE + 2 * (a + bb * N1);
        fx = tf_add(fx, tf_mul(val, tf{prm.src_vals[vi], src_lo[vi]}));
        fy = tf_add(fy, tf_mul(val, tf{prm.src_vals[vi + 1], src_lo[vi + 1]}));
      }
    }
    const tf ax = tf_mul(fx, minv_s[k]), ay = tf_mul(fy, minv_s[k]);
    const int ri = (Y - b.RYa) * BXW + (X - b.RXa);
    const int oi = oy * OBW + (X - b.OXa);
    const float2 u = rU[ri], cu = rCU[ri], w = oW[oi], cw = oCW[oi];
    const tf ux{u.x, -cu.x}, uy{u.y, -cu.y}, wx{w.x, -cw.x}, wy{w.y, -cw.y};
    for (int q = r0; q < r1; q++) {
      const int r = prm.tile_rec_idx[q], re = prm.rec_elem[r], rx = re % prm.mx, ry = re / prm.mx;
      const int a = X - rx * P, bb = Y - ry * P;
      if (a >= 0 && a <= P && bb >= 0 && bb <= P) {
        float *rb = stp.rbuf_out + ((size_t)r * NPE + a + bb * N1) * 12;
        const tf vx = tf_add(wx, tf_mul(hdt, ax)), vy = tf_add(wy, tf_mul(hdt, ay));
        const tf uxn = tf_norm(ux), uyn = tf_norm(uy);
        rb[0] = uxn.h; rb[1] = uyn.h; rb[2] = vx.h; rb[3] = vy.h; rb[4] = ax.h; rb[5] = ay.h;
        rb[6] = uxn.l; rb[7] = uyn.l; rb[8] = vx.l; rb[9] = vy.l; rb[10] = ax.l; rb[11] = ay.l;
      }
    }
    const tf wxn = tf_add(wx, tf_mul(dt, ax)), wyn = tf_add(wy, tf_mul(dt, ay));
    const tf uxn = tf_add(ux, tf_mul(dt, wxn)), uyn = tf_add(uy, tf_mul(dt, wyn));
    const size_t n = (size_t)Y * pitch + X;
    u_out[n] = make_float2(uxn.h, uyn.h);
    w_out[n] = make_float2(wxn.h, wyn.h);
    cu_out[n] = make_float2(-uxn.l, -uyn.l);
    cw_out[n] = make_float2(-wxn.l, -wyn.l);
    if (a_out) {
      a_out[n] = make_float2(ax.h, ay.h);
      a_out[(size_t)prm.ny_g * pitch + n] = make_float2(ax.l, ay.l);   // low parts after the high parts
    }
  }
  __syncthreads();   // stage s, the owned buffer and the exchange buffers are free again
  return true;
}

// this thread's (element, line) work item, the same for every tile
template <int P, int TE, bool WE>
__device__ __forceinline__ void item_of(int &el, int &j, bool &valid)
{
  typedef Geo<P, TE> G;
  constexpr int N1 = G::N1;
  if constexpr (WE) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = lane / N1;
    el = w * G::EPW + sub;
    j = lane - sub * N1;
    valid = (sub < G::EPW) && (el < G::NE);
  } else {
    el = threadIdx.x / N1;
    j = threadIdx.x - el * N1;
    valid = threadIdx.x < G::ITEMS;
  }
}

// DF: the two-float mode (KAHAN storage, tile_body_df); WE: the warp-aligned item mapping.
// Thread 0 issues, at the start of each tile, the next tile's region (and owned boxes,
// NOB = 2) or this tile's owned boxes (NOB = 1, on their own barrier), into the buffers
// the previous tile freed.  Except in the two-float mode the per-tile constants come with
// the copies (AC): the cell constants with the region, 1/M and the tile's source/receiver
// bounds with the owned boxes.
template <int P, int TE, int NT, bool KAHAN, int NOB = owned_buffers(P),
          int MINB = min_blocks(Layout<P, TE, KAHAN, NOB>::TOTAL), bool DF = false, bool WE = false>
__global__ void __launch_bounds__(NT, MINB)
persist_step(const __grid_constant__ CUtensorMap tm_u, const __grid_constant__ CUtensorMap tm_cu,
             const __grid_constant__ CUtensorMap tm_w, const __grid_constant__ CUtensorMap tm_cw,
             const __grid_constant__ CUtensorMap tm_c, const __grid_constant__ CUtensorMap tm_m, const Params prm)
{
  constexpr bool AC = !DF;   // tm_c: cell constants (float4 per cell), tm_m: 1/M
  typedef Geo<P, TE> G;
  typedef Layout<P, TE, KAHAN, NOB, DF, AC> L;
  constexpr int NEX = G::NEX;
  static_assert(WE ? NT >= 32 * G::NW : NT >= G::ITEMS, "one (element, line) item per thread");
  static_assert(NOB == 1 || NOB == 2, "one or two owned-box buffers");
  static_assert(!DF || (KAHAN && NOB == 1), "the two-float mode keeps the Kahan storage and one owned buffer");
  const float *W = c_w[P - 1];
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *stage0 = smem;
  unsigned char *stage1 = smem + L::STAGE;
  unsigned char *ob0 = smem + 2 * L::STAGE;                                             // owned w (cw)
  unsigned char *ob1 = ob0 + (NOB - 1) * L::OWNB;
  float2 *X1 = reinterpret_cast<float2 *>(smem + 2 * L::STAGE + NOB * L::OWNB);          // eta derivatives, then element forces
  float2 *X2 = reinterpret_cast<float2 *>(smem + 2 * L::STAGE + NOB * L::OWNB + L::XCH); // eta fluxes
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * L::STAGE + NOB * L::OWNB + 2 * L::XCH);
  const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]), bo0 = smem_u32(&bars[2]);

  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    mbar_init(bo0, 1);
    fence_barrier_init();
    prefetch_map(&tm_u); prefetch_map(&tm_w);
    if (KAHAN) { prefetch_map(&tm_cu); prefetch_map(&tm_cw); }
    if (AC) { prefetch_map(&tm_c); prefetch_map(&tm_m); }
  }
  __syncthreads();
  if (blockIdx.x == 0 && prm.record) sample_rows<P, DF>(prm, prm.rbuf_in, prm.trace_row);

  int el, j;
  bool valid;
  item_of<P, TE, WE>(el, j, valid);
  const int ecy = el / NEX, ecx = el - (el / NEX) * NEX;
  const float wj = valid ? W[j] : 0.f;

  // tile coordinates advance by the grid size without a division per tile
  int t = blockIdx.x;
  int tx = t % prm.ntx, ty = t / prm.ntx;
  const int dtx = gridDim.x % prm.ntx, dty = gridDim.x / prm.ntx;
  auto bnd = [&](int x, int y) { return prm.tile_bounds + (y * prm.ntx + x); };
  if (t < prm.ntiles && threadIdx.x == 0) {
    if (NOB == 2) issue_both<P, TE, KAHAN, AC>(tx, ty, stage0, ob0, bar0, &tm_u, &tm_cu, &tm_w, &tm_cw, &tm_c, &tm_m, bnd(tx, ty));
    else issue_region<P, TE, KAHAN, AC>(tx, ty, stage0, bar0, &tm_u, &tm_cu, &tm_c);
  }
  for (int it = 0; t < prm.ntiles; it++, t += gridDim.x) {
    const int s = it & 1;
    const uint32_t bar = s ? bar1 : bar0;
    const uint32_t parity = (it >> 1) & 1;
    int txn = tx + dtx, tyn = ty + dty;
    if (txn >= prm.ntx) { txn -= prm.ntx; tyn++; }
    // this tile's owned w (cw) with one owned buffer, the next tile's with two, and the
    // next tile's region into the other stage (each buffer was freed by the barrier
    // that ended the previous tile)
    const int tn = t + gridDim.x;
    unsigned char *ob = (NOB == 2 && s) ? ob1 : ob0;
    const uint32_t par_o = (uint32_t)(it & 1);   // the owned barrier (one owned buffer)
    if (threadIdx.x == 0) {
      fence_proxy_async();
      if (NOB == 1) issue_owned<P, TE, KAHAN, AC>(tx, ty, ob0, bo0, &tm_w, &tm_cw, &tm_m, bnd(tx, ty));
      if (tn < prm.ntiles) {
        if (NOB == 2)
          issue_both<P, TE, KAHAN, AC>(txn, tyn, s ? stage0 : stage1, s ? ob0 : ob1, s ? bar0 : bar1, &tm_u, &tm_cu, &tm_w,
                                       &tm_cw, &tm_c, &tm_m, bnd(txn, tyn));
        else
          issue_region<P, TE, KAHAN, AC>(txn, tyn, s ? stage0 : stage1, s ? bar0 : bar1, &tm_u, &tm_cu, &tm_c);
      }
    }
    bool ok;
    if constexpr (DF)
      ok = tile_body_df<P, TE, NT, true, WE>(prm, StepPtrs{prm.stf, prm.rbuf_out, prm.a_out}, tx, ty, s ? stage1 : stage0,
                                             bar, parity, ob, bo0, par_o, reinterpret_cast<float4 *>(X1),
                                             reinterpret_cast<float4 *>(X2), valid, el, j, ecx, ecy);
    else
      ok = tile_body<P, TE, NT, KAHAN, NOB == 1, WE, AC>(prm, StepPtrs{prm.stf, prm.rbuf_out, prm.a_out}, tx, ty,
                                                         s ? stage1 : stage0, bar, parity, ob, bo0, par_o, X1, X2, valid,
                                                         el, j, ecx, ecy, wj);
    if (!ok) {
      if (threadIdx.x == 0) {
        atomicExch(prm.err, 1);
        // let this CTA's copies in flight land before the shared memory is released
        mbar_wait_bounded(bar, parity);
        if (NOB == 1) mbar_wait_bounded(bo0, par_o);
        if (tn < prm.ntiles) mbar_wait_bounded(s ? bar0 : bar1, ((it + 1) >> 1) & 1);
      }
      return;
    }
    tx = txn;
    ty = tyn;
  }
}

// Many independent shots of one degree in one persistent launch.  The CTAs walk
// a flattened (shot, tile) list.  Each shot's parameters come from a table in
// global memory that depends only on which field buffer is the input; the
// per-step pointers are derived from the step's index within its block (kblk):
//   stf       = shot.stf + kblk * nsrc                     (block staging [shot][K][nsrc])
//   rbuf out  = kblk even ? shot.rbuf_out : shot.rbuf_in  (receiver ping-pong)
//   trace row = shot.trace_row + kblk * 7 * nrec           (block staging [shot][K][nrec][7])
// so the launches of a block are the same on every repetition (graph replay).
__device__ __forceinline__ const float *batch_rbuf(const Params &sh, int kblk)
{
  return (kblk & 1) ? sh.rbuf_in : sh.rbuf_out;
}

template <int P, int TE, int NT, bool KAHAN, int NOB = owned_buffers(P),
          int MINB = min_blocks(Layout<P, TE, KAHAN, NOB>::TOTAL), bool WE = false>
__global__ void __launch_bounds__(NT, MINB)
persist_batch(const __grid_constant__ BatchArgs ba)
{
  typedef Geo<P, TE> G;
  typedef Layout<P, TE, KAHAN, NOB> L;
  constexpr int NEX = G::NEX;
  static_assert(WE ? NT >= 32 * G::NW : NT >= G::ITEMS, "one (element, line) item per thread");
  static_assert(NOB == 1 || NOB == 2, "one or two owned-box buffers");
  const float *W = c_w[P - 1];
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char *stage0 = smem;
  unsigned char *stage1 = smem + L::STAGE;
  unsigned char *ob0 = smem + 2 * L::STAGE;
  unsigned char *ob1 = ob0 + (NOB - 1) * L::OWNB;
  float2 *X1 = reinterpret_cast<float2 *>(smem + 2 * L::STAGE + NOB * L::OWNB);
  float2 *X2 = reinterpret_cast<float2 *>(smem + 2 * L::STAGE + NOB * L::OWNB + L::XCH);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * L::STAGE + NOB * L::OWNB + 2 * L::XCH);
  const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]), bo0 = smem_u32(&bars[2]);

  if (threadIdx.x == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    mbar_init(bo0, 1);
    fence_barrier_init();
  }
  __syncthreads();
  // receivers of the previous step of this block, one CTA per shot
  if (ba.kblk > 0)
    for (int sh = blockIdx.x; sh < ba.nshots; sh += gridDim.x) {
      const Params &q = ba.shots[sh];
      if (q.nrec > 0) sample_rows<P>(q, batch_rbuf(q, ba.kblk - 1), q.trace_row + (size_t)(ba.kblk - 1) * 7 * q.nrec);
    }

  int el, j;
  bool valid;
  item_of<P, TE, WE>(el, j, valid);
  const int ecy = el / NEX, ecx = el - (el / NEX) * NEX;
  const float wj = valid ? W[j] : 0.f;

  // The shots' parameters are a kernel parameter (constant bank), so a tile reads
  // its shot's directly.  Every thread keeps the work items of this tile and the
  // next in registers (the list entry two tiles ahead is loaded one tile early);
  // thread 0 issues the next tile's copies at the top of this tile, as in the
  // single-shot kernel.
  const int stride = gridDim.x;
  int w = blockIdx.x;
  int2 cur = make_int2(0, 0), nxt = make_int2(0, 0);
  if (w < ba.nitems) cur = ba.items[w];
  if (w + stride < ba.nitems) nxt = ba.items[w + stride];
  if (w < ba.nitems && threadIdx.x == 0) {
    const CUtensorMap *m = ba.maps + 4 * cur.x;
    if (NOB == 2) issue_both<P, TE, KAHAN>(cur.y & 0xFFFF, cur.y >> 16, stage0, ob0, bar0, m, m + 1, m + 2, m + 3);
    else issue_region<P, TE, KAHAN>(cur.y & 0xFFFF, cur.y >> 16, stage0, bar0, m, m + 1);
  }
  for (int it = 0; w < ba.nitems; it++, w += stride) {
    const int s = it & 1;
    const uint32_t bar = s ? bar1 : bar0;
    const uint32_t parity = (it >> 1) & 1;
    const int wn = w + stride;
    unsigned char *ob = (NOB == 2 && s) ? ob1 : ob0;
    const uint32_t par_o = (uint32_t)(it & 1);   // the owned barrier (one owned buffer)
    const int2 nn = (wn + stride < ba.nitems) ? ba.items[wn + stride] : make_int2(0, 0);   // for the next tile
    if (threadIdx.x == 0) {
      fence_proxy_async();
      if (NOB == 1) {
        const CUtensorMap *mc = ba.maps + 4 * cur.x;
        issue_owned<P, TE, KAHAN>(cur.y & 0xFFFF, cur.y >> 16, ob0, bo0, mc + 2, mc + 3);
      }
      if (wn < ba.nitems) {
        const CUtensorMap *m = ba.maps + 4 * nxt.x;
        if (NOB == 2)
          issue_both<P, TE, KAHAN>(nxt.y & 0xFFFF, nxt.y >> 16, s ? stage0 : stage1, s ? ob0 : ob1, s ? bar0 : bar1, m,
                                   m + 1, m + 2, m + 3);
        else
          issue_region<P, TE, KAHAN>(nxt.y & 0xFFFF, nxt.y >> 16, s ? stage0 : stage1, s ? bar0 : bar1, m, m + 1);
      }
    }
    // this step's pointers of the tile's shot
    const Params &sp = ba.shots[cur.x];
    const StepPtrs stp{sp.stf + (size_t)ba.kblk * sp.nsrc, const_cast<float *>(batch_rbuf(sp, ba.kblk)),
                       ba.write_a ? sp.a_out : nullptr};
    if (!tile_body<P, TE, NT, KAHAN, NOB == 1, WE>(sp, stp, cur.y & 0xFFFF, cur.y >> 16, s ? stage1 : stage0, bar,
                                                   parity, ob, bo0, par_o, X1, X2, valid, el, j, ecx, ecy, wj)) {
      if (threadIdx.x == 0) {
        atomicExch(ba.err, 1);
        mbar_wait_bounded(bar, parity);
        if (NOB == 1) mbar_wait_bounded(bo0, par_o);
        if (wn < ba.nitems) mbar_wait_bounded(s ? bar0 : bar1, ((it + 1) >> 1) & 1);
      }
      return;
    }
    cur = nxt;
    nxt = nn;
  }
}

// receivers of the last step (kblk) of a block of batched steps, one CTA per shot
template <int P>
__global__ void persist_record_batch(const Params *shots, int nshots, int kblk)
{
  if ((int)blockIdx.x >= nshots) return;
  const Params &q = shots[blockIdx.x];
  if (q.nrec > 0) sample_rows<P>(q, batch_rbuf(q, kblk), q.trace_row + (size_t)kblk * 7 * q.nrec);
}

// receiver rows of the last step of a block
template <int P, bool DF = false>
__global__ void persist_record(const Params prm)
{
  sample_rows<P, DF>(prm, prm.rbuf_in, prm.trace_row);
}

}  // namespace se2p
