// se2gpu_persist_params.h -- launch parameters of the persistent FP32 step kernel.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

namespace se2p {

struct Params {
  int mx, my, nx_g, ny_g, pitch;   // pitch: padded row length (nodes) of the device arrays
  int ntx, nty, ntiles;
  // outputs (padded layout, float2 per node)
  float2 *u_out, *w_out, *cu_out, *cw_out;
  float2 *a_out;                   // optional: a_k (last step of a block); two-float mode: its low
                                   // parts follow at a_out + ny_g*pitch
  // inputs not loaded by TMA
  // Two-float mode: every table below is followed in the same allocation by its low
  // parts (value = hi + lo): minv by ny_g*pitch floats, lam and mu by mx*my, J00 and
  // iJ00 by mx, J11 and iJ11 by my, src_vals by nsrc*2*npe.
  const float *minv;               // padded, 1/M
  const float *lam, *mu;           // per cell
  const float *J00, *J11, *iJ00, *iJ11;
  // the constants of a cell as the plain and Kahan modes use them: (lam detJ, mu detJ,
  // d xi/dx, d eta/dy), detJ = J00 J11, each product rounded to float
  const float4 *cellc;
  float dt, half_dt;
  float dt_lo, half_dt_lo;         // two-float mode: dt = dt + dt_lo, dt/2 = half_dt + half_dt_lo
  int nsrc;
  const int *src_elem;
  const float *src_vals;           // [nsrc][2*npe]
  const double *stf;               // this step's values per source
  // receivers
  int nrec;
  const int *rec_elem;
  float *rbuf_out;                 // [nrec][npe][6] (u, v, a) of this step's receiver elements
                                   // (two-float mode: [nrec][npe][12], the 6 high then the 6 low parts)
  const float *rbuf_in;            // previous step's, sampled into trace_row when record != 0
  int record;
  const int *rec_gll;
  const double *Dd, *iJ00d, *iJ11d;
  double *trace_row;
  int *err;                        // error flag (bounded waits)
  // per-tile lists (CSR over tiles) of the sources and receivers whose element
  // touches the tile's owned nodes, built on the host
  const int *tile_src_off, *tile_src_idx, *tile_rec_off, *tile_rec_idx;
  // per tile: (first source, end of sources, first receiver, end of receivers) in the lists
  const int4 *tile_bounds;
};

// shots per batched launch: their parameters travel in the kernel's parameter space
// (constant bank), 96 x 312 B of the 32 KB a kernel parameter may take
#define SE2P_BATCH_SHOTS 96

// arguments of one batched step (up to SE2P_BATCH_SHOTS shots of one degree).  A
// shot's rbuf_out / rbuf_in are its two receiver buffers (written at even / odd steps
// of a block); stf and trace_row point at the shot's block staging.
struct BatchArgs {
  const CUtensorMap *maps;     // [shot][4]: region u, region cu, owned w, owned cw of the input buffers
  const int2 *items;           // (shot, ty << 16 | tx) work list of tile coordinates
  int nshots, nitems;
  int kblk;                    // step index within the block
  int write_a;                 // store a_k (last step of a block)
  int *err;
  Params shots[SE2P_BATCH_SHOTS];   // per shot, for this step's input buffer
};
static_assert(sizeof(BatchArgs) <= 32764, "a kernel parameter holds at most 32764 bytes");

}  // namespace se2p
