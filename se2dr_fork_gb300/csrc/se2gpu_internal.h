// se2gpu_internal.h -- the solver handle's layout and the helpers that the
// single-shot API (se2gpu_api.cu) shares with the batched ensemble
// (se2gpu_ensemble.cu).  Not part of the public interface.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "se2gpu.h"
#include "se2gpu_persist_params.h"

struct se2gpu_solver {
  int pageable;      // the device reads and writes pageable host memory (cudaDevAttrPageableMemoryAccess)
  int mx, my, p, n1, npe, nx_g, ny_g, precision;
  long nnodes;
  int nsrc, nrec, trace_cap, rows_written;
  bool pending_record;
  double dt;
  int device, nsm;
  cudaStream_t stream, own_stream;
  size_t tsize;                  // compute precision (4 or 8 bytes)
  // FP64 state: two buffer sets of packed u, v, a
  void *f64[2][3];
  int cur;
  // FP32 leapfrog state (padded): u, w, cu, cw per buffer set, a of the last step
  int pitch;
  float2 *pu[2], *pw[2], *pcu[2], *pcw[2], *pa;
  float *pminv, *rbuf[2];
  unsigned long long *mass_bad;  // first node with a mass that is not positive (device check at create)
  cudaEvent_t side_done[2];      // se2gpu_create: set-up work on side streams not yet joined
  int rlast;
  CUtensorMap maps[2][6];        // per input buffer set: region u, cu, owned w, cw; cell constants, 1/M
  float4 *cellc;                 // plain and Kahan modes: (lam detJ, mu detJ, d xi/dx, d eta/dy) per cell
  int4 *tile_bounds;             // per tile: source and receiver list bounds
  int pgrid, pconfig, pntx, pnty;
  int *tile_src_off, *tile_src_idx, *tile_rec_off, *tile_rec_idx;
  std::vector<int> *src_elem_h, *rec_elem_h;
  int *err_dev;
  // tables in compute precision
  void *mass, *lam, *mu, *J00, *J11, *iJ00, *iJ11, *D, *wq, *src_vals;
  double *Dd, *iJ00d, *iJ11d, *stf_dev, *traces, *norm_part;
  int stf_cap;
  int *src_elem, *rec_node, *rec_elem, *rec_gll;
  void *scratch_u, *scratch_f;   // assemble_linear_form staging (packed)
  long launches;
  int ntx, nty, nblocks;         // FP64 tiles
  char err[512];
};

// FP32 persistent-kernel parameters of a handle (no per-step pointers set)
se2p::Params se2gpu_internal_f32_params(se2gpu_solver *h);
// set the thread's message returned by se2gpu_last_error(NULL)
void se2gpu_internal_set_error(const char *msg);
