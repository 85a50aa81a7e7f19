// se2gpu_persist_launch.h -- host entry points of the persistent FP32 kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "se2gpu_persist_params.h"

namespace se2p {

// Tile configurations of the persistent kernels, X(degree, elements per tile edge,
// threads, owned-box buffers (0: owned_buffers(degree)), CTAs per SM the registers are
// sized for (0: as many as the shared memory allows, up to 3), item mapping (0: one
// thread per (element, line) in order, threads >= (edge + 1)^2 (degree + 1); 1:
// warp-aligned, 32 / (degree + 1) whole elements per warp, whose three element phases
// synchronise within the warp, threads = 32 x warps)).  Degree 4: 7x7 at 2 CTAs per SM
// (92-96 registers) is the fastest, with two owned buffers; sized for 3 CTAs it is capped
// at 64 registers and runs slower.  default_config gives each degree's fastest.  The
// two-float mode uses the same list with one owned buffer.  New configurations go at the
// end of their degree's list: the autotuner's cache and default_config refer to them by
// position.
#define SE2P_CONFIGS(X)                                                                      \
  X(1, 15, 512, 0, 0, 0) X(1, 11, 288, 0, 0, 0) X(1, 15, 512, 0, 0, 1)                       \
  X(2, 12, 512, 2, 2, 0) X(2, 10, 384, 0, 0, 0) X(2, 8, 256, 0, 0, 0) X(2, 10, 416, 0, 0, 1) \
  X(3, 7, 256, 0, 0, 0) X(3, 8, 352, 0, 0, 0) X(3, 7, 256, 0, 0, 1)                          \
  X(4, 7, 320, 1, 2, 0) X(4, 7, 320, 2, 0, 0) X(4, 6, 256, 2, 0, 0) X(4, 8, 416, 0, 0, 0)    \
  X(4, 7, 352, 1, 2, 1) X(4, 6, 288, 2, 0, 1)                                                \
  X(5, 6, 320, 0, 0, 0) X(5, 5, 224, 0, 0, 0) X(5, 6, 320, 0, 0, 1)                          \
  X(6, 5, 256, 0, 0, 0) X(6, 4, 192, 0, 0, 0) X(6, 5, 288, 0, 0, 1)                          \
  X(7, 4, 224, 0, 0, 0) X(7, 5, 288, 0, 0, 0) X(7, 4, 224, 0, 0, 1)                          \
  X(8, 4, 256, 0, 0, 0) X(8, 3, 160, 0, 0, 0) X(8, 4, 288, 0, 0, 1)

// arithmetic modes of the persistent step kernel
enum { MODE_PLAIN = 0, MODE_KAHAN = 1, MODE_DF = 2 };

struct TileShape {
  int tex, tey, nt, region_w, region_h, own_w, own_h;
  int owned_buffers;   // 2: the next tile's owned boxes arrive a tile ahead; 1: during the tile
  int cell_box;        // cell-constant box edge (elements, float4 each)
  int minv_w;          // 1/M box width (floats; the box is own_h high)
  size_t smem;
};

cudaError_t set_tables(int p, const double *D, const double *w1d);   // constant-memory D, w (current device)
int num_configs(int p);                                               // tile configurations for degree p
int default_config(int p);                                            // a new handle's (plain and Kahan modes)
// mode: MODE_PLAIN, MODE_KAHAN or MODE_DF (the batched kernel: plain or Kahan)
int config_shape(int p, int config, int mode, TileShape *s);
cudaError_t prepare(int p, int config, int mode);                     // dynamic shared-memory limit
int occupancy(int p, int config, int mode, bool batch = false);       // resident CTAs per SM
// maps: region u, region cu, owned w, owned cw of the input state, cell constants, 1/M
cudaError_t launch_step(int p, int config, int mode, const CUtensorMap *maps, const Params &prm, int grid,
                        cudaStream_t st);
cudaError_t launch_record(int p, const Params &prm, cudaStream_t st, bool df = false);

// the two-float kernels (their own translation unit, with its own constant tables)
cudaError_t df_set_tables(int p, const double *D, const double *w1d);
const void *df_kernel(int p, int config, size_t *smem);
cudaError_t df_launch_record(int p, const Params &prm, cudaStream_t st);
// batched step of many shots of degree p (tables in device memory), and the
// receiver rows of a block's last step
cudaError_t launch_batch(int p, int config, bool kahan, const BatchArgs &ba, int grid, cudaStream_t st);
cudaError_t launch_record_batch(int p, const Params *shots, int nshots, int kblk, cudaStream_t st);
int make_map(CUtensorMap *map, void *base, int nx, int ny, int pitch, int bw, int bh);      // float2 nodes
int make_map_f32(CUtensorMap *map, void *base, int nx, int ny, int pitch, int bw, int bh);  // float nodes
int make_map_cells(CUtensorMap *map, void *base, int mx, int my, int box);                 // float4 cells
// (al: the low parts of a in the two-float mode, else null)
cudaError_t launch_norms(const float2 *u, const float2 *w, const float2 *cu, const float2 *cw, const float2 *a,
                         const float2 *al, int nx, int ny, int pitch, double dt, double *part, int nblocks,
                         cudaStream_t st);
// the bounded wait on a barrier nothing arrives at (EXPIRY_TEST_POLLS polls): raises
// *err and writes the wait's duration in ns to *ns
constexpr long EXPIRY_TEST_POLLS = 256;
cudaError_t launch_wait_expiry_test(int *err, unsigned long long *ns, cudaStream_t st);

}  // namespace se2p
