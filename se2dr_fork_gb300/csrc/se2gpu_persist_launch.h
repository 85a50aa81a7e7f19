// se2gpu_persist_launch.h -- host entry points of the persistent FP32 kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "se2gpu_persist_params.h"

namespace se2p {

struct TileShape {
  int tex, tey, nt, region_w, region_h, own_w, own_h;
  int owned_buffers;   // 2: the next tile's owned boxes arrive a tile ahead; 1: during the tile
  size_t smem;
};

cudaError_t set_tables(int p, const double *D, const double *w1d);   // constant-memory D, w (current device)
int num_configs(int p);                                               // tile configurations for degree p
int config_shape(int p, int config, bool kahan, TileShape *s);
cudaError_t prepare(int p, int config, bool kahan);                   // dynamic shared-memory limit
int occupancy(int p, int config, bool kahan, bool batch = false);     // resident CTAs per SM
// maps: region u, region cu, owned w, owned cw of the input state
cudaError_t launch_step(int p, int config, bool kahan, const CUtensorMap *maps, const Params &prm, int grid,
                        cudaStream_t st);
cudaError_t launch_record(int p, const Params &prm, cudaStream_t st);
// batched step of many shots of degree p (tables in device memory), and the
// receiver rows of a block's last step
cudaError_t launch_batch(int p, int config, bool kahan, const BatchArgs &ba, int grid, cudaStream_t st);
cudaError_t launch_record_batch(int p, const Params *shots, int nshots, int kblk, cudaStream_t st);
int make_map(CUtensorMap *map, void *base, int nx, int ny, int pitch, int bw, int bh);
cudaError_t launch_norms(const float2 *u, const float2 *w, const float2 *cu, const float2 *cw, const float2 *a, int nx,
                         int ny, int pitch, double dt, double *part, int nblocks, cudaStream_t st);
// the bounded wait on a barrier nothing arrives at (EXPIRY_TEST_POLLS polls): raises
// *err and writes the wait's duration in ns to *ns
constexpr long EXPIRY_TEST_POLLS = 256;
cudaError_t launch_wait_expiry_test(int *err, unsigned long long *ns, cudaStream_t st);

}  // namespace se2p
