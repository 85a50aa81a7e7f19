// se2gpu_launch.h -- launch entry points of the per-precision kernel units.
#pragma once
#include <cuda_runtime.h>
#include "se2gpu_kernels.cuh"

namespace se2 {

// elements per tile edge for degree p
int tile_edge(int p);

// FP64, reference operation order
cudaError_t prepare_f64(int p);  // raise the dynamic shared-memory limit (current device)
size_t smem_f64(int p);
cudaError_t launch_step_f64(int p, const StepParams<double> &prm, int nblocks, cudaStream_t st);
cudaError_t launch_record_f64(int p, const StepParams<double> &prm, cudaStream_t st);

// FP32 internal force (plain arithmetic; FP32 stepping uses the persistent kernels)
cudaError_t prepare_f32(int p);
cudaError_t launch_step_f32(int p, const StepParams<float> &prm, int nblocks, cudaStream_t st);

}  // namespace se2
