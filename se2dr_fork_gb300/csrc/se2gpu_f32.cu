// se2gpu_f32.cu -- FP32 instantiations of the tiled step kernel, degrees 1..8.  They
// serve the FP32 internal-force entry point (se2gpu_assemble_linear_form[_device] on
// an FP32 handle, plain arithmetic); FP32 time stepping runs the persistent kernels of
// se2gpu_f32p.cu.
#include "se2gpu_launch.h"

namespace se2 {

template <int P>
static cudaError_t prep()
{
  return cudaFuncSetAttribute(step_kernel<P, float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_layout<P, float, false>().total);
}

template <int P>
static cudaError_t launch(const StepParams<float> &prm, int nblocks, cudaStream_t st)
{
  step_kernel<P, float, false><<<nblocks, 256, smem_layout<P, float, false>().total, st>>>(prm);
  return cudaGetLastError();
}

#define SE2_DISPATCH(fn, ...)                                               \
  switch (p) {                                                              \
    case 1: return fn<1>(__VA_ARGS__); case 2: return fn<2>(__VA_ARGS__);   \
    case 3: return fn<3>(__VA_ARGS__); case 4: return fn<4>(__VA_ARGS__);   \
    case 5: return fn<5>(__VA_ARGS__); case 6: return fn<6>(__VA_ARGS__);   \
    case 7: return fn<7>(__VA_ARGS__); case 8: return fn<8>(__VA_ARGS__);   \
    default: break;                                                         \
  }

cudaError_t prepare_f32(int p) { SE2_DISPATCH(prep) return cudaErrorInvalidValue; }
cudaError_t launch_step_f32(int p, const StepParams<float> &prm, int nblocks, cudaStream_t st)
{
  SE2_DISPATCH(launch, prm, nblocks, st)
  return cudaErrorInvalidValue;
}

}  // namespace se2
