// se2gpu_f32.cu -- FP32 instantiations (plain and Kahan-compensated), degrees 1..8.
#include "se2gpu_launch.h"

namespace se2 {

template <int P, bool K>
static cudaError_t prep1()
{
  return cudaFuncSetAttribute(step_kernel<P, float, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_layout<P, float, K>().total);
}
template <int P>
static cudaError_t prep(bool kahan) { return kahan ? prep1<P, true>() : prep1<P, false>(); }

template <int P>
static cudaError_t launch(bool kahan, const StepParams<float> &prm, int nblocks, cudaStream_t st)
{
  if (kahan) step_kernel<P, float, true><<<nblocks, 256, smem_layout<P, float, true>().total, st>>>(prm);
  else step_kernel<P, float, false><<<nblocks, 256, smem_layout<P, float, false>().total, st>>>(prm);
  return cudaGetLastError();
}

template <int P>
static cudaError_t record(const StepParams<float> &prm, cudaStream_t st)
{
  record_kernel<P, float><<<1, 128, 0, st>>>(prm);
  return cudaGetLastError();
}

template <int P>
static size_t smem(bool kahan) { return kahan ? smem_layout<P, float, true>().total : smem_layout<P, float, false>().total; }

#define SE2_DISPATCH(fn, ...)                                               \
  switch (p) {                                                              \
    case 1: return fn<1>(__VA_ARGS__); case 2: return fn<2>(__VA_ARGS__);   \
    case 3: return fn<3>(__VA_ARGS__); case 4: return fn<4>(__VA_ARGS__);   \
    case 5: return fn<5>(__VA_ARGS__); case 6: return fn<6>(__VA_ARGS__);   \
    case 7: return fn<7>(__VA_ARGS__); case 8: return fn<8>(__VA_ARGS__);   \
    default: break;                                                         \
  }

cudaError_t prepare_f32(int p, bool kahan) { SE2_DISPATCH(prep, kahan) return cudaErrorInvalidValue; }
cudaError_t launch_step_f32(int p, bool kahan, const StepParams<float> &prm, int nblocks, cudaStream_t st)
{
  SE2_DISPATCH(launch, kahan, prm, nblocks, st)
  return cudaErrorInvalidValue;
}
cudaError_t launch_record_f32(int p, const StepParams<float> &prm, cudaStream_t st) { SE2_DISPATCH(record, prm, st) return cudaErrorInvalidValue; }
size_t smem_f32(int p, bool kahan) { SE2_DISPATCH(smem, kahan) return 0; }

}  // namespace se2
