// se2gpu_f64.cu -- FP64 (reference operation order) instantiations, degrees 1..8.
#include "se2gpu_launch.h"

namespace se2 {

int tile_edge(int p)
{
  switch (p) {
    case 1: return Tile<1>::TE; case 2: return Tile<2>::TE; case 3: return Tile<3>::TE; case 4: return Tile<4>::TE;
    case 5: return Tile<5>::TE; case 6: return Tile<6>::TE; case 7: return Tile<7>::TE; case 8: return Tile<8>::TE;
    default: return 0;
  }
}

template <int P>
static cudaError_t prep()
{
  return cudaFuncSetAttribute(step_kernel<P, double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_layout<P, double, false>().total);
}

template <int P>
static cudaError_t launch(const StepParams<double> &prm, int nblocks, cudaStream_t st)
{
  step_kernel<P, double, false><<<nblocks, 256, smem_layout<P, double, false>().total, st>>>(prm);
  return cudaGetLastError();
}

template <int P>
static cudaError_t record(const StepParams<double> &prm, cudaStream_t st)
{
  record_kernel<P, double><<<1, 128, 0, st>>>(prm);
  return cudaGetLastError();
}

#define SE2_DISPATCH(fn, ...)                                               \
  switch (p) {                                                              \
    case 1: return fn<1>(__VA_ARGS__); case 2: return fn<2>(__VA_ARGS__);   \
    case 3: return fn<3>(__VA_ARGS__); case 4: return fn<4>(__VA_ARGS__);   \
    case 5: return fn<5>(__VA_ARGS__); case 6: return fn<6>(__VA_ARGS__);   \
    case 7: return fn<7>(__VA_ARGS__); case 8: return fn<8>(__VA_ARGS__);   \
    default: return cudaErrorInvalidValue;                                  \
  }

cudaError_t prepare_f64(int p) { SE2_DISPATCH(prep) }
cudaError_t launch_step_f64(int p, const StepParams<double> &prm, int nblocks, cudaStream_t st) { SE2_DISPATCH(launch, prm, nblocks, st) }
cudaError_t launch_record_f64(int p, const StepParams<double> &prm, cudaStream_t st) { SE2_DISPATCH(record, prm, st) }

size_t smem_f64(int p)
{
  switch (p) {
    case 1: return smem_layout<1, double, false>().total; case 2: return smem_layout<2, double, false>().total;
    case 3: return smem_layout<3, double, false>().total; case 4: return smem_layout<4, double, false>().total;
    case 5: return smem_layout<5, double, false>().total; case 6: return smem_layout<6, double, false>().total;
    case 7: return smem_layout<7, double, false>().total; case 8: return smem_layout<8, double, false>().total;
    default: return 0;
  }
}

}  // namespace se2
