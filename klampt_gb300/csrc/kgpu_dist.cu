// kgpu_dist.cu — signed distance, soft-min and adjoint kernels.
#include "kgpu_device.cuh"

namespace kgpu {

cudaError_t launch_distance(const KWorldDev&, const Scratch&, int, const float*, int, double, double*, int*,
                            double*, float*, int, int, cudaStream_t)
{
  return cudaErrorNotSupported;
}

cudaError_t launch_softmin(const KWorldDev&, const Scratch&, int, const float*, int, int, double, double*,
                           float*, int, int, cudaStream_t)
{
  return cudaErrorNotSupported;
}

}  // namespace kgpu
