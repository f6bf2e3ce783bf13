// 3D instantiations of the spreading kernel.
#include "gbn_kernels.cuh"

namespace gbn {
cudaError_t launch_spread3d(const SpreadArgs& a, cudaStream_t st) { return dispatch_spread<3>(a, st); }
cudaError_t launch_spread_stream3d(const SpreadArgs& a, cudaStream_t st) {
  return dispatch_spread_stream3d(a, st);
}
}  // namespace gbn
