// 2D instantiations of the spreading kernel.
#include "gbn_kernels.cuh"

namespace gbn {
cudaError_t launch_spread2d(const SpreadArgs& a, cudaStream_t st) { return dispatch_spread<2>(a, st); }
cudaError_t launch_spread_stream2d(const SpreadArgs& a, cudaStream_t st) {
  return dispatch_spread_stream2d(a, st);
}
}  // namespace gbn
