// 2D instantiations of the interpolation and kernel-derivative kernels.
#include "gbn_kernels.cuh"

namespace gbn {
cudaError_t launch_interp2d(const InterpArgs& a, cudaStream_t st) { return dispatch_interp<2>(a, st); }
cudaError_t launch_grad2d(const GradArgs& a, cudaStream_t st) { return dispatch_grad<2>(a, st); }
}  // namespace gbn
