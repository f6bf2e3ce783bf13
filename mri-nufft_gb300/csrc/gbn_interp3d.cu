// 3D instantiations of the interpolation and kernel-derivative kernels.
#include "gbn_kernels.cuh"

namespace gbn {
cudaError_t launch_interp3d(const InterpArgs& a, cudaStream_t st) { return dispatch_interp<3>(a, st); }
cudaError_t launch_grad3d(const GradArgs& a, cudaStream_t st) { return dispatch_grad<3>(a, st); }
}  // namespace gbn
