// Pruned 3D transforms on 256^3 fine grids fused with the pad / crop passes
// (see gbn_fft256.cu).
#pragma once

#include <vector>

#include "gbn_passes.cuh"

namespace gbn {

// 3D plans whose fine grid is 256 on every axis
bool fft256_fits(const Geom& g);

// W256^(b k1), entry k1 * 16 + b (k1, b < 16), as 512 floats (re, im)
std::vector<float> fft256_twiddles();

// raises the dynamic shared-memory limit of the crop kernel (once, outside
// any stream capture)
cudaError_t fft256_prepare();

// op: pad (pa: image, coil maps, 1/phihat, scale) and the pruned transform
// of sign isign into pa.fine (pa.ntr grids); every fine cell is written.
cudaError_t launch_fft256_op(const PadArgs& pa, const float2* tw, int isign, cudaStream_t st);

// adjoint: the pruned transform of sign isign of `fine` (ca.ntr grids, read
// and overwritten) and the crop / coil combine of ca into ca.out.
cudaError_t launch_fft256_adj(const CropArgs& ca, float2* fine, const float2* tw, int isign,
                              cudaStream_t st);

// Toeplitz Gram of a pass (pa.ntr = ca.ntr transforms): pad, forward
// transform, multiply by the real circulant spectrum K (256^3), inverse
// transform and crop, with the x transforms and the multiply in one pass
// over the (y, z) lines; the fine grids hold only intermediate line data.
cudaError_t launch_fft256_gram(const PadArgs& pa, const CropArgs& ca, const float* K,
                               const float2* tw, cudaStream_t st);

}  // namespace gbn
