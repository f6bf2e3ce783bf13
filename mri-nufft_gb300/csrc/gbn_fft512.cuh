// Pruned 2D transforms on 512 x 512 fine grids fused with the pad / crop
// passes (see gbn_fft512.cu).
#pragma once

#include <vector>

#include "gbn_passes.cuh"

namespace gbn {

// 2D plans whose fine grid is 512 on both axes
bool fft512_fits(const Geom& g);

// W512^(b k1), entry k1 * 16 + b (k1 < 32, b < 16), as 1024 floats (re, im)
std::vector<float> fft512_twiddles();

// raises the dynamic shared-memory limit of the kernels (once, outside any
// stream capture)
cudaError_t fft512_prepare();

// op: pad and the pruned transform of sign isign into pa.fine (pa.ntr
// grids); every fine cell is written.
cudaError_t launch_fft512_op(const PadArgs& pa, const float2* tw, int isign, cudaStream_t st);

// adjoint: the pruned transform of sign isign of `fine` (ca.ntr grids, read
// and overwritten) and the crop / coil combine of ca into ca.out.
cudaError_t launch_fft512_adj(const CropArgs& ca, float2* fine, const float2* tw, int isign,
                              cudaStream_t st);

// Toeplitz Gram of a pass: pad, forward transform, multiply by the real
// circulant spectrum K (512^2), inverse transform and crop, with the x
// transforms and the multiply in one pass over the y columns.
cudaError_t launch_fft512_gram(const PadArgs& pa, const CropArgs& ca, const float* K,
                               const float2* tw, cudaStream_t st);

}  // namespace gbn
