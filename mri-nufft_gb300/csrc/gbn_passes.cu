// Fused passes around the FFT on the oversampled grid, and FP64 reductions.
//
// pad pass  (type 2, before the forward FFT): one write of every fine cell;
//   cells that hold an image mode n get x_n * s_n * prod_d 1/phihat_d(n_d),
//   every other cell gets 0.  The SENSE product, the deapodisation and the
//   zero padding are one pass, so no separate elementwise kernel runs.
// crop pass (type 1, after the inverse FFT): reads only the N^d cells that
//   hold image modes, divides by phihat, scales, and either writes each
//   transform (calibrationless) or conjugate-multiplies by the coil maps and
//   sums over coils into one image (SENSE coil combine), optionally adding to
//   what is already there (coil chunks).
#include "gbn_passes.cuh"

namespace gbn {


template <int DIM>
__global__ void pad_kernel(PadArgs a) {
  pad_body<DIM>(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int DIM>
__global__ void crop_kernel(CropArgs a) {
  crop_body<DIM>(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}


cudaError_t launch_pad(const PadArgs& a, cudaStream_t st) {
  int64_t blocks = (a.g.G + 255) / 256;
  if (a.g.dim == 2) pad_kernel<2><<<(unsigned)blocks, 256, 0, st>>>(a);
  else pad_kernel<3><<<(unsigned)blocks, 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_crop(const CropArgs& a, cudaStream_t st) {
  int64_t blocks = (a.g.Nimg + 255) / 256;
  if (a.g.dim == 2) crop_kernel<2><<<(unsigned)blocks, 256, 0, st>>>(a);
  else crop_kernel<3><<<(unsigned)blocks, 256, 0, st>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 reductions (CG dot products and residual norms)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// out[0] += sum |x|^2 ; out must be zeroed by the caller
__global__ void norm2_kernel(const float2* __restrict__ x, int64_t n, double* out) {
  __shared__ double sm[32];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float2 v = x[i];
    acc += (double)v.x * v.x + (double)v.y * v.y;
  }
  acc = warp_sum(acc);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sm[wid] = acc;
  __syncthreads();
  if (wid == 0) {
    acc = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0.0;
    acc = warp_sum(acc);
    if (lane == 0) atomicAdd(out, acc);
  }
}

// out[0..1] += sum a_i * b_i  (non-conjugating complex dot, as numpy.dot)
__global__ void dotu_kernel(const float2* __restrict__ a, const float2* __restrict__ b,
                            int64_t n, int conj_a, double* out) {
  __shared__ double sr[32], si[32];
  double ar = 0.0, ai = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float2 x = a[i], y = b[i];
    double xr = x.x, xi = conj_a ? -(double)x.y : (double)x.y;
    ar += xr * y.x - xi * y.y;
    ai += xr * y.y + xi * y.x;
  }
  ar = warp_sum(ar);
  ai = warp_sum(ai);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sr[wid] = ar; si[wid] = ai; }
  __syncthreads();
  if (wid == 0) {
    ar = lane < (int)(blockDim.x >> 5) ? sr[lane] : 0.0;
    ai = lane < (int)(blockDim.x >> 5) ? si[lane] : 0.0;
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if (lane == 0) {
      atomicAdd(out, ar);
      atomicAdd(out + 1, ai);
    }
  }
}

static int reduce_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 1216 ? (b < 1 ? 1 : b) : 1216);  // 8 CTAs per SM on 152 SMs
}

cudaError_t launch_norm2(const float2* x, int64_t n, double* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
  if (e != cudaSuccess) return e;
  norm2_kernel<<<reduce_blocks(n), 256, 0, st>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t launch_dotu(const float2* a, const float2* b, int64_t n, int conj_a, double* out,
                        cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  dotu_kernel<<<reduce_blocks(n), 256, 0, st>>>(a, b, n, conj_a, out);
  return cudaGetLastError();
}

}  // namespace gbn
