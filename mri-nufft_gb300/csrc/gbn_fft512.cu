// Pruned 2D transforms on 512 x 512 fine grids (2D images of up to 512
// modes per axis whose oversampled grid is 512, e.g. 256^2 at sigma = 2),
// fused with the pad and crop passes.  The 3D counterpart is gbn_fft256.cu;
// the layouts below follow it.
//
// Axis 0 (x) has stride 512 cells, axis 1 (y) is contiguous.  The image
// modes of an N-point axis occupy the fine indices [0, N - N/2) and
// [512 - N/2, 512).
//
//   op      y lines of the x-mode rows, pad fused into the loads
//           (x * s * scale / phihat on the y modes), all 512 entries
//           written; x lines of every y (mode entries in, all out).
//   adjoint x lines of every y (all in, mode entries out); y lines of the
//           x-mode rows (all in), crop fused into the stores: divide by
//           phihat, scale, and for coil maps conj(s_c) v_c added into the
//           image with float2 atomics (the image is cleared first unless the
//           call accumulates).
//   Toeplitz Gram (512^2 circulant grid): the op's y pass, one pass over
//           the x lines doing the forward transform, the multiply by the
//           real spectrum and the inverse transform, then the adjoint's y
//           pass with the crop.
//
// A 512-point line transform is a four-step of a 32-point and a 16-point
// DFT in registers with one exchange through shared memory:
//   n = 16 a + b (a < 32, b < 16), k = k1 + 32 k2 (k1 < 32, k2 < 16),
//   Y_b[k1] = sum_a x[16 a + b] W32^(a k1),   Z_b[k1] = Y_b[k1] W512^(b k1),
//   X[k1 + 32 k2] = sum_b Z_b[k1] W16^(b k2).
// A thread owns one (line, b) in the first step (the 32-point DFT, two
// 16-point DFTs and a radix-2 combine) and the two (line, k1 = b, b + 16) of
// the second.  For a 256-point image axis the mode entries of a line are
// the rows a < 8 and a >= 24 and the outputs k2 < 4 and k2 >= 12, known at
// compile time (kHalf); other sizes test each entry at run time (kModes).
// After the forward transform's second step the thread (line, b) holds
// X[b + 16 h + 32 k2] (h < 2, k2 < 16), which are the inputs x[16 a' + b]
// (a' = h + 2 k2) of the next 512-point transform's first step: the Gram's
// inverse transform needs no exchange in between.
//
// Thread layouts (256 threads, 16 lines per CTA): y lines put lanes on b of
// two lines (128-byte row segments; exchange buffer [line][k1][b], row
// pitch 17); x lines put lanes on 16 consecutive y columns (exchange buffer
// [k1][b][y]).
#include "gbn_fft512.cuh"

#include <cmath>
#include <vector>

#include "gbn_dft.cuh"

namespace gbn {

namespace {

using namespace dft;

constexpr int kL = 16;     // lines per CTA
constexpr int kT = 256;    // threads per CTA
constexpr int kN = 512;    // fine axis

// W32^k = (cos(pi k / 16), -sin(pi k / 16)), k < 16
__device__ __forceinline__ float2 w32(int k) {
  constexpr float c[9] = {1.0f,
                          0.98078528040323044f,
                          0.92387953251128674f,
                          0.83146961230254524f,
                          0.70710678118654752f,
                          0.55557023301960218f,
                          0.38268343236508977f,
                          0.19509032201612825f,
                          0.0f};
  return k <= 8 ? make_float2(c[k], -c[8 - k]) : make_float2(-c[16 - k], -c[k - 8]);
}

// 32-point DFT, natural order in and out.  HALF_IN: x[8 .. 23] are zero and
// not read.
template <bool HALF_IN = false>
__device__ __forceinline__ void dft32(float2 (&x)[32]) {
  float2 e[16], o[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    e[j] = x[2 * j];
    o[j] = x[2 * j + 1];
  }
  dft16<HALF_IN>(e);
  dft16<HALF_IN>(o);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const float2 ev = e[pos16(k)];
    const float2 ov = f2mul(o[pos16(k)], w32(k));
    x[k] = f2add(ev, ov);
    x[k + 16] = f2sub(ev, ov);
  }
}

__device__ __forceinline__ bool is_mode(int m, int n) {
  const int h = n >> 1;
  return m < n - h || m >= kN - h;
}
__device__ __forceinline__ int mode_to_img(int m, int n) {
  const int h = n >> 1;
  return m < n - h ? m + h : m - kN + h;
}
__device__ __forceinline__ int img_to_fine(int i, int n) {
  const int k = i - (n >> 1);
  return k < 0 ? k + kN : k;
}

enum : int { kAll = 0, kHalf = 1, kModes = 2 };
// input entry n = 16 a + b
template <int SET>
__device__ __forceinline__ bool in_on(int a, int b, int n) {
  if (SET == kAll) return true;
  if (SET == kHalf) return a < 8 || a >= 24;
  return is_mode(16 * a + b, n);
}
template <int SET>
__device__ __forceinline__ int in_img(int a, int b, int n) {
  if (SET == kHalf) return a < 8 ? 16 * a + b + 128 : 16 * a + b - 384;
  return mode_to_img(16 * a + b, n);
}
// output entry k = k1 + 32 k2
template <int SET>
__device__ __forceinline__ bool out_on(int k1, int k2, int n) {
  if (SET == kAll) return true;
  if (SET == kHalf) return k2 < 4 || k2 >= 12;
  return is_mode(k1 + 32 * k2, n);
}

constexpr size_t kYSmem = (512 + kL * 32 * 17) * sizeof(float2);   // twiddles + exchange
constexpr size_t kXSmem = (512 + 32 * 16 * kL) * sizeof(float2);

// ---------------------------------------------------------------- y lines, pad fused
// blockIdx.x: 16 consecutive x image rows; blockIdx.y: transform.  SET: the y
// modes.  3 CTAs per SM (80 registers): 23.5 against 26.9 us at 2 CTAs and
// 126 registers for 64 transforms; the other kernels measured slower at 3.
template <int SET>
__global__ void __launch_bounds__(kT, 3)
f512_pad_y_kernel(PadArgs a, const float2* __restrict__ tw, int conj) {
  extern __shared__ float2 s_dyn[];
  float2* const s_tw = s_dyn;
  float2* const s_x = s_tw + 512;
  const Geom& g = a.g;
  const int n0 = g.n[0], n1 = g.n[1];
  s_tw[threadIdx.x] = tw[threadIdx.x];
  s_tw[threadIdx.x + kT] = tw[threadIdx.x + kT];
  const int b = threadIdx.x & 15, l = threadIdx.x >> 4;
  const int ix = blockIdx.x * kL + l;
  const bool valid = ix < n0;
  const int c = blockIdx.y;
  const int64_t irow = (int64_t)(valid ? ix : 0) * n1;
  const float2* img = a.smaps ? a.img : a.img + (int64_t)c * g.Nimg;
  const float2* sm = a.smaps ? a.smaps + (int64_t)c * g.Nimg : nullptr;
  float f0 = a.scale;
  if (a.dec[0]) f0 *= a.dec[0][valid ? ix : 0];
  float2 x[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) {
    float2 v = make_float2(0.f, 0.f);
    if (valid && in_on<SET>(q, b, n1)) {
      const int i1 = in_img<SET>(q, b, n1);
      v = img[irow + i1];
      if (a.conj_in) v = f2conj(v);
      if (sm) {
        float2 s = sm[irow + i1];
        if (a.conj_in) s = f2conj(s);
        v = f2mul(v, s);
      }
      v = f2scale(v, a.dec[1] ? f0 * a.dec[1][i1] : f0);
      if (conj) v = f2conj(v);
    }
    x[q] = v;
  }
  __syncthreads();  // twiddle table
  dft32<SET == kHalf>(x);
  float2* row = s_x + l * (32 * 17);
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) row[k1 * 17 + b] = f2mul(x[k1], s_tw[k1 * 16 + b]);
  __syncthreads();
  if (!valid) return;
  float2* out = a.fine + (int64_t)c * g.G + (int64_t)img_to_fine(ix, n0) * kN;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k1 = b + 16 * h;
    float2 w[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = row[k1 * 17 + q];
    dft16(w);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      const float2 v = w[pos16(k2)];
      out[k1 + 32 * k2] = conj ? f2conj(v) : v;
    }
  }
}

// ---------------------------------------------------------------- x lines
struct F512Lines {
  float2* data;   // ntr grids of G cells
  int64_t G;
  int n_axis;     // image size along x
  int conj;
  const float2* tw;
};

// blockIdx.x: 16 consecutive y columns; blockIdx.y: transform.  IN / OUT:
// the x entries read / written.
template <int IN, int OUT>
__global__ void __launch_bounds__(kT, 2) f512_x_kernel(F512Lines a) {
  extern __shared__ float2 s_dyn[];
  float2* const s_tw = s_dyn;
  float2* const s_x = s_tw + 512;
  s_tw[threadIdx.x] = a.tw[threadIdx.x];
  s_tw[threadIdx.x + kT] = a.tw[threadIdx.x + kT];
  const int l = threadIdx.x & 15, b = threadIdx.x >> 4;
  float2* base = a.data + (int64_t)blockIdx.y * a.G + blockIdx.x * kL + l;
  float2 x[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) {
    float2 v = make_float2(0.f, 0.f);
    if (in_on<IN>(q, b, a.n_axis)) {
      v = base[(16 * q + b) * kN];
      if (a.conj) v = f2conj(v);
    }
    x[q] = v;
  }
  __syncthreads();  // twiddle table
  dft32<IN == kHalf>(x);
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) s_x[(k1 * 16 + b) * kL + l] = f2mul(x[k1], s_tw[k1 * 16 + b]);
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k1 = b + 16 * h;
    float2 w[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = s_x[(k1 * 16 + q) * kL + l];
    dft16<false, OUT == kHalf>(w);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      if (out_on<OUT>(k1, k2, a.n_axis)) {
        const float2 v = w[pos16(k2)];
        base[(k1 + 32 * k2) * kN] = a.conj ? f2conj(v) : v;
      }
    }
  }
}

// ---------------------------------------------------------------- y lines, crop fused
// blockIdx.x: 16 consecutive x image rows; blockIdx.y: transform.  SET: the y modes.
template <int SET>
__global__ void __launch_bounds__(kT, 2)
f512_crop_y_kernel(CropArgs a, const float2* __restrict__ tw, int conj) {
  extern __shared__ float2 s_dyn[];
  float2* const s_tw = s_dyn;
  float2* const s_x = s_tw + 512;
  const Geom& g = a.g;
  const int n0 = g.n[0], n1 = g.n[1];
  s_tw[threadIdx.x] = tw[threadIdx.x];
  s_tw[threadIdx.x + kT] = tw[threadIdx.x + kT];
  const int b = threadIdx.x & 15, l = threadIdx.x >> 4;
  const int ix = blockIdx.x * kL + l;
  const bool valid = ix < n0;
  const int c = blockIdx.y;
  const float2* in = a.fine + (int64_t)c * g.G + (int64_t)img_to_fine(valid ? ix : 0, n0) * kN;
  float2 x[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) {
    const float2 v = valid ? in[16 * q + b] : make_float2(0.f, 0.f);
    x[q] = conj ? f2conj(v) : v;
  }
  __syncthreads();  // twiddle table
  dft32(x);
  float2* row = s_x + l * (32 * 17);
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) row[k1 * 17 + b] = f2mul(x[k1], s_tw[k1 * 16 + b]);
  __syncthreads();
  if (!valid) return;
  float f0 = a.scale;
  if (a.dec[0]) f0 *= a.dec[0][ix];
  const int64_t irow = (int64_t)ix * n1;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k1 = b + 16 * h;
    float2 w[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = row[k1 * 17 + q];
    dft16<false, SET == kHalf>(w);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      if (!out_on<SET>(k1, k2, n1)) continue;
      const int i1 = mode_to_img(k1 + 32 * k2, n1);
      float2 v = w[pos16(k2)];
      if (conj) v = f2conj(v);
      v = f2scale(v, a.dec[1] ? f0 * a.dec[1][i1] : f0);
      if (a.smaps) {
        const float2 s = a.smaps[(int64_t)c * g.Nimg + irow + i1];
        atomicAdd(a.out + irow + i1, make_float2(s.x * v.x + s.y * v.y, s.x * v.y - s.y * v.x));
      } else {
        float2* dst = a.out + (int64_t)c * g.Nimg + irow + i1;
        if (a.accumulate) v = f2add(v, *dst);
        *dst = v;
      }
    }
  }
}

// ---------------------------------------------------------------- x lines of the Toeplitz Gram
// Forward x transform (x-mode entries in), multiply by the real spectrum K,
// inverse x transform (x-mode entries out), per (y column, transform).
// blockIdx.x: 16 consecutive y columns; blockIdx.y: transform
template <int SET>
__global__ void __launch_bounds__(kT, 2)
f512_x_kmul_kernel(float2* data, int64_t G, int n0, const float* __restrict__ K,
                   const float2* __restrict__ tw) {
  extern __shared__ float2 s_dyn[];
  float2* const s_tw = s_dyn;
  float2* const s_x = s_tw + 512;
  s_tw[threadIdx.x] = tw[threadIdx.x];
  s_tw[threadIdx.x + kT] = tw[threadIdx.x + kT];
  const int l = threadIdx.x & 15, b = threadIdx.x >> 4;
  const int y = blockIdx.x * kL + l;
  float2* base = data + (int64_t)blockIdx.y * G + y;
  float2 x[32];
#pragma unroll
  for (int q = 0; q < 32; ++q)
    x[q] = in_on<SET>(q, b, n0) ? base[(16 * q + b) * kN] : make_float2(0.f, 0.f);
  __syncthreads();  // twiddle table
  dft32<SET == kHalf>(x);
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) s_x[(k1 * 16 + b) * kL + l] = f2mul(x[k1], s_tw[k1 * 16 + b]);
  __syncthreads();
  // X[b + 16 h + 32 k2] -> conj(K X) as the inverse transform's x[16 (h + 2 k2) + b]
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k1 = b + 16 * h;
    float2 w[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = s_x[(k1 * 16 + q) * kL + l];
    dft16(w);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2)
      x[h + 2 * k2] = f2conj(f2scale(w[pos16(k2)], K[(k1 + 32 * k2) * kN + y]));
  }
  dft32(x);
  __syncthreads();  // every thread has read its forward exchange entries
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) s_x[(k1 * 16 + b) * kL + l] = f2mul(x[k1], s_tw[k1 * 16 + b]);
  __syncthreads();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int k1 = b + 16 * h;
    float2 w[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) w[q] = s_x[(k1 * 16 + q) * kL + l];
    dft16<false, SET == kHalf>(w);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2)
      if (out_on<SET>(k1, k2, n0)) base[(k1 + 32 * k2) * kN] = f2conj(w[pos16(k2)]);
  }
}

template <typename F>
cudaError_t set_smem(F* k, size_t bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

F512Lines x_lines(float2* fine, const Geom& g, const float2* tw, int conj) {
  F512Lines x{};
  x.data = fine;
  x.G = g.G;
  x.n_axis = g.n[0];
  x.conj = conj;
  x.tw = tw;
  return x;
}

}  // namespace

bool fft512_fits(const Geom& g) { return g.dim == 2 && g.nf[0] == kN && g.nf[1] == kN; }

std::vector<float> fft512_twiddles() {
  // entry k1 * 16 + b (k1 < 32, b < 16): W512^(b k1), as (re, im)
  std::vector<float> t(1024);
  const double pi = 3.14159265358979323846;
  for (int k1 = 0; k1 < 32; ++k1)
    for (int b = 0; b < 16; ++b) {
      const int e = k1 * 16 + b;
      t[2 * e] = (float)std::cos(2.0 * pi * b * k1 / 512.0);
      t[2 * e + 1] = (float)-std::sin(2.0 * pi * b * k1 / 512.0);
    }
  return t;
}

cudaError_t fft512_prepare() {
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  chk(set_smem(f512_pad_y_kernel<kHalf>, kYSmem));
  chk(set_smem(f512_pad_y_kernel<kModes>, kYSmem));
  chk(set_smem(f512_crop_y_kernel<kHalf>, kYSmem));
  chk(set_smem(f512_crop_y_kernel<kModes>, kYSmem));
  chk(set_smem(f512_x_kernel<kHalf, kAll>, kXSmem));
  chk(set_smem(f512_x_kernel<kModes, kAll>, kXSmem));
  chk(set_smem(f512_x_kernel<kAll, kHalf>, kXSmem));
  chk(set_smem(f512_x_kernel<kAll, kModes>, kXSmem));
  chk(set_smem(f512_x_kmul_kernel<kHalf>, kXSmem));
  chk(set_smem(f512_x_kmul_kernel<kModes>, kXSmem));
  return e;
}

cudaError_t launch_fft512_op(const PadArgs& pa, const float2* tw, int isign, cudaStream_t st) {
  const Geom& g = pa.g;
  const int conj = isign > 0;
  const dim3 gy((g.n[0] + kL - 1) / kL, pa.ntr);
  if (g.n[1] == 256) f512_pad_y_kernel<kHalf><<<gy, kT, kYSmem, st>>>(pa, tw, conj);
  else f512_pad_y_kernel<kModes><<<gy, kT, kYSmem, st>>>(pa, tw, conj);
  const F512Lines x = x_lines(pa.fine, g, tw, conj);
  const dim3 gx(kN / kL, pa.ntr);
  if (g.n[0] == 256) f512_x_kernel<kHalf, kAll><<<gx, kT, kXSmem, st>>>(x);
  else f512_x_kernel<kModes, kAll><<<gx, kT, kXSmem, st>>>(x);
  return cudaGetLastError();
}

cudaError_t launch_fft512_adj(const CropArgs& ca, float2* fine, const float2* tw, int isign,
                              cudaStream_t st) {
  const Geom& g = ca.g;
  const int conj = isign > 0;
  const F512Lines x = x_lines(fine, g, tw, conj);
  const dim3 gx(kN / kL, ca.ntr);
  if (g.n[0] == 256) f512_x_kernel<kAll, kHalf><<<gx, kT, kXSmem, st>>>(x);
  else f512_x_kernel<kAll, kModes><<<gx, kT, kXSmem, st>>>(x);
  if (ca.smaps && !ca.accumulate) {  // the coil sum is added into the image
    cudaError_t e = cudaMemsetAsync(ca.out, 0, sizeof(float2) * (size_t)g.Nimg, st);
    if (e != cudaSuccess) return e;
  }
  const dim3 gy((g.n[0] + kL - 1) / kL, ca.ntr);
  if (g.n[1] == 256) f512_crop_y_kernel<kHalf><<<gy, kT, kYSmem, st>>>(ca, tw, conj);
  else f512_crop_y_kernel<kModes><<<gy, kT, kYSmem, st>>>(ca, tw, conj);
  return cudaGetLastError();
}

cudaError_t launch_fft512_gram(const PadArgs& pa, const CropArgs& ca, const float* K,
                               const float2* tw, cudaStream_t st) {
  const Geom& g = pa.g;
  const dim3 gy((g.n[0] + kL - 1) / kL, pa.ntr);
  if (g.n[1] == 256) f512_pad_y_kernel<kHalf><<<gy, kT, kYSmem, st>>>(pa, tw, 0);
  else f512_pad_y_kernel<kModes><<<gy, kT, kYSmem, st>>>(pa, tw, 0);
  const dim3 gx(kN / kL, pa.ntr);
  if (g.n[0] == 256) f512_x_kmul_kernel<kHalf><<<gx, kT, kXSmem, st>>>(pa.fine, g.G, g.n[0], K, tw);
  else f512_x_kmul_kernel<kModes><<<gx, kT, kXSmem, st>>>(pa.fine, g.G, g.n[0], K, tw);
  if (ca.smaps && !ca.accumulate) {
    cudaError_t e = cudaMemsetAsync(ca.out, 0, sizeof(float2) * (size_t)g.Nimg, st);
    if (e != cudaSuccess) return e;
  }
  if (g.n[1] == 256) f512_crop_y_kernel<kHalf><<<gy, kT, kYSmem, st>>>(ca, tw, 1);
  else f512_crop_y_kernel<kModes><<<gy, kT, kYSmem, st>>>(ca, tw, 1);
  return cudaGetLastError();
}

}  // namespace gbn
