// Pruned 3D transforms on 256^3 fine grids, fused with the pad and crop
// passes.
//
// The image modes of an N-point axis occupy the fine indices [0, N - N/2)
// and [256 - N/2, 256).  A type-2 transform (op) therefore starts from a
// grid that is non-zero only on the (x mode, y mode, z mode) cells, and a
// type-1 transform (adjoint) keeps only those cells of its result.  The
// library's cuFFT path writes every fine cell in the pad pass and runs full
// 2D transforms over the mode planes, then 1D transforms along x.  Here each
// axis is a separate pass of 256-point line transforms that reads only the
// lines and entries that can be non-zero and writes only the entries that a
// later pass reads:
//
//   op      z lines of the (x mode, y mode) columns, pad fused into the
//           loads (x * s * scale / phihat), 128 of 256 inputs per line;
//           y lines of the x-mode planes (mode entries in, all out);
//           x lines of every (y, z) (mode entries in, all out).
//   adjoint x lines of every (y, z) (all in, mode entries out);
//           y lines of the x-mode planes (all in, mode entries out);
//           z lines of the (x mode, y mode) columns (all in, mode entries
//           out), crop fused into the stores (divide by phihat, scale, and
//           the SENSE coil combine sum_c conj(s_c) v_c over the pass's coils).
//   Toeplitz Gram (256^3 circulant grid): the op's z and y passes, one pass
//           over the (y, z) lines doing the forward x transform, the
//           multiply by the spectrum and the inverse x transform, then the
//           adjoint's y and z passes.
//
// For a 128^3 image this moves about 350 MB per coil and transform against
// about 670 MB for the pad pass plus the pruned cuFFT passes.  For 128-point
// image axes the entries of a line that hold modes are whole rows of the
// four-step layout (q < 4 and q >= 12 below), a compile-time set (kHalf);
// other sizes test each entry at run time (kModes).
//
// A 256-point line transform is two 16-point DFTs in registers with one
// exchange through shared memory (four-step: n = 16 a + b, k = k1 + 16 k2):
//   Y_b[k1] = sum_a x[16 a + b] W16^(a k1),   Z_b[k1] = Y_b[k1] W256^(b k1),
//   X[k1 + 16 k2] = sum_b Z_b[k1] W16^(b k2).
// A thread owns one (line, b) in the first step and one (line, k1) in the
// second.  The 16-point DFT is radix 4 x 4.  The exponent sign is -1; a +1
// transform conjugates its inputs and outputs.  The twiddles W256^(b k1)
// come from a table computed in double precision on the host, laid out
// [k1][b] so that lanes running over b read consecutive entries.
//
// Thread layouts (256 threads, 16 lines per CTA):
//   z lines (contiguous in memory): lanes run over b (first step) or k1
//     (second step) of two lines, so each global access is a 128-byte row
//     segment; the exchange buffer [line][k1][b] has a row pitch of 17
//     cells, which keeps both steps free of bank conflicts;
//   x / y lines (stride 256 or 65536 cells): lanes run over 16 consecutive
//     z columns, so each global access is again a 128-byte segment; the
//     exchange buffer is [k1][b][z].
#include "gbn_fft256.cuh"
#include "gbn_dft.cuh"

#include <cmath>
#include <vector>

namespace gbn {

namespace {

using namespace dft;

constexpr int kF256Lines = 16;       // lines per CTA
constexpr int kF256Threads = 256;

// modes of an n-point axis on the 256-point fine axis
__device__ __forceinline__ bool is_mode(int m, int n) {
  const int h = n >> 1;
  return m < n - h || m >= 256 - h;
}
__device__ __forceinline__ int mode_to_img(int m, int n) {  // image array index of fine index m
  const int h = n >> 1;
  return m < n - h ? m + h : m - 256 + h;
}
__device__ __forceinline__ int img_to_fine(int i, int n) {
  const int k = i - (n >> 1);
  return k < 0 ? k + 256 : k;
}

// Entry m = 16 q + b of a line, for the mode sets of the transformed axis:
// kAll (every entry), kHalf (n = 128: the modes are the rows q < 4 and
// q >= 12, known at compile time in the unrolled loops), kModes (any n <= 256).
enum : int { kAll = 0, kHalf = 1, kModes = 2 };
template <int SET>
__device__ __forceinline__ bool entry_on(int q, int b, int n) {
  if (SET == kAll) return true;
  if (SET == kHalf) return q < 4 || q >= 12;
  return is_mode(16 * q + b, n);
}
template <int SET>
__device__ __forceinline__ int entry_img(int q, int b, int n) {  // image index of a mode entry
  if (SET == kHalf) return q < 4 ? 16 * q + b + 64 : 16 * q + b - 192;
  return mode_to_img(16 * q + b, n);
}

// ---------------------------------------------------------------- z lines, pad fused
// blockIdx.x: 16 consecutive (ix, iy) image columns; blockIdx.y: transform;
// SET: the z modes (kHalf for n2 = 128, else kModes)
template <int SET>
__global__ void __launch_bounds__(kF256Threads)
f256_pad_z_kernel(PadArgs a, const float2* __restrict__ tw, int conj) {
  __shared__ float2 s_tw[256];
  __shared__ float2 s_x[kF256Lines * 16 * 17];
  const Geom& g = a.g;
  const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
  s_tw[threadIdx.x] = tw[threadIdx.x];
  const int b = threadIdx.x & 15, l = threadIdx.x >> 4;
  const int line = blockIdx.x * kF256Lines + l;
  const bool valid = line < n0 * n1;
  const int ix = valid ? line / n1 : 0, iy = valid ? line - ix * n1 : 0;
  const int c = blockIdx.y;
  const int64_t irow = ((int64_t)ix * n1 + iy) * n2;
  const float2* img = a.smaps ? a.img : a.img + (int64_t)c * g.Nimg;
  const float2* sm = a.smaps ? a.smaps + (int64_t)c * g.Nimg : nullptr;
  float f0 = a.scale;
  if (a.dec[0]) f0 *= a.dec[0][ix];
  if (a.dec[1]) f0 *= a.dec[1][iy];
  float2 x[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    float2 v = make_float2(0.f, 0.f);
    if (valid && entry_on<SET>(q, b, n2)) {
      const int i2 = entry_img<SET>(q, b, n2);
      v = img[irow + i2];
      if (a.conj_in) v = f2conj(v);
      if (sm) {
        float2 s = sm[irow + i2];
        if (a.conj_in) s = f2conj(s);
        v = f2mul(v, s);
      }
      v = f2scale(v, a.dec[2] ? f0 * a.dec[2][i2] : f0);
      if (conj) v = f2conj(v);
    }
    x[q] = v;
  }
  __syncthreads();  // twiddle table
  dft16<SET == kHalf>(x);
  float2* row = s_x + l * (16 * 17);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) row[k1 * 17 + b] = f2mul(x[pos16(k1)], s_tw[k1 * 16 + b]);
  __syncthreads();
  const int k1 = b;
#pragma unroll
  for (int q = 0; q < 16; ++q) x[q] = row[k1 * 17 + q];
  dft16(x);
  if (!valid) return;
  float2* out = a.fine + (int64_t)c * g.G +
                ((int64_t)img_to_fine(ix, n0) * 256 + img_to_fine(iy, n1)) * 256 + k1;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    const float2 v = x[pos16(k2)];
    out[16 * k2] = conj ? f2conj(v) : v;
  }
}

// ---------------------------------------------------------------- x / y lines
struct F256Lines {
  float2* data;       // ntr grids of G cells
  int64_t G;
  int64_t line_stride;   // cells between consecutive entries of a line
  int64_t outer_stride;  // cells between consecutive outer indices
  int outer_modes;       // outer index o is an image index of an n_outer-point axis
  int n_outer;
  int n_axis;            // image size along the transformed axis
  int in_prune;          // only mode entries are read (the others are zero)
  int out_prune;         // only mode entries are written
  int conj;
  const float2* tw;
};

// blockIdx.x: 16 consecutive z columns; blockIdx.y: outer index; blockIdx.z: transform
// IN / OUT: the entries read / written (kAll, kHalf, kModes of n_axis)
template <int MINB, int IN, int OUT>
__global__ void __launch_bounds__(kF256Threads, MINB) f256_lines_kernel(F256Lines a) {
  __shared__ float2 s_tw[256];
  __shared__ float2 s_x[16 * 16 * kF256Lines];
  s_tw[threadIdx.x] = a.tw[threadIdx.x];
  const int l = threadIdx.x & 15, b = threadIdx.x >> 4;
  const int z = blockIdx.x * kF256Lines + l;
  const int o = a.outer_modes ? img_to_fine(blockIdx.y, a.n_outer) : (int)blockIdx.y;
  float2* base = a.data + (int64_t)blockIdx.z * a.G + o * a.outer_stride + z;
  float2 x[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    float2 v = make_float2(0.f, 0.f);
    if (entry_on<IN>(q, b, a.n_axis)) {
      v = base[(16 * q + b) * a.line_stride];
      if (a.conj) v = f2conj(v);
    }
    x[q] = v;
  }
  __syncthreads();  // twiddle table
  dft16<IN == kHalf>(x);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) s_x[(k1 * 16 + b) * 16 + l] = f2mul(x[pos16(k1)], s_tw[k1 * 16 + b]);
  __syncthreads();
  const int k1 = b;
#pragma unroll
  for (int q = 0; q < 16; ++q) x[q] = s_x[(k1 * 16 + q) * 16 + l];
  dft16<false, OUT == kHalf>(x);
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    if (entry_on<OUT>(k2, k1, a.n_axis)) {
      const float2 v = x[pos16(k2)];
      base[(k1 + 16 * k2) * a.line_stride] = a.conj ? f2conj(v) : v;
    }
  }
}

// ---------------------------------------------------------------- z lines, crop fused
// blockIdx.x: 16 consecutive (ix, iy) image columns; the CTA runs every
// transform of the pass and, with coil maps, sums them into one image
constexpr size_t kCropSmem = (256 + kF256Lines * 16 * 17 + kF256Lines * 16 * 16) * sizeof(float2);

template <int MINB, int SET>
__global__ void __launch_bounds__(kF256Threads, MINB)
f256_z_crop_kernel(CropArgs a, const float2* __restrict__ tw, int conj) {
  // dynamic: twiddles, the exchange buffer, and the coil sums [line][k2][k1]
  // (thread (line, k1) owns its 16 entries)
  extern __shared__ float2 s_dyn[];
  float2* const s_tw = s_dyn;
  float2* const s_x = s_tw + 256;
  float2* const s_acc = s_x + kF256Lines * 16 * 17;
  const Geom& g = a.g;
  const int n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
  s_tw[threadIdx.x] = tw[threadIdx.x];
  const int b = threadIdx.x & 15, l = threadIdx.x >> 4;
  const int line = blockIdx.x * kF256Lines + l;
  const bool valid = line < n0 * n1;
  const int ix = valid ? line / n1 : 0, iy = valid ? line - ix * n1 : 0;
  const int64_t irow = ((int64_t)ix * n1 + iy) * n2;
  const int64_t frow = ((int64_t)img_to_fine(ix, n0) * 256 + img_to_fine(iy, n1)) * 256;
  float f0 = a.scale;
  if (a.dec[0]) f0 *= a.dec[0][ix];
  if (a.dec[1]) f0 *= a.dec[1][iy];
  float2* row = s_x + l * (16 * 17);
  const int k1 = b;
  float2* acc = s_acc + l * 256 + k1;  // entry k2 at acc[16 * k2]
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) acc[16 * k2] = make_float2(0.f, 0.f);
  for (int c = 0; c < a.ntr; ++c) {
    const float2* in = a.fine + (int64_t)c * g.G + frow;
    float2 x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float2 v = valid ? in[16 * q + b] : make_float2(0.f, 0.f);
      x[q] = conj ? f2conj(v) : v;
    }
    __syncthreads();  // twiddle table; the previous transform's exchange reads are done
    dft16(x);
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) row[kk * 17 + b] = f2mul(x[pos16(kk)], s_tw[kk * 16 + b]);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) x[q] = row[k1 * 17 + q];
    dft16<false, SET == kHalf>(x);
    if (!valid) continue;
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) {
      if (!entry_on<SET>(k2, k1, n2)) continue;
      const int i2 = entry_img<SET>(k2, k1, n2);
      float2 v = x[pos16(k2)];
      if (conj) v = f2conj(v);
      if (a.smaps) {
        const float2 s = a.smaps[(int64_t)c * g.Nimg + irow + i2];
        const float2 o = acc[16 * k2];
        acc[16 * k2] = make_float2(o.x + s.x * v.x + s.y * v.y, o.y + s.x * v.y - s.y * v.x);
      } else {
        const float f = a.dec[2] ? f0 * a.dec[2][i2] : f0;
        float2 r = f2scale(v, f);
        float2* dst = a.out + (int64_t)c * g.Nimg + irow + i2;
        if (a.accumulate) r = f2add(r, *dst);
        *dst = r;
      }
    }
  }
  if (!a.smaps || !valid) return;
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    if (!entry_on<SET>(k2, k1, n2)) continue;
    const int i2 = entry_img<SET>(k2, k1, n2);
    const float f = a.dec[2] ? f0 * a.dec[2][i2] : f0;
    float2 r = f2scale(acc[16 * k2], f);
    float2* dst = a.out + irow + i2;
    if (a.accumulate) r = f2add(r, *dst);
    *dst = r;
  }
}

// ---------------------------------------------------------------- x lines of the Toeplitz Gram
// Forward x transform (x-mode entries in), multiply by the real kernel K,
// inverse x transform (x-mode entries out) of every (y, z) line, for every
// transform of the pass, without writing the full grid.  After the forward
// transform's second step thread (z, k1) holds X[k1 + 16 k2], k2 = 0 .. 15,
// which are exactly the inputs x[16 a + b] (a = k2) of the inverse
// transform's first step for b = k1, so the two transforms share one layout.
// blockIdx.x: 16 consecutive z columns; blockIdx.y: y
template <int SET>
__global__ void __launch_bounds__(kF256Threads, 4)
f256_x_kmul_kernel(float2* data, int64_t G, int ntr, int n0, const float* __restrict__ K,
                   const float2* __restrict__ tw) {
  __shared__ float2 s_tw[256];
  __shared__ float2 s_x[16 * 16 * kF256Lines];
  s_tw[threadIdx.x] = tw[threadIdx.x];
  const int l = threadIdx.x & 15, b = threadIdx.x >> 4;
  const int z = blockIdx.x * kF256Lines + l;
  const int64_t col = (int64_t)blockIdx.y * 256 + z;
  constexpr int64_t XS = 256 * 256;  // x stride
  float kk[16];  // K at x = b + 16 k2 (b is k1 in the forward transform's second step)
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) kk[k2] = K[(b + 16 * k2) * XS + col];
  for (int c = 0; c < ntr; ++c) {
    float2* base = data + (int64_t)c * G + col;
    float2 x[16];
#pragma unroll
    for (int q = 0; q < 16; ++q)
      x[q] = entry_on<SET>(q, b, n0) ? base[(16 * q + b) * XS] : make_float2(0.f, 0.f);
    __syncthreads();  // twiddles; the previous transform's exchange reads are done
    dft16<SET == kHalf>(x);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) s_x[(k1 * 16 + b) * 16 + l] = f2mul(x[pos16(k1)], s_tw[k1 * 16 + b]);
    __syncthreads();
    // thread (z, k1 = b): X[k1 + 16 k2] -> conj(K X) as the inverse transform's x[16 k2 + k1]
    float2 y[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) y[q] = s_x[(b * 16 + q) * 16 + l];
    dft16(y);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) x[k2] = f2conj(f2scale(y[pos16(k2)], kk[k2]));
    dft16(x);
    __syncthreads();  // every thread has read its forward exchange entries
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) s_x[(k1 * 16 + b) * 16 + l] = f2mul(x[pos16(k1)], s_tw[k1 * 16 + b]);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) y[q] = s_x[(b * 16 + q) * 16 + l];
    dft16<false, SET == kHalf>(y);
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2)
      if (entry_on<SET>(k2, b, n0)) base[(b + 16 * k2) * XS] = f2conj(y[pos16(k2)]);
  }
}

}  // namespace

cudaError_t fft256_prepare() {
  return cudaFuncSetAttribute(f256_z_crop_kernel<3, kModes>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCropSmem);
}

bool fft256_fits(const Geom& g) {
  return g.dim == 3 && g.nf[0] == 256 && g.nf[1] == 256 && g.nf[2] == 256;
}

std::vector<float> fft256_twiddles() {
  // entry k1 * 16 + b: W256^(b k1) = exp(-2 pi i b k1 / 256), as (re, im)
  std::vector<float> t(512);
  const double pi = 3.14159265358979323846;
  for (int k1 = 0; k1 < 16; ++k1)
    for (int b = 0; b < 16; ++b) {
      const int e = k1 * 16 + b;
      t[2 * e] = (float)std::cos(2.0 * pi * b * k1 / 256.0);
      t[2 * e + 1] = (float)-std::sin(2.0 * pi * b * k1 / 256.0);
    }
  return t;
}

namespace {
// 4 CTAs per SM (64 registers, a few bytes of spills) measured 5 % faster
// than 3 CTAs at 80 registers on the 128^3 passes
void lines(const F256Lines& a, dim3 grid, cudaStream_t st) {
  const bool half = a.n_axis == 128;
  if (a.in_prune) {
    if (half) f256_lines_kernel<4, kHalf, kAll><<<grid, kF256Threads, 0, st>>>(a);
    else f256_lines_kernel<4, kModes, kAll><<<grid, kF256Threads, 0, st>>>(a);
  } else if (a.out_prune) {
    if (half) f256_lines_kernel<4, kAll, kHalf><<<grid, kF256Threads, 0, st>>>(a);
    else f256_lines_kernel<4, kAll, kModes><<<grid, kF256Threads, 0, st>>>(a);
  } else {
    f256_lines_kernel<4, kAll, kAll><<<grid, kF256Threads, 0, st>>>(a);
  }
}

void pad_z(const PadArgs& pa, const float2* tw, int conj, cudaStream_t st) {
  const int nl = pa.g.n[0] * pa.g.n[1];
  const dim3 grid((nl + kF256Lines - 1) / kF256Lines, pa.ntr);
  if (pa.g.n[2] == 128) f256_pad_z_kernel<kHalf><<<grid, kF256Threads, 0, st>>>(pa, tw, conj);
  else f256_pad_z_kernel<kModes><<<grid, kF256Threads, 0, st>>>(pa, tw, conj);
}

// coil sums in shared memory: 3 CTAs per SM (69 against 86 us with the sums
// in registers at 2 CTAs per SM, 4 coils of a 128^3 image); the runtime mode
// test (kModes) also for n2 = 128: the kHalf instance measured 90 us
cudaError_t z_crop(const CropArgs& ca, const float2* tw, int conj, cudaStream_t st) {
  const int nl = ca.g.n[0] * ca.g.n[1];
  const unsigned nb = (nl + kF256Lines - 1) / kF256Lines;
  f256_z_crop_kernel<3, kModes><<<nb, kF256Threads, kCropSmem, st>>>(ca, tw, conj);
  return cudaGetLastError();
}

F256Lines y_lines(float2* fine, const Geom& g, const float2* tw, int in_prune, int conj) {
  F256Lines y{};
  y.data = fine;
  y.G = g.G;
  y.line_stride = 256;
  y.outer_stride = 256 * 256;
  y.outer_modes = 1;
  y.n_outer = g.n[0];
  y.n_axis = g.n[1];
  y.in_prune = in_prune;
  y.out_prune = !in_prune;
  y.conj = conj;
  y.tw = tw;
  return y;
}

F256Lines x_lines(float2* fine, const Geom& g, const float2* tw, int in_prune, int conj) {
  F256Lines x{};
  x.data = fine;
  x.G = g.G;
  x.line_stride = 256 * 256;
  x.outer_stride = 256;
  x.outer_modes = 0;
  x.n_outer = 256;
  x.n_axis = g.n[0];
  x.in_prune = in_prune;
  x.out_prune = !in_prune;
  x.conj = conj;
  x.tw = tw;
  return x;
}
}  // namespace

cudaError_t launch_fft256_op(const PadArgs& pa, const float2* tw, int isign, cudaStream_t st) {
  const Geom& g = pa.g;
  const int conj = isign > 0;
  pad_z(pa, tw, conj, st);
  lines(y_lines(pa.fine, g, tw, 1, conj), dim3(256 / kF256Lines, g.n[0], pa.ntr), st);
  lines(x_lines(pa.fine, g, tw, 1, conj), dim3(256 / kF256Lines, 256, pa.ntr), st);
  return cudaGetLastError();
}

cudaError_t launch_fft256_adj(const CropArgs& ca, float2* fine, const float2* tw, int isign,
                              cudaStream_t st) {
  const Geom& g = ca.g;
  const int conj = isign > 0;
  lines(x_lines(fine, g, tw, 0, conj), dim3(256 / kF256Lines, 256, ca.ntr), st);
  lines(y_lines(fine, g, tw, 0, conj), dim3(256 / kF256Lines, g.n[0], ca.ntr), st);
  return z_crop(ca, tw, conj, st);
}

cudaError_t launch_fft256_gram(const PadArgs& pa, const CropArgs& ca, const float* K,
                               const float2* tw, cudaStream_t st) {
  const Geom& g = pa.g;
  pad_z(pa, tw, 0, st);
  lines(y_lines(pa.fine, g, tw, 1, 0), dim3(256 / kF256Lines, g.n[0], pa.ntr), st);
  const dim3 grid(256 / kF256Lines, 256);
  if (g.n[0] == 128)
    f256_x_kmul_kernel<kHalf><<<grid, kF256Threads, 0, st>>>(pa.fine, g.G, pa.ntr, g.n[0], K, tw);
  else
    f256_x_kmul_kernel<kModes><<<grid, kF256Threads, 0, st>>>(pa.fine, g.G, pa.ntr, g.n[0], K, tw);
  lines(y_lines(pa.fine, g, tw, 0, 1), dim3(256 / kF256Lines, g.n[0], pa.ntr), st);
  return z_crop(ca, tw, 1, st);
}

}  // namespace gbn
