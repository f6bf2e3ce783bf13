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
// Toeplitz embedding of A^H W A
// ---------------------------------------------------------------------------
// fine[t][i] *= K[i]: K is read once per cell for all ntr grids
__global__ void kmul_kernel(float2* __restrict__ fine, const float* __restrict__ K, int64_t G,
                            int ntr) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < G;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float k = K[i];
    for (int t = 0; t < ntr; ++t) {
      float2 v = fine[(int64_t)t * G + i];
      fine[(int64_t)t * G + i] = make_float2(v.x * k, v.y * k);
    }
  }
}

// dst (circulant grid, nf per axis) <- psf (2N modes per axis, mode m at
// array index m + N) for lags |m| < N at index m mod nf; other cells 0
__global__ void toep_place_kernel(Geom gt, const float2* __restrict__ psf,
                                  float2* __restrict__ dst) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= gt.G) return;
  int64_t r = idx, src = 0;
  bool inside = true;
  int p[3] = {0, 0, 0};
  for (int d = gt.dim - 1; d >= 0; --d) {
    p[d] = (int)(r % gt.nf[d]);
    r /= gt.nf[d];
  }
  for (int d = 0; d < gt.dim; ++d) {
    const int N = gt.n[d], P = gt.nf[d];
    int m;
    if (p[d] < N) m = p[d];
    else if (p[d] > P - N) m = p[d] - P;
    else { inside = false; break; }
    src = src * (2 * N) + (m + N);
  }
  dst[idx] = inside ? psf[src] : make_float2(0.f, 0.f);
}

__global__ void real_part_kernel(const float2* __restrict__ src, float* __restrict__ dst, int64_t n,
                                 float scale) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i].x * scale;
}

__global__ void fill_weights_kernel(const float* __restrict__ w, float2* __restrict__ out,
                                    int64_t M) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < M;
       j += (int64_t)gridDim.x * blockDim.x)
    out[j] = make_float2(w ? w[j] : 1.0f, 0.0f);
}

static unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

cudaError_t launch_kmul(float2* fine, const float* K, int64_t G, int ntr, cudaStream_t st) {
  kmul_kernel<<<grid_for(G), 256, 0, st>>>(fine, K, G, ntr);
  return cudaGetLastError();
}

cudaError_t launch_toep_place(const Geom& gt, const float2* psf, float2* dst, cudaStream_t st) {
  toep_place_kernel<<<(unsigned)((gt.G + 255) / 256), 256, 0, st>>>(gt, psf, dst);
  return cudaGetLastError();
}

cudaError_t launch_real_part(const float2* src, float* dst, int64_t n, float scale, cudaStream_t st) {
  real_part_kernel<<<grid_for(n), 256, 0, st>>>(src, dst, n, scale);
  return cudaGetLastError();
}

cudaError_t launch_fill_weights(const float* w, float2* out, int64_t M, cudaStream_t st) {
  if (M == 0) return cudaSuccess;
  fill_weights_kernel<<<grid_for(M), 256, 0, st>>>(w, out, M);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Off-resonance interpolator passes
// ---------------------------------------------------------------------------
__global__ void orc_reduce_kernel(const float2* __restrict__ yl, const float2* __restrict__ Bt,
                                  float2* __restrict__ y, int nb, int L, int C, int64_t M,
                                  int64_t NK) {
  const int64_t total = (int64_t)nb * C * M;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i % M;
    const int64_t bc = i / M;
    const int64_t b = bc / C, c = bc - b * C;
    const float2* brow = Bt + (j % NK) * L;
    float2 acc = make_float2(0.f, 0.f);
    for (int l = 0; l < L; ++l) {
      const float2 w = brow[l];
      const float2 v = yl[((b * L + l) * C + c) * M + j];
      acc.x += w.x * v.x - w.y * v.y;
      acc.y += w.x * v.y + w.y * v.x;
    }
    y[i] = acc;
  }
}

__global__ void orc_expand_kernel(const float2* __restrict__ y, const float2* __restrict__ Bt,
                                  float2* __restrict__ yl, int nb, int L, int C, int64_t M,
                                  int64_t NK) {
  const int64_t total = (int64_t)nb * C * M;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i % M;
    const int64_t bc = i / M;
    const int64_t b = bc / C, c = bc - b * C;
    const float2* brow = Bt + (j % NK) * L;
    const float2 v = y[i];
    for (int l = 0; l < L; ++l) {
      const float2 w = brow[l];  // conj(w) * v
      yl[((b * L + l) * C + c) * M + j] = make_float2(w.x * v.x + w.y * v.y, w.x * v.y - w.y * v.x);
    }
  }
}

cudaError_t launch_orc_reduce(const float2* yl, const float2* Bt, float2* y, int nb, int L, int C,
                              int64_t M, int64_t NK, cudaStream_t st) {
  if ((int64_t)nb * C * M == 0) return cudaSuccess;
  orc_reduce_kernel<<<grid_for((int64_t)nb * C * M), 256, 0, st>>>(yl, Bt, y, nb, L, C, M, NK);
  return cudaGetLastError();
}

cudaError_t launch_orc_expand(const float2* y, const float2* Bt, float2* yl, int nb, int L, int C,
                              int64_t M, int64_t NK, cudaStream_t st) {
  if ((int64_t)nb * C * M == 0) return cudaSuccess;
  orc_expand_kernel<<<grid_for((int64_t)nb * C * M), 256, 0, st>>>(y, Bt, yl, nb, L, C, M, NK);
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

// ---------------------------------------------------------------------------
// Device-side solver updates (no host synchronisation inside a solve)
// ---------------------------------------------------------------------------
namespace gbn {

// state layout (doubles): [0,1] dot(g_new, g_new)  [2,3] dot(g_new, g)
//                         [4,5] dot(g, g)          [6] |g_new|^2  [7] done flag
__global__ void cg_update_kernel(int64_t n, const float2* __restrict__ gnew, float2* grad,
                                 float2* vel, float2* img, const double* st, const float* L,
                                 float tol) {
  if (st[7] != 0.0) return;
  const double nrm = sqrt(st[6]);
  if (!(nrm > (double)tol)) return;  // the state kernel marks the solve done
  // beta = (dot(gn, gn) - dot(gn, g)) / dot(g, g) (complex), then numpy's
  // max(0, beta): kept when Re > 0 or (Re == 0 and Im > 0), else 0
  const double nr = st[0] - st[2], ni = st[1] - st[3], dr = st[4], di = st[5];
  const double dd = dr * dr + di * di;
  double br = (nr * dr + ni * di) / dd;
  double bi = (ni * dr - nr * di) / dd;
  if (!(br > 0.0 || (br == 0.0 && bi > 0.0))) {
    br = 0.0;
    bi = 0.0;
  }
  const float fbr = (float)br, fbi = (float)bi, invL = 1.0f / *L;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 g = gnew[i];
    const float2 v = vel[i];
    const float2 nv = make_float2(g.x + fbr * v.x - fbi * v.y, g.y + fbr * v.y + fbi * v.x);
    vel[i] = nv;
    float2 x = img[i];
    x.x -= nv.x * invL;
    x.y -= nv.y * invL;
    img[i] = x;
    grad[i] = g;
  }
}

__global__ void cg_state_kernel(double* st, float tol) {
  if (st[7] == 0.0 && !(sqrt(st[6]) > (double)tol)) st[7] = 1.0;
}

// power method state (doubles): [0] |x_new|^2 [1] x_norm [2] L [3] converged
__global__ void power_normalize_kernel(int64_t n, const float2* __restrict__ xnew, float2* x,
                                       const double* st) {
  if (st[3] != 0.0) return;
  const float inv = (float)(1.0 / sqrt(st[0]));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = xnew[i];
    x[i] = make_float2(v.x * inv, v.y * inv);
  }
}

__global__ void power_state_kernel(double* st, float* L) {
  if (st[3] != 0.0) return;
  const double nn = sqrt(st[0]);
  st[2] = nn;
  *L = (float)nn;
  if (fabs(st[1] - nn) < 1e-6) st[3] = 1.0;
  st[1] = nn;
}

// x *= sqrt(num2 / den2), both squared norms on the device
__global__ void scale_ratio_kernel(int64_t n, float2* x, const double* num2, const double* den2) {
  const float s = (float)sqrt(*num2 / *den2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float2 v = x[i];
    x[i] = make_float2(v.x * s, v.y * s);
  }
}

static unsigned elem_blocks(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)(b < 1216 ? (b < 1 ? 1 : b) : 1216);
}

__global__ void neg_copy_kernel(const float2* __restrict__ in, float2* __restrict__ out, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = make_float2(-v.x, -v.y);
  }
}

__global__ void cg_dots_kernel(const float2* __restrict__ gn, const float2* __restrict__ g,
                               int64_t n, double* st) {
  __shared__ double sm[7][32];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = gn[i], b = g[i];
    const double ar = a.x, ai = a.y, br = b.x, bi = b.y;
    acc[0] += ar * ar - ai * ai;  // dotu(gn, gn) (non-conjugating)
    acc[1] += 2.0 * ar * ai;
    acc[2] += ar * br - ai * bi;  // dotu(gn, g)
    acc[3] += ar * bi + ai * br;
    acc[4] += br * br - bi * bi;  // dotu(g, g)
    acc[5] += 2.0 * br * bi;
    acc[6] += ar * ar + ai * ai;  // |gn|^2
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    double v = warp_sum(acc[k]);
    if (lane == 0) sm[k][wid] = v;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      double v = lane < (int)(blockDim.x >> 5) ? sm[k][lane] : 0.0;
      v = warp_sum(v);
      if (lane == 0) atomicAdd(&st[k], v);
    }
  }
}

cudaError_t launch_neg_copy(const float2* in, float2* out, int64_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  neg_copy_kernel<<<elem_blocks(n), 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t launch_cg_dots(const float2* gnew, const float2* grad, int64_t n, double* st,
                           cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(st, 0, 7 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  cg_dots_kernel<<<reduce_blocks(n), 256, 0, s>>>(gnew, grad, n, st);
  return cudaGetLastError();
}

cudaError_t launch_cg_update(int64_t n, const float2* gnew, float2* grad, float2* vel, float2* img,
                             double* st, const float* L, float tol, cudaStream_t s) {
  cg_update_kernel<<<elem_blocks(n), 256, 0, s>>>(n, gnew, grad, vel, img, st, L, tol);
  cg_state_kernel<<<1, 1, 0, s>>>(st, tol);
  return cudaGetLastError();
}

cudaError_t launch_power_step(int64_t n, const float2* xnew, float2* x, double* st, float* L,
                              cudaStream_t s) {
  power_normalize_kernel<<<elem_blocks(n), 256, 0, s>>>(n, xnew, x, st);
  power_state_kernel<<<1, 1, 0, s>>>(st, L);
  return cudaGetLastError();
}

cudaError_t launch_scale_ratio(int64_t n, float2* x, const double* num2, const double* den2,
                               cudaStream_t s) {
  scale_ratio_kernel<<<elem_blocks(n), 256, 0, s>>>(n, x, num2, den2);
  return cudaGetLastError();
}

}  // namespace gbn
