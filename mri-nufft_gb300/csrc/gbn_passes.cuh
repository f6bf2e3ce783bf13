// Fused pad / crop passes and FP64 reductions.
#pragma once

#include "gbn_internal.cuh"

namespace gbn {

struct PadArgs {
  Geom g;
  const float2* img;    // SENSE: one image; calibrationless: ntr images
  const float2* smaps;  // SENSE: ntr coil maps (null: calibrationless)
  const float* dec[3];  // 1/phihat per axis, indexed by image array index (null: 1)
  float2* fine;         // ntr fine grids (every cell written)
  int ntr;
  int conj_in;          // use conj(img) and conj(smaps)
  float scale;
};

struct CropArgs {
  Geom g;
  const float2* fine;   // ntr fine grids
  const float2* smaps;  // SENSE coil maps (null: calibrationless)
  const float* dec[3];  // 1/phihat per axis (null: 1)
  float2* out;          // SENSE: one image; calibrationless: ntr images
  int ntr;
  int accumulate;       // out += result
  float scale;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // conj(a) * b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// pad pass for fine cell idx (see gbn_passes.cu)
template <int DIM>
__device__ __forceinline__ void pad_body(const PadArgs& a, const int64_t idx) {
  const Geom& g = a.g;
  if (idx >= g.G) return;
  int m[3] = {0, 0, 0};
  {
    int64_t r = idx;
    for (int d = DIM - 1; d >= 0; --d) {
      m[d] = (int)(r % g.nf[d]);
      r /= g.nf[d];
    }
  }
  bool inside = true;
  int64_t ii = 0;
  float f = a.scale;
  for (int d = 0; d < DIM; ++d) {
    int h = g.n[d] / 2;              // floor(N/2)
    int hi = g.n[d] - h;             // modes 0 .. hi-1 at the start
    int n;
    if (m[d] < hi) n = m[d];
    else if (m[d] >= g.nf[d] - h) n = m[d] - g.nf[d];
    else { inside = false; break; }
    int i = n + h;
    ii = ii * g.n[d] + i;
    if (a.dec[d]) f *= a.dec[d][i];
  }
  if (!inside) {
    for (int c = 0; c < a.ntr; ++c) a.fine[(int64_t)c * g.G + idx] = make_float2(0.f, 0.f);
    return;
  }
  if (a.smaps) {
    float2 x = a.img[ii];
    if (a.conj_in) x = conjf2(x);
    for (int c = 0; c < a.ntr; ++c) {
      float2 s = a.smaps[(int64_t)c * g.Nimg + ii];
      if (a.conj_in) s = conjf2(s);
      float2 v = cmul(x, s);
      a.fine[(int64_t)c * g.G + idx] = make_float2(v.x * f, v.y * f);
    }
  } else {
    for (int c = 0; c < a.ntr; ++c) {
      float2 x = a.img[(int64_t)c * g.Nimg + ii];
      if (a.conj_in) x = conjf2(x);
      a.fine[(int64_t)c * g.G + idx] = make_float2(x.x * f, x.y * f);
    }
  }
}

// crop pass for image pixel idx (see gbn_passes.cu)
template <int DIM>
__device__ __forceinline__ void crop_body(const CropArgs& a, const int64_t idx) {
  const Geom& g = a.g;
  if (idx >= g.Nimg) return;
  int64_t r = idx;
  int64_t mlin = 0;
  float f = a.scale;
  int i[3] = {0, 0, 0};
  for (int d = DIM - 1; d >= 0; --d) {
    i[d] = (int)(r % g.n[d]);
    r /= g.n[d];
  }
  for (int d = 0; d < DIM; ++d) {
    int n = i[d] - g.n[d] / 2;
    int m = n < 0 ? n + g.nf[d] : n;
    mlin = mlin * g.nf[d] + m;
    if (a.dec[d]) f *= a.dec[d][i[d]];
  }
  if (a.smaps) {
    float2 acc = make_float2(0.f, 0.f);
    for (int c = 0; c < a.ntr; ++c) {
      float2 v = a.fine[(int64_t)c * g.G + mlin];
      float2 s = a.smaps[(int64_t)c * g.Nimg + idx];
      float2 p = cmulc(s, v);
      acc.x += p.x;
      acc.y += p.y;
    }
    acc.x *= f;
    acc.y *= f;
    if (a.accumulate) {
      float2 o = a.out[idx];
      acc.x += o.x;
      acc.y += o.y;
    }
    a.out[idx] = acc;
  } else {
    for (int c = 0; c < a.ntr; ++c) {
      float2 v = a.fine[(int64_t)c * g.G + mlin];
      float2 r = make_float2(v.x * f, v.y * f);
      if (a.accumulate) {
        float2 o = a.out[(int64_t)c * g.Nimg + idx];
        r.x += o.x;
        r.y += o.y;
      }
      a.out[(int64_t)c * g.Nimg + idx] = r;
    }
  }
}

// Toeplitz embedding helpers: fine[t][i] *= K[i] for ntr grids of G cells;
// the lag-ordered placement of a type-1 transform on 2N modes into the
// circulant grid gt (lags |m| < N at m mod nf, zero elsewhere); real part
// with a scale; complex weights from real ones (null: ones).
cudaError_t launch_kmul(float2* fine, const float* K, int64_t G, int ntr, cudaStream_t st);
cudaError_t launch_toep_place(const Geom& gt, const float2* psf, float2* dst, cudaStream_t st);
cudaError_t launch_real_part(const float2* src, float* dst, int64_t n, float scale, cudaStream_t st);
cudaError_t launch_fill_weights(const float* w, float2* out, int64_t M, cudaStream_t st);
// out = -in (n complex values)
cudaError_t launch_neg_copy(const float2* in, float2* out, int64_t n, cudaStream_t st);
// CG reductions in one pass (FP64): st[0..1] = dotu(gn, gn), st[2..3] =
// dotu(gn, g), st[4..5] = dotu(g, g), st[6] = |gn|^2; st[7] is kept
cudaError_t launch_cg_dots(const float2* gnew, const float2* grad, int64_t n, double* st,
                           cudaStream_t s);
// Off-resonance time interpolators (B: NK x L, row-major; sample j of a
// shot uses row j mod NK): reduce y[b][c][j] = sum_l B[j][l] yl[b][l C + c][j];
// expand yl[b][l C + c][j] = conj(B[j][l]) y[b][c][j].
cudaError_t launch_orc_reduce(const float2* yl, const float2* Bt, float2* y, int nb, int L, int C,
                              int64_t M, int64_t NK, cudaStream_t st);
cudaError_t launch_orc_expand(const float2* y, const float2* Bt, float2* yl, int nb, int L, int C,
                              int64_t M, int64_t NK, cudaStream_t st);
cudaError_t launch_pad(const PadArgs& a, cudaStream_t st);
cudaError_t launch_crop(const CropArgs& a, cudaStream_t st);
cudaError_t launch_norm2(const float2* x, int64_t n, double* out, cudaStream_t st);
cudaError_t launch_dotu(const float2* a, const float2* b, int64_t n, int conj_a, double* out,
                        cudaStream_t st);
cudaError_t launch_cg_update(int64_t n, const float2* gnew, float2* grad, float2* vel, float2* img,
                             double* st, const float* L, float tol, cudaStream_t s);
cudaError_t launch_power_step(int64_t n, const float2* xnew, float2* x, double* st, float* L,
                              cudaStream_t s);
cudaError_t launch_scale_ratio(int64_t n, float2* x, const double* num2, const double* den2,
                               cudaStream_t s);

}  // namespace gbn
