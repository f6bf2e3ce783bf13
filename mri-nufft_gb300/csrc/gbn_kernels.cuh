// Spreading (type 1), interpolation (type 2) and kernel-derivative
// interpolation kernels over bin-sorted samples.
//
// One CTA handles one subproblem: up to `maxsub` samples of one bin.  The
// padded fine-grid tile of the bin (bin extent + w cells per axis, with
// periodic wrap) is staged in shared memory for `CG` transforms (coils) at a
// time.  Kernel weights are evaluated once per sample and axis per coil pass
// and reused by every coil of the pass.
//   interp: tile <- fine grid (coalesced rows), each thread gathers its
//           samples' w^d footprints from shared memory;
//   spread: threads scatter into the shared tile with shared-memory atomics,
//           then the tile is added to the fine grid with vector float2 global
//           atomics (tiles of neighbouring bins overlap by w cells, so the
//           halo cells receive contributions from several CTAs).
#pragma once

#include "gbn_internal.cuh"

// Full unrolling for compile-time widths only; the runtime-width fallback
// keeps rolled loops so that it compiles quickly.
#define GBN_UNROLL _Pragma("unroll")

namespace gbn {

// W > 0: compile-time width; W == 0: runtime width g.w <= 16.
template <int W>
struct WidthTraits {
  static constexpr int WM = W > 0 ? W : 16;
};

template <int W>
__device__ __forceinline__ int weights_rt(float u, const Geom& g, float* wt) {
  constexpr int WM = WidthTraits<W>::WM;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;
  float s = u - g.halfw;
  int i0 = (int)ceilf(s);
  float x0 = (float)i0 - u;
GBN_UNROLL
  for (int t = 0; t < WM; ++t)
    wt[t] = (W > 0 || t < w) ? es_eval(x0 + (float)t, g.beta, g.inv_halfw) : 0.0f;
  return i0;
}

template <int W>
__device__ __forceinline__ int weights_rt_d(float u, const Geom& g, float* wt, float* dw) {
  constexpr int WM = WidthTraits<W>::WM;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;
  float s = u - g.halfw;
  int i0 = (int)ceilf(s);
  float x0 = (float)i0 - u;
GBN_UNROLL
  for (int t = 0; t < WM; ++t) {
    bool on = (W > 0 || t < w);
    wt[t] = on ? es_eval(x0 + (float)t, g.beta, g.inv_halfw) : 0.0f;
    // d/du phi(m - u) = -phi'(m - u)
    dw[t] = on ? -es_deriv(x0 + (float)t, g.beta, g.inv_halfw) : 0.0f;
  }
  return i0;
}

template <int DIM>
__device__ __forceinline__ void bin_origin(const Geom& g, int b, int* o) {
  // bins are numbered with axis 0 slowest
  int r = b;
  for (int d = DIM - 1; d >= 0; --d) {
    int bd = r % g.nb[d];
    r /= g.nb[d];
    o[d] = bd * g.bs[d] - (g.w >> 1);
  }
}

// fine-grid linear offset of tile cell r (row-major over pd) with wrap
template <int DIM>
__device__ __forceinline__ int64_t tile_to_fine(const Geom& g, const int* o, int r) {
  if (DIM == 2) {
    int i1 = r % g.pd[1];
    int i0 = r / g.pd[1];
    int m0 = wrap_idx(o[0] + i0, g.nf[0]);
    int m1 = wrap_idx(o[1] + i1, g.nf[1]);
    return (int64_t)m0 * g.nf[1] + m1;
  } else {
    int i2 = r % g.pd[2];
    int q = r / g.pd[2];
    int i1 = q % g.pd[1];
    int i0 = q / g.pd[1];
    int m0 = wrap_idx(o[0] + i0, g.nf[0]);
    int m1 = wrap_idx(o[1] + i1, g.nf[1]);
    int m2 = wrap_idx(o[2] + i2, g.nf[2]);
    return ((int64_t)m0 * g.nf[1] + m1) * g.nf[2] + m2;
  }
}

// ---------------------------------------------------------------------------
// Interpolation
// ---------------------------------------------------------------------------
template <int DIM, int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS)
interp_kernel(InterpArgs a) {
  constexpr int WM = WidthTraits<W>::WM;
  extern __shared__ float2 tile[];
  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<DIM>(g, b, o);
  const int T = g.tile;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;

  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    for (int idx = threadIdx.x; idx < nc * T; idx += blockDim.x) {
      int cc = idx / T;
      int r = idx - cc * T;
      tile[idx] = a.fine[(int64_t)(c0 + cc) * g.G + tile_to_fine<DIM>(g, o, r)];
    }
    __syncthreads();
    for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
      const int pos = p0 + s;
      float w0[WM], w1[WM], w2[WM];
      int l0 = weights_rt<W>(a.s.u[0][pos], g, w0) - o[0];
      int l1 = weights_rt<W>(a.s.u[1][pos], g, w1) - o[1];
      int l2 = 0;
      if (DIM == 3) l2 = weights_rt<W>(a.s.u[2][pos], g, w2) - o[2];
      float ar[CG], ai[CG];
GBN_UNROLL
      for (int cc = 0; cc < CG; ++cc) { ar[cc] = 0.f; ai[cc] = 0.f; }
      if (DIM == 2) {
GBN_UNROLL
        for (int t0 = 0; t0 < WL; ++t0) {
          {
            const float2* row = tile + (l0 + t0) * g.pd[1] + l1;
GBN_UNROLL
            for (int cc = 0; cc < CG; ++cc) {
              float sr = 0.f, si = 0.f;
GBN_UNROLL
              for (int t1 = 0; t1 < WL; ++t1) {
                {
                  float2 v = row[cc * T + t1];
                  sr = fmaf(w1[t1], v.x, sr);
                  si = fmaf(w1[t1], v.y, si);
                }
              }
              ar[cc] = fmaf(w0[t0], sr, ar[cc]);
              ai[cc] = fmaf(w0[t0], si, ai[cc]);
            }
          }
        }
      } else {
GBN_UNROLL
        for (int t0 = 0; t0 < WL; ++t0) {
          {
GBN_UNROLL
            for (int t1 = 0; t1 < WL; ++t1) {
              {
                const float wy = w0[t0] * w1[t1];
                const float2* row = tile + ((l0 + t0) * g.pd[1] + (l1 + t1)) * g.pd[2] + l2;
GBN_UNROLL
                for (int cc = 0; cc < CG; ++cc) {
                  float sr = 0.f, si = 0.f;
GBN_UNROLL
                  for (int t2 = 0; t2 < WL; ++t2) {
                    {
                      float2 v = row[cc * T + t2];
                      sr = fmaf(w2[t2], v.x, sr);
                      si = fmaf(w2[t2], v.y, si);
                    }
                  }
                  ar[cc] = fmaf(wy, sr, ar[cc]);
                  ai[cc] = fmaf(wy, si, ai[cc]);
                }
              }
            }
          }
        }
      }
      const int j = a.s.perm[pos];
      if (a.mode == INTERP_PIPE) {
        // single transform: w_j <- w_j / |scale * v_j|
        float2 cur = a.out[j];
        float mag = a.scale * sqrtf(ar[0] * ar[0] + ai[0] * ai[0]);
        a.out[j] = make_float2(cur.x / mag, cur.y / mag);
      } else {
GBN_UNROLL
        for (int cc = 0; cc < CG; ++cc) {
          if (cc < nc) {
            const int64_t oi = (int64_t)(c0 + cc) * a.s.M + j;
            float2 r = make_float2(a.scale * ar[cc], a.scale * ai[cc]);
            if (a.mode == INTERP_RESID) {
              float2 ob = a.obs[oi];
              r.x -= ob.x;
              r.y -= ob.y;
              if (a.density) {
                float dj = a.density[j];
                r.x *= dj;
                r.y *= dj;
              }
            }
            a.out[oi] = r;
          }
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Spreading
// ---------------------------------------------------------------------------
template <int DIM, int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS)
spread_kernel(SpreadArgs a) {
  constexpr int WM = WidthTraits<W>::WM;
  extern __shared__ float2 tile[];
  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<DIM>(g, b, o);
  const int T = g.tile;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;
  float* tf = reinterpret_cast<float*>(tile);

  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    for (int idx = threadIdx.x; idx < nc * T; idx += blockDim.x) tile[idx] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
      const int pos = p0 + s;
      const int j = a.s.perm[pos];
      float dj = a.scale;
      if (a.density) dj *= a.density[j];
      float2 v[CG];
GBN_UNROLL
      for (int cc = 0; cc < CG; ++cc) {
        if (cc < nc) {
          float2 x = a.in[(int64_t)(c0 + cc) * a.s.M + j];
          v[cc] = make_float2(x.x * dj, x.y * dj);
        } else {
          v[cc] = make_float2(0.f, 0.f);
        }
      }
      float w0[WM], w1[WM], w2[WM];
      int l0 = weights_rt<W>(a.s.u[0][pos], g, w0) - o[0];
      int l1 = weights_rt<W>(a.s.u[1][pos], g, w1) - o[1];
      int l2 = 0;
      if (DIM == 3) l2 = weights_rt<W>(a.s.u[2][pos], g, w2) - o[2];
      if (DIM == 2) {
GBN_UNROLL
        for (int t0 = 0; t0 < WL; ++t0) {
          {
            const int rbase = (l0 + t0) * g.pd[1] + l1;
GBN_UNROLL
            for (int t1 = 0; t1 < WL; ++t1) {
              {
                const float k = w0[t0] * w1[t1];
GBN_UNROLL
                for (int cc = 0; cc < CG; ++cc) {
                  if (cc < nc) {
                    float* p = tf + 2 * (cc * T + rbase + t1);
                    atomicAdd(p, k * v[cc].x);
                    atomicAdd(p + 1, k * v[cc].y);
                  }
                }
              }
            }
          }
        }
      } else {
GBN_UNROLL
        for (int t0 = 0; t0 < WL; ++t0) {
          {
GBN_UNROLL
            for (int t1 = 0; t1 < WL; ++t1) {
              {
                const float wy = w0[t0] * w1[t1];
                const int rbase = ((l0 + t0) * g.pd[1] + (l1 + t1)) * g.pd[2] + l2;
GBN_UNROLL
                for (int t2 = 0; t2 < WL; ++t2) {
                  {
                    const float k = wy * w2[t2];
GBN_UNROLL
                    for (int cc = 0; cc < CG; ++cc) {
                      if (cc < nc) {
                        float* p = tf + 2 * (cc * T + rbase + t2);
                        atomicAdd(p, k * v[cc].x);
                        atomicAdd(p + 1, k * v[cc].y);
                      }
                    }
                  }
                }
              }
            }
          }
        }
      }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nc * T; idx += blockDim.x) {
      float2 v = tile[idx];
      if (v.x != 0.f || v.y != 0.f) {
        int cc = idx / T;
        int r = idx - cc * T;
        float2* dst = a.fine + (int64_t)(c0 + cc) * g.G + tile_to_fine<DIM>(g, o, r);
        atomicAdd(dst, v);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Kernel-derivative interpolation: grad[j, d] += Re(a_j * scale * uscale_d *
// sum_m B[m] d/du_d phi(m - u_j)), a_j = conj(dy_j) (conj_a) or dy_j.
// ---------------------------------------------------------------------------
template <int DIM, int W>
__global__ void __launch_bounds__(GBN_THREADS)
grad_kernel(GradArgs a, int conj_a) {
  constexpr int WM = WidthTraits<W>::WM;
  extern __shared__ float2 tile[];
  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<DIM>(g, b, o);
  const int T = g.tile;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;

  for (int c = 0; c < a.ntr; ++c) {
    for (int idx = threadIdx.x; idx < T; idx += blockDim.x)
      tile[idx] = a.fine[(int64_t)c * g.G + tile_to_fine<DIM>(g, o, idx)];
    __syncthreads();
    for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
      const int pos = p0 + s;
      float w0[WM], w1[WM], w2[WM], d0[WM], d1[WM], d2[WM];
      int l0 = weights_rt_d<W>(a.s.u[0][pos], g, w0, d0) - o[0];
      int l1 = weights_rt_d<W>(a.s.u[1][pos], g, w1, d1) - o[1];
      int l2 = 0;
      if (DIM == 3) l2 = weights_rt_d<W>(a.s.u[2][pos], g, w2, d2) - o[2];
      float gr[3] = {0.f, 0.f, 0.f}, gi[3] = {0.f, 0.f, 0.f};
      if (DIM == 2) {
        for (int t0 = 0; t0 < w; ++t0) {
          const float2* row = tile + (l0 + t0) * g.pd[1] + l1;
          float sr = 0.f, si = 0.f, dr = 0.f, di = 0.f;
          for (int t1 = 0; t1 < w; ++t1) {
            float2 v = row[t1];
            sr = fmaf(w1[t1], v.x, sr);
            si = fmaf(w1[t1], v.y, si);
            dr = fmaf(d1[t1], v.x, dr);
            di = fmaf(d1[t1], v.y, di);
          }
          gr[0] = fmaf(d0[t0], sr, gr[0]);
          gi[0] = fmaf(d0[t0], si, gi[0]);
          gr[1] = fmaf(w0[t0], dr, gr[1]);
          gi[1] = fmaf(w0[t0], di, gi[1]);
        }
      } else {
        for (int t0 = 0; t0 < w; ++t0) {
          for (int t1 = 0; t1 < w; ++t1) {
            const float2* row = tile + ((l0 + t0) * g.pd[1] + (l1 + t1)) * g.pd[2] + l2;
            float sr = 0.f, si = 0.f, dr = 0.f, di = 0.f;
            for (int t2 = 0; t2 < w; ++t2) {
              float2 v = row[t2];
              sr = fmaf(w2[t2], v.x, sr);
              si = fmaf(w2[t2], v.y, si);
              dr = fmaf(d2[t2], v.x, dr);
              di = fmaf(d2[t2], v.y, di);
            }
            const float a0 = d0[t0] * w1[t1], a1 = w0[t0] * d1[t1], a2 = w0[t0] * w1[t1];
            gr[0] = fmaf(a0, sr, gr[0]);
            gi[0] = fmaf(a0, si, gi[0]);
            gr[1] = fmaf(a1, sr, gr[1]);
            gi[1] = fmaf(a1, si, gi[1]);
            gr[2] = fmaf(a2, dr, gr[2]);
            gi[2] = fmaf(a2, di, gi[2]);
          }
        }
      }
      const int j = a.s.perm[pos];
      float2 av = a.dy[(int64_t)c * a.s.M + j];
      if (conj_a) av.y = -av.y;
GBN_UNROLL
      for (int d = 0; d < DIM; ++d) {
        // Re(av * (gr + i gi))
        float re = av.x * gr[d] - av.y * gi[d];
        a.grad[(int64_t)j * DIM + d] += a.scale * g.uscale[d] * re;
      }
    }
    __syncthreads();
  }
}

template <int DIM, int W, int CG>
cudaError_t launch_interp_t(const InterpArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  size_t smem = (size_t)CG * a.g.tile * sizeof(float2);
  auto k = interp_kernel<DIM, W, CG>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.s.nsub, GBN_THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int DIM, int W, int CG>
cudaError_t launch_spread_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  size_t smem = (size_t)CG * a.g.tile * sizeof(float2);
  auto k = spread_kernel<DIM, W, CG>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.s.nsub, GBN_THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int DIM, int W>
cudaError_t launch_grad_t(const GradArgs& a, int conj_a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  size_t smem = (size_t)a.g.tile * sizeof(float2);
  auto k = grad_kernel<DIM, W>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.s.nsub, GBN_THREADS, smem, st>>>(a, conj_a);
  return cudaGetLastError();
}

template <int DIM, int CG>
cudaError_t dispatch_interp_w(const InterpArgs& a, cudaStream_t st) {
  // w = 7 is the width of mri-nufft's default eps = 1e-6 at upsampfac 2;
  // every other width runs the runtime-width kernel.
  if (a.g.w == 7) return launch_interp_t<DIM, 7, CG>(a, st);
  return launch_interp_t<DIM, 0, CG>(a, st);
}

template <int DIM, int CG>
cudaError_t dispatch_spread_w(const SpreadArgs& a, cudaStream_t st) {
  // w = 7 is the width of mri-nufft's default eps = 1e-6 at upsampfac 2;
  // every other width runs the runtime-width kernel.
  if (a.g.w == 7) return launch_spread_t<DIM, 7, CG>(a, st);
  return launch_spread_t<DIM, 0, CG>(a, st);
}

template <int DIM>
cudaError_t dispatch_interp(const InterpArgs& a, cudaStream_t st) {
  int cg = a.mode == INTERP_PIPE ? 1 : coils_per_pass(a.g, a.ntr);
  if (cg >= 2) return dispatch_interp_w<DIM, 4>(a, st);
  return dispatch_interp_w<DIM, 1>(a, st);
}

template <int DIM>
cudaError_t dispatch_spread(const SpreadArgs& a, cudaStream_t st) {
  int cg = coils_per_pass(a.g, a.ntr);
  if (cg >= 2) return dispatch_spread_w<DIM, 4>(a, st);
  return dispatch_spread_w<DIM, 1>(a, st);
}

template <int DIM>
cudaError_t dispatch_grad(const GradArgs& a, cudaStream_t st) {
  // runtime-width kernel: the derivative path is not the throughput path
  return launch_grad_t<DIM, 0>(a, a.conj_a, st);
}

}  // namespace gbn
