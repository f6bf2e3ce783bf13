// Pipe density iterations that allocate nothing (gbn_pipe_static).
//
// Some callers cannot allocate device memory when they need this step: a
// process whose device memory is already handed to a framework's pool (JAX
// and TensorFlow reserve most of it at start-up, so cudaMalloc fails), or a
// real-time scanner reconstruction service that forbids allocation after
// start-up to keep its latency predictable.  For them this entry point runs
// the same iteration as gbn_pipe on a spread-only plan, but its only scratch,
// the image-size grid, is a fixed file-scope device array.  The bin sort of a
// plan needs scratch too, so the samples are used in the caller's order:
// spreading adds to the grid with float2 global atomics and interpolation
// reads it through the cache hierarchy.
//
// The array holds GBN_STATIC_GRID_CELLS complex64 cells (16 MiB) on every GPU
// that loads the library, for the life of the process.  Host code cannot use
// the array's name as a device address, so every call looks the address up
// with cudaGetSymbolAddress on the current device (a lookup that allocates
// nothing and stays valid across a device reset, which a cached pointer would
// not).  The first call on a device also loads the module there, so it should
// come before any stream capture.  Every call shares the array, and each
// iteration clears it before spreading; calls whose work overlaps on the GPU
// (other streams, other threads) race on it and must be serialised by the
// caller.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "gbn_internal.cuh"
#include "gbnufft.h"

namespace {

static __device__ __align__(256) float2 g_static_grid[GBN_STATIC_GRID_CELLS];

using gbn::fold_coord;
using gbn::wrap_idx;

struct StaticGeom {
  int dim;
  int nf[3];
  float uscale[3];
  int w;
  float beta, halfw, inv_halfw;
};

__device__ __forceinline__ float es(float x, const StaticGeom& g) {
  float z = x * g.inv_halfw;
  float t = 1.0f - z * z;
  return t > 0.0f ? __expf(g.beta * (sqrtf(t) - 1.0f)) : 0.0f;
}

// footprint of one sample along one axis: first cell and the w weights
__device__ __forceinline__ int footprint(float k, const StaticGeom& g, int d, float* wt) {
  float u = fold_coord(k, g.uscale[d], g.nf[d]);
  int i0 = (int)ceilf(u - g.halfw);
  float x0 = (float)i0 - u;
  for (int t = 0; t < g.w; ++t) wt[t] = es(x0 + (float)t, g);
  return i0;
}

template <int DIM>
__global__ void static_spread_kernel(StaticGeom g, int64_t M, const float* __restrict__ k0,
                                     const float* __restrict__ k1, const float* __restrict__ k2,
                                     const float2* __restrict__ c, float2* grid) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  float w0[16], w1[16], w2[16];
  int a0 = footprint(k0[j], g, 0, w0);
  int a1 = footprint(k1[j], g, 1, w1);
  int a2 = DIM == 3 ? footprint(k2[j], g, 2, w2) : 0;
  const float2 v = c[j];
  for (int t0 = 0; t0 < g.w; ++t0) {
    const int m0 = wrap_idx(a0 + t0, g.nf[0]);
    for (int t1 = 0; t1 < g.w; ++t1) {
      const float k = w0[t0] * w1[t1];
      const int64_t r = (int64_t)m0 * g.nf[1] + wrap_idx(a1 + t1, g.nf[1]);
      if (DIM == 2) {
        atomicAdd(grid + r, make_float2(k * v.x, k * v.y));
      } else {
        for (int t2 = 0; t2 < g.w; ++t2) {
          const float kk = k * w2[t2];
          atomicAdd(grid + r * g.nf[2] + wrap_idx(a2 + t2, g.nf[2]),
                    make_float2(kk * v.x, kk * v.y));
        }
      }
    }
  }
}

// w_j <- w_j / |scale2 * interp(grid)_j|
template <int DIM>
__global__ void static_interp_divide_kernel(StaticGeom g, int64_t M, const float* __restrict__ k0,
                                            const float* __restrict__ k1,
                                            const float* __restrict__ k2,
                                            const float2* __restrict__ grid, float2* w,
                                            float scale2) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  float w0[16], w1[16], w2[16];
  int a0 = footprint(k0[j], g, 0, w0);
  int a1 = footprint(k1[j], g, 1, w1);
  int a2 = DIM == 3 ? footprint(k2[j], g, 2, w2) : 0;
  float sr = 0.f, si = 0.f;
  for (int t0 = 0; t0 < g.w; ++t0) {
    const int m0 = wrap_idx(a0 + t0, g.nf[0]);
    for (int t1 = 0; t1 < g.w; ++t1) {
      const float k = w0[t0] * w1[t1];
      const int64_t r = (int64_t)m0 * g.nf[1] + wrap_idx(a1 + t1, g.nf[1]);
      if (DIM == 2) {
        const float2 v = grid[r];
        sr = fmaf(k, v.x, sr);
        si = fmaf(k, v.y, si);
      } else {
        float rr = 0.f, ri = 0.f;
        for (int t2 = 0; t2 < g.w; ++t2) {
          const float2 v = grid[r * g.nf[2] + wrap_idx(a2 + t2, g.nf[2])];
          rr = fmaf(w2[t2], v.x, rr);
          ri = fmaf(w2[t2], v.y, ri);
        }
        sr = fmaf(k, rr, sr);
        si = fmaf(k, ri, si);
      }
    }
  }
  const float mag = scale2 * sqrtf(sr * sr + si * si);
  const float2 cur = w[j];
  w[j] = make_float2(cur.x / mag, cur.y / mag);
}

int fail_static(int code, const std::string& msg) {
  gbn::set_last_error(msg.c_str());
  return code;
}

}  // namespace

extern "C" int gbn_pipe_static(int dim, const int64_t* n_modes, double osf, double eps, int64_t M,
                               const float* k0, const float* k1, const float* k2, void* w,
                               int iters, float scale2, gbn_stream stream) {
  gbn::set_last_error("");
  if (dim != 2 && dim != 3) return fail_static(GBN_ERR_ARG, "dim must be 2 or 3");
  if (!n_modes) return fail_static(GBN_ERR_ARG, "null n_modes");
  if (!(eps > 0.0 && eps < 1.0)) return fail_static(GBN_ERR_ARG, "eps must be in (0, 1)");
  if (M < 0 || M > ((int64_t)1 << 31) - 1) return fail_static(GBN_ERR_ARG, "M out of range");
  if (iters < 0) return fail_static(GBN_ERR_ARG, "iters must be >= 0");
  if (M > 0 && (!k0 || !k1 || (dim == 3 && !k2) || !w))
    return fail_static(GBN_ERR_ARG, "null coordinates or weights");
  StaticGeom g{};
  g.dim = dim;
  int64_t cells = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < dim) {
      if (n_modes[d] < 1) return fail_static(GBN_ERR_ARG, "image size must be >= 1");
      // cells <= GBN_STATIC_GRID_CELLS before this factor, so the test
      // below cannot overflow and the product stays within the array
      if (n_modes[d] > GBN_STATIC_GRID_CELLS / cells) {
        return fail_static(GBN_ERR_ARG,
                           "grid exceeds the static grid of " +
                               std::to_string((long long)GBN_STATIC_GRID_CELLS) +
                               " cells (16 MiB); use a plan (gbn_plan_create + gbn_pipe) instead");
      }
      cells *= n_modes[d];
      g.nf[d] = (int)n_modes[d];
      g.uscale[d] = (float)((double)n_modes[d] / (2.0 * M_PI));
    } else {
      g.nf[d] = 1;
      g.uscale[d] = 0.f;
    }
  }
  // kernel width and shape: the rule gbn_plan_create uses (osf <= 1 takes
  // the osf = 2 kernel there too)
  int wd;
  double beta;
  gbn::kernel_params(eps, osf, &wd, &beta);
  g.w = wd;
  g.beta = (float)beta;
  g.halfw = 0.5f * wd;
  g.inv_halfw = 2.0f / wd;

  float2* grid = nullptr;
  {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_grid);
    if (e != cudaSuccess)
      return fail_static(GBN_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    grid = static_cast<float2*>(p);
  }
  if (M == 0 || iters == 0) return GBN_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)((M + 255) / 256);
  float2* wv = static_cast<float2*>(w);
  const float* kk2 = dim == 3 ? k2 : k1;
  cudaError_t e = cudaSuccess;
  for (int it = 0; it < iters; ++it) {
    e = cudaMemsetAsync(grid, 0, sizeof(float2) * (size_t)cells, st);
    if (e != cudaSuccess) return fail_static(GBN_ERR_CUDA, std::string("clear grid: ") + cudaGetErrorString(e));
    if (dim == 2) {
      static_spread_kernel<2><<<blocks, 256, 0, st>>>(g, M, k0, k1, kk2, wv, grid);
      static_interp_divide_kernel<2><<<blocks, 256, 0, st>>>(g, M, k0, k1, kk2, grid, wv, scale2);
    } else {
      static_spread_kernel<3><<<blocks, 256, 0, st>>>(g, M, k0, k1, kk2, wv, grid);
      static_interp_divide_kernel<3><<<blocks, 256, 0, st>>>(g, M, k0, k1, kk2, grid, wv, scale2);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail_static(GBN_ERR_CUDA, std::string("pipe kernels: ") + cudaGetErrorString(e));
  }
  return GBN_OK;
}
