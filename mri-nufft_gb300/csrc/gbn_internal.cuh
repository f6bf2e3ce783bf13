// Internal definitions of the GB300 NUFFT library (not part of the C ABI).
//
// Geometry conventions (shared by every kernel):
//   * image axis d pairs with sample coordinate column d; axis dim-1 is the
//     fastest in memory (C order), matching mri-nufft's image arrays
//     (operators/base.py:738-746) and its NDFT (nudft_numpy.py:12-55);
//   * a sample coordinate k in radians maps to fine-grid units
//     u = k * nf / (2 pi), folded into [0, nf);
//   * image mode n (n in [-floor(N/2), N - floor(N/2))) lives at fine index
//     n mod nf, and at image array index n + floor(N/2);
//   * the exponential-of-semicircle kernel of width w (cells) is
//     phi(x) = exp(beta * (sqrt(1 - (2x/w)^2) - 1)) for |x| < w/2, else 0.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#define GBN_MAXDIM 3
#define GBN_THREADS 256

namespace gbn {

struct Geom {
  int dim;
  int n[3];      // image modes per axis (unused axes = 1)
  int nf[3];     // fine grid per axis (unused axes = 1)
  int bs[3];     // bin size per axis (unused axes = 1)
  int nb[3];     // number of bins per axis
  int pd[3];     // padded tile extent per axis = bs + w (unused axes = 1)
  int w;         // kernel width in cells
  float beta;    // ES shape parameter
  float halfw;   // w / 2
  float inv_halfw;  // 2 / w
  float uscale[3];  // nf / (2 pi) per axis
  int64_t G;     // fine cells per transform
  int64_t Nimg;  // image pixels per transform
  int tile;      // padded tile cells = prod(pd)
  int interp_cg; // coils per interp tile pass (0: automatic)
  int method_interp;  // 0: automatic (3D tiles, 2D warp-cooperative), 1: direct from the
                      // fine grid, 3: double-buffered tiles, 4: warp-cooperative,
                      // 5: 3D tile warp-cooperative, 6: tiles
  int method_spread;  // 0: automatic, 1: global atomics, 2: warp-cooperative atomics,
                      // 3: 3D column streaming, 4: 3D bin-tile rows,
                      // 5: 3D quadrant streaming (8 x 8 bins),
                      // 6: 3D quadrant tiles on the tensor cores (8 x 8 bins, w = 7)
  int interp_threads; // CTA size of the tile interp kernel (0: 128)
  int spread_cg;      // coils per pass of the streaming spreader (0: automatic)
  int quad_minb;      // resident CTAs per SM of the 4-coil quadrant spreader (0: 3)
  int quad_packed;    // 0: scalar accumulators in the quadrant spreader (default 1: (re, im) pairs)
};

// Work table of one sorted trajectory.
struct Sorted {
  int64_t M;
  const int* perm;        // sorted position -> original sample index
  const float* u[3];      // sorted fine-grid coordinates per axis
  const int* sub_bin;     // subproblem -> bin
  const int* sub_start;   // subproblem -> first sorted position
  const int* sub_count;   // subproblem -> number of samples
  int nsub;
  int maxsub;             // largest subproblem
};

// Interp epilogues.
enum InterpMode : int {
  INTERP_STORE = 0,   // out[c][j] = scale * v
  INTERP_RESID = 1,   // out[c][j] = (scale * v - obs[c][j]) * density[j]
  INTERP_PIPE = 2,    // w[j] = w[j] / |scale * v|   (one transform)
};

struct InterpArgs {
  Geom g;
  Sorted s;
  const float2* fine;   // ntr fine grids, G cells each
  float2* out;          // ntr x M (original sample order)
  const float2* obs;    // INTERP_RESID: ntr x M
  const float* density; // optional, M
  int ntr;              // transforms in this launch
  float scale;
  int mode;
};

struct SpreadArgs {
  Geom g;
  Sorted s;
  const float2* in;     // ntr x M strengths (original sample order)
  const float* density; // optional, M
  float2* fine;         // ntr fine grids (accumulated into)
  int ntr;
  float scale;
};

// Kernel-derivative interpolation: gradient of k-space values with respect
// to the sample coordinates.
struct GradArgs {
  Geom g;
  Sorted s;
  const float2* fine;   // ntr fine grids
  const float2* dy;     // ntr x M cotangents
  float* grad;          // M x dim, accumulated (+=)
  int ntr;
  float scale;          // the nf/(2 pi) chain factor per axis comes from g.uscale
  int conj_a;           // 1: grad += Re(conj(dy) * dv); 0: grad += Re(dy * dv)
};

__host__ __device__ inline int imin(int a, int b) { return a < b ? a : b; }

__device__ __forceinline__ int wrap_idx(int i, int n) {
  // n >= 1; tiles never reach beyond one period for nf >= 2w, but a modulo
  // keeps tiny grids correct too.
  int r = i % n;
  return r < 0 ? r + n : r;
}

__device__ __forceinline__ float es_eval(float x, float beta, float inv_halfw) {
  float z = x * inv_halfw;
  float t = 1.0f - z * z;
  return t > 0.0f ? __expf(beta * (sqrtf(t) - 1.0f)) : 0.0f;
}

// derivative d phi / dx
__device__ __forceinline__ float es_deriv(float x, float beta, float inv_halfw) {
  float z = x * inv_halfw;
  float t = 1.0f - z * z;
  if (t <= 1e-12f) return 0.0f;
  float st = sqrtf(t);
  float ph = __expf(beta * (st - 1.0f));
  return -ph * beta * z * inv_halfw / st;
}

// Fold a coordinate in radians to fine-grid units in [0, nf].  Non-finite
// or huge inputs (whose fold is not exact) map to 0, so that every stored
// coordinate lies in the bin it was sorted into and every footprint stays
// inside its shared-memory tile.
__device__ __forceinline__ float fold_coord(float k, float uscale, int nf) {
  float u = k * uscale;
  float fnf = (float)nf;
  u = u - fnf * floorf(u / fnf);
  if (!(u >= 0.0f && u <= fnf)) u = 0.0f;
  return u;
}

__device__ __forceinline__ int cell_of(float u, int nf) {
  int f = (int)floorf(u);
  f = f < 0 ? 0 : f;
  return f > nf - 1 ? nf - 1 : f;
}

// Kernel width and shape from the published exponential-of-semicircle rules
// (finufft paper, Barnett, Magland & af Klinteberg, SISC 2019, and the finufft
// docs); every entry point that builds a kernel takes them from here:
//   sigma 2:     w = ceil(-log10(eps / 10)), beta = c(w) * w with
//                c = 2.20, 2.26, 2.38 for w = 2, 3, 4 and 2.30 otherwise;
//   other sigma: w = ceil(-ln(eps) / (pi sqrt(1 - 1/sigma))),
//                beta = 0.97 * pi * w * (1 - 1 / (2 sigma));
//   w is clamped to [2, 16].  A sigma <= 1 (spread-only grids whose caller
//   gave no oversampling) takes the sigma = 2 rule.
inline void kernel_params(double eps, double sigma, int* w_out, double* beta_out) {
  const double pi = 3.14159265358979323846;
  if (!(sigma > 1.0)) sigma = 2.0;
  int w;
  if (sigma == 2.0) w = (int)__builtin_ceil(-__builtin_log10(eps / 10.0));
  else w = (int)__builtin_ceil(-__builtin_log(eps) / (pi * __builtin_sqrt(1.0 - 1.0 / sigma)));
  if (w < 2) w = 2;
  if (w > 16) w = 16;
  double beta;
  if (sigma == 2.0) {
    const double c = w == 2 ? 2.20 : w == 3 ? 2.26 : w == 4 ? 2.38 : 2.30;
    beta = c * w;
  } else {
    beta = 0.97 * pi * w * (1.0 - 1.0 / (2.0 * sigma));
  }
  *w_out = w;
  *beta_out = beta;
}

// Sets the message returned by gbn_last_error() on the calling thread.
void set_last_error(const char* msg);

// Launchers implemented in the per-dimension translation units.
cudaError_t launch_interp2d(const InterpArgs& a, cudaStream_t st);
cudaError_t launch_interp3d(const InterpArgs& a, cudaStream_t st);
cudaError_t launch_spread2d(const SpreadArgs& a, cudaStream_t st);
cudaError_t launch_spread3d(const SpreadArgs& a, cudaStream_t st);
// column-streaming spreaders; a.s is the column-chunk table
cudaError_t launch_spread_stream3d(const SpreadArgs& a, cudaStream_t st);
cudaError_t launch_spread_stream2d(const SpreadArgs& a, cudaStream_t st);
cudaError_t launch_grad2d(const GradArgs& a, cudaStream_t st);
cudaError_t launch_grad3d(const GradArgs& a, cudaStream_t st);

// Shared-memory budget for the tiles of one CTA.
constexpr int kTileSmemBudget = 112 * 1024;

// coils per interp tile pass: 1 (or the plan's override), halved until the
// tiles fit the shared-memory budget and do not exceed the transform count.
inline int coils_per_pass(const Geom& g, int ntr) {
  size_t t = (size_t)g.tile * sizeof(float2);
  int cg = g.interp_cg > 0 ? g.interp_cg : 1;
  while (cg > 1 && (cg > ntr || (size_t)cg * t > (size_t)kTileSmemBudget)) cg >>= 1;
  return cg;
}

// 3D tiles up to 16 x 16 x 16 cells use the row spreading kernel (two coils
// per pass); 2D, and wider kernels, use the sample-driven global-atomic one.
inline bool rows_fit(const Geom& g) {
  return g.dim == 3 && g.w <= 8 && g.pd[0] <= 16 && g.pd[1] <= 16 && g.pd[2] <= 16;
}

// Widths up to 7 with column cross-sections of at most 16 x 16 rows (3D) or
// 32 rows (2D), and a last-axis extent that fits the kernels' 14-bit sample
// header, use the column-streaming spreaders (an 8-cell register window
// along the last axis).
inline bool stream_fit(const Geom& g) {
  if (g.w > 7 || !(g.method_spread == 0 || g.method_spread == 3 || g.method_spread == 5 ||
                   g.method_spread == 6))
    return false;
  if (g.dim == 2) return g.pd[0] <= 32 && g.nf[1] <= 16000;
  return g.dim == 3 && g.bs[0] <= 15 && g.bs[1] <= 15 && g.pd[0] <= 16 && g.pd[1] <= 16 &&
         g.nf[2] <= 16000;
}

// Samples per chunk of the column-streaming spreaders (3D, 2D).
constexpr int kStreamChunk = 512;
constexpr int kStreamChunk2 = 256;

}  // namespace gbn
