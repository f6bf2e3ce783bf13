// C ABI of the GB300 NUFFT library: plans, point setting, operator calls.
//
// The pipelines (per pass of up to `ntrans` transforms):
//   op  : pad pass (SENSE product, 1/phihat, zero pad) -> cuFFT -> interp
//   adj : zero fine grid -> spread (density applied) -> cuFFT -> crop pass
//         (1/phihat, scale, conj(smaps) coil sum)
//   dc  : pad -> cuFFT -> interp with residual epilogue (scale*v - y)*d
//         -> zero -> spread -> cuFFT -> crop (coil sum)
//   pipe: zero -> spread -> interp with divide epilogue, on the N grid
#include <cufft.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "gbn_batch.cuh"
#include "gbn_fft256.cuh"
#include "gbn_fft512.cuh"
#include "gbn_internal.cuh"
#include "gbn_passes.cuh"
#include "gbn_sort.cuh"
#include "gbnufft.h"

using namespace gbn;

namespace {

thread_local std::string g_err;

struct Fail {
  int code;
};

[[noreturn]] void fail(int code, const std::string& msg) {
  g_err = msg;
  throw Fail{code};
}

void ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    fail(GBN_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
  }
  fail(GBN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void ckfft(cufftResult r, const char* what) {
  if (r == CUFFT_SUCCESS) return;
  if (r == CUFFT_ALLOC_FAILED) fail(GBN_ERR_NOMEM, std::string(what) + ": cuFFT allocation failed");
  fail(GBN_ERR_CUFFT, std::string(what) + ": cuFFT error " + std::to_string((int)r));
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) ck(cudaSetDevice(dev), "cudaSetDevice");
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

template <typename T>
T* dev_alloc(size_t count, int64_t& tally, const char* what) {
  if (count == 0) count = 1;
  void* p = nullptr;
  ck(cudaMalloc(&p, count * sizeof(T)), what);
  tally += (int64_t)(count * sizeof(T));
  return static_cast<T*>(p);
}

void dev_free(void* p) {
  if (p) cudaFree(p);
}

// smallest even integer >= n with no prime factor other than 2, 3, 5
int64_t next_smooth_even(int64_t n) {
  if (n <= 2) return 2;
  if (n % 2) ++n;
  for (;; n += 2) {
    int64_t r = n;
    for (int p : {2, 3, 5})
      while (r % p == 0) r /= p;
    if (r == 1) return n;
  }
}

// Gauss-Legendre nodes/weights on [-1, 1] (Newton on P_q, Golub-free)
void gauss_legendre(int q, std::vector<double>& x, std::vector<double>& wts) {
  x.assign(q, 0.0);
  wts.assign(q, 0.0);
  for (int i = 0; i < (q + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (q + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int k = 1; k <= q; ++k) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * k - 1.0) * z * p2 - (k - 1.0) * p3) / k;
      }
      pp = q * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-15) break;
    }
    x[i] = -z;
    x[q - 1 - i] = z;
    wts[i] = wts[q - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

// 1 / phihat(n) for the N modes of one axis (array index i <-> mode i - N/2),
// phihat(k) = int_{-w/2}^{w/2} phi(x) cos(2 pi k x / nf) dx in FP64.
std::vector<float> deconv_factors(int N, int64_t nf, int w, double beta) {
  std::vector<double> x, wt;
  const int q = 2 * w + 48;
  gauss_legendre(q, x, wt);
  const double h = 0.5 * w;
  std::vector<double> xs(q), fs(q);
  for (int i = 0; i < q; ++i) {
    xs[i] = h * x[i];
    double z = xs[i] / h;
    double t = 1.0 - z * z;
    fs[i] = t > 0 ? std::exp(beta * (std::sqrt(t) - 1.0)) * h * wt[i] : 0.0;
  }
  std::vector<float> out(N);
  for (int i = 0; i < N; ++i) {
    double k = (double)(i - N / 2);
    double s = 0.0;
    for (int j = 0; j < q; ++j) s += fs[j] * std::cos(2.0 * M_PI * k * xs[j] / (double)nf);
    out[i] = (float)(1.0 / s);
  }
  return out;
}

}  // namespace

void gbn::set_last_error(const char* msg) { g_err = msg; }

struct gbn_plan_s {
  Geom g{};
  int ntrans = 1;
  int spread_only = 0;
  int device = 0;
  int nsm = 152;
  double eps = 1e-6, sigma = 2.0, beta = 0.0;
  int64_t bytes = 0;

  float* dec[3] = {nullptr, nullptr, nullptr};
  float2* fine = nullptr;
  float2* kbuf = nullptr;  // ntrans x M residual scratch for dc
  int64_t kbuf_cap = 0;

  // sort state
  int64_t M = -1, Mcap = 0, subcap = 0;
  int64_t point_bytes = 0;  // device bytes of the per-point arrays
  int maxsub = 256;
  int maxsub_cap = 512;
  int nsub = 0;
  SortBuffers sb{};
  int nbins = 0;           // bins of the sort
  int64_t bin_bytes = 0;   // device bytes of the per-bin arrays

  // 3D column streaming: the sort is keyed on (x bin, y bin, z cell); the
  // interp / grad table groups bs2 consecutive z cells (the bins of g), the
  // spread table cuts each column into chunks of <= kStreamChunk samples
  int stream_spread = 0;
  int ngrp = 0;            // interp groups (bins of g)
  int ncol = 0;            // columns
  int* grp = nullptr;      // group-table scratch, 4 x (ngrp + ncol)
  int* ssub = nullptr;     // spread chunk table, 3 x sscap
  int64_t sscap = 0;
  int nsub_s = 0;
  int maxsub_s = 0;

  std::map<int, cufftHandle> ffts;

  // Pruned 3D transforms.  The image occupies the planes |n0| < N0/2 of
  // axis 0 (indices [0, lo) and [nf0 - hi, nf0)), so a transform whose input
  // is confined there (after padding) runs 2D (axes 1, 2) FFTs over those
  // planes only, then 1D FFTs along axis 0; a transform whose output is only
  // read there (before cropping) runs the same two steps in reverse order.
  // The planes of consecutive transforms' hi and lo ranges are contiguous,
  // so T transforms take T + 1 batched 2D calls.
  bool prune = false;
  cufftHandle pl_lo = 0, pl_span = 0, pl_hi = 0, pl_x = 0;

  // 256^3 fine grids: the fused pruned line transforms of gbn_fft256.cu
  // replace the pad pass, cuFFT and the crop pass of op / adj / dc
  bool fft256 = false;
  float2* tw256 = nullptr;  // W256^k table
  // 512^2 fine grids (2D): the same with the 512-point line transforms of
  // gbn_fft512.cu
  bool fft512 = false;
  float2* tw512 = nullptr;  // W512^(b k1) table

  // per-stage CUDA-event timing (gbn_profile) and kernel launch count
  bool prof = false;
  std::vector<cudaEvent_t> evpool;
  size_t evnext = 0;
  std::vector<std::pair<size_t, size_t>> spans[GBN_STAGES];
  int64_t launches = 0;

  size_t record(cudaStream_t st) {
    if (evnext == evpool.size()) {
      cudaEvent_t e;
      ck(cudaEventCreate(&e), "cudaEventCreate");
      evpool.push_back(e);
    }
    ck(cudaEventRecord(evpool[evnext], st), "cudaEventRecord");
    return evnext++;
  }

  ~gbn_plan_s() {
    for (auto e : evpool) cudaEventDestroy(e);
    for (auto& kv : ffts) cufftDestroy(kv.second);
    for (cufftHandle h : {pl_lo, pl_span, pl_hi, pl_x})
      if (h) cufftDestroy(h);
    for (int d = 0; d < 3; ++d) dev_free(dec[d]);
    dev_free(fine);
    dev_free(kbuf);
    dev_free(tw256);
    dev_free(tw512);
    free_points();
    free_bins();
    dev_free(sb.d_total);
  }

  void free_bins() {
    dev_free(sb.bin_count);
    dev_free(sb.bin_start);
    dev_free(sb.nsub_bin);
    dev_free(sb.sub_off);
    dev_free(sb.scan_scratch);
    dev_free(grp);
    sb.bin_count = sb.bin_start = sb.nsub_bin = sb.sub_off = sb.scan_scratch = grp = nullptr;
    bytes -= bin_bytes;
    bin_bytes = 0;
  }

  // (Re)allocates the per-bin arrays for the current geometry.
  void setup_bins() {
    free_bins();
    stream_spread = stream_fit(g) ? 1 : 0;
    const int last = g.dim - 1;
    ngrp = g.nb[0] * g.nb[1] * g.nb[2];
    ncol = ngrp / g.nb[last];
    nbins = stream_spread ? ncol * g.nf[last] : ngrp;
    const int64_t b0 = bytes;
    sb.bin_count = dev_alloc<int>(nbins, bytes, "bins");
    sb.bin_start = dev_alloc<int>(nbins, bytes, "bins");
    sb.nsub_bin = dev_alloc<int>(nbins, bytes, "bins");
    sb.sub_off = dev_alloc<int>(nbins, bytes, "bins");
    sb.scan_scratch = dev_alloc<int>(scan_scratch_ints(nbins), bytes, "scan");
    if (stream_spread) grp = dev_alloc<int>(4 * ((size_t)ngrp + ncol), bytes, "bin groups");
    bin_bytes = bytes - b0;
  }

  void free_points() {
    dev_free(sb.bin_of);
    dev_free(sb.rank_of);
    dev_free(sb.perm);
    for (int d = 0; d < 3; ++d) dev_free(sb.u[d]);
    dev_free(sb.sub_bin);
    dev_free(sb.sub_start);
    dev_free(sb.sub_count);
    dev_free(ssub);
    ssub = nullptr;
    sscap = 0;
    sb.bin_of = sb.rank_of = sb.perm = sb.sub_bin = sb.sub_start = sb.sub_count = nullptr;
    sb.u[0] = sb.u[1] = sb.u[2] = nullptr;
  }

  Sorted sorted() const {
    Sorted s{};
    s.M = M;
    s.perm = sb.perm;
    for (int d = 0; d < 3; ++d) s.u[d] = sb.u[d];
    s.sub_bin = sb.sub_bin;
    s.sub_start = sb.sub_start;
    s.sub_count = sb.sub_count;
    s.nsub = nsub;
    s.maxsub = maxsub;
    return s;
  }

  // the table the spreader walks: column chunks when streaming
  Sorted sorted_spread() const {
    Sorted s = sorted();
    if (stream_spread) {
      s.sub_bin = ssub;
      s.sub_start = ssub + sscap;
      s.sub_count = ssub + 2 * sscap;
      s.nsub = nsub_s;
      s.maxsub = maxsub_s;
    }
    return s;
  }

  cufftHandle fft(int batch) {
    auto it = ffts.find(batch);
    if (it != ffts.end()) return it->second;
    cufftHandle h;
    int n[3];
    for (int d = 0; d < g.dim; ++d) n[d] = g.nf[d];
    ckfft(cufftPlanMany(&h, g.dim, n, nullptr, 1, (int)g.G, nullptr, 1, (int)g.G, CUFFT_C2C,
                        batch),
          "cufftPlanMany");
    size_t ws = 0;
    cufftGetSize(h, &ws);
    bytes += (int64_t)ws;
    ffts[batch] = h;
    return h;
  }

  // prune_mode: 0 full transform, 1 input confined to the image planes,
  // 2 output read on the image planes only
  void exec_fft(int batch, float2* data, int isign, cudaStream_t st, int prune_mode = 0);

  cufftHandle make_plan(int rank, int* n, int* embed, int stride, int dist, int batch) {
    cufftHandle h;
    ckfft(cufftPlanMany(&h, rank, n, embed, stride, dist, embed, stride, dist, CUFFT_C2C, batch),
          "cufftPlanMany");
    size_t ws = 0;
    cufftGetSize(h, &ws);
    bytes += (int64_t)ws;
    return h;
  }

  void make_pruned_plans() {
    const int lo = g.n[0] - g.n[0] / 2, hi = g.n[0] / 2;
    const int P = g.nf[1] * g.nf[2];
    int n2[2] = {g.nf[1], g.nf[2]};
    pl_lo = make_plan(2, n2, nullptr, 1, P, lo);
    if (hi > 0) {
      pl_span = make_plan(2, n2, nullptr, 1, P, lo + hi);
      pl_hi = make_plan(2, n2, nullptr, 1, P, hi);
    }
    int n1[1] = {g.nf[0]};
    int e1[1] = {g.nf[0]};
    pl_x = make_plan(1, n1, e1, P, 1, P);
  }
};

// Records CUDA events around one stage launch when profiling is enabled.
struct Span {
  gbn_plan_s* p;
  int stage;
  cudaStream_t st;
  size_t a = (size_t)-1;
  Span(gbn_plan_s* p_, int stage_, cudaStream_t st_) : p(p_), stage(stage_), st(st_) {
    if (p->prof) a = p->record(st);
  }
  ~Span() {
    if (a != (size_t)-1) {
      size_t b = p->record(st);
      p->spans[stage].push_back({a, b});
    }
  }
};

void gbn_plan_s::exec_fft(int batch, float2* data, int isign, cudaStream_t st, int prune_mode) {
    Span span(this, GBN_STAGE_FFT, st);
    if (prune && prune_mode != 0) {
      if (!pl_x) make_pruned_plans();
      const int dir = isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE;
      auto run = [&](cufftHandle h, float2* d) {
        ckfft(cufftSetStream(h, st), "cufftSetStream");
        ckfft(cufftExecC2C(h, reinterpret_cast<cufftComplex*>(d), reinterpret_cast<cufftComplex*>(d),
                           dir),
              "cufftExecC2C");
      };
      const int64_t P = (int64_t)g.nf[1] * g.nf[2];
      const int hi = g.n[0] / 2;
      auto planes = [&]() {
        if (hi == 0) {
          for (int t = 0; t < batch; ++t) run(pl_lo, data + t * g.G);
          return;
        }
        run(pl_lo, data);
        for (int t = 0; t + 1 < batch; ++t) run(pl_span, data + t * g.G + (g.nf[0] - hi) * P);
        run(pl_hi, data + (batch - 1) * g.G + (g.nf[0] - hi) * P);
      };
      auto columns = [&]() {
        for (int t = 0; t < batch; ++t) run(pl_x, data + t * g.G);
      };
      if (prune_mode == 1) {
        planes();
        columns();
      } else {
        columns();
        planes();
      }
      return;
    }
    cufftHandle h = fft(batch);
    ckfft(cufftSetStream(h, st), "cufftSetStream");
    ckfft(cufftExecC2C(h, reinterpret_cast<cufftComplex*>(data),
                       reinterpret_cast<cufftComplex*>(data),
                       isign < 0 ? CUFFT_FORWARD : CUFFT_INVERSE),
          "cufftExecC2C");
}

namespace {

void require_points(gbn_plan p) {
  if (!p) fail(GBN_ERR_ARG, "null plan");
  if (p->M < 0) fail(GBN_ERR_STATE, "gbn_setpts has not been called on this plan");
}

void run_interp(gbn_plan p, const InterpArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return;
  Span span(p, GBN_STAGE_INTERP, st);
  ck(a.g.dim == 2 ? launch_interp2d(a, st) : launch_interp3d(a, st), "interp kernel");
  p->launches++;
}
void run_spread(gbn_plan p, const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return;
  Span span(p, GBN_STAGE_SPREAD, st);
  // 2D: the streaming spreader for several transforms per call, the
  // warp-cooperative one (any sort order) for a single transform
  const bool stream = p->stream_spread && (a.g.dim == 3 || a.ntr >= 2);
  ck(stream ? (a.g.dim == 2 ? launch_spread_stream2d(a, st) : launch_spread_stream3d(a, st))
            : (a.g.dim == 2 ? launch_spread2d(a, st) : launch_spread3d(a, st)),
     "spread kernel");
  p->launches++;
}
void run_pad(gbn_plan p, const PadArgs& a, cudaStream_t st) {
  Span span(p, GBN_STAGE_PAD, st);
  ck(launch_pad(a, st), "pad pass");
  p->launches++;
}
void run_crop(gbn_plan p, const CropArgs& a, cudaStream_t st) {
  Span span(p, GBN_STAGE_CROP, st);
  ck(launch_crop(a, st), "crop pass");
  p->launches++;
}
// op: pad + forward transform (fused line transforms on 256^3 grids)
void run_pad_fft(gbn_plan p, const PadArgs& a, int isign, cudaStream_t st) {
  if (p->fft512) {
    Span span(p, GBN_STAGE_FFT, st);
    ck(launch_fft512_op(a, p->tw512, isign, st), "fused pad + transform");
    p->launches += 2;
    return;
  }
  if (p->fft256) {
    Span span(p, GBN_STAGE_FFT, st);
    ck(launch_fft256_op(a, p->tw256, isign, st), "fused pad + transform");
    p->launches += 3;
    return;
  }
  run_pad(p, a, st);
  p->exec_fft(a.ntr, p->fine, isign, st, 1);
}
// adjoint: inverse transform + crop
void run_fft_crop(gbn_plan p, const CropArgs& a, int isign, cudaStream_t st) {
  if (p->fft512) {
    Span span(p, GBN_STAGE_FFT, st);
    ck(launch_fft512_adj(a, const_cast<float2*>(a.fine), p->tw512, isign, st),
       "fused transform + crop");
    p->launches += 2;
    return;
  }
  if (p->fft256) {
    Span span(p, GBN_STAGE_FFT, st);
    ck(launch_fft256_adj(a, p->fine, p->tw256, isign, st), "fused transform + crop");
    p->launches += 3;
    return;
  }
  p->exec_fft(a.ntr, p->fine, isign, st, 2);
  run_crop(p, a, st);
}
void run_zero(gbn_plan p, float2* dst, size_t cells, cudaStream_t st) {
  Span span(p, GBN_STAGE_ZERO, st);
  ck(cudaMemsetAsync(dst, 0, sizeof(float2) * cells, st), "zero grid");
}
void run_grad(gbn_plan p, const GradArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return;
  Span span(p, GBN_STAGE_GRAD, st);
  ck(a.g.dim == 2 ? launch_grad2d(a, st) : launch_grad3d(a, st), "gradient kernel");
  p->launches++;
}

PadArgs pad_args(gbn_plan p, const float2* img, const float2* smaps, int ntr, int conj_in) {
  PadArgs a{};
  a.g = p->g;
  a.img = img;
  a.smaps = smaps;
  for (int d = 0; d < 3; ++d) a.dec[d] = p->dec[d];
  a.fine = p->fine;
  a.ntr = ntr;
  a.conj_in = conj_in;
  a.scale = 1.0f;
  return a;
}

CropArgs crop_args(gbn_plan p, const float2* smaps, float2* out, int ntr, int accumulate,
                   float scale) {
  CropArgs a{};
  a.g = p->g;
  a.fine = p->fine;
  a.smaps = smaps;
  for (int d = 0; d < 3; ++d) a.dec[d] = p->dec[d];
  a.out = out;
  a.ntr = ntr;
  a.accumulate = accumulate;
  a.scale = scale;
  return a;
}

InterpArgs interp_args(gbn_plan p, const float2* fine, float2* out, int ntr, float scale,
                       int mode) {
  InterpArgs a{};
  a.g = p->g;
  a.s = p->sorted();
  a.fine = fine;
  a.out = out;
  a.ntr = ntr;
  a.scale = scale;
  a.mode = mode;
  return a;
}

SpreadArgs spread_args(gbn_plan p, const float2* in, const float* density, float2* fine,
                       int ntr, float scale) {
  SpreadArgs a{};
  a.g = p->g;
  a.s = p->sorted_spread();
  a.in = in;
  a.density = density;
  a.fine = fine;
  a.ntr = ntr;
  a.scale = scale;
  return a;
}

// Iterate transform passes.  SENSE: pass = (batch b, coils c0..c0+T);
// calibrationless: pass = rows r0..r0+T of the flattened (B*C) stack.
template <typename F>
void for_each_pass(gbn_plan p, bool sense, int B, int C, F&& f) {
  const int T = p->ntrans;
  if (sense) {
    for (int b = 0; b < B; ++b)
      for (int c0 = 0; c0 < C; c0 += T) f(b, c0, imin(T, C - c0));
  } else {
    const int R = B * C;
    for (int r0 = 0; r0 < R; r0 += T) f(-1, r0, imin(T, R - r0));
  }
}

void check_counts(int B, int C) {
  if (B < 1 || C < 1) fail(GBN_ERR_ARG, "n_batchs and n_coils must be >= 1");
}

template <typename F>
int guarded(gbn_plan p, F&& f) {
  try {
    if (!p) fail(GBN_ERR_ARG, "null plan");
    DeviceGuard dg(p->device);
    f();
    return GBN_OK;
  } catch (const Fail& e) {
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return GBN_ERR_NOMEM;
  } catch (...) {
    g_err = "unexpected error";
    return GBN_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

int gbn_version(void) { return 100; }

const char* gbn_last_error(void) { return g_err.c_str(); }

int gbn_plan_create(int dim, const int64_t* n_modes, double upsampfac, double eps, int ntrans,
                    int spread_only, int device, gbn_plan* out) {
  g_err.clear();
  if (!out) {
    g_err = "null output pointer";
    return GBN_ERR_ARG;
  }
  *out = nullptr;
  gbn_plan p = nullptr;
  try {
    if (dim != 2 && dim != 3) fail(GBN_ERR_ARG, "dim must be 2 or 3");
    if (!n_modes) fail(GBN_ERR_ARG, "null n_modes");
    if (!(eps > 0.0) || !(eps < 1.0)) fail(GBN_ERR_ARG, "eps must be in (0, 1)");
    if (!(upsampfac > 1.0) && !spread_only) fail(GBN_ERR_ARG, "upsampfac must be > 1");
    if (ntrans < 1) fail(GBN_ERR_ARG, "ntrans must be >= 1");
    int ndev = 0;
    ck(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) fail(GBN_ERR_ARG, "invalid device ordinal");
    DeviceGuard dg(device);
    p = new gbn_plan_s();
    p->device = device;
    p->ntrans = ntrans;
    p->spread_only = spread_only ? 1 : 0;
    p->eps = eps;
    p->sigma = upsampfac;
    cudaDeviceProp prop;
    ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    p->nsm = prop.multiProcessorCount;
    int w;
    double beta;
    kernel_params(eps, upsampfac > 1.0 ? upsampfac : 2.0, &w, &beta);
    p->beta = beta;
    Geom& g = p->g;
    g.dim = dim;
    g.w = w;
    g.beta = (float)beta;
    g.halfw = 0.5f * w;
    g.inv_halfw = 2.0f / w;
    g.G = 1;
    g.Nimg = 1;
    // 2D: 19-cell x bins (with w <= 7 the padded column is at most 26 rows,
    // two overlapping 16-row halves of a warp in the streaming spreader)
    int binsz2[2] = {19, 32};
    int binsz3[3] = {8, 8, 8};
    // tuning overrides: GBN_BINS2="b0,b1", GBN_BINS3="b0,b1,b2", GBN_INTERP_CG=1|2|4
    if (const char* e = std::getenv(dim == 2 ? "GBN_BINS2" : "GBN_BINS3")) {
      int v[3] = {0, 0, 0};
      if (std::sscanf(e, "%d,%d,%d", &v[0], &v[1], &v[2]) >= dim)
        for (int d = 0; d < dim; ++d)
          if (v[d] >= 1 && v[d] <= 64) (dim == 2 ? binsz2[d] : binsz3[d]) = v[d];
    }
    if (const char* e = std::getenv("GBN_INTERP_CG")) g.interp_cg = std::atoi(e);
    if (const char* e = std::getenv("GBN_SPREAD_CG")) g.spread_cg = std::atoi(e);
    if (const char* e = std::getenv("GBN_QUAD_MINB")) g.quad_minb = std::atoi(e);
    g.quad_packed = 1;
    if (const char* e = std::getenv("GBN_QUAD_PACKED")) g.quad_packed = std::atoi(e);
    if (const char* e = std::getenv("GBN_INTERP"))
      g.method_interp = std::strcmp(e, "gm") == 0   ? 1
                        : std::strcmp(e, "db") == 0 ? 3
                        : std::strcmp(e, "wc") == 0 ? 4
                        : std::strcmp(e, "twc") == 0 ? 5
                        : std::strcmp(e, "tile") == 0 ? 6
                                                     : 0;
    if (const char* e = std::getenv("GBN_INTERP_THREADS")) {
      int v = std::atoi(e);
      if (v == 64 || v == 128 || v == 256) g.interp_threads = v;
    }
    if (const char* e = std::getenv("GBN_SPREAD"))
      g.method_spread = std::strcmp(e, "gm") == 0       ? 1
                        : std::strcmp(e, "wc") == 0     ? 2
                        : std::strcmp(e, "stream") == 0 ? 3
                        : std::strcmp(e, "rows") == 0   ? 4
                        : std::strcmp(e, "quad") == 0   ? 5
                        : std::strcmp(e, "mma") == 0    ? 6
                                                        : 0;
    for (int d = 0; d < 3; ++d) {
      if (d < dim) {
        int64_t N = n_modes[d];
        if (N < 1 || N > (1 << 20)) fail(GBN_ERR_ARG, "image size out of range");
        int64_t nf;
        if (spread_only) nf = N;
        else {
          int64_t want = (int64_t)std::ceil(upsampfac * (double)N);
          if (want < 2 * w) want = 2 * w;
          nf = next_smooth_even(want);
        }
        g.n[d] = (int)N;
        g.nf[d] = (int)nf;
        int bs = dim == 2 ? binsz2[d] : binsz3[d];
        if (bs > nf) bs = (int)nf;
        g.bs[d] = bs;
        g.nb[d] = (int)((nf + bs - 1) / bs);
        g.pd[d] = bs + w;
        g.uscale[d] = (float)((double)nf / (2.0 * M_PI));
      } else {
        g.n[d] = g.nf[d] = g.bs[d] = g.nb[d] = g.pd[d] = 1;
        g.uscale[d] = 0.f;
      }
      g.G *= g.nf[d];
      g.Nimg *= g.n[d];
    }
    if (g.G > ((int64_t)1 << 31) - 1) fail(GBN_ERR_ARG, "fine grid larger than 2^31 cells");
    g.tile = g.pd[0] * g.pd[1] * g.pd[2];
    if ((int64_t)g.tile * 8 > kTileSmemBudget) fail(GBN_ERR_ARG, "tile does not fit shared memory");
    if (!spread_only) {
      for (int d = 0; d < dim; ++d) {
        std::vector<float> f = deconv_factors(g.n[d], g.nf[d], w, beta);
        p->dec[d] = dev_alloc<float>(f.size(), p->bytes, "deconv factors");
        ck(cudaMemcpy(p->dec[d], f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice),
           "copy deconv factors");
      }
    }
    {
      const char* e = std::getenv("GBN_FFT_PRUNE");
      p->prune = dim == 3 && !spread_only && g.nf[0] > g.n[0] && !(e && std::atoi(e) == 0);
      const char* f = std::getenv("GBN_FUSED_FFT");
      p->fft256 = !spread_only && fft256_fits(g) && !(f && std::atoi(f) == 0);
      if (p->fft256) {
        std::vector<float> t = fft256_twiddles();
        p->tw256 = dev_alloc<float2>(256, p->bytes, "transform twiddles");
        ck(cudaMemcpy(p->tw256, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice),
           "copy transform twiddles");
        ck(fft256_prepare(), "transform kernel attributes");
      }
      p->fft512 = !spread_only && fft512_fits(g) && !(f && std::atoi(f) == 0);
      if (p->fft512) {
        std::vector<float> t = fft512_twiddles();
        p->tw512 = dev_alloc<float2>(512, p->bytes, "transform twiddles");
        ck(cudaMemcpy(p->tw512, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice),
           "copy transform twiddles");
        ck(fft512_prepare(), "transform kernel attributes");
      }
    }
    p->fine = dev_alloc<float2>((size_t)ntrans * g.G, p->bytes, "fine grid");
    p->setup_bins();
    p->sb.d_total = dev_alloc<int>(2, p->bytes, "scan");
    *out = p;
    return GBN_OK;
  } catch (const Fail& e) {
    delete p;
    return e.code;
  } catch (const std::bad_alloc&) {
    delete p;
    g_err = "host allocation failed";
    return GBN_ERR_NOMEM;
  }
}

int gbn_plan_destroy(gbn_plan plan) {
  if (!plan) return GBN_OK;
  int dev = plan->device;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != dev) cudaSetDevice(dev);
  delete plan;
  if (prev >= 0 && prev != dev) cudaSetDevice(prev);
  return GBN_OK;
}

int gbn_plan_info(gbn_plan p, int* width, double* beta, int64_t* nf, int* bins) {
  if (!p) {
    g_err = "null plan";
    return GBN_ERR_ARG;
  }
  if (width) *width = p->g.w;
  if (beta) *beta = p->beta;
  for (int d = 0; d < 3; ++d) {
    if (nf) nf[d] = p->g.nf[d];
    if (bins) bins[d] = p->g.bs[d];
  }
  return GBN_OK;
}

int gbn_plan_device_bytes(gbn_plan p, int64_t* bytes) {
  if (!p || !bytes) {
    g_err = "null argument";
    return GBN_ERR_ARG;
  }
  *bytes = p->bytes;
  return GBN_OK;
}

int gbn_setpts(gbn_plan p, int64_t M, const float* k0, const float* k1, const float* k2,
               gbn_stream stream) {
  return guarded(p, [&] {
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (M < 0 || M > ((int64_t)1 << 31) - 1) fail(GBN_ERR_ARG, "M out of range");
    if (M > 0 && (!k0 || !k1 || (p->g.dim == 3 && !k2))) fail(GBN_ERR_ARG, "null coordinates");
    // subproblem size: aim at >= 4 subproblems per SM, 32..1024 samples
    int64_t target = M / (4 * (int64_t)p->nsm);
    int cap = p->maxsub_cap;
    if (const char* e = std::getenv("GBN_MAXSUB")) {
      int v = std::atoi(e);
      if (v >= 32 && v <= 65536) cap = v;
    }
    int maxsub = 32;
    while (maxsub < target && maxsub < cap) maxsub <<= 1;
    // interp / grad subproblems are cut finer than the spread chunks: at most
    // one sample per thread of the 128-thread tile interp (its weights then
    // stay in registers across coils; measured 2.5 % faster in 3D than 512)
    const int maxsub_i = [&] {
      if (!p->stream_spread) return maxsub;
      const char* e = std::getenv("GBN_INTERP_MAXSUB");
      int v = e ? std::atoi(e) : 128;
      if (v < 32) v = 128;
      return v < maxsub ? v : maxsub;
    }();
    int64_t subcap = M / maxsub_i + (M < p->ngrp ? M : p->ngrp) + 1;
    // spread chunks of the streaming kernel: one CTA batch at most
    const int chunk = p->g.dim == 2 ? kStreamChunk2 : kStreamChunk;
    const int maxsub_s = maxsub < chunk ? maxsub : chunk;
    int64_t sscap = p->stream_spread ? M / maxsub_s + (M < p->ncol ? M : p->ncol) + 1 : 0;
    if (M > p->Mcap || subcap > p->subcap || sscap > p->sscap) {
      // free the previous point buffers before the new ones (bytes tally)
      int64_t cap = M > p->Mcap ? M : p->Mcap;
      int64_t scap = subcap > p->subcap ? subcap : p->subcap;
      int64_t sscap2 = sscap > p->sscap ? sscap : p->sscap;
      p->free_points();
      p->bytes -= p->point_bytes;
      p->point_bytes = 0;
      p->Mcap = p->subcap = p->sscap = 0;
      const int64_t b0 = p->bytes;
      p->sb.bin_of = dev_alloc<int>(cap, p->bytes, "sort scratch");
      p->sb.rank_of = dev_alloc<int>(cap, p->bytes, "sort scratch");
      p->sb.perm = dev_alloc<int>(cap, p->bytes, "permutation");
      for (int d = 0; d < p->g.dim; ++d) p->sb.u[d] = dev_alloc<float>(cap, p->bytes, "coords");
      p->sb.sub_bin = dev_alloc<int>(scap, p->bytes, "subproblems");
      p->sb.sub_start = dev_alloc<int>(scap, p->bytes, "subproblems");
      p->sb.sub_count = dev_alloc<int>(scap, p->bytes, "subproblems");
      if (sscap2 > 0) p->ssub = dev_alloc<int>(3 * sscap2, p->bytes, "spread chunks");
      p->point_bytes = p->bytes - b0;
      p->Mcap = cap;
      p->subcap = scap;
      p->sscap = sscap2;
    }
    const float* k[3] = {k0, k1, k2};
    p->maxsub = maxsub_i;
    p->maxsub_s = maxsub_s;
    int totals[2] = {0, 0};
    if (p->stream_spread) {
      const Geom& g = p->g;
      const int last = g.dim - 1;
      Geom gs = g;  // sort key: the bins of the other axes, then the last-axis cell
      gs.bs[last] = 1;
      gs.nb[last] = g.nf[last];
      ck(sort_points(gs, M, k, maxsub, p->sb, st, false), "sort");
      int* q = p->grp;
      GroupBuffers gi{q, q + p->ngrp, q + 2 * p->ngrp, q + 3 * p->ngrp,
                      p->sb.sub_bin, p->sb.sub_start, p->sb.sub_count};
      q += 4 * (size_t)p->ngrp;
      GroupBuffers gc{q, q + p->ncol, q + 2 * p->ncol, q + 3 * p->ncol,
                      p->ssub, p->ssub + p->sscap, p->ssub + 2 * p->sscap};
      ck(build_group_table(p->ngrp, g.nb[last], g.bs[last], g.nf[last], maxsub_i, p->sb, gi,
                           p->sb.d_total, st),
         "interp groups");
      ck(build_group_table(p->ncol, 1, g.nf[last], g.nf[last], maxsub_s, p->sb, gc,
                           p->sb.d_total + 1, st),
         "spread chunks");
    } else {
      ck(sort_points(p->g, M, k, maxsub, p->sb, st, true), "sort");
    }
    ck(cudaMemcpyAsync(totals, p->sb.d_total, sizeof(totals), cudaMemcpyDeviceToHost, st),
       "copy subproblem count");
    ck(cudaStreamSynchronize(st), "setpts sync");
    const int total = totals[0];
    if (total > p->subcap || (p->stream_spread && totals[1] > p->sscap))
      fail(GBN_ERR_CUDA, "subproblem table overflow");
    p->nsub_s = p->stream_spread ? totals[1] : 0;
    p->nsub = total;
    p->M = M;
  });
}

int gbn_op(gbn_plan p, const void* img, const void* smaps, void* ksp, int B, int C,
           float scale, int isign, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    check_counts(B, C);
    if (!img || (!ksp && p->M > 0)) fail(GBN_ERR_ARG, "null image or k-space pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const float2* x = static_cast<const float2*>(img);
    const float2* s = static_cast<const float2*>(smaps);
    float2* y = static_cast<float2*>(ksp);
    const Geom& g = p->g;
    if (p->spread_only) {
      if (s) fail(GBN_ERR_ARG, "coil maps are not supported on a spread-only plan");
      // the image array is the fine grid
      for (int r0 = 0; r0 < B * C; r0 += p->ntrans) {
        int T = imin(p->ntrans, B * C - r0);
        run_interp(p, interp_args(p, x + (int64_t)r0 * g.G, y + (int64_t)r0 * p->M, T,
                                      scale, INTERP_STORE), st);
      }
      return;
    }
    for_each_pass(p, s != nullptr, B, C, [&](int b, int c0, int T) {
      PadArgs pa = s ? pad_args(p, x + (int64_t)b * g.Nimg, s + (int64_t)c0 * g.Nimg, T, 0)
                     : pad_args(p, x + (int64_t)c0 * g.Nimg, nullptr, T, 0);
      run_pad_fft(p, pa, isign, st);
      int64_t row = s ? (int64_t)b * C + c0 : c0;
      run_interp(p, interp_args(p, p->fine, y + row * p->M, T, scale, INTERP_STORE), st);
    });
  });
}

int gbn_adj(gbn_plan p, const void* ksp, const float* density, const void* smaps, void* img,
            int B, int C, float scale, int isign, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    check_counts(B, C);
    if (!img || (!ksp && p->M > 0)) fail(GBN_ERR_ARG, "null image or k-space pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const float2* y = static_cast<const float2*>(ksp);
    const float2* s = static_cast<const float2*>(smaps);
    float2* x = static_cast<float2*>(img);
    const Geom& g = p->g;
    if (p->spread_only) {
      if (s) fail(GBN_ERR_ARG, "coil maps are not supported on a spread-only plan");
      for (int r0 = 0; r0 < B * C; r0 += p->ntrans) {
        int T = imin(p->ntrans, B * C - r0);
        float2* dst = x + (int64_t)r0 * g.G;
        run_zero(p, dst, (size_t)T * g.G, st);
        run_spread(p, spread_args(p, y + (int64_t)r0 * p->M, density, dst, T, scale), st);
      }
      return;
    }
    for_each_pass(p, s != nullptr, B, C, [&](int b, int c0, int T) {
      run_zero(p, p->fine, (size_t)T * g.G, st);
      int64_t row = s ? (int64_t)b * C + c0 : c0;
      run_spread(p, spread_args(p, y + row * p->M, density, p->fine, T, 1.0f), st);
      CropArgs ca = s ? crop_args(p, s + (int64_t)c0 * g.Nimg, x + (int64_t)b * g.Nimg, T,
                                  c0 > 0, scale)
                      : crop_args(p, nullptr, x + (int64_t)c0 * g.Nimg, T, 0, scale);
      run_fft_crop(p, ca, isign, st);
    });
  });
}

int gbn_dc(gbn_plan p, const void* img, const void* obs, const float* density,
           const void* smaps, void* grad, int B, int C, float scale, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    check_counts(B, C);
    if (p->spread_only) fail(GBN_ERR_ARG, "data consistency needs a full NUFFT plan");
    if (!img || !grad || (!obs && p->M > 0)) fail(GBN_ERR_ARG, "null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const float2* x = static_cast<const float2*>(img);
    const float2* yo = static_cast<const float2*>(obs);
    const float2* s = static_cast<const float2*>(smaps);
    float2* gr = static_cast<float2*>(grad);
    const Geom& g = p->g;
    int64_t need = (int64_t)p->ntrans * (p->M > 0 ? p->M : 1);
    if (need > p->kbuf_cap) {
      dev_free(p->kbuf);
      p->bytes -= p->kbuf_cap * 8;
      p->kbuf = nullptr;
      p->kbuf_cap = 0;
      p->kbuf = dev_alloc<float2>(need, p->bytes, "residual buffer");
      p->kbuf_cap = need;
    }
    for_each_pass(p, s != nullptr, B, C, [&](int b, int c0, int T) {
      PadArgs pa = s ? pad_args(p, x + (int64_t)b * g.Nimg, s + (int64_t)c0 * g.Nimg, T, 0)
                     : pad_args(p, x + (int64_t)c0 * g.Nimg, nullptr, T, 0);
      run_pad_fft(p, pa, -1, st);
      int64_t row = s ? (int64_t)b * C + c0 : c0;
      InterpArgs ia = interp_args(p, p->fine, p->kbuf, T, scale, INTERP_RESID);
      ia.obs = yo + row * p->M;
      ia.density = density;
      run_interp(p, ia, st);
      run_zero(p, p->fine, (size_t)T * g.G, st);
      run_spread(p, spread_args(p, p->kbuf, nullptr, p->fine, T, 1.0f), st);
      CropArgs ca = s ? crop_args(p, s + (int64_t)c0 * g.Nimg, gr + (int64_t)b * g.Nimg, T,
                                  c0 > 0, scale)
                      : crop_args(p, nullptr, gr + (int64_t)c0 * g.Nimg, T, 0, scale);
      run_fft_crop(p, ca, +1, st);
    });
  });
}

int gbn_pipe(gbn_plan p, void* w, int iters, float scale2, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    if (!p->spread_only) fail(GBN_ERR_ARG, "pipe needs a spread-only plan");
    if (!w && p->M > 0) fail(GBN_ERR_ARG, "null weights");
    if (iters < 0) fail(GBN_ERR_ARG, "iters must be >= 0");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    float2* wv = static_cast<float2*>(w);
    const Geom& g = p->g;
    for (int it = 0; it < iters; ++it) {
      run_zero(p, p->fine, (size_t)g.G, st);
      run_spread(p, spread_args(p, wv, nullptr, p->fine, 1, 1.0f), st);
      run_interp(p, interp_args(p, p->fine, wv, 1, scale2, INTERP_PIPE), st);
    }
  });
}

static void grad_traj_common(gbn_plan p, const float2* img, const float2* s, const float2* a,
                             float* grad, int B, int C, float scale, int adjoint,
                             cudaStream_t st) {
  const Geom& g = p->g;
  if (p->M > 0)
    ck(cudaMemsetAsync(grad, 0, sizeof(float) * (size_t)p->M * g.dim, st), "zero gradient");
  for_each_pass(p, s != nullptr, B, C, [&](int b, int c0, int T) {
    PadArgs pa = s ? pad_args(p, img + (int64_t)b * g.Nimg, s + (int64_t)c0 * g.Nimg, T, adjoint)
                   : pad_args(p, img + (int64_t)c0 * g.Nimg, nullptr, T, adjoint);
    run_pad_fft(p, pa, adjoint ? +1 : -1, st);
    int64_t row = s ? (int64_t)b * C + c0 : c0;
    GradArgs ga{};
    ga.g = g;
    ga.s = p->sorted();
    ga.fine = p->fine;
    ga.dy = a + row * p->M;
    ga.grad = grad;
    ga.ntr = T;
    ga.scale = scale;
    ga.conj_a = adjoint ? 0 : 1;
    run_grad(p, ga, st);
  });
}

int gbn_grad_traj_op(gbn_plan p, const void* img, const void* smaps, const void* dy,
                     float* grad, int B, int C, float scale, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    check_counts(B, C);
    if (p->spread_only) fail(GBN_ERR_ARG, "needs a full NUFFT plan");
    if (!img || ((!dy || !grad) && p->M > 0)) fail(GBN_ERR_ARG, "null pointer");
    grad_traj_common(p, static_cast<const float2*>(img), static_cast<const float2*>(smaps),
                     static_cast<const float2*>(dy), grad, B, C, scale, 0,
                     reinterpret_cast<cudaStream_t>(stream));
  });
}

int gbn_grad_traj_adj(gbn_plan p, const void* dx, const void* smaps, const void* y, float* grad,
                      int B, int C, float scale, gbn_stream stream) {
  return guarded(p, [&] {
    require_points(p);
    check_counts(B, C);
    if (p->spread_only) fail(GBN_ERR_ARG, "needs a full NUFFT plan");
    if (!dx || ((!y || !grad) && p->M > 0)) fail(GBN_ERR_ARG, "null pointer");
    grad_traj_common(p, static_cast<const float2*>(dx), static_cast<const float2*>(smaps),
                     static_cast<const float2*>(y), grad, B, C, scale, 1,
                     reinterpret_cast<cudaStream_t>(stream));
  });
}

int gbn_profile(gbn_plan p, int enable) {
  return guarded(p, [&] {
    for (int i = 0; i < GBN_STAGES; ++i) p->spans[i].clear();
    p->evnext = 0;
    p->launches = 0;
    p->prof = enable != 0;
  });
}

int gbn_profile_read(gbn_plan p, int stage, double* total_ms, int64_t* count) {
  return guarded(p, [&] {
    if (stage < -1 || stage >= GBN_STAGES) fail(GBN_ERR_ARG, "unknown stage");
    double ms = 0.0;
    int64_t n = 0;
    for (int i = (stage < 0 ? 0 : stage); i < (stage < 0 ? GBN_STAGES : stage + 1); ++i) {
      for (auto& sp : p->spans[i]) {
        ck(cudaEventSynchronize(p->evpool[sp.second]), "cudaEventSynchronize");
        float t = 0.f;
        ck(cudaEventElapsedTime(&t, p->evpool[sp.first], p->evpool[sp.second]), "elapsed");
        ms += t;
      }
      n += (int64_t)p->spans[i].size();
    }
    if (total_ms) *total_ms = ms;
    if (count) *count = stage < 0 ? p->launches : n;
  });
}

int gbn_plan_tune(gbn_plan p, const int* bins, int interp_method, int maxsub_cap) {
  return guarded(p, [&] {
    Geom& g = p->g;
    if (bins) {
      Geom t = g;
      for (int d = 0; d < g.dim; ++d) {
        if (bins[d] < 1 || bins[d] > 64) fail(GBN_ERR_ARG, "bin sizes must be in [1, 64]");
        t.bs[d] = bins[d] > g.nf[d] ? g.nf[d] : bins[d];
        t.nb[d] = (g.nf[d] + t.bs[d] - 1) / t.bs[d];
        t.pd[d] = t.bs[d] + g.w;
      }
      t.tile = t.pd[0] * t.pd[1] * t.pd[2];
      if ((int64_t)t.tile * 8 > kTileSmemBudget) fail(GBN_ERR_ARG, "tile does not fit shared memory");
      g = t;
      p->setup_bins();
      p->M = -1;  // points must be set again
    }
    if (interp_method >= 0) {
      if (interp_method > 5 || interp_method == 2) fail(GBN_ERR_ARG, "unknown interpolation method");
      g.method_interp = interp_method;
    }
    if (maxsub_cap > 0) {
      if (maxsub_cap < 32 || maxsub_cap > 65536) fail(GBN_ERR_ARG, "maxsub_cap must be in [32, 65536]");
      p->maxsub_cap = maxsub_cap;
      p->M = -1;
    }
  });
}

static int simple_status(cudaError_t e) {
  if (e == cudaSuccess) return GBN_OK;
  g_err = cudaGetErrorString(e);
  return GBN_ERR_CUDA;
}

int gbn_cg_update(int64_t n, const void* grad_new, void* grad, void* velocity, void* image,
                  double* state, const float* lipschitz, float tol, gbn_stream stream) {
  g_err.clear();
  if (n < 0 || !state || !lipschitz || (n > 0 && (!grad_new || !grad || !velocity || !image))) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  return simple_status(launch_cg_update(n, static_cast<const float2*>(grad_new),
                                        static_cast<float2*>(grad), static_cast<float2*>(velocity),
                                        static_cast<float2*>(image), state, lipschitz, tol,
                                        reinterpret_cast<cudaStream_t>(stream)));
}

int gbn_power_step(int64_t n, const void* x_new, void* x, double* state, float* lipschitz,
                   gbn_stream stream) {
  g_err.clear();
  if (n < 0 || !state || !lipschitz || (n > 0 && (!x_new || !x))) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  return simple_status(launch_power_step(n, static_cast<const float2*>(x_new),
                                         static_cast<float2*>(x), state, lipschitz,
                                         reinterpret_cast<cudaStream_t>(stream)));
}

int gbn_scale_ratio(int64_t n, void* x, const double* num2, const double* den2, gbn_stream stream) {
  g_err.clear();
  if (n < 0 || !num2 || !den2 || (n > 0 && !x)) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  return simple_status(launch_scale_ratio(n, static_cast<float2*>(x), num2, den2,
                                          reinterpret_cast<cudaStream_t>(stream)));
}

int gbn_orc_reduce(const void* yl, const void* B, void* y, int nb, int L, int C, int64_t M,
                   int64_t NK, gbn_stream stream) {
  g_err.clear();
  if (nb < 1 || L < 1 || C < 1 || M < 0 || NK < 1 || M % NK != 0 ||
      (M > 0 && (!yl || !B || !y))) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  return simple_status(launch_orc_reduce(static_cast<const float2*>(yl), static_cast<const float2*>(B),
                                         static_cast<float2*>(y), nb, L, C, M, NK,
                                         reinterpret_cast<cudaStream_t>(stream)));
}

int gbn_orc_expand(const void* y, const void* B, void* yl, int nb, int L, int C, int64_t M,
                   int64_t NK, gbn_stream stream) {
  g_err.clear();
  if (nb < 1 || L < 1 || C < 1 || M < 0 || NK < 1 || M % NK != 0 ||
      (M > 0 && (!yl || !B || !y))) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  return simple_status(launch_orc_expand(static_cast<const float2*>(y), static_cast<const float2*>(B),
                                         static_cast<float2*>(yl), nb, L, C, M, NK,
                                         reinterpret_cast<cudaStream_t>(stream)));
}

int gbn_norm2_f64(const void* x, int64_t n, double* out, gbn_stream stream) {
  g_err.clear();
  if ((!x && n > 0) || !out || n < 0) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  cudaError_t e = launch_norm2(static_cast<const float2*>(x), n, out,
                               reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return GBN_ERR_CUDA;
  }
  return GBN_OK;
}

int gbn_dotu_f64(const void* a, const void* b, int64_t n, int conj_a, double* out,
                 gbn_stream stream) {
  g_err.clear();
  if (((!a || !b) && n > 0) || !out || n < 0) {
    g_err = "invalid argument";
    return GBN_ERR_ARG;
  }
  cudaError_t e = launch_dotu(static_cast<const float2*>(a), static_cast<const float2*>(b), n,
                              conj_a, out, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return GBN_ERR_CUDA;
  }
  return GBN_OK;
}

}  // extern "C"

// ----------------------------------------------------------------------------
// Toeplitz embedding of A^H W A
// ----------------------------------------------------------------------------
struct gbn_toep_s {
  gbn_plan inner = nullptr;  // circulant grid (n = N, nf >= 2N), FFT plans, fine grids
  float* K = nullptr;        // real kernel spectrum, inner->g.G cells
  int device = 0;
  ~gbn_toep_s() {
    DeviceGuard dg(device);
    dev_free(K);
    if (inner) gbn_plan_destroy(inner);
  }
};

namespace {
void chk(int rc) {
  if (rc != GBN_OK) throw Fail{rc};  // the message is already set
}

// A^H W A x by the Toeplitz embedding for every batch item and coil: per coil
// pass zero-pad (x * s_c), FFT, multiply by K, inverse FFT, crop with the
// conj(s_c) coil sum, times scale / prod(nf); `accumulate` adds every pass
// to what `out` holds.
void toep_apply(gbn_toep t, const void* img, const void* smaps, void* out, int B, int C,
                float scale, bool accumulate, cudaStream_t st) {
  gbn_plan p = t->inner;
  check_counts(B, C);
  if (!img || !out) fail(GBN_ERR_ARG, "null image pointer");
  const float2* x = static_cast<const float2*>(img);
  const float2* s = static_cast<const float2*>(smaps);
  float2* o = static_cast<float2*>(out);
  const Geom& g = p->g;
  const float sc = (float)((double)scale / (double)g.G);  // inverse-FFT normalisation
  for_each_pass(p, s != nullptr, B, C, [&](int b, int c0, int T) {
    PadArgs pa = s ? pad_args(p, x + (int64_t)b * g.Nimg, s + (int64_t)c0 * g.Nimg, T, 0)
                   : pad_args(p, x + (int64_t)c0 * g.Nimg, nullptr, T, 0);
    pa.dec[0] = pa.dec[1] = pa.dec[2] = nullptr;
    CropArgs ca = s ? crop_args(p, s + (int64_t)c0 * g.Nimg, o + (int64_t)b * g.Nimg, T,
                                accumulate || c0 > 0, sc)
                    : crop_args(p, nullptr, o + (int64_t)c0 * g.Nimg, T, accumulate, sc);
    ca.dec[0] = ca.dec[1] = ca.dec[2] = nullptr;
    if (p->fft256) {  // the x transforms and the multiply in one pass over the lines
      Span span(p, GBN_STAGE_FFT, st);
      ck(launch_fft256_gram(pa, ca, t->K, p->tw256, st), "fused Toeplitz Gram");
      p->launches += 5;
      return;
    }
    if (p->fft512) {
      Span span(p, GBN_STAGE_FFT, st);
      ck(launch_fft512_gram(pa, ca, t->K, p->tw512, st), "fused Toeplitz Gram");
      p->launches += 3;
      return;
    }
    run_pad_fft(p, pa, -1, st);
    {
      Span span(p, GBN_STAGE_KMUL, st);
      ck(launch_kmul(p->fine, t->K, g.G, T, st), "Toeplitz multiply");
      p->launches++;
    }
    run_fft_crop(p, ca, +1, st);
  });
}
}  // namespace

extern "C" {

int gbn_toep_create(gbn_plan p, int64_t M, const float* k0, const float* k1, const float* k2,
                    const float* weights, gbn_toep* out, gbn_stream stream) {
  if (!out) {
    g_err = "null output handle";
    return GBN_ERR_ARG;
  }
  *out = nullptr;
  gbn_plan q = nullptr;
  float2* w2 = nullptr;
  float2* psf = nullptr;
  gbn_toep t = nullptr;
  int rc = guarded(p, [&] {
    if (p->spread_only) fail(GBN_ERR_ARG, "the Toeplitz embedding needs a full NUFFT plan");
    if (M < 0 || M > ((int64_t)1 << 31) - 1) fail(GBN_ERR_ARG, "M out of range");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const Geom& g = p->g;
    int64_t n1[3] = {1, 1, 1}, n2[3] = {1, 1, 1};
    int64_t P2 = 1;
    for (int d = 0; d < g.dim; ++d) {
      n1[d] = g.n[d];
      n2[d] = 2 * (int64_t)g.n[d];
      P2 *= n2[d];
    }
    int64_t tmp = 0;
    // psf: type-1 transform of the weights on 2N modes
    chk(gbn_plan_create(g.dim, n2, 2.0, p->eps, 1, 0, p->device, &q));
    chk(gbn_setpts(q, M, k0, k1, k2, stream));
    w2 = dev_alloc<float2>((size_t)M, tmp, "Toeplitz weights");
    ck(launch_fill_weights(weights, w2, M, st), "Toeplitz weights");
    psf = dev_alloc<float2>((size_t)P2, tmp, "Toeplitz psf");
    chk(gbn_adj(q, w2, nullptr, nullptr, psf, 1, 1, 1.0f, +1, stream));
    // circulant grid and the kernel spectrum
    t = new gbn_toep_s();
    t->device = p->device;
    chk(gbn_plan_create(g.dim, n1, 2.0, p->eps, p->ntrans, 0, p->device, &t->inner));
    gbn_plan in = t->inner;
    ck(launch_toep_place(in->g, psf, in->fine, st), "Toeplitz placement");
    in->exec_fft(1, in->fine, -1, st, 0);
    int64_t kb = 0;
    t->K = dev_alloc<float>((size_t)in->g.G, kb, "Toeplitz kernel");
    in->bytes += kb;
    ck(launch_real_part(in->fine, t->K, in->g.G, 1.0f, st), "Toeplitz kernel");
    ck(cudaStreamSynchronize(st), "Toeplitz kernel sync");
  });
  {
    DeviceGuard dg(p ? p->device : 0);
    dev_free(w2);
    dev_free(psf);
    if (q) gbn_plan_destroy(q);
  }
  if (rc != GBN_OK) {
    delete t;
    return rc;
  }
  *out = t;
  return GBN_OK;
}

int gbn_toep_info(gbn_toep t, int64_t* nf) {
  if (!t || !nf) {
    g_err = "null argument";
    return GBN_ERR_ARG;
  }
  for (int d = 0; d < 3; ++d) nf[d] = t->inner->g.nf[d];
  return GBN_OK;
}

int gbn_toep_kernel(gbn_toep t, float* dst, gbn_stream stream) {
  if (!t || !dst) {
    g_err = "null argument";
    return GBN_ERR_ARG;
  }
  return guarded(t->inner, [&] {
    ck(cudaMemcpyAsync(dst, t->K, sizeof(float) * t->inner->g.G, cudaMemcpyDeviceToDevice,
                       reinterpret_cast<cudaStream_t>(stream)),
       "copy Toeplitz kernel");
  });
}

int gbn_toep_apply(gbn_toep t, const void* img, const void* smaps, void* out, int B, int C,
                   float scale, gbn_stream stream) {
  if (!t) {
    g_err = "null Toeplitz handle";
    return GBN_ERR_ARG;
  }
  return guarded(t->inner, [&] {
    toep_apply(t, img, smaps, out, B, C, scale, false, reinterpret_cast<cudaStream_t>(stream));
  });
}

int gbn_toep_cg_iter(gbn_toep t, void* image, const void* smaps, const void* rhs, void* grad,
                     void* grad_new, void* velocity, double* state, const float* lipschitz, int B,
                     int C, float scale, float tol, gbn_stream stream) {
  if (!t) {
    g_err = "null Toeplitz handle";
    return GBN_ERR_ARG;
  }
  return guarded(t->inner, [&] {
    if (!image || !rhs || !grad || !grad_new || !velocity || !state || !lipschitz)
      fail(GBN_ERR_ARG, "null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const Geom& g = t->inner->g;
    const int64_t n = (int64_t)B * (smaps ? 1 : C) * g.Nimg;
    float2* gn = static_cast<float2*>(grad_new);
    ck(launch_neg_copy(static_cast<const float2*>(rhs), gn, n, st), "CG gradient");
    toep_apply(t, image, smaps, gn, B, C, scale, true, st);
    ck(launch_cg_dots(gn, static_cast<const float2*>(grad), n, state, st), "CG dots");
    ck(launch_cg_update(n, gn, static_cast<float2*>(grad), static_cast<float2*>(velocity),
                        static_cast<float2*>(image), state, lipschitz, tol, st),
       "CG update");
    t->inner->launches += 4;
  });
}

int gbn_toep_power_iter(gbn_toep t, void* x, void* x_new, double* state, float* lipschitz,
                        float scale, gbn_stream stream) {
  if (!t) {
    g_err = "null Toeplitz handle";
    return GBN_ERR_ARG;
  }
  return guarded(t->inner, [&] {
    if (!x || !x_new || !state || !lipschitz) fail(GBN_ERR_ARG, "null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t n = t->inner->g.Nimg;
    toep_apply(t, x, nullptr, x_new, 1, 1, scale, false, st);
    ck(launch_norm2(static_cast<const float2*>(x_new), n, state, st), "power norm");
    ck(launch_power_step(n, static_cast<const float2*>(x_new), static_cast<float2*>(x), state,
                         lipschitz, st),
       "power step");
    t->inner->launches += 3;
  });
}

int gbn_toep_plan(gbn_toep t, gbn_plan* out) {
  if (!t || !out) {
    g_err = "null argument";
    return GBN_ERR_ARG;
  }
  *out = t->inner;
  return GBN_OK;
}

int gbn_toep_destroy(gbn_toep t) {
  delete t;
  return GBN_OK;
}

}  // extern "C"

// ----------------------------------------------------------------------------
// Batches of independent plans
// ----------------------------------------------------------------------------
// Instances with the same fine grid share one contiguous pool of fine grids,
// so that one batched cuFFT call per grid size serves all of them.
struct FftGroup {
  int nf[3];
  int dim;
  int64_t G;
  int slots;  // sum of the members' ntrans
  float2* pool = nullptr;
  cufftHandle plan = 0;
};

struct gbn_batch_s {
  std::vector<gbn_plan> plans;
  std::vector<BatchInst> h_inst;
  std::vector<FftGroup> groups;
  BatchInst* d_inst = nullptr;
  WorkItem* d_work = nullptr;
  BatchTables t{};
  int device = 0;
  bool bound = false;
  ~gbn_batch_s() {
    for (auto& gr : groups) {
      if (gr.plan) cufftDestroy(gr.plan);
      dev_free(gr.pool);
    }
    dev_free(d_inst);
    dev_free(d_work);
  }
};

extern "C" {

int gbn_batch_create(int n, const gbn_plan* plans, gbn_batch* out) {
  g_err.clear();
  if (!out || !plans || n < 1) {
    g_err = "invalid batch arguments";
    return GBN_ERR_ARG;
  }
  *out = nullptr;
  gbn_batch b = nullptr;
  try {
    DeviceGuard dg(plans[0] ? plans[0]->device : 0);
    b = new gbn_batch_s();
    b->device = plans[0] ? plans[0]->device : 0;
    int64_t tmp = 0;
    std::vector<WorkItem> sub, fblk, iblk, sblk;
    size_t tile_bytes = 0;
    bool w7 = true, rows = true;
    for (int i = 0; i < n; ++i) {
      gbn_plan p = plans[i];
      if (!p) fail(GBN_ERR_ARG, "null plan in batch");
      if (p->M < 0) fail(GBN_ERR_STATE, "every plan of a batch needs gbn_setpts first");
      if (p->spread_only) fail(GBN_ERR_ARG, "spread-only plans cannot be batched");
      if (p->device != b->device) fail(GBN_ERR_ARG, "plans of a batch must share a device");
      if (p->g.dim != plans[0]->g.dim) fail(GBN_ERR_ARG, "plans of a batch must share dim");
      w7 = w7 && p->g.w == 7;
      if (plans[0]->g.w != p->g.w) fail(GBN_ERR_ARG, "plans of a batch must share the kernel width");
      rows = rows && rows_fit(p->g);
      b->plans.push_back(p);
      BatchInst bi{};
      bi.g = p->g;
      bi.s = p->sorted();
      bi.fine = p->fine;
      for (int d = 0; d < 3; ++d) bi.dec[d] = p->dec[d];
      b->h_inst.push_back(bi);
      for (int s = 0; s < p->nsub; ++s) sub.push_back({i, s});
      const int64_t cblock = (int64_t)GBN_THREADS * 16;  // cells per pad / zero / crop item
      for (int64_t k = 0; k < (p->g.G + cblock - 1) / cblock; ++k) fblk.push_back({i, (int)k});
      for (int64_t k = 0; k < (p->g.Nimg + cblock - 1) / cblock; ++k) iblk.push_back({i, (int)k});
      const int sblock = 256;  // samples per batched sample-block work item
      for (int64_t k = 0; k < (p->M + sblock - 1) / sblock; ++k) sblk.push_back({i, (int)k});
      size_t tb = (size_t)p->g.tile * sizeof(float2);
      if (tb > tile_bytes) tile_bytes = tb;
    }
    // group instances by fine-grid shape; each group gets one pool and one
    // cuFFT plan over all its coil slots
    for (int i = 0; i < n; ++i) {
      gbn_plan p = plans[i];
      int gi = -1;
      for (size_t k = 0; k < b->groups.size(); ++k) {
        const FftGroup& gr = b->groups[k];
        if (gr.nf[0] == p->g.nf[0] && gr.nf[1] == p->g.nf[1] && gr.nf[2] == p->g.nf[2]) gi = (int)k;
      }
      if (gi < 0) {
        FftGroup gr;
        for (int d = 0; d < 3; ++d) gr.nf[d] = p->g.nf[d];
        gr.dim = p->g.dim;
        gr.G = p->g.G;
        gr.slots = 0;
        b->groups.push_back(gr);
        gi = (int)b->groups.size() - 1;
      }
      b->groups[gi].slots += p->ntrans;
    }
    for (auto& gr : b->groups) {
      gr.pool = dev_alloc<float2>((size_t)gr.slots * gr.G, tmp, "batch fine-grid pool");
      int nn[3] = {gr.nf[0], gr.nf[1], gr.nf[2]};
      ckfft(cufftPlanMany(&gr.plan, gr.dim, nn, nullptr, 1, (int)gr.G, nullptr, 1, (int)gr.G,
                          CUFFT_C2C, gr.slots),
            "cufftPlanMany");
    }
    {
      std::vector<int> used(b->groups.size(), 0);
      for (int i = 0; i < n; ++i) {
        gbn_plan p = plans[i];
        for (size_t k = 0; k < b->groups.size(); ++k) {
          FftGroup& gr = b->groups[k];
          if (gr.nf[0] == p->g.nf[0] && gr.nf[1] == p->g.nf[1] && gr.nf[2] == p->g.nf[2]) {
            b->h_inst[i].fine = gr.pool + (int64_t)used[k] * gr.G;
            used[k] += p->ntrans;
            break;
          }
        }
      }
    }
    std::vector<WorkItem> all;
    all.insert(all.end(), sub.begin(), sub.end());
    all.insert(all.end(), fblk.begin(), fblk.end());
    all.insert(all.end(), iblk.begin(), iblk.end());
    all.insert(all.end(), sblk.begin(), sblk.end());
    b->d_inst = dev_alloc<BatchInst>(n, tmp, "batch instances");
    b->d_work = dev_alloc<WorkItem>(all.size(), tmp, "batch work tables");
    if (!all.empty())
      ck(cudaMemcpy(b->d_work, all.data(), all.size() * sizeof(WorkItem), cudaMemcpyHostToDevice),
         "copy work tables");
    BatchTables& t = b->t;
    t.inst = b->d_inst;
    t.sub = b->d_work;
    t.nsub = (int)sub.size();
    t.fblk = b->d_work + sub.size();
    t.nfblk = (int)fblk.size();
    t.iblk = t.fblk + fblk.size();
    t.niblk = (int)iblk.size();
    t.sblk = t.iblk + iblk.size();
    t.nsblk = (int)sblk.size();
    t.dim = plans[0]->g.dim;
    t.w7 = w7 ? 1 : 0;
    t.rows = rows ? 1 : 0;
    t.tile_bytes = tile_bytes;
    t.grid = plans[0]->nsm * 4;
    ck(batch_prepare(t), "batch kernel attributes");
    *out = b;
    return GBN_OK;
  } catch (const Fail& e) {
    delete b;
    return e.code;
  } catch (const std::bad_alloc&) {
    delete b;
    g_err = "host allocation failed";
    return GBN_ERR_NOMEM;
  }
}

int gbn_batch_bind(gbn_batch b, void* const* imgs, const void* const* smaps, void* const* ksps,
                   const float* const* densities, const float* scales, const int* n_coils) {
  g_err.clear();
  if (!b || !imgs || !ksps || !scales || !n_coils) {
    g_err = "invalid batch bind arguments";
    return GBN_ERR_ARG;
  }
  try {
    DeviceGuard dg(b->device);
    for (size_t i = 0; i < b->plans.size(); ++i) {
      gbn_plan p = b->plans[i];
      BatchInst& bi = b->h_inst[i];
      if (n_coils[i] < 1 || n_coils[i] > p->ntrans)
        fail(GBN_ERR_ARG, "instance " + std::to_string(i) + ": n_coils must be in [1, plan ntrans]");
      if (!imgs[i] || (!ksps[i] && p->M > 0)) fail(GBN_ERR_ARG, "null buffer in batch bind");
      bi.img = static_cast<float2*>(imgs[i]);
      bi.smaps = smaps ? static_cast<const float2*>(smaps[i]) : nullptr;
      bi.ksp = static_cast<float2*>(ksps[i]);
      bi.density = densities ? densities[i] : nullptr;
      bi.scale = scales[i];
      bi.ncoils = n_coils[i];
    }
    ck(cudaMemcpy(b->d_inst, b->h_inst.data(), b->h_inst.size() * sizeof(BatchInst),
                  cudaMemcpyHostToDevice),
       "copy batch descriptors");
    b->bound = true;
    return GBN_OK;
  } catch (const Fail& e) {
    return e.code;
  }
}

static int batch_run(gbn_batch b, bool adjoint, gbn_stream stream) {
  g_err.clear();
  if (!b) {
    g_err = "null batch";
    return GBN_ERR_ARG;
  }
  if (!b->bound) {
    g_err = "gbn_batch_bind has not been called";
    return GBN_ERR_STATE;
  }
  try {
    DeviceGuard dg(b->device);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    auto ffts = [&](int dir) {
      for (auto& gr : b->groups) {
        ckfft(cufftSetStream(gr.plan, st), "cufftSetStream");
        ckfft(cufftExecC2C(gr.plan, reinterpret_cast<cufftComplex*>(gr.pool),
                           reinterpret_cast<cufftComplex*>(gr.pool), dir),
              "cufftExecC2C");
      }
    };
    if (!adjoint) {
      ck(batch_pad(b->t, st), "batch pad");
      ffts(CUFFT_FORWARD);
      ck(batch_interp(b->t, st), "batch interp");
    } else {
      ck(batch_zero(b->t, st), "batch zero");
      ck(batch_spread(b->t, st), "batch spread");
      ffts(CUFFT_INVERSE);
      ck(batch_crop(b->t, st), "batch crop");
    }
    return GBN_OK;
  } catch (const Fail& e) {
    return e.code;
  }
}

int gbn_batch_op(gbn_batch b, gbn_stream stream) { return batch_run(b, false, stream); }
int gbn_batch_adj(gbn_batch b, gbn_stream stream) { return batch_run(b, true, stream); }

int gbn_batch_destroy(gbn_batch b) {
  if (!b) return GBN_OK;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != b->device) cudaSetDevice(b->device);
  delete b;
  if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
  return GBN_OK;
}

}  // extern "C"
