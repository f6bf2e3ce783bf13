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

#include <cstdlib>

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

// Largest number of tile rows (all axes but the last) whose fine-grid offsets
// are tabulated in shared memory; larger tiles compute them per load.
constexpr int kMaxTileRows = 1024;

// Fine-grid offsets of the rows of the padded tile at origin o (periodic
// wrap), computed once per subproblem so that the per-transform tile loads
// need no integer division.  Returns the table, or nullptr if the tile has
// more rows than the table holds.  The caller synchronises before use.
template <int DIM>
__device__ __forceinline__ const int* tile_rows_init(const Geom& g, const int* o, int* table) {
  const int nrows = DIM == 2 ? g.pd[0] : g.pd[0] * g.pd[1];
  if (nrows > kMaxTileRows) return nullptr;
  for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
    int off;
    if (DIM == 2) {
      off = wrap_idx(o[0] + r, g.nf[0]) * g.nf[1];
    } else {
      const int i1 = r % g.pd[1];
      const int i0 = r / g.pd[1];
      off = (wrap_idx(o[0] + i0, g.nf[0]) * g.nf[1] + wrap_idx(o[1] + i1, g.nf[1])) * g.nf[2];
    }
    table[r] = off;  // fine grids hold < 2^31 cells
  }
  return table;
}

// Stage the padded tiles of `nc` transforms (from transform c0 on) into shared
// memory.  Rows of the tile (all axes but the last) are spread over groups of
// `seg` threads, seg = a power of two >= the last tile extent, so that the
// row's cells load contiguously.  Row offsets come from `rowoff` (see
// tile_rows_init) when given.
template <int DIM>
__device__ __forceinline__ void load_tiles(float2* tile, const float2* __restrict__ fine,
                                           const Geom& g, const int* o, int c0, int nc,
                                           const int* rowoff = nullptr) {
  const int last = DIM - 1;
  const int pl = g.pd[last];
  int seg = 16;
  while (seg < pl) seg <<= 1;
  const int rows_per_tile = DIM == 2 ? g.pd[0] : g.pd[0] * g.pd[1];
  const int col = threadIdx.x & (seg - 1);
  const int step = blockDim.x / seg;
  if (col >= pl) return;
  const int mc = wrap_idx(o[last] + col, g.nf[last]);
  if (rowoff) {
    for (int cc = 0; cc < nc; ++cc) {
      const float2* src = fine + (int64_t)(c0 + cc) * g.G + mc;
      float2* dst = tile + cc * rows_per_tile * pl + col;
      for (int r = threadIdx.x / seg; r < rows_per_tile; r += step) dst[r * pl] = src[rowoff[r]];
    }
    return;
  }
  const int nrows = nc * rows_per_tile;
  for (int r = threadIdx.x / seg; r < nrows; r += step) {
    const int cc = r / rows_per_tile;
    const int rr = r - cc * rows_per_tile;
    int64_t rowbase;
    if (DIM == 2) {
      rowbase = (int64_t)wrap_idx(o[0] + rr, g.nf[0]) * g.nf[1];
    } else {
      const int i1 = rr % g.pd[1];
      const int i0 = rr / g.pd[1];
      rowbase = ((int64_t)wrap_idx(o[0] + i0, g.nf[0]) * g.nf[1] + wrap_idx(o[1] + i1, g.nf[1])) *
                g.nf[2];
    }
    tile[(int64_t)r * pl + col] = fine[(int64_t)(c0 + cc) * g.G + rowbase + mc];
  }
}

// Asynchronous global -> shared copies of one tile (cp.async, 8 bytes per
// cell), with the same row / column split as load_tiles.
__device__ __forceinline__ void cp_async8(float2* dst, const float2* src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int DIM>
__device__ __forceinline__ void load_tile_async(float2* tile, const float2* __restrict__ fine,
                                                const Geom& g, const int* o, const int* rowoff) {
  const int last = DIM - 1;
  const int pl = g.pd[last];
  int seg = 16;
  while (seg < pl) seg <<= 1;
  const int nrows = DIM == 2 ? g.pd[0] : g.pd[0] * g.pd[1];
  const int col = threadIdx.x & (seg - 1);
  if (col >= pl) return;
  const int step = blockDim.x / seg;
  const int mc = wrap_idx(o[last] + col, g.nf[last]);
  if (rowoff) {
    for (int r = threadIdx.x / seg; r < nrows; r += step)
      cp_async8(tile + r * pl + col, fine + rowoff[r] + mc);
    return;
  }
  for (int r = threadIdx.x / seg; r < nrows; r += step) {
    int64_t rowbase;
    if (DIM == 2) {
      rowbase = (int64_t)wrap_idx(o[0] + r, g.nf[0]) * g.nf[1];
    } else {
      const int i1 = r % g.pd[1];
      const int i0 = r / g.pd[1];
      rowbase = ((int64_t)wrap_idx(o[0] + i0, g.nf[0]) * g.nf[1] + wrap_idx(o[1] + i1, g.nf[1])) *
                g.nf[2];
    }
    cp_async8(tile + r * pl + col, fine + rowbase + mc);
  }
}

// ---------------------------------------------------------------------------
// Interpolation
// ---------------------------------------------------------------------------
// Footprint sum of one sample over the staged tiles of CG transforms.  The
// (re, im) sums are carried as pairs by two-wide FMAs.
template <int DIM, int W, int CG>
__device__ __forceinline__ void interp_footprint(const float2* cur, const Geom& g, int T,
                                                 const float* w0, const float* w1, const float* w2,
                                                 int l0, int l1, int l2, float* ar, float* ai) {
  constexpr int WM = WidthTraits<W>::WM;
  const int WL = W > 0 ? W : g.w;
  float2 acc[CG];
GBN_UNROLL
  for (int cc = 0; cc < CG; ++cc) acc[cc] = make_float2(0.f, 0.f);
  const float* wl = DIM == 2 ? w1 : w2;  // weights of the last axis
  float2 wp[WM];
GBN_UNROLL
  for (int t = 0; t < WM; ++t) wp[t] = make_float2(wl[t], wl[t]);
  if (DIM == 2) {
GBN_UNROLL
    for (int t0 = 0; t0 < WL; ++t0) {
      const float2* row = cur + (l0 + t0) * g.pd[1] + l1;
      const float2 wx = make_float2(w0[t0], w0[t0]);
GBN_UNROLL
      for (int cc = 0; cc < CG; ++cc) {
        float2 sv = make_float2(0.f, 0.f);
GBN_UNROLL
        for (int t1 = 0; t1 < WL; ++t1) sv = __ffma2_rn(wp[t1], row[cc * T + t1], sv);
        acc[cc] = __ffma2_rn(wx, sv, acc[cc]);
      }
    }
  } else {
GBN_UNROLL
    for (int t0 = 0; t0 < WL; ++t0) {
GBN_UNROLL
      for (int t1 = 0; t1 < WL; ++t1) {
        const float wy = w0[t0] * w1[t1];
        const float2 wyp = make_float2(wy, wy);
        const float2* row = cur + ((l0 + t0) * g.pd[1] + (l1 + t1)) * g.pd[2] + l2;
GBN_UNROLL
        for (int cc = 0; cc < CG; ++cc) {
          float2 sv = make_float2(0.f, 0.f);
GBN_UNROLL
          for (int t2 = 0; t2 < WL; ++t2) sv = __ffma2_rn(wp[t2], row[cc * T + t2], sv);
          acc[cc] = __ffma2_rn(wyp, sv, acc[cc]);
        }
      }
    }
  }
GBN_UNROLL
  for (int cc = 0; cc < CG; ++cc) {
    ar[cc] = acc[cc].x;
    ai[cc] = acc[cc].y;
  }
}

// Interp epilogue of one sample (original index j) for transforms c0 .. c0+nc-1.
template <int CG>
__device__ __forceinline__ void interp_store(const InterpArgs& a, int j, int c0, int nc,
                                             const float* ar, const float* ai) {
  if (a.mode == INTERP_PIPE) {
    // single transform: w_j <- w_j / |scale * v_j|
    float2 cur = a.out[j];
    float mag = a.scale * sqrtf(ar[0] * ar[0] + ai[0] * ai[0]);
    a.out[j] = make_float2(cur.x / mag, cur.y / mag);
    return;
  }
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

// One CTA per subproblem.  When the subproblem has at most one sample per
// thread, each thread evaluates its sample's kernel weights once and keeps
// them in registers for every transform pass; larger subproblems evaluate
// them per pass.
template <int DIM, int W, int CG>
__device__ __forceinline__ void interp_body(const InterpArgs& a, const int sub) {
  constexpr int WM = WidthTraits<W>::WM;
  extern __shared__ float2 tile[];
  const Geom& g = a.g;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<DIM>(g, b, o);
  const int T = g.tile;

  __shared__ int s_rowoff[kMaxTileRows];
  const int* rowoff = tile_rows_init<DIM>(g, o, s_rowoff);

  const bool cached = cnt <= (int)blockDim.x;
  float cw0[WM], cw1[WM], cw2[WM];
  int cl0 = 0, cl1 = 0, cl2 = 0, cj = -1;
  if (cached) {
    // Every footprint load of a lane is its sample's tile origin plus an
    // offset common to all lanes, so the bank conflicts of all w^d loads are
    // fixed by the origins: a 64-bit load is served per half-warp, and lanes
    // whose origins differ by a non-zero multiple of 16 cells (a float2 spans
    // two of the 32 banks) are serialised, while lanes on the same cell share
    // one broadcast.  The samples are sorted by (origin mod 16, origin) and
    // the runs of equal origins are dealt round-robin to the half-warps; in
    // a model of the 3D kooshball this takes the wavefronts per half-warp
    // load from 2.0 (sort order) to 1.29 (ideal 1).
    __shared__ int s_hist[16];
    __shared__ int s_slot[GBN_THREADS];
    __shared__ int s_key[GBN_THREADS];   // origin cell, by residue bucket
    __shared__ int s_who[GBN_THREADS];   // sample index, by residue bucket
    if (threadIdx.x < 16) s_hist[threadIdx.x] = 0;
    s_slot[threadIdx.x] = -1;
    __syncthreads();
    int r = 0, rank = 0, base = 0;
    if ((int)threadIdx.x < cnt) {
      const int pos = p0 + threadIdx.x;
      const int l0 = (int)ceilf(a.s.u[0][pos] - g.halfw) - o[0];
      const int l1 = (int)ceilf(a.s.u[1][pos] - g.halfw) - o[1];
      base = l0 * g.pd[1] + l1;
      if (DIM == 3) base = base * g.pd[2] + (int)ceilf(a.s.u[2][pos] - g.halfw) - o[2];
      r = base & 15;
      rank = atomicAdd(&s_hist[r], 1);
    }
    __syncthreads();
    int boff = 0, bcnt = 0;
    if ((int)threadIdx.x < cnt) {
      for (int q = 0; q < r; ++q) boff += s_hist[q];
      bcnt = s_hist[r];
      s_key[boff + rank] = base;
      s_who[boff + rank] = threadIdx.x;
    }
    __syncthreads();
    int sp = 0;
    if ((int)threadIdx.x < cnt) {  // rank by (origin, index) inside the bucket
      sp = boff;
      for (int q = boff; q < boff + bcnt; ++q) {
        const int kq = s_key[q], wq = s_who[q];
        sp += kq < base || (kq == base && wq < (int)threadIdx.x);
      }
    }
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      s_key[sp] = base;
      s_who[sp] = threadIdx.x;
    }
    __syncthreads();
    // Run r goes to half-warp r mod nh after the runs dealt there before it;
    // lanes past 16 move to the free lanes of other half-warps (prefix sums
    // of the overflow and free counts).  Everything is parallel over the
    // CTA; in the model it keeps 98 % of the gain of a sequential deal that
    // skips full half-warps.
    __shared__ int s_rpos[GBN_THREADS];  // lane of run r's first sample in its half-warp
    __shared__ int s_wcnt[GBN_THREADS / 32];
    __shared__ int s_hfill[16], s_fpre[17], s_opre[17];
    int* const s_rstart = s_key;  // run start positions (written after the key reads)
    const int nh = (cnt + 15) >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int p = threadIdx.x;
    const bool in = p < cnt;
    const bool st = in && (p == 0 || s_key[p] != s_key[p - 1]);
    const unsigned bal = __ballot_sync(0xffffffffu, st);
    if (lane == 0) s_wcnt[warp] = __popc(bal);
    __syncthreads();
    int wpre = 0, nruns = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      if (q < warp) wpre += s_wcnt[q];
      nruns += s_wcnt[q];
    }
    const int run = wpre + __popc(bal & ((2u << lane) - 1u)) - 1;  // starts at or before p
    if (st) s_rstart[run] = p;
    __syncthreads();
    if ((int)threadIdx.x < nh) {
      int acc = 0;
      for (int rr = threadIdx.x; rr < nruns; rr += nh) {
        s_rpos[rr] = acc;
        acc += (rr + 1 < nruns ? s_rstart[rr + 1] : cnt) - s_rstart[rr];
      }
      s_hfill[threadIdx.x] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int f = 0, ov = 0;
      for (int h = 0; h < nh; ++h) {
        s_fpre[h] = f;
        s_opre[h] = ov;
        const int fl = s_hfill[h];
        f += fl < 16 ? 16 - fl : 0;
        ov += fl > 16 ? fl - 16 : 0;
      }
      s_fpre[nh] = f;
      s_opre[nh] = ov;
    }
    __syncthreads();
    if (in) {
      const int h = run % nh;
      const int ln = s_rpos[run] + (p - s_rstart[run]);
      if (ln < 16) {
        s_slot[h * 16 + ln] = s_who[p];
      } else {  // k-th overflow sample -> k-th free lane
        const int k = s_opre[h] + ln - 16;
        int hh = 0;
        while (hh + 1 < nh && s_fpre[hh + 1] <= k) ++hh;
        s_slot[hh * 16 + s_hfill[hh] + (k - s_fpre[hh])] = s_who[p];
      }
    }
    __syncthreads();
    const int sidx = s_slot[threadIdx.x];
    if (sidx >= 0) {
      const int pos = p0 + sidx;
      cl0 = weights_rt<W>(a.s.u[0][pos], g, cw0) - o[0];
      cl1 = weights_rt<W>(a.s.u[1][pos], g, cw1) - o[1];
      if (DIM == 3) cl2 = weights_rt<W>(a.s.u[2][pos], g, cw2) - o[2];
      cj = a.s.perm[pos];
    }
  }
  __syncthreads();

  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    if (rowoff) {
      // asynchronous copies: every cell of the tile in flight at once
      for (int cc = 0; cc < nc; ++cc)
        load_tile_async<DIM>(tile + cc * T, a.fine + (int64_t)(c0 + cc) * g.G, g, o, rowoff);
      cp_async_commit();
      cp_async_wait<0>();
    } else {
      load_tiles<DIM>(tile, a.fine, g, o, c0, nc);
    }
    __syncthreads();
    float ar[CG], ai[CG];
    if (cached) {
      if (cj >= 0) {
        interp_footprint<DIM, W, CG>(tile, g, T, cw0, cw1, cw2, cl0, cl1, cl2, ar, ai);
        interp_store<CG>(a, cj, c0, nc, ar, ai);
      }
    } else {
      for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
        const int pos = p0 + s;
        float w0[WM], w1[WM], w2[WM];
        int l0 = weights_rt<W>(a.s.u[0][pos], g, w0) - o[0];
        int l1 = weights_rt<W>(a.s.u[1][pos], g, w1) - o[1];
        int l2 = 0;
        if (DIM == 3) l2 = weights_rt<W>(a.s.u[2][pos], g, w2) - o[2];
        interp_footprint<DIM, W, CG>(tile, g, T, w0, w1, w2, l0, l1, l2, ar, ai);
        interp_store<CG>(a, a.s.perm[pos], c0, nc, ar, ai);
      }
    }
    __syncthreads();
  }
}

// 128-thread CTAs; at least 5 resident per SM keeps registers <= 96 a thread
constexpr int kInterpThreads = 128;

template <int DIM, int W, int CG>
__global__ void __launch_bounds__(kInterpThreads, 5)
interp_kernel(InterpArgs a) {
  interp_body<DIM, W, CG>(a, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Interpolation with double-buffered tiles: each thread keeps the weights of
// its (at most S) samples in registers for all transforms, and the tile of
// transform c+1 streams into shared memory with cp.async while transform c
// is interpolated.  maxsub <= S * GBN_THREADS.
// ---------------------------------------------------------------------------
template <int DIM, int W, int S>
__global__ void __launch_bounds__(GBN_THREADS)
interp_db_kernel(InterpArgs a) {
  extern __shared__ float2 tiles[];
  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<DIM>(g, b, o);
  const int T = g.tile;
  float w0[S][W], w1[S][W], w2[S][W];
  int l0[S], l1[S], l2[S], jj[S];
#pragma unroll
  for (int q = 0; q < S; ++q) {
    const int s = threadIdx.x + q * GBN_THREADS;
    jj[q] = -1;
    l0[q] = l1[q] = l2[q] = 0;
    if (s < cnt) {
      const int pos = p0 + s;
      jj[q] = a.s.perm[pos];
      l0[q] = weights_rt<W>(a.s.u[0][pos], g, w0[q]) - o[0];
      l1[q] = weights_rt<W>(a.s.u[1][pos], g, w1[q]) - o[1];
      if (DIM == 3) l2[q] = weights_rt<W>(a.s.u[2][pos], g, w2[q]) - o[2];
    }
  }
  __shared__ int s_rowoff[kMaxTileRows];
  const int* rowoff = tile_rows_init<DIM>(g, o, s_rowoff);
  __syncthreads();
  load_tile_async<DIM>(tiles, a.fine, g, o, rowoff);
  cp_async_commit();
  for (int c = 0; c < a.ntr; ++c) {
    if (c + 1 < a.ntr) {
      load_tile_async<DIM>(tiles + ((c + 1) & 1) * T, a.fine + (int64_t)(c + 1) * g.G, g, o, rowoff);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float2* tile = tiles + (c & 1) * T;
#pragma unroll
    for (int q = 0; q < S; ++q) {
      if (jj[q] < 0) continue;
      float ar = 0.f, ai = 0.f;
      if (DIM == 2) {
#pragma unroll
        for (int t0 = 0; t0 < W; ++t0) {
          const float2* row = tile + (l0[q] + t0) * g.pd[1] + l1[q];
          float sr = 0.f, si = 0.f;
#pragma unroll
          for (int t1 = 0; t1 < W; ++t1) {
            const float2 v = row[t1];
            sr = fmaf(w1[q][t1], v.x, sr);
            si = fmaf(w1[q][t1], v.y, si);
          }
          ar = fmaf(w0[q][t0], sr, ar);
          ai = fmaf(w0[q][t0], si, ai);
        }
      } else {
#pragma unroll
        for (int t0 = 0; t0 < W; ++t0) {
#pragma unroll
          for (int t1 = 0; t1 < W; ++t1) {
            const float2* row = tile + ((l0[q] + t0) * g.pd[1] + (l1[q] + t1)) * g.pd[2] + l2[q];
            float sr = 0.f, si = 0.f;
#pragma unroll
            for (int t2 = 0; t2 < W; ++t2) {
              const float2 v = row[t2];
              sr = fmaf(w2[q][t2], v.x, sr);
              si = fmaf(w2[q][t2], v.y, si);
            }
            const float k = w0[q][t0] * w1[q][t1];
            ar = fmaf(k, sr, ar);
            ai = fmaf(k, si, ai);
          }
        }
      }
      const int j = jj[q];
      if (a.mode == INTERP_PIPE) {
        float2 cur = a.out[j];
        float mag = a.scale * sqrtf(ar * ar + ai * ai);
        a.out[j] = make_float2(cur.x / mag, cur.y / mag);
      } else {
        const int64_t oi = (int64_t)c * a.s.M + j;
        float2 r = make_float2(a.scale * ar, a.scale * ai);
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
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Interpolation straight from the fine grid (no shared-memory tile): thread
// per sorted sample, weights evaluated once and reused by every transform,
// footprint cells read through L1 (consecutive sorted samples of a warp read
// overlapping cells).
// ---------------------------------------------------------------------------
template <int DIM, int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS, 4)
interp_gm_kernel(InterpArgs a) {
  constexpr int WM = WidthTraits<W>::WM;
  const Geom& g = a.g;
  const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= a.s.M) return;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;
  const int j = a.s.perm[pos];
  float w0[WM], w1[WM], w2[WM];
  int m0[WM], m1[WM], m2[WM];
  int i0 = weights_rt<W>(a.s.u[0][pos], g, w0);
  int i1 = weights_rt<W>(a.s.u[1][pos], g, w1);
  int i2 = 0;
  if (DIM == 3) i2 = weights_rt<W>(a.s.u[2][pos], g, w2);
GBN_UNROLL
  for (int t = 0; t < WL; ++t) {
    m0[t] = wrap_idx(i0 + t, g.nf[0]);
    m1[t] = wrap_idx(i1 + t, g.nf[1]);
    if (DIM == 3) m2[t] = wrap_idx(i2 + t, g.nf[2]);
  }
  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    float ar[CG], ai[CG];
#pragma unroll
    for (int cc = 0; cc < CG; ++cc) ar[cc] = ai[cc] = 0.f;
#pragma unroll 1
    for (int t0 = 0; t0 < WL; ++t0) {
#pragma unroll 1
      for (int t1 = 0; t1 < WL; ++t1) {
        const int64_t r = (int64_t)m0[t0] * g.nf[1] + m1[t1];
        const float k = w0[t0] * w1[t1];
#pragma unroll
        for (int cc = 0; cc < CG; ++cc) {
          if (cc < nc) {
            const float2* base = a.fine + (int64_t)(c0 + cc) * g.G;
            float sr = 0.f, si = 0.f;
            if (DIM == 2) {
              const float2 v = __ldg(base + r);
              sr = v.x;
              si = v.y;
            } else {
              const float2* row = base + r * g.nf[2];
GBN_UNROLL
              for (int t2 = 0; t2 < WL; ++t2) {
                const float2 v = __ldg(row + m2[t2]);
                sr = fmaf(w2[t2], v.x, sr);
                si = fmaf(w2[t2], v.y, si);
              }
            }
            ar[cc] = fmaf(k, sr, ar[cc]);
            ai[cc] = fmaf(k, si, ai[cc]);
          }
        }
      }
    }
#pragma unroll
    for (int cc = 0; cc < CG; ++cc) {
      if (cc >= nc) continue;
      if (a.mode == INTERP_PIPE) {
        float2 cur = a.out[j];
        float mag = a.scale * sqrtf(ar[cc] * ar[cc] + ai[cc] * ai[cc]);
        a.out[j] = make_float2(cur.x / mag, cur.y / mag);
      } else {
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

// ---------------------------------------------------------------------------
// Warp-cooperative interpolation straight from the fine grid (w = 7).
// Eight lanes serve one sample: lane l reads footprint cells along the last
// axis at offset l (7 contiguous float2 per row, i.e. 56 coalesced bytes per
// sample), so one warp instruction loads the rows of four samples in a few
// sectors; partial sums are combined with three butterfly shuffles.  The
// kernel weights of a sample stay in registers for every transform.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void interp_wc_body(const InterpArgs& a, const int64_t warp_id) {
  constexpr int W = 7;
  const Geom& g = a.g;
  const int lane = threadIdx.x & 31;
  const int sub = lane >> 3, l = lane & 7;
  const int64_t pos = warp_id * 4 + sub;
  const bool valid = pos < a.s.M;
  const bool act = valid && l < W;
  float w0[W], w1[W];
  float wl = 0.f;
  int rb[W];  // row index m0 * nf1 (< 2^31: fine grids are capped at 2^31 cells)
  int m1[W];
  int ml = 0, j = 0;
  if (valid) {
    j = a.s.perm[pos];
    const float u0 = a.s.u[0][pos], u1 = a.s.u[1][pos];
    const int i0 = weights_rt<W>(u0, g, w0);
    if (DIM == 2) {
      const float s1 = u1 - g.halfw;
      const int i1 = (int)ceilf(s1);
      wl = l < W ? es_eval((float)(i1 + l) - u1, g.beta, g.inv_halfw) : 0.f;
      ml = wrap_idx(i1 + l, g.nf[1]);
#pragma unroll
      for (int t = 0; t < W; ++t) rb[t] = wrap_idx(i0 + t, g.nf[0]) * g.nf[1];
    } else {
      const int i1 = weights_rt<W>(u1, g, w1);
      const float u2 = a.s.u[2][pos];
      const int i2 = (int)ceilf(u2 - g.halfw);
      wl = l < W ? es_eval((float)(i2 + l) - u2, g.beta, g.inv_halfw) : 0.f;
      ml = wrap_idx(i2 + l, g.nf[2]);
#pragma unroll
      for (int t = 0; t < W; ++t) {
        rb[t] = wrap_idx(i0 + t, g.nf[0]) * g.nf[1];
        m1[t] = wrap_idx(i1 + t, g.nf[1]);
      }
    }
  }
  for (int c = 0; c < a.ntr; ++c) {
    const float2* base = a.fine + (int64_t)c * g.G;
    float ar = 0.f, ai = 0.f;
    if (act) {
      // (re, im) sums carried as pairs by two-wide FMAs
      float2 acc = make_float2(0.f, 0.f);
      if (DIM == 2) {
#pragma unroll
        for (int t0 = 0; t0 < W; ++t0)
          acc = __ffma2_rn(make_float2(w0[t0], w0[t0]), __ldg(base + rb[t0] + ml), acc);
      } else {
#pragma unroll
        for (int t0 = 0; t0 < W; ++t0) {
          float2 sv = make_float2(0.f, 0.f);
#pragma unroll
          for (int t1 = 0; t1 < W; ++t1)
            sv = __ffma2_rn(make_float2(w1[t1], w1[t1]),
                            __ldg(base + (int64_t)(rb[t0] + m1[t1]) * g.nf[2] + ml), sv);
          acc = __ffma2_rn(make_float2(w0[t0], w0[t0]), sv, acc);
        }
      }
      ar = acc.x * wl;
      ai = acc.y * wl;
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o);
      ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (valid && l == 0) {
      if (a.mode == INTERP_PIPE) {
        float2 cur = a.out[j];
        float mag = a.scale * sqrtf(ar * ar + ai * ai);
        a.out[j] = make_float2(cur.x / mag, cur.y / mag);
      } else {
        const int64_t oi = (int64_t)c * a.s.M + j;
        float2 r = make_float2(a.scale * ar, a.scale * ai);
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

template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS, 4)
interp_wc_kernel(InterpArgs a) {
  interp_wc_body<DIM>(a, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

// ---------------------------------------------------------------------------
// Tile + warp-cooperative interpolation (3D, w = 7).  Per subproblem the
// samples' local footprint origins and weights are computed once into shared
// memory; then for each transform the padded tile is staged in shared memory
// and every warp serves groups of four samples with eight lanes each (lane l
// reads the 7-cell rows at offset l: conflict-free, 56 contiguous bytes per
// sample), reducing with butterfly shuffles.  Sparse bins keep all warps
// busy because work is spread by sample groups, not by threads.
// ---------------------------------------------------------------------------
constexpr int kTwcMaxSub = 256;

static __global__ void __launch_bounds__(GBN_THREADS)
interp_twc3d_kernel(InterpArgs a) {
  constexpr int W = 7;
  extern __shared__ float2 tile[];
  __shared__ float s_w0[kTwcMaxSub][8], s_w1[kTwcMaxSub][8], s_w2[kTwcMaxSub][8];
  __shared__ int s_off[kTwcMaxSub], s_j[kTwcMaxSub];
  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<3>(g, b, o);
  for (int s = threadIdx.x; s < cnt; s += blockDim.x) {
    const int pos = p0 + s;
    float wt[W];
    const int l0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o[0];
#pragma unroll
    for (int t = 0; t < 8; ++t) s_w0[s][t] = t < W ? wt[t] : 0.f;
    const int l1 = weights_rt<W>(a.s.u[1][pos], g, wt) - o[1];
#pragma unroll
    for (int t = 0; t < 8; ++t) s_w1[s][t] = t < W ? wt[t] : 0.f;
    const int l2 = weights_rt<W>(a.s.u[2][pos], g, wt) - o[2];
#pragma unroll
    for (int t = 0; t < 8; ++t) s_w2[s][t] = t < W ? wt[t] : 0.f;
    s_off[s] = (l0 * g.pd[1] + l1) * g.pd[2] + l2;
    s_j[s] = a.s.perm[pos];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int q = lane >> 3, l = lane & 7;
  const int ngroups = (cnt + 3) >> 2;
  const int pd12 = g.pd[1] * g.pd[2];
  __shared__ int s_rowoff[kMaxTileRows];
  const int* rowoff = tile_rows_init<3>(g, o, s_rowoff);
  for (int c = 0; c < a.ntr; ++c) {
    __syncthreads();  // previous tile consumed, sample and row tables written
    load_tiles<3>(tile, a.fine, g, o, c, 1, rowoff);
    __syncthreads();
    for (int gi = warp; gi < ngroups; gi += (GBN_THREADS / 32)) {
      const int s = gi * 4 + q;
      const bool valid = s < cnt;
      float ar = 0.f, ai = 0.f;
      if (valid && l < W) {
        const float2* t = tile + s_off[s] + l;
        const float wl = s_w2[s][l];
#pragma unroll
        for (int t0 = 0; t0 < W; ++t0) {
          float sr = 0.f, si = 0.f;
#pragma unroll
          for (int t1 = 0; t1 < W; ++t1) {
            const float2 v = t[t0 * pd12 + t1 * g.pd[2]];
            const float w1 = s_w1[s][t1];
            sr = fmaf(w1, v.x, sr);
            si = fmaf(w1, v.y, si);
          }
          const float w0 = s_w0[s][t0];
          ar = fmaf(w0, sr, ar);
          ai = fmaf(w0, si, ai);
        }
        ar *= wl;
        ai *= wl;
      }
#pragma unroll
      for (int m = 1; m < 8; m <<= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, m);
        ai += __shfl_xor_sync(0xffffffffu, ai, m);
      }
      if (valid && l == 0) {
        const int j = s_j[s];
        if (a.mode == INTERP_PIPE) {
          float2 cur = a.out[j];
          float mag = a.scale * sqrtf(ar * ar + ai * ai);
          a.out[j] = make_float2(cur.x / mag, cur.y / mag);
        } else {
          const int64_t oi = (int64_t)c * a.s.M + j;
          float2 r = make_float2(a.scale * ar, a.scale * ai);
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
}

// ---------------------------------------------------------------------------
// Spreading, 3D "row ownership" kernel (no shared-memory atomics).
//
// Shared-memory float atomics are compare-and-swap loops on this GPU, and the
// dense k-space centre of radial trajectories makes them contend, so the 3D
// spreader is output-driven inside each bin tile: thread t owns one row
// (i0, i1) of the padded tile (P0 x P1 <= 16 x 16 rows, all P2 <= 16 cells
// along axis 2) and keeps its cells in registers.  Samples of the subproblem
// are staged in shared memory in batches of 256 (local footprint origin, the
// axis-0/1 weights and a dense 16-cell axis-2 weight row); every thread walks
// the batch and accumulates the samples whose footprint covers its row.
// Each warp owns two rows of i0, so most warps skip a sample uniformly.
// The tile is then added to the fine grid with float2 global atomics (tiles
// of neighbouring bins overlap by w cells).
// ---------------------------------------------------------------------------
constexpr int kRowBatch = 256;

template <int W, int CG>
__device__ __forceinline__ void spread_rows3d_body(const SpreadArgs& a, const int sub) {
  constexpr int WM = W > 0 ? W : 8;
  __shared__ int s_a0[kRowBatch], s_a1[kRowBatch];
  __shared__ float s_w0[kRowBatch][8], s_w1[kRowBatch][8];
  __shared__ __align__(16) float s_w2[kRowBatch][16];
  __shared__ float2 s_c[CG][kRowBatch];
  const Geom& g = a.g;
  const int b = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = a.s.sub_count[sub];
  int o[3];
  bin_origin<3>(g, b, o);
  const int w = W > 0 ? W : g.w;
  // warp w owns rows i0 = 2w, 2w+1 (16 lanes each along i1): a footprint of
  // 7 consecutive i0 rows touches 4 warps
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i0 = 2 * warp + (lane >> 4);
  const int i1 = lane & 15;
  const bool own = i0 < g.pd[0] && i1 < g.pd[1];

  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    float ar[CG][16], ai[CG][16];
#pragma unroll
    for (int cc = 0; cc < CG; ++cc)
#pragma unroll
      for (int z = 0; z < 16; ++z) ar[cc][z] = ai[cc][z] = 0.f;

    for (int q0 = 0; q0 < cnt; q0 += kRowBatch) {
      const int nb = imin(kRowBatch, cnt - q0);
      if ((int)threadIdx.x < nb) {
        const int t = threadIdx.x;
        const int pos = p0 + q0 + t;
        const int j = a.s.perm[pos];
        float wt[WidthTraits<W>::WM];
        s_a0[t] = weights_rt<W>(a.s.u[0][pos], g, wt) - o[0];
#pragma unroll
        for (int k = 0; k < 8; ++k) s_w0[t][k] = k < w ? wt[k] : 0.f;
        s_a1[t] = weights_rt<W>(a.s.u[1][pos], g, wt) - o[1];
#pragma unroll
        for (int k = 0; k < 8; ++k) s_w1[t][k] = k < w ? wt[k] : 0.f;
        int a2 = weights_rt<W>(a.s.u[2][pos], g, wt) - o[2];
#pragma unroll
        for (int z = 0; z < 16; ++z) {
          int k = z - a2;
          float v = 0.f;
#pragma unroll
          for (int kk = 0; kk < WidthTraits<W>::WM; ++kk)
            if (kk == k && kk < w) v = wt[kk];
          s_w2[t][z] = v;
        }
        float dj = a.scale;
        if (a.density) dj *= a.density[j];
#pragma unroll
        for (int cc = 0; cc < CG; ++cc) {
          float2 x = cc < nc ? a.in[(int64_t)(c0 + cc) * a.s.M + j] : make_float2(0.f, 0.f);
          s_c[cc][t] = make_float2(x.x * dj, x.y * dj);
        }
      }
      __syncthreads();
      if (own) {
        for (int s = 0; s < nb; ++s) {
          const unsigned r0 = (unsigned)(i0 - s_a0[s]);
          const unsigned r1 = (unsigned)(i1 - s_a1[s]);
          if (r0 < (unsigned)w && r1 < (unsigned)w) {
            const float k = s_w0[s][r0] * s_w1[s][r1];
            float wz[16];
            const float4* w4 = reinterpret_cast<const float4*>(s_w2[s]);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              float4 v = w4[q];
              wz[4 * q] = v.x;
              wz[4 * q + 1] = v.y;
              wz[4 * q + 2] = v.z;
              wz[4 * q + 3] = v.w;
            }
#pragma unroll
            for (int cc = 0; cc < CG; ++cc) {
              const float2 c = s_c[cc][s];
              const float vr = k * c.x, vi = k * c.y;
#pragma unroll
              for (int z = 0; z < 16; ++z) {
                ar[cc][z] = fmaf(vr, wz[z], ar[cc][z]);
                ai[cc][z] = fmaf(vi, wz[z], ai[cc][z]);
              }
            }
          }
        }
      }
      __syncthreads();
    }
    if (own) {
      const int m0 = wrap_idx(o[0] + i0, g.nf[0]);
      const int m1 = wrap_idx(o[1] + i1, g.nf[1]);
      const int64_t rowbase = ((int64_t)m0 * g.nf[1] + m1) * g.nf[2];
#pragma unroll
      for (int cc = 0; cc < CG; ++cc) {
        if (cc < nc) {
          float2* dst = a.fine + (int64_t)(c0 + cc) * g.G + rowbase;
#pragma unroll
          for (int z = 0; z < 16; ++z) {
            if (z < g.pd[2] && (ar[cc][z] != 0.f || ai[cc][z] != 0.f))
              atomicAdd(dst + wrap_idx(o[2] + z, g.nf[2]), make_float2(ar[cc][z], ai[cc][z]));
          }
        }
      }
    }
  }
}

template <int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS, 2)
spread_rows3d_kernel(SpreadArgs a) {
  spread_rows3d_body<W, CG>(a, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Spreading, 3D column-streaming kernel (widths w <= 7).
//
// With the sort keyed on (x bin, y bin, z cell), the samples of one column
// of bins (bs0 x bs1 cells across, the whole z extent) arrive in z order.  A
// CTA takes a chunk of <= kStreamBatch consecutive samples of one column.
// Thread t owns row (i0, i1) of the column's padded (bs0 + w) x (bs1 + w)
// cross-section (two i0 rows per warp, as in the row kernel) and keeps a
// window of 8 z cells in registers: cell z lives in slot z & 7.  A sample in
// z cell f covers cells [f - w/2, f - w/2 + 7], so the window is anchored at
// zb = f - floor(w/2); when the samples reach a later anchor, the slots whose
// cells fall out of the window are added to the fine grid (float2 global
// atomics) and cleared.  Each sample's z weights are staged already rotated
// into slot order, so the accumulation indexes registers statically.
// Against the bin-tile row kernel each sample updates 8 register cells per
// coil instead of 16, the kernel weights are evaluated once per chunk for all
// coils, and a fine cell is flushed once per chunk rather than once per
// overlapping tile.
// ---------------------------------------------------------------------------
constexpr int kStreamBatch = kStreamChunk;

// dynamic shared memory of the streaming kernel for CG coils per pass
__host__ __device__ constexpr size_t stream_smem_bytes(int cg) {
  return (size_t)kStreamBatch * (sizeof(unsigned) + 24 * sizeof(float)) +
         (size_t)cg * kStreamBatch * sizeof(float2);
}

__device__ __forceinline__ int wrap_near(int i, int n) {
  // one period of correction covers every window cell when n >= 8; the
  // modulo keeps tiny grids correct
  int m = i < 0 ? i + n : (i >= n ? i - n : i);
  return (unsigned)m < (unsigned)n ? m : wrap_idx(i, n);
}

// Adds window slot K (fine cell z) of every coil to the fine grid and clears it.
template <int K, int CG>
__device__ __forceinline__ void stream_flush(float (&ar)[CG][8], float (&ai)[CG][8], bool own,
                                             float2* fb, int z, int nf2, int G, int nc) {
  if (own) {
    float2* dst = fb + wrap_near(z, nf2);
#pragma unroll
    for (int cc = 0; cc < CG; ++cc) {
      if (cc < nc && (ar[cc][K] != 0.f || ai[cc][K] != 0.f))
        atomicAdd(dst, make_float2(ar[cc][K], ai[cc][K]));
      dst += G;
    }
  }
#pragma unroll
  for (int cc = 0; cc < CG; ++cc) ar[cc][K] = ai[cc][K] = 0.f;
}

// Flushes the window slots set in `mask` (slot k holds cell zb + ((k - zb) & 7)).
template <int CG>
__device__ __forceinline__ void stream_flush_mask(unsigned mask, int zb, float (&ar)[CG][8],
                                                  float (&ai)[CG][8], bool own, float2* fb,
                                                  int nf2, int G, int nc) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (mask & (1u << k)) {
      const int z = zb + ((k - zb) & 7);
      if (k == 0) stream_flush<0, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 1) stream_flush<1, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 2) stream_flush<2, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 3) stream_flush<3, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 4) stream_flush<4, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 5) stream_flush<5, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 6) stream_flush<6, CG>(ar, ai, own, fb, z, nf2, G, nc);
      if (k == 7) stream_flush<7, CG>(ar, ai, own, fb, z, nf2, G, nc);
    }
  }
}

template <int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS, 2)
spread_stream3d_kernel(SpreadArgs a) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  float* s_w2 = reinterpret_cast<float*>(s_raw);           // [kStreamBatch][8], slot order
  float* s_w0 = s_w2 + kStreamBatch * 8;                    // [kStreamBatch][8]
  float* s_w1 = s_w0 + kStreamBatch * 8;                    // [kStreamBatch][8]
  float2* s_c = reinterpret_cast<float2*>(s_w1 + kStreamBatch * 8);  // [CG][kStreamBatch]
  // per sample: window anchor + 8 (bits 0-15), local row offsets a0, a1
  // (bits 16-19, 20-23), mask of the warps whose rows it covers (bits 24-31)
  unsigned* s_hd = reinterpret_cast<unsigned*>(s_c + CG * kStreamBatch);

  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int col = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = imin(a.s.sub_count[sub], kStreamBatch);
  const int w = W > 0 ? W : g.w;
  const int hw = w >> 1;
  const int o0 = (col / g.nb[1]) * g.bs[0] - hw;
  const int o1 = (col % g.nb[1]) * g.bs[1] - hw;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // warp w owns rows i0 = 2w, 2w+1 (16 lanes each along i1)
  const int i0 = 2 * warp + (lane >> 4);
  const int i1 = lane & 15;
  const bool own = i0 < g.pd[0] && i1 < g.pd[1];
  const int nf2 = g.nf[2];
  // fine grids hold < 2^31 cells
  const int G = (int)g.G;
  const int rowbase = own ? (wrap_idx(o0 + i0, g.nf[0]) * g.nf[1] + wrap_idx(o1 + i1, g.nf[1])) * nf2 : 0;

  // geometry of the chunk, once for every coil
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int pos = p0 + t;
    float wt[WidthTraits<W>::WM];
    const int a0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o0;  // 0 .. bs0
#pragma unroll
    for (int k = 0; k < 8; ++k) s_w0[t * 8 + k] = k < w ? wt[k] : 0.f;
    const int a1 = weights_rt<W>(a.s.u[1][pos], g, wt) - o1;  // 0 .. bs1
#pragma unroll
    for (int k = 0; k < 8; ++k) s_w1[t * 8 + k] = k < w ? wt[k] : 0.f;
    const float u2 = a.s.u[2][pos];
    const int zs = cell_of(u2, nf2) - hw;
    const int off = weights_rt<W>(u2, g, wt) - zs;  // 0 or 1
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int m = k - off;
      float v = 0.f;
#pragma unroll
      for (int kk = 0; kk < WidthTraits<W>::WM; ++kk)
        if (kk == m && kk < w) v = wt[kk];
      s_w2[t * 8 + ((zs + k) & 7)] = v;
    }
    unsigned wm = 0;
#pragma unroll
    for (int q = 0; q < GBN_THREADS / 32; ++q)
      if (a0 <= 2 * q + 1 && a0 + w > 2 * q) wm |= 1u << q;
    s_hd[t] = (unsigned)(zs + 8) | ((unsigned)a0 << 16) | ((unsigned)a1 << 20) | (wm << 24);
  }

  const unsigned mybit = 1u << (24 + warp);
  // blockIdx.y selects a group of gridDim.y-way split transform passes
  const int per_cta = ((a.ntr + CG - 1) / CG + gridDim.y - 1) / gridDim.y * CG;
  const int c_end = imin(a.ntr, (int)(blockIdx.y + 1) * per_cta);
  for (int c0 = blockIdx.y * per_cta; c0 < c_end; c0 += CG) {
    const int nc = imin(CG, c_end - c0);
    // strengths of this pass's coils
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
      const int j = a.s.perm[p0 + t];
      float dj = a.scale;
      if (a.density) dj *= a.density[j];
#pragma unroll
      for (int cc = 0; cc < CG; ++cc) {
        float2 x = cc < nc ? a.in[(int64_t)(c0 + cc) * a.s.M + j] : make_float2(0.f, 0.f);
        s_c[cc * kStreamBatch + t] = make_float2(x.x * dj, x.y * dj);
      }
    }
    __syncthreads();
    float ar[CG][8], ai[CG][8];
#pragma unroll
    for (int cc = 0; cc < CG; ++cc)
#pragma unroll
      for (int k = 0; k < 8; ++k) ar[cc][k] = ai[cc][k] = 0.f;
    float2* const fb = a.fine + (int64_t)c0 * g.G + rowbase;
    int zb = cnt > 0 ? (int)(s_hd[0] & 0xffffu) - 8 : 0;  // window: cells zb .. zb + 7

#pragma unroll 1
    for (int s = 0; s < cnt; ++s) {
      const unsigned hd = s_hd[s];
      const int zs = (int)(hd & 0xffffu) - 8;
      if (zs != zb) {  // the same for every thread: flush the cells that leave the window
        const int steps = imin(zs - zb, 8);
        const unsigned m = (1u << steps) - 1u, r = (unsigned)zb & 7u;
        stream_flush_mask<CG>(((m << r) | (m >> (8u - r))) & 0xffu, zb, ar, ai, own, fb, nf2, G, nc);
        zb = zs;
      }
      if (hd & mybit) {  // warp-uniform
        const unsigned r0 = (unsigned)(i0 - (int)((hd >> 16) & 15u));
        const unsigned r1 = (unsigned)(i1 - (int)((hd >> 20) & 15u));
        if (own && r0 < (unsigned)w && r1 < (unsigned)w) {
          const float kw = s_w0[s * 8 + r0] * s_w1[s * 8 + r1];
          const float4* w4 = reinterpret_cast<const float4*>(s_w2 + s * 8);
          const float4 wa = w4[0], wb = w4[1];
          const float wz[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
          for (int cc = 0; cc < CG; ++cc) {
            const float2 c = s_c[cc * kStreamBatch + s];
            const float vr = kw * c.x, vi = kw * c.y;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              ar[cc][k] = fmaf(vr, wz[k], ar[cc][k]);
              ai[cc][k] = fmaf(vi, wz[k], ai[cc][k]);
            }
          }
        }
      }
    }
    stream_flush_mask<CG>(0xffu, zb, ar, ai, own, fb, nf2, G, nc);
    __syncthreads();  // s_c is restaged by the next pass
  }
}

// The same for window accumulators held as (re, im) pairs.
template <int K, int CG>
__device__ __forceinline__ void stream_flush2(float2 (&acc)[CG][8], bool own, float2* fb, int z,
                                              int nf2, int G, int nc) {
  if (own) {
    float2* dst = fb + wrap_near(z, nf2);
#pragma unroll
    for (int cc = 0; cc < CG; ++cc) {
      if (cc < nc && (acc[cc][K].x != 0.f || acc[cc][K].y != 0.f)) atomicAdd(dst, acc[cc][K]);
      dst += G;
    }
  }
#pragma unroll
  for (int cc = 0; cc < CG; ++cc) acc[cc][K] = make_float2(0.f, 0.f);
}

template <int CG>
__device__ __forceinline__ void stream_flush_mask2(unsigned mask, int zb, float2 (&acc)[CG][8],
                                                   bool own, float2* fb, int nf2, int G, int nc) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if (mask & (1u << k)) {
      const int z = zb + ((k - zb) & 7);
      if (k == 0) stream_flush2<0, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 1) stream_flush2<1, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 2) stream_flush2<2, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 3) stream_flush2<3, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 4) stream_flush2<4, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 5) stream_flush2<5, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 6) stream_flush2<6, CG>(acc, own, fb, z, nf2, G, nc);
      if (k == 7) stream_flush2<7, CG>(acc, own, fb, z, nf2, G, nc);
    }
  }
}

// ---------------------------------------------------------------------------
// Spreading, 3D quadrant-streaming kernel (8 x 8 bins, widths w <= 7).
//
// The column-streaming kernel above gives every thread of a 256-thread CTA
// one row of the column's 15 x 15 cross-section, so a sample's 7 x 7
// footprint keeps 49 of 256 threads busy while all 8 warps step through it.
// Here the chunk of an 8 x 8 column is split by footprint origin into four
// 4 x 4 quadrants, one 128-thread CTA each: the CTA keeps the
// chunk's samples of its quadrant, in z order, and its threads own the rows
// of the quadrant's (4 + w) x (4 + w) cross-section (121 rows for w = 7), so
// a sample occupies about 3 of the 4 warps.  Quadrant cross-sections overlap
// by w rows, which the float2 flush atomics absorb.  The z window, rotated
// weights and flush rules are those of the column kernel.
// ---------------------------------------------------------------------------
constexpr int kQuadThreads = 128;
constexpr int kQuadRound = 256;  // samples staged at a time

__host__ __device__ constexpr size_t quad_smem_bytes(int cg) {
  return (size_t)kQuadRound * (sizeof(unsigned) + 24 * sizeof(float)) +
         (size_t)cg * kQuadRound * sizeof(float2) + (size_t)kStreamBatch * sizeof(short);
}

// PACKED: the window accumulators are (re, im) pairs updated by two-wide
// FP32 fused multiply-adds (one instruction per cell and coil).
template <int W, int CG, int MINB, bool PACKED = false>
__global__ void __launch_bounds__(kQuadThreads, MINB)
spread_quad3d_kernel(SpreadArgs a) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  float* s_w2 = reinterpret_cast<float*>(s_raw);           // [kQuadRound][8], slot order
  float* s_w0 = s_w2 + kQuadRound * 8;                      // [kQuadRound][8]
  float* s_w1 = s_w0 + kQuadRound * 8;                      // [kQuadRound][8]
  float2* s_c = reinterpret_cast<float2*>(s_w1 + kQuadRound * 8);  // [CG][kQuadRound]
  // per sample: window anchor + 8 (bits 0-15), quadrant row offsets a0, a1
  // (bits 16-19, 20-23), mask of the warps whose rows it covers (bits 24-27)
  unsigned* s_hd = reinterpret_cast<unsigned*>(s_c + CG * kQuadRound);
  short* s_list = reinterpret_cast<short*>(s_hd + kQuadRound);  // chunk indices, z order
  __shared__ int s_wsum[kQuadThreads / 32];

  const Geom& g = a.g;
  // the four quadrants of a chunk are consecutive blocks, so that they run
  // together and their overlapping rows meet in L2
  const int sub = blockIdx.x >> 2;
  const int col = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = imin(a.s.sub_count[sub], kStreamBatch);
  const int w = W > 0 ? W : g.w;
  const int hw = w >> 1;
  const int qx = (blockIdx.x >> 1) & 1, qy = blockIdx.x & 1;
  const int b0 = (col / g.nb[1]) * g.bs[0] - hw;  // column origin (footprint frame)
  const int b1 = (col % g.nb[1]) * g.bs[1] - hw;
  const int o0 = b0 + 4 * qx, o1 = b1 + 4 * qy;   // quadrant origin
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pdq = 4 + w;
  const int i0 = threadIdx.x / pdq, i1 = threadIdx.x - i0 * pdq;
  const bool own = (int)threadIdx.x < pdq * pdq;
  const int nf2 = g.nf[2];
  const int G = (int)g.G;
  const int rowbase = own ? (wrap_idx(o0 + i0, g.nf[0]) * g.nf[1] + wrap_idx(o1 + i1, g.nf[1])) * nf2 : 0;

  // the chunk's samples whose footprint starts in this quadrant, in order
  int n_own = 0;
  for (int base = 0; base < cnt; base += kQuadThreads) {
    const int t = base + threadIdx.x;
    bool mine = false;
    if (t < cnt) {
      const int a0 = (int)ceilf(a.s.u[0][p0 + t] - g.halfw) - b0;  // 0 .. 8
      const int a1 = (int)ceilf(a.s.u[1][p0 + t] - g.halfw) - b1;
      mine = (a0 >= 4) == (qx == 1) && (a1 >= 4) == (qy == 1);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, mine);
    if (lane == 0) s_wsum[warp] = __popc(bal);
    __syncthreads();
    int before = n_own, total = 0;
#pragma unroll
    for (int q = 0; q < kQuadThreads / 32; ++q) {
      if (q < warp) before += s_wsum[q];
      total += s_wsum[q];
    }
    if (mine) s_list[before + __popc(bal & ((1u << lane) - 1u))] = (short)t;
    n_own += total;
    __syncthreads();
  }
  if (n_own == 0) return;

  auto stage_geometry = [&](int r0, int nr) {
    for (int t = threadIdx.x; t < nr; t += blockDim.x) {
      const int pos = p0 + s_list[r0 + t];
      float wt[WidthTraits<W>::WM];
      const int a0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o0;  // 0 .. 4
#pragma unroll
      for (int k = 0; k < 8; ++k) s_w0[t * 8 + k] = k < w ? wt[k] : 0.f;
      const int a1 = weights_rt<W>(a.s.u[1][pos], g, wt) - o1;
#pragma unroll
      for (int k = 0; k < 8; ++k) s_w1[t * 8 + k] = k < w ? wt[k] : 0.f;
      const float u2 = a.s.u[2][pos];
      const int zs = cell_of(u2, nf2) - hw;
      const int off = weights_rt<W>(u2, g, wt) - zs;  // 0 or 1
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int m = k - off;
        float v = 0.f;
#pragma unroll
        for (int kk = 0; kk < WidthTraits<W>::WM; ++kk)
          if (kk == m && kk < w) v = wt[kk];
        s_w2[t * 8 + ((zs + k) & 7)] = v;
      }
      // warp q's threads own quadrant rows (32 q) / pdq .. (32 q + 31) / pdq along x
      unsigned wm = 0;
#pragma unroll
      for (int q = 0; q < kQuadThreads / 32; ++q)
        if (a0 <= imin((32 * q + 31) / pdq, pdq - 1) && a0 + w - 1 >= (32 * q) / pdq) wm |= 1u << q;
      s_hd[t] = (unsigned)(zs + 8) | ((unsigned)a0 << 16) | ((unsigned)a1 << 20) | (wm << 24);
    }
  };
  const bool once = n_own <= kQuadRound;
  if (once) stage_geometry(0, n_own);

  const unsigned mybit = 1u << (24 + warp);
  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
    float ar[PACKED ? 1 : CG][8], ai[PACKED ? 1 : CG][8];
    float2 acc[PACKED ? CG : 1][8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
#pragma unroll
      for (int cc = 0; cc < (PACKED ? 1 : CG); ++cc) ar[cc][k] = ai[cc][k] = 0.f;
#pragma unroll
      for (int cc = 0; cc < (PACKED ? CG : 1); ++cc) acc[cc][k] = make_float2(0.f, 0.f);
    }
    float2* const fb = a.fine + (int64_t)c0 * g.G + rowbase;
    int zb = 0;
    auto flush = [&](unsigned mask) {
      if constexpr (PACKED) stream_flush_mask2<CG>(mask, zb, acc, own, fb, nf2, G, nc);
      else stream_flush_mask<CG>(mask, zb, ar, ai, own, fb, nf2, G, nc);
    };
    for (int r0 = 0; r0 < n_own; r0 += kQuadRound) {
      const int nr = imin(kQuadRound, n_own - r0);
      if (!once) stage_geometry(r0, nr);
      for (int t = threadIdx.x; t < nr; t += blockDim.x) {
        const int j = a.s.perm[p0 + s_list[r0 + t]];
        float dj = a.scale;
        if (a.density) dj *= a.density[j];
#pragma unroll
        for (int cc = 0; cc < CG; ++cc) {
          float2 x = cc < nc ? a.in[(int64_t)(c0 + cc) * a.s.M + j] : make_float2(0.f, 0.f);
          s_c[cc * kQuadRound + t] = make_float2(x.x * dj, x.y * dj);
        }
      }
      __syncthreads();
      if (r0 == 0) zb = (int)(s_hd[0] & 0xffffu) - 8;  // window: cells zb .. zb + 7
#pragma unroll 1
      for (int s = 0; s < nr; ++s) {
        const unsigned hd = s_hd[s];
        const int zs = (int)(hd & 0xffffu) - 8;
        if (zs != zb) {  // the same for every thread: flush the cells that leave the window
          const int steps = imin(zs - zb, 8);
          const unsigned m = (1u << steps) - 1u, r = (unsigned)zb & 7u;
          flush(((m << r) | (m >> (8u - r))) & 0xffu);
          zb = zs;
        }
        if (hd & mybit) {  // warp-uniform
          const unsigned r0w = (unsigned)(i0 - (int)((hd >> 16) & 15u));
          const unsigned r1w = (unsigned)(i1 - (int)((hd >> 20) & 15u));
          if (own && r0w < (unsigned)w && r1w < (unsigned)w) {
            const float kw = s_w0[s * 8 + r0w] * s_w1[s * 8 + r1w];
            const float4* w4 = reinterpret_cast<const float4*>(s_w2 + s * 8);
            const float4 wa = w4[0], wb = w4[1];
            const float wz[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
            for (int cc = 0; cc < CG; ++cc) {
              const float2 c = s_c[cc * kQuadRound + s];
              if constexpr (PACKED) {
                const float2 v = __fmul2_rn(c, make_float2(kw, kw));
#pragma unroll
                for (int k = 0; k < 8; ++k)
                  acc[cc][k] = __ffma2_rn(v, make_float2(wz[k], wz[k]), acc[cc][k]);
              } else {
                const float vr = kw * c.x, vi = kw * c.y;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                  ar[cc][k] = fmaf(vr, wz[k], ar[cc][k]);
                  ai[cc][k] = fmaf(vi, wz[k], ai[cc][k]);
                }
              }
            }
          }
        }
      }
      __syncthreads();  // staged strengths (and geometry) are replaced next
    }
    flush(0xffu);
  }
}

// ---------------------------------------------------------------------------
// Spreading, 2D column-streaming kernel (widths w <= 7).
//
// The sort is keyed on (x bin, y cell) with bs0 + w <= 32, so the samples of
// one column (bs0 cells along x, the whole y extent) arrive in y order.  A
// CTA takes a chunk of <= kStream2Batch consecutive samples of one column;
// lane l of every warp owns row i0 = l of the column's padded cross-section
// (32 rows along x) and keeps an 8-cell window along y in registers (cell y
// in slot y & 7), for the CG transforms of its warp; the CTA's warps cover
// different transforms of the same staged samples.  Samples in y cell f
// cover cells [f - w/2, f - w/2 + 7]; when the anchor moves, the slots that
// leave the window are added to the fine grid with float2 atomics.  The
// kernel weights are evaluated once per chunk for every transform.
// ---------------------------------------------------------------------------
constexpr int kStream2Batch = kStreamChunk2;

// dynamic shared memory of the 2D streaming kernel for `coils` transforms per pass
__host__ __device__ constexpr size_t stream2_smem_bytes(int coils) {
  return (size_t)kStream2Batch * (sizeof(unsigned) + 16 * sizeof(float)) +
         (size_t)coils * kStream2Batch * sizeof(float2);
}

template <int W, int CG>
__global__ void __launch_bounds__(GBN_THREADS, 2)
spread_stream2d_kernel(SpreadArgs a) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const int nw = blockDim.x >> 5;
  float* s_w1 = reinterpret_cast<float*>(s_raw);        // [batch][8], slot order (y)
  float* s_w0 = s_w1 + kStream2Batch * 8;                // [batch][8] (x)
  float2* s_c = reinterpret_cast<float2*>(s_w0 + kStream2Batch * 8);  // [nw * CG][batch]
  // per sample: window anchor + 8 (bits 0-13), local row offset a0 (bits 14-19)
  unsigned* s_hd = reinterpret_cast<unsigned*>(s_c + nw * CG * kStream2Batch);

  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int col = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = imin(a.s.sub_count[sub], kStream2Batch);
  const int w = W > 0 ? W : g.w;
  const int hw = w >> 1;
  const int o0 = col * g.bs[0] - hw;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool own = lane < g.pd[0];
  const int nf1 = g.nf[1];
  const int G = (int)g.G;  // fine grids hold < 2^31 cells
  const int rowbase = own ? wrap_idx(o0 + lane, g.nf[0]) * nf1 : 0;

  // geometry of the chunk, once for every transform
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int pos = p0 + t;
    float wt[WidthTraits<W>::WM];
    const int a0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o0;  // 0 .. bs0
#pragma unroll
    for (int k = 0; k < 8; ++k) s_w0[t * 8 + k] = k < w ? wt[k] : 0.f;
    const float u1 = a.s.u[1][pos];
    const int zs = cell_of(u1, nf1) - hw;
    const int off = weights_rt<W>(u1, g, wt) - zs;  // 0 or 1
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int m = k - off;
      float v = 0.f;
#pragma unroll
      for (int kk = 0; kk < WidthTraits<W>::WM; ++kk)
        if (kk == m && kk < w) v = wt[kk];
      s_w1[t * 8 + ((zs + k) & 7)] = v;
    }
    s_hd[t] = (unsigned)(zs + 8) | ((unsigned)a0 << 14);
  }

  // blockIdx.y selects the group of nw * CG transforms (one pass)
  const int per_pass = nw * CG;
  for (int cp = blockIdx.y * per_pass; cp < a.ntr && cp < (int)(blockIdx.y + 1) * per_pass;
       cp += per_pass) {
    __syncthreads();  // geometry staged
    for (int i = threadIdx.x; i < per_pass * cnt; i += blockDim.x) {
      const int k = i / cnt, t = i - k * cnt;
      const int c = cp + k;
      float2 v = make_float2(0.f, 0.f);
      if (c < a.ntr) {
        const int j = a.s.perm[p0 + t];
        float dj = a.scale;
        if (a.density) dj *= a.density[j];
        const float2 x = a.in[(int64_t)c * a.s.M + j];
        v = make_float2(x.x * dj, x.y * dj);
      }
      s_c[k * kStream2Batch + t] = v;
    }
    __syncthreads();
    const int c0 = cp + warp * CG;
    const int nc = imin(CG, a.ntr - c0);
    if (nc <= 0 || cnt == 0) continue;
    float2 acc[CG][8];  // (re, im) pairs, two-wide FMAs
#pragma unroll
    for (int cc = 0; cc < CG; ++cc)
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[cc][k] = make_float2(0.f, 0.f);
    float2* const fb = a.fine + (int64_t)c0 * g.G + rowbase;
    const float2* sc = s_c + warp * CG * kStream2Batch;
    int zb = (int)(s_hd[0] & 0x3fffu) - 8;
#pragma unroll 1
    for (int s = 0; s < cnt; ++s) {
      const unsigned hd = s_hd[s];
      const int zs = (int)(hd & 0x3fffu) - 8;
      if (zs != zb) {  // the same for every lane: flush the cells that leave the window
        const int steps = imin(zs - zb, 8);
        const unsigned m = (1u << steps) - 1u, r = (unsigned)zb & 7u;
        stream_flush_mask2<CG>(((m << r) | (m >> (8u - r))) & 0xffu, zb, acc, own, fb, nf1, G, nc);
        zb = zs;
      }
      const unsigned r0 = (unsigned)(lane - (int)((hd >> 14) & 63u));
      if (own && r0 < (unsigned)w) {
        const float kw = s_w0[s * 8 + r0];
        const float4* w4 = reinterpret_cast<const float4*>(s_w1 + s * 8);
        const float4 wa = w4[0], wb = w4[1];
        const float wz[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
        for (int cc = 0; cc < CG; ++cc) {
          const float2 v = __fmul2_rn(sc[cc * kStream2Batch + s], make_float2(kw, kw));
#pragma unroll
          for (int k = 0; k < 8; ++k) acc[cc][k] = __ffma2_rn(v, make_float2(wz[k], wz[k]), acc[cc][k]);
        }
      }
    }
    stream_flush_mask2<CG>(0xffu, zb, acc, own, fb, nf1, G, nc);
  }
}

// ---------------------------------------------------------------------------
// Spreading, 2D half-warp streaming kernel (x bins of <= 19 cells, w <= 7).
//
// The column kernel gives lane l of a warp row l of a 32-row column, so a
// sample's w rows keep w of 32 lanes busy.  Here the two half-warps take the
// chunk's samples by footprint origin a0 (half 0: a0 < 17 - w, rows 0..15;
// half 1: the rest, rows 17 - w .. 32 - w), each half in z order, and a
// warp-iteration advances both halves by one sample: a warp updates two
// samples per step with the same instruction stream.  Windows, rotated
// weights, flush rules and transforms per warp are those of the column
// kernel; the rows both halves own are flushed by both.
// ---------------------------------------------------------------------------
template <int W, int CG, int MINB = 2>
__global__ void __launch_bounds__(GBN_THREADS, MINB)
spread_half2d_kernel(SpreadArgs a) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const int nw = blockDim.x >> 5;
  float* s_w1 = reinterpret_cast<float*>(s_raw);        // [batch][8], slot order (y)
  float* s_w0 = s_w1 + kStream2Batch * 8;                // [batch][8] (x)
  float2* s_c = reinterpret_cast<float2*>(s_w0 + kStream2Batch * 8);  // [nw * CG][batch]
  // per sample: window anchor + 8 (bits 0-13), local row offset a0 (bits 14-19)
  unsigned* s_hd = reinterpret_cast<unsigned*>(s_c + nw * CG * kStream2Batch);
  short* s_list = reinterpret_cast<short*>(s_hd + kStream2Batch);  // [2][batch], z order
  __shared__ int s_wsum[GBN_THREADS / 32][2];

  const Geom& g = a.g;
  const int sub = blockIdx.x;
  const int col = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = imin(a.s.sub_count[sub], kStream2Batch);
  const int w = W > 0 ? W : g.w;
  const int hw = w >> 1;
  const int S = 17 - w;  // first footprint origin of half 1
  const int o0 = col * g.bs[0] - hw;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4;
  const int row = (lane & 15) + (half ? S : 0);
  const bool own = row < g.pd[0];
  const int nf1 = g.nf[1];
  const int G = (int)g.G;  // fine grids hold < 2^31 cells
  const int rowbase = own ? wrap_idx(o0 + row, g.nf[0]) * nf1 : 0;

  // geometry of the chunk, once for every transform
  for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
    const int pos = p0 + t;
    float wt[WidthTraits<W>::WM];
    const int a0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o0;  // 0 .. bs0
#pragma unroll
    for (int k = 0; k < 8; ++k) s_w0[t * 8 + k] = k < w ? wt[k] : 0.f;
    const float u1 = a.s.u[1][pos];
    const int zs = cell_of(u1, nf1) - hw;
    const int off = weights_rt<W>(u1, g, wt) - zs;  // 0 or 1
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int m = k - off;
      float v = 0.f;
#pragma unroll
      for (int kk = 0; kk < WidthTraits<W>::WM; ++kk)
        if (kk == m && kk < w) v = wt[kk];
      s_w1[t * 8 + ((zs + k) & 7)] = v;
    }
    s_hd[t] = (unsigned)(zs + 8) | ((unsigned)a0 << 14);
  }
  __syncthreads();
  // the samples of each half, in order
  int n0 = 0, n1 = 0;
  for (int base = 0; base < cnt; base += blockDim.x) {
    const int t = base + threadIdx.x;
    const bool h1 = t < cnt && (int)((s_hd[t] >> 14) & 63u) >= S;
    const bool h0 = t < cnt && !h1;
    const unsigned b0 = __ballot_sync(0xffffffffu, h0), b1 = __ballot_sync(0xffffffffu, h1);
    if (lane == 0) {
      s_wsum[warp][0] = __popc(b0);
      s_wsum[warp][1] = __popc(b1);
    }
    __syncthreads();
    int pre0 = n0, pre1 = n1, tot0 = 0, tot1 = 0;
    for (int q = 0; q < nw; ++q) {
      if (q < warp) {
        pre0 += s_wsum[q][0];
        pre1 += s_wsum[q][1];
      }
      tot0 += s_wsum[q][0];
      tot1 += s_wsum[q][1];
    }
    const unsigned lt = (1u << lane) - 1u;
    if (h0) s_list[pre0 + __popc(b0 & lt)] = (short)t;
    if (h1) s_list[kStream2Batch + pre1 + __popc(b1 & lt)] = (short)t;
    n0 += tot0;
    n1 += tot1;
    __syncthreads();
  }
  const int nmine = half ? n1 : n0;
  const int nmax = n0 > n1 ? n0 : n1;
  const short* lst = s_list + (half ? kStream2Batch : 0);

  // blockIdx.y selects the group of nw * CG transforms (one pass)
  const int per_pass = nw * CG;
  for (int cp = blockIdx.y * per_pass; cp < a.ntr && cp < (int)(blockIdx.y + 1) * per_pass;
       cp += per_pass) {
    __syncthreads();  // lists staged; s_c free
    for (int i = threadIdx.x; i < per_pass * cnt; i += blockDim.x) {
      const int k = i / cnt, t = i - k * cnt;
      const int c = cp + k;
      float2 v = make_float2(0.f, 0.f);
      if (c < a.ntr) {
        const int j = a.s.perm[p0 + t];
        float dj = a.scale;
        if (a.density) dj *= a.density[j];
        const float2 x = a.in[(int64_t)c * a.s.M + j];
        v = make_float2(x.x * dj, x.y * dj);
      }
      s_c[k * kStream2Batch + t] = v;
    }
    __syncthreads();
    const int c0 = cp + warp * CG;
    const int nc = imin(CG, a.ntr - c0);
    if (nc <= 0 || cnt == 0) continue;
    float2 acc[CG][8];  // (re, im) pairs, two-wide FMAs
#pragma unroll
    for (int cc = 0; cc < CG; ++cc)
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[cc][k] = make_float2(0.f, 0.f);
    float2* const fb = a.fine + (int64_t)c0 * g.G + rowbase;
    const float2* sc = s_c + warp * CG * kStream2Batch;
    int zb = nmine > 0 ? (int)(s_hd[lst[0]] & 0x3fffu) - 8 : 0;
#pragma unroll 1
    for (int it = 0; it < nmax; ++it) {
      if (it < nmine) {
        const int s = lst[it];
        const unsigned hd = s_hd[s];
        const int zs = (int)(hd & 0x3fffu) - 8;
        if (zs != zb) {  // the same for every lane of the half
          const int steps = imin(zs - zb, 8);
          const unsigned m = (1u << steps) - 1u, r = (unsigned)zb & 7u;
          stream_flush_mask2<CG>(((m << r) | (m >> (8u - r))) & 0xffu, zb, acc, own, fb, nf1, G, nc);
          zb = zs;
        }
        const unsigned r0 = (unsigned)(row - (int)((hd >> 14) & 63u));
        if (own && r0 < (unsigned)w) {
          const float kw = s_w0[s * 8 + r0];
          const float4* w4 = reinterpret_cast<const float4*>(s_w1 + s * 8);
          const float4 wa = w4[0], wb = w4[1];
          const float wz[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
          for (int cc = 0; cc < CG; ++cc) {
            const float2 v = __fmul2_rn(sc[cc * kStream2Batch + s], make_float2(kw, kw));
#pragma unroll
            for (int k = 0; k < 8; ++k) acc[cc][k] = __ffma2_rn(v, make_float2(wz[k], wz[k]), acc[cc][k]);
          }
        }
      }
    }
    stream_flush_mask2<CG>(0xffu, zb, acc, own, fb, nf1, G, nc);
  }
}

template <int W, int CG>
cudaError_t launch_spread_half2d_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  int nw = (a.ntr + CG - 1) / CG;
  if (nw > GBN_THREADS / 32) nw = GBN_THREADS / 32;
  const int passes = (a.ntr + nw * CG - 1) / (nw * CG);
  if (passes > 65535) return cudaErrorInvalidValue;
  const size_t smem = stream2_smem_bytes(nw * CG) + 2 * kStream2Batch * sizeof(short);
  // full 256-thread CTAs at 3 per SM (80 registers, 32 bytes of spills):
  // stack-of-stars spread 6.30 against 6.67 ms; CTAs of fewer warps keep 2
  // (104 registers, no spills; the 8-coil differentiable step measured 5 %
  // slower with the spills)
  auto k = nw == GBN_THREADS / 32 ? spread_half2d_kernel<W, CG, 3> : spread_half2d_kernel<W, CG, 2>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<dim3(a.s.nsub, passes), nw * 32, smem, st>>>(a);
  return cudaGetLastError();
}

template <int W, int CG>
cudaError_t launch_spread_stream2d_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  int nw = (a.ntr + CG - 1) / CG;
  if (nw > GBN_THREADS / 32) nw = GBN_THREADS / 32;
  const int passes = (a.ntr + nw * CG - 1) / (nw * CG);
  if (passes > 65535) return cudaErrorInvalidValue;
  const size_t smem = stream2_smem_bytes(nw * CG);
  auto k = spread_stream2d_kernel<W, CG>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<dim3(a.s.nsub, passes), nw * 32, smem, st>>>(a);
  return cudaGetLastError();
}

// a.s is the column-chunk table (sub_bin = x-bin index)
// two transforms per warp (four spill registers: measured 11 % slower on the
// 1024-transform stack-of-stars spread)
inline cudaError_t dispatch_spread_stream2d(const SpreadArgs& a, cudaStream_t st) {
  const int cg = (a.ntr >= 2 && a.g.spread_cg != 1) ? 2 : 1;
  // x bins of <= 19 cells: half-warp kernel unless GBN_SPREAD=stream
  if (a.g.bs[0] <= 19 && a.g.method_spread != 3) {
    if (a.g.w == 7)
      return cg == 2 ? launch_spread_half2d_t<7, 2>(a, st) : launch_spread_half2d_t<7, 1>(a, st);
    return cg == 2 ? launch_spread_half2d_t<0, 2>(a, st) : launch_spread_half2d_t<0, 1>(a, st);
  }
  if (a.g.w == 7)
    return cg == 2 ? launch_spread_stream2d_t<7, 2>(a, st) : launch_spread_stream2d_t<7, 1>(a, st);
  return cg == 2 ? launch_spread_stream2d_t<0, 2>(a, st) : launch_spread_stream2d_t<0, 1>(a, st);
}

// ---------------------------------------------------------------------------
// Spreading, sample-driven kernel with global vector atomics (2D, and any
// width the row kernel does not cover).  Threads take consecutive sorted
// samples, so the float2 reductions of a warp land on nearby cells of the
// same L2 sectors.
// ---------------------------------------------------------------------------
template <int DIM, int W>
__device__ __forceinline__ void spread_gm_body(const SpreadArgs& a, const int64_t pos) {
  constexpr int WM = WidthTraits<W>::WM;
  const Geom& g = a.g;
  if (pos >= a.s.M) return;
  const int w = W > 0 ? W : g.w;
  const int WL = W > 0 ? W : w;
  const int j = a.s.perm[pos];
  float w0[WM], w1[WM], w2[WM];
  int m0[WM], m1[WM], m2[WM];
  int i0 = weights_rt<W>(a.s.u[0][pos], g, w0);
  int i1 = weights_rt<W>(a.s.u[1][pos], g, w1);
  int i2 = 0;
  if (DIM == 3) i2 = weights_rt<W>(a.s.u[2][pos], g, w2);
GBN_UNROLL
  for (int t = 0; t < WL; ++t) {
    m0[t] = wrap_idx(i0 + t, g.nf[0]);
    m1[t] = wrap_idx(i1 + t, g.nf[1]);
    if (DIM == 3) m2[t] = wrap_idx(i2 + t, g.nf[2]);
  }
  float dj = a.scale;
  if (a.density) dj *= a.density[j];
  for (int c = 0; c < a.ntr; ++c) {
    float2 x = a.in[(int64_t)c * a.s.M + j];
    const float vr = x.x * dj, vi = x.y * dj;
    float2* base = a.fine + (int64_t)c * g.G;
GBN_UNROLL
    for (int t0 = 0; t0 < WL; ++t0) {
GBN_UNROLL
      for (int t1 = 0; t1 < WL; ++t1) {
        const float k = w0[t0] * w1[t1];
        const int64_t r = (int64_t)m0[t0] * g.nf[1] + m1[t1];
        if (DIM == 2) {
          atomicAdd(base + r, make_float2(k * vr, k * vi));
        } else {
GBN_UNROLL
          for (int t2 = 0; t2 < WL; ++t2) {
            const float kk = k * w2[t2];
            atomicAdd(base + r * g.nf[2] + m2[t2], make_float2(kk * vr, kk * vi));
          }
        }
      }
    }
  }
}

template <int DIM, int W>
__global__ void __launch_bounds__(GBN_THREADS)
spread_gm_kernel(SpreadArgs a) {
  spread_gm_body<DIM, W>(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// Warp-cooperative spreading with global vector atomics (w = 7).  Eight lanes
// serve one sorted sample: lane l adds to the footprint cells at offset l of
// the last axis, so each warp instruction issues the float2 reductions of
// four samples onto 7 contiguous cells each (two 32-byte sectors per sample
// instead of one sector per lane).
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ void spread_wc_body(const SpreadArgs& a, const int64_t warp_id) {
  constexpr int W = 7;
  const Geom& g = a.g;
  const int lane = threadIdx.x & 31;
  const int q = lane >> 3, l = lane & 7;
  const int64_t pos = warp_id * 4 + q;
  if (pos >= a.s.M || l >= W) return;
  const int j = a.s.perm[pos];
  float w0[W], w1[W];
  int r0[W], m1[W];
  const int i0 = weights_rt<W>(a.s.u[0][pos], g, w0);
  float wl;
  int ml;
  if (DIM == 2) {
    const float u1 = a.s.u[1][pos];
    const int i1 = (int)ceilf(u1 - g.halfw);
    wl = es_eval((float)(i1 + l) - u1, g.beta, g.inv_halfw);
    ml = wrap_idx(i1 + l, g.nf[1]);
  } else {
    const int i1 = weights_rt<W>(a.s.u[1][pos], g, w1);
    const float u2 = a.s.u[2][pos];
    const int i2 = (int)ceilf(u2 - g.halfw);
    wl = es_eval((float)(i2 + l) - u2, g.beta, g.inv_halfw);
    ml = wrap_idx(i2 + l, g.nf[2]);
#pragma unroll
    for (int t = 0; t < W; ++t) m1[t] = wrap_idx(i1 + t, g.nf[1]);
  }
#pragma unroll
  for (int t = 0; t < W; ++t) r0[t] = wrap_idx(i0 + t, g.nf[0]) * g.nf[1];
  float dj = a.scale * wl;
  if (a.density) dj *= a.density[j];
  for (int c = 0; c < a.ntr; ++c) {
    const float2 x = a.in[(int64_t)c * a.s.M + j];
    const float vr = x.x * dj, vi = x.y * dj;
    float2* base = a.fine + (int64_t)c * g.G;
#pragma unroll
    for (int t0 = 0; t0 < W; ++t0) {
      if (DIM == 2) {
        atomicAdd(base + r0[t0] + ml, make_float2(w0[t0] * vr, w0[t0] * vi));
      } else {
#pragma unroll
        for (int t1 = 0; t1 < W; ++t1) {
          const float k = w0[t0] * w1[t1];
          atomicAdd(base + (int64_t)(r0[t0] + m1[t1]) * g.nf[2] + ml, make_float2(k * vr, k * vi));
        }
      }
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS, 4)
spread_wc_kernel(SpreadArgs a) {
  spread_wc_body<DIM>(a, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
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

  __shared__ int s_rowoff[kMaxTileRows];
  const int* rowoff = tile_rows_init<DIM>(g, o, s_rowoff);
  __syncthreads();
  for (int c = 0; c < a.ntr; ++c) {
    load_tiles<DIM>(tile, a.fine, g, o, c, 1, rowoff);
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
  // 128-thread CTAs: subproblems average fewer samples than 256, and smaller
  // CTAs wait less at the per-coil tile barriers (measured 4 % faster in 3D)
  const int threads = a.g.interp_threads == 64 ? 64 : kInterpThreads;
  k<<<a.s.nsub, threads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int W, int CG>
cudaError_t launch_spread_rows_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  spread_rows3d_kernel<W, CG><<<a.s.nsub, GBN_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

template <int W, int CG>
cudaError_t launch_spread_stream_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  const size_t smem = stream_smem_bytes(CG);
  auto k = spread_stream3d_kernel<W, CG>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // one CTA per chunk runs every transform pass (the kernel also accepts a
  // split of the passes over blockIdx.y groups)
  k<<<dim3(a.s.nsub, 1), GBN_THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int W, int CG, int MINB = 4, bool PACKED = false>
cudaError_t launch_spread_quad_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  const size_t smem = quad_smem_bytes(CG);
  auto k = spread_quad3d_kernel<W, CG, MINB, PACKED>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<(unsigned)(4 * (int64_t)a.s.nsub), kQuadThreads, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gbn

#include "gbn_mma_spread.cuh"

namespace gbn {

// a.s is the column-chunk table (sub_bin = column index)
inline cudaError_t dispatch_spread_stream3d(const SpreadArgs& a, cudaStream_t st) {
  int cg = a.ntr >= 3 ? 4 : a.ntr;
  if (a.g.spread_cg == 1 || a.g.spread_cg == 2 || a.g.spread_cg == 4) cg = imin(cg, a.g.spread_cg);
  // 8 x 8 bins: quadrant CTAs (measured 7 % faster than whole columns on the
  // 3D kooshball); GBN_SPREAD=stream keeps the column kernel
  if (a.g.method_spread == 6 && a.g.w == 7 && a.g.bs[0] == 8 && a.g.bs[1] == 8)
    return launch_spread_mma3d(a, st);
  if ((a.g.method_spread == 0 || a.g.method_spread == 5) && a.g.bs[0] == 8 && a.g.bs[1] == 8) {
    if (a.g.w == 7) {
      // 4 coils per pass at 3 CTAs per SM (170 registers, no spills;
      // measured 7.08 against 7.63 ms at 4 CTAs per SM, whose 128-register
      // cap spills, on the 16-coil 3D kooshball); GBN_QUAD_MINB=4 keeps 4
      // CTAs; GBN_SPREAD_CG=8 runs 8 coils per pass at 2 CTAs per SM (7.50 ms)
      if (a.g.spread_cg == 8 && a.ntr >= 8)
        return a.g.quad_packed != 0 ? launch_spread_quad_t<7, 8, 2, true>(a, st)
                                    : launch_spread_quad_t<7, 8, 2>(a, st);
      // (re, im) accumulator pairs with two-wide FMAs (measured 6.11 against
      // 7.09 ms on the 16-coil 3D kooshball); GBN_QUAD_PACKED=0 keeps scalar
      // accumulators
      if (cg == 4 && a.g.quad_packed != 0) return launch_spread_quad_t<7, 4, 3, true>(a, st);
      if (cg == 4 && a.g.quad_minb == 4) return launch_spread_quad_t<7, 4, 4>(a, st);
      if (cg == 4) return launch_spread_quad_t<7, 4, 3>(a, st);
      return cg == 2 ? launch_spread_quad_t<7, 2>(a, st) : launch_spread_quad_t<7, 1>(a, st);
    }
    if (cg == 4) return launch_spread_quad_t<0, 4>(a, st);
    return cg == 2 ? launch_spread_quad_t<0, 2>(a, st) : launch_spread_quad_t<0, 1>(a, st);
  }
  if (a.g.w == 7) {
    if (cg == 4) return launch_spread_stream_t<7, 4>(a, st);
    return cg == 2 ? launch_spread_stream_t<7, 2>(a, st) : launch_spread_stream_t<7, 1>(a, st);
  }
  if (cg == 4) return launch_spread_stream_t<0, 4>(a, st);
  return cg == 2 ? launch_spread_stream_t<0, 2>(a, st) : launch_spread_stream_t<0, 1>(a, st);
}

template <int DIM, int W>
cudaError_t launch_spread_gm_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.M == 0) return cudaSuccess;
  unsigned blocks = (unsigned)((a.s.M + GBN_THREADS - 1) / GBN_THREADS);
  spread_gm_kernel<DIM, W><<<blocks, GBN_THREADS, 0, st>>>(a);
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

template <int DIM, int W>
cudaError_t launch_interp_gm_t(const InterpArgs& a, cudaStream_t st) {
  if (a.s.M == 0) return cudaSuccess;
  unsigned blocks = (unsigned)((a.s.M + GBN_THREADS - 1) / GBN_THREADS);
  if (a.ntr > 1 && a.mode != INTERP_PIPE && a.g.interp_cg != 1)
    interp_gm_kernel<DIM, W, 4><<<blocks, GBN_THREADS, 0, st>>>(a);
  else
    interp_gm_kernel<DIM, W, 1><<<blocks, GBN_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

template <int DIM, int S>
cudaError_t launch_interp_db_t(const InterpArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  size_t smem = 2 * (size_t)a.g.tile * sizeof(float2);
  auto k = interp_db_kernel<DIM, 7, S>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<a.s.nsub, GBN_THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_interp_wc_t(const InterpArgs& a, cudaStream_t st) {
  if (a.s.M == 0) return cudaSuccess;
  const int64_t warps = (a.s.M + 3) / 4;
  const unsigned blocks = (unsigned)((warps * 32 + GBN_THREADS - 1) / GBN_THREADS);
  interp_wc_kernel<DIM><<<blocks, GBN_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

inline cudaError_t launch_interp_twc(const InterpArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  size_t smem = (size_t)a.g.tile * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(interp_twc3d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  interp_twc3d_kernel<<<a.s.nsub, GBN_THREADS, smem, st>>>(a);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t dispatch_interp(const InterpArgs& a, cudaStream_t st) {
  // 2D at w = 7 defaults to the warp-cooperative direct kernel (measured 1.1x
  // the tile kernel with its bank-aware lane order on the 1024-transform
  // stack-of-stars, 2.7x before it); 3D to tiles.  GBN_INTERP=tile forces tiles.
  if (a.g.w == 7 && (a.g.method_interp == 4 || (DIM == 2 && a.g.method_interp == 0)))
    return launch_interp_wc_t<DIM>(a, st);
  if (DIM == 3 && a.g.method_interp == 5 && a.g.w == 7 && a.s.maxsub <= kTwcMaxSub)
    return launch_interp_twc(a, st);
  // default for the w = 7 kernel: double-buffered tiles with register weights
  if (a.g.method_interp == 3 && a.g.w == 7 && a.s.maxsub <= 2 * GBN_THREADS &&
      2 * (size_t)a.g.tile * sizeof(float2) <= (size_t)kTileSmemBudget) {
    if (a.s.maxsub <= GBN_THREADS) return launch_interp_db_t<DIM, 1>(a, st);
    return launch_interp_db_t<DIM, 2>(a, st);
  }
  if (a.g.method_interp == 1) {
    if (a.g.w == 7) return launch_interp_gm_t<DIM, 7>(a, st);
    return launch_interp_gm_t<DIM, 0>(a, st);
  }
  int cg = a.mode == INTERP_PIPE ? 1 : coils_per_pass(a.g, a.ntr);
  if (cg >= 4) return dispatch_interp_w<DIM, 4>(a, st);
  if (cg == 2) return dispatch_interp_w<DIM, 2>(a, st);
  return dispatch_interp_w<DIM, 1>(a, st);
}


template <int DIM>
cudaError_t launch_spread_wc_t(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.M == 0) return cudaSuccess;
  const int64_t warps = (a.s.M + 3) / 4;
  const unsigned blocks = (unsigned)((warps * 32 + GBN_THREADS - 1) / GBN_THREADS);
  spread_wc_kernel<DIM><<<blocks, GBN_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

template <int DIM>
cudaError_t dispatch_spread(const SpreadArgs& a, cudaStream_t st) {
  // 2D at w = 7 defaults to warp-cooperative atomics (2.5x the per-sample
  // atomics); 3D to the row kernel
  if (a.g.w == 7 && (a.g.method_spread == 2 || (DIM == 2 && a.g.method_spread == 0)))
    return launch_spread_wc_t<DIM>(a, st);
  if (DIM == 3 && rows_fit(a.g) && a.g.method_spread != 1) {
    if (a.g.w == 7) return a.ntr > 1 ? launch_spread_rows_t<7, 2>(a, st) : launch_spread_rows_t<7, 1>(a, st);
    return a.ntr > 1 ? launch_spread_rows_t<0, 2>(a, st) : launch_spread_rows_t<0, 1>(a, st);
  }
  if (a.g.w == 7) return launch_spread_gm_t<DIM, 7>(a, st);
  return launch_spread_gm_t<DIM, 0>(a, st);
}

template <int DIM>
cudaError_t dispatch_grad(const GradArgs& a, cudaStream_t st) {
  // runtime-width kernel: the derivative path is not the throughput path
  return launch_grad_t<DIM, 0>(a, a.conj_a, st);
}

}  // namespace gbn
