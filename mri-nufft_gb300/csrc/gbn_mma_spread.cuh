// Spreading, 3D quadrant kernel on the tensor cores (w = 7, 8 x 8 bins).
//
// The work of the quadrant-streaming spreader (gbn_kernels.cuh) is a sum of
// rank-one updates: a quadrant's (4 + w) x (4 + w) = 121 cross-section rows
// (padded to M = 128) receive, for each of its samples s in z order,
//   G[row, cell z, coil c] += wx(s, x_row) wy(s, y_row) * wz(s, z) c_s,
// which over a block of 16 consecutive samples is the matrix product
//   D[row, (slot, coil, re/im)] += A[row, s] B[s, (slot, coil, re/im)]
// with A[row, s] = wx wy (zero outside the footprint) and B[s, ...] =
// wz(s, cell of the slot) times the real or imaginary part of the strength.
// The accumulator D lives in registers as mma.sync m16n8k16 fragments: each
// warp owns 32 rows, the N = 128 columns are 16 ring slots of the z axis
// (cell z in slot z & 15) times 4 coils times (re, im), so a lane holds the
// (re, im) pair of coil (lane & 3) for 4 rows of every slot.  A block takes
// up to 16 samples whose cells lie within 8 of its first sample's cell, so
// that every footprint fits the ring [zb, zb + 16) with zb = first cell - 3;
// the slots of the cells below the next block's zb are added to the fine
// grid with float2 atomics and cleared before that block.
//
// Precision: A and B are split into bf16 high and low parts (x = hi + lo,
// lo the bf16 rounding of x - hi) and D += Ah Bh + Ah Bl + Al Bh; the
// dropped Al Bl term and the rounding of the low parts leave about 2^-16
// relative error per product, accumulated in fp32.
#pragma once

#include "gbn_internal.cuh"

namespace gbn {

constexpr int kMmaThreads = 128;
constexpr int kMmaRound = 256;  // samples staged at a time
constexpr int kMmaCG = 4;       // coils per pass

__host__ __device__ constexpr size_t mma_spread_smem_bytes() {
  return (size_t)kMmaRound * sizeof(int)                 // headers
         + (size_t)kMmaRound * 24 * sizeof(float)        // wx, wy, wz (8 each)
         + (size_t)kMmaCG * kMmaRound * sizeof(float2)   // strengths
         + (size_t)2 * 16 * 32 * sizeof(uint2)           // B fragments, hi and lo
         + (size_t)kStreamChunk * sizeof(short);         // chunk indices in z order
}

__device__ __forceinline__ void bf16x3_split(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  // hi packs bf16(v1):bf16(v0) (v0 in the low half, the lower k index of a
  // fragment register); lo packs the bf16 rounding of the residuals
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(v1), "f"(v0));
  const float h0 = __uint_as_float(hi << 16);
  const float h1 = __uint_as_float(hi & 0xffff0000u);
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(v1 - h1), "f"(v0 - h0));
}

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                          uint32_t b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

template <int W>
__global__ void __launch_bounds__(kMmaThreads, 2) spread_mma3d_kernel(SpreadArgs a) {
  static_assert(W == 7, "the tensor-core spreader is written for w = 7");
  constexpr int CG = kMmaCG;
  extern __shared__ __align__(16) unsigned char s_raw[];
  uint2* s_bh = reinterpret_cast<uint2*>(s_raw);            // [16 slots][32 lanes]
  uint2* s_bl = s_bh + 16 * 32;
  float* s_wx = reinterpret_cast<float*>(s_bl + 16 * 32);   // [kMmaRound][8]
  float* s_wy = s_wx + kMmaRound * 8;
  float* s_wz = s_wy + kMmaRound * 8;
  float2* s_c = reinterpret_cast<float2*>(s_wz + kMmaRound * 8);  // [CG][kMmaRound]
  // per sample: x, y footprint origins in the quadrant (bits 0-3, 4-7), first
  // z cell minus (cell - 3) (bit 8), z cell (bits 12-31)
  int* s_hd = reinterpret_cast<int*>(s_c + CG * kMmaRound);
  short* s_list = reinterpret_cast<short*>(s_hd + kMmaRound);
  __shared__ int s_wsum[kMmaThreads / 32];

  const Geom& g = a.g;
  const int sub = blockIdx.x >> 2;
  const int col = a.s.sub_bin[sub];
  const int p0 = a.s.sub_start[sub];
  const int cnt = imin(a.s.sub_count[sub], kStreamChunk);
  constexpr int hw = W >> 1;
  const int qx = (blockIdx.x >> 1) & 1, qy = blockIdx.x & 1;
  const int b0 = (col / g.nb[1]) * g.bs[0] - hw;  // column origin (footprint frame)
  const int b1 = (col % g.nb[1]) * g.bs[1] - hw;
  const int o0 = b0 + 4 * qx, o1 = b1 + 4 * qy;   // quadrant origin
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int nf2 = g.nf[2];
  const int G = (int)g.G;
  constexpr int PQ = 4 + W;  // cross-section rows per axis

  // the chunk's samples whose footprint starts in this quadrant, in order
  int n_own = 0;
  for (int base = 0; base < cnt; base += kMmaThreads) {
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
    for (int q = 0; q < kMmaThreads / 32; ++q) {
      if (q < warp) before += s_wsum[q];
      total += s_wsum[q];
    }
    if (mine) s_list[before + __popc(bal & ((1u << lane) - 1u))] = (short)t;
    n_own += total;
    __syncthreads();
  }
  if (n_own == 0) return;

  // the lane's 4 rows: (m-tile mt, half h) -> row 32 warp + 16 mt + gq + 8 h
  int rx[4], ry[4], rb[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = 32 * warp + 16 * (q >> 1) + gq + 8 * (q & 1);
    rx[q] = r / PQ;
    ry[q] = r - rx[q] * PQ;
    rb[q] = r < PQ * PQ ? (wrap_idx(o0 + rx[q], g.nf[0]) * g.nf[1] + wrap_idx(o1 + ry[q], g.nf[1])) * nf2
                        : -1;
  }

  auto stage_geometry = [&](int r0, int nr) {
    for (int t = threadIdx.x; t < nr; t += blockDim.x) {
      const int pos = p0 + s_list[r0 + t];
      float wt[W];
      const int a0 = weights_rt<W>(a.s.u[0][pos], g, wt) - o0;  // 0 .. 4
#pragma unroll
      for (int k = 0; k < 8; ++k) s_wx[t * 8 + k] = k < W ? wt[k] : 0.f;
      const int a1 = weights_rt<W>(a.s.u[1][pos], g, wt) - o1;
#pragma unroll
      for (int k = 0; k < 8; ++k) s_wy[t * 8 + k] = k < W ? wt[k] : 0.f;
      const float u2 = a.s.u[2][pos];
      const int cell = cell_of(u2, nf2);
      const int off = weights_rt<W>(u2, g, wt) - (cell - hw);  // 0 or 1
#pragma unroll
      for (int k = 0; k < 8; ++k) s_wz[t * 8 + k] = k < W ? wt[k] : 0.f;
      s_hd[t] = a0 | (a1 << 4) | (off << 8) | (cell << 12);
    }
  };
  const bool once = n_own <= kMmaRound;
  if (once) stage_geometry(0, n_own);

  float d[2][16][4];
  for (int c0 = 0; c0 < a.ntr; c0 += CG) {
    const int nc = imin(CG, a.ntr - c0);
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
      for (int j = 0; j < 16; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) d[mt][j][e] = 0.f;
    const bool coil_ok = tq < nc;
    float2* const fc = a.fine + (int64_t)(c0 + tq) * G;
    bool have = false;
    int zb = 0;  // the ring holds cells zb .. zb + 15

    // adds the ring slots in `mask` to the fine grid and clears them
    auto flush = [&](unsigned mask) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        if (mask & (1u << j)) {
          const int z = wrap_near(zb + ((j - zb) & 15), nf2);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float vr = d[q >> 1][j][2 * (q & 1)], vi = d[q >> 1][j][2 * (q & 1) + 1];
            if (coil_ok && rb[q] >= 0 && (vr != 0.f || vi != 0.f))
              atomicAdd(fc + rb[q] + z, make_float2(vr, vi));
            d[q >> 1][j][2 * (q & 1)] = 0.f;
            d[q >> 1][j][2 * (q & 1) + 1] = 0.f;
          }
        }
      }
    };

    for (int r0 = 0; r0 < n_own; r0 += kMmaRound) {
      const int nr = imin(kMmaRound, n_own - r0);
      if (!once) stage_geometry(r0, nr);
      for (int t = threadIdx.x; t < nr; t += blockDim.x) {
        const int j = a.s.perm[p0 + s_list[r0 + t]];
        float dj = a.scale;
        if (a.density) dj *= a.density[j];
#pragma unroll
        for (int cc = 0; cc < CG; ++cc) {
          float2 x = cc < nc ? a.in[(int64_t)(c0 + cc) * a.s.M + j] : make_float2(0.f, 0.f);
          s_c[cc * kMmaRound + t] = make_float2(x.x * dj, x.y * dj);
        }
      }
      __syncthreads();
      int s = 0;
      while (s < nr) {
        // block: up to 16 samples within 8 cells of the first one (uniform)
        const int cell0 = s_hd[s] >> 12;
        int n = 1;
        while (n < 16 && s + n < nr && (s_hd[s + n] >> 12) <= cell0 + 8) ++n;
        const int zn = cell0 - hw;
        if (have && zn > zb) {
          unsigned mask = 0;
          const int zend = imin(zn, zb + 16);
          for (int z = zb; z < zend; ++z) mask |= 1u << (z & 15);
          flush(mask);
        }
        have = true;
        zb = zn;
        __syncthreads();  // the previous block's B fragments are consumed
        // B fragments: entry (slot j, lane L) holds samples 2t', 2t'+1,
        // 2t'+8, 2t'+9 of column n = g' = (coil, re/im)
        for (int e = threadIdx.x; e < 16 * 32; e += blockDim.x) {
          const int j = e >> 5, L = e & 31;
          const int gg = L >> 2, tt = L & 3;
          const int cc = gg >> 1, ri = gg & 1;
          const int z = zb + ((j - zb) & 15);
          float v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int k = 2 * tt + (q & 1) + 8 * (q >> 1);
            float val = 0.f;
            if (k < n) {
              const int hd = s_hd[s + k];
              const int dz = z - ((hd >> 12) - hw + ((hd >> 8) & 1));
              if ((unsigned)dz < (unsigned)W) {
                const float2 c = s_c[cc * kMmaRound + s + k];
                val = s_wz[(s + k) * 8 + dz] * (ri ? c.y : c.x);
              }
            }
            v[q] = val;
          }
          uint2 h, l;
          bf16x3_split(v[0], v[1], h.x, l.x);
          bf16x3_split(v[2], v[3], h.y, l.y);
          s_bh[e] = h;
          s_bl[e] = l;
        }
        // A fragments: rows of the lane, samples 2 tq, 2 tq + 1, 2 tq + 8, 2 tq + 9
        float av[4][4];  // [row q][sample slot k]
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const int k = 2 * tq + (kk & 1) + 8 * (kk >> 1);
          int hd = 0;
          if (k < n) hd = s_hd[s + k];
          const int ax = hd & 15, ay = (hd >> 4) & 15;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int dx = rx[q] - ax, dy = ry[q] - ay;
            float val = 0.f;
            if (k < n && (unsigned)dx < (unsigned)W && (unsigned)dy < (unsigned)W)
              val = s_wx[(s + k) * 8 + dx] * s_wy[(s + k) * 8 + dy];
            av[q][kk] = val;
          }
        }
        uint32_t ah[2][4], al[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          // a0: (row g, k 2t..2t+1), a1: (row g+8, k 2t..), a2: (row g, k 2t+8..), a3: (row g+8, k 2t+8..)
          bf16x3_split(av[2 * mt][0], av[2 * mt][1], ah[mt][0], al[mt][0]);
          bf16x3_split(av[2 * mt + 1][0], av[2 * mt + 1][1], ah[mt][1], al[mt][1]);
          bf16x3_split(av[2 * mt][2], av[2 * mt][3], ah[mt][2], al[mt][2]);
          bf16x3_split(av[2 * mt + 1][2], av[2 * mt + 1][3], ah[mt][3], al[mt][3]);
        }
        __syncthreads();  // B fragments written
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const uint2 bh = s_bh[j * 32 + lane];
          const uint2 bl = s_bl[j * 32 + lane];
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            mma_16816(d[mt][j], al[mt], bh.x, bh.y);
            mma_16816(d[mt][j], ah[mt], bl.x, bl.y);
            mma_16816(d[mt][j], ah[mt], bh.x, bh.y);
          }
        }
        s += n;
      }
      __syncthreads();  // staged strengths (and geometry) are replaced next
    }
    flush(0xffffu);
  }
}

inline cudaError_t launch_spread_mma3d(const SpreadArgs& a, cudaStream_t st) {
  if (a.s.nsub == 0) return cudaSuccess;
  const size_t smem = mma_spread_smem_bytes();
  auto k = spread_mma3d_kernel<7>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<(unsigned)(4 * (int64_t)a.s.nsub), kMmaThreads, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gbn
