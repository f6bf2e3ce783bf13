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
  return (size_t)2 * 16 * 32 * sizeof(uint2)             // B fragments, hi and lo
         + (size_t)kMmaRound * 49 * sizeof(uint32_t)     // x-y weight products, bf16 hi | lo
         + (size_t)kMmaRound * 8 * sizeof(float)         // wz
         + (size_t)kMmaCG * kMmaRound * sizeof(float2)   // strengths
         + (size_t)kMmaRound * sizeof(int)               // headers
         + (size_t)kStreamChunk * sizeof(short);         // chunk indices in z order
}

// bf16 high part of v and bf16 rounding of the residual, packed hi | lo << 16
__device__ __forceinline__ uint32_t bf16_hilo(float v) {
  uint32_t h;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(h) : "f"(0.f), "f"(v));  // low half = bf16(v)
  const float r = v - __uint_as_float(h << 16);
  uint32_t l;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(l) : "f"(r), "f"(0.f));  // high half = bf16(r)
  return (h & 0xffffu) | (l & 0xffff0000u);
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
  uint2* s_bh = reinterpret_cast<uint2*>(s_raw);                // [16 slots][32 lanes]
  uint2* s_bl = s_bh + 16 * 32;
  uint32_t* s_p = reinterpret_cast<uint32_t*>(s_bl + 16 * 32);  // [kMmaRound][49]
  float* s_wz = reinterpret_cast<float*>(s_p + kMmaRound * 49);   // [kMmaRound][8]
  float2* s_c = reinterpret_cast<float2*>(s_wz + kMmaRound * 8);  // [CG][kMmaRound]
  // per sample: x, y footprint origins in the quadrant (bits 0-3, 4-7), first
  // footprint cell along z minus (cell - 3) (bit 8), z cell (bits 12-31)
  int* s_hd = reinterpret_cast<int*>(s_c + CG * kMmaRound);
  short* s_list = reinterpret_cast<short*>(s_hd + kMmaRound);
  unsigned short* s_bh16 = reinterpret_cast<unsigned short*>(s_bh);
  unsigned short* s_bl16 = reinterpret_cast<unsigned short*>(s_bl);
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

  // geometry of a round: header, the 7 x 7 products wx wy (bf16 hi | lo),
  // the z weights
  auto stage_geometry = [&](int r0, int nr) {
    for (int t = threadIdx.x; t < nr; t += blockDim.x) {
      const int pos = p0 + s_list[r0 + t];
      float wx[W], wy[W], wz[W];
      const int a0 = weights_rt<W>(a.s.u[0][pos], g, wx) - o0;  // 0 .. 4
      const int a1 = weights_rt<W>(a.s.u[1][pos], g, wy) - o1;
      const float u2 = a.s.u[2][pos];
      const int cell = cell_of(u2, nf2);
      const int off = weights_rt<W>(u2, g, wz) - (cell - hw);  // 0 or 1
#pragma unroll
      for (int i = 0; i < W; ++i)
#pragma unroll
        for (int k = 0; k < W; ++k) s_p[t * 49 + i * W + k] = bf16_hilo(wx[i] * wy[k]);
#pragma unroll
      for (int k = 0; k < 8; ++k) s_wz[t * 8 + k] = k < W ? wz[k] : 0.f;
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
        // block: up to 16 samples in cells within 8 of the first one's, so
        // that every footprint lies in [cell0 - 3, cell0 + 13) (uniform)
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
        {
          // B: thread -> (sample k of the block, column n = (coil, re/im));
          // its 16 slots, the footprint's 7 nonzero, into the fragment layout
          // (entry (slot, lane n * 4 + (k & 7) / 2), word k / 8, half k & 1)
          const int k = threadIdx.x >> 3, nn = threadIdx.x & 7;
          const int L = nn * 4 + ((k & 7) >> 1);
          const int hoff = (k >> 3) * 2 + (k & 1);
          float cv = 0.f;
          int dz0 = 0;
          if (k < n) {
            const float2 c = s_c[(nn >> 1) * kMmaRound + s + k];
            cv = (nn & 1) ? c.y : c.x;
            const int hd = s_hd[s + k];
            dz0 = (hd >> 12) - hw + ((hd >> 8) & 1) - zb;  // 0 .. 9
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int dz = ((j - zb - dz0) & 15);  // footprint offset of slot j
            const bool on = k < n && dz < W;
            const float v = on ? s_wz[on ? (s + k) * 8 + dz : 0] * cv : 0.f;
            const uint32_t hl = bf16_hilo(v);
            s_bh16[(j * 32 + L) * 4 + hoff] = (unsigned short)(hl & 0xffffu);
            s_bl16[(j * 32 + L) * 4 + hoff] = (unsigned short)(hl >> 16);
          }
        }
        // A fragments from the product table: rows of the lane, samples
        // 2 tq, 2 tq + 1 (word 0) and 2 tq + 8, 2 tq + 9 (word 1)
        uint32_t ah[2][4], al[2][4];
#pragma unroll
        for (int kp = 0; kp < 2; ++kp) {
          const int k0 = 2 * tq + 8 * kp;
          uint32_t pv[2][4];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int k = k0 + e;
            const int hd = k < n ? s_hd[s + k] : (15 | (15 << 4));
            const int ax = hd & 15, ay = (hd >> 4) & 15;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int dx = rx[q] - ax, dy = ry[q] - ay;
              const bool on = (unsigned)dx < (unsigned)W && (unsigned)dy < (unsigned)W;
              // the index stays inside the table when the entry is off
              const uint32_t pe = s_p[on ? (s + k) * 49 + dx * W + dy : 0];
              pv[e][q] = on ? pe : 0u;
            }
          }
#pragma unroll
          for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              // register 2 kp + h of m-tile mt: row (mt, h), samples k0, k0 + 1
              const uint32_t x0 = pv[0][2 * mt + h], x1 = pv[1][2 * mt + h];
              ah[mt][2 * kp + h] = __byte_perm(x0, x1, 0x5410);
              al[mt][2 * kp + h] = __byte_perm(x0, x1, 0x7632);
            }
        }
        __syncthreads();  // B fragments written
#pragma unroll
        for (int j0 = 0; j0 < 16; j0 += 4) {
          uint2 bh[4], bl[4];
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            bh[jj] = s_bh[(j0 + jj) * 32 + lane];
            bl[jj] = s_bl[(j0 + jj) * 32 + lane];
          }
#pragma unroll
          for (int jj = 0; jj < 4; ++jj)
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma_16816(d[mt][j0 + jj], al[mt], bh[jj].x, bh[jj].y);
#pragma unroll
          for (int jj = 0; jj < 4; ++jj)
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma_16816(d[mt][j0 + jj], ah[mt], bl[jj].x, bl[jj].y);
#pragma unroll
          for (int jj = 0; jj < 4; ++jj)
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) mma_16816(d[mt][j0 + jj], ah[mt], bh[jj].x, bh[jj].y);
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
