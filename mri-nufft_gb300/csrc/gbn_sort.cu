// Bin sort of the non-uniform points (the "setpts" step).
//
// A counting sort over spatial bins of the fine grid:
//   1. each sample is folded to fine-grid units, assigned its bin and a rank
//      inside the bin with a warp-aggregated atomic (lanes of one warp that
//      share a bin receive consecutive ranks in lane order, so runs of
//      consecutive input samples stay contiguous after the sort and the
//      gathers / scatters of k-space data in spread / interp coalesce);
//   2. an exclusive scan of the bin histogram gives bin start offsets;
//   3. a scatter writes the permutation and the sorted coordinates;
//   4. bins are cut into subproblems of at most `maxsub` samples (one CTA
//      each in spread / interp), which balances the dense k-space centre of
//      radial and spiral trajectories.
#include "gbn_sort.cuh"

namespace gbn {

__global__ void bin_count_kernel(Geom g, int64_t M, const float* __restrict__ k0,
                                 const float* __restrict__ k1, const float* __restrict__ k2,
                                 int* __restrict__ bin_of, int* __restrict__ rank_of,
                                 int* __restrict__ bin_count) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned active = __ballot_sync(0xffffffffu, j < M);
  if (j >= M) return;
  const float* ks[3] = {k0, k1, k2};
  int b = 0;
  for (int d = 0; d < g.dim; ++d) {
    float u = fold_coord(ks[d][j], g.uscale[d], g.nf[d]);
    int f = cell_of(u, g.nf[d]);
    b = b * g.nb[d] + f / g.bs[d];
  }
  const int lane = threadIdx.x & 31;
  unsigned peers = __match_any_sync(active, b);
  int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&bin_count[b], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  bin_of[j] = b;
  rank_of[j] = base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void scatter_kernel(Geom g, int64_t M, const float* __restrict__ k0,
                               const float* __restrict__ k1, const float* __restrict__ k2,
                               const int* __restrict__ bin_of, const int* __restrict__ rank_of,
                               const int* __restrict__ bin_start, int* __restrict__ perm,
                               float* __restrict__ u0, float* __restrict__ u1,
                               float* __restrict__ u2) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  int pos = bin_start[bin_of[j]] + rank_of[j];
  perm[pos] = (int)j;
  u0[pos] = fold_coord(k0[j], g.uscale[0], g.nf[0]);
  u1[pos] = fold_coord(k1[j], g.uscale[1], g.nf[1]);
  if (g.dim == 3) u2[pos] = fold_coord(k2[j], g.uscale[2], g.nf[2]);
}

__global__ void nsub_kernel(int nbins, const int* __restrict__ bin_count, int maxsub,
                            int* __restrict__ nsub) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  nsub[b] = (bin_count[b] + maxsub - 1) / maxsub;
}

__global__ void fill_sub_kernel(int nbins, const int* __restrict__ bin_count,
                                const int* __restrict__ bin_start,
                                const int* __restrict__ sub_off, int maxsub,
                                int* __restrict__ sub_bin, int* __restrict__ sub_start,
                                int* __restrict__ sub_count) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  int cnt = bin_count[b];
  int off = sub_off[b];
  for (int s = 0; s * maxsub < cnt; ++s) {
    sub_bin[off + s] = b;
    sub_start[off + s] = bin_start[b] + s * maxsub;
    sub_count[off + s] = imin(maxsub, cnt - s * maxsub);
  }
}

// Groups of K consecutive bins along the last axis (bins of one column are
// contiguous in the sorted order): group gi = column * ngz + gz covers the
// bins of layers [gz*K, min(nl, gz*K + K)) of its column.
__global__ void group_kernel(int ngroups, int ngz, int K, int nl, const int* __restrict__ bin_count,
                             const int* __restrict__ bin_start, int* __restrict__ grp_count,
                             int* __restrict__ grp_start) {
  int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= ngroups) return;
  const int col = gi / ngz, gz = gi - col * ngz;
  const int l0 = gz * K;
  const int l1 = imin(nl, l0 + K);
  const int64_t b = (int64_t)col * nl;
  int c = 0;
  for (int l = l0; l < l1; ++l) c += bin_count[b + l];
  grp_count[gi] = c;
  grp_start[gi] = bin_start[b + l0];
}

// ---------------------------------------------------------------------------
// Exclusive scan of int arrays (block scan + scan of block sums + add).
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// exclusive scan of one tile; returns the tile total to thread 0
__device__ int block_excl_scan(int* vals /*kScanItems*/, int* smem /*32*/) {
  int local = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    int v = vals[i];
    vals[i] = local;
    local += v;
  }
  int incl = warp_incl_scan(local);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 31) smem[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int v = lane < (kScanThreads / 32) ? smem[lane] : 0;
    v = warp_incl_scan(v);
    smem[lane] = v;
  }
  __syncthreads();
  int warp_prefix = wid > 0 ? smem[wid - 1] : 0;
  int excl = warp_prefix + incl - local;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) vals[i] += excl;
  int total = smem[(kScanThreads / 32) - 1];
  __syncthreads();
  return total;
}

__global__ void __launch_bounds__(kScanThreads)
scan_tiles_kernel(const int* __restrict__ in, int* __restrict__ out, int n,
                  int* __restrict__ tile_sums) {
  __shared__ int smem[32];
  int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int vals[kScanItems];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) vals[i] = (base + i < n) ? in[base + i] : 0;
  int total = block_excl_scan(vals, smem);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) out[base + i] = vals[i];
  if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = total;
}

__global__ void add_tile_offsets_kernel(int* __restrict__ out, int n,
                                        const int* __restrict__ tile_off) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] += tile_off[i / kScanTile];
}

// total = out[n-1] + in[n-1]
__global__ void scan_total_kernel(const int* in, const int* out, int n, int* total) {
  *total = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

size_t scan_scratch_ints(int n) {
  int tiles = (n + kScanTile - 1) / kScanTile;
  return (size_t)2 * (tiles + 1) + 8;
}

cudaError_t exclusive_scan(const int* in, int* out, int n, int* scratch, int* total,
                           cudaStream_t st) {
  if (n <= 0) return cudaMemsetAsync(total, 0, sizeof(int), st);
  int tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles > kScanTile) return cudaErrorInvalidValue;  // > 16.7 M entries
  int* sums = scratch;
  int* sums_scan = scratch + tiles + 1;
  scan_tiles_kernel<<<tiles, kScanThreads, 0, st>>>(in, out, n, tiles > 1 ? sums : nullptr);
  if (tiles > 1) {
    scan_tiles_kernel<<<1, kScanThreads, 0, st>>>(sums, sums_scan, tiles, nullptr);
    add_tile_offsets_kernel<<<(n + 255) / 256, 256, 0, st>>>(out, n, sums_scan);
  }
  scan_total_kernel<<<1, 1, 0, st>>>(in, out, n, total);
  return cudaGetLastError();
}

cudaError_t build_group_table(int ngroups, int ngz, int K, int nl, int maxsub,
                              const SortBuffers& sb, const GroupBuffers& gb, int* d_total,
                              cudaStream_t st) {
  int bb = (ngroups + 255) / 256;
  group_kernel<<<bb, 256, 0, st>>>(ngroups, ngz, K, nl, sb.bin_count, sb.bin_start, gb.grp_count,
                                   gb.grp_start);
  nsub_kernel<<<bb, 256, 0, st>>>(ngroups, gb.grp_count, maxsub, gb.nsub_grp);
  cudaError_t e = exclusive_scan(gb.nsub_grp, gb.grp_off, ngroups, sb.scan_scratch, d_total, st);
  if (e != cudaSuccess) return e;
  fill_sub_kernel<<<bb, 256, 0, st>>>(ngroups, gb.grp_count, gb.grp_start, gb.grp_off, maxsub,
                                      gb.sub_bin, gb.sub_start, gb.sub_count);
  return cudaGetLastError();
}

cudaError_t sort_points(const Geom& g, int64_t M, const float* const k[3], int maxsub,
                        const SortBuffers& sb, cudaStream_t st, bool subproblems) {
  const int nbins = g.nb[0] * g.nb[1] * g.nb[2];
  cudaError_t e = cudaMemsetAsync(sb.bin_count, 0, sizeof(int) * nbins, st);
  if (e != cudaSuccess) return e;
  const float* k2 = g.dim == 3 ? k[2] : k[1];
  if (M > 0) {
    int blocks = (int)((M + 255) / 256);
    bin_count_kernel<<<blocks, 256, 0, st>>>(g, M, k[0], k[1], k2, sb.bin_of, sb.rank_of,
                                             sb.bin_count);
  }
  e = exclusive_scan(sb.bin_count, sb.bin_start, nbins, sb.scan_scratch, sb.d_total, st);
  if (e != cudaSuccess) return e;
  if (M > 0) {
    int blocks = (int)((M + 255) / 256);
    scatter_kernel<<<blocks, 256, 0, st>>>(g, M, k[0], k[1], k2, sb.bin_of, sb.rank_of,
                                           sb.bin_start, sb.perm, sb.u[0], sb.u[1], sb.u[2]);
  }
  if (!subproblems) return cudaGetLastError();
  int bb = (nbins + 255) / 256;
  nsub_kernel<<<bb, 256, 0, st>>>(nbins, sb.bin_count, maxsub, sb.nsub_bin);
  e = exclusive_scan(sb.nsub_bin, sb.sub_off, nbins, sb.scan_scratch, sb.d_total, st);
  if (e != cudaSuccess) return e;
  fill_sub_kernel<<<bb, 256, 0, st>>>(nbins, sb.bin_count, sb.bin_start, sb.sub_off, maxsub,
                                      sb.sub_bin, sb.sub_start, sb.sub_count);
  return cudaGetLastError();
}

}  // namespace gbn
