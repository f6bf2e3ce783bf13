// Device buffers and entry points of the bin sort.
#pragma once

#include "gbn_internal.cuh"

namespace gbn {

struct SortBuffers {
  int* bin_of;        // M   (scratch)
  int* rank_of;       // M   (scratch)
  int* bin_count;     // nbins
  int* bin_start;     // nbins
  int* nsub_bin;      // nbins
  int* sub_off;       // nbins
  int* scan_scratch;  // scan_scratch_ints(nbins)
  int* d_total;       // 1
  int* perm;          // M
  float* u[3];        // M each (u[2] unused in 2D)
  int* sub_bin;       // subproblem capacity
  int* sub_start;
  int* sub_count;
};

size_t scan_scratch_ints(int n);
cudaError_t exclusive_scan(const int* in, int* out, int n, int* scratch, int* total,
                           cudaStream_t st);
// Sorts M points with coordinates k[d] (radians, device float32).  On return
// (stream-ordered) sb.d_total holds the number of subproblems.
cudaError_t sort_points(const Geom& g, int64_t M, const float* const k[3], int maxsub,
                        const SortBuffers& sb, cudaStream_t st);

}  // namespace gbn
