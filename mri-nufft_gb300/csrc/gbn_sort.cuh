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

// A subproblem table over groups of consecutive bins along the last axis.
struct GroupBuffers {
  int* grp_count;   // ngroups
  int* grp_start;   // ngroups
  int* nsub_grp;    // ngroups
  int* grp_off;     // ngroups
  int* sub_bin;     // subproblem -> group
  int* sub_start;
  int* sub_count;
};

size_t scan_scratch_ints(int n);
// Builds gb's subproblem table (chunks of <= maxsub samples per group) from a
// finished sort; d_total receives the number of subproblems.
cudaError_t build_group_table(int ngroups, int ngz, int K, int nl, int maxsub,
                              const SortBuffers& sb, const GroupBuffers& gb, int* d_total,
                              cudaStream_t st);
cudaError_t exclusive_scan(const int* in, int* out, int n, int* scratch, int* total,
                           cudaStream_t st);
// Sorts M points with coordinates k[d] (radians, device float32) by the bins
// of g.  With `subproblems`, also cuts every bin into subproblems of at most
// maxsub samples; on return (stream-ordered) sb.d_total holds their number.
cudaError_t sort_points(const Geom& g, int64_t M, const float* const k[3], int maxsub,
                        const SortBuffers& sb, cudaStream_t st, bool subproblems);

}  // namespace gbn
