// Persistent batched kernels: a fixed grid of CTAs strides over a work table
// that covers every instance of the batch, so one launch per stage serves all
// instances whatever their sizes (pad, zero, interp, spread, crop).  The
// per-item work is the single-plan kernels' bodies.
#include "gbn_batch.cuh"
#include "gbn_kernels.cuh"
#include "gbn_passes.cuh"

namespace gbn {

namespace {

constexpr int kSampleBlock = 256;                 // samples per sblk item
constexpr int kCellsPerThread = 16;               // fblk / iblk items: 4096 cells
constexpr int kGroupsPerWarp = kSampleBlock / 4 / (GBN_THREADS / 32);  // 4-sample groups

__device__ __forceinline__ PadArgs pad_of(const BatchInst& b) {
  PadArgs a;
  a.g = b.g;
  a.img = b.img;
  a.smaps = b.smaps;
  a.dec[0] = b.dec[0];
  a.dec[1] = b.dec[1];
  a.dec[2] = b.dec[2];
  a.fine = b.fine;
  a.ntr = b.ncoils;
  a.conj_in = 0;
  a.scale = 1.0f;
  return a;
}

template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS) batch_pad_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nfblk; w += gridDim.x) {
    const WorkItem it = t.fblk[w];
    __shared__ PadArgs a;
    __syncthreads();
    if (threadIdx.x == 0) a = pad_of(t.inst[it.inst]);
    __syncthreads();
    const int64_t base = (int64_t)it.idx * GBN_THREADS * kCellsPerThread + threadIdx.x;
#pragma unroll 4
    for (int k = 0; k < kCellsPerThread; ++k) pad_body<DIM>(a, base + (int64_t)k * GBN_THREADS);
  }
}

__global__ void __launch_bounds__(GBN_THREADS) batch_zero_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nfblk; w += gridDim.x) {
    const WorkItem it = t.fblk[w];
    const BatchInst& b = t.inst[it.inst];
    const int64_t G = b.g.G;
    float2* fine = b.fine;
    const int nc = b.ncoils;
    const int64_t base = (int64_t)it.idx * GBN_THREADS * kCellsPerThread + threadIdx.x;
    for (int k = 0; k < kCellsPerThread; ++k) {
      const int64_t idx = base + (int64_t)k * GBN_THREADS;
      if (idx < G)
        for (int c = 0; c < nc; ++c) fine[(int64_t)c * G + idx] = make_float2(0.f, 0.f);
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS) batch_crop_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.niblk; w += gridDim.x) {
    const WorkItem it = t.iblk[w];
    __shared__ CropArgs a;
    __syncthreads();
    if (threadIdx.x == 0) {
      const BatchInst& b = t.inst[it.inst];
      a.g = b.g;
      a.fine = b.fine;
      a.smaps = b.smaps;
      a.dec[0] = b.dec[0];
      a.dec[1] = b.dec[1];
      a.dec[2] = b.dec[2];
      a.out = b.img;
      a.ntr = b.ncoils;
      a.accumulate = 0;
      a.scale = b.scale;
    }
    __syncthreads();
    const int64_t base = (int64_t)it.idx * GBN_THREADS * kCellsPerThread + threadIdx.x;
#pragma unroll 4
    for (int k = 0; k < kCellsPerThread; ++k) crop_body<DIM>(a, base + (int64_t)k * GBN_THREADS);
  }
}

template <int DIM, int W>
__global__ void __launch_bounds__(GBN_THREADS) batch_interp_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nsub; w += gridDim.x) {
    const WorkItem it = t.sub[w];
    const BatchInst& b = t.inst[it.inst];
    InterpArgs a;
    a.g = b.g;
    a.s = b.s;
    a.fine = b.fine;
    a.out = b.ksp;
    a.obs = nullptr;
    a.density = nullptr;
    a.ntr = b.ncoils;
    a.scale = b.scale;
    a.mode = INTERP_STORE;
    interp_body<DIM, W, 1>(a, it.idx);  // ends with a barrier
  }
}

__device__ __forceinline__ SpreadArgs spread_of(const BatchInst& b) {
  SpreadArgs a;
  a.g = b.g;
  a.s = b.s;
  a.in = b.ksp;
  a.density = b.density;
  a.fine = b.fine;
  a.ntr = b.ncoils;
  a.scale = 1.0f;
  return a;
}

template <int DIM, int W>
__global__ void __launch_bounds__(GBN_THREADS) batch_spread_gm_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nsblk; w += gridDim.x) {
    const WorkItem it = t.sblk[w];
    const SpreadArgs a = spread_of(t.inst[it.inst]);
    spread_gm_body<DIM, W>(a, (int64_t)it.idx * kSampleBlock + threadIdx.x);
  }
}

// warp-cooperative kernels over blocks of 32 sorted samples (8 warps x 4)
template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS, 4) batch_interp_wc_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nsblk; w += gridDim.x) {
    const WorkItem it = t.sblk[w];
    // the instance's arguments live in shared memory: the bodies read them
    // at shared-memory (broadcast) cost instead of from spilled registers
    __shared__ InterpArgs a;
    __syncthreads();
    if (threadIdx.x == 0) {
      const BatchInst& b = t.inst[it.inst];
      a.g = b.g;
      a.s = b.s;
      a.fine = b.fine;
      a.out = b.ksp;
      a.obs = nullptr;
      a.density = nullptr;
      a.ntr = b.ncoils;
      a.scale = b.scale;
      a.mode = INTERP_STORE;
    }
    __syncthreads();
    const int64_t w0 = ((int64_t)it.idx * (GBN_THREADS / 32) + (threadIdx.x >> 5)) * kGroupsPerWarp;
    for (int k = 0; k < kGroupsPerWarp; ++k) interp_wc_body<DIM>(a, w0 + k);
  }
}

template <int DIM>
__global__ void __launch_bounds__(GBN_THREADS, 4) batch_spread_wc_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nsblk; w += gridDim.x) {
    const WorkItem it = t.sblk[w];
    __shared__ SpreadArgs a;
    __syncthreads();
    if (threadIdx.x == 0) a = spread_of(t.inst[it.inst]);
    __syncthreads();
    const int64_t w0 = ((int64_t)it.idx * (GBN_THREADS / 32) + (threadIdx.x >> 5)) * kGroupsPerWarp;
    for (int k = 0; k < kGroupsPerWarp; ++k) spread_wc_body<DIM>(a, w0 + k);
  }
}

template <int W>
__global__ void __launch_bounds__(GBN_THREADS, 2) batch_spread_rows_kernel(BatchTables t) {
  for (int w = blockIdx.x; w < t.nsub; w += gridDim.x) {
    const WorkItem it = t.sub[w];
    const SpreadArgs a = spread_of(t.inst[it.inst]);
    spread_rows3d_body<W, 2>(a, it.idx);
    __syncthreads();
  }
}

}  // namespace

cudaError_t batch_prepare(const BatchTables& t) {
  // dynamic shared memory of the interp tiles (set outside any stream capture)
  if (t.dim == 2) {
    if (t.w7) return cudaFuncSetAttribute(batch_interp_kernel<2, 7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.tile_bytes);
    return cudaFuncSetAttribute(batch_interp_kernel<2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.tile_bytes);
  }
  if (t.w7) return cudaFuncSetAttribute(batch_interp_kernel<3, 7>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.tile_bytes);
  return cudaFuncSetAttribute(batch_interp_kernel<3, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.tile_bytes);
}

cudaError_t batch_pad(const BatchTables& t, cudaStream_t st) {
  if (t.nfblk == 0) return cudaSuccess;
  if (t.dim == 2) batch_pad_kernel<2><<<t.grid, GBN_THREADS, 0, st>>>(t);
  else batch_pad_kernel<3><<<t.grid, GBN_THREADS, 0, st>>>(t);
  return cudaGetLastError();
}

cudaError_t batch_zero(const BatchTables& t, cudaStream_t st) {
  if (t.nfblk == 0) return cudaSuccess;
  batch_zero_kernel<<<t.grid, GBN_THREADS, 0, st>>>(t);
  return cudaGetLastError();
}

cudaError_t batch_crop(const BatchTables& t, cudaStream_t st) {
  if (t.niblk == 0) return cudaSuccess;
  if (t.dim == 2) batch_crop_kernel<2><<<t.grid, GBN_THREADS, 0, st>>>(t);
  else batch_crop_kernel<3><<<t.grid, GBN_THREADS, 0, st>>>(t);
  return cudaGetLastError();
}

cudaError_t batch_interp(const BatchTables& t, cudaStream_t st) {
  if (t.dim == 2 && t.w7) {
    if (t.nsblk == 0) return cudaSuccess;
    batch_interp_wc_kernel<2><<<t.grid, GBN_THREADS, 0, st>>>(t);
    return cudaGetLastError();
  }
  if (t.nsub == 0) return cudaSuccess;
  const size_t smem = t.tile_bytes;
  if (t.dim == 2) {
    if (t.w7) batch_interp_kernel<2, 7><<<t.grid, GBN_THREADS, smem, st>>>(t);
    else batch_interp_kernel<2, 0><<<t.grid, GBN_THREADS, smem, st>>>(t);
  } else {
    if (t.w7) batch_interp_kernel<3, 7><<<t.grid, GBN_THREADS, smem, st>>>(t);
    else batch_interp_kernel<3, 0><<<t.grid, GBN_THREADS, smem, st>>>(t);
  }
  return cudaGetLastError();
}

cudaError_t batch_spread(const BatchTables& t, cudaStream_t st) {
  if (t.dim == 3 && t.rows) {
    if (t.nsub == 0) return cudaSuccess;
    if (t.w7) batch_spread_rows_kernel<7><<<t.grid, GBN_THREADS, 0, st>>>(t);
    else batch_spread_rows_kernel<0><<<t.grid, GBN_THREADS, 0, st>>>(t);
  } else {
    if (t.nsblk == 0) return cudaSuccess;
    if (t.w7) {
      if (t.dim == 2) batch_spread_wc_kernel<2><<<t.grid, GBN_THREADS, 0, st>>>(t);
      else batch_spread_wc_kernel<3><<<t.grid, GBN_THREADS, 0, st>>>(t);
    } else {
      // blocks of 32 samples: threads past the block's 32 samples idle
      if (t.dim == 2) batch_spread_gm_kernel<2, 0><<<t.grid, GBN_THREADS, 0, st>>>(t);
      else batch_spread_gm_kernel<3, 0><<<t.grid, GBN_THREADS, 0, st>>>(t);
    }
  }
  return cudaGetLastError();
}

}  // namespace gbn
