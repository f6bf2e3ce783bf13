// Batched execution of many independent NUFFT instances (uneven image size,
// sample count and coil count) in persistent launches driven by work tables.
#pragma once

#include "gbn_internal.cuh"

namespace gbn {

// Everything one instance needs on the device: its geometry, sorted
// trajectory, fine grids and the buffers bound to the batch.
struct BatchInst {
  Geom g;
  Sorted s;
  float2* fine;          // ncoils fine grids
  const float* dec[3];   // 1/phihat per axis
  float2* img;           // SENSE: one image; calibrationless: ncoils images
  const float2* smaps;   // ncoils maps or null
  float2* ksp;           // ncoils x M
  const float* density;  // M or null
  float scale;
  int ncoils;
};

// One unit of work: instance index and a subproblem / block index.
struct WorkItem {
  int inst;
  int idx;
};

struct BatchTables {
  const BatchInst* inst;
  const WorkItem* sub;  int nsub;     // (instance, subproblem)
  const WorkItem* fblk; int nfblk;    // (instance, block of 4096 fine cells)
  const WorkItem* iblk; int niblk;    // (instance, block of 4096 image pixels)
  const WorkItem* sblk; int nsblk;    // (instance, block of 256 sorted samples)
  int dim;
  int w7;                             // every instance has kernel width 7
  int rows;                           // 3D: every tile fits the row spreader
  size_t tile_bytes;                  // largest interp tile
  int grid;                           // persistent CTAs per launch
};

cudaError_t batch_pad(const BatchTables& t, cudaStream_t st);
cudaError_t batch_zero(const BatchTables& t, cudaStream_t st);
cudaError_t batch_interp(const BatchTables& t, cudaStream_t st);
cudaError_t batch_spread(const BatchTables& t, cudaStream_t st);
cudaError_t batch_crop(const BatchTables& t, cudaStream_t st);
cudaError_t batch_prepare(const BatchTables& t);

}  // namespace gbn
