// Fused pad / crop passes and FP64 reductions.
#pragma once

#include "gbn_internal.cuh"

namespace gbn {

struct PadArgs {
  Geom g;
  const float2* img;    // SENSE: one image; calibrationless: ntr images
  const float2* smaps;  // SENSE: ntr coil maps (null: calibrationless)
  const float* dec[3];  // 1/phihat per axis, indexed by image array index
  float2* fine;         // ntr fine grids (every cell written)
  int ntr;
  int conj_in;          // use conj(img) and conj(smaps)
  float scale;
};

struct CropArgs {
  Geom g;
  const float2* fine;   // ntr fine grids
  const float2* smaps;  // SENSE coil maps (null: calibrationless)
  const float* dec[3];
  float2* out;          // SENSE: one image; calibrationless: ntr images
  int ntr;
  int accumulate;       // SENSE: out += result
  float scale;
};

cudaError_t launch_pad(const PadArgs& a, cudaStream_t st);
cudaError_t launch_crop(const CropArgs& a, cudaStream_t st);
cudaError_t launch_norm2(const float2* x, int64_t n, double* out, cudaStream_t st);
cudaError_t launch_dotu(const float2* a, const float2* b, int64_t n, int conj_a, double* out,
                        cudaStream_t st);

}  // namespace gbn
