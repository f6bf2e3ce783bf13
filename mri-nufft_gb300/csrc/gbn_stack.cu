// Stacked NUFFT z-axis passes (stack-of-stars / stack-of-spirals).
//
// mri-nufft's stacked operator (src/mrinufft/operators/stacked.py:178-330)
// applies, per coil, a centred orthonormal DFT along the last image axis
// (fftshift(fft(ifftshift(x), norm="ortho")) / sqrt(2)), keeps the z_index
// planes, and runs a 2D NUFFT on every kept plane of every coil; the adjoint
// scatters the planes back, inverts the DFT and combines the coils.  Here
// the passes around cuFFT are fused kernels:
//   forward: pad    P[c][x][y][(z - h) mod Nz] = (s_c x)[x][y][z]   (h = Nz/2)
//            cuFFT along z (C Nx Ny transforms of Nz contiguous cells)
//            gather out[c NZ + k][x][y] = P[c][x][y][(zi_k - h) mod Nz] / sqrt(2 Nz)
//   adjoint: scatter (zero P, then the kept planes / sqrt(2 Nz)),
//            inverse cuFFT along z,
//            crop  img[x][y][z] = sum_c conj(s_c) P[c][x][y][(z - h) mod Nz]
//            (calibless: one image per coil).
#include <cufft.h>

#include <cmath>
#include <map>
#include <string>
#include <vector>

#include "gbnufft.h"
#include "gbn_internal.cuh"

namespace gbn {
namespace {

struct StackGeom {
  int nx, ny, nz;  // image shape (z is the stacked, last axis)
  int nzi;         // kept planes
  int64_t nxy;     // nx * ny
  int64_t nimg;    // nx * ny * nz
};

__device__ __forceinline__ float2 cmul_(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc_(float2 a, float2 b) {  // conj(a) * b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// one thread per (c, x, y, z) cell of the padded stack
__global__ void stack_pad_kernel(StackGeom g, const float2* __restrict__ img,
                                 const float2* __restrict__ smaps, float2* __restrict__ P, int C) {
  const int64_t total = (int64_t)C * g.nimg;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / g.nimg;
    const int64_t r = i - c * g.nimg;  // (x, y, z) of the image, z fastest
    const int z = (int)(r % g.nz);
    const int64_t col = r / g.nz;
    float2 v;
    if (smaps) v = cmul_(img[r], smaps[i]);
    else v = img[i];
    int zz = z - g.nz / 2;
    if (zz < 0) zz += g.nz;
    P[(c * g.nxy + col) * g.nz + zz] = v;
  }
}

// one thread per (c, k, x, y) output cell
__global__ void stack_gather_kernel(StackGeom g, const float2* __restrict__ P,
                                    const int* __restrict__ zpos, float2* __restrict__ out, int C,
                                    float scale) {
  const int64_t total = (int64_t)C * g.nzi * g.nxy;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t plane = i / g.nxy;  // c * nzi + k
    const int64_t col = i - plane * g.nxy;
    const int64_t c = plane / g.nzi;
    const int k = (int)(plane - c * g.nzi);
    const float2 v = P[(c * g.nxy + col) * g.nz + zpos[k]];
    out[i] = make_float2(v.x * scale, v.y * scale);
  }
}

// adjoint of the gather: P (zeroed by the caller) at the kept planes
__global__ void stack_scatter_kernel(StackGeom g, const float2* __restrict__ in,
                                     const int* __restrict__ zpos, float2* __restrict__ P, int C,
                                     float scale) {
  const int64_t total = (int64_t)C * g.nzi * g.nxy;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t plane = i / g.nxy;
    const int64_t col = i - plane * g.nxy;
    const int64_t c = plane / g.nzi;
    const int k = (int)(plane - c * g.nzi);
    const float2 v = in[i];
    P[(c * g.nxy + col) * g.nz + zpos[k]] = make_float2(v.x * scale, v.y * scale);
  }
}

// adjoint of the pad: coil combine (SENSE) or per-coil images
__global__ void stack_crop_kernel(StackGeom g, const float2* __restrict__ P,
                                  const float2* __restrict__ smaps, float2* __restrict__ img, int C,
                                  int accumulate) {
  const int64_t total = smaps ? g.nimg : (int64_t)C * g.nimg;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c0 = smaps ? 0 : i / g.nimg;
    const int64_t r = i - c0 * g.nimg;
    const int z = (int)(r % g.nz);
    const int64_t col = r / g.nz;
    int zz = z - g.nz / 2;
    if (zz < 0) zz += g.nz;
    float2 acc;
    if (smaps) {
      acc = make_float2(0.f, 0.f);
      for (int c = 0; c < C; ++c) {
        const float2 p = cmulc_(smaps[(int64_t)c * g.nimg + r], P[((int64_t)c * g.nxy + col) * g.nz + zz]);
        acc.x += p.x;
        acc.y += p.y;
      }
    } else {
      acc = P[(c0 * g.nxy + col) * g.nz + zz];
    }
    if (accumulate) {
      const float2 o = img[i];
      acc.x += o.x;
      acc.y += o.y;
    }
    img[i] = acc;
  }
}

unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 64) b = 152 * 64;
  return (unsigned)b;
}

}  // namespace
}  // namespace gbn

using namespace gbn;

struct gbn_stack_s {
  StackGeom g{};
  int device = 0;
  int* zpos = nullptr;     // kept planes as positions in the shifted z axis
  float2* P = nullptr;     // C x nx x ny x nz work stack
  int64_t pcap = 0;        // cells of P
  std::map<int, cufftHandle> ffts;
  ~gbn_stack_s() {
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device) cudaSetDevice(device);
    for (auto& kv : ffts) cufftDestroy(kv.second);
    if (zpos) cudaFree(zpos);
    if (P) cudaFree(P);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
  }
};

namespace {

int stack_fail(int code, const std::string& msg) {
  set_last_error(msg.c_str());
  return code;
}

int ck_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GBN_OK;
  cudaGetLastError();
  return stack_fail(e == cudaErrorMemoryAllocation ? GBN_ERR_NOMEM : GBN_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

struct DevSwitch {
  int prev = -1;
  explicit DevSwitch(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DevSwitch() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

// work stack and z-FFT plan for C coils
int stack_prepare(gbn_stack s, int C, cufftHandle* plan) {
  const int64_t need = (int64_t)C * s->g.nimg;
  if (need > s->pcap) {
    if (s->P) cudaFree(s->P);
    s->P = nullptr;
    s->pcap = 0;
    int rc = ck_cuda(cudaMalloc(&s->P, sizeof(float2) * need), "stack work array");
    if (rc) return rc;
    s->pcap = need;
  }
  auto it = s->ffts.find(C);
  if (it == s->ffts.end()) {
    cufftHandle h;
    int n[1] = {s->g.nz};
    const int64_t batch = (int64_t)C * s->g.nxy;
    if (batch > 0x7fffffff) return stack_fail(GBN_ERR_ARG, "stack too large for one z-FFT plan");
    cufftResult r = cufftPlanMany(&h, 1, n, nullptr, 1, s->g.nz, nullptr, 1, s->g.nz, CUFFT_C2C,
                                  (int)batch);
    if (r != CUFFT_SUCCESS)
      return stack_fail(r == CUFFT_ALLOC_FAILED ? GBN_ERR_NOMEM : GBN_ERR_CUFFT,
                        "cufftPlanMany (stack z-FFT): error " + std::to_string((int)r));
    it = s->ffts.emplace(C, h).first;
  }
  *plan = it->second;
  return GBN_OK;
}

int exec_z(cufftHandle h, float2* P, int dir, cudaStream_t st) {
  cufftResult r = cufftSetStream(h, st);
  if (r == CUFFT_SUCCESS)
    r = cufftExecC2C(h, reinterpret_cast<cufftComplex*>(P), reinterpret_cast<cufftComplex*>(P), dir);
  if (r != CUFFT_SUCCESS) return stack_fail(GBN_ERR_CUFFT, "cufftExecC2C (stack z-FFT): error " + std::to_string((int)r));
  return GBN_OK;
}

}  // namespace

extern "C" {

int gbn_stack_create(const int64_t* shape, const int* z_index, int n_index, int device,
                     gbn_stack* out) {
  if (!out || !shape || (!z_index && n_index > 0) || n_index < 1)
    return stack_fail(GBN_ERR_ARG, "invalid stack arguments");
  *out = nullptr;
  for (int d = 0; d < 3; ++d)
    if (shape[d] < 1 || shape[d] > (1 << 20)) return stack_fail(GBN_ERR_ARG, "stack shape out of range");
  const int nz = (int)shape[2];
  std::vector<int> pos(n_index);
  for (int k = 0; k < n_index; ++k) {
    if (z_index[k] < 0 || z_index[k] >= nz) return stack_fail(GBN_ERR_ARG, "z_index out of range");
    int p = z_index[k] - nz / 2;  // frequency of the shifted index, as a DFT bin
    pos[k] = p < 0 ? p + nz : p;
  }
  DevSwitch dg(device);
  gbn_stack s = new gbn_stack_s();
  s->device = device;
  s->g.nx = (int)shape[0];
  s->g.ny = (int)shape[1];
  s->g.nz = nz;
  s->g.nzi = n_index;
  s->g.nxy = shape[0] * shape[1];
  s->g.nimg = s->g.nxy * nz;
  int rc = ck_cuda(cudaMalloc(&s->zpos, sizeof(int) * n_index), "stack z positions");
  if (!rc)
    rc = ck_cuda(cudaMemcpy(s->zpos, pos.data(), sizeof(int) * n_index, cudaMemcpyHostToDevice),
                 "stack z positions");
  if (rc) {
    delete s;
    return rc;
  }
  *out = s;
  return GBN_OK;
}

int gbn_stack_fwd(gbn_stack s, const void* img, const void* smaps, void* out, int C,
                  gbn_stream stream) {
  if (!s || !img || !out || C < 1) return stack_fail(GBN_ERR_ARG, "invalid stack arguments");
  DevSwitch dg(s->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cufftHandle h;
  int rc = stack_prepare(s, C, &h);
  if (rc) return rc;
  const StackGeom& g = s->g;
  stack_pad_kernel<<<blocks_for((int64_t)C * g.nimg), 256, 0, st>>>(
      g, static_cast<const float2*>(img), static_cast<const float2*>(smaps), s->P, C);
  if ((rc = ck_cuda(cudaGetLastError(), "stack pad"))) return rc;
  if ((rc = exec_z(h, s->P, CUFFT_FORWARD, st))) return rc;
  const float scale = (float)(1.0 / std::sqrt(2.0 * g.nz));
  stack_gather_kernel<<<blocks_for((int64_t)C * g.nzi * g.nxy), 256, 0, st>>>(
      g, s->P, s->zpos, static_cast<float2*>(out), C, scale);
  return ck_cuda(cudaGetLastError(), "stack gather");
}

int gbn_stack_adj(gbn_stack s, const void* in, const void* smaps, void* img, int C, int accumulate,
                  gbn_stream stream) {
  if (!s || !in || !img || C < 1) return stack_fail(GBN_ERR_ARG, "invalid stack arguments");
  DevSwitch dg(s->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cufftHandle h;
  int rc = stack_prepare(s, C, &h);
  if (rc) return rc;
  const StackGeom& g = s->g;
  if ((rc = ck_cuda(cudaMemsetAsync(s->P, 0, sizeof(float2) * (size_t)C * g.nimg, st), "stack zero")))
    return rc;
  const float scale = (float)(1.0 / std::sqrt(2.0 * g.nz));
  stack_scatter_kernel<<<blocks_for((int64_t)C * g.nzi * g.nxy), 256, 0, st>>>(
      g, static_cast<const float2*>(in), s->zpos, s->P, C, scale);
  if ((rc = ck_cuda(cudaGetLastError(), "stack scatter"))) return rc;
  if ((rc = exec_z(h, s->P, CUFFT_INVERSE, st))) return rc;
  const int64_t n = smaps ? g.nimg : (int64_t)C * g.nimg;
  stack_crop_kernel<<<blocks_for(n), 256, 0, st>>>(g, s->P, static_cast<const float2*>(smaps),
                                                   static_cast<float2*>(img), C, accumulate);
  return ck_cuda(cudaGetLastError(), "stack crop");
}

int gbn_stack_destroy(gbn_stack s) {
  delete s;
  return GBN_OK;
}

}  // extern "C"
