// Complex helpers and in-register 4- and 16-point DFTs shared by the fused
// line transforms (gbn_fft256.cu, gbn_fft512.cu).  Exponent sign -1
// throughout; a +1 transform conjugates its inputs and outputs.
#pragma once

#include <cuda_runtime.h>

namespace gbn {
namespace dft {

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 f2conj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 f2scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// 4-point DFT, exponent sign -1, in place
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = f2add(a0, a2), t1 = f2sub(a0, a2), t2 = f2add(a1, a3), t3 = f2sub(a1, a3);
  a0 = f2add(t0, t2);
  a2 = f2sub(t0, t2);
  a1 = make_float2(t1.x + t3.y, t1.y - t3.x);  // t1 - i t3
  a3 = make_float2(t1.x - t3.y, t1.y + t3.x);  // t1 + i t3
}

// 4-point DFT whose inputs a1, a2 are zero (not read)
__device__ __forceinline__ void dft4_in03(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 p = a0, q = a3;
  a0 = f2add(p, q);
  a2 = f2sub(p, q);
  a1 = make_float2(p.x - q.y, p.y + q.x);  // p + i q
  a3 = make_float2(p.x + q.y, p.y - q.x);  // p - i q
}

// 4-point DFT of which only the outputs a0, a3 are used (a1, a2 are left stale)
__device__ __forceinline__ void dft4_out03(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 t0 = f2add(a0, a2), t1 = f2sub(a0, a2), t2 = f2add(a1, a3), t3 = f2sub(a1, a3);
  a0 = f2add(t0, t2);
  a3 = make_float2(t1.x - t3.y, t1.y + t3.x);
}

// 16-point DFT, exponent sign -1: x[n] in natural order in, X[k] at x[pos16(k)] out.
// HALF_IN: x[4 .. 11] are zero and not read (the inputs of a 128-mode axis,
// n = 16 q + b with q < 4 or q >= 12); HALF_OUT: only X[k], k < 4 or k >= 12,
// are computed (the outputs such an axis keeps).  The IEEE arithmetic does
// not let the compiler drop additions of constant zeros by itself.
__device__ __forceinline__ int pos16(int k) { return 4 * (k & 3) + (k >> 2); }

template <bool HALF_IN = false, bool HALF_OUT = false>
__device__ __forceinline__ void dft16(float2 (&x)[16]) {
  // W16^k = (cos(2 pi k / 16), -sin(2 pi k / 16))
  constexpr float c1 = 0.92387953251128674f;  // cos(pi / 8)
  constexpr float s1 = 0.38268343236508977f;  // sin(pi / 8)
  constexpr float r2 = 0.70710678118654752f;  // sqrt(1 / 2)
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    if (HALF_IN) dft4_in03(x[r], x[r + 4], x[r + 8], x[r + 12]);
    else dft4(x[r], x[r + 4], x[r + 8], x[r + 12]);
  }
  // x[r + 4 s] *= W16^(r s)
  x[5] = f2mul(x[5], make_float2(c1, -s1));    // r 1, s 1
  x[9] = f2mul(x[9], make_float2(r2, -r2));    // r 1, s 2
  x[13] = f2mul(x[13], make_float2(s1, -c1));  // r 1, s 3
  x[6] = f2mul(x[6], make_float2(r2, -r2));    // r 2, s 1
  x[10] = make_float2(x[10].y, -x[10].x);      // r 2, s 2: W16^4 = -i
  x[14] = f2mul(x[14], make_float2(-r2, -r2)); // r 2, s 3: W16^6
  x[7] = f2mul(x[7], make_float2(s1, -c1));    // r 3, s 1: W16^3
  x[11] = f2mul(x[11], make_float2(-r2, -r2)); // r 3, s 2: W16^6
  x[15] = f2mul(x[15], make_float2(-c1, s1));  // r 3, s 3: W16^9
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (HALF_OUT) dft4_out03(x[4 * s], x[4 * s + 1], x[4 * s + 2], x[4 * s + 3]);
    else dft4(x[4 * s], x[4 * s + 1], x[4 * s + 2], x[4 * s + 3]);
  }
}

}  // namespace dft
}  // namespace gbn
