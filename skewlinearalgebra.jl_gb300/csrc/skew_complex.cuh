// ComplexF64 helpers for the complex skew-Hermitian kernels (interleaved re, im:
// the layout of Julia's ComplexF64 and of CUDA's double2).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "skew_common.cuh"

namespace skew {

struct __align__(16) zc {
  double re, im;
};

__device__ __forceinline__ zc zadd(zc a, zc b) { return zc{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ zc zsub(zc a, zc b) { return zc{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ zc zconj(zc a) { return zc{a.re, neg(a.im)}; }
// a * b
__device__ __forceinline__ zc zmul(zc a, zc b) {
  return zc{fma(a.re, b.re, -(a.im * b.im)), fma(a.re, b.im, a.im * b.re)};
}
// a * conj(b)
__device__ __forceinline__ zc zmulc(zc a, zc b) {
  return zc{fma(a.re, b.re, a.im * b.im), fma(a.im, b.re, -(a.re * b.im))};
}
// conj(a) * b
__device__ __forceinline__ zc zcmul(zc a, zc b) {
  return zc{fma(a.re, b.re, a.im * b.im), fma(a.re, b.im, -(a.im * b.re))};
}
// a * b + c
__device__ __forceinline__ zc zfma(zc a, zc b, zc c) {
  return zc{fma(a.re, b.re, fma(neg(a.im), b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im))};
}
// 1 / b with the components scaled by max(|re|, |im|) first (no overflow of |b|^2)
__device__ __forceinline__ zc zinv(zc b) {
  const double s = fmax(fabs(b.re), fabs(b.im));
  if (s == 0.0) return zc{INFINITY, 0.0};
  const double br = b.re / s, bi = b.im / s;
  const double d = fma(br, br, bi * bi) * s;
  return zc{br / d, neg(bi) / d};
}

}  // namespace skew
