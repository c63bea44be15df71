// Shared device helpers for libskewgpu (sm_103a, FP64).
//
// Cost model this code is written against (measured on GB300): the FP64 pipe of
// an SM sub-partition retires one warp-wide DFMA every 64 cycles (1.19 TFLOP/s
// per GPU), whatever the number of active lanes; a double divide or square
// root costs about ten DFMAs.  So: every FP64 instruction should carry 32
// useful lanes, scalar FP64 work stays off the critical path where it can, and
// integer index arithmetic, loads and shuffles are close to free.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/skewgpu.h"

namespace skew {

constexpr int WARP = 32;

// Negation by flipping the sign bit on the integer pipe (keeps the FP64 pipe free).
__device__ __forceinline__ double neg(double x) {
  return __hiloint2double(__double2hiint(x) ^ 0x80000000, __double2loint(x));
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Block-wide sum for a block of NW warps; red must hold NW doubles. All threads
// get the result.  Contains two __syncthreads().
template <int NW>
__device__ __forceinline__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = x;
  __syncthreads();
  double s = 0;
#pragma unroll
  for (int i = 0; i < NW; i++) s += red[i];
  __syncthreads();
  return s;
}

// Householder reflector parameters following hessenberg.jl:26-44 (householder!):
// beta = -sign(alpha) * hypot(alpha, |x|), tau = 1 - alpha/beta, v = [1; x/(alpha-beta)].
// ss = |x|^2 (sum of squares of the part below alpha); xnorm_scaled >= 0 is |x|
// computed with scaling, supplied by the caller only when ss over/underflowed
// (then hypot is used, as the reference does).  One division is shared by tau
// and the scale: with d = alpha - beta and r = 1/(beta*d), 1/beta = d*r and
// 1/d = beta*r.
struct Reflector {
  double tau, beta, scale;
};
__device__ __forceinline__ bool ss_needs_scaling(double ss) { return !(ss < 1e290) || (ss > 0.0 && ss < 1e-290); }

__device__ __forceinline__ Reflector make_reflector(double alpha, double ss, double xnorm_scaled) {
  Reflector R;
  if (ss == 0.0 && alpha == 0.0) {  // :38-41
    R.tau = 0.0;
    R.beta = 0.0;
    R.scale = 0.0;
    return R;
  }
  double h;
  if (xnorm_scaled < 0.0 && fabs(alpha) < 1e145) {
    h = sqrt(fma(alpha, alpha, ss));
  } else {
    h = hypot(alpha, xnorm_scaled < 0.0 ? sqrt(ss) : xnorm_scaled);
  }
  const double beta = alpha > 0.0 ? neg(h) : h;  // :33
  const double d = alpha - beta;                 // never cancels: beta has the opposite sign
  if (fabs(h) < 1e150 && fabs(h) > 1e-150) {
    const double r = 1.0 / (beta * d);
    R.tau = neg(d * (d * r));  // 1 - alpha/beta = -d/beta
    R.scale = beta * r;        // 1/(alpha - beta)
  } else {
    R.tau = 1.0 - alpha / beta;
    R.scale = 1.0 / d;
  }
  R.beta = beta;
  return R;
}

// Sum over the 32 lanes of 32 per-lane values at once (butterfly transpose):
// on return lane L holds sum_lanes v[L].  31 adds instead of 32 x 5.
__device__ __forceinline__ double warp_transpose_sum32(double (&v)[32]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = lane & s;
#pragma unroll
    for (int i = 0; i < s; i++) {
      const double send = up ? v[i] : v[i + s];
      const double keep = up ? v[i + s] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  return v[0];
}

// Reduce per-thread partial values part[0..npair) (npair <= 32) over the block
// into out[0..npair); scratch holds NW*32 doubles.
template <int NT>
__device__ void block_reduce_pairs(double (&part)[32], int npair, double* scratch, double* out) {
  constexpr int NW = NT / 32;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double mine = warp_transpose_sum32(part);  // lane L holds the warp's sum for slot L
  scratch[w * 32 + lane] = mine;
  __syncthreads();
  if ((int)threadIdx.x < npair) {
    double acc = 0.0;
#pragma unroll
    for (int q = 0; q < NW; q++) acc += scratch[q * 32 + threadIdx.x];
    out[threadIdx.x] = acc;
  }
  __syncthreads();
}

// Pair (l1 < l2) of 8 columns -> slot; 28 slots.
__device__ __forceinline__ int pair_slot(int l1, int l2) { return l1 * 8 - (l1 * (l1 + 1)) / 2 + (l2 - l1 - 1); }

// Bounded spin on a device flag: returns false if `limit` polls pass first.
__device__ __forceinline__ bool spin_until_geq(const volatile unsigned* flag, unsigned target, long long limit) {
  for (long long it = 0; it < limit; it++) {
    if (*flag >= target) return true;
    __nanosleep(64);
  }
  return false;
}

}  // namespace skew

namespace skew {

// Multisection for the target-th smallest eigenvalue (0-based) of a symmetric
// tridiagonal, given count(x) = number of eigenvalues smaller than x (Sturm).
// Groups of p lanes (p a power of two, p <= 32) share one eigenvalue: each step
// the p lanes count at p interior points of [lo, hi] and the group keeps the
// sub-interval [x_{j-1}, x_j] where x_j is the first point whose count exceeds
// the target, so the bracket count(lo) <= target < count(hi) holds by
// construction.  The interval shrinks (p+1)-fold per step until it is below
// max(2 eps max(|lo|, |hi|), abstol).  All 32 lanes of the warp must call this
// (active = false for a group with nothing to find).  Returns the midpoint.
template <class Count>
__device__ double group_multisect(double lo, double hi, int target, double abstol, int p, bool active, Count count) {
  const int lane = threadIdx.x & 31;
  const int g = lane / p, gl = lane - g * p;
  const unsigned gmask = (p == 32) ? 0xffffffffu : (((1u << p) - 1u) << (g * p));
  const double inv = 1.0 / (double)(p + 1);
  bool run = active;
  for (int it = 0; it < 256; it++) {
    const double w = hi - lo;
    if (run && !(w > fmax(2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)), abstol))) run = false;
    if (!__any_sync(0xffffffffu, run)) break;
    const double x = lo + w * ((double)(gl + 1) * inv);
    const bool below = run ? (count(x) <= target) : true;
    const unsigned bits = __ballot_sync(0xffffffffu, below) & gmask;
    if (run) {
      const unsigned above = ~bits & gmask;  // points whose count exceeds the target
      const int j = above ? (__ffs(above) - 1 - g * p) : p;  // first such point (p: none)
      const double nlo = (j == 0) ? lo : lo + w * ((double)j * inv);
      const double nhi = (j == p) ? hi : lo + w * ((double)(j + 1) * inv);
      lo = nlo;
      hi = nhi;
    }
  }
  return 0.5 * (lo + hi);
}

// lanes per eigenvalue for m eigenvalues on a GPU with `sms` SMs: enough groups
// to give every SM sub-partition a warp, at most a warp per eigenvalue
__host__ __device__ inline int multisect_lanes(int m, int sms) {
  const long long want = (long long)sms * 4 * 32 / (m > 0 ? m : 1);
  int p = 1;
  while (p < 32 && 2LL * p <= want) p *= 2;
  return p;
}

}  // namespace skew
