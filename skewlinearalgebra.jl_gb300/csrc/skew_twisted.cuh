// Twisted-factorisation eigenvector of one symmetric tridiagonal (diagonal dg,
// or zero if dg is null; off-diagonal e) for an eigenvalue sig, computed by one
// thread.  Used by the whole-GPU kernels of skew_tdvec.cu and by the per-matrix
// stagnation fallback of skew_eigen.cu.
//
//   pass 1: the stationary pivots D+ of T - sig I = L+ D+ L+^T (top-down), stored;
//   pass 2: the progressive pivots D- of T - sig I = U- D- U-^T (bottom-up), stored,
//           and the twist r = argmin |gamma_r|, gamma_r = D+_r + D-_r - (T_rr - sig);
//   pass 3: z_r = 1, z_i = -(e_i / D+_i) z_{i+1} above r, z_{i+1} = -(e_i / D-_{i+1}) z_i
//           below (a zero neighbour falls back on the three-term relation of the
//           row between).
// (Dhillon and Parlett's twisted factorisation, without relatively robust
// representations.)  Pivots below pivmin in magnitude are replaced by -pivmin.
//
// Each lane works on its own block of rows [lo, hi): where the tridiagonal
// splits (e_i = 0), an eigenvalue shared by several blocks gets one vector per
// block (tdvec_block assigns the blocks).  Rows outside the block are zero.
// The 32 lanes of a warp walk the union of their blocks in lockstep, so that
// without splits every load and store is a whole line.
// Storage is interleaved: entry i of the vector of thread k at [i * KP + k] (32
// consecutive k per warp).  All 32 lanes must call this together (warp
// shuffles).  Returns sum of z_i^2.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"

namespace skew {

constexpr int TW_PF = 8;  // rows prefetched per chunk

__device__ __forceinline__ int warp_min_int(int x) {
  for (int o = 16; o > 0; o >>= 1) x = min(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}
__device__ __forceinline__ int warp_max_int(int x) {
  for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Sturm count restricted to rows [lo, hi): eigenvalues of that block below x.
__device__ __forceinline__ int block_sturm(const double* __restrict__ e, const double* __restrict__ dg, int lo, int hi,
                                           double x, double pivmin) {
  double q = (dg ? dg[lo] : 0.0) - x;
  if (fabs(q) <= pivmin) q = neg(pivmin);
  int c = (q < 0.0);
  for (int i = lo + 1; i < hi; i++) {
    const double ei = e[i - 1];
    q = ((dg ? dg[i] : 0.0) - x) - (ei * ei) / q;
    if (fabs(q) <= pivmin) q = neg(pivmin);
    c += (q < 0.0);
  }
  return c;
}

// The block of rows for the j-th copy (0-based) of an eigenvalue sig: blocks
// are the maximal row ranges joined by nonzero e_i; the blocks holding an
// eigenvalue within [sig - delta, sig + delta] are taken in order and the j-th
// such eigenvalue decides.  Without splits this is [0, n).
__device__ __forceinline__ void tdvec_block(const double* __restrict__ e, const double* __restrict__ dg, int n,
                                            double sig, double delta, int j, double pivmin, int* lo_out,
                                            int* hi_out) {
  int lo = 0, cum = 0;
  for (int i = 0; i < n; i++) {
    if (i + 1 < n && e[i] != 0.0) continue;
    const int hi = i + 1;  // block [lo, hi)
    if (lo == 0 && hi == n) break;
    const int c = block_sturm(e, dg, lo, hi, sig + delta, pivmin) - block_sturm(e, dg, lo, hi, sig - delta, pivmin);
    if (cum + c > j) {
      *lo_out = lo;
      *hi_out = hi;
      return;
    }
    cum += c;
    lo = hi;
  }
  *lo_out = 0;
  *hi_out = n;
}

__device__ __forceinline__ double twisted_vector(const double* __restrict__ e, const double* __restrict__ dg, int n,
                                                 double sig, double pivmin, int64_t KP, int k, int lo, int hi,
                                                 double* __restrict__ dp, double* __restrict__ dm,
                                                 double* __restrict__ z) {
  const double nsig = neg(sig);
#define TW_DIAG(i) (dg ? dg[i] - sig : nsig)
  const int lomin = warp_min_int(lo), himax = warp_max_int(hi);
  if (lo > 0 || hi < n)  // rows outside the block are zero
    for (int i = 0; i < n; i++)
      if (i < lo || i >= hi) z[(int64_t)i * KP + k] = 0.0;

  // pass 1: T - sigma I = L+ D+ L+^T on [lo, hi), D+ stored
  double d = 0.0;
  for (int i = lomin; i < himax; i++) {
    if (i == lo) d = TW_DIAG(lo);
    if (i >= lo && i < hi) {
      if (fabs(d) <= pivmin) d = neg(pivmin);
      dp[(int64_t)i * KP + k] = d;
      if (i + 1 < hi) {
        const double ei = e[i];
        d = TW_DIAG(i + 1) - (ei * ei) / d;
      }
    }
  }
  // pass 2: T - sigma I = U- D- U-^T (bottom-up), D- stored; twist r = argmin |gamma|
  double best = INFINITY;
  int r = hi - 1;
  {
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) {
      const int i = himax - 1 - j;
      cur[j] = (i >= lo && i < hi) ? dp[(int64_t)i * KP + k] : 0.0;
    }
    for (int i0 = himax - 1; i0 >= lomin; i0 -= TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - TW_PF - j;
        nxt[j] = (i >= lo && i < hi) ? dp[(int64_t)i * KP + k] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - j;
        if (i == hi - 1) d = TW_DIAG(hi - 1);
        if (i >= lo && i < hi) {
          if (fabs(d) <= pivmin) d = neg(pivmin);
          dm[(int64_t)i * KP + k] = d;
          const double g = fabs(cur[j] + d - TW_DIAG(i));  // gamma_i = D+_i + D-_i - (T_ii - sigma)
          if (g < best) {
            best = g;
            r = i;
          }
          if (i > lo) {
            const double ei = e[i - 1];
            d = TW_DIAG(i - 1) - (ei * ei) / d;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) cur[j] = nxt[j];
    }
  }
  // pass 3: z_r = 1; z_i = -(e_i / D+_i) z_{i+1} above r, z_{i+1} = -(e_i / D-_{i+1}) z_i below.
  // A zero neighbour falls back on the three-term relation of the row between.
  z[(int64_t)r * KP + k] = 1.0;
  double nrm = 1.0;
  const int rmax = warp_max_int(r), rmin = warp_min_int(r);
  {  // top part, rows rmax-1 .. lomin in lockstep, lanes active on [lo, r)
    double z1 = 1.0, z2 = 0.0;
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) {
      const int i = rmax - 1 - j;
      cur[j] = (i >= lo && i < r) ? dp[(int64_t)i * KP + k] : 1.0;
    }
    for (int i0 = rmax - 1; i0 >= lomin; i0 -= TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - TW_PF - j;
        nxt[j] = (i >= lo && i < r) ? dp[(int64_t)i * KP + k] : 1.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - j;
        if (i >= lo && i < r) {
          const double ei = e[i];
          double zi;
          if (z1 != 0.0)
            zi = neg(ei / cur[j]) * z1;
          else
            zi = (ei != 0.0) ? neg(e[i + 1] / ei) * z2 : 0.0;
          z[(int64_t)i * KP + k] = zi;
          nrm = fma(zi, zi, nrm);
          z2 = z1;
          z1 = zi;
        }
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) cur[j] = nxt[j];
    }
  }
  {  // bottom part, rows rmin+1 .. himax-1, lanes active on (r, hi)
    double z1 = 1.0, z0 = 0.0;  // z_i, z_{i-1}
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) {
      const int i = rmin + j;
      cur[j] = (i >= r && i + 1 < hi) ? dm[(int64_t)(i + 1) * KP + k] : 1.0;
    }
    for (int i0 = rmin; i0 <= himax - 2; i0 += TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 + TW_PF + j;
        nxt[j] = (i >= r && i + 1 < hi) ? dm[(int64_t)(i + 1) * KP + k] : 1.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 + j;
        if (i >= r && i + 1 < hi) {
          const double ei = e[i];
          double zn;
          if (z1 != 0.0)
            zn = neg(ei / cur[j]) * z1;
          else
            zn = (ei != 0.0 && i > lo) ? neg(e[i - 1] / ei) * z0 : 0.0;
          z[(int64_t)(i + 1) * KP + k] = zn;
          nrm = fma(zn, zn, nrm);
          z0 = z1;
          z1 = zn;
        }
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) cur[j] = nxt[j];
    }
  }
#undef TW_DIAG
  return nrm;
}

}  // namespace skew
