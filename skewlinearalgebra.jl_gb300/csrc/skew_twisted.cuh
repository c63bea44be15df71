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
// Storage is interleaved: entry i of the vector of thread k at [i * KP + k], so
// the 32 lanes of a warp (32 consecutive k) read and write whole lines; all 32
// lanes must call this together (warp shuffles).  Returns sum of z_i^2.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"

namespace skew {

constexpr int TW_PF = 8;  // rows prefetched per chunk

__device__ __forceinline__ double twisted_vector(const double* __restrict__ e, const double* __restrict__ dg, int n,
                                                 double sig, double pivmin, int64_t KP, int k,
                                                 double* __restrict__ dp, double* __restrict__ dm,
                                                 double* __restrict__ z) {
  const double nsig = neg(sig);
#define TW_DIAG(i) (dg ? dg[i] - sig : nsig)

  // pass 1: T - sigma I = L+ D+ L+^T, D+ stored
  double d = TW_DIAG(0);
  for (int i = 0; i < n; i++) {
    if (fabs(d) <= pivmin) d = neg(pivmin);
    dp[(int64_t)i * KP + k] = d;
    if (i + 1 < n) {
      const double ei = e[i];
      d = TW_DIAG(i + 1) - (ei * ei) / d;
    }
  }
  // pass 2: T - sigma I = U- D- U-^T (bottom-up), D- stored; twist r = argmin |gamma|
  double best = INFINITY;
  int r = n - 1;
  d = TW_DIAG(n - 1);
  {
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) cur[j] = (n - 1 - j >= 0) ? dp[(int64_t)(n - 1 - j) * KP + k] : 0.0;
    for (int i0 = n - 1; i0 >= 0; i0 -= TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - TW_PF - j;
        nxt[j] = (i >= 0) ? dp[(int64_t)i * KP + k] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - j;
        if (i >= 0) {
          if (fabs(d) <= pivmin) d = neg(pivmin);
          dm[(int64_t)i * KP + k] = d;
          const double g = fabs(cur[j] + d - TW_DIAG(i));  // gamma_i = D+_i + D-_i - (T_ii - sigma)
          if (g < best) {
            best = g;
            r = i;
          }
          if (i > 0) {
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
  int rmax = r, rmin = r;
  for (int o = 16; o > 0; o >>= 1) {
    rmax = max(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    rmin = min(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
  }
  {  // top part, rows rmax-1 .. 0 in lockstep (coalesced), lanes active below their r
    double z1 = 1.0, z2 = 0.0;
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) cur[j] = (rmax - 1 - j >= 0) ? dp[(int64_t)(rmax - 1 - j) * KP + k] : 1.0;
    for (int i0 = rmax - 1; i0 >= 0; i0 -= TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - TW_PF - j;
        nxt[j] = (i >= 0) ? dp[(int64_t)i * KP + k] : 1.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 - j;
        if (i >= 0 && i < r) {
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
  {  // bottom part, rows rmin+1 .. n-1, lanes active above their r
    double z1 = 1.0, z0 = 0.0;  // z_i, z_{i-1}
    double cur[TW_PF], nxt[TW_PF];
#pragma unroll
    for (int j = 0; j < TW_PF; j++) cur[j] = (rmin + 1 + j < n) ? dm[(int64_t)(rmin + 1 + j) * KP + k] : 1.0;
    for (int i0 = rmin; i0 <= n - 2; i0 += TW_PF) {
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 + TW_PF + j;
        nxt[j] = (i + 1 < n) ? dm[(int64_t)(i + 1) * KP + k] : 1.0;
      }
#pragma unroll
      for (int j = 0; j < TW_PF; j++) {
        const int i = i0 + j;
        if (i <= n - 2 && i >= r) {
          const double ei = e[i];
          double zn;
          if (z1 != 0.0)
            zn = neg(ei / cur[j]) * z1;
          else
            zn = (ei != 0.0 && i > 0) ? neg(e[i - 1] / ei) * z0 : 0.0;
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
