// Eigenvectors of one large real skew matrix (n > 1024) on the whole GPU.
//
// The reference solves the tridiagonal eigenproblem by implicit QR with the
// rotations accumulated into Qodd / Qeven (skewtrieigen_divided!, skeweigen.jl:
// 322-457) and, when the shifts stagnate, through the symmetric tridiagonal
// SymTridiagonal(0, ev) (skewtrieigen_backup!, skeweigen.jl:470-489).  The QR
// chain is serial (about 2n^2 dependent rotations), which one GPU thread cannot
// run at n = 8192 in reasonable time.  This file computes the same
// decomposition the way the fallback formulates it:
//   1. eigenvalues sigma_k > 0 of SymTridiagonal(0, ev) by bisection (skew_qr.cu),
//      sorted descending (the reference's fallback order: vals = -eigvals(H));
//   2. one eigenvector w_k of SymTridiagonal(0, ev) per sigma_k, one thread
//      each, from the twisted factorisation of T - sigma I: the stationary
//      L D L^T (top-down) and progressive U D U^T (bottom-up) pivots, the twist
//      index r = argmin |gamma_r|, and the vector by the two recurrences out of
//      r (the twisted-factorisation eigenvector of Dhillon and Parlett's MRRR,
//      here without the relatively robust representations);
//   3. the even-row and odd-row parts of the w_k are the left and right singular
//      vectors of the bidiagonal coupling; each set is made orthonormal by one
//      symmetric (Lowdin) correction restricted to a band of LW neighbours in
//      the sorted spectrum, which keeps residuals at the eps level;
//   4. the skew eigenvectors in the tridiagonal basis follow the fallback's
//      pattern (real on odd 1-based rows, imaginary on even rows, sign flipped
//      every pair); the vector of -sigma_k is the conjugate of that of sigma_k;
//   5. back-transformation X <- Q X with the stored reflectors, panel by panel in
//      compact WY form (Q_b = I - V T V^T, dlarft-style T), each CTA owning a
//      strip of 32 columns (no inter-CTA dependence);
//   6. the +sigma columns are mirrored from the -sigma columns (Vr equal, Vi
//      negated).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_internal.h"
#include "skew_twisted.cuh"

namespace skew {

constexpr int TW_NT = 64;  // threads per CTA of the twisted kernel (one vector each)
constexpr int LW = 16;     // half-width of the Lowdin band
constexpr int WB = 64;     // reflectors per compact-WY panel
constexpr int SW = 32;     // columns per back-transformation strip
constexpr int RC = 32;     // rows per staged chunk

struct TdvecLayout {
  int n, h, K, KP;  // n, positive eigenvalues, vectors (h + n odd), padded to 32
  int npan;         // WY panels
  int full;         // 1: general symmetric tridiagonal (diagonal dg), one vector per eigenvalue (K = n)
  const double* dg; // diagonal (full mode) or null (zero diagonal)
  // batches of equal-size problems (full mode): problem mb = blockIdx.z uses the
  // workspace block mb (mstride doubles apart) and inputs mb * (n, n, 8) apart
  size_t mstride;
  double* dp;       // n x KP
  double* dm;       // n x KP
  double* z;        // n x KP
  double* nrm2;     // KP
  double* bandU;    // KP x (LW + 1) raw dots over even rows
  double* bandV;    // KP x (LW + 1) raw dots over odd rows
  double* T;        // npan x WB x WB
  // gate != null: every kernel of the pipeline returns at once unless *gate ==
  // gate_on (two pipelines are queued and the device picks one, no host sync)
  const int* gate;
  int gate_on;
};

// problem mb of the launch (blockIdx.z of the batched kernels, 0 for one matrix)
__device__ __forceinline__ bool gated_off(const TdvecLayout& L, int mb = 0) {
  return L.gate && L.gate[mb] != L.gate_on;
}

size_t large_eigen_ws_doubles(int n);

static TdvecLayout layout(int n, double* ws, bool full = false, const double* dg = nullptr) {
  TdvecLayout L;
  L.n = n;
  L.h = n / 2;
  L.K = full ? n : L.h + (n & 1);
  L.full = full ? 1 : 0;
  L.dg = dg;
  L.mstride = large_eigen_ws_doubles(n);
  L.KP = (L.K + 31) / 32 * 32;
  L.npan = (n - 2 + WB - 1) / WB;
  const size_t big = (size_t)n * L.KP;
  L.dp = ws;
  L.dm = L.dp + big;
  L.z = L.dm + big;
  L.nrm2 = L.z + big;
  L.bandU = L.nrm2 + L.KP;
  L.bandV = L.bandU + (size_t)L.KP * (LW + 1);
  L.T = L.bandV + (size_t)L.KP * (LW + 1);
  L.gate = nullptr;
  L.gate_on = 0;
  return L;
}

size_t large_eigen_ws_doubles(int n) {
  const int KP = (n + 31) / 32 * 32;  // covers both modes (K <= n)
  const int npan = (n - 2 + WB - 1) / WB;
  return 3 * (size_t)n * KP + KP + 2 * (size_t)KP * (LW + 1) + (size_t)std::max(npan, 1) * WB * WB + 64;
}

// the layout of problem mb of a batch (mb = 0: unchanged)
__device__ __forceinline__ TdvecLayout at_problem(TdvecLayout L, int mb) {
  if (mb == 0) return L;
  const size_t o = (size_t)mb * L.mstride;
  L.dp += o;
  L.dm += o;
  L.z += o;
  L.nrm2 += o;
  L.bandU += o;
  L.bandV += o;
  L.T += o;
  if (L.dg) L.dg += (size_t)mb * L.n;
  return L;
}

// ---------------------------------------------------------------------------
// 2. twisted factorisation eigenvectors, one thread per sigma
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TW_NT) twisted_kernel(const double* __restrict__ e, const double* __restrict__ vals,
                                                        const double* __restrict__ bp, TdvecLayout L0) {
  const int mb = blockIdx.z;
  if (gated_off(L0, mb)) return;
  const TdvecLayout L = at_problem(L0, mb);
  e += (size_t)mb * L.n;
  vals += (size_t)mb * L.n;
  bp += (size_t)mb * 8;
  const int k = blockIdx.x * TW_NT + threadIdx.x;
  if (k >= L.KP) return;  // KP is a multiple of 32: whole warps leave together
  const int n = L.n;
  const int64_t KP = L.KP;
  // sigma: the k-th eigenvalue (full mode: ascending list; skew mode: descending
  // positive values, then 0 for odd n); padded lanes solve a dummy vector
  const double sig = L.full ? (k < L.K ? vals[k] : vals[L.K - 1]) : ((k < L.h) ? vals[k] : 0.0);
  const double pivmin = bp[1];
  // copy index j among equal eigenvalues (the list is sorted) -> the block of rows
  const double scale = L.full ? fmax(fabs(bp[0]), fabs(bp[2])) : bp[0];
  // 8 times the bisection tolerance, and above the pivot guard (counts cannot
  // resolve below pivmin: a zero matrix has only eigenvalues there)
  const double delta = fmax(16.0 * 2.220446049250313e-16 * (scale + fabs(sig)), 4.0 * pivmin);
  int lo = 0, hi = n;
  if (k < L.K) {
    int j = 0;
    for (int q = k - 1; q >= 0; q--) {
      const double sq = L.full ? vals[q] : ((q < L.h) ? vals[q] : 0.0);
      if (fabs(sq - sig) > delta) break;
      j++;
    }
    tdvec_block(e, L.dg, n, sig, delta, j, pivmin, &lo, &hi);
  }
  L.nrm2[k] = twisted_vector(e, L.dg, n, sig, pivmin, KP, k, lo, hi, L.dp, L.dm, L.z);
}

// unit parts: X(i,k) = s_k z(i,k).  Skew mode: even-row and odd-row parts each of
// unit length, s_k = sqrt(2)/|z_k| (sigma > 0) or 1/|z_k| (the zero-eigenvalue
// vector, even rows only); full mode: s_k = 1/|z_k|.  X may be L.dp.
__global__ void tdvec_normalize_kernel(TdvecLayout L0, double* X0) {
  if (gated_off(L0, blockIdx.z)) return;
  const TdvecLayout L = at_problem(L0, blockIdx.z);
  double* X = X0 + (size_t)blockIdx.z * L0.mstride;
  const int64_t KP = L.KP;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)L.n * KP;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / KP), k = (int)(q - (int64_t)i * KP);
    double x = 0.0;
    if (k < L.K) {
      if (L.full)
        x = rsqrt(L.nrm2[k]) * L.z[q];
      else if (!((i & 1) && k >= L.h))
        x = ((k < L.h) ? 1.4142135623730951 : 1.0) * rsqrt(L.nrm2[k]) * L.z[q];
    }
    X[q] = x;
  }
}

// ---------------------------------------------------------------------------
// 3. banded Gram entries: raw dots of vector k with k + d (d = 0..LW), over the
//    even rows (U) and the odd rows (V) separately
// ---------------------------------------------------------------------------
constexpr int BD_NT = 256;
constexpr int BD_COLS = 32 + LW;
constexpr int BD_PAIRS = 32 * (LW + 1);
constexpr int BD_PER = (BD_PAIRS + BD_NT - 1) / BD_NT;

__global__ void __launch_bounds__(BD_NT) band_dots_kernel(TdvecLayout L0, const double* X0) {
  if (gated_off(L0, blockIdx.z)) return;
  const TdvecLayout L = at_problem(L0, blockIdx.z);
  const double* X = X0 + (size_t)blockIdx.z * L0.mstride;
  __shared__ double zs[RC][BD_COLS + 1];
  const int k0 = blockIdx.x * 32;
  const int n = L.n;
  const int64_t KP = L.KP;
  double accU[BD_PER], accV[BD_PER];
#pragma unroll
  for (int q = 0; q < BD_PER; q++) accU[q] = accV[q] = 0.0;
  for (int i0 = 0; i0 < n; i0 += RC) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < RC * BD_COLS; idx += BD_NT) {
      const int rr = idx / BD_COLS, cc = idx - rr * BD_COLS;
      const int i = i0 + rr, k = k0 + cc;
      zs[rr][cc] = (i < n && k < L.K) ? X[(int64_t)i * KP + k] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < BD_PER; q++) {
      const int pr = threadIdx.x + q * BD_NT;
      if (pr < BD_PAIRS) {
        const int kk = pr % 32, dd = pr / 32;
        double su = 0.0, sv = 0.0;
        for (int rr = 0; rr < RC; rr += 2) {  // i0 is even, so rr even <-> even row
          su = fma(zs[rr][kk], zs[rr][kk + dd], su);
          sv = fma(zs[rr + 1][kk], zs[rr + 1][kk + dd], sv);
        }
        accU[q] += su;
        accV[q] += sv;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < BD_PER; q++) {
    const int pr = threadIdx.x + q * BD_NT;
    if (pr < BD_PAIRS) {
      const int kk = pr % 32, dd = pr / 32;
      const int k = k0 + kk;
      L.bandU[(int64_t)k * (LW + 1) + dd] = accU[q];
      L.bandV[(int64_t)k * (LW + 1) + dd] = accV[q];
    }
  }
}

// ---------------------------------------------------------------------------
// 3. one symmetric correction pass  Y = X - 1/2 X E  over the band,
//    E(k, j) = X_k . X_j - delta_kj per part (skew mode: even rows / odd rows;
//    the zero-eigenvalue vector has no odd part; full mode: all rows)
// ---------------------------------------------------------------------------
constexpr int LA_NT = 256;
constexpr int LA_COLS = 32 + 2 * LW;

__global__ void __launch_bounds__(LA_NT) band_apply_kernel(TdvecLayout L0, const double* X0, double* Y0) {
  if (gated_off(L0, blockIdx.z)) return;
  const TdvecLayout L = at_problem(L0, blockIdx.z);
  const double* X = X0 + (size_t)blockIdx.z * L0.mstride;
  double* Y = Y0 + (size_t)blockIdx.z * L0.mstride;
  __shared__ double xs[RC][LA_COLS + 1];
  __shared__ double eU[32][2 * LW + 1], eV[32][2 * LW + 1];
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int n = L.n;
  const int64_t KP = L.KP;
  for (int idx = threadIdx.x; idx < RC * LA_COLS; idx += LA_NT) {
    const int rr = idx / LA_COLS, cc = idx - rr * LA_COLS;
    const int i = i0 + rr, k = k0 - LW + cc;
    xs[rr][cc] = (i < n && k >= 0 && k < L.K) ? X[(int64_t)i * KP + k] : 0.0;
  }
  for (int idx = threadIdx.x; idx < 32 * (2 * LW + 1); idx += LA_NT) {
    const int kk = idx / (2 * LW + 1), dd = idx - kk * (2 * LW + 1) - LW;
    const int k = k0 + kk, j = k + dd;
    double u = 0.0, v = 0.0;
    if (k < L.K && j >= 0 && j < L.K) {
      const int lo = min(k, j), off = abs(dd);
      const double du = L.bandU[(int64_t)lo * (LW + 1) + off], dv = L.bandV[(int64_t)lo * (LW + 1) + off];
      const double id = (dd == 0) ? 1.0 : 0.0;
      if (L.full) {
        u = v = du + dv - id;
      } else {
        u = du - id;
        v = (k >= L.h || j >= L.h) ? 0.0 : dv - id;
      }
    }
    eU[kk][dd + LW] = u;
    eV[kk][dd + LW] = v;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx % 32, rr = idx / 32;  // consecutive threads: consecutive k (interleaved rows)
    const int i = i0 + rr, k = k0 + kk;
    if (i >= n || k >= KP) continue;
    double acc = xs[rr][kk + LW];
    if (k < L.K) {
      const double(*E)[2 * LW + 1] = (i & 1) ? eV : eU;
#pragma unroll 11
      for (int dd = -LW; dd <= LW; dd++) acc = fma(-0.5 * E[kk][dd + LW], xs[rr][kk + LW + dd], acc);
    }
    Y[(int64_t)i * KP + k] = acc;
  }
}

// skew mode: the -sigma eigenvectors in the tridiagonal basis into the columns n-1-k
// of Vr / Vi (real on even 0-based rows, imaginary on odd rows, sign flipped every
// pair, |w| = 1); the zero-eigenvalue vector (odd n) into column h
__global__ void __launch_bounds__(LA_NT) tdvec_write_skew_kernel(TdvecLayout L, const double* __restrict__ X,
                                                                 double* __restrict__ Vr, double* __restrict__ Vi,
                                                                 int64_t ldv) {
  if (gated_off(L)) return;
  __shared__ double out[RC][33];
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int n = L.n;
  const int64_t KP = L.KP;
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx % 32, rr = idx / 32;
    const int i = i0 + rr, k = k0 + kk;
    double o = 0.0;
    if (i < n && k < L.K) {
      o = X[(int64_t)i * KP + k];
      if (k < L.h) o *= 0.7071067811865476;
      if ((i >> 1) & 1) o = neg(o);
    }
    out[rr][kk] = o;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx / RC, rr = idx - kk * RC;  // consecutive threads: consecutive rows of a column
    const int i = i0 + rr, k = k0 + kk;
    if (i >= n || k >= L.K) continue;
    const int col = (k < L.h) ? n - 1 - k : L.h;
    const double o = out[rr][kk];
    if ((i & 1) == 0) {
      Vr[i + (int64_t)col * ldv] = o;
      if (k < L.h) Vi[i + (int64_t)col * ldv] = 0.0;
    } else {
      Vr[i + (int64_t)col * ldv] = 0.0;
      if (k < L.h) Vi[i + (int64_t)col * ldv] = o;
    }
  }
}

// full mode: Y(:, k) = X(:, k) (n x n, ld n), problem blockIdx.z n^2 apart
__global__ void __launch_bounds__(LA_NT) tdvec_write_full_kernel(TdvecLayout L0, const double* X0, double* Y) {
  __shared__ double out[RC][33];
  const int n = L0.n;
  const double* X = X0 + (size_t)blockIdx.z * L0.mstride;
  Y += (size_t)blockIdx.z * n * n;
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int64_t KP = L0.KP;
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx % 32, rr = idx / 32;
    const int i = i0 + rr, k = k0 + kk;
    out[rr][kk] = (i < n && k < L0.K) ? X[(int64_t)i * KP + k] : 0.0;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx / RC, rr = idx - kk * RC;
    const int i = i0 + rr, k = k0 + kk;
    if (i < n && k < L0.K) Y[i + (int64_t)k * n] = out[rr][kk];
  }
}

// normalise, then three correction passes (each squares the departure from
// orthogonality; clusters of nearly equal eigenvalues need more than one);
// returns the array holding the result (L.dp or L.dm)
static double* tdvec_orthogonalize(const TdvecLayout& L, int batch, cudaStream_t st) {
  const int64_t tot = (int64_t)L.n * L.KP;
  tdvec_normalize_kernel<<<dim3((unsigned)std::min<int64_t>((tot + 255) / 256, 4096), 1, batch), 256, 0, st>>>(L, L.dp);
  double* X = L.dp;
  double* Y = L.dm;
  for (int pass = 0; pass < 3; pass++) {
    band_dots_kernel<<<dim3(L.KP / 32, 1, batch), BD_NT, 0, st>>>(L, X);
    band_apply_kernel<<<dim3(L.KP / 32, (L.n + RC - 1) / RC, batch), LA_NT, 0, st>>>(L, X, Y);
    double* t = X;
    X = Y;
    Y = t;
  }
  return X;
}

// Eigenvectors of the symmetric tridiagonal with diagonal dg and off-diagonal e
// for the ascending eigenvalues mu (bp: bound, pivmin), into Y (n x n, ld n).
// Problems mb < batch lie n (dg, e, mu), 8 (bp), n^2 (Y) and
// large_eigen_ws_doubles(n) (ws) apart.
cudaError_t symtri_vectors(const double* dg, const double* e, int n, const double* mu, const double* bp, double* Y,
                           double* ws, int batch, cudaStream_t st) {
  const TdvecLayout L = layout(n, ws, true, dg);
  twisted_kernel<<<dim3(L.KP / TW_NT + (L.KP % TW_NT ? 1 : 0), 1, batch), TW_NT, 0, st>>>(e, mu, bp, L);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  double* X = tdvec_orthogonalize(L, batch, st);
  tdvec_write_full_kernel<<<dim3(L.KP / 32, (n + RC - 1) / RC, batch), LA_NT, 0, st>>>(L, X, Y);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// 5. compact WY factors T_b (dlarft, forward, columnwise) of each panel
// ---------------------------------------------------------------------------
// Reflector c (0 <= c <= n-3) lives in column c of A below the diagonal: v_c = 0
// above row c+1, v_c[c+1] = 1, v_c[c+2:] = A[c+2:, c]; tau_c = 0 means H_c = I.
__device__ __forceinline__ double refl_at(const double* A, int64_t lda, const double* tau, int row, int c) {
  if (row < c + 1 || tau[c] == 0.0) return 0.0;
  return (row == c + 1) ? 1.0 : A[row + (int64_t)c * lda];
}

constexpr int WT_NT = 256;
constexpr int WT_RC = 16;  // rows per staged chunk of the factor kernel

// One array holds both: the lower triangle of M is the Gram matrix G = V^T V
// (symmetric, so G(l, i) is read as M(i, l)), the upper triangle and diagonal
// receive T as the recurrence produces it (a diagonal G entry is never needed).
__global__ void __launch_bounds__(WT_NT) wy_factor_kernel(const double* __restrict__ A, int64_t lda,
                                                          const double* __restrict__ tau, TdvecLayout L) {
  if (gated_off(L)) return;
  __shared__ double Vs[WT_RC][WB + 1];
  __shared__ double M[WB][WB + 1];
  const int b = blockIdx.x;
  const int n = L.n;
  const int c0 = b * WB, c1 = min(c0 + WB, n - 2), nb = c1 - c0;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[a][q] = 0.0;
  for (int r0 = c0 + 1; r0 < n; r0 += WT_RC) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < WT_RC * WB; idx += WT_NT) {
      const int cc = idx / WT_RC, rr = idx - cc * WT_RC;
      const int row = r0 + rr, c = c0 + cc;
      Vs[rr][cc] = (row < n && cc < nb) ? refl_at(A, lda, tau, row, c) : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < WT_RC; rr++) {
      double va[4], vb[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        va[a] = Vs[rr][ty + 16 * a];
        vb[a] = Vs[rr][tx + 16 * a];
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[a][q] = fma(va[a], vb[q], acc[a][q]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int i = ty + 16 * a, j = tx + 16 * q;
      M[i][j] = (i > j) ? acc[a][q] : 0.0;  // G below the diagonal, T (zero so far) on and above
    }
  __syncthreads();
  // T(i,i) = tau_i; T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i)
  for (int i = 0; i < nb; i++) {
    const double ti = tau[c0 + i];
    if (threadIdx.x < i) {
      const int j = threadIdx.x;
      double s = 0.0;
      for (int l = j; l < i; l++) s = fma(M[j][l], M[i][l], s);
      M[j][i] = neg(ti) * s;
    }
    if (threadIdx.x == 0) M[i][i] = ti;
    __syncthreads();
  }
  double* Tg = L.T + (size_t)b * WB * WB;
  for (int idx = threadIdx.x; idx < WB * WB; idx += WT_NT) {
    const int i = idx / WB, j = idx % WB;
    Tg[idx] = (j >= i) ? M[i][j] : 0.0;
  }
}

// ---------------------------------------------------------------------------
// 5. X <- Q X, one CTA per strip of SW columns, panels last to first:
//    W = V^T X, W <- T W, X <- X - V W
// ---------------------------------------------------------------------------
constexpr int BT_NT = 256;

struct StripParams {
  const double* A;
  int64_t lda;
  const double* tau;
  TdvecLayout L;
  double* Xr;  // columns [cr0, n) of Vr
  double* Xi;  // columns [ci0, n) of Vi
  int64_t ldv;
  int cr0, ci0, nstr_r;  // strips over Vr first
};

__global__ void __launch_bounds__(BT_NT) back_strip_kernel(StripParams P) {
  if (gated_off(P.L)) return;
  extern __shared__ __align__(16) double bsm[];
  double(*Ts)[WB + 1] = reinterpret_cast<double(*)[WB + 1]>(bsm);                   // WB x (WB+1)
  double(*Ws)[SW + 1] = reinterpret_cast<double(*)[SW + 1]>(bsm + WB * (WB + 1));  // WB x (SW+1)
  double(*Vs)[WB + 1] = reinterpret_cast<double(*)[WB + 1]>(bsm + WB * (WB + 1) + WB * (SW + 1));  // RC x (WB+1)
  double(*Xs)[SW + 1] =
      reinterpret_cast<double(*)[SW + 1]>(bsm + WB * (WB + 1) + WB * (SW + 1) + RC * (WB + 1));  // RC x (SW+1)
  const int n = P.L.n;
  const int s = blockIdx.x;
  double* X;
  int col0, ncol;
  if (s < P.nstr_r) {
    X = P.Xr;
    col0 = P.cr0 + s * SW;
  } else {
    X = P.Xi;
    col0 = P.ci0 + (s - P.nstr_r) * SW;
  }
  ncol = min(SW, n - col0);
  X += (int64_t)col0 * P.ldv;
  const int64_t ldx = P.ldv;
  // thread tiles: W (WB x SW = 64 x 32): 4 x 2 per thread; X chunk (RC x SW = 32 x 32): 2 x 2 per thread
  const int wr = (threadIdx.x >> 4) * 4, wc = (threadIdx.x & 15) * 2;
  const int xr = (threadIdx.x >> 4) * 2, xc = (threadIdx.x & 15) * 2;
  for (int b = P.L.npan - 1; b >= 0; b--) {
    const int c0 = b * WB, c1 = min(c0 + WB, n - 2), nb = c1 - c0;
    __syncthreads();
    for (int idx = threadIdx.x; idx < WB * WB; idx += BT_NT)
      Ts[idx / WB][idx % WB] = P.L.T[(size_t)b * WB * WB + idx];
    // W = V^T X over rows c0+1 .. n-1
    double w[4][2];
#pragma unroll
    for (int a = 0; a < 4; a++) w[a][0] = w[a][1] = 0.0;
    for (int r0 = c0 + 1; r0 < n; r0 += RC) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < RC * WB; idx += BT_NT) {
        const int cc = idx / RC, rr = idx - cc * RC;
        const int row = r0 + rr;
        Vs[rr][cc] = (row < n && cc < nb) ? refl_at(P.A, P.lda, P.tau, row, c0 + cc) : 0.0;
      }
      for (int idx = threadIdx.x; idx < RC * SW; idx += BT_NT) {
        const int cc = idx / RC, rr = idx - cc * RC;
        const int row = r0 + rr;
        Xs[rr][cc] = (row < n && cc < ncol) ? X[row + (int64_t)cc * ldx] : 0.0;
      }
      __syncthreads();
#pragma unroll 8
      for (int rr = 0; rr < RC; rr++) {
        const double x0 = Xs[rr][wc], x1 = Xs[rr][wc + 1];
#pragma unroll
        for (int a = 0; a < 4; a++) {
          const double v = Vs[rr][wr + a];
          w[a][0] = fma(v, x0, w[a][0]);
          w[a][1] = fma(v, x1, w[a][1]);
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
      Ws[wr + a][wc] = w[a][0];
      Ws[wr + a][wc + 1] = w[a][1];
    }
    __syncthreads();
    // W <- T W (T upper triangular)
    double tw[4][2];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      tw[a][0] = tw[a][1] = 0.0;
      const int i = wr + a;
      for (int l = i; l < WB; l++) {
        const double t = Ts[i][l];
        tw[a][0] = fma(t, Ws[l][wc], tw[a][0]);
        tw[a][1] = fma(t, Ws[l][wc + 1], tw[a][1]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < 4; a++) {
      Ws[wr + a][wc] = tw[a][0];
      Ws[wr + a][wc + 1] = tw[a][1];
    }
    // X <- X - V W over rows c0+1 .. n-1 (X chunk staged: coalesced column reads and writes)
    for (int r0 = c0 + 1; r0 < n; r0 += RC) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < RC * WB; idx += BT_NT) {
        const int cc = idx / RC, rr = idx - cc * RC;
        const int row = r0 + rr;
        Vs[rr][cc] = (row < n && cc < nb) ? refl_at(P.A, P.lda, P.tau, row, c0 + cc) : 0.0;
      }
      for (int idx = threadIdx.x; idx < RC * SW; idx += BT_NT) {
        const int cc = idx / RC, rr = idx - cc * RC;
        const int row = r0 + rr;
        Xs[rr][cc] = (row < n && cc < ncol) ? X[row + (int64_t)cc * ldx] : 0.0;
      }
      __syncthreads();
      double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
#pragma unroll 8
      for (int l = 0; l < WB; l++) {
        const double w0 = Ws[l][xc], w1 = Ws[l][xc + 1];
        const double v0 = Vs[xr][l], v1 = Vs[xr + 1][l];
        acc[0][0] = fma(v0, w0, acc[0][0]);
        acc[0][1] = fma(v0, w1, acc[0][1]);
        acc[1][0] = fma(v1, w0, acc[1][0]);
        acc[1][1] = fma(v1, w1, acc[1][1]);
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int q = 0; q < 2; q++) Xs[xr + a][xc + q] -= acc[a][q];
      __syncthreads();
      for (int idx = threadIdx.x; idx < RC * SW; idx += BT_NT) {
        const int cc = idx / RC, rr = idx - cc * RC;
        const int row = r0 + rr;
        if (row < n && cc < ncol) X[row + (int64_t)cc * ldx] = Xs[rr][cc];
      }
    }
  }
}

// 6. +sigma columns: Vr[:, k] = Vr[:, n-1-k], Vi[:, k] = -Vi[:, n-1-k]; odd n: Vi[:, h] = 0
__global__ void mirror_kernel(double* __restrict__ Vr, double* __restrict__ Vi, int64_t ldv, int n,
                              const int* __restrict__ gate) {
  if (gate && *gate != 0) return;  // the skew-mode pipeline only
  const int h = n / 2;
  const int k = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (k < h) {
      const int64_t src = i + (int64_t)(n - 1 - k) * ldv, dst = i + (int64_t)k * ldv;
      Vr[dst] = Vr[src];
      Vi[dst] = neg(Vi[src]);
    } else {
      Vi[i + (int64_t)h * ldv] = 0.0;  // k == h only launched for odd n
    }
  }
}

static size_t strip_smem_bytes() {
  return sizeof(double) * ((size_t)WB * (WB + 1) + (size_t)WB * (SW + 1) + (size_t)RC * (WB + 1) + (size_t)RC * (SW + 1));
}

// Batched skew-mode write and mirror for G problems of one size (per-problem output
// pointers Vr[idx[mb]], Vi[idx[mb]], leading dimension n): the same as
// tdvec_write_skew_kernel and mirror_kernel.
__global__ void __launch_bounds__(LA_NT) tdvec_write_skew_batch_kernel(TdvecLayout L0, const double* X0,
                                                                       double* const* Vr_all, double* const* Vi_all,
                                                                       const int32_t* idx) {
  if (gated_off(L0, blockIdx.z)) return;
  __shared__ double out[RC][33];
  const int mb = blockIdx.z;
  const TdvecLayout L = at_problem(L0, mb);
  const double* X = X0 + (size_t)mb * L0.mstride;
  double* Vr = Vr_all[idx[mb]];
  double* Vi = Vi_all[idx[mb]];
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int n = L.n;
  const int64_t ldv = n;
  const int64_t KP = L.KP;
  for (int q = threadIdx.x; q < RC * 32; q += LA_NT) {
    const int kk = q % 32, rr = q / 32;
    const int i = i0 + rr, k = k0 + kk;
    double o = 0.0;
    if (i < n && k < L.K) {
      o = X[(int64_t)i * KP + k];
      if (k < L.h) o *= 0.7071067811865476;
      if ((i >> 1) & 1) o = neg(o);
    }
    out[rr][kk] = o;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < RC * 32; q += LA_NT) {
    const int kk = q / RC, rr = q - kk * RC;
    const int i = i0 + rr, k = k0 + kk;
    if (i >= n || k >= L.K) continue;
    const int col = (k < L.h) ? n - 1 - k : L.h;
    const double o = out[rr][kk];
    if ((i & 1) == 0) {
      Vr[i + (int64_t)col * ldv] = o;
      Vi[i + (int64_t)col * ldv] = 0.0;
    } else {
      Vr[i + (int64_t)col * ldv] = 0.0;
      Vi[i + (int64_t)col * ldv] = (k < L.h) ? o : 0.0;
    }
  }
}

__global__ void mirror_batch_kernel(double* const* Vr_all, double* const* Vi_all, const int32_t* idx, int n,
                                    const int* __restrict__ gate) {
  if (gate && gate[blockIdx.z] != 0) return;  // the skew-mode pipeline only
  double* Vr = Vr_all[idx[blockIdx.z]];
  double* Vi = Vi_all[idx[blockIdx.z]];
  const int h = n / 2;
  const int k = blockIdx.y;
  const int64_t ldv = n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (k < h) {
      const int64_t src = i + (int64_t)(n - 1 - k) * ldv, dst = i + (int64_t)k * ldv;
      Vr[dst] = Vr[src];
      Vi[dst] = neg(Vi[src]);
    } else {
      Vi[i + (int64_t)h * ldv] = 0.0;  // k == h only launched for odd n
    }
  }
}

// ---------------------------------------------------------------------------
// Several zero eigenvalues.  Where ev has exact zeros, the tridiagonal is a direct
// sum of blocks and each odd-size block brings one zero eigenvalue.  More zero
// eigenvalues than n mod 2 do not fit the +-sigma pairing of the skew mode, so the
// whole problem is then solved in full mode, as the reference's fallback
// skewtrieigen_backup! (skeweigen.jl:470-489) solves it: every eigenpair of
// SymTridiagonal(0, ev), each column laid out on its own.
// ---------------------------------------------------------------------------
constexpr int OB_NT = 1024;

// gate <- 1 when the exact splits of ev leave more odd-size blocks than n mod 2, else
// 0; for full mode also mu[j] = -vals[j] (ascending) and bpf = (bound, pivmin, -bound).
// One CTA per problem (blockIdx.x; ev, vals, mu n apart, bp, bpf 8 apart): each thread
// summarises a contiguous chunk of ev (first and last zero and the odd gaps between its
// zeros), thread 0 joins the chunks in order.
__global__ void __launch_bounds__(OB_NT) odd_blocks_kernel(const double* __restrict__ ev, int n,
                                                           const double* __restrict__ vals,
                                                           const double* __restrict__ bp, int* __restrict__ gate,
                                                           double* __restrict__ mu, double* __restrict__ bpf) {
  __shared__ int first[OB_NT], last[OB_NT], odd[OB_NT];
  const int mb = blockIdx.x;
  ev += (size_t)mb * n;
  vals += (size_t)mb * n;
  mu += (size_t)mb * n;
  bp += (size_t)mb * 8;
  bpf += (size_t)mb * 8;
  gate += mb;
  const int m = n - 1;  // entries of ev; a zero at ev[i] ends a block at row i
  const int chunk = (m + OB_NT - 1) / OB_NT;
  const int t = threadIdx.x;
  int f = -1, l = -1, c = 0;
  for (int i = t * chunk; i < min(m, (t + 1) * chunk); i++) {
    if (ev[i] == 0.0) {
      if (l >= 0) c += (i - l) & 1;
      else f = i;
      l = i;
    }
  }
  first[t] = f;
  last[t] = l;
  odd[t] = c;
  for (int j = t; j < n; j += OB_NT) mu[j] = -vals[j];
  __syncthreads();
  if (t == 0) {
    int prev = -1, count = 0;  // previous zero position (-1: the start of row 0)
    for (int q = 0; q < OB_NT; q++) {
      if (first[q] < 0) continue;
      count += ((first[q] - prev) & 1) + odd[q];
      prev = last[q];
    }
    count += ((n - 1 - prev) & 1);  // the last block
    *gate = (count > (n & 1)) ? 1 : 0;
    bpf[0] = bp[0];
    bpf[1] = bp[1];
    bpf[2] = -bp[0];
  }
}

// full mode into the fallback's layout (skeweigen.jl:476-487): column j holds the
// eigenvector w_j of SymTridiagonal(0, ev) for mu_j = -vals_j, real on even 0-based
// rows and imaginary on odd rows, with the sign (-1)^(i/2) of row pair i/2
__global__ void __launch_bounds__(LA_NT) tdvec_write_fallback_kernel(TdvecLayout L, const double* __restrict__ X,
                                                                     double* __restrict__ Vr,
                                                                     double* __restrict__ Vi, int64_t ldv) {
  if (gated_off(L)) return;
  __shared__ double out[RC][33];
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int n = L.n;
  const int64_t KP = L.KP;
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx % 32, rr = idx / 32;
    const int i = i0 + rr, k = k0 + kk;
    double o = 0.0;
    if (i < n && k < L.K) {
      o = X[(int64_t)i * KP + k];
      if ((i >> 1) & 1) o = neg(o);
    }
    out[rr][kk] = o;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < RC * 32; idx += LA_NT) {
    const int kk = idx / RC, rr = idx - kk * RC;
    const int i = i0 + rr, k = k0 + kk;
    if (i >= n || k >= L.K) continue;
    const double o = out[rr][kk];
    const int64_t at = i + (int64_t)k * ldv;
    Vr[at] = (i & 1) ? 0.0 : o;
    Vi[at] = (i & 1) ? o : 0.0;
  }
}

// the same for problem blockIdx.z of a batch: Vr[idx[mb]], Vi[idx[mb]] (n x n, ld n)
__global__ void __launch_bounds__(LA_NT) tdvec_write_fallback_batch_kernel(TdvecLayout L0, const double* X0,
                                                                           double* const* Vr_all,
                                                                           double* const* Vi_all,
                                                                           const int32_t* idx) {
  const int mb = blockIdx.z;
  if (gated_off(L0, mb)) return;
  __shared__ double out[RC][33];
  const TdvecLayout L = at_problem(L0, mb);
  const double* X = X0 + (size_t)mb * L0.mstride;
  double* Vr = Vr_all[idx[mb]];
  double* Vi = Vi_all[idx[mb]];
  const int k0 = blockIdx.x * 32, i0 = blockIdx.y * RC;
  const int n = L.n;
  const int64_t KP = L.KP;
  for (int q = threadIdx.x; q < RC * 32; q += LA_NT) {
    const int kk = q % 32, rr = q / 32;
    const int i = i0 + rr, k = k0 + kk;
    double o = 0.0;
    if (i < n && k < L.K) {
      o = X[(int64_t)i * KP + k];
      if ((i >> 1) & 1) o = neg(o);
    }
    out[rr][kk] = o;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < RC * 32; q += LA_NT) {
    const int kk = q / RC, rr = q - kk * RC;
    const int i = i0 + rr, k = k0 + kk;
    if (i >= n || k >= L.K) continue;
    const double o = out[rr][kk];
    const int64_t at = i + (int64_t)k * n;
    Vr[at] = (i & 1) ? 0.0 : o;
    Vi[at] = (i & 1) ? o : 0.0;
  }
}

static cudaError_t back_transform(const double* A, int64_t lda, const double* tau, const TdvecLayout& L, double* Vr,
                                  double* Vi, int64_t ldv, int cr0, int ci0, cudaStream_t st) {
  const int n = L.n;
  wy_factor_kernel<<<L.npan, WT_NT, 0, st>>>(A, lda, tau, L);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  StripParams P;
  P.A = A;
  P.lda = lda;
  P.tau = tau;
  P.L = L;
  P.Xr = Vr;
  P.Xi = Vi;
  P.ldv = ldv;
  P.cr0 = cr0;
  P.ci0 = ci0;
  P.nstr_r = (n - cr0 + SW - 1) / SW;
  const int nstr_i = (n - ci0 + SW - 1) / SW;
  static std::atomic<uint64_t> raised{0};
  e = raise_smem_limit_once((const void*)back_strip_kernel, raised);
  if (e != cudaSuccess) return e;
  back_strip_kernel<<<P.nstr_r + nstr_i, BT_NT, strip_smem_bytes(), st>>>(P);
  return cudaGetLastError();
}

size_t large_eigen_aux_doubles(int n) { return (size_t)n + 8; }

// gate (device int) and aux (large_eigen_aux_doubles(n)) are scratch of the caller.
cudaError_t large_eigen_vectors(const double* A, int64_t lda, int n, const double* tau, const double* ev,
                                const double* vals, const double* bp, double* Vr, double* Vi, int64_t ldv, double* ws,
                                int* gate, double* aux, cudaStream_t st) {
  if (n < 3) return cudaErrorInvalidValue;
  double* mu = aux;
  double* bpf = aux + n;
  odd_blocks_kernel<<<1, OB_NT, 0, st>>>(ev, n, vals, bp, gate, mu, bpf);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // skew mode (gate == 0): -sigma vectors, back-transformed, +sigma mirrored
  TdvecLayout L = layout(n, ws);
  L.gate = gate;
  L.gate_on = 0;
  twisted_kernel<<<L.KP / TW_NT + (L.KP % TW_NT ? 1 : 0), TW_NT, 0, st>>>(ev, vals, bp, L);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double* X = tdvec_orthogonalize(L, 1, st);
  tdvec_write_skew_kernel<<<dim3(L.KP / 32, (n + RC - 1) / RC), LA_NT, 0, st>>>(L, X, Vr, Vi, ldv);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (A) {  // A == null: a tridiagonal input, Q = I
    // -sigma columns and the zero vector of Vr, -sigma columns of Vi
    e = back_transform(A, lda, tau, L, Vr, Vi, ldv, L.h, L.h + (n & 1), st);
    if (e != cudaSuccess) return e;
  }
  mirror_kernel<<<dim3((n + 255) / 256, L.h + (n & 1)), 256, 0, st>>>(Vr, Vi, ldv, n, gate);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // full mode (gate == 1): every eigenpair, each column back-transformed
  TdvecLayout F = layout(n, ws, true, nullptr);
  F.gate = gate;
  F.gate_on = 1;
  twisted_kernel<<<F.KP / TW_NT + (F.KP % TW_NT ? 1 : 0), TW_NT, 0, st>>>(ev, mu, bpf, F);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  X = tdvec_orthogonalize(F, 1, st);
  tdvec_write_fallback_kernel<<<dim3(F.KP / 32, (n + RC - 1) / RC), LA_NT, 0, st>>>(F, X, Vr, Vi, ldv);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (A) return back_transform(A, lda, tau, F, Vr, Vi, ldv, 0, 0, st);
  return cudaSuccess;
}


// Batched skew-mode vectors for G problems of one size.  ws holds each problem's
// workspace (large_eigen_ws_doubles(n), mstride apart), then per problem the
// full-mode inputs mu (n), bpf (8) and the gate (as in large_eigen_vectors).
size_t skew_vectors_batch_ws_doubles(int n) { return large_eigen_ws_doubles(n) + (size_t)n + 16; }

cudaError_t skew_vectors_batch(const double* e_g, int n, int G, const double* vals_g, const double* bp_g,
                               double* const* Vr, double* const* Vi, const int32_t* idx, double* ws,
                               cudaStream_t st) {
  if (n < 3 || G <= 0) return cudaErrorInvalidValue;
  double* aux = ws + (size_t)G * large_eigen_ws_doubles(n);
  double* mu = aux;
  double* bpf = aux + (size_t)G * n;
  int* gate = (int*)(bpf + (size_t)G * 8);
  odd_blocks_kernel<<<G, OB_NT, 0, st>>>(e_g, n, vals_g, bp_g, gate, mu, bpf);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // skew mode (gate 0): the -sigma vectors, then the +sigma mirror
  TdvecLayout L = layout(n, ws);
  L.gate = gate;
  L.gate_on = 0;
  twisted_kernel<<<dim3(L.KP / TW_NT + (L.KP % TW_NT ? 1 : 0), 1, G), TW_NT, 0, st>>>(e_g, vals_g, bp_g, L);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double* X = tdvec_orthogonalize(L, G, st);
  tdvec_write_skew_batch_kernel<<<dim3(L.KP / 32, (n + RC - 1) / RC, G), LA_NT, 0, st>>>(L, X, Vr, Vi, idx);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  mirror_batch_kernel<<<dim3((n + 255) / 256, L.h + (n & 1), G), 256, 0, st>>>(Vr, Vi, idx, n, gate);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // full mode (gate 1): every eigenpair in the fallback's layout
  TdvecLayout F = layout(n, ws, true, nullptr);
  F.gate = gate;
  F.gate_on = 1;
  twisted_kernel<<<dim3(F.KP / TW_NT + (F.KP % TW_NT ? 1 : 0), 1, G), TW_NT, 0, st>>>(e_g, mu, bpf, F);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  X = tdvec_orthogonalize(F, G, st);
  tdvec_write_fallback_batch_kernel<<<dim3(F.KP / 32, (n + RC - 1) / RC, G), LA_NT, 0, st>>>(F, X, Vr, Vi, idx);
  return cudaGetLastError();
}

}  // namespace skew
