// Batched and small-matrix kernels: one CTA per skew matrix.
//
// Working copy.  A CTA works on a full-storage copy W of its matrix (both
// triangles kept, W[j,i] = -W[i,j]).  In the batched path W lives in dynamic
// shared memory when the size bucket fits (template SM = true: every access is
// a shared-memory instruction), otherwise in a per-CTA slot of a global
// workspace; in the single-matrix path W is the caller's matrix itself (in
// place, as hessenberg!/logabspfaffian! are).  Leading dimensions of private
// copies are odd so transposed stores do not conflict in shared-memory banks.
//
// Forward reduction, step k (reflector acting on indices k+1..n-1):
//   1. p = tau_k * W[k+1:n, k+1:n] v_k       (full-row products, lanes = rows)
//   2. W[i,j] += v_i p_j - p_i v_j, k < j < i, mirrored (two-sided H W H; exact
//      for skew W since v^T W v = 0).  While warps 1.. update the bulk, warp 0
//      updates column k+1 first and builds reflector k+1 from it (householder!,
//      hessenberg.jl:26-44), so the serial norm/sqrt/divide chain of the next
//      step is hidden behind this step's update.
// Steps 1 and 2 cost m^2 FMAs each (4/3 n^3 flops in total).
//
// Gradient (the adjoint of log|Pf|; the reference has no rrule):
// d log|Pf(A)|/dA = 1/2 A^{-T} = -1/2 A^{-1} = Q (-1/2 T^{-1}) Q^T with
// Q = H_0 H_1 ... H_{n-3}.  Starting from M = -1/2 T^{-1}, the reflectors are
// applied innermost first in blocks of GNB.  A block Q_b = I - V T_b V^T
// (compact WY, T_b upper triangular) acts as one skew rank-2*GNB update:
//   X = M V,  Z = X T_b^T,  K = V^T X,  C = T_b K T_b^T,  Z' = Z - 1/2 V C,
//   Q_b M Q_b^T = M + V Z'^T - Z' V^T,
// which is the same 2 n m FMAs per reflector as applying them one at a time, but
// as register-tiled products that read M once per block instead of once per
// reflector.  Only the strictly lower triangle of M is kept while the blocks run
// (M is skew): X reads the upper entries as -M^T, the update writes no mirror, and
// one pass at the end fills the upper triangle.  That halves the gradient's live
// set, so that two CTAs per SM on n = 256 matrices keep it in L2.
//
// Zero structure.  T^{-1} is nonzero only where row and column differ in parity,
// and below the diagonal only at (odd row, even column).  With r0 the first row of
// the current block, the rows and columns above r0 are untouched except through
// the updates of the blocks already applied, and by induction over the blocks the
// odd columns j < r0 of M stay zero in every row >= r0 (so the odd rows i < r0 are
// zero in every column >= r0).  Hence X_i = 0 for odd i < r0 and the update leaves
// the odd columns j < r0 unchanged (its term there is V_i . Z'_j with Z'_j = 0).
// Skipping both is exact and cuts the gradient from n^3 to 5/6 n^3 FMAs.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "skew_common.cuh"
#include "skew_internal.h"

namespace skew {

constexpr int GNB = 8;  // reflectors per block in the gradient

// ---------------------------------------------------------------------------
// Matrix accessors: shared-memory (offset into the dynamic shared array) or
// global (pointer).  Distinct types so shared accesses compile to shared-memory
// instructions.
// ---------------------------------------------------------------------------
extern __shared__ __align__(16) double dsm[];

struct SMat {
  int off, ld;
  __device__ __forceinline__ double& at(int i, int j) const { return dsm[off + i + j * ld]; }
};
struct GMat {
  double* p;
  int64_t ld;
  __device__ __forceinline__ double& at(int i, int j) const { return p[i + (int64_t)j * ld]; }
};

// ---------------------------------------------------------------------------
// Shared-memory layout (doubles)
// ---------------------------------------------------------------------------
struct Smem {
  double *ev, *tau, *red, *T, *P, *K, *C;
  double *vb0, *vb1, *p, *ypart;  // forward view of the union
  double *Vs, *Zs, *Xp;           // gradient view of the union
  int nmax;
};

// Forward view: vb0, vb1, p (nmax each), then row-product partials (up to
// (nw + strips - 1) x 32).  Gradient view: V and Z (GNB x nmax each), then the
// partials of X = G V (2 nw slots of 32 x GNB).
__host__ __device__ inline int union_doubles(int nmax, int nw) {
  const int f = (3 + nw) * nmax;
  const int g = 2 * GNB * nmax + 2 * nw * 32 * GNB;
  return f > g ? f : g;
}
__host__ __device__ inline int fixed_doubles(int nmax) { return 2 * nmax + 64 + 4 * GNB * GNB; }
__host__ __device__ inline int smem_doubles(int nmax, int nw) {
  return fixed_doubles(nmax) + union_doubles(nmax, nw);
}

__device__ __forceinline__ Smem carve(int nmax) {
  Smem s;
  s.nmax = nmax;
  s.ev = dsm;
  s.tau = dsm + nmax;
  s.red = dsm + 2 * nmax;
  s.T = s.red + 64;
  s.P = s.T + GNB * GNB;
  s.K = s.P + GNB * GNB;
  s.C = s.K + GNB * GNB;
  double* u = s.C + GNB * GNB;
  s.vb0 = u;
  s.vb1 = u + nmax;
  s.p = u + 2 * nmax;
  s.ypart = u + 3 * nmax;
  s.Vs = u;
  s.Zs = u + GNB * nmax;
  s.Xp = u + 2 * GNB * nmax;
  return s;
}

template <int NW>
__device__ double block_maxabs(double x, double* red) {
  x = fabs(x);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = x;
  __syncthreads();
  double s = 0;
#pragma unroll
  for (int i = 0; i < NW; i++) s = fmax(s, red[i]);
  __syncthreads();
  return s;
}

// ---------------------------------------------------------------------------
// Copy-in with the exact skew check (isskewhermitian, skewhermitian.jl:84-94)
// ---------------------------------------------------------------------------
template <int NT, class MW>
__device__ bool copy_in(const double* __restrict__ A, int64_t lda, const MW& W, bool inplace, int n, bool check) {
  int bad = 0;
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += NT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    const double a = A[i + (int64_t)j * lda];
    if (!inplace) W.at(i, j) = a;
    if (check) bad |= !(a == -A[j + (int64_t)i * lda]);
  }
  return __syncthreads_or(bad) == 0;
}

// Working copy from page-locked host memory (A contiguous, leading dimension n):
// eight loads in flight per thread before their stores, so a warp keeps 2 KB of
// requests on the host link instead of 256 bytes.
template <int NT, class MW>
__device__ void copy_in_host(const double* __restrict__ A, const MW& W, int n) {
  constexpr int U = 8;
  const int64_t total = (int64_t)n * n;
  int64_t e0 = threadIdx.x;
  for (; e0 + (int64_t)(U - 1) * NT < total; e0 += (int64_t)U * NT) {
    double a[U];
#pragma unroll
    for (int u = 0; u < U; u++) a[u] = A[e0 + (int64_t)u * NT];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t e = e0 + (int64_t)u * NT;
      const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
      W.at(i, j) = a[u];
    }
  }
  for (; e0 < total; e0 += NT) {
    const int j = (int)(e0 / n), i = (int)(e0 - (int64_t)j * n);
    W.at(i, j) = A[e0];
  }
  __syncthreads();
}

// The finished gradient (n x n, contiguous, written by this CTA) to its
// page-locked host destination.
template <int NT>
__device__ void copy_out_host(const double* __restrict__ G, double* __restrict__ Gh, int n) {
  constexpr int U = 4;
  const int64_t total = (int64_t)n * n;
  int64_t e0 = threadIdx.x;
  for (; e0 + (int64_t)(U - 1) * NT < total; e0 += (int64_t)U * NT) {
    double a[U];
#pragma unroll
    for (int u = 0; u < U; u++) a[u] = G[e0 + (int64_t)u * NT];
#pragma unroll
    for (int u = 0; u < U; u++) Gh[e0 + (int64_t)u * NT] = a[u];
  }
  for (; e0 < total; e0 += NT) Gh[e0] = G[e0];
}

// ---------------------------------------------------------------------------
// Forward reduction
// ---------------------------------------------------------------------------

// Reflector for column c computed by the whole block (first column only).
template <int NT, class MW>
__device__ void reflector_block(const MW& W, int n, int c, const Smem& s, double* vout) {
  constexpr int NW = NT / 32;
  double part = 0.0;
  for (int r = c + 2 + (int)threadIdx.x; r < n; r += NT) {
    const double x = W.at(r, c);
    part = fma(x, x, part);
  }
  const double ss = block_sum<NW>(part, s.red);
  double xn = -1.0;
  if (ss_needs_scaling(ss)) {  // block-uniform rare path: norm with scaling
    double mx = 0.0;
    for (int r = c + 2 + (int)threadIdx.x; r < n; r += NT) mx = fmax(mx, fabs(W.at(r, c)));
    mx = block_maxabs<NW>(mx, s.red);
    double q = 0.0;
    if (mx > 0.0)
      for (int r = c + 2 + (int)threadIdx.x; r < n; r += NT) {
        const double x = W.at(r, c) / mx;
        q = fma(x, x, q);
      }
    q = block_sum<NW>(q, s.red);
    xn = mx * sqrt(q);
  }
  const Reflector R = make_reflector(W.at(c + 1, c), ss, xn);
  if (threadIdx.x == 0) {
    s.ev[c] = R.beta;
    s.tau[c] = R.tau;
  }
  for (int r = c + 1 + (int)threadIdx.x; r < n; r += NT) {
    const double vr = (R.tau == 0.0) ? 0.0 : (r == c + 1 ? 1.0 : W.at(r, c) * R.scale);
    vout[r] = vr;
    W.at(r, c) = vr;
  }
  __syncthreads();
}

// Warp 0 during step k: update column k+1 with (v_k, p_k), then build reflector
// k+1 from it into vout, ev[k+1], tau[k+1] and column k+1 of W.
template <class MW>
__device__ void lookahead_warp(const MW& W, int n, int k, const double* v, const double* p, double tauk,
                               const Smem& s, double* vout) {
  const int lane = threadIdx.x & 31;
  const int c = k + 1;
  const double vc = v[c], pc = p[c];
  double part = 0.0;
  for (int r = c + 1 + lane; r < n; r += 32) {
    double a = W.at(r, c);
    if (tauk != 0.0) a = fma(v[r], pc, fma(neg(p[r]), vc, a));
    W.at(r, c) = a;
    if (r >= c + 2) part = fma(a, a, part);
  }
  __syncwarp();
  const double ss = warp_sum(part);
  double xn = -1.0;
  if (ss_needs_scaling(ss)) {  // warp-uniform rare path
    double mx = 0.0;
    for (int r = c + 2 + lane; r < n; r += 32) mx = fmax(mx, fabs(W.at(r, c)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    double q = 0.0;
    if (mx > 0.0)
      for (int r = c + 2 + lane; r < n; r += 32) {
        const double x = W.at(r, c) / mx;
        q = fma(x, x, q);
      }
    xn = mx * sqrt(warp_sum(q));
  }
  const Reflector R = make_reflector(W.at(c + 1, c), ss, xn);
  if (lane == 0) {
    s.ev[c] = R.beta;
    s.tau[c] = R.tau;
  }
  for (int r = c + 1 + lane; r < n; r += 32) {
    const double vr = (R.tau == 0.0) ? 0.0 : (r == c + 1 ? 1.0 : W.at(r, c) * R.scale);
    vout[r] = vr;
    W.at(r, c) = vr;
  }
}

// Row products over S strips of 32 rows (lanes = rows) and mc columns.  When the
// strips do not divide evenly over the NW warps, the (strip, column) units, strip
// by strip, are cut into NW equal runs, one per warp: a run covers a piece of one
// or more strips, and piece (warp w, strip si) writes its partial sums to slot
// w + si, which no other piece uses (the runs are ordered), so at most NW + S - 1
// slots.  The partials of a row are then added in warp order.
struct StripSplit {
  int U;   // units per warp (0: whole strips, round robin)
  int mc;  // columns per strip
  __device__ __forceinline__ int first_warp(int si) const { return (si * mc) / U; }
  __device__ __forceinline__ int last_warp(int si) const { return ((si + 1) * mc - 1) / U; }
};

template <int NW>
__device__ __forceinline__ StripSplit strip_split(int S, int mc, int max_slots) {
  StripSplit sp;
  sp.mc = mc;
  sp.U = (S % NW == 0 || NW + S - 1 > max_slots) ? 0 : (S * mc + NW - 1) / NW;
  return sp;
}

// Dot of row i of W with v over columns [cb, ce), four loads in flight.
template <class MW>
__device__ __forceinline__ double row_dot(const MW& W, int i, int cb, int ce, const double* v) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int j = cb;
  for (; j + 3 < ce; j += 4) {
    const double w0 = W.at(i, j), w1 = W.at(i, j + 1), w2 = W.at(i, j + 2), w3 = W.at(i, j + 3);
    a0 = fma(w0, v[j], a0);
    a1 = fma(w1, v[j + 1], a1);
    a2 = fma(w2, v[j + 2], a2);
    a3 = fma(w3, v[j + 3], a3);
  }
  for (; j < ce; j++) a0 = fma(W.at(i, j), v[j], a0);
  return (a0 + a1) + (a2 + a3);
}

// p_i = tau * sum_{j >= c0} W[i,j] v_j for i >= r0.  Lanes are rows; whole strips per
// warp when they divide evenly, else the balanced split above.  Ends with p visible
// to the whole block.
template <int NT, class MW>
__device__ void rowprod(const MW& W, int n, int r0, int c0, const double* v, double tau, const Smem& s) {
  constexpr int NW = NT / 32;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mr = n - r0, mc = n - c0;
  const int S = (mr + 31) >> 5;
  const StripSplit sp = strip_split<NW>(S, mc, 1 << 30);
  if (sp.U == 0) {
    for (int si = w; si < S; si += NW) {
      const int i = r0 + si * 32 + lane;
      if (i < n) s.p[i] = tau * row_dot(W, i, c0, n, v);
    }
    __syncthreads();
    return;
  }
  const int u1 = min(S * mc, (w + 1) * sp.U);
  for (int u = w * sp.U; u < u1;) {
    const int si = u / mc;
    const int i = r0 + si * 32 + lane;
    if (i < n) s.ypart[(w + si) * 32 + lane] = row_dot(W, i, c0 + (u - si * mc), c0 + min(mc, u1 - si * mc), v);
    u = (si + 1) * mc;
  }
  __syncthreads();
  for (int i = r0 + (int)threadIdx.x; i < n; i += NT) {
    const int t = i - r0, si = t >> 5, ln = t & 31;
    double y = 0.0;
    for (int ww = sp.first_warp(si); ww <= sp.last_warp(si); ww++) y += s.ypart[(ww + si) * 32 + ln];
    s.p[i] = tau * y;
  }
  __syncthreads();
}

// Rank-2 skew update of the lower triangle {jstart <= j < i <= n-1}, mirrored.
// Participating thread t of T; elements dealt from the flattened triangle,
// four per iteration so four loads are in flight.
template <class MW>
__device__ void update_tri(const MW& W, int n, int jstart, const double* v, const double* p, int t, int T) {
  int j = jstart, r = t;
  while (j < n - 1 && r >= n - 1 - j) {
    r -= n - 1 - j;
    j++;
  }
  while (j < n - 1) {
    int jj[4], ii[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      jj[q] = j;
      ii[q] = j + 1 + r;
      if (j < n - 1) {
        r += T;
        while (j < n - 1 && r >= n - 1 - j) {
          r -= n - 1 - j;
          j++;
        }
      }
    }
    double a[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (jj[q] < n - 1) a[q] = W.at(ii[q], jj[q]);
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (jj[q] < n - 1) {
        const int i = ii[q], jc = jj[q];
        const double x = fma(v[i], p[jc], fma(neg(p[i]), v[jc], a[q]));
        W.at(i, jc) = x;
        W.at(jc, i) = neg(x);
      }
  }
}

template <int NT, class MW>
__device__ void forward(const MW& W, int n, const Smem& s) {
  if (n <= 1) return;
  if (n == 2) {
    if (threadIdx.x == 0) {
      s.ev[0] = W.at(1, 0);  // final real 1x1 step: tau = 0, beta = x (hessenberg.jl:27-29)
      s.tau[0] = 0.0;
    }
    __syncthreads();
    return;
  }
  reflector_block<NT>(W, n, 0, s, s.vb0);
  for (int k = 0; k + 2 < n; k++) {
    const double* v = (k & 1) ? s.vb1 : s.vb0;
    double* vn = (k & 1) ? s.vb0 : s.vb1;
    const double tauk = s.tau[k];
    if (tauk != 0.0) rowprod<NT>(W, n, k + 1, k + 1, v, tauk, s);
    const int w = threadIdx.x >> 5;
    if (k + 1 <= n - 3) {
      if (w == 0)
        lookahead_warp(W, n, k, v, s.p, tauk, s, vn);
      else if (tauk != 0.0)
        update_tri(W, n, k + 2, v, s.p, (int)threadIdx.x - 32, NT - 32);
    } else if (tauk != 0.0) {
      update_tri(W, n, k + 1, v, s.p, (int)threadIdx.x, NT);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    s.ev[n - 2] = W.at(n - 1, n - 2);
    s.tau[n - 2] = 0.0;
  }
  __syncthreads();
}

// log|Pf| and sign from ev and tau (pfaffian.jl:167-179):
//   log|Pf| = sum_{odd i} log|ev_i|, sign = prod sign(-ev_i) * (-1)^{#tau != 0}.
template <int NT>
__device__ void pfaffian_from_tridiag(int n, const Smem& s, double* logpf, double* sign) {
  constexpr int NW = NT / 32;
  const int h = n / 2;
  double lp = 0.0;
  int npos = 0, nzero = 0, ntau = 0;
  for (int a = threadIdx.x; a < h; a += NT) {
    const double e = s.ev[2 * a];
    lp += log(fabs(e));
    npos += (e > 0.0);
    nzero += (e == 0.0);
  }
  for (int a = threadIdx.x; a < n - 1; a += NT) ntau += (s.tau[a] != 0.0);
  const int tflip = __syncthreads_count((npos + ntau) & 1);
  const int tzero = __syncthreads_count(nzero > 0);
  const double total = block_sum<NW>(lp, s.red);
  if (threadIdx.x == 0) {
    *logpf = total;
    *sign = tzero ? 0.0 : ((tflip & 1) ? -1.0 : 1.0);
  }
}

// ---------------------------------------------------------------------------
// Gradient
// ---------------------------------------------------------------------------

// M = -1/2 T^{-1} (even n, all odd-position ev nonzero), its lower triangle and
// diagonal (the strictly upper triangle is filled at the end of the gradient).
// With O = even 0-based indices and E = odd ones, T = [[0, B], [-B^T, 0]] where
// B is lower bidiagonal (diag d_a = -ev[2a], sub s_a = ev[2a-1]) and
// T^{-1} = [[0, -B^{-T}], [B^{-1}, 0]]:  T^{-1}[2a+1, 2b] = (B^{-1})_{ab}
//   = (1/d_b) prod_{c=b+1..a} (-s_c/d_c)   for a >= b, zero otherwise; these are
// the only nonzero entries below the diagonal.
template <int NT>
__device__ void tinv_init(const GMat& G, int n, const Smem& s) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += NT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    if (i >= j) G.at(i, j) = 0.0;
  }
  const int h = n / 2;
  double* ratio = s.Vs;  // -s_c/d_c = ev[2c-1]/ev[2c], 1 <= c < h
  for (int c = 1 + (int)threadIdx.x; c < h; c += NT) ratio[c] = s.ev[2 * c - 1] / s.ev[2 * c];
  __syncthreads();
  for (int b = threadIdx.x; b < h; b += NT) {
    double x = 0.5 / s.ev[2 * b];  // -1/2 * (1/d_b)
    for (int a = b; a < h; a++) {
      G.at(2 * a + 1, 2 * b) = x;
      if (a + 1 < h) x *= ratio[a + 1];
    }
  }
  __syncthreads();
}

// G <- Q G Q^T, G holding -1/2 T^{-1} on entry (its lower triangle and diagonal);
// reflectors from W's lower part.  Only the lower triangle is read and written while
// the blocks run; the upper triangle is written at the end as -G^T.
template <int NT, class MW>
__device__ void gradient(const MW& W, const GMat& G, int n, const Smem& s) {
  constexpr int NW = NT / 32;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int nref = n - 2;  // reflectors 0..n-3 (reflector n-2 is the trivial 1x1)
  double* Vs = s.Vs;       // V block, row-major: Vs[(r - k0 - 1) * GNB + l]
  double* Zs = s.Zs;       // X, then Z', row-major: Zs[i * GNB + l]
  double* Xp = s.Xp;       // partial products / reduction scratch
  for (int kend = nref; kend > 0; kend -= GNB) {
    const int k0 = max(0, kend - GNB), nb = kend - k0;
    const int r0 = k0 + 1, m = n - r0;
    // 1. stage V (m x GNB; columns past nb are zero)
    for (int idx = tid; idx < m * GNB; idx += NT) {
      const int rr = idx / GNB, l = idx - rr * GNB;
      const int r = r0 + rr, kk = k0 + l;
      double val = 0.0;
      if (l < nb) val = (r < kk + 1) ? 0.0 : (r == kk + 1 ? 1.0 : W.at(r, kk));
      Vs[idx] = val;
    }
    __syncthreads();
    // 2. Gram P = V^T V (pairs l1 < l2), then T_b (forward, columnwise)
    {
      double part[32];
#pragma unroll
      for (int q = 0; q < 32; q++) part[q] = 0.0;
      for (int rr = tid; rr < m; rr += NT) {
        double vr[GNB];
#pragma unroll
        for (int l = 0; l < GNB; l++) vr[l] = Vs[rr * GNB + l];
#pragma unroll
        for (int l1 = 0; l1 < GNB; l1++)
#pragma unroll
          for (int l2 = l1 + 1; l2 < GNB; l2++) part[pair_slot(l1, l2)] = fma(vr[l1], vr[l2], part[pair_slot(l1, l2)]);
      }
      block_reduce_pairs<NT>(part, 28, Xp, s.P);
      if (w == 0) {  // T[l][l] = tau_l, T[0:l, l] = -tau_l T[0:l, 0:l] P[0:l, l]
        for (int q = lane; q < GNB * GNB; q += 32) s.T[q] = 0.0;
        __syncwarp();
        for (int l = 0; l < nb; l++) {
          const double tl = s.tau[k0 + l];
          double acc = 0.0;
          if (lane < l)
            for (int j = lane; j < l; j++) acc = fma(s.T[lane * GNB + j], s.P[pair_slot(j, l)], acc);
          __syncwarp();
          if (lane < l) s.T[lane * GNB + l] = neg(tl * acc);
          if (lane == l) s.T[l * GNB + l] = tl;
          __syncwarp();
        }
      }
      __syncthreads();
    }
    // 3. X = G[:, r0:n] V  (n x GNB), lanes = rows, (strip, chunk) items.  Only the
    //    rows >= r0 and the even rows above r0 are computed (the odd ones are zero):
    //    virtual row t is row r0 + t for t < m and row 2 (t - m) after that.
    //    Strips are split over the warps as in rowprod (partials: 2 NW slots).
    const int nvr = m + ((r0 + 1) >> 1);
    {
      const int S = (nvr + 31) >> 5;
      const StripSplit sp = strip_split<NW>(S, m, 2 * NW);
      // X row i over columns [cb, ce): G[i, j] from the lower triangle, G[j, i] negated
      // above the diagonal (strided reads that hit L2: a load feeds GNB FMAs)
      auto xrow = [&](int i, int cb, int ce, double* acc) {
#pragma unroll
        for (int l = 0; l < GNB; l++) acc[l] = 0.0;
        for (int j = cb; j < ce; j++) {
          const double g = (j < i) ? G.at(i, j) : ((j > i) ? neg(G.at(j, i)) : 0.0);
          const double* vj = Vs + (j - r0) * GNB;
#pragma unroll
          for (int l = 0; l < GNB; l++) acc[l] = fma(g, vj[l], acc[l]);
        }
      };
      // the rows of strip si over columns [cb, ce), one row per lane.  A strip of at
      // most 16 rows (the last one) would leave lanes idle for the whole column loop,
      // so groups of p2 lanes (p2 the power of two >= its rows) take slices of the
      // columns and add their partials by xor shuffles; lane L < rows then holds row
      // 32 si + L.  Returns the strip's rows.
      auto xstrip = [&](int si, int cb, int ce, double* acc) -> int {
        const int rs = min(32, nvr - 32 * si);
        if (rs > 16) {
          const int t = si * 32 + lane;
          if (lane < rs) {
            xrow(t < m ? r0 + t : 2 * (t - m), cb, ce, acc);
          } else {
#pragma unroll
            for (int l = 0; l < GNB; l++) acc[l] = 0.0;
          }
          return rs;
        }
        int p2 = 1;
        while (p2 < rs) p2 <<= 1;
        const int g = lane / p2, rl = lane - g * p2, groups = 32 / p2;
        const int seg = (ce - cb + groups - 1) / groups;
        const int sb = cb + g * seg, se = min(ce, sb + seg);
        const int t = si * 32 + rl;
        if (rl < rs && sb < se) {
          xrow(t < m ? r0 + t : 2 * (t - m), sb, se, acc);
        } else {
#pragma unroll
          for (int l = 0; l < GNB; l++) acc[l] = 0.0;
        }
        for (int o = p2; o < 32; o <<= 1) {
#pragma unroll
          for (int l = 0; l < GNB; l++) acc[l] += __shfl_xor_sync(0xffffffffu, acc[l], o);
        }
        return rs;
      };
      if (sp.U == 0) {
        for (int si = w; si < S; si += NW) {
          double acc[GNB];
          const int rs = xstrip(si, r0, n, acc);
          const int t = si * 32 + lane;
          if (lane < rs) {
            const int i = t < m ? r0 + t : 2 * (t - m);
#pragma unroll
            for (int l = 0; l < GNB; l++) Zs[i * GNB + l] = acc[l];
          }
        }
      } else {
        const int u1 = min(S * m, (w + 1) * sp.U);
        for (int u = w * sp.U; u < u1;) {
          const int si = u / m;
          double acc[GNB];
          const int rs = xstrip(si, r0 + (u - si * m), r0 + min(m, u1 - si * m), acc);
          if (lane < rs) {
#pragma unroll
            for (int l = 0; l < GNB; l++) Xp[((w + si) * 32 + lane) * GNB + l] = acc[l];
          }
          u = (si + 1) * m;
        }
      }
      for (int idx = tid; idx < (r0 >> 1) * GNB; idx += NT) {  // the odd rows above r0
        const int i = 2 * (idx / GNB) + 1, l = idx % GNB;
        Zs[i * GNB + l] = 0.0;
      }
      __syncthreads();
      if (sp.U != 0) {
        for (int idx = tid; idx < nvr * GNB; idx += NT) {
          const int t = idx / GNB, l = idx - t * GNB;
          const int i = t < m ? r0 + t : 2 * (t - m);
          const int si = t >> 5, ln = t & 31;
          double x = 0.0;
          for (int ww = sp.first_warp(si); ww <= sp.last_warp(si); ww++) x += Xp[((ww + si) * 32 + ln) * GNB + l];
          Zs[i * GNB + l] = x;
        }
        __syncthreads();
      }
    }
    // 4. K = V^T X over the rows of V (skew: pairs l1 < l2); Ch = -1/2 T K T^T
    {
      double part[32];
#pragma unroll
      for (int q = 0; q < 32; q++) part[q] = 0.0;
      for (int rr = tid; rr < m; rr += NT) {
        double vr[GNB], xr[GNB];
#pragma unroll
        for (int l = 0; l < GNB; l++) {
          vr[l] = Vs[rr * GNB + l];
          xr[l] = Zs[(r0 + rr) * GNB + l];
        }
#pragma unroll
        for (int l1 = 0; l1 < GNB; l1++)
#pragma unroll
          for (int l2 = l1 + 1; l2 < GNB; l2++) part[pair_slot(l1, l2)] = fma(vr[l1], xr[l2], part[pair_slot(l1, l2)]);
      }
      block_reduce_pairs<NT>(part, 28, Xp, s.K);
      if (w == 0) {
        double* Kf = s.C;  // full skew K
        for (int q = lane; q < GNB * GNB; q += 32) {
          const int l1 = q / GNB, l2 = q - l1 * GNB;
          Kf[q] = (l1 < l2) ? s.K[pair_slot(l1, l2)] : (l1 > l2 ? neg(s.K[pair_slot(l2, l1)]) : 0.0);
        }
        __syncwarp();
        for (int q = lane; q < GNB * GNB; q += 32) {  // TK = T Kf (into P, free now)
          const int a = q / GNB, b = q - a * GNB;
          double acc = 0.0;
          for (int c = a; c < GNB; c++) acc = fma(s.T[a * GNB + c], Kf[c * GNB + b], acc);
          s.P[q] = acc;
        }
        __syncwarp();
        for (int q = lane; q < GNB * GNB; q += 32) {  // Ch = -1/2 (T K) T^T (into K)
          const int a = q / GNB, b = q - a * GNB;
          double acc = 0.0;
          for (int c = b; c < GNB; c++) acc = fma(s.P[a * GNB + c], s.T[b * GNB + c], acc);
          s.K[q] = -0.5 * acc;
        }
      }
      __syncthreads();
    }
    // 5. Z' = X T^T + V Ch  (only rows of V get the V Ch term; the odd rows above r0
    //    stay zero)
    for (int t = tid; t < nvr; t += NT) {
      const int i = t < m ? r0 + t : 2 * (t - m);
      double x[GNB], z[GNB];
#pragma unroll
      for (int l = 0; l < GNB; l++) x[l] = Zs[i * GNB + l];
#pragma unroll
      for (int l = 0; l < GNB; l++) {
        double acc = 0.0;
#pragma unroll
        for (int c = l; c < GNB; c++) acc = fma(x[c], s.T[l * GNB + c], acc);
        z[l] = acc;
      }
      if (i >= r0) {
        double vr[GNB];
#pragma unroll
        for (int l = 0; l < GNB; l++) vr[l] = Vs[(i - r0) * GNB + l];
#pragma unroll
        for (int l = 0; l < GNB; l++) {
          double acc = z[l];
#pragma unroll
          for (int c = 0; c < GNB; c++) acc = fma(vr[c], s.K[c * GNB + l], acc);
          z[l] = acc;
        }
      }
#pragma unroll
      for (int l = 0; l < GNB; l++) Zs[i * GNB + l] = z[l];
    }
    __syncthreads();
    // 6. G[i,j] += V_i . Z'_j - Z'_i . V_j for i >= r0, j < i (lower triangle only).
    //    Row strips of 32, strip si holding rows [ib, ib + 32), ib = n - 32(si+1)
    //    (aligned to the last row, the partial strip is the one next to r0, which
    //    has the fewest columns).  Items of a strip: the even columns below r0 in
    //    blocks of 32 (the odd ones do not change; V_j = 0 there, so only V_i . Z'_j),
    //    the columns [r0, ib) in blocks of 32 ending at ib (below every row of the
    //    strip: no per-lane bound), and the diagonal triangle.  A warp instruction
    //    costs the FP64 pipe the same with idle lanes, so the triangle (31 steps at
    //    half the lanes row by row) runs as a 16 x 16 square, two 8 x 8 squares and
    //    four 8-row triangles: 8 + 4 + 7 steps.
    {
      const int S = (m + 31) >> 5;
      const int nec = (r0 + 1) >> 1;  // even columns below r0
      const int eb = (nec + 31) >> 5;
      auto nfull = [&](int si) {
        const int ib = n - 32 * (si + 1);
        return ib > r0 ? (ib - r0 + 31) >> 5 : 0;
      };
      // G[i, j] += V_i . Z'_j - Z'_i . V_j (j >= r0)
      auto elem = [&](int i, int j, const double* vi, const double* zi) {
        const double* zj = Zs + j * GNB;
        const double* vj = Vs + (j - r0) * GNB;
        double a0 = G.at(i, j), a1 = 0.0;
#pragma unroll
        for (int l = 0; l < GNB; l += 2) {
          a0 = fma(vi[l], zj[l], a0);
          a1 = fma(vi[l + 1], zj[l + 1], a1);
        }
#pragma unroll
        for (int l = 0; l < GNB; l += 2) {
          a0 = fma(neg(zi[l]), vj[l], a0);
          a1 = fma(neg(zi[l + 1]), vj[l + 1], a1);
        }
        G.at(i, j) = a0 + a1;
      };
      auto load_row = [&](int i, double* vi, double* zi) {
#pragma unroll
        for (int l = 0; l < GNB; l++) {
          vi[l] = Vs[(i - r0) * GNB + l];
          zi[l] = Zs[i * GNB + l];
        }
      };
      int total = 0;
      for (int si = 0; si < S; si++) total += eb + nfull(si) + 1;
      for (int item = w; item < total; item += NW) {
        int si = 0, rem = item;
        for (;;) {
          const int nbk = eb + nfull(si) + 1;
          if (rem < nbk) break;
          rem -= nbk;
          si++;
        }
        const int ib = n - 32 * (si + 1);
        double vi[GNB], zi[GNB];
        if (rem < eb) {  // even columns j < r0
          const int i = ib + lane;  // below r0 in the partial strip: idle
          if (i >= r0) {
#pragma unroll
            for (int l = 0; l < GNB; l++) vi[l] = Vs[(i - r0) * GNB + l];
            const int qe = min(32 * rem + 32, nec);
            for (int q = 32 * rem; q < qe; q++) {
              const int j = 2 * q;
              const double* zj = Zs + j * GNB;
              double a0 = G.at(i, j), a1 = 0.0;
#pragma unroll
              for (int l = 0; l < GNB; l += 2) {
                a0 = fma(vi[l], zj[l], a0);
                a1 = fma(vi[l + 1], zj[l + 1], a1);
              }
              G.at(i, j) = a0 + a1;
            }
          }
        } else if (rem < eb + nfull(si)) {  // columns [jb, je) below the strip (ib > r0)
          const int je = ib - 32 * (rem - eb), jb = max(r0, je - 32);
          const int i = ib + lane;
          load_row(i, vi, zi);
          for (int j = jb; j < je; j++) elem(i, j, vi, zi);
        } else if (ib >= r0) {  // the diagonal triangle of rows and columns [ib, ib + 32)
          {  // rows 16..31 x columns 0..15: two lanes per row, 8 columns each
            const int i = ib + 16 + (lane & 15), j0 = ib + ((lane >> 4) << 3);
            load_row(i, vi, zi);
#pragma unroll 1
            for (int q = 0; q < 8; q++) elem(i, j0 + q, vi, zi);
          }
          {  // rows 8..15 x columns 0..7 and rows 24..31 x columns 16..23: 4 columns each
            const int k = lane & 15, h = lane >> 4;
            const int i = ib + 16 * h + 8 + (k & 7), j0 = ib + 16 * h + ((k >> 3) << 2);
            load_row(i, vi, zi);
#pragma unroll 1
            for (int q = 0; q < 4; q++) elem(i, j0 + q, vi, zi);
          }
          {  // the four 8-row triangles on the diagonal
            const int t = lane >> 3, r = lane & 7;
            const int i = ib + 8 * t + r, j0 = ib + 8 * t;
            load_row(i, vi, zi);
            for (int q = 0; q < r; q++) elem(i, j0 + q, vi, zi);
          }
        } else {  // the partial strip: rows [r0, ib + 32), columns [r0, row)
          const int i = ib + lane;
          if (i >= r0) {
            load_row(i, vi, zi);
            for (int j = r0; j < i; j++) elem(i, j, vi, zi);
          }
        }
      }
      __syncthreads();
    }
  }
  // the upper triangle: G[j, i] = -G[i, j] for j < i (consecutive threads write
  // consecutive rows of a column; the reads are strided and hit L2)
  const int64_t total = (int64_t)n * n;
  for (int64_t e = tid; e < total; e += NT) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    if (j < i) G.at(j, i) = neg(G.at(i, j));
  }
  __syncthreads();
}

template <int NT>
__device__ void fill(const GMat& G, int n, double val) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += NT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    G.at(i, j) = val;
  }
}

// One matrix, start to finish.
struct Job {
  const double* A;
  int64_t lda;
  int n;
  double* G;  // gradient output or null
  int64_t ldg;
  double* logpf;
  double* sign;
  double* ev_out;    // optional (n-1)
  double* tau_out;   // optional (n-1)
  double* refl_out;  // optional n x n: the reduced matrix (reflectors below the subdiagonal)
  int* status;
  bool check;
  bool want_pf;
  bool host_in;  // A in page-locked host memory (batched path: lda == n, never in place)
};

template <int NT, class MW>
__device__ void run_job(const Job& J, const MW& W, bool inplace, const Smem& s) {
  const int n = J.n;
  bool ok = true;
  if (J.host_in) {
    copy_in_host<NT>(J.A, W, n);
    if (J.check) {  // on the working copy: no strided reads over the host link
      int bad = 0;
      for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += NT) {
        const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
        bad |= !(W.at(i, j) == -W.at(j, i));
      }
      ok = __syncthreads_or(bad) == 0;
    }
  } else {
    ok = copy_in<NT>(J.A, J.lda, W, inplace, n, J.check);
  }
  const GMat G{J.G, J.ldg};
  if (!ok) {
    if (threadIdx.x == 0) {
      if (J.logpf) *J.logpf = nan("");
      if (J.sign) *J.sign = nan("");
      if (J.status) *J.status = SKEW_NOT_SKEW;
    }
    if (J.G) fill<NT>(G, n, nan(""));
    __syncthreads();
    return;
  }
  const bool odd = (n & 1);
  if (J.want_pf && odd) {  // pfaffian.jl:169
    if (threadIdx.x == 0) {
      *J.logpf = -INFINITY;
      *J.sign = 0.0;
      if (J.status) *J.status = SKEW_SINGULAR;
    }
    if (J.G) fill<NT>(G, n, nan(""));
    __syncthreads();
    if (!J.ev_out) return;
  }
  forward<NT>(W, n, s);
  if (J.refl_out) {
    const int64_t total = (int64_t)n * n;
    for (int64_t e = threadIdx.x; e < total; e += NT) {
      const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
      J.refl_out[e] = W.at(i, j);
    }
  }
  if (J.ev_out || J.tau_out)
    for (int a = threadIdx.x; a < n - 1; a += NT) {
      if (J.ev_out) J.ev_out[a] = s.ev[a];
      if (J.tau_out) J.tau_out[a] = s.tau[a];
    }
  if (!J.want_pf || odd) {
    if (threadIdx.x == 0 && J.status && !J.want_pf) *J.status = SKEW_OK;
    __syncthreads();
    return;
  }
  __shared__ double s_lp, s_sg;
  pfaffian_from_tridiag<NT>(n, s, &s_lp, &s_sg);
  __syncthreads();
  const double lp = s_lp, sg = s_sg;
  if (threadIdx.x == 0) {
    *J.logpf = lp;
    *J.sign = sg;
    if (J.status) *J.status = (sg == 0.0) ? SKEW_SINGULAR : SKEW_OK;
  }
  if (J.G) {
    if (sg == 0.0) {
      fill<NT>(G, n, nan(""));
    } else {
      tinv_init<NT>(G, n, s);
      gradient<NT>(W, G, n, s);
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Persistent batched kernel over order[begin:end) (matrices sorted largest
// first); CTAs take the next matrix from an atomic counter.  With a split, the
// slice is two regions, [begin, split) holding the largest matrices (half the work)
// and [split, end) the rest, each with its own counter.  The CTAs of the first half
// of the grid start in the first region and those of the second half in the second
// (one CTA of each per SM), both largest first; a CTA whose region is empty takes
// from the other.  Co-resident CTAs then hold a large and a smaller working copy
// instead of two large ones in the same phase (less L2 overflow), and the launch
// still ends on the smallest matrices.
// HOST: the inputs are read from, and the gradients written to, page-locked host
// memory (a separate instantiation, so the device-resident kernels are unchanged).
template <int NT, bool SM, bool HOST>
__global__ void __launch_bounds__(NT) batch_kernel(BatchParams P, int tridiag_only) {
  const Smem s = carve(P.nmax);
  const int woff = smem_doubles(P.nmax, NT / 32);
  __shared__ int s_next;
  for (;;) {
    if (threadIdx.x == 0) {
      if (P.split > P.begin) {
        const int second = blockIdx.x >= (gridDim.x >> 1) ? 1 : 0;
        int t = P.end;
        for (int pass = 0; pass < 2; pass++) {
          const int r = second ^ pass;  // region: 0 [begin, split), 1 [split, end)
          const int x = (int)atomicAdd(P.counter + r, 1u) + (r ? P.split : P.begin);
          if (x < (r ? P.end : P.split)) {
            t = x;
            break;
          }
        }
        s_next = t;
      } else {
        s_next = (int)atomicAdd(P.counter, 1u) + P.begin;
      }
    }
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= P.end) break;
    const int b = P.order[t];
    const int n = P.n[b];
    Job J;
    J.A = P.A[b];
    J.lda = n;
    J.n = n;
    J.G = tridiag_only ? nullptr : (P.grad ? P.grad[b] : nullptr);
    J.ldg = n;
    J.logpf = tridiag_only ? nullptr : P.logpf + b;
    J.sign = tridiag_only ? nullptr : P.sign + b;
    J.ev_out = P.ev_out ? P.ev_out + P.ev_off[b] : nullptr;
    J.tau_out = P.tau_out ? P.tau_out + P.ev_off[b] : nullptr;
    J.refl_out = P.refl_out ? P.refl_out[b] : nullptr;
    J.status = tridiag_only ? nullptr : P.status + b;
    J.check = P.check != 0;
    J.want_pf = !tridiag_only;
    J.host_in = HOST && P.host_in != 0;
    if constexpr (SM) {
      const SMat W{woff, n | 1};
      run_job<NT>(J, W, false, s);
    } else {
      const GMat W{P.gws + (size_t)blockIdx.x * P.gws_slot, (int64_t)(n | 1)};
      run_job<NT>(J, W, false, s);
    }
    // run_job ends with a barrier after its last write of G
    if constexpr (HOST)
      if (J.G && P.grad_host) copy_out_host<NT>(J.G, P.grad_host[b], n);
  }
}

// Single matrix, in place (W = A), one CTA.
template <int NT>
__global__ void __launch_bounds__(NT) single_kernel(SingleParams P) {
  const Smem s = carve(P.n > 0 ? P.n : 1);
  Job J;
  J.A = P.A;
  J.lda = P.lda;
  J.n = P.n;
  J.G = P.G;
  J.ldg = P.ldg;
  J.logpf = P.logpf;
  J.sign = P.sign;
  J.ev_out = P.ev;
  J.tau_out = P.tau;
  J.refl_out = nullptr;
  J.status = P.info;
  J.check = P.check != 0;
  J.want_pf = P.want_pf != 0;
  J.host_in = false;
  const GMat W{P.A, P.lda};
  run_job<NT>(J, W, true, s);
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
constexpr int NT_SMALL = 128;   // shared-memory buckets up to n = 96
constexpr int NT_LARGE = 256;   // shared-memory buckets above 96 (one CTA per SM)
constexpr int NT_GLOBAL = 512;  // optional global-memory variant: one CTA of 16 warps per SM

// Threads per CTA: the bucket's choice (from the handle's tuning table), or the
// default for the working copy's location: 128 for shared-memory copies up to
// n = 96, 256 above and for global-memory copies (measured best on GB300).
static int threads_for(int nmax, bool smem_matrix, int nt) {
  if (smem_matrix) {
    if (nt == 128 || nt == 256 || nt == 512) return nt;
    return nmax <= 96 ? NT_SMALL : NT_LARGE;
  }
  return nt == NT_GLOBAL ? NT_GLOBAL : NT_LARGE;
}

size_t batch_smem_bytes(int nmax, bool smem_matrix, int nt_req) {
  const int nt = threads_for(nmax, smem_matrix, nt_req);
  size_t b = sizeof(double) * (size_t)smem_doubles(nmax, nt / 32);
  if (smem_matrix) b += sizeof(double) * (size_t)nmax * (size_t)(nmax | 1);
  return b;
}

// Per-instantiation record of the devices on which the shared-memory limit of
// batch_kernel<NT, SM> has been raised (shared by the launch and the occupancy query).
template <int NT, bool SM, bool HOST>
std::atomic<uint64_t> g_smem_raised{0};

template <int NT, bool SM, bool HOST>
static cudaError_t launch_t(const BatchParams& P, int grid, size_t smem, cudaStream_t st, int tridiag_only) {
  cudaError_t e = raise_smem_limit_once((const void*)batch_kernel<NT, SM, HOST>, g_smem_raised<NT, SM, HOST>);
  if (e != cudaSuccess) return e;
  batch_kernel<NT, SM, HOST><<<grid, NT, smem, st>>>(P, tridiag_only);
  return cudaGetLastError();
}

template <bool HOST>
static cudaError_t launch_pf(const BatchParams& P, int grid, cudaStream_t st, bool tridiag_only) {
  const bool sm = P.smem_matrix != 0;
  const size_t smem = batch_smem_bytes(P.nmax, sm, P.nt);
  const int nt = threads_for(P.nmax, sm, P.nt);
  if (sm && nt == 128) return launch_t<128, true, HOST>(P, grid, smem, st, tridiag_only);
  if (sm && nt == 256) return launch_t<256, true, HOST>(P, grid, smem, st, tridiag_only);
  if (sm) return launch_t<512, true, HOST>(P, grid, smem, st, tridiag_only);
  if (nt == NT_LARGE) return launch_t<NT_LARGE, false, HOST>(P, grid, smem, st, tridiag_only);
  return launch_t<NT_GLOBAL, false, HOST>(P, grid, smem, st, tridiag_only);
}

cudaError_t launch_batch_pf(const BatchParams& P, int grid, cudaStream_t st, bool tridiag_only) {
  if (P.host_in || P.grad_host) return launch_pf<true>(P, grid, st, tridiag_only);
  return launch_pf<false>(P, grid, st, tridiag_only);
}

cudaError_t launch_single(const SingleParams& P, cudaStream_t st) {
  const int nmax = P.n > 0 ? P.n : 1;
  const size_t smem = sizeof(double) * (size_t)smem_doubles(nmax, NT_LARGE / 32);
  cudaError_t e =
      cudaFuncSetAttribute(single_kernel<NT_LARGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  single_kernel<NT_LARGE><<<1, NT_LARGE, smem, st>>>(P);
  return cudaGetLastError();
}

int batch_threads() { return NT_LARGE; }

// Occupancy of the device-resident instantiation (the host one has the same
// shared memory and launch bounds).
template <int NT, bool SM>
static int occ_t(size_t smem) {
  int occ = 0;
  cudaError_t e = raise_smem_limit_once((const void*)batch_kernel<NT, SM, false>, g_smem_raised<NT, SM, false>);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel<NT, SM, false>, NT, smem);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return 1;
  }
  return occ;
}

int batch_occupancy(int nmax, bool smem_matrix, int nt_req) {
  const size_t smem = batch_smem_bytes(nmax, smem_matrix, nt_req);
  const int nt = threads_for(nmax, smem_matrix, nt_req);
  if (smem_matrix && nt == 128) return occ_t<128, true>(smem);
  if (smem_matrix && nt == 256) return occ_t<256, true>(smem);
  if (smem_matrix) return occ_t<512, true>(smem);
  if (nt == NT_LARGE) return occ_t<NT_LARGE, false>(smem);
  return occ_t<NT_GLOBAL, false>(smem);
}

}  // namespace skew
