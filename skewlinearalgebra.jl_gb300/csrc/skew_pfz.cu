// Pfaffian of a complex skew-symmetric matrix (A == -transpose(A)) by
// Parlett-Reid elimination with pivoting: pfaffian.jl:98-137 (_pfaffian!, the
// running product) and :193-233 (_logabspfaffian!, log|Pf| and cis(phase)).
//
// Step k (0-based, k = 0, 2, ..., n-2; p = k + 1):
//   kp = argmax_{i > k} |A[i,k]| (first maximum); if kp != p swap rows and
//   columns p <-> kp (phase += pi, pf = -pf); z = A[p,k]; z == 0 -> Pf = 0;
//   the reference's pivot is A[k,p] = -z: logpf += log|z|, phase += angle(-z),
//   pf *= -z; tau_i = A[i,k] / z and c_i = A[i,p] for i > p;
//   A[i,j] += tau_i c_j - tau_j c_i on the trailing block i, j > p.
// (The reference divides A[k,j] by A[k,p]; for a skew-symmetric A both are the
// negated lower entries, so the quotient is the same.)
//
// GB300 design.  Only the strictly lower triangle is stored and updated (the
// update keeps A skew-symmetric, so the upper half is its negation): half the
// reference's work, 8 DFMA per entry and step, which makes the elimination
// FP64-pipe bound (2 DFMA/clk/SM) in shared memory and in L2 alike.  The
// symmetric swap is never written back: after the swap only row/column kp of
// the trailing block changes, and its new values are the old column p (which
// the step reads but never writes), so the update reads them from there, and
// tau and c are formed from the old entries through the permutation.  Each
// step is then two phases, "T" (pivot, tau, c) and "U" (update), separated by
// one barrier each; the argmax for the next step is taken in phase U while the
// first trailing column is written.
//
//   pfz_cta_kernel  one CTA per matrix (batches; small single matrices): the
//                   packed triangle in shared memory when it fits, else in a
//                   per-CTA global slot; __syncthreads between the phases.
//   pfz_grid_kernel one large matrix, in place on its lower triangle, over a
//                   cooperative grid with bounded grid barriers; the update is
//                   tiled 32 rows x 16 columns per warp (tau_i, c_i held in
//                   registers for the tile), reads through L2 (__ldcg).
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <atomic>

#include "../../include/skewgpu.h"
#include "skew_common.cuh"
#include "skew_complex.cuh"
#include "skew_internal.h"

namespace skew {

namespace {

constexpr double PFZ_PI = 3.141592653589793;

__device__ __forceinline__ zc zneg(zc a) { return zc{-a.re, -a.im}; }

// Argmax keys.  Julia's argmax(abs.(x)) takes the first maximum, with NaN above
// every number.  A key is the bit pattern of a non-negative double (|x| or |x|^2)
// read as an unsigned integer, which orders like the value; every NaN maps to one
// pattern above +Inf.  Comparisons and reductions then run on the integer pipe:
// on this part a warp-wide FP64 instruction costs the FP64 pipe as much as a full
// warp's work, so the serial pivot search must not use it.
typedef unsigned long long u64;
constexpr u64 KEY_NAN = 0x7FF8000000000000ull;
constexpr int NO_ROW = INT_MAX;
__device__ __forceinline__ u64 key_of(double v) {
  const u64 b = (u64)__double_as_longlong(v);
  return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull ? KEY_NAN : b;
}
__device__ __forceinline__ bool key_better(u64 a, int i, u64 b, int j) { return a > b || (a == b && i < j); }

__device__ __forceinline__ void warp_argmax(u64& v, int& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const u64 w = __shfl_xor_sync(0xffffffffu, v, o);
    const int j = __shfl_xor_sync(0xffffffffu, i, o);
    if (key_better(w, j, v, i)) {
      v = w;
      i = j;
    }
  }
}

// x == -y as IEEE comparisons of both parts (so +0 == -0 and NaN never equal),
// on the integer pipe.
__device__ __forceinline__ bool neg_equal_part(double a, double b) {
  const u64 x = (u64)__double_as_longlong(a), y = (u64)__double_as_longlong(b);
  const u64 mag = 0x7FFFFFFFFFFFFFFFull;
  if ((x & mag) > 0x7FF0000000000000ull || (y & mag) > 0x7FF0000000000000ull) return false;  // NaN
  return x == (y ^ 0x8000000000000000ull) || ((x | y) & mag) == 0;
}
__device__ __forceinline__ bool neg_equal(zc x, zc y) {
  return neg_equal_part(x.re, y.re) && neg_equal_part(x.im, y.im);
}

__device__ __forceinline__ bool is_zero_bits(zc z) {
  return (((u64)__double_as_longlong(z.re) | (u64)__double_as_longlong(z.im)) << 1) == 0;
}

// x + ti * cj - tj * ci
__device__ __forceinline__ zc rank2(zc x, zc ti, zc cj, zc tj, zc ci) {
  zc r;
  r.re = fma(ti.re, cj.re, fma(-ti.im, cj.im, fma(-tj.re, ci.re, fma(tj.im, ci.im, x.re))));
  r.im = fma(ti.re, cj.im, fma(ti.im, cj.re, fma(-tj.re, ci.im, fma(-tj.im, ci.re, x.im))));
  return r;
}

// 1/b with an exact power-of-two prescale and one real division.
__device__ __forceinline__ zc zrcp(zc b) {
  int e;
  frexp(fmax(fabs(b.re), fabs(b.im)), &e);
  const double s = ldexp(1.0, -max(e, -1021));
  const double br = b.re * s, bi = b.im * s;
  const double r = 1.0 / fma(br, br, bi * bi);
  return zc{(br * r) * s, (-bi * r) * s};
}

// Key |x|^2 (two FP64 operations; Julia's abs is hypot).  Outside [2^-1000, 2^1000]
// the squares lose the order, and the caller repeats the search with hypot.
__device__ __forceinline__ u64 sqkey(zc x) { return key_of(fma(x.re, x.re, x.im * x.im)); }
__device__ __forceinline__ bool sqkey_ok(u64 k) {
  return k >= 0x0170000000000000ull /* 2^-1000 */ && k <= 0x7E70000000000000ull /* 2^1000 */;
}
__device__ __forceinline__ u64 abskey(zc x) { return key_of(hypot(x.re, x.im)); }

// Compensated sums (hi + lo) for log|Pf| and the phase: the reference adds the
// n/2 terms in one FP64 running sum, whose rounding (and that of the phase's
// multiples of pi) grows with n; these sums stay within a few ulps.
struct DD {
  double hi, lo;
};
__device__ __forceinline__ DD two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  const double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return DD{s, e};
}
__device__ __forceinline__ DD dd_add(DD a, double b) {
  const DD t = two_sum(a.hi, b);
  return DD{t.hi, __dadd_rn(a.lo, t.lo)};
}
__device__ __forceinline__ DD dd_warp_sum(DD a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double h = __shfl_xor_sync(0xffffffffu, a.hi, o);
    const double l = __shfl_xor_sync(0xffffffffu, a.lo, o);
    const DD t = two_sum(a.hi, h);
    a = DD{t.hi, __dadd_rn(__dadd_rn(a.lo, l), t.lo)};
  }
  return a;
}
constexpr double TWO_PI_HI = 6.283185307179586;        // 2 pi rounded to FP64
constexpr double TWO_PI_LO = 2.4492935982947064e-16;   // 2 pi - TWO_PI_HI
constexpr double PI_LO = 1.2246467991473532e-16;       // pi - PFZ_PI

// The outputs of one elimination from its recorded pivots (piv[t] = -A[p,k] of
// step t, the reference's A[k,k+1]), on one warp (all lanes call):
//   log|Pf| = sum_t log|piv_t|, phase = swaps * pi + sum_t angle(piv_t),
//   Pf = (-1)^swaps prod_t piv_t (sequential, without contraction, as the
//   reference's running product; the sign flips commute exactly).
// The sums are taken across lanes, so that no single lane runs a chain of
// FP64 transcendentals per step.
__device__ void pf_finish_warp(const zc* piv, int npiv, int swaps, int status, int b, double* logpf, double* phase,
                               double* pf, int* st) {
  const int lane = threadIdx.x & 31;
  DD lp{0.0, 0.0}, an{0.0, 0.0};
  if (status == SKEW_OK && (logpf || phase)) {
    for (int t = lane; t < npiv; t += 32) {
      const zc z = piv[t];
      lp = dd_add(lp, log(hypot(z.re, z.im)));
      an = dd_add(an, atan2(z.im, z.re));
    }
    lp = dd_warp_sum(lp);
    an = dd_warp_sum(an);
  }
  if (lane != 0) return;
  double c, sn;
  zc pr;
  if (status == SKEW_OK) {
    // phase mod 2 pi: the angle sum reduced with a two-part 2 pi, and swaps * pi
    // replaced by its parity (cis depends on the phase mod 2 pi only)
    const double k2 = rint(an.hi * (1.0 / TWO_PI_HI));
    double r = fma(-k2, TWO_PI_HI, an.hi);
    r = fma(-k2, TWO_PI_LO, r) + an.lo;
    if (swaps & 1) r = (r + PFZ_PI) + PI_LO;
    sincos(r, &sn, &c);
    pr = zc{1.0, 0.0};
    if (pf) {
      for (int t = 0; t < npiv; t++) {
        const zc z = piv[t];
        const double re = __dsub_rn(__dmul_rn(pr.re, z.re), __dmul_rn(pr.im, z.im));
        const double im = __dadd_rn(__dmul_rn(pr.re, z.im), __dmul_rn(pr.im, z.re));
        pr = zc{re, im};
      }
      if (swaps & 1) pr = zneg(pr);
    }
  } else if (status == SKEW_SINGULAR) {  // (-Inf, 0) and Pf = 0, pfaffian.jl:130, :227
    lp = DD{-INFINITY, 0.0};
    c = sn = 0.0;
    pr = zc{0.0, 0.0};
  } else {
    lp = DD{nan(""), 0.0};
    c = sn = nan("");
    pr = zc{nan(""), nan("")};
  }
  if (logpf) logpf[b] = lp.hi + lp.lo;
  if (phase) {
    phase[2 * b] = c;
    phase[2 * b + 1] = sn;
  }
  if (pf) {
    pf[2 * b] = pr.re;
    pf[2 * b + 1] = pr.im;
  }
  if (st) st[b] = status;
}

// Packed strictly-lower storage: column j holds rows j+1 .. n-1, from pk_col(j).
__device__ __forceinline__ int64_t pk_col(int n, int j) { return (int64_t)j * (2 * n - j - 1) / 2 - j - 1; }
__device__ __forceinline__ int64_t pk(int n, int i, int j) { return pk_col(n, j) + i; }

}  // namespace

// ===========================================================================
// One CTA per matrix
// ===========================================================================
// Shared memory: tau[n], cc[n], piv[n/2 + 1], then (SM) the packed triangle.
// SM (P.smem_matrix) is a template parameter so that the triangle's accesses
// compile to shared-memory instructions rather than generic ones.
template <int NT, bool SM>
__global__ void __launch_bounds__(NT) pfz_cta_kernel(PfzParams P) {
  constexpr int NW = NT / 32;
  extern __shared__ __align__(16) unsigned char pfz_smem[];
  __shared__ zc s_z, s_rz;
  __shared__ int s_kp, s_swaps;
  const int n = P.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  zc* tau = (zc*)pfz_smem;
  zc* cc = tau + n;
  zc* piv = cc + n;
  zc* L = SM ? piv + n / 2 + 1 : P.gws + (int64_t)blockIdx.x * P.slot;

  // Warp 0, after writing column q of the trailing block: the next pivot
  // (kp = first argmax over rows > q), z = A[kp,q], 1/z, recorded as step t.
  auto next_pivot = [&](int q, int t, u64 bv, int bi) {
    warp_argmax(bv, bi);
    __syncwarp();
    if (!sqkey_ok(bv)) {  // squares out of range (or zero, NaN): repeat with hypot
      bv = 0;
      bi = NO_ROW;
      for (int i = q + 1 + lane; i < n; i += 32) {
        const u64 h = abskey(L[pk(n, i, q)]);
        if (key_better(h, i, bv, bi)) {
          bv = h;
          bi = i;
        }
      }
      warp_argmax(bv, bi);
    }
    if (bi <= q || bi >= n) bi = q + 1;  // unreachable: column q has rows below q
    if (lane == 0) {
      const zc z = L[pk(n, bi, q)];
      s_kp = bi;
      s_z = z;
      s_rz = zrcp(z);
      piv[t] = zneg(z);
      s_swaps += (bi != q + 1);
    }
  };

  for (int b = blockIdx.x; b < P.count; b += gridDim.x) {
    const zc* A = P.A + (int64_t)b * P.stride;
    // isskewsymmetric(A): A == -transpose(A) elementwise (skewhermitian.jl:101-110).
    // Even n > 0 checks after the copy below (every entry of A read once, coalesced).
    if (P.check && ((n & 1) || n == 0)) {
      int bad = 0;
      for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += NT) {
        const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
        bad |= !neg_equal(A[i + (int64_t)j * P.lda], A[j + (int64_t)i * P.lda]);
      }
      if (__syncthreads_or(bad)) {
        if (warp == 0) pf_finish_warp(piv, 0, 0, SKEW_NOT_SKEW, b, P.logpf, P.phase, P.pf, P.status);
        continue;
      }
    }
    if (n & 1) {  // pfaffian.jl:97, :195
      if (warp == 0) pf_finish_warp(piv, 0, 0, SKEW_SINGULAR, b, P.logpf, P.phase, P.pf, P.status);
      continue;
    }
    if (n == 0) {
      if (warp == 0) pf_finish_warp(piv, 0, 0, SKEW_OK, b, P.logpf, P.phase, P.pf, P.status);
      continue;
    }
    for (int j = warp; j < n - 1; j += NW) {  // four loads in flight per lane
      const double2* col = (const double2*)(A + (int64_t)j * P.lda);
      zc* dst = L + pk_col(n, j);
      for (int i0 = j + 1; i0 < n; i0 += 128) {
        double2 v[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const int i = i0 + 32 * r + lane;
          if (i < n) v[r] = __ldg(col + i);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const int i = i0 + 32 * r + lane;
          if (i < n) dst[i] = zc{v[r].x, v[r].y};
        }
      }
    }
    if (P.check) {  // the upper triangle and the diagonal of A against the copied lower triangle
      __syncthreads();
      int bad = 0;
      for (int j = warp; j < n; j += NW) {
        const zc* col = A + (int64_t)j * P.lda;
        for (int i = lane; i <= j; i += 32) {
          const zc a = col[i];
          bad |= !neg_equal(a, i == j ? a : L[pk(n, j, i)]);
        }
      }
      if (__syncthreads_or(bad)) {
        if (warp == 0) pf_finish_warp(piv, 0, 0, SKEW_NOT_SKEW, b, P.logpf, P.phase, P.pf, P.status);
        continue;
      }
    }
    if (threadIdx.x == 0) s_swaps = 0;
    __syncthreads();
    if (warp == 0) {  // pivot of step 0 (column 0)
      u64 bv = 0;
      int bi = NO_ROW;
      for (int i = 1 + lane; i < n; i += 32) {
        const u64 v = sqkey(L[pk(n, i, 0)]);
        if (key_better(v, i, bv, bi)) {
          bv = v;
          bi = i;
        }
      }
      next_pivot(0, 0, bv, bi);
    }
    __syncthreads();
    int status = SKEW_OK;
    for (int k = 0; k < n - 1; k += 2) {
      const int p = k + 1;
      // ---- phase T: tau and c from the unswapped entries ----
      const int kp = s_kp;
      if (is_zero_bits(s_z)) {  // pfaffian.jl:127-129, :226-228
        status = SKEW_SINGULAR;
        break;
      }
      const zc rz = s_rz;
      for (int i = p + 1 + threadIdx.x; i < n; i += NT) {
        tau[i] = zmul(L[pk(n, i == kp ? p : i, k)], rz);
        zc c;
        if (i == kp)
          c = zneg(L[pk(n, kp, p)]);
        else if (i < kp)
          c = zneg(L[pk(n, kp, i)]);
        else
          c = L[pk(n, i, kp)];
        cc[i] = c;
      }
      __syncthreads();
      // ---- phase U: the trailing triangle as one list of entries ----
      // Columns a and m-2-a of the m x m trailing block are paired into runs of
      // length m (the middle column alone when m is even), and the runs are
      // numbered one after the other: entry e is run e / m, offset e % m.  Run 0
      // starts with the next pivot column (its m - 1 entries, e < m - 1), which
      // warp 0 updates before the pivot search; the rest goes out in chunks of
      // 64 entries, so that only the last chunk of a step has idle lanes (an
      // FP64 warp instruction costs the FP64 pipe the same with idle lanes).
      const int m = n - p - 1;
      const int q = p + 1;
      auto update = [&](int e) -> zc {
        const int v = e / m, off = e - v * m;
        const int lena = m - 1 - v;
        const int j = off < lena ? q + v : q + m - 2 - v;
        const int i = off < lena ? j + 1 + off : j + 1 + (off - lena);
        zc* dst = L + pk(n, i, j);
        zc x;
        if (i == kp)
          x = zneg(L[pk(n, j, p)]);  // new A[kp,j] = old A[p,j]
        else if (j == kp)
          x = L[pk(n, i, p)];  // new A[i,kp] = old A[i,p]
        else
          x = *dst;
        x = rank2(x, tau[i], cc[j], tau[j], cc[i]);
        *dst = x;
        return x;
      };
      if (m >= 2) {
        const int total = m * (m - 1) / 2;
        if (warp == 0) {
          u64 bv = 0;
          int bi = NO_ROW;
          for (int e = lane; e < m - 1; e += 32) {
            const zc x = update(e);
            const u64 key = sqkey(x);
            if (key_better(key, q + 1 + e, bv, bi)) {
              bv = key;
              bi = q + 1 + e;
            }
          }
          next_pivot(q, (k + 2) / 2, bv, bi);
        }
        // chunks of CH entries, all loads of a chunk issued before its FMAs
        constexpr int R = 2, CH = 32 * R;
        const int w0 = NW >= 4 ? 1 : 0, nw = NW - w0;
        if (warp >= w0) {
          for (int c0 = m - 1 + (warp - w0) * CH; c0 < total; c0 += nw * CH) {
            int ii[R], jj[R];
            zc x[R], ti[R], ci[R], tj[R], cj[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
              const int e = min(c0 + 32 * r + lane, total - 1);  // past the end: a repeat, not stored
              const int v = e / m, off = e - v * m;
              const int lena = m - 1 - v;
              const int j = off < lena ? q + v : q + m - 2 - v;
              const int i = off < lena ? j + 1 + off : j + 1 + (off - lena);
              ii[r] = i;
              jj[r] = j;
              if (i == kp)
                x[r] = zneg(L[pk(n, j, p)]);  // new A[kp,j] = old A[p,j]
              else if (j == kp)
                x[r] = L[pk(n, i, p)];  // new A[i,kp] = old A[i,p]
              else
                x[r] = L[pk(n, i, j)];
              ti[r] = tau[i];
              ci[r] = cc[i];
              tj[r] = tau[j];
              cj[r] = cc[j];
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
              if (c0 + 32 * r + lane < total) L[pk(n, ii[r], jj[r])] = rank2(x[r], ti[r], cj[r], tj[r], ci[r]);
            }
          }
        }
      }
      __syncthreads();
    }
    if (warp == 0) pf_finish_warp(piv, n / 2, s_swaps, status, b, P.logpf, P.phase, P.pf, P.status);
    __syncthreads();  // the next matrix reuses the storage
  }
}

// ===========================================================================
// One matrix over a cooperative grid
// ===========================================================================
namespace {
constexpr int GZ_NT = 512;
constexpr int GZ_NW = GZ_NT / 32;
constexpr int GZ_TC = 16;  // columns per tile (rows per tile: 32, one per lane)
constexpr long long GZ_POLL_LIMIT = 1LL << 24;  // default polls before a grid barrier gives up

__device__ __forceinline__ zc ldz(const zc* p) {
  const double2 v = __ldcg((const double2*)p);
  return zc{v.x, v.y};
}
__device__ __forceinline__ void stz(zc* p, zc x) { __stcg((double2*)p, make_double2(x.re, x.im)); }

// Grid barrier on a monotonic arrival counter: barrier number b ends when the
// counter reaches (b + 1) * gridDim.x, so each CTA makes one atomic and then
// polls with acquire loads (no reset and no second word).  Bounded: false if
// it gave up (error recorded) or another CTA did.
// poll_limit bounds the wait; the CTA skip_cta (>= 0) never arrives, so the others'
// waits run out (a test of the timeout path) while it waits, bounded, for that.
__device__ bool pfz_gsync(unsigned* sync, int* err, long long poll_limit, int skip_cta) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && (int)blockIdx.x == skip_cta) {
    volatile int* verr = err;
    long long it = 0;
    while (!*verr && ++it <= poll_limit) __nanosleep(32);
    s_ok = 0;
  } else if (threadIdx.x == 0) {
    volatile int* verr = err;
    __threadfence();
    const unsigned old = atomicAdd(sync, 1u);
    const unsigned target = (old / gridDim.x + 1) * gridDim.x;
    int ok = 1;
    long long it = 0;
    for (;;) {
      unsigned cur;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(sync) : "memory");
      if ((int)(cur - target) >= 0) break;
      if ((++it & 63) == 0) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (it > poll_limit) {
          atomicExch(err, 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    s_ok = ok && !*verr;
  }
  __syncthreads();
  return s_ok != 0;
}
}  // namespace

__global__ void __launch_bounds__(GZ_NT) pfz_grid_kernel(PfzGridParams P) {
  __shared__ u64 s_v[GZ_NW];
  __shared__ int s_i[GZ_NW];
  __shared__ int s_kp;
  __shared__ zc s_z, s_rz;
  __shared__ zc s_tc[GZ_NW][2 * GZ_TC];  // per warp: tau, c of the tile's columns
  const int n = P.n;
  const int64_t lda = P.lda;
  zc* A = P.A;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warp-major numbering: consecutive tiles go to different SMs, so that every
  // CTA gets a share of the full tiles near the bottom of the triangle
  const int gw = warp * gridDim.x + blockIdx.x, GW = gridDim.x * GZ_NW;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  if (P.notskew && *P.notskew != 0.0) {
    if (blockIdx.x == 0 && warp == 0) pf_finish_warp(P.piv, 0, 0, SKEW_NOT_SKEW, 0, P.logpf, P.phase, P.pf, P.info);
    return;
  }
  if (n & 1) {  // pfaffian.jl:97, :195
    if (blockIdx.x == 0 && warp == 0) pf_finish_warp(P.piv, 0, 0, SKEW_SINGULAR, 0, P.logpf, P.phase, P.pf, P.info);
    return;
  }
#define AZ(i, j) (A + (i) + (int64_t)(j) * lda)
  // argmax partials of column 0, one per 32 rows
  int nparts = (n - 1 + 31) / 32;
  for (int u = gw; u < nparts; u += GW) {
    const int i = 1 + u * 32 + lane;
    u64 bv = 0;
    int bi = NO_ROW;
    if (i < n) {
      bv = abskey(ldz(AZ(i, 0)));
      bi = i;
    }
    warp_argmax(bv, bi);
    if (lane == 0) {
      P.part_v[u] = bv;
      P.part_i[u] = bi;
    }
  }
  int status = SKEW_OK, swaps = 0;
  if (!pfz_gsync(P.sync, P.err, P.poll_limit, P.skip_cta)) return;
  for (int k = 0; k < n - 1; k += 2) {
    const int p = k + 1, q = p + 1, m = n - q;
    // ---- phase T: the pivot (every CTA reduces the partials), tau and c ----
    {
      u64 bv = 0;
      int bi = NO_ROW;
      for (int u = threadIdx.x; u < nparts; u += GZ_NT) {
        const u64 v = __ldcg(P.part_v + u);
        const int i = __ldcg(P.part_i + u);
        if (key_better(v, i, bv, bi)) {
          bv = v;
          bi = i;
        }
      }
      warp_argmax(bv, bi);
      if (lane == 0) {
        s_v[warp] = bv;
        s_i[warp] = bi;
      }
      __syncthreads();
      if (warp == 0) {
        bv = lane < GZ_NW ? s_v[lane] : 0;
        bi = lane < GZ_NW ? s_i[lane] : NO_ROW;
        warp_argmax(bv, bi);
        if (bi <= k || bi >= n) bi = k + 1;  // unreachable: the partials cover rows k+1 .. n-1
        if (lane == 0) {
          const zc z = ldz(AZ(bi, k));
          s_kp = bi;
          s_z = z;
          s_rz = zrcp(z);
        }
      }
      __syncthreads();
    }
    const int kp = s_kp;
    const zc z = s_z;
    if (is_zero_bits(z)) {  // pfaffian.jl:127-129, :226-228
      status = SKEW_SINGULAR;
      break;
    }
    if (lead) {
      P.piv[k / 2] = zneg(z);
      swaps += (kp != p);
    }
    const zc rz = s_rz;
    for (int i = q + blockIdx.x * GZ_NT + threadIdx.x; i < n; i += gridDim.x * GZ_NT) {
      const zc t = zmul(ldz(AZ(i == kp ? p : i, k)), rz);
      zc c;
      if (i == kp)
        c = zneg(ldz(AZ(kp, p)));
      else if (i < kp)
        c = zneg(ldz(AZ(kp, i)));
      else
        c = ldz(AZ(i, kp));
      stz(P.tau + i, t);
      stz(P.cc + i, c);
    }
    if (!pfz_gsync(P.sync, P.err, P.poll_limit, P.skip_cta)) return;
    // ---- phase U: 32 x 16 tiles of the trailing lower triangle ----
    const int nrb = (m + 31) / 32, ncb = (m + GZ_TC - 1) / GZ_TC;
    zc* tcw = s_tc[warp];
    for (int u = gw; u < nrb * ncb; u += GW) {
      const int rb = u / ncb, cb = u - rb * ncb;
      const int r0 = q + rb * 32, c0 = q + cb * GZ_TC;
      const int rlast = min(n - 1, r0 + 31);
      if (c0 >= rlast) continue;  // no entry below the diagonal
      const int ncol = min(GZ_TC, rlast - c0);  // columns c0 .. c0+ncol-1 (j < i needs j < rlast)
      __syncwarp();
      if (lane < ncol)
        tcw[lane] = ldz(P.tau + c0 + lane);
      else if (lane >= 16 && lane - 16 < ncol)
        tcw[GZ_TC + lane - 16] = ldz(P.cc + c0 + lane - 16);
      const int i = r0 + lane;
      const bool row_ok = i < n;
      zc ti = zc{0.0, 0.0}, ci = zc{0.0, 0.0};
      zc x[GZ_TC];
      if (row_ok) {
        ti = ldz(P.tau + i);
        ci = ldz(P.cc + i);
      }
#pragma unroll
      for (int jj = 0; jj < GZ_TC; jj++) {
        const int j = c0 + jj;
        x[jj] = zc{0.0, 0.0};
        if (jj < ncol && row_ok && i > j) {
          if (i == kp)
            x[jj] = zneg(ldz(AZ(j, p)));  // new A[kp,j] = old A[p,j]
          else if (j == kp)
            x[jj] = ldz(AZ(i, p));  // new A[i,kp] = old A[i,p]
          else
            x[jj] = ldz(AZ(i, j));
        }
      }
      __syncwarp();
      u64 bv = 0;
      int bi = NO_ROW;
#pragma unroll
      for (int jj = 0; jj < GZ_TC; jj++) {
        const int j = c0 + jj;
        if (jj < ncol && row_ok && i > j) {
          const zc r = rank2(x[jj], ti, tcw[GZ_TC + jj], tcw[jj], ci);
          stz(AZ(i, j), r);
          if (j == q) {
            bv = abskey(r);
            bi = i;
          }
        }
      }
      if (cb == 0) {
        warp_argmax(bv, bi);
        if (lane == 0) {
          P.part_v[rb] = bv;
          P.part_i[rb] = bi;
        }
      }
    }
    nparts = nrb;
    if (!pfz_gsync(P.sync, P.err, P.poll_limit, P.skip_cta)) return;
  }
#undef AZ
  if (blockIdx.x == 0 && warp == 0) {
    swaps = __shfl_sync(0xffffffffu, swaps, 0);
    __syncwarp();
    pf_finish_warp(P.piv, n / 2, swaps, status, 0, P.logpf, P.phase, P.pf, P.info);
  }
}

// ===========================================================================
// Launchers
// ===========================================================================
size_t pfz_cta_smem(int n, bool smem_matrix) {
  size_t b = (2 * (size_t)n + n / 2 + 1) * sizeof(zc);
  if (smem_matrix) b += (size_t)n * (n - 1) / 2 * sizeof(zc);
  return b;
}

// forced: the tuning key pfz_nt (64/128/256/512 for the shared-memory kernel), or 0
static int pfz_threads(int n, bool smem_matrix, int forced) {
  if (!smem_matrix) return 512;
  if (forced == 64 || forced == 128 || forced == 256 || forced == 512) return forced;
  // measured on GB300 (batches of 1024-4096): 128 threads best at n = 64, 256 at
  // n = 96 (+10 % over 128), 512 at n = 128-160 (+3-5 % over 256)
  if (n <= 48) return 64;
  if (n <= 72) return 128;
  if (n <= 112) return 256;
  return 512;
}

template <int NT, bool SM>
static cudaError_t pfz_launch_t(const PfzParams& P, int grid, size_t smem, cudaStream_t st) {
  static std::atomic<uint64_t> raised{0};
  cudaError_t e = raise_smem_limit_once((const void*)pfz_cta_kernel<NT, SM>, raised);
  if (e != cudaSuccess) return e;
  pfz_cta_kernel<NT, SM><<<grid, NT, smem, st>>>(P);
  return cudaGetLastError();
}

template <int NT, bool SM>
static int pfz_occ_t(size_t smem) {
  static std::atomic<uint64_t> raised{0};
  int occ = 0;
  cudaError_t e = raise_smem_limit_once((const void*)pfz_cta_kernel<NT, SM>, raised);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pfz_cta_kernel<NT, SM>, NT, smem);
  if (e != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return 1;
  }
  return occ;
}

bool pfz_smem_fits(int n) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return pfz_cta_smem(n, true) + 1024 <= (size_t)optin;  // + the kernel's static shared memory
}

int pfz_cta_occupancy(int n, bool smem_matrix, int nt) {
  const size_t smem = pfz_cta_smem(n, smem_matrix);
  if (!smem_matrix) return pfz_occ_t<512, false>(smem);
  switch (pfz_threads(n, true, nt)) {
    case 64: return pfz_occ_t<64, true>(smem);
    case 128: return pfz_occ_t<128, true>(smem);
    case 256: return pfz_occ_t<256, true>(smem);
    default: return pfz_occ_t<512, true>(smem);
  }
}

cudaError_t launch_pfz_cta(const PfzParams& P, int grid, cudaStream_t st) {
  const bool sm = P.smem_matrix != 0;
  const size_t smem = pfz_cta_smem(P.n, sm);
  if (!sm) return pfz_launch_t<512, false>(P, grid, smem, st);
  switch (pfz_threads(P.n, true, P.nt)) {
    case 64: return pfz_launch_t<64, true>(P, grid, smem, st);
    case 128: return pfz_launch_t<128, true>(P, grid, smem, st);
    case 256: return pfz_launch_t<256, true>(P, grid, smem, st);
    default: return pfz_launch_t<512, true>(P, grid, smem, st);
  }
}

__global__ void pfz_check_kernel(const zc* __restrict__ A, int64_t lda, int n, double* flag) {
  const int64_t total = (int64_t)n * n;
  int bad = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    bad |= !neg_equal(A[i + (int64_t)j * lda], A[j + (int64_t)i * lda]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) flag[0] = 1.0;
}

__global__ void pfz_merge_err_kernel(const int* err, int* info, double* logpf, double* phase, double* pf) {
  if (*err) {
    if (info) *info = SKEW_TIMEOUT;
    if (logpf) *logpf = nan("");
    if (phase) phase[0] = phase[1] = nan("");
    if (pf) pf[0] = pf[1] = nan("");
  }
}

size_t pfz_grid_ws_doubles(int n) {
  // tau, cc (n complex each), pivots (n/2 + 1 complex), partials (values, indices),
  // sync words, error flag, check flag
  const size_t parts = (size_t)(n + 31) / 32 + 1;
  return 4 * (size_t)n + 2 * (size_t)(n / 2 + 1) + 2 * parts + 8;
}

cudaError_t launch_pfz_grid(zc* A, int64_t lda, int n, int check, double* logpf, double* phase, double* pf,
                            int* info, double* ws, int sms, const Tuning& T, cudaStream_t st) {
  PfzGridParams P;
  P.poll_limit = T.wait_polls > 0 ? T.wait_polls : GZ_POLL_LIMIT;
  P.skip_cta = T.wait_skip_cta;
  P.A = A;
  P.lda = lda;
  P.n = n;
  P.tau = (zc*)ws;
  P.cc = P.tau + n;
  const size_t parts = (size_t)(n + 31) / 32 + 1;
  P.piv = P.cc + n;
  double* pv = ws + 4 * (size_t)n + 2 * (size_t)(n / 2 + 1);
  P.part_v = (unsigned long long*)pv;
  P.part_i = (int*)(pv + parts);
  double* tailw = pv + 2 * parts;
  P.sync = (unsigned*)tailw;           // 2 words
  P.err = (int*)(tailw + 1);           // 1 word
  double* flag = tailw + 2;            // not-skew flag
  P.notskew = check ? flag : nullptr;
  P.logpf = logpf;
  P.phase = phase;
  P.pf = pf;
  P.info = info;
  cudaError_t e = cudaMemsetAsync(tailw, 0, 3 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  if (check) {
    pfz_check_kernel<<<2 * sms, 256, 0, st>>>(A, lda, n, flag);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pfz_grid_kernel, GZ_NT, 0);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorNotSupported;
  // fewer CTAs for smaller matrices: the two grid barriers per step cost more
  // with more CTAs, and the trailing block holds less work
  int grid = std::min(sms, std::max(16, n / 8));
  if (T.pfz_ctas > 0) grid = std::max(1, std::min(sms * occ, T.pfz_ctas));
  void* args[] = {&P};
  e = cudaLaunchCooperativeKernel((const void*)pfz_grid_kernel, dim3(grid), dim3(GZ_NT), args, 0, st);
  if (e != cudaSuccess) return e;
  pfz_merge_err_kernel<<<1, 1, 0, st>>>(P.err, info, logpf, phase, pf);
  return cudaGetLastError();
}

}  // namespace skew
