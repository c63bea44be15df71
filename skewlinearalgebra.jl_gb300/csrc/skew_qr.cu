// Skew-symmetric tridiagonal eigenvalues.
//
// Batched path: the implicit-QR iteration of skewtrieigvals!
// (skeweigen.jl:105-156) with its exact tolerances, shift, deflation order and
// stagnation rule, one matrix per thread.  The iteration is a serial chain of
// Givens rotations; since the FP64 pipe charges a warp instruction the same
// whether one lane or 32 are active, 32 matrices share each warp (matrices are
// sorted by size, so warp-mates run similar trip counts).  A matrix whose
// shifts stagnate is handed to a second kernel that solves the reference's
// fallback, the eigenvalues of SymTridiagonal(0, ev) (skeweigen.jl:134-137,
// 463-468), with one CTA per matrix and one eigenvalue per thread.
//
// Single large matrix: bisection with Sturm counts on the equivalent
// zero-diagonal symmetric tridiagonal SymTridiagonal(0, ev), one eigenvalue per
// thread across the whole GPU.  Values come out sorted descending, the order the
// reference itself returns from its fallback (skeweigen.jl:134-137, 463-468).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_internal.h"
#include "skew_twisted.cuh"

namespace skew {

// getgivens (skeweigen.jl:3-7): nm = hypot(a, b); (1, 0) if nm == 0, else
// (a/nm, b/nm).  The QR steps below round every product and sum separately (no
// fused multiply-add), as the reference's Float64 code does: the iteration's
// deflation decisions depend on the last bits of ev, so matching the reference's
// rounding keeps the GPU on the reference's trajectory.
__device__ __forceinline__ void givens(double a, double b, double& c, double& s) {
  const double nm = hypot(a, b);
  if (nm == 0.0) {
    c = 1.0;
    s = 0.0;
    return;
  }
  c = __ddiv_rn(a, nm);
  s = __ddiv_rn(b, nm);
}

// reducetozero (skeweigen.jl:11-47) for odd sizes; n = N-1 (even), G unused for values.
__device__ void reducetozero_dev(double* ev, int n) {
  if (n == 0) return;
  double bulge = 0.0, c, s;
  if (n > 2) {
    const double a = ev[n - 3], b = ev[n - 2], g = ev[n - 1];
    givens(-b, g, c, s);
    ev[n - 3] = __dmul_rn(ev[n - 3], c);
    ev[n - 2] = __dsub_rn(__dmul_rn(c, b), __dmul_rn(s, g));
    ev[n - 1] = 0.0;
    bulge = __dmul_rn(neg(s), a);
    for (int i = n - 2; i >= 4; i -= 2) {
      const double a2 = ev[i - 3], b2 = ev[i - 2];
      givens(-b2, bulge, c, s);
      ev[i - 3] = __dmul_rn(ev[i - 3], c);
      ev[i - 2] = __dsub_rn(__dmul_rn(c, b2), __dmul_rn(s, bulge));
      bulge = __dmul_rn(neg(s), a2);
    }
  }
  const double b = (n == 2 ? ev[1] : bulge);
  const double a = ev[0];
  givens(-a, b, c, s);
  ev[0] = __dsub_rn(__dmul_rn(c, a), __dmul_rn(s, b));
  if (n == 2) ev[1] = __dadd_rn(__dmul_rn(s, a), __dmul_rn(b, c));
}

// implicitstep_novec (skeweigen.jl:73-103); n = active size - 1, start 1-based.
// The chain is serial: step i needs the rotation of step i-1.  The three entries
// a step reads besides ev[i+1] are the ones the previous step just wrote, so they
// are carried in registers instead of going through memory, and ev[i+1], which no
// step of this sweep has touched yet, is loaded one step ahead.  Every store of
// the reference's step is still made, in the same order, so ev holds the same
// values at every step and after an early return.
__device__ int implicitstep_dev(double* ev, int n, int start) {
  double bulge = 0.0;
  const double shift = __dmul_rn(ev[n - 1], ev[n - 1]);
  const double tol = 2.220446049250313e-16;  // eps(Float64)
  double a = 0.0;              // ev[i-2] (zero at i == start, as the reference's alpha)
  double b = ev[start - 1];    // ev[i-1]
  double g = ev[start];        // ev[i]
  double z = (start < n - 1) ? ev[start + 1] : 0.0;  // ev[i+1], untouched this sweep
  for (int i = start; i <= n - 1; i++) {
    const double zn = (i + 2 <= n - 1) ? ev[i + 2] : 0.0;  // next step's ev[i+1]
    double c, s;
    if (i > start) {
      givens(a, bulge, c, s);
    } else {
      const double x1 = __dadd_rn(__dsub_rn(neg(__dmul_rn(a, a)), __dmul_rn(b, b)), shift);
      const double x2 = __dadd_rn(neg(__dmul_rn(a, bulge)), __dmul_rn(b, g));
      givens(x1, x2, c, s);
    }
    if (i > 1) ev[i - 2] = __dadd_rn(__dmul_rn(c, a), __dmul_rn(s, bulge));
    const double nb = __dsub_rn(__dmul_rn(c, b), __dmul_rn(s, g));
    const double ng = __dadd_rn(__dmul_rn(s, b), __dmul_rn(c, g));
    ev[i - 1] = nb;
    ev[i] = ng;
    if (i < n - 1) {
      const double nz = __dmul_rn(z, c);
      ev[i + 1] = nz;
      bulge = __dmul_rn(s, z);
      if (fabs(bulge) < tol && fabs(nb) < tol) return i + 1;
      a = nb;
      b = ng;
      g = nz;
      z = zn;
    }
  }
  return start;
}

// Number of eigenvalues of SymTridiagonal(0, e) (size n) smaller than x: the
// count of negative pivots of the LDL^T factorisation of (T - x I), a pivot
// smaller than pivmin in magnitude being replaced by -pivmin before it is
// counted and used.
__device__ int sturm_count(const double* e, int n, double x, double pivmin) {
  double q = -x;
  if (fabs(q) <= pivmin) q = -pivmin;
  int c = (q < 0.0);
  for (int i = 1; i < n; i++) {
    const double ei = e[i - 1];
    q = -x - (ei * ei) / q;
    if (fabs(q) <= pivmin) q = -pivmin;
    c += (q < 0.0);
  }
  return c;
}

// skewtrieigvals! (skeweigen.jl:105-156).  ev (N-1 entries) is destroyed;
// vals[N] receives the imaginary parts in the reference's order.  On stagnation
// the active size n is returned in *fb_n (vals[0..n) and ev[0..n-1) are then
// left to the fallback kernel).
__device__ int skewtrieigvals_dev(double* ev, int N, double* vals, int* fb_n, int max_iter_cap) {
  int n = N;
  for (int i = 0; i < N; i++) vals[i] = 0.0;
  if (n & 1) {
    n -= 1;
    reducetozero_dev(ev, n);
  }
  const double tol = 10.0 * 2.220446049250313e-16;
  const int max_iter = max_iter_cap > 0 ? max_iter_cap : 30 * n;
  int iter = 0, count_static = 0, start = 1;
  double mem = 1.0;
  while (n > 2 && iter < max_iter) {
    start = implicitstep_dev(ev, n - 1, start);
    while (n > 2 && fabs(ev[n - 2]) <= tol) {
      vals[n - 1] = 0.0;
      n -= 1;
    }
    while (n > 2 && fabs(ev[n - 3]) <= tol * fabs(ev[n - 2])) {
      vals[n - 2] = ev[n - 2];
      vals[n - 1] = neg(ev[n - 2]);
      n -= 2;
    }
    if (start > n - 2) start = 1;
    if (n > 1 && fabs(mem - ev[n - 2]) < 0.0001 * fabs(ev[n - 2])) {
      count_static += 1;
      if (count_static > 4) {  // stagnation: symmetric tridiagonal fallback (:134-137)
        *fb_n = n;
        return SKEW_FALLBACK_USED;
      }
    } else {
      count_static = 0;
    }
    mem = (n > 1 ? ev[n - 2] : 0.0);
    iter += 1;
  }
  if (n == 2) {
    vals[0] = ev[0];
    vals[1] = neg(ev[0]);
    return SKEW_OK;
  }
  if (n <= 1) {
    if (n == 1) vals[0] = 0.0;
    return SKEW_OK;
  }
  return SKEW_NO_CONVERGENCE;
}

__global__ void batch_trieig_kernel(TrieigParams P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P.count) return;
  const int b = P.order[t];
  const int N = P.n[b];
  double* ev = P.evwork + P.ev_off[b];
  if (P.evwork != P.ev_all)
    for (int i = 0; i + 1 < N; i++) ev[i] = P.ev_all[P.ev_off[b] + i];
  int fb_n = 0;
  const int st = (N >= 1) ? skewtrieigvals_dev(ev, N, P.vals[b], &fb_n, P.max_iter) : SKEW_OK;
  if (st == SKEW_FALLBACK_USED) {
    const unsigned k = atomicAdd(P.fallback, 1u);
    P.fallback[2 + k] = (unsigned)b;
    P.fallback[2 + P.count + k] = (unsigned)fb_n;
  }
  if (P.status) P.status[b] = st;
}

constexpr int FB_NT = 256;

// The reference's fallback for matrices whose shifts stagnated: values[1:n] =
// -eigvals(SymTridiagonal(0, ev[1:n-1])) (skeweigen.jl:134-137, 463-468), i.e.
// the eigenvalues in descending order.  One CTA per matrix (taken from a work
// counter), one eigenvalue per thread by Sturm-count bisection.
__global__ void __launch_bounds__(FB_NT) batch_fallback_kernel(TrieigParams P) {
  __shared__ int s_item;
  __shared__ double red[2][FB_NT / 32];
  const unsigned nfb = *(volatile unsigned*)P.fallback;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(P.fallback + 1, 1u);
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= (int)nfb) break;
    const int b = (int)P.fallback[2 + item];
    const int n = (int)P.fallback[2 + P.count + item];
    const double* e = P.evwork + P.ev_off[b];
    double* vals = P.vals[b];
    double bound = 0.0, emax2 = 0.0;
    for (int i = threadIdx.x; i < n; i += FB_NT) {
      const double l = (i > 0 ? fabs(e[i - 1]) : 0.0), r = (i + 1 < n ? fabs(e[i]) : 0.0);
      bound = fmax(bound, l + r);
      if (i + 1 < n) emax2 = fmax(emax2, e[i] * e[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      bound = fmax(bound, __shfl_xor_sync(0xffffffffu, bound, o));
      emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = bound;
      red[1][threadIdx.x >> 5] = emax2;
    }
    __syncthreads();
    bound = 0.0;
    emax2 = 0.0;
    for (int w = 0; w < FB_NT / 32; w++) {
      bound = fmax(bound, red[0][w]);
      emax2 = fmax(emax2, red[1][w]);
    }
    __syncthreads();
    const double pivmin = 2.2250738585072014e-308 * fmax(1.0, emax2);
    bound = bound * (1.0 + 1e-14) + 1e-300;
    for (int k = threadIdx.x; k < n; k += FB_NT) {  // k-th largest = (n-1-k)-th smallest
      double lo = -bound, hi = bound;
      for (int it = 0; it < 120 && hi - lo > 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300; it++) {
        const double mid = 0.5 * (lo + hi);
        if (sturm_count(e, n, mid, pivmin) <= n - 1 - k)
          lo = mid;
        else
          hi = mid;
      }
      vals[k] = 0.5 * (lo + hi);
    }
  }
}

cudaError_t launch_batch_trieig(const TrieigParams& P, cudaStream_t st) {
  if (P.count <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(P.fallback, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  const int bs = 32;
  batch_trieig_kernel<<<(P.count + bs - 1) / bs, bs, 0, st>>>(P);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  batch_fallback_kernel<<<P.grid > 0 ? P.grid : 1, FB_NT, 0, st>>>(P);
  return cudaGetLastError();
}

// Gershgorin bound and pivmin in one small kernel so the host never waits.
__global__ void bisect_prep_kernel(const double* __restrict__ e, int n, double* __restrict__ out2) {
  __shared__ double red[2][32];
  double bound = 0.0, emax2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double l = (i > 0 ? fabs(e[i - 1]) : 0.0), r = (i + 1 < n ? fabs(e[i]) : 0.0);
    bound = fmax(bound, l + r);
    if (i + 1 < n) emax2 = fmax(emax2, e[i] * e[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    bound = fmax(bound, __shfl_xor_sync(0xffffffffu, bound, o));
    emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = bound;
    red[1][threadIdx.x >> 5] = emax2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0, m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      b = fmax(b, red[0][w]);
      m = fmax(m, red[1][w]);
    }
    out2[0] = b * (1.0 + 1e-14) + 1e-300;
    out2[1] = 2.2250738585072014e-308 * fmax(1.0, m);
  }
}

// The positive eigenvalues of SymTridiagonal(0, e): the k-th largest (k < n/2) by
// a group of p lanes (multisection to relative precision: the zero-diagonal Sturm
// count resolves the tiny singular values of the bidiagonal coupling, and their
// twisted eigenvectors need them accurate); vals[k] and vals[n-1-k] = -vals[k]
// written together; odd n: vals[n/2] = 0.
__global__ void bisect_kernel_dev(const double* __restrict__ e, int n, const double* __restrict__ bp,
                                  double* __restrict__ vals, int p) {
  const int h = n / 2;
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / p;  // eigenvalue index of the lane's group
  const int gl = (threadIdx.x & 31) % p;
  if ((n & 1) && gid == 0 && gl == 0 && blockIdx.x == 0) vals[h] = 0.0;
  const double bound = bp[0], pivmin = bp[1];
  const bool active = gid < h;
  const double x = group_multisect(0.0, bound, n - 1 - (active ? gid : 0), 4.0 * pivmin, p, active,
                                   [&](double y) { return sturm_count(e, n, y, pivmin); });
  if (active && gl == 0) {
    vals[gid] = x;
    vals[n - 1 - gid] = neg(x);
  }
}

cudaError_t launch_tridiag_bisect(const double* ev, int n, double* vals_im, double* scratch2, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  bisect_prep_kernel<<<1, 256, 0, st>>>(ev, n, scratch2);
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int h = n / 2;
  const int p = multisect_lanes(h, sms);
  const long long threads = ((long long)std::max(h, 1) * p + 31) / 32 * 32;
  const int bs = 128;
  bisect_kernel_dev<<<(unsigned)((threads + bs - 1) / bs), bs, 0, st>>>(ev, n, scratch2, vals_im, p);
  return cudaGetLastError();
}

// The same for G problems of one size n (subdiagonals e_g, n apart): per problem the
// bounds {bound, pivmin} into bp_g (8 apart) and the values (descending, exact
// +-pairs) into vals_g (n apart) and into vals_out[idx[mb]].
__global__ void bisect_prep_batch_kernel(const double* __restrict__ e_g, int n, double* __restrict__ bp_g) {
  __shared__ double red[2][32];
  const double* e = e_g + (size_t)blockIdx.x * n;
  double bound = 0.0, emax2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double l = (i > 0 ? fabs(e[i - 1]) : 0.0), r = (i + 1 < n ? fabs(e[i]) : 0.0);
    bound = fmax(bound, l + r);
    if (i + 1 < n) emax2 = fmax(emax2, e[i] * e[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    bound = fmax(bound, __shfl_xor_sync(0xffffffffu, bound, o));
    emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = bound;
    red[1][threadIdx.x >> 5] = emax2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0, m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      b = fmax(b, red[0][w]);
      m = fmax(m, red[1][w]);
    }
    double* bp = bp_g + (size_t)blockIdx.x * 8;
    bp[0] = b * (1.0 + 1e-14) + 1e-300;
    bp[1] = 2.2250738585072014e-308 * fmax(1.0, m);
  }
}

__global__ void bisect_batch_kernel(const double* __restrict__ e_g, int n, const double* __restrict__ bp_g,
                                    double* __restrict__ vals_g, double* const* __restrict__ vals_out,
                                    const int32_t* __restrict__ idx, int p) {
  const int mb = blockIdx.y;
  const double* e = e_g + (size_t)mb * n;
  const double* bp = bp_g + (size_t)mb * 8;
  double* vals = vals_g + (size_t)mb * n;
  double* out = vals_out[idx[mb]];
  const int h = n / 2;
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / p;
  const int gl = (threadIdx.x & 31) % p;
  if ((n & 1) && gid == 0 && gl == 0 && blockIdx.x == 0) {
    vals[h] = 0.0;
    out[h] = 0.0;
  }
  const double bound = bp[0], pivmin = bp[1];
  const bool active = gid < h;
  const double x = group_multisect(0.0, bound, n - 1 - (active ? gid : 0), 4.0 * pivmin, p, active,
                                   [&](double y) { return sturm_count(e, n, y, pivmin); });
  if (active && gl == 0) {
    vals[gid] = x;
    vals[n - 1 - gid] = neg(x);
    out[gid] = x;
    out[n - 1 - gid] = neg(x);
  }
}

cudaError_t launch_tridiag_bisect_batch(const double* e_g, int n, int G, double* bp_g, double* vals_g,
                                        double* const* vals_out, const int32_t* idx, cudaStream_t st) {
  if (n <= 0 || G <= 0) return cudaSuccess;
  bisect_prep_batch_kernel<<<G, 256, 0, st>>>(e_g, n, bp_g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int h = n / 2;
  // lanes per eigenvalue: the whole batch shares the machine
  const int p = multisect_lanes(std::max(1, h * G), sms);
  const long long threads = ((long long)std::max(h, 1) * p + 31) / 32 * 32;
  const int bs = 128;
  bisect_batch_kernel<<<dim3((unsigned)((threads + bs - 1) / bs), G), bs, 0, st>>>(e_g, n, bp_g, vals_g, vals_out,
                                                                                   idx, p);
  return cudaGetLastError();
}

// Selected eigenvalues of a symmetric tridiagonal (diagonal dg or zero, off-diagonal
// e): the ascending eigenvalues lambda_{i0 .. i0+m-1} with
//   irange (il, iu, 1-based):  i0 = il - 1, m = iu - il + 1;
//   interval [-vh, -vl):       i0 = #lambda < -vh, m = #lambda < -vl - i0;
// written negated (out[k] = -lambda_{i0+k}, i.e. descending), as the reference's
// eigvals!(A, irange) / eigvals!(A, vl, vh) negate the eigenvalues of
// SymTridiagonal(0, ev) (eigen.jl:57-73) or of Hermitian(iA) (eigen.jl:29-41).
// bnd: sym_bound ? {bound, pivmin} (spectrum in [-bound, bound]) : {lo, pivmin, hi}.
// *count = m.  Groups of p lanes, one eigenvalue each; groups beyond m idle.
__global__ void select_kernel(const double* __restrict__ e, const double* __restrict__ dg, int n,
                              const double* __restrict__ bnd, int sym_bound, int by_index, int il, int iu, double vl,
                              double vh, double* __restrict__ out, int* __restrict__ count, int p) {
  const double lo = sym_bound ? neg(bnd[0]) : bnd[0];
  const double hi = sym_bound ? bnd[0] : bnd[2];
  const double pivmin = bnd[1];
  int i0, m;
  if (by_index) {
    i0 = il - 1;
    m = iu - il + 1;
  } else {
    i0 = block_sturm(e, dg, 0, n, neg(vh), pivmin);
    m = block_sturm(e, dg, 0, n, neg(vl), pivmin) - i0;
  }
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) / p;
  const int gl = (threadIdx.x & 31) % p;
  if (blockIdx.x == 0 && threadIdx.x == 0 && count) *count = m;
  const bool active = k < m;
  double x = group_multisect(lo, hi, active ? i0 + k : 0, 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)), p,
                             active, [&](double y) { return block_sturm(e, dg, 0, n, y, pivmin); });
  if (n == 1) x = dg ? dg[0] : 0.0;  // the 1 x 1 eigenvalue itself (the reference returns A[1,1])
  if (active && gl == 0) out[k] = neg(x);
}

cudaError_t launch_select(const double* e, const double* dg, int n, const double* bnd, int sym_bound, int by_index,
                          int il, int iu, double vl, double vh, double* out, int* count, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int m = by_index ? std::max(iu - il + 1, 1) : n;  // eigenvalues to find (at most)
  const int p = multisect_lanes(m, sms);
  const long long threads = ((long long)m * p + 31) / 32 * 32;
  select_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(e, dg, n, bnd, sym_bound, by_index, il, iu, vl, vh,
                                                                   out, count, p);
  return cudaGetLastError();
}

// Gershgorin bound and pivmin of SymTridiagonal(0, e) into bnd[0..1] (no eigenvalue search)
cudaError_t launch_tridiag_bounds(const double* ev, int n, double* bnd, cudaStream_t st) {
  bisect_prep_kernel<<<1, 256, 0, st>>>(ev, n, bnd);
  return cudaGetLastError();
}

}  // namespace skew
