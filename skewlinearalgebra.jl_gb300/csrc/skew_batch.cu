// Batched and small-matrix kernels: one CTA per skew matrix.
//
// Working copy.  A CTA works on a full-storage copy W of its matrix (both
// triangles kept, W[j,i] = -W[i,j]).  In the batched path W lives in dynamic
// shared memory when the size bucket fits, otherwise in a per-CTA slot of a
// global workspace; in the single-matrix path W is the caller's matrix itself
// (in place, as hessenberg!/logabspfaffian! are).  The code is the same for all
// three (generic addressing).  Leading dimensions of private copies are odd so
// that transposed stores do not conflict in shared-memory banks.
//
// Reduction step k (reflector acting on indices k+1..n-1, m = n-k-1):
//   1. ss = |W[k+2:n, k]|^2                        (block reduction)
//   2. beta, tau, scale as householder! does (hessenberg.jl:26-44); every
//      thread computes them redundantly, which costs the FP64 pipe no more
//      than one thread would and saves a broadcast barrier
//   3. v = [1; W[k+2:n,k]*scale], stored back into column k (the reflector,
//      v[1] = 1 on the subdiagonal as the reference stores it)
//   4. p = tau * W[k+1:n, k+1:n] v                 (full-row products)
//   5. W[i,j] += v_i p_j - p_i v_j for k < j < i, mirrored to W[j,i]
// Step 5 is the two-sided application H W H = W + v p^T - p v^T, exact for a
// skew W because v^T W v = 0.  Steps 4 and 5 cost m^2 FMAs each, the minimum for
// this reduction (4/3 n^3 flops in total); the reference's unblocked tail
// (skewhess!, hessenberg.jl:70-90) spends 4 m^2 on the same step.  The elements
// of step 5 are dealt out from the flattened lower triangle so every FP64
// instruction carries 32 useful lanes.
//
// Gradient (the spec adjoint; the reference has no rrule):
// d log|Pf(A)|/dA = 1/2 A^{-T} = -1/2 A^{-1} = Q (-1/2 T^{-1}) Q^T with
// Q = H_0 H_1 ... H_{n-3}.  Starting from M = -1/2 T^{-1}, the reflectors are
// applied innermost first with the same two-sided update, now over all n rows
// (2 n m FMAs per reflector, 2 n^3 flops in total).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"
#include "skew_internal.h"

namespace skew {

constexpr int BT = 128;  // threads per CTA
constexpr int NW = BT / WARP;

// Shared vectors (nmax entries each) carved from dynamic shared memory.
struct Vecs {
  double* v;      // reflector
  double* p;      // tau * W v
  double* ypart;  // NW partial row products, stride nmax
  double* ev;     // subdiagonal of T
  double* tau;    // reflector scalars
  double* red;    // NW doubles of scratch for block reductions
  int nmax;
};

__host__ __device__ constexpr int vec_doubles(int nmax) { return (4 + NW) * nmax + 2 * NW; }

__device__ __forceinline__ Vecs carve(double* base, int nmax) {
  Vecs s;
  s.v = base;
  s.p = base + nmax;
  s.ypart = base + 2 * nmax;
  s.ev = base + (2 + NW) * nmax;
  s.tau = base + (3 + NW) * nmax;
  s.red = base + (4 + NW) * nmax;
  s.nmax = nmax;
  return s;
}

// Copy A (lda) into W (ldw).  With check, verifies A == -A^T exactly
// (isskewhermitian, skewhermitian.jl:84-94).  Returns false if not skew.
__device__ bool copy_in(const double* __restrict__ A, int64_t lda, double* W, int64_t ldw, int n, bool check) {
  int bad = 0;
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += BT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    const double a = A[i + (int64_t)j * lda];
    if (W != A) W[i + (int64_t)j * ldw] = a;
    if (check) bad |= !(a == -A[j + (int64_t)i * lda]);
  }
  return __syncthreads_or(bad) == 0;
}

// Block-wide max of |x| (for the scaled-norm fallback).
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

// p_i = tau * sum_{j in [c0, n)} W[i,j] v_j for rows i in [r0, n).  Each warp
// takes one of NW column chunks; partial sums meet in shared memory.  Ends with
// p visible to the whole block.
__device__ void rowprod(const double* W, int64_t ldw, int n, int r0, int c0, const Vecs& s, double tau) {
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  const int m = n - c0;
  const int chunk = (m + NW - 1) / NW;
  const int cb = c0 + w * chunk;
  const int ce = min(n, cb + chunk);
  double* yp = s.ypart + (size_t)w * s.nmax;
  for (int i0 = r0; i0 < n; i0 += WARP) {
    const int i = i0 + l;
    if (i < n) {
      const double* row = W + i;
      double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
      int j = cb;
      for (; j + 3 < ce; j += 4) {
        a0 = fma(row[(int64_t)j * ldw], s.v[j], a0);
        a1 = fma(row[(int64_t)(j + 1) * ldw], s.v[j + 1], a1);
        a2 = fma(row[(int64_t)(j + 2) * ldw], s.v[j + 2], a2);
        a3 = fma(row[(int64_t)(j + 3) * ldw], s.v[j + 3], a3);
      }
      for (; j < ce; j++) a0 = fma(row[(int64_t)j * ldw], s.v[j], a0);
      yp[i] = (a0 + a1) + (a2 + a3);
    }
  }
  __syncthreads();
  for (int i = r0 + (int)threadIdx.x; i < n; i += BT) {
    double y = s.ypart[i];
#pragma unroll
    for (int q = 1; q < NW; q++) y += s.ypart[(size_t)q * s.nmax + i];
    s.p[i] = tau * y;
  }
  __syncthreads();
}

// Two-sided update W += v p^T - p v^T on the region {i in [o, n), j < i, j >= j0}
// (lower triangle only, mirrored to the upper).  v_j = 0 for j < o, so the
// rectangle j in [j0, o) needs one FMA per element and the triangle two.
// Elements are dealt out column by column from the flattened region.
__device__ void skew_update(double* W, int64_t ldw, int n, int o, int j0, const Vecs& s) {
  // column j holds rows max(j+1, o) .. n-1
  auto collen = [&](int j) { return n - max(j + 1, o); };
  int j = j0, r = threadIdx.x;
  while (j < n - 1 && r >= collen(j)) {
    r -= collen(j);
    j++;
  }
  while (j < n - 1) {
    const int i = max(j + 1, o) + r;
    double* pij = W + i + (int64_t)j * ldw;
    double a = *pij;
    const double vi = s.v[i];
    const double pj = s.p[j];
    if (j >= o) a = fma(neg(s.p[i]), s.v[j], a);
    a = fma(vi, pj, a);
    *pij = a;
    W[j + (int64_t)i * ldw] = neg(a);
    r += BT;
    while (j < n - 1 && r >= collen(j)) {
      r -= collen(j);
      j++;
    }
  }
}

// Householder reduction of the n x n skew matrix in W to tridiagonal form.
// Fills s.ev[0..n-2], s.tau[0..n-2]; W keeps the reflectors in its lower part.
__device__ void reduce(double* W, int64_t ldw, int n, const Vecs& s) {
  for (int k = 0; k + 2 < n; k++) {
    // (1) sum of squares below the subdiagonal
    double part = 0.0;
    for (int r = k + 2 + (int)threadIdx.x; r < n; r += BT) {
      const double x = W[r + (int64_t)k * ldw];
      part = fma(x, x, part);
    }
    const double ss = block_sum<NW>(part, s.red);
    const double alpha = W[(k + 1) + (int64_t)k * ldw];
    double xn = -1.0;
    if (ss_needs_scaling(ss)) {  // block-uniform rare path: norm with scaling
      double mx = 0.0;
      for (int r = k + 2 + (int)threadIdx.x; r < n; r += BT) mx = fmax(mx, fabs(W[r + (int64_t)k * ldw]));
      mx = block_maxabs(mx, s.red);
      double q = 0.0;
      for (int r = k + 2 + (int)threadIdx.x; r < n; r += BT) {
        const double x = W[r + (int64_t)k * ldw] / mx;
        q = fma(x, x, q);
      }
      q = block_sum<NW>(q, s.red);
      xn = mx * sqrt(q);
    }
    // (2) reflector, computed redundantly by every thread
    const Reflector R = make_reflector(alpha, ss, xn);
    if (threadIdx.x == 0) {
      s.ev[k] = R.beta;
      s.tau[k] = R.tau;
    }
    // (3) v into shared memory and back into column k
    for (int r = k + 1 + (int)threadIdx.x; r < n; r += BT) {
      double vr;
      if (R.tau == 0.0)
        vr = 0.0;  // zero column: x .= 0 (hessenberg.jl:40)
      else
        vr = (r == k + 1) ? 1.0 : W[r + (int64_t)k * ldw] * R.scale;
      s.v[r] = vr;
      W[r + (int64_t)k * ldw] = vr;
    }
    __syncthreads();
    if (R.tau == 0.0) continue;
    // (4) p = tau * W22 v
    rowprod(W, ldw, n, k + 1, k + 1, s, R.tau);
    // (5) W22 += v p^T - p v^T
    skew_update(W, ldw, n, k + 1, k + 1, s);
    __syncthreads();
  }
  if (n >= 2 && threadIdx.x == 0) {  // final real 1x1 step: tau = 0, beta = x (hessenberg.jl:27-29)
    s.ev[n - 2] = W[(n - 1) + (int64_t)(n - 2) * ldw];
    s.tau[n - 2] = 0.0;
  }
  __syncthreads();
}

// log|Pf| and sign from ev and tau (pfaffian.jl:167-179):
//   log|Pf| = sum_{odd i} log|ev_i|, sign = prod sign(-ev_i) * (-1)^{#tau != 0}.
__device__ void pfaffian_from_tridiag(int n, const Vecs& s, double* logpf, double* sign) {
  const int h = n / 2;
  double lp = 0.0;
  int npos = 0, nzero = 0, ntau = 0;
  for (int a = threadIdx.x; a < h; a += BT) {
    const double e = s.ev[2 * a];
    lp += log(fabs(e));
    npos += (e > 0.0);
    nzero += (e == 0.0);
  }
  for (int a = threadIdx.x; a < n - 1; a += BT) ntau += (s.tau[a] != 0.0);
  // parity of (#ev_odd > 0) + (#tau != 0), summed over threads on the integer pipe
  const int tflip = __syncthreads_count((npos + ntau) & 1);
  const int tzero = __syncthreads_count(nzero > 0);
  const double total = block_sum<NW>(lp, s.red);
  if (threadIdx.x == 0) {
    *logpf = total;
    *sign = tzero ? 0.0 : ((tflip & 1) ? -1.0 : 1.0);
  }
}

// M = -1/2 T^{-1} (even n, all odd-position ev nonzero), full storage in G.
// With O = even 0-based indices and E = odd ones, T = [[0, B], [-B^T, 0]] where
// B is lower bidiagonal (diag d_a = -ev[2a], sub s_a = ev[2a-1]), and
// T^{-1} = [[0, -B^{-T}], [B^{-1}, 0]]:  T^{-1}[2a+1, 2b] = (B^{-1})_{ab}
//   = (1/d_b) prod_{c=b+1..a} (-s_c/d_c)   for a >= b, zero otherwise.
__device__ void tinv_init(double* G, int64_t ldg, int n, const Vecs& s) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += BT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    G[i + (int64_t)j * ldg] = 0.0;
  }
  const int h = n / 2;
  // ratios -s_c/d_c = ev[2c-1]/ev[2c] into s.p[c], 1 <= c < h
  for (int c = 1 + (int)threadIdx.x; c < h; c += BT) s.p[c] = s.ev[2 * c - 1] / s.ev[2 * c];
  __syncthreads();
  for (int b = threadIdx.x; b < h; b += BT) {
    double x = 0.5 / s.ev[2 * b];  // -1/2 * (1/d_b) = -1/2 * (-1/ev[2b])
    for (int a = b; a < h; a++) {
      G[(2 * a + 1) + (int64_t)(2 * b) * ldg] = x;
      G[(2 * b) + (int64_t)(2 * a + 1) * ldg] = neg(x);
      if (a + 1 < h) x *= s.p[a + 1];
    }
  }
  __syncthreads();
}

// G = Q M Q^T with M already in G, reflectors k = n-3..0 taken from W.
__device__ void backapply(double* G, int64_t ldg, const double* W, int64_t ldw, int n, const Vecs& s) {
  for (int k = n - 3; k >= 0; k--) {
    const double tau = s.tau[k];
    if (tau == 0.0) continue;
    for (int r = k + 1 + (int)threadIdx.x; r < n; r += BT) s.v[r] = W[r + (int64_t)k * ldw];
    __syncthreads();
    rowprod(G, ldg, n, 0, k + 1, s, tau);
    skew_update(G, ldg, n, k + 1, 0, s);
    __syncthreads();
  }
}

__device__ void fill(double* G, int64_t ldg, int n, double val) {
  const int64_t total = (int64_t)n * n;
  for (int64_t e = threadIdx.x; e < total; e += BT) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    G[i + (int64_t)j * ldg] = val;
  }
}

// One matrix, start to finish.  W may alias A (in-place single-matrix path).
struct Job {
  const double* A;
  int64_t lda;
  int n;
  double* W;
  int64_t ldw;
  double* G;  // gradient output or null
  int64_t ldg;
  double* logpf;
  double* sign;
  double* ev_out;   // optional (n-1)
  double* tau_out;  // optional (n-1)
  int* status;
  bool check;
  bool want_pf;
};

__device__ void run_job(const Job& J, const Vecs& s) {
  const int n = J.n;
  const bool ok = copy_in(J.A, J.lda, J.W, J.ldw, n, J.check);
  if (!ok) {
    if (threadIdx.x == 0) {
      if (J.logpf) *J.logpf = nan("");
      if (J.sign) *J.sign = nan("");
      if (J.status) *J.status = SKEW_NOT_SKEW;
    }
    if (J.G) fill(J.G, J.ldg, n, nan(""));
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
    if (J.G) fill(J.G, J.ldg, n, nan(""));
    __syncthreads();
    if (!J.ev_out) return;
  }
  reduce(J.W, J.ldw, n, s);
  if (J.ev_out || J.tau_out)
    for (int a = threadIdx.x; a < n - 1; a += BT) {
      if (J.ev_out) J.ev_out[a] = s.ev[a];
      if (J.tau_out) J.tau_out[a] = s.tau[a];
    }
  if (!J.want_pf || odd) {
    if (threadIdx.x == 0 && J.status && !J.want_pf) *J.status = SKEW_OK;
    __syncthreads();
    return;
  }
  __shared__ double s_lp, s_sg;
  pfaffian_from_tridiag(n, s, &s_lp, &s_sg);
  __syncthreads();
  const double lp = s_lp, sg = s_sg;
  if (threadIdx.x == 0) {
    *J.logpf = lp;
    *J.sign = sg;
    if (J.status) *J.status = (sg == 0.0) ? SKEW_SINGULAR : SKEW_OK;
  }
  if (J.G) {
    if (sg == 0.0) {
      fill(J.G, J.ldg, n, nan(""));
    } else {
      tinv_init(J.G, J.ldg, n, s);
      backapply(J.G, J.ldg, J.W, J.ldw, n, s);
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// Persistent batched kernel over order[begin:end) (matrices sorted largest
// first); CTAs take the next matrix from an atomic counter.
__global__ void __launch_bounds__(BT) batch_pf_kernel(BatchParams P) {
  extern __shared__ __align__(16) double dsm[];
  const Vecs s = carve(dsm, P.nmax);
  double* smat = dsm + vec_doubles(P.nmax);
  __shared__ int s_next;
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(P.counter, 1u) + P.begin;
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
    J.ldw = n | 1;
    J.W = P.smem_matrix ? smat : P.gws + (size_t)blockIdx.x * P.gws_slot;
    J.G = P.grad ? P.grad[b] : nullptr;
    J.ldg = n;
    J.logpf = P.logpf + b;
    J.sign = P.sign + b;
    J.ev_out = P.ev_out ? P.ev_out + P.ev_off[b] : nullptr;
    J.tau_out = nullptr;
    J.status = P.status + b;
    J.check = P.check != 0;
    J.want_pf = true;
    run_job(J, s);
  }
}

// Batched reduction to tridiagonal form only (eigvals front end): ev_out[b].
__global__ void __launch_bounds__(BT) batch_tridiag_kernel(BatchParams P) {
  extern __shared__ __align__(16) double dsm[];
  const Vecs s = carve(dsm, P.nmax);
  double* smat = dsm + vec_doubles(P.nmax);
  __shared__ int s_next;
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(P.counter, 1u) + P.begin;
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
    J.ldw = n | 1;
    J.W = P.smem_matrix ? smat : P.gws + (size_t)blockIdx.x * P.gws_slot;
    J.G = nullptr;
    J.ldg = n;
    J.logpf = nullptr;
    J.sign = nullptr;
    J.ev_out = P.ev_out + P.ev_off[b];
    J.tau_out = nullptr;
    J.status = nullptr;
    J.check = P.check != 0;
    J.want_pf = false;
    run_job(J, s);
  }
}

// Single matrix, in place (W = A), one CTA.
__global__ void __launch_bounds__(BT) single_kernel(SingleParams P) {
  extern __shared__ __align__(16) double dsm[];
  const Vecs s = carve(dsm, P.n > 0 ? P.n : 1);
  Job J;
  J.A = P.A;
  J.lda = P.lda;
  J.n = P.n;
  J.W = P.A;
  J.ldw = P.lda;
  J.G = P.G;
  J.ldg = P.ldg;
  J.logpf = P.logpf;
  J.sign = P.sign;
  J.ev_out = P.ev;
  J.tau_out = P.tau;
  J.status = P.info;
  J.check = P.check != 0;
  J.want_pf = P.want_pf != 0;
  run_job(J, s);
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
size_t batch_smem_bytes(int nmax, bool smem_matrix) {
  size_t b = sizeof(double) * (size_t)vec_doubles(nmax);
  if (smem_matrix) b += sizeof(double) * (size_t)nmax * (size_t)(nmax | 1);
  return b;
}

cudaError_t launch_batch_pf(const BatchParams& P, int grid, cudaStream_t st, bool tridiag_only) {
  const size_t smem = batch_smem_bytes(P.nmax, P.smem_matrix != 0);
  cudaError_t e;
  if (tridiag_only) {
    e = cudaFuncSetAttribute(batch_tridiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    batch_tridiag_kernel<<<grid, BT, smem, st>>>(P);
  } else {
    e = cudaFuncSetAttribute(batch_pf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    batch_pf_kernel<<<grid, BT, smem, st>>>(P);
  }
  return cudaGetLastError();
}

cudaError_t launch_single(const SingleParams& P, cudaStream_t st) {
  const size_t smem = batch_smem_bytes(P.n > 0 ? P.n : 1, false);
  cudaError_t e = cudaFuncSetAttribute(single_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  single_kernel<<<1, BT, smem, st>>>(P);
  return cudaGetLastError();
}

int batch_threads() { return BT; }

int batch_occupancy(size_t smem) {
  int occ = 0;
  if (cudaFuncSetAttribute(batch_pf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_pf_kernel, BT, smem) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return 1;
  }
  return occ;
}

}  // namespace skew
