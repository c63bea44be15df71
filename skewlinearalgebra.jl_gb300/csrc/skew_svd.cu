// Singular values and vectors from the eigenpairs (eigen.jl:110-144, tridiag.jl:526-555),
// the way the reference forms them:
//   svdvals:  |imag(eigenvalues)| sorted descending;
//   svd:      the eigenvalues' imaginary parts lambda stably sorted by |lambda| descending
//             (sortperm(vals; by = abs, rev = true)), U = the eigenvectors in that order,
//             S = |lambda|, V = -i U with the columns of negative lambda negated, so that
//             A = U diag(S) V^H.
// For ComplexF64 the reference takes svd(Hermitian(i A)), which LinearAlgebra forms from
// eigen(Hermitian(i A)) by the same sort and sign rule; with i A = W diag(-lambda) W^H
// this is the same U, S, V in terms of the skew-Hermitian eigenpairs (the LAPACK
// ascending order of -lambda is the descending order of lambda used here).
//
// svd_rank_kernel: a stable rank sort (rank of i = #{|v_j| > |v_i|} + #{j < i : |v_j| == |v_i|})
// on integer keys, shared-memory tiles of the batch's values; O(n^2) comparisons on the
// integer pipe, far below the eigen solve it follows.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_complex.cuh"
#include "skew_internal.h"

namespace skew {

namespace {
typedef unsigned long long u64;
constexpr int RS_NT = 256;

// |v| as an ordered integer key; every NaN above +Inf (Julia's isless order, reversed).
__device__ __forceinline__ u64 abs_key(double v) {
  const u64 b = (u64)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
  return b > 0x7FF0000000000000ull ? 0x7FF8000000000000ull : b;
}
}  // namespace

// perm[b][k] = index of the k-th value of problem b by |v| descending (stable);
// S[b][k] = |v| of it; sgn[b][k] = -1 where that value is negative, else 1.
__global__ void __launch_bounds__(RS_NT) svd_rank_kernel(const double* __restrict__ vals, int n, int64_t vstride,
                                                         int* __restrict__ perm, double* __restrict__ S,
                                                         int64_t sstride, double* __restrict__ sgn) {
  __shared__ u64 tile[RS_NT];
  const int b = blockIdx.y;
  const double* v = vals + (int64_t)b * vstride;
  const int i = blockIdx.x * RS_NT + threadIdx.x;
  const double vi = i < n ? v[i] : 0.0;
  const u64 ki = abs_key(vi);
  int rank = 0;
  for (int t0 = 0; t0 < n; t0 += RS_NT) {
    __syncthreads();
    if (t0 + threadIdx.x < n) tile[threadIdx.x] = abs_key(v[t0 + threadIdx.x]);
    __syncthreads();
    const int cnt = min(RS_NT, n - t0);
    for (int t = 0; t < cnt; t++) {
      const u64 kj = tile[t];
      const int j = t0 + t;
      rank += (kj > ki) || (kj == ki && j < i);
    }
  }
  if (i < n) {
    if (perm) perm[(int64_t)b * n + rank] = i;
    if (S) S[(int64_t)b * sstride + rank] = fabs(vi);
    if (sgn) sgn[(int64_t)b * n + rank] = vi < 0.0 ? -1.0 : 1.0;
  }
}

// U[:, k] = W[:, perm[k]] (real and imaginary planes, leading dimension ld).
__global__ void svd_gather_d_kernel(const double* __restrict__ Wr, const double* __restrict__ Wi, int n, int64_t ld,
                                    const int* __restrict__ perm, double* __restrict__ Ur, double* __restrict__ Ui) {
  const int k = blockIdx.y;
  const int64_t src = (int64_t)perm[k] * ld, dst = (int64_t)k * ld;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    Ur[dst + r] = Wr[src + r];
    Ui[dst + r] = Wi[src + r];
  }
}

// V[:, k] = -i sgn[k] U[:, k]:  (Vr, Vi) = sgn (Ui, -Ur).
__global__ void svd_vmake_d_kernel(const double* __restrict__ Ur, const double* __restrict__ Ui, int n, int64_t ld,
                                   const double* __restrict__ sgn, double* __restrict__ Vr, double* __restrict__ Vi) {
  const int k = blockIdx.y;
  const double s = sgn[k];
  const int64_t o = (int64_t)k * ld;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    Vr[o + r] = s * Ui[o + r];
    Vi[o + r] = -s * Ur[o + r];
  }
}

// Complex interleaved forms of the two kernels above.
__global__ void svd_gather_z_kernel(const zc* __restrict__ W, int n, int64_t ld, const int* __restrict__ perm,
                                    zc* __restrict__ U) {
  const int k = blockIdx.y;
  const int64_t src = (int64_t)perm[k] * ld, dst = (int64_t)k * ld;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) U[dst + r] = W[src + r];
}

__global__ void svd_vmake_z_kernel(const zc* __restrict__ U, int n, int64_t ld, const double* __restrict__ sgn,
                                   zc* __restrict__ V) {
  const int k = blockIdx.y;
  const double s = sgn[k];
  const int64_t o = (int64_t)k * ld;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const zc u = U[o + r];
    V[o + r] = zc{s * u.im, -s * u.re};
  }
}

cudaError_t launch_svd_rank(const double* vals, int n, int64_t vstride, int batch, int* perm, double* S,
                            int64_t sstride, double* sgn, cudaStream_t st) {
  if (n <= 0 || batch <= 0) return cudaSuccess;
  svd_rank_kernel<<<dim3((n + RS_NT - 1) / RS_NT, batch), RS_NT, 0, st>>>(vals, n, vstride, perm, S, sstride, sgn);
  return cudaGetLastError();
}

static dim3 col_grid(int n) { return dim3((unsigned)std::min(8, (n + 255) / 256), (unsigned)n); }

cudaError_t launch_svd_vectors_d(const double* Wr, const double* Wi, int n, int64_t ld, const int* perm,
                                 const double* sgn, double* Ur, double* Ui, double* Vr, double* Vi, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  svd_gather_d_kernel<<<col_grid(n), 256, 0, st>>>(Wr, Wi, n, ld, perm, Ur, Ui);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  svd_vmake_d_kernel<<<col_grid(n), 256, 0, st>>>(Ur, Ui, n, ld, sgn, Vr, Vi);
  return cudaGetLastError();
}

cudaError_t launch_svd_vectors_z(const double* W, int n, int64_t ld, const int* perm, const double* sgn, double* U,
                                 double* V, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  svd_gather_z_kernel<<<col_grid(n), 256, 0, st>>>((const zc*)W, n, ld, perm, (zc*)U);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  svd_vmake_z_kernel<<<col_grid(n), 256, 0, st>>>((const zc*)U, n, ld, sgn, (zc*)V);
  return cudaGetLastError();
}

}  // namespace skew
