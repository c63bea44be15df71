// ComplexF64 skew-Hermitian Householder tridiagonalisation (the complex branches
// of hessenberg.jl: householder! :26-44 with complex alpha, skewhess! :70-90,
// skewlatrd! :92-131 with the alpha correction of :123-126, the trailing update
// of skewblockedhess! :158-166).
//
// For column c with x = A[c+1:n, c] (alpha = x[1]):
//   beta = -sign(Re alpha) hypot(|alpha|, |x[2:]|) (real), tau = 1 - alpha/beta,
//   v = [1; x[2:] / (alpha - beta)]; zero column -> tau = 0, v = 0, beta = 0.
//   The last step (a 1 x 1 column) is a phase that makes the last subdiagonal real.
// With p = A22 v, W = tau p and a = tau (W^H v) / 2, w = W + a v, the update
//   A22 += v w^H - w v^H
// equals H^H A22 H for H = I - tau v v^H (the term a v restores the v v^H part
// that v^H A22 v, purely imaginary, contributes).  The lower triangle is updated,
// the upper one mirrored as -conj, and the diagonal only receives the purely
// imaginary part 2i Im(v_j conj(w_j)), as the blocked reference's
// Omega - Omega^H does.  On exit A holds the reflectors below the subdiagonal
// (v[1] = 1 on the subdiagonal), ev the real subdiagonal, dvim = imag(diag(A)).
//
// Two forms: zhess_cta_kernel, one CTA per matrix (batched, or the tail of a
// large reduction); and per-column multi-CTA kernels for large n (reflector,
// matvec partials over (row block, column chunk) tiles, combination, and the
// rank-2 update on 32 x 32 tiles of the lower triangle with a transposed mirror).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_complex.cuh"
#include "skew_funcs.cuh"
#include "skew_internal.h"

namespace skew {

constexpr int ZNT = 256;
constexpr int ZNW = ZNT / 32;

// ---------------------------------------------------------------------------
// reflector from (alpha, amax, ss) with |x[2:]| = amax * sqrt(ss)
// ---------------------------------------------------------------------------
struct ZRefl {
  zc tau, scale;
  double beta;
};

__device__ ZRefl zrefl(zc alpha, double xnorm) {
  ZRefl R;
  if (xnorm == 0.0 && alpha.re == 0.0 && alpha.im == 0.0) {
    R.tau = zc{0.0, 0.0};
    R.scale = zc{0.0, 0.0};
    R.beta = 0.0;
    return R;
  }
  const double h = hypot(hypot(alpha.re, alpha.im), xnorm);
  const double beta = (alpha.re > 0.0) ? neg(h) : h;
  R.beta = beta;
  R.tau = zc{1.0 - alpha.re / beta, neg(alpha.im / beta)};
  R.scale = zinv(zc{alpha.re - beta, alpha.im});
  return R;
}

// ---------------------------------------------------------------------------
// one CTA per matrix
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_max(double x, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = x;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < ZNW; i++) s = fmax(s, red[i]);
  __syncthreads();
  return s;
}

__global__ void __launch_bounds__(ZNT) zhess_cta_kernel(ZHessParams P) {
  extern __shared__ __align__(16) double zsm[];  // v (nmax complex) | w (nmax complex)
  zc* vs = reinterpret_cast<zc*>(zsm);
  zc* ws = vs + P.nmax;
  __shared__ double red[ZNW];
  __shared__ int s_next;
  __shared__ ZRefl s_R;
  for (;;) {
    if (threadIdx.x == 0) s_next = P.counter ? (int)atomicAdd(P.counter, 1u) : (int)blockIdx.x;
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= P.count) break;
    const int b = P.order ? P.order[t] : t;
    const bool one = (P.W == nullptr);  // matrices given directly: W1 + b * stride
    const int n = one ? P.n1 : P.n[b];
    const int64_t ld = one ? P.ld1 : n;
    const int64_t off = one ? (int64_t)b * P.n1 : P.off[b];
    zc* W = one ? reinterpret_cast<zc*>(P.W1) + (int64_t)b * P.stride : reinterpret_cast<zc*>(P.W[b]);
    zc* tau = reinterpret_cast<zc*>(P.tau) + off;
    double* ev = P.ev + off;
    for (int c = 0; c + 1 < n; c++) {
      const int m = n - c - 1;
      zc* x = W + (c + 1) + (int64_t)c * ld;
      double amax = 0.0;
      for (int i = 1 + threadIdx.x; i < m; i += ZNT) amax = fmax(amax, fmax(fabs(x[i].re), fabs(x[i].im)));
      amax = block_max(amax, red);
      double ss = 0.0;
      if (amax > 0.0) {
        const double inv = 1.0 / amax;
        for (int i = 1 + threadIdx.x; i < m; i += ZNT) {
          const double a = x[i].re * inv, bb = x[i].im * inv;
          ss = fma(a, a, fma(bb, bb, ss));
        }
      }
      ss = block_sum<ZNW>(ss, red);
      if (threadIdx.x == 0) {
        s_R = zrefl(x[0], amax * sqrt(ss));
        ev[c] = s_R.beta;
        tau[c] = s_R.tau;
      }
      __syncthreads();
      const ZRefl R = s_R;
      const bool zero = (R.tau.re == 0.0 && R.tau.im == 0.0);
      for (int i = threadIdx.x; i < m; i += ZNT) {
        const zc v = zero ? zc{0.0, 0.0} : (i == 0 ? zc{1.0, 0.0} : zmul(x[i], R.scale));
        x[i] = v;
        vs[i] = v;
      }
      __syncthreads();
      if (zero) continue;  // H = I: nothing to update
      zc* A22 = W + (c + 1) + (int64_t)(c + 1) * ld;
      // p = A22 v  (rows by threads, coalesced down each column; eight loads in
      // flight per thread: the working copy of a batch lives in L2)
      for (int i = threadIdx.x; i < m; i += ZNT) {
        zc a0{0.0, 0.0}, a1{0.0, 0.0}, a2{0.0, 0.0}, a3{0.0, 0.0};
        const zc* row = A22 + i;
        int j = 0;
        for (; j + 7 < m; j += 8) {
          zc x[8];
#pragma unroll
          for (int u = 0; u < 8; u++) x[u] = row[(int64_t)(j + u) * ld];
          a0 = zfma(x[0], vs[j], a0);
          a1 = zfma(x[1], vs[j + 1], a1);
          a2 = zfma(x[2], vs[j + 2], a2);
          a3 = zfma(x[3], vs[j + 3], a3);
          a0 = zfma(x[4], vs[j + 4], a0);
          a1 = zfma(x[5], vs[j + 5], a1);
          a2 = zfma(x[6], vs[j + 6], a2);
          a3 = zfma(x[7], vs[j + 7], a3);
        }
        for (; j < m; j++) a0 = zfma(row[(int64_t)j * ld], vs[j], a0);
        ws[i] = zmul(R.tau, zadd(zadd(a0, a1), zadd(a2, a3)));  // W = tau p
      }
      __syncthreads();
      // a = tau (W^H v) / 2
      double dr = 0.0, di = 0.0;
      for (int i = threadIdx.x; i < m; i += ZNT) {
        const zc d = zcmul(ws[i], vs[i]);  // conj(W_i) v_i
        dr += d.re;
        di += d.im;
      }
      dr = block_sum<ZNW>(dr, red);
      di = block_sum<ZNW>(di, red);
      const zc a = zmul(R.tau, zc{0.5 * dr, 0.5 * di});
      for (int i = threadIdx.x; i < m; i += ZNT) ws[i] = zfma(a, vs[i], ws[i]);
      __syncthreads();
      // A22 += v w^H - w v^H on the lower triangle (diagonal included), mirrored.
      // The triangle is walked column by column as one list of m (m + 1) / 2 entries
      // (no division per entry); four entries per thread and iteration, loads first.
      {
        int j = 0, r = threadIdx.x;  // entry (j + r, j): column j has m - j entries
        while (j < m && r >= m - j) {
          r -= m - j;
          j++;
        }
        while (j < m) {
          int jj[4], ii[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            jj[u] = j;
            ii[u] = j + r;
            if (j < m) {
              r += ZNT;
              while (j < m && r >= m - j) {
                r -= m - j;
                j++;
              }
            }
          }
          zc a[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (jj[u] < m) a[u] = A22[ii[u] + (int64_t)jj[u] * ld];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            if (jj[u] >= m) continue;
            const int i = ii[u], jc = jj[u];
            const zc vi = vs[i], wi = ws[i];
            if (i == jc) {
              a[u].im += 2.0 * (vi.im * wi.re - vi.re * wi.im);  // 2 Im(v conj(w))
              A22[i + (int64_t)i * ld] = a[u];
            } else {
              const zc vj = vs[jc], wj = ws[jc];
              const zc uu = zsub(zadd(a[u], zmulc(vi, wj)), zmulc(wi, vj));  // + v_i conj(w_j) - w_i conj(v_j)
              A22[i + (int64_t)jc * ld] = uu;
              A22[jc + (int64_t)i * ld] = zc{neg(uu.re), uu.im};  // -conj(u)
            }
          }
        }
      }
      __syncthreads();
    }
    if (P.dvim) {
      double* dv = P.dvim + off;
      for (int k = threadIdx.x; k < n; k += ZNT) dv[k] = W[k + (int64_t)k * ld].im;
    }
    __syncthreads();
    if (!P.counter) break;
  }
}

size_t zhess_cta_smem_bytes(int nmax) { return sizeof(double) * 4 * (size_t)(nmax > 0 ? nmax : 1); }

cudaError_t launch_zhess_cta(const ZHessParams& P, int grid, cudaStream_t st) {
  static std::atomic<uint64_t> raised{0};
  cudaError_t e = raise_smem_limit_once((const void*)zhess_cta_kernel, raised);
  if (e != cudaSuccess) return e;
  zhess_cta_kernel<<<grid, ZNT, zhess_cta_smem_bytes(P.nmax), st>>>(P);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// multi-CTA per-column reduction of one large matrix
// ---------------------------------------------------------------------------
constexpr int ZR_NT = 1024;  // reflector / combine CTA
constexpr int ZMV_ROWS = 256, ZMV_CH = 256;
constexpr int ZU_T = 32;

struct ZColWs {
  zc* v;       // m
  zc* w;       // m
  zc* part;    // nchunk x n
  ZRefl* R;    // 1
};

__global__ void __launch_bounds__(ZR_NT) zcol_refl_kernel(zc* A, int64_t lda, int n, int c, zc* tau, double* ev,
                                                          ZColWs ws) {
  __shared__ double red[ZR_NT / 32];
  __shared__ ZRefl s_R;
  const int m = n - c - 1;
  zc* x = A + (c + 1) + (int64_t)c * lda;
  double amax = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += ZR_NT) amax = fmax(amax, fmax(fabs(x[i].re), fabs(x[i].im)));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = amax;
  __syncthreads();
  amax = 0.0;
  for (int i = 0; i < ZR_NT / 32; i++) amax = fmax(amax, red[i]);
  __syncthreads();
  double ss = 0.0;
  if (amax > 0.0) {
    const double inv = 1.0 / amax;
    for (int i = 1 + threadIdx.x; i < m; i += ZR_NT) {
      const double a = x[i].re * inv, bb = x[i].im * inv;
      ss = fma(a, a, fma(bb, bb, ss));
    }
  }
  ss = block_sum<ZR_NT / 32>(ss, red);
  if (threadIdx.x == 0) {
    s_R = zrefl(x[0], amax * sqrt(ss));
    ev[c] = s_R.beta;
    tau[c] = s_R.tau;
    *ws.R = s_R;
  }
  __syncthreads();
  const ZRefl R = s_R;
  const bool zero = (R.tau.re == 0.0 && R.tau.im == 0.0);
  for (int i = threadIdx.x; i < m; i += ZR_NT) {
    const zc v = zero ? zc{0.0, 0.0} : (i == 0 ? zc{1.0, 0.0} : zmul(x[i], R.scale));
    x[i] = v;
    ws.v[i] = v;
  }
}

// partial p over a (row block, column chunk) tile: part[chunk][i] = sum_j A22[i,j] v_j
__global__ void __launch_bounds__(ZMV_ROWS) zcol_matvec_kernel(const zc* __restrict__ A, int64_t lda, int n, int c,
                                                               ZColWs ws) {
  __shared__ zc sv[ZMV_CH];
  const int m = n - c - 1;
  const int i = blockIdx.x * ZMV_ROWS + threadIdx.x;
  const int j0 = blockIdx.y * ZMV_CH, j1 = min(j0 + ZMV_CH, m);
  for (int j = j0 + threadIdx.x; j < j1; j += ZMV_ROWS) sv[j - j0] = ws.v[j];
  __syncthreads();
  if (i >= m) return;
  const zc* A22 = A + (c + 1) + (int64_t)(c + 1) * lda;
  zc a0{0.0, 0.0}, a1{0.0, 0.0}, a2{0.0, 0.0}, a3{0.0, 0.0};
  int j = j0;
  for (; j + 3 < j1; j += 4) {
    a0 = zfma(A22[i + (int64_t)j * lda], sv[j - j0], a0);
    a1 = zfma(A22[i + (int64_t)(j + 1) * lda], sv[j + 1 - j0], a1);
    a2 = zfma(A22[i + (int64_t)(j + 2) * lda], sv[j + 2 - j0], a2);
    a3 = zfma(A22[i + (int64_t)(j + 3) * lda], sv[j + 3 - j0], a3);
  }
  for (; j < j1; j++) a0 = zfma(A22[i + (int64_t)j * lda], sv[j - j0], a0);
  ws.part[(int64_t)blockIdx.y * n + i] = zadd(zadd(a0, a1), zadd(a2, a3));
}

// p = sum of partials (fixed order), W = tau p, a = tau (W^H v)/2, w = W + a v
__global__ void __launch_bounds__(ZR_NT) zcol_combine_kernel(int n, int c, int nchunk, ZColWs ws) {
  __shared__ double red[ZR_NT / 32];
  const int m = n - c - 1;
  const ZRefl R = *ws.R;
  double dr = 0.0, di = 0.0;
  for (int i = threadIdx.x; i < m; i += ZR_NT) {
    zc p{0.0, 0.0};
    for (int k = 0; k < nchunk; k++) p = zadd(p, ws.part[(int64_t)k * n + i]);
    const zc W = zmul(R.tau, p);
    ws.w[i] = W;
    const zc d = zcmul(W, ws.v[i]);
    dr += d.re;
    di += d.im;
  }
  dr = block_sum<ZR_NT / 32>(dr, red);
  di = block_sum<ZR_NT / 32>(di, red);
  const zc a = zmul(R.tau, zc{0.5 * dr, 0.5 * di});
  for (int i = threadIdx.x; i < m; i += ZR_NT) ws.w[i] = zfma(a, ws.v[i], ws.w[i]);
}

// A22 += v w^H - w v^H on lower 32 x 32 tiles (ti >= tj), upper tile mirrored
__global__ void __launch_bounds__(ZU_T * 8) zcol_update_kernel(zc* A, int64_t lda, int n, int c, ZColWs ws) {
  __shared__ zc tile[ZU_T][ZU_T + 1];
  __shared__ zc svi[ZU_T], swi[ZU_T], svj[ZU_T], swj[ZU_T];
  const int m = n - c - 1;
  // linear block index -> (ti, tj), tj <= ti
  const long long q = blockIdx.x;
  int ti = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
  while ((long long)ti * (ti + 1) / 2 > q) ti--;
  while ((long long)(ti + 1) * (ti + 2) / 2 <= q) ti++;
  const int tj = (int)(q - (long long)ti * (ti + 1) / 2);
  const int i0 = ti * ZU_T, j0 = tj * ZU_T;
  zc* A22 = A + (c + 1) + (int64_t)(c + 1) * lda;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  if (threadIdx.x < ZU_T) {
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.x;
    svi[threadIdx.x] = (i < m) ? ws.v[i] : zc{0.0, 0.0};
    swi[threadIdx.x] = (i < m) ? ws.w[i] : zc{0.0, 0.0};
    svj[threadIdx.x] = (j < m) ? ws.v[j] : zc{0.0, 0.0};
    swj[threadIdx.x] = (j < m) ? ws.w[j] : zc{0.0, 0.0};
  }
  __syncthreads();
  for (int jj = ty; jj < ZU_T; jj += 8) {
    const int i = i0 + tx, j = j0 + jj;
    zc u{0.0, 0.0};
    if (i < m && j < m && i >= j) {
      zc* p = A22 + i + (int64_t)j * lda;
      const zc vi = svi[tx], wi = swi[tx], vj = svj[jj], wj = swj[jj];
      if (i == j) {
        u = *p;
        u.im += 2.0 * (vi.im * wi.re - vi.re * wi.im);
      } else {
        u = zsub(zadd(*p, zmulc(vi, wj)), zmulc(wi, vj));
      }
      *p = u;
    }
    tile[jj][tx] = u;
  }
  if (ti == tj) {
    __syncthreads();
    // diagonal tile: mirror the strictly lower part into the upper part
    for (int jj = ty; jj < ZU_T; jj += 8) {
      const int i = i0 + jj, j = j0 + tx;  // element (i, j) of the upper part: row i < column j
      if (i < m && j < m && i < j) A22[i + (int64_t)j * lda] = zc{neg(tile[jj][tx].re), tile[jj][tx].im};
    }
    return;
  }
  __syncthreads();
  // off-diagonal tile: A22[j, i] = -conj(A22[i, j]) (rows j0.., columns i0..), coalesced along j
  for (int ii = ty; ii < ZU_T; ii += 8) {
    const int j = j0 + tx, i = i0 + ii;
    if (i < m && j < m) A22[j + (int64_t)i * lda] = zc{neg(tile[tx][ii].re), tile[tx][ii].im};
  }
}

__global__ void zdiag_im_kernel(const zc* __restrict__ A, int64_t lda, int n, double* dvim) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dvim[k] = A[k + (int64_t)k * lda].im;
}

cudaError_t launch_zdiag_im(const double* A, int64_t lda, int n, double* dvim, cudaStream_t st) {
  if (!dvim || n <= 0) return cudaSuccess;
  zdiag_im_kernel<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const zc*>(A), lda, n, dvim);
  return cudaGetLastError();
}

constexpr int ZTAIL = 96;  // trailing columns left to the one-CTA kernel

size_t zhess_large_ws_doubles(int n) {
  const int nchunk = (n + ZMV_CH - 1) / ZMV_CH;
  return (2 * (2 * (size_t)n) + 2 * (size_t)nchunk * n + 8 + 31) & ~(size_t)31;
}

cudaError_t zhess_large(double* Ad, int64_t lda, int n, double* taud, double* ev, double* dvim, double* wsd,
                        cudaStream_t st) {
  zc* A = reinterpret_cast<zc*>(Ad);
  zc* tau = reinterpret_cast<zc*>(taud);
  ZColWs ws;
  ws.v = reinterpret_cast<zc*>(wsd);
  ws.w = ws.v + n;
  ws.part = ws.w + n;
  const int nchunk_max = (n + ZMV_CH - 1) / ZMV_CH;
  ws.R = reinterpret_cast<ZRefl*>(ws.part + (size_t)nchunk_max * n);
  cudaError_t e;
  const int cend = n - 1 - ZTAIL;  // columns [0, cend) here, the rest by the one-CTA kernel
  for (int c = 0; c < cend; c++) {
    const int m = n - c - 1;
    zcol_refl_kernel<<<1, ZR_NT, 0, st>>>(A, lda, n, c, tau, ev, ws);
    const int nrb = (m + ZMV_ROWS - 1) / ZMV_ROWS, nch = (m + ZMV_CH - 1) / ZMV_CH;
    zcol_matvec_kernel<<<dim3(nrb, nch), ZMV_ROWS, 0, st>>>(A, lda, n, c, ws);
    zcol_combine_kernel<<<1, ZR_NT, 0, st>>>(n, c, nch, ws);
    const long long nt = (m + ZU_T - 1) / ZU_T;
    zcol_update_kernel<<<(unsigned)(nt * (nt + 1) / 2), ZU_T * 8, 0, st>>>(A, lda, n, c, ws);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  // tail: the trailing (n - c0) x (n - c0) block with the one-CTA kernel (in place, ld = lda)
  const int c0 = cend > 0 ? cend : 0;
  ZHessParams P;
  P.W = nullptr;
  P.W1 = reinterpret_cast<double*>(A + c0 + (int64_t)c0 * lda);
  P.n1 = n - c0;
  P.ld1 = lda;
  P.stride = 0;
  P.n = nullptr;
  P.off = nullptr;
  P.order = nullptr;
  P.count = 1;
  P.nmax = n - c0;
  P.counter = nullptr;
  P.tau = reinterpret_cast<double*>(tau + c0);
  P.ev = ev + c0;
  P.dvim = nullptr;
  e = launch_zhess_cta(P, 1, st);
  if (e != cudaSuccess) return e;
  zdiag_im_kernel<<<(n + 255) / 256, 256, 0, st>>>(A, lda, n, dvim);
  return cudaGetLastError();
}


// ===========================================================================
// Complex eigenproblem.  The reference solves eigen(Hermitian(i A)) by LAPACK
// (eigen.jl:101-106; eigvals :18-27: values -mu, mu ascending, so the imaginary
// parts come out descending).  Here: A = Q T Q^H from the reduction above, then
// i T = D S D^H with S real symmetric tridiagonal (diagonal -dvim, off-diagonal
// |ev|) and D = diag(d), d_1 = 1, d_{k+1} = d_k i sign(ev_k) (the phase scaling
// of to_symtridiagonal, tridiag.jl:558-583); S = Y diag(mu) Y^T by bisection and
// twisted-factorisation eigenvectors; the eigenvectors of A are Q D Y.
// ===========================================================================

// S's diagonal and off-diagonal, the phases, Gershgorin bound and pivmin:
// bp[0] = lower bound, bp[1] = pivmin, bp[2] = upper bound.
__global__ void __launch_bounds__(1024) zprep_kernel(const double* __restrict__ ev, const double* __restrict__ dvim,
                                                    int n, double* __restrict__ dg, double* __restrict__ off,
                                                    zc* __restrict__ ph, double* __restrict__ bp) {
  const size_t mb = blockIdx.x;  // problem of a batch: arrays n (bp: 8) apart
  ev += mb * n;
  dvim += mb * n;
  dg += mb * n;
  off += mb * n;
  ph += mb * n;
  bp += mb * 8;
  __shared__ double red[3][32];
  double lo = INFINITY, hi = -INFINITY, e2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = neg(dvim[i]);
    const double l = (i > 0) ? fabs(ev[i - 1]) : 0.0, r = (i + 1 < n) ? fabs(ev[i]) : 0.0;
    dg[i] = d;
    if (i + 1 < n) {
      off[i] = r;
      e2 = fmax(e2, r * r);
    }
    lo = fmin(lo, d - l - r);
    hi = fmax(hi, d + l + r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    e2 = fmax(e2, __shfl_xor_sync(0xffffffffu, e2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = lo;
    red[1][threadIdx.x >> 5] = hi;
    red[2][threadIdx.x >> 5] = e2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      lo = fmin(lo, red[0][w]);
      hi = fmax(hi, red[1][w]);
      e2 = fmax(e2, red[2][w]);
    }
    const double span = fmax(fabs(lo), fabs(hi));
    bp[0] = lo - 1e-14 * span - 1e-300;
    bp[1] = 2.2250738585072014e-308 * fmax(1.0, e2);
    bp[2] = hi + 1e-14 * span + 1e-300;
    // phases: d_{k+1} = d_k * (i sign(ev_k)), i^k times the sign product
    int quarter = 0;  // d_k = i^quarter
    ph[0] = zc{1.0, 0.0};
    for (int k = 0; k + 1 < n; k++) {
      quarter = (quarter + ((ev[k] < 0.0) ? 3 : 1)) & 3;
      const double re = (quarter == 0) ? 1.0 : ((quarter == 2) ? -1.0 : 0.0);
      const double im = (quarter == 1) ? 1.0 : ((quarter == 3) ? -1.0 : 0.0);
      ph[k + 1] = zc{re, im};
    }
  }
}

// SkewHermTridiagonal{ComplexF64} input (complex subdiagonal ev, imaginary diagonal
// dvim or none): to_symtridiagonal (tridiag.jl:558-583) gives S = SymTridiagonal(-dvim,
// |ev|) and the phases d_1 = 1, d_{k+1} = d_k (i ev_k) / |ev_k|; bnd = {lo, pivmin, hi}.
__global__ void __launch_bounds__(1024) zprep_tri_kernel(const zc* __restrict__ ev, const double* __restrict__ dvim,
                                                        int n, double* __restrict__ dg, double* __restrict__ off,
                                                        zc* __restrict__ ph, double* __restrict__ bp) {
  __shared__ double red[3][32];
  double lo = INFINITY, hi = -INFINITY, e2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = dvim ? neg(dvim[i]) : 0.0;
    const double l = (i > 0) ? hypot(ev[i - 1].re, ev[i - 1].im) : 0.0;
    const double r = (i + 1 < n) ? hypot(ev[i].re, ev[i].im) : 0.0;
    dg[i] = d;
    if (i + 1 < n) {
      off[i] = r;
      e2 = fmax(e2, r * r);
    }
    lo = fmin(lo, d - l - r);
    hi = fmax(hi, d + l + r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    e2 = fmax(e2, __shfl_xor_sync(0xffffffffu, e2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = lo;
    red[1][threadIdx.x >> 5] = hi;
    red[2][threadIdx.x >> 5] = e2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
      lo = fmin(lo, red[0][w]);
      hi = fmax(hi, red[1][w]);
      e2 = fmax(e2, red[2][w]);
    }
    const double span = fmax(fabs(lo), fabs(hi));
    bp[0] = lo - 1e-14 * span - 1e-300;
    bp[1] = 2.2250738585072014e-308 * fmax(1.0, e2);
    bp[2] = hi + 1e-14 * span + 1e-300;
    zc d{1.0, 0.0};
    ph[0] = d;
    for (int k = 0; k + 1 < n; k++) {
      const double a = hypot(ev[k].re, ev[k].im);
      if (a > 0.0) d = zmul(d, zc{neg(ev[k].im) / a, ev[k].re / a});  // (i ev_k) / |ev_k|
      ph[k + 1] = d;
    }
  }
}

cudaError_t zsymtri_prep(const double* ev, const double* dvim, int n, double* dg, double* off, double* ph,
                         double* bnd, cudaStream_t st) {
  zprep_kernel<<<1, 1024, 0, st>>>(ev, dvim, n, dg, off, reinterpret_cast<zc*>(ph), bnd);
  return cudaGetLastError();
}

// number of eigenvalues of S smaller than x (pivots of LDL^T(S - x I), pivmin guard)
__device__ int zsturm(const double* dg, const double* off, int n, double x, double pivmin) {
  double q = dg[0] - x;
  if (fabs(q) <= pivmin) q = neg(pivmin);
  int c = (q < 0.0);
  for (int i = 1; i < n; i++) {
    const double e = off[i - 1];
    q = (dg[i] - x) - (e * e) / q;
    if (fabs(q) <= pivmin) q = neg(pivmin);
    c += (q < 0.0);
  }
  return c;
}

// mu_k = k-th smallest eigenvalue of S by a group of p lanes (multisection,
// absolute tolerance eps * max|Gershgorin bound|); vals_im[k] = -mu_k
__global__ void zbisect_kernel(const double* __restrict__ dg, const double* __restrict__ off, int n, int batch,
                               const double* __restrict__ bp, double* __restrict__ mu, double* __restrict__ vals_im,
                               int p) {
  const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / p;
  const int gl = (threadIdx.x & 31) % p;
  const bool active = gid < (long long)n * batch;
  const size_t mb = active ? (size_t)(gid / n) : 0;
  const int k = active ? (int)(gid - (long long)mb * n) : 0;
  dg += mb * n;
  off += mb * n;
  bp += mb * 8;
  const double lo = bp[0], hi = bp[2], pivmin = bp[1];
  const double x = group_multisect(lo, hi, active ? k : 0, 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)), p,
                                   active, [&](double y) { return zsturm(dg, off, n, y, pivmin); });
  if (active && gl == 0) {
    if (mu) mu[mb * n + k] = x;
    vals_im[mb * n + k] = neg(x);
  }
}

// V(:, k) = D Y(:, k)
__global__ void zassemble_kernel(const double* __restrict__ Y, const zc* __restrict__ ph, int n, zc* __restrict__ V,
                                 int64_t ldv) {
  const size_t mb = blockIdx.z;  // problem mb: Y, V n^2 (V: ldv n) apart, ph n apart
  Y += mb * n * n;
  ph += mb * n;
  V += mb * (size_t)ldv * n;
  const int k = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double y = Y[i + (int64_t)k * n];
    V[i + (int64_t)k * ldv] = zc{ph[i].re * y, ph[i].im * y};
  }
}

// ---------------------------------------------------------------------------
// complex compact WY: Q_b = H_c0 ... H_c1-1 = I - V T V^H, T(i,i) = tau_i,
// T(0:i, i) = -tau_i T(0:i, 0:i) (V(:, 0:i)^H v_i); X <- Q X by strips
// ---------------------------------------------------------------------------
constexpr int ZWB = 32;  // reflectors per panel
constexpr int ZSW = 16;  // complex columns per strip
constexpr int ZRC = 16;  // rows per staged chunk (one X element per thread)

__device__ __forceinline__ zc zrefl_at(const zc* A, int64_t lda, const zc* tau, int row, int c) {
  if (row < c + 1 || (tau[c].re == 0.0 && tau[c].im == 0.0)) return zc{0.0, 0.0};
  return (row == c + 1) ? zc{1.0, 0.0} : A[row + (int64_t)c * lda];
}

__global__ void __launch_bounds__(256) zwy_factor_kernel(const zc* __restrict__ A, int64_t lda,
                                                         const zc* __restrict__ tau, int n, zc* __restrict__ Tg) {
  __shared__ zc Vs[16][ZWB + 1];
  __shared__ zc M[ZWB][ZWB + 1];  // lower: G = V^H V, upper + diagonal: T
  const size_t mb = blockIdx.y;   // problem mb: A lda*n, tau n, T gridDim.x panels apart
  A += mb * (size_t)lda * n;
  tau += mb * n;
  Tg += mb * gridDim.x * (size_t)ZWB * ZWB;
  const int b = blockIdx.x;
  const int c0 = b * ZWB, c1 = min(c0 + ZWB, n - 1), nb = c1 - c0;
  const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;  // G (32 x 32): 2 x 2 per thread
  zc acc[2][2] = {{{0.0, 0.0}, {0.0, 0.0}}, {{0.0, 0.0}, {0.0, 0.0}}};
  for (int r0 = c0 + 1; r0 < n; r0 += 16) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < 16 * ZWB; idx += 256) {
      const int cc = idx / 16, rr = idx - cc * 16;
      const int row = r0 + rr;
      Vs[rr][cc] = (row < n && cc < nb) ? zrefl_at(A, lda, tau, row, c0 + cc) : zc{0.0, 0.0};
    }
    __syncthreads();
    for (int rr = 0; rr < 16; rr++) {
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int q = 0; q < 2; q++) acc[a][q] = zfma(zconj(Vs[rr][ty + 16 * a]), Vs[rr][tx + 16 * q], acc[a][q]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int i = ty + 16 * a, j = tx + 16 * q;  // acc = v_i^H v_j = G(i, j)
      M[i][j] = (i > j) ? acc[a][q] : zc{0.0, 0.0};
    }
  __syncthreads();
  for (int i = 0; i < nb; i++) {
    const zc ti = tau[c0 + i];
    if (threadIdx.x < i) {
      const int j = threadIdx.x;
      zc s{0.0, 0.0};
      for (int l = j; l < i; l++) s = zfma(M[j][l], zconj(M[i][l]), s);  // G(l, i) = conj(G(i, l))
      M[j][i] = zmul(zc{neg(ti.re), neg(ti.im)}, s);
    }
    if (threadIdx.x == 0) M[i][i] = ti;
    __syncthreads();
  }
  zc* T = Tg + (size_t)b * ZWB * ZWB;
  for (int idx = threadIdx.x; idx < ZWB * ZWB; idx += 256) {
    const int i = idx / ZWB, j = idx % ZWB;
    T[idx] = (j >= i) ? M[i][j] : zc{0.0, 0.0};
  }
}

__global__ void __launch_bounds__(256) zback_strip_kernel(const zc* __restrict__ A, int64_t lda,
                                                          const zc* __restrict__ tau, int n, const zc* __restrict__ Tg,
                                                          int npan, zc* __restrict__ X, int64_t ldx, int ncols) {
  __shared__ zc Ts[ZWB][ZWB + 1];
  __shared__ zc Ws[ZWB][ZSW + 1];
  __shared__ zc Vs[ZRC][ZWB + 1];
  __shared__ zc Xs[ZRC][ZSW + 1];
  const size_t mb = blockIdx.y;  // problem mb: A lda*n, tau n, T npan panels, X ldx*ncols apart
  A += mb * (size_t)lda * n;
  tau += mb * n;
  Tg += mb * (size_t)npan * ZWB * ZWB;
  X += mb * (size_t)ldx * ncols;
  const int col0 = blockIdx.x * ZSW;
  const int ncol = min(ZSW, ncols - col0);
  X += (int64_t)col0 * ldx;
  // W (32 x 16): 2 per thread (rows wr, wr+16); X chunk (16 x 16): 1 per thread
  const int wc = threadIdx.x & 15, wr = threadIdx.x >> 4;
  for (int b = npan - 1; b >= 0; b--) {
    const int c0 = b * ZWB, c1 = min(c0 + ZWB, n - 1), nb = c1 - c0;
    __syncthreads();
    for (int idx = threadIdx.x; idx < ZWB * ZWB; idx += 256) Ts[idx / ZWB][idx % ZWB] = Tg[(size_t)b * ZWB * ZWB + idx];
    zc w0{0.0, 0.0}, w1{0.0, 0.0};
    for (int r0 = c0 + 1; r0 < n; r0 += ZRC) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < ZRC * ZWB; idx += 256) {
        const int cc = idx / ZRC, rr = idx - cc * ZRC;
        const int row = r0 + rr;
        Vs[rr][cc] = (row < n && cc < nb) ? zrefl_at(A, lda, tau, row, c0 + cc) : zc{0.0, 0.0};
      }
      for (int idx = threadIdx.x; idx < ZRC * ZSW; idx += 256) {
        const int cc = idx / ZRC, rr = idx - cc * ZRC;
        const int row = r0 + rr;
        Xs[rr][cc] = (row < n && cc < ncol) ? X[row + (int64_t)cc * ldx] : zc{0.0, 0.0};
      }
      __syncthreads();
#pragma unroll 4
      for (int rr = 0; rr < ZRC; rr++) {
        const zc x = Xs[rr][wc];
        w0 = zfma(zconj(Vs[rr][wr]), x, w0);
        w1 = zfma(zconj(Vs[rr][wr + 16]), x, w1);
      }
    }
    Ws[wr][wc] = w0;
    Ws[wr + 16][wc] = w1;
    __syncthreads();
    zc t0{0.0, 0.0}, t1{0.0, 0.0};
    for (int l = wr; l < ZWB; l++) t0 = zfma(Ts[wr][l], Ws[l][wc], t0);
    for (int l = wr + 16; l < ZWB; l++) t1 = zfma(Ts[wr + 16][l], Ws[l][wc], t1);
    __syncthreads();
    Ws[wr][wc] = t0;
    Ws[wr + 16][wc] = t1;
    for (int r0 = c0 + 1; r0 < n; r0 += ZRC) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < ZRC * ZWB; idx += 256) {
        const int cc = idx / ZRC, rr = idx - cc * ZRC;
        const int row = r0 + rr;
        Vs[rr][cc] = (row < n && cc < nb) ? zrefl_at(A, lda, tau, row, c0 + cc) : zc{0.0, 0.0};
      }
      for (int idx = threadIdx.x; idx < ZRC * ZSW; idx += 256) {
        const int cc = idx / ZRC, rr = idx - cc * ZRC;
        const int row = r0 + rr;
        Xs[rr][cc] = (row < n && cc < ncol) ? X[row + (int64_t)cc * ldx] : zc{0.0, 0.0};
      }
      __syncthreads();
      zc a0{0.0, 0.0};
#pragma unroll 8
      for (int l = 0; l < ZWB; l++) a0 = zfma(Vs[wr][l], Ws[l][wc], a0);
      Xs[wr][wc] = zsub(Xs[wr][wc], a0);
      __syncthreads();
      for (int idx = threadIdx.x; idx < ZRC * ZSW; idx += 256) {
        const int cc = idx / ZRC, rr = idx - cc * ZRC;
        const int row = r0 + rr;
        if (row < n && cc < ncol) X[row + (int64_t)cc * ldx] = Xs[rr][cc];
      }
    }
  }
}

// workspace segments are rounded to 32 doubles so that every complex array is 16-byte aligned
static inline size_t seg(size_t d) { return (d + 31) & ~(size_t)31; }

size_t zeigen_ws_doubles(int n, int batch) {
  const int npan = (n - 1 + ZWB - 1) / ZWB;
  const size_t B = (size_t)(batch > 0 ? batch : 1);
  return 3 * seg(B * n)                      // dg, off, mu
         + seg(2 * B * n)                    // phases
         + seg(8 * B)                        // bp
         + seg(B * n * n)                    // Y
         + seg(2 * B * std::max(npan, 1) * ZWB * ZWB)  // T factors
         + B * large_eigen_ws_doubles(n) + 64;
}

// Eigen-decomposition of `batch` reduced matrices of size n (A: the reflectors,
// lda*n apart; tau, ev, dvim, vals_im n apart): vals_im (descending) and, if
// V != null, the eigenvectors V (ldv*n apart).
cudaError_t zeigen_from_tridiag(const double* Ad, int64_t lda, int n, const double* taud, const double* ev,
                                const double* dvim, double* vals_im, double* Vd, int64_t ldv, double* ws, int batch,
                                cudaStream_t st) {
  const int npan = (n - 1 + ZWB - 1) / ZWB;
  const size_t B = (size_t)batch;
  double* dg = ws;
  double* off = dg + seg(B * n);
  double* mu = off + seg(B * n);
  zc* ph = reinterpret_cast<zc*>(mu + seg(B * n));
  double* bp = mu + seg(B * n) + seg(2 * B * n);
  double* Y = bp + seg(8 * B);
  zc* Tg = reinterpret_cast<zc*>(Y + seg(B * n * n));
  double* tws = Y + seg(B * n * n) + seg(2 * B * std::max(npan, 1) * ZWB * ZWB);
  zprep_kernel<<<batch, 1024, 0, st>>>(ev, dvim, n, dg, off, ph, bp);
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int p = multisect_lanes(n * batch, sms);
  const long long threads = ((long long)n * batch * p + 31) / 32 * 32;
  zbisect_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(dg, off, n, batch, bp, mu, vals_im, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !Vd) return e;
  e = symtri_vectors(dg, off, n, mu, bp, Y, tws, batch, st);
  if (e != cudaSuccess) return e;
  zc* V = reinterpret_cast<zc*>(Vd);
  zassemble_kernel<<<dim3((n + 255) / 256, n, batch), 256, 0, st>>>(Y, ph, n, V, ldv);
  e = cudaGetLastError();
  if (e != cudaSuccess || n < 2) return e;
  const zc* A = reinterpret_cast<const zc*>(Ad);
  const zc* tau = reinterpret_cast<const zc*>(taud);
  zwy_factor_kernel<<<dim3(npan, batch), 256, 0, st>>>(A, lda, tau, n, Tg);
  zback_strip_kernel<<<dim3((n + ZSW - 1) / ZSW, batch), 256, 0, st>>>(A, lda, tau, n, Tg, npan, V, ldv, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// complex products for exp and its adjoint: C = op(A) op(B), op in {N, H}
// (32 x 32 output tiles, 2 x 2 per thread, K in chunks of 16)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zgemm_kernel(int n, const zc* __restrict__ A, int64_t lda, int ha,
                                                    const zc* __restrict__ B, int64_t ldb, int hb, zc* __restrict__ C,
                                                    int64_t ldc) {
  __shared__ zc As[32][17];
  __shared__ zc Bs[16][33];
  const size_t mb = blockIdx.z;  // problem mb: each operand ld*n apart
  A += mb * (size_t)lda * n;
  B += mb * (size_t)ldb * n;
  C += mb * (size_t)ldc * n;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // rows i0 + tx + 16a, columns j0 + ty + 16q
  zc acc[2][2] = {{{0.0, 0.0}, {0.0, 0.0}}, {{0.0, 0.0}, {0.0, 0.0}}};
  for (int k0 = 0; k0 < n; k0 += 16) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * 16; idx += 256) {
      // A tile (32 rows x 16 k): element (i, k) = A[i, k] or conj(A[k, i])
      int r, kk;
      if (!ha) { r = idx & 31; kk = idx >> 5; } else { kk = idx & 15; r = idx >> 4; }
      const int i = i0 + r, k = k0 + kk;
      zc a{0.0, 0.0};
      if (i < n && k < n) a = ha ? zconj(A[k + (int64_t)i * lda]) : A[i + (int64_t)k * lda];
      As[r][kk] = a;
      // B tile (16 k x 32 cols): element (k, j) = B[k, j] or conj(B[j, k])
      int c2, k2;
      if (!hb) { k2 = idx & 15; c2 = idx >> 4; } else { c2 = idx & 31; k2 = idx >> 5; }
      const int j = j0 + c2, kb = k0 + k2;
      zc bv{0.0, 0.0};
      if (j < n && kb < n) bv = hb ? zconj(B[j + (int64_t)kb * ldb]) : B[kb + (int64_t)j * ldb];
      Bs[k2][c2] = bv;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; kk++) {
      const zc a0 = As[tx][kk], a1 = As[tx + 16][kk];
      const zc b0 = Bs[kk][ty], b1 = Bs[kk][ty + 16];
      acc[0][0] = zfma(a0, b0, acc[0][0]);
      acc[0][1] = zfma(a0, b1, acc[0][1]);
      acc[1][0] = zfma(a1, b0, acc[1][0]);
      acc[1][1] = zfma(a1, b1, acc[1][1]);
    }
  }
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int i = i0 + tx + 16 * a, j = j0 + ty + 16 * q;
      if (i < n && j < n) C[i + (int64_t)j * ldc] = acc[a][q];
    }
}

// mode 0: P(:, k) = V(:, k) f(i mu_k)   (F = P V^H for the function `func`)
// mode 1: M(j, k) <- conj(Phi(j, k)) M(j, k), Phi(j,k) = e^{i(mu_j+mu_k)/2} sinc((mu_j-mu_k)/2)
__global__ void zscale_kernel(int mode, int func, int n, const double* __restrict__ mu, const zc* __restrict__ V,
                              int64_t ldv, zc* __restrict__ M, int64_t ldm, int* __restrict__ status) {
  const size_t mb = blockIdx.z;  // problem mb: mu n, V ldv*n, M ldm*n apart
  mu += mb * n;
  V += mb * (size_t)ldv * n;
  M += mb * (size_t)ldm * n;
  const int k = blockIdx.y;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    if (mode == 0) {
      double fa, fb;
      bool sing = false;
      skew_scalar_func(func, mu[k], &fa, &fb, &sing);
      if (sing && j == 0 && status) status[mb] = SKEW_SINGULAR;
      M[j + (int64_t)k * ldm] = zmul(V[j + (int64_t)k * ldv], zc{fa, fb});
    } else {
      const double a = mu[j], bb = mu[k];
      const double d = 0.5 * (a - bb);
      const double sc = (fabs(d) < 1e-8) ? fma(neg(d) * d, 1.0 / 6.0, 1.0) : sin(d) / d;
      double s, c;
      sincos(0.5 * (a + bb), &s, &c);
      M[j + (int64_t)k * ldm] = zmul(M[j + (int64_t)k * ldm], zc{c * sc, neg(s) * sc});
    }
  }
}

// O <- (O + s O^H) / 2 in place (s = +1 Hermitian part, -1 skew-Hermitian part)
__global__ void zsymmetrize_kernel(int n, zc* __restrict__ O, int64_t ldo, int s) {
  O += (size_t)blockIdx.z * ldo * n;
  const int64_t tot = (int64_t)n * n;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(q / n), i = (int)(q - (int64_t)j * n);
    if (i < j) continue;
    zc* pij = O + i + (int64_t)j * ldo;
    if (i == j) {  // Hermitian: real diagonal; skew-Hermitian: imaginary diagonal
      if (s > 0)
        pij->im = 0.0;
      else
        pij->re = 0.0;
      continue;
    }
    zc* pji = O + j + (int64_t)i * ldo;
    const zc x = *pij, y = *pji;
    const zc u = zc{0.5 * (x.re + s * y.re), 0.5 * (x.im - s * y.im)};  // (x + s conj(y)) / 2
    *pij = u;
    *pji = zc{s * u.re, neg(s * u.im)};  // s conj(u)
  }
}

cudaError_t zfunc_from_eigen(int mode, int func, int n, const double* vals_im, const double* Vd, int64_t ldv,
                             const double* Cd, int64_t ldc, double* Od, int64_t ldo, double* ws, int batch,
                             int* status, cudaStream_t st) {
  const zc* V = reinterpret_cast<const zc*>(Vd);
  zc* O = reinterpret_cast<zc*>(Od);
  zc* T1 = reinterpret_cast<zc*>(ws);
  zc* T2 = T1 + (size_t)batch * n * n;
  const dim3 g((n + 31) / 32, (n + 31) / 32, batch);
  const dim3 gs((n + 255) / 256, n, batch);
  if (mode == 0) {  // F = V diag(f(i mu)) V^H, then its (skew-)Hermitian part
    zscale_kernel<<<gs, 256, 0, st>>>(0, func, n, vals_im, V, ldv, T1, n, status);
    zgemm_kernel<<<g, 256, 0, st>>>(n, T1, n, 0, V, ldv, 1, O, ldo);
    const int sym = skew_func_symmetry(func);
    if (sym != 0) {
      const int64_t tot = (int64_t)n * n;
      zsymmetrize_kernel<<<dim3((unsigned)std::min<int64_t>((tot + 255) / 256, 1024), 1, batch), 256, 0, st>>>(
          n, O, ldo, sym);
    }
  } else {  // G = V (conj(Phi) o (V^H C V)) V^H
    const zc* C = reinterpret_cast<const zc*>(Cd);
    zgemm_kernel<<<g, 256, 0, st>>>(n, V, ldv, 1, C, ldc, 0, T1, n);   // V^H C
    zgemm_kernel<<<g, 256, 0, st>>>(n, T1, n, 0, V, ldv, 0, T2, n);    // (V^H C) V
    zscale_kernel<<<gs, 256, 0, st>>>(1, 0, n, vals_im, V, ldv, T2, n, nullptr);
    zgemm_kernel<<<g, 256, 0, st>>>(n, V, ldv, 0, T2, n, 0, T1, n);    // V M
    zgemm_kernel<<<g, 256, 0, st>>>(n, T1, n, 0, V, ldv, 1, O, ldo);   // (V M) V^H
  }
  return cudaGetLastError();
}

size_t zfunc_ws_doubles(int n, int batch) { return 4 * (size_t)batch * n * n + 32; }

// eigen of a SkewHermTridiagonal{ComplexF64}: vals_im (descending) and, if V != null,
// V = D Y (no reflectors); ws: zeigen_ws_doubles(n, 1)
cudaError_t zeigen_tridiag(const double* evd, const double* dvim, int n, double* vals_im, double* Vd, int64_t ldv,
                           double* ws, cudaStream_t st) {
  double* dg = ws;
  double* off = dg + seg(n);
  double* mu = off + seg(n);
  zc* ph = reinterpret_cast<zc*>(mu + seg(n));
  double* bp = mu + seg(n) + seg(2 * (size_t)n);
  double* Y = bp + seg(8);
  const int npan = (n - 1 + ZWB - 1) / ZWB;
  double* tws = Y + seg((size_t)n * n) + seg(2 * (size_t)std::max(npan, 1) * ZWB * ZWB);
  zprep_tri_kernel<<<1, 1024, 0, st>>>(reinterpret_cast<const zc*>(evd), dvim, n, dg, off, ph, bp);
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int p = multisect_lanes(n, sms);
  const long long threads = ((long long)n * p + 31) / 32 * 32;
  zbisect_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(dg, off, n, 1, bp, mu, vals_im, p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !Vd) return e;
  e = symtri_vectors(dg, off, n, mu, bp, Y, tws, 1, st);
  if (e != cudaSuccess) return e;
  zassemble_kernel<<<dim3((n + 255) / 256, n, 1), 256, 0, st>>>(Y, ph, n, reinterpret_cast<zc*>(Vd), ldv);
  return cudaGetLastError();
}

}  // namespace skew
