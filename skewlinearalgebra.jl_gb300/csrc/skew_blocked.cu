// Blocked Householder tridiagonalisation of one large skew matrix across the
// whole GPU (the skewblockedhess! / skewlatrd! structure of hessenberg.jl:92-173).
//
// Panels of NB columns.  For panel column c (local index i = c - p):
//   sym_kernel   : y = A[c+1:n, c+1:n] v  (full rows of the trailing matrix as it
//                  was at the panel start), u1 = W[c+1:n, 0:i]^T v and
//                  u2 = A[c+1:n, p:c]^T v.  v = [1; A[c+2:n, c] * scale] is formed
//                  on the fly from the reflector scalars.  Partial sums go to
//                  per-chunk buffers (deterministic, no floating-point atomics).
//   fin_kernel   : writes v into column c, W[:, i] = tau (y + A_p u1 - W_p u2)
//                  (hessenberg.jl:114-121), then applies the panel so far to
//                  column c+1 (hessenberg.jl:100-107) and accumulates its norm.
//                  The last CTA to finish (atomic ticket, no waiting) builds
//                  reflector c+1 (householder!, hessenberg.jl:26-44).
// After NB columns, upd_kernel applies A22 += V W^T - W V^T (hessenberg.jl:158-166)
// to the lower triangle of the trailing matrix in 64 x 64 register-tiled blocks
// and mirrors each block to the upper triangle.  The last <= 128 columns are
// reduced by the one-CTA kernel of skew_batch.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"
#include "skew_internal.h"

namespace skew {

constexpr int BNB = 64;        // panel width
constexpr int SYM_ROWS = 256;  // rows per sym CTA (one per thread)
constexpr int FIN_ROWS = 64;   // rows per fin CTA (4 threads per row)
constexpr int UPD_T = 64;      // update tile edge
constexpr int TAIL = 128;      // columns left to the one-CTA kernel

struct BlockedWs {
  double* W;      // n x BNB, column-major, ld n (rows indexed globally)
  double* ypart;  // max_chunks x n
  double* upart;  // max_symtiles x (2 * BNB)
  double* sspart; // max_fintiles
  double* scal;   // 3 per column: beta, tau, scale
  unsigned* ticket;
  int max_chunks, max_symtiles, max_fintiles;
};

size_t blocked_ws_doubles(int n) {
  const int max_chunks = 64;
  const int max_symtiles = (n + SYM_ROWS - 1) / SYM_ROWS;
  const int max_fintiles = (n + FIN_ROWS - 1) / FIN_ROWS;
  return (size_t)n * BNB + (size_t)max_chunks * n + (size_t)max_symtiles * 2 * BNB + max_fintiles + 3 * (size_t)n +
         8;
}

static BlockedWs carve_ws(double* base, int n) {
  BlockedWs w;
  w.max_chunks = 64;
  w.max_symtiles = (n + SYM_ROWS - 1) / SYM_ROWS;
  w.max_fintiles = (n + FIN_ROWS - 1) / FIN_ROWS;
  double* p = base;
  w.W = p;
  p += (size_t)n * BNB;
  w.ypart = p;
  p += (size_t)w.max_chunks * n;
  w.upart = p;
  p += (size_t)w.max_symtiles * 2 * BNB;
  w.sspart = p;
  p += w.max_fintiles;
  w.scal = p;
  p += 3 * (size_t)n;
  w.ticket = (unsigned*)p;
  return w;
}

__device__ __forceinline__ double vval(const double* A, int64_t lda, int c, int r, double scale, double tau) {
  // reflector c at row r (r >= c+1) before it is written back into A
  if (tau == 0.0) return 0.0;
  return (r == c + 1) ? 1.0 : A[r + (int64_t)c * lda] * scale;
}

// ---------------------------------------------------------------------------
// Reflector for column c from its (already updated) entries, one CTA.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) col0_kernel(double* A, int64_t lda, int n, int c, double* scal, double* ev,
                                                   double* tau) {
  __shared__ double red[8];
  double part = 0.0;
  for (int r = c + 2 + threadIdx.x; r < n; r += 256) {
    const double x = A[r + (int64_t)c * lda];
    part = fma(x, x, part);
  }
  double ss = block_sum<8>(part, red);
  double xn = -1.0;
  if (ss_needs_scaling(ss)) {
    double mx = 0.0;
    for (int r = c + 2 + threadIdx.x; r < n; r += 256) mx = fmax(mx, fabs(A[r + (int64_t)c * lda]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double rm[8];
    if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = 0.0;
    for (int q = 0; q < 8; q++) mx = fmax(mx, rm[q]);
    double qq = 0.0;
    if (mx > 0.0)
      for (int r = c + 2 + threadIdx.x; r < n; r += 256) {
        const double x = A[r + (int64_t)c * lda] / mx;
        qq = fma(x, x, qq);
      }
    qq = block_sum<8>(qq, red);
    xn = mx * sqrt(qq);
  }
  if (threadIdx.x == 0) {
    const Reflector R = make_reflector(A[(c + 1) + (int64_t)c * lda], ss, xn);
    scal[3 * c + 0] = R.beta;
    scal[3 * c + 1] = R.tau;
    scal[3 * c + 2] = R.scale;
    ev[c] = R.beta;
    tau[c] = R.tau;
  }
}

// ---------------------------------------------------------------------------
// sym_kernel: grid (row tiles, column chunks).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SYM_ROWS) sym_kernel(const double* __restrict__ A, int64_t lda, int n, int p, int c,
                                                       BlockedWs ws, int nchunk, int chunk) {
  __shared__ double sv[512 + 8];
  const int i = c - p;
  const double tau = ws.scal[3 * c + 1], scale = ws.scal[3 * c + 2];
  const int r0 = c + 1;
  const int tile = blockIdx.x, ch = blockIdx.y;
  const int r = r0 + tile * SYM_ROWS + threadIdx.x;
  const int cb = r0 + ch * chunk, ce = min(n, cb + chunk);
  // stage v over this CTA's column chunk
  for (int j = cb + threadIdx.x; j < ce; j += SYM_ROWS) sv[j - cb] = vval(A, lda, c, j, scale, tau);
  __syncthreads();
  if (r < n) {
    const double* row = A + r;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0, a7 = 0;
    int j = cb;
    for (; j + 7 < ce; j += 8) {
      const double w0 = row[(int64_t)j * lda], w1 = row[(int64_t)(j + 1) * lda], w2 = row[(int64_t)(j + 2) * lda],
                   w3 = row[(int64_t)(j + 3) * lda], w4 = row[(int64_t)(j + 4) * lda], w5 = row[(int64_t)(j + 5) * lda],
                   w6 = row[(int64_t)(j + 6) * lda], w7 = row[(int64_t)(j + 7) * lda];
      const double* vv = sv + (j - cb);
      a0 = fma(w0, vv[0], a0);
      a1 = fma(w1, vv[1], a1);
      a2 = fma(w2, vv[2], a2);
      a3 = fma(w3, vv[3], a3);
      a4 = fma(w4, vv[4], a4);
      a5 = fma(w5, vv[5], a5);
      a6 = fma(w6, vv[6], a6);
      a7 = fma(w7, vv[7], a7);
    }
    for (; j < ce; j++) a0 = fma(row[(int64_t)j * lda], sv[j - cb], a0);
    ws.ypart[(size_t)ch * n + r] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  }
  // panel dot products, chunk-0 CTAs only: warp q handles dots q, q+8, ...
  if (ch == 0 && i > 0) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rb = r0 + tile * SYM_ROWS, re = min(n, rb + SYM_ROWS);
    for (int d = w; d < 2 * i; d += 8) {
      const int j = d < i ? d : d - i;
      const double* col = (d < i) ? (ws.W + (size_t)j * n) : (A + (int64_t)(p + j) * lda);
      double acc = 0.0;
      for (int rr = rb + lane; rr < re; rr += 32) acc = fma(col[rr], vval(A, lda, c, rr, scale, tau), acc);
      acc = warp_sum(acc);
      if (lane == 0) ws.upart[(size_t)tile * 2 * BNB + d] = acc;
    }
  }
}

// ---------------------------------------------------------------------------
// fin_kernel: grid = row tiles of FIN_ROWS over [c+1, n); 4 threads per row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) fin_kernel(double* __restrict__ A, int64_t lda, int n, int p, int c,
                                                  int last_in_panel, BlockedWs ws, int nchunk, int nsymtiles,
                                                  double* ev, double* tauo) {
  __shared__ double su[2 * BNB];       // u1 (0..i-1), u2 (BNB..BNB+i-1)
  __shared__ double sWrow[BNB + 1];    // W[c+1, 0..i]
  __shared__ double sArow[BNB + 1];    // A[c+1, p..c]  (reflector entries of row c+1)
  __shared__ double red[8];
  __shared__ bool s_last;
  const int i = c - p;
  const double tau = ws.scal[3 * c + 1], scale = ws.scal[3 * c + 2];
  const int r0 = c + 1;
  const int tid = threadIdx.x;
  // 1. u1, u2: sum the per-tile partials in a fixed order
  for (int d = tid; d < 2 * i; d += 256) {
    double s = 0.0;
    for (int t = 0; t < nsymtiles; t++) s += ws.upart[(size_t)t * 2 * BNB + d];
    if (d < i)
      su[d] = s;
    else
      su[BNB + d - i] = s;
  }
  __syncthreads();
  // 2. W[c+1, i] redundantly in every CTA (needed by the column c+1 update)
  if (tid < 32) {
    const int lane = tid;
    double acc = 0.0;
    for (int j = lane; j < i; j += 32)
      acc = fma(A[r0 + (int64_t)(p + j) * lda], su[j], fma(-ws.W[(size_t)j * n + r0], su[BNB + j], acc));
    acc = warp_sum(acc);
    if (lane == 0) {
      double y = 0.0;
      for (int q = 0; q < nchunk; q++) y += ws.ypart[(size_t)q * n + r0];
      sWrow[i] = tau * (y + acc);
    }
    for (int j = lane; j < i; j += 32) {
      sWrow[j] = ws.W[(size_t)j * n + r0];
      sArow[j] = A[r0 + (int64_t)(p + j) * lda];
    }
    if (lane == 0) sArow[i] = (tau == 0.0) ? 0.0 : 1.0;  // v_c at row c+1
  }
  __syncthreads();
  // 3. own rows: write v into column c, W[r, i], update column c+1, norm partial.
  //    All lanes take part in the shuffles; only memory accesses are guarded.
  const int row = r0 + blockIdx.x * FIN_ROWS + (tid >> 2);
  const int g = tid & 3;
  const bool valid = row < n;
  double vr = 0.0, acc = 0.0;
  if (valid) {
    vr = vval(A, lda, c, row, scale, tau);
    for (int j = g; j < i; j += 4)
      acc = fma(A[row + (int64_t)(p + j) * lda], su[j], fma(-ws.W[(size_t)j * n + row], su[BNB + j], acc));
  }
  acc += __shfl_xor_sync(0xffffffffu, acc, 1);
  acc += __shfl_xor_sync(0xffffffffu, acc, 2);
  double y = 0.0;
  if (valid && g == 0)
    for (int q = 0; q < nchunk; q++) y += ws.ypart[(size_t)q * n + row];
  y = __shfl_sync(0xffffffffu, y, (tid & 31) & ~3);
  double wri = tau * (y + acc);
  if (row == r0) wri = sWrow[i];  // one value for W[c+1, i] everywhere
  if (valid && g == 0) {
    ws.W[(size_t)i * n + row] = wri;
    A[row + (int64_t)c * lda] = vr;
  }
  double sspart = 0.0;
  const bool doupd = valid && !last_in_panel && row >= c + 2;
  double u = 0.0;
  if (doupd)
    for (int j = g; j <= i; j += 4) {
      // A[row, c+1] += sum_{j<=i} A[row, p+j] W[c+1, j] - W[row, j] A[c+1, p+j]
      const double arj = (j == i) ? vr : A[row + (int64_t)(p + j) * lda];
      const double wrj = (j == i) ? wri : ws.W[(size_t)j * n + row];
      u = fma(arj, sWrow[j], fma(-wrj, sArow[j], u));
    }
  u += __shfl_xor_sync(0xffffffffu, u, 1);
  u += __shfl_xor_sync(0xffffffffu, u, 2);
  if (doupd && g == 0) {
    const double anew = A[row + (int64_t)(c + 1) * lda] + u;
    A[row + (int64_t)(c + 1) * lda] = anew;
    if (row >= c + 3) sspart = anew * anew;
  }
  if (last_in_panel) return;
  // 4. norm partial of column c+1 (rows c+3..) and the last-CTA reflector
  const double ss_blk = block_sum<8>(sspart, red);
  if (tid == 0) ws.sspart[blockIdx.x] = ss_blk;
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    const unsigned t = atomicAdd(ws.ticket, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (tid == 0) {
    double ss = 0.0;
    for (int t = 0; t < (int)gridDim.x; t++) ss += ((volatile double*)ws.sspart)[t];
    *ws.ticket = 0u;
    const int c1 = c + 1;
    if (c1 <= n - 3) {
      double xn = -1.0;
      if (ss_needs_scaling(ss)) {
        double mx = 0.0;
        for (int r = c1 + 2; r < n; r++) mx = fmax(mx, fabs(((volatile double*)A)[r + (int64_t)c1 * lda]));
        double qq = 0.0;
        if (mx > 0.0)
          for (int r = c1 + 2; r < n; r++) {
            const double x = ((volatile double*)A)[r + (int64_t)c1 * lda] / mx;
            qq = fma(x, x, qq);
          }
        xn = mx * sqrt(qq);
      }
      const double alpha = ((volatile double*)A)[(c1 + 1) + (int64_t)c1 * lda];
      const Reflector R = make_reflector(alpha, ss, xn);
      ws.scal[3 * c1 + 0] = R.beta;
      ws.scal[3 * c1 + 1] = R.tau;
      ws.scal[3 * c1 + 2] = R.scale;
      ev[c1] = R.beta;
      tauo[c1] = R.tau;
    }
  }
}

// ---------------------------------------------------------------------------
// upd_kernel: A22 += V W^T - W V^T on the lower triangle of [q, n)^2, mirrored.
// One CTA per 64 x 64 lower tile; 256 threads, 4 x 4 elements per thread.
// V[r, l] = A[r, p + l], W[r, l] = ws.W[l * n + r].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) upd_kernel(double* __restrict__ A, int64_t lda, int n, int p, int nbp, int q,
                                                  const double* __restrict__ Wb) {
  constexpr int KC = 16;
  // operand panels during the k loop, then the transposed tile for the mirror
  __shared__ double sbuf[UPD_T * (UPD_T + 1)];
  double (*sVR)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf);
  double (*sWR)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + KC * UPD_T);
  double (*sVC)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + 2 * KC * UPD_T);
  double (*sWC)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + 3 * KC * UPD_T);
  double (*sT)[UPD_T + 1] = reinterpret_cast<double (*)[UPD_T + 1]>(sbuf);
  // tile index -> (ti, tj), ti >= tj
  const int t = blockIdx.x;
  int ti = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= t) ti++;
  while (ti * (ti + 1) / 2 > t) ti--;
  const int tj = t - ti * (ti + 1) / 2;
  const int R0 = q + ti * UPD_T, C0 = q + tj * UPD_T;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;
  for (int k0 = 0; k0 < nbp; k0 += KC) {
    const int kc = min(KC, nbp - k0);
    for (int idx = threadIdx.x; idx < KC * UPD_T; idx += 256) {
      const int kk = idx / UPD_T, rr = idx - kk * UPD_T;
      double vr = 0.0, wr = 0.0, vc = 0.0, wc = 0.0;
      if (kk < kc) {
        const int l = k0 + kk;
        const int gr = R0 + rr, gc = C0 + rr;
        if (gr < n) {
          vr = A[gr + (int64_t)(p + l) * lda];
          wr = Wb[(size_t)l * n + gr];
        }
        if (gc < n) {
          vc = A[gc + (int64_t)(p + l) * lda];
          wc = Wb[(size_t)l * n + gc];
        }
      }
      sVR[kk][rr] = vr;
      sWR[kk][rr] = wr;
      sVC[kk][rr] = vc;
      sWC[kk][rr] = wc;
    }
    __syncthreads();
    for (int kk = 0; kk < kc; kk++) {
      double vR[4], wR[4], vC[4], wC[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        vR[a] = sVR[kk][tx + 16 * a];
        wR[a] = sWR[kk][tx + 16 * a];
        vC[a] = sVC[kk][ty + 16 * a];
        wC[a] = sWC[kk][ty + 16 * a];
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = fma(vR[a], wC[b], fma(-wR[a], vC[b], acc[a][b]));
    }
    __syncthreads();
  }
  // apply to the lower part, stash the new values for the mirror
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int rr = tx + 16 * a, cc = ty + 16 * b;
      const int gr = R0 + rr, gc = C0 + cc;
      double val = 0.0;
      if (gr < n && gc < n && gr > gc) {
        double* pa = A + gr + (int64_t)gc * lda;
        val = *pa + acc[a][b];
        *pa = val;
      }
      sT[rr][cc] = val;
    }
  __syncthreads();
  // mirror: A[gc, gr] = -A[gr, gc]; lanes along cc for coalescing
  for (int idx = threadIdx.x; idx < UPD_T * UPD_T; idx += 256) {
    const int rr = idx / UPD_T, cc = idx - rr * UPD_T;
    const int gr = R0 + rr, gc = C0 + cc;
    if (gr < n && gc < n && gr > gc) A[gc + (int64_t)gr * lda] = neg(sT[rr][cc]);
  }
}

// flag[0] = 1.0 if A != -A^T anywhere (isskewhermitian, skewhermitian.jl:84-94).
// flag must be zero before the launch.
__global__ void check_skew_kernel(const double* __restrict__ A, int64_t lda, int n, double* flag) {
  const int64_t total = (int64_t)n * n;
  int bad = 0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(e / n), i = (int)(e - (int64_t)j * n);
    bad |= !(A[i + (int64_t)j * lda] == -A[j + (int64_t)i * lda]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) flag[0] = 1.0;
}

cudaError_t launch_check_skew(const double* A, int64_t lda, int n, double* flag, int sms, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(double), st);
  if (e != cudaSuccess) return e;
  check_skew_kernel<<<2 * sms, 256, 0, st>>>(A, lda, n, flag);
  return cudaGetLastError();
}

// log|Pf| and sign from ev and tau for one matrix (used after the blocked path).
// notskew (nullable) is the flag of check_skew_kernel.
__global__ void __launch_bounds__(256) pf_from_tridiag_kernel(const double* ev, const double* tau, int n,
                                                              double* logpf, double* sign, int* info,
                                                              const double* notskew) {
  __shared__ double red[8];
  if (notskew && notskew[0] != 0.0) {
    if (threadIdx.x == 0) {
      *logpf = nan("");
      *sign = nan("");
      if (info) *info = SKEW_NOT_SKEW;
    }
    return;
  }
  if (n & 1) {
    if (threadIdx.x == 0) {
      *logpf = -INFINITY;
      *sign = 0.0;
      if (info) *info = SKEW_SINGULAR;
    }
    return;
  }
  double lp = 0.0;
  int npos = 0, nzero = 0, ntau = 0;
  for (int a = threadIdx.x; a < n / 2; a += 256) {
    const double e = ev[2 * a];
    lp += log(fabs(e));
    npos += (e > 0.0);
    nzero += (e == 0.0);
  }
  for (int a = threadIdx.x; a < n - 1; a += 256) ntau += (tau[a] != 0.0);
  const int tflip = __syncthreads_count((npos + ntau) & 1);
  const int tzero = __syncthreads_count(nzero > 0);
  const double total = block_sum<8>(lp, red);
  if (threadIdx.x == 0) {
    *logpf = total;
    *sign = tzero ? 0.0 : ((tflip & 1) ? -1.0 : 1.0);
    if (info) *info = tzero ? SKEW_SINGULAR : SKEW_OK;
  }
}

cudaError_t launch_pf_from_tridiag(const double* ev, const double* tau, int n, double* logpf, double* sign, int* info,
                                   const double* notskew, cudaStream_t st) {
  pf_from_tridiag_kernel<<<1, 256, 0, st>>>(ev, tau, n, logpf, sign, info, notskew);
  return cudaGetLastError();
}

// Host driver.  ws must hold blocked_ws_doubles(n) doubles; A is reduced in place.
cudaError_t blocked_hessenberg(double* A, int64_t lda, int n, double* tau, double* ev, int* info, double* wsbase,
                               int sms, cudaStream_t st) {
  BlockedWs ws = carve_ws(wsbase, n);
  cudaError_t e = cudaMemsetAsync(ws.ticket, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  int p = 0;
  if (n - p > TAIL) {
    col0_kernel<<<1, 256, 0, st>>>(A, lda, n, 0, ws.scal, ev, tau);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  while (n - p > TAIL) {
    // panel columns p .. p+nbp-1; keep at least TAIL columns for the tail
    const int nbp = min(BNB, n - TAIL - p);
    for (int i = 0; i < nbp; i++) {
      const int c = p + i;
      const int m = n - (c + 1);
      const int symtiles = (m + SYM_ROWS - 1) / SYM_ROWS;
      int nchunk = max((2 * sms + symtiles - 1) / symtiles, (m + 511) / 512);  // chunk <= 512 (sv stage)
      nchunk = max(1, min(nchunk, min(ws.max_chunks, (m + 31) / 32)));
      const int chunk = (m + nchunk - 1) / nchunk;
      nchunk = (m + chunk - 1) / chunk;
      sym_kernel<<<dim3(symtiles, nchunk), SYM_ROWS, 0, st>>>(A, lda, n, p, c, ws, nchunk, chunk);
      const int fintiles = (m + FIN_ROWS - 1) / FIN_ROWS;
      fin_kernel<<<fintiles, 256, 0, st>>>(A, lda, n, p, c, i == nbp - 1 ? 1 : 0, ws, nchunk, symtiles, ev, tau);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    const int q = p + nbp;
    const int mt = (n - q + UPD_T - 1) / UPD_T;
    upd_kernel<<<mt * (mt + 1) / 2, 256, 0, st>>>(A, lda, n, p, nbp, q, ws.W);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    p = q;
    if (n - p > TAIL) {
      col0_kernel<<<1, 256, 0, st>>>(A, lda, n, p, ws.scal, ev, tau);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
  }
  // tail: one CTA, in place on A[p:n, p:n]
  SingleParams P;
  P.A = A + p + (int64_t)p * lda;
  P.lda = lda;
  P.n = n - p;
  P.G = nullptr;
  P.ldg = 0;
  P.logpf = nullptr;
  P.sign = nullptr;
  P.ev = ev + p;
  P.tau = tau + p;
  P.info = info;
  P.check = 0;
  P.want_pf = 0;
  return launch_single(P, st);
}

}  // namespace skew
