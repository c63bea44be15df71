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
#include <stdlib.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_internal.h"

namespace skew {

constexpr int BNB = 64;        // largest panel width of the multi-launch path
constexpr int PNB_MAX = 128;   // largest panel width of the persistent kernel
constexpr int SYM_ROWS = 256;  // rows per sym CTA (one per thread)
constexpr int FIN_ROWS = 64;   // rows per fin CTA (4 threads per row)
constexpr int PF_ROWS = 16;    // persistent kernel, phase B: smallest row block
constexpr int UPD_T = 64;      // update tile edge
constexpr int TAIL = 128;      // columns left to the one-CTA kernel

struct BlockedWs {
  double* W;      // n x PNB_MAX, column-major, ld n (rows indexed globally)
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
  const int max_fintiles = (n + PF_ROWS - 1) / PF_ROWS;  // covers FIN_ROWS row tiles too
  return (size_t)n * PNB_MAX + (size_t)max_chunks * n + (size_t)max_symtiles * 2 * BNB + max_fintiles + 3 * (size_t)n +
         8;
}

static BlockedWs carve_ws(double* base, int n) {
  BlockedWs w;
  w.max_chunks = 64;
  w.max_symtiles = (n + SYM_ROWS - 1) / SYM_ROWS;
  w.max_fintiles = (n + PF_ROWS - 1) / PF_ROWS;
  double* p = base;
  w.W = p;
  p += (size_t)n * PNB_MAX;
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
  // panel dot products u1 = W_p^T v, u2 = A_p^T v over this tile's rows: dot d
  // goes to chunk CTA d mod nchunk; each warp covers 32 rows of the tile.
  if (i > 0) {
    __shared__ double svr[SYM_ROWS];
    __shared__ double sred[8][8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rb = r0 + tile * SYM_ROWS;
    const int rr = rb + threadIdx.x;
    svr[threadIdx.x] = (rr < n) ? vval(A, lda, c, rr, scale, tau) : 0.0;
    __syncthreads();
    const int ndots = 2 * i;
    for (int d0 = ch * 8; d0 < ndots; d0 += nchunk * 8) {
      // up to 8 dots at a time: warp w sums its 32 rows for each
      const int nd = min(8, ndots - d0);
      for (int q = 0; q < nd; q++) {
        const int d = d0 + q;
        const int j = d < i ? d : d - i;
        const double* col = (d < i) ? (ws.W + (size_t)j * n) : (A + (int64_t)(p + j) * lda);
        const double x = (rr < n) ? col[rr] * svr[threadIdx.x] : 0.0;
        const double sw = warp_sum(x);
        if (lane == 0) sred[q][w] = sw;
      }
      __syncthreads();
      if ((int)threadIdx.x < nd) {
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q++) acc += sred[threadIdx.x][q];
        ws.upart[(size_t)tile * 2 * BNB + d0 + threadIdx.x] = acc;
      }
      __syncthreads();
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
  // 1. u1, u2: sum the per-tile partials in a fixed order (two threads per dot)
  {
    __shared__ double uhalf[2][2 * BNB];
    const int d = tid & 127, half = tid >> 7;
    if (d < 2 * i) {
      double s = 0.0;
      for (int t = half; t < nsymtiles; t += 2) s += ws.upart[(size_t)t * 2 * BNB + d];
      uhalf[half][d] = s;
    }
    __syncthreads();
    if (tid < 2 * i) {
      const double s = uhalf[0][tid] + uhalf[1][tid];
      if (tid < i)
        su[tid] = s;
      else
        su[BNB + tid - i] = s;
    }
  }
  __syncthreads();
  // 2. W[c+1, i] redundantly in every CTA (needed by the column c+1 update)
  if (tid < 32) {
    const int lane = tid;
    double acc = 0.0;
    for (int j = lane; j < i; j += 32)
      acc = fma(A[r0 + (int64_t)(p + j) * lda], su[j], fma(-ws.W[(size_t)j * n + r0], su[BNB + j], acc));
    double y = 0.0;
    for (int q = lane; q < nchunk; q += 32) y += ws.ypart[(size_t)q * n + r0];
    acc = warp_sum(acc + y);
    if (lane == 0) sWrow[i] = tau * acc;
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
  if (valid)
    for (int q = g; q < nchunk; q += 4) y += ws.ypart[(size_t)q * n + row];
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
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
  if (tid < 32) {
    double ss = 0.0;
    for (int t = tid; t < (int)gridDim.x; t += 32) ss += ((volatile double*)ws.sspart)[t];
    ss = warp_sum(ss);
    if (tid != 0) return;
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
// Panels of nb columns (at most BNB).
cudaError_t blocked_hessenberg(double* A, int64_t lda, int n, double* tau, double* ev, int* info, double* wsbase,
                               int sms, int nb, cudaStream_t st) {
  BlockedWs ws = carve_ws(wsbase, n);
  nb = std::max(1, std::min(BNB, nb));
  cudaError_t e = cudaMemsetAsync(ws.ticket, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  int p = 0;
  if (n - p > TAIL) {
    col0_kernel<<<1, 256, 0, st>>>(A, lda, n, 0, ws.scal, ev, tau);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  while (n - p > TAIL) {
    // panel columns p .. p+nbp-1; keep at least TAIL columns for the tail
    const int nbp = min(nb, n - TAIL - p);
    for (int i = 0; i < nbp; i++) {
      const int c = p + i;
      const int m = n - (c + 1);
      const int symtiles = (m + SYM_ROWS - 1) / SYM_ROWS;
      int nchunk = max((2 * sms + symtiles - 1) / symtiles, (m + 511) / 512);  // chunk <= 512 (sv stage)
      nchunk = max(1, min(nchunk, min(ws.max_chunks, (m + 63) / 64)));          // chunk >= 64
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


// ===========================================================================
// Persistent variant: one cooperative launch runs every panel.  One CTA per SM;
// the phases of a panel column are separated by a grid barrier instead of a
// kernel boundary:
//   A  v staged in shared memory; warps take work items from an atomic counter:
//      the 2i panel dot products (one warp per dot over all rows, so u1/u2 are
//      complete without partial sums) and the (32-row, column-chunk) tiles of
//      y = A22 v (partial sums per chunk, summed in a fixed order in B).
//   B  row blocks: v into column c, W[:, i], the update of column c+1 and the
//      norm partials of column c+1.
//   then every CTA builds reflector c+1 itself from the norm partials (same data,
//   same order, so all CTAs agree) and no third barrier is needed.
// After a panel, D applies the trailing update tile by tile (atomic counter).
// Everything another CTA may have written during the kernel is read with
// L2-only loads (__ldcg): L1 is not coherent across SMs inside one launch.
// Grid barriers spin on a generation counter with a bounded number of polls;
// on timeout the kernel records an error and every CTA returns.
// ===========================================================================
constexpr int P_NT = 256;
constexpr int P_NW = P_NT / 32;
constexpr long long BAR_POLL_LIMIT = 1LL << 22;  // default: x ~1 us per poll (L2 read + sleep): ~4 s

struct PersistParams {
  double* A;
  int64_t lda;
  int n, pend;  // panels cover reflector columns [0, pend)
  int nb;       // panel width (<= the kernel's NBC)
  double* tau;
  double* ev;
  double* W;       // n x nb
  double* ypart;   // maxck x n
  double* u;       // 2 * NBC (u1, then u2 at NBC)
  double* sspart;  // row-block norm partials
  unsigned* sync;  // [0] barrier count, [1] barrier generation, [2] item counter
  int* err;
  int maxck;
  int items_per_warp;  // matvec tiles per warp and column (chunk count)
  long long poll_limit;  // polls before a grid barrier gives up
  int skip_cta;          // >= 0: this CTA never arrives (the waits run out: a test of the timeout)
};

__device__ __forceinline__ double ldg2(const double* p) { return __ldcg(p); }

// Grid barrier; false if it gave up (error recorded) or another CTA did.
__device__ bool gsync(const PersistParams& P) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = P.sync + 1;
    volatile int* err = P.err;
    const unsigned g = *gen;
    __threadfence();
    int ok = 1;
    if ((int)blockIdx.x == P.skip_cta) {
      // no arrival: the others give up after poll_limit polls; wait (bounded) for that
      long long it = 0;
      while (!*err && ++it <= P.poll_limit) __nanosleep(100);
      ok = 0;
    } else if (atomicAdd(P.sync, 1u) == gridDim.x - 1) {
      atomicExch(P.sync, 0u);
      __threadfence();
      atomicAdd(P.sync + 1, 1u);
    } else {
      long long it = 0;
      while (*gen == g) {
        if (*err) {
          ok = 0;
          break;
        }
        if (++it > P.poll_limit) {
          atomicExch(P.err, 1);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    s_ok = ok && !*err;
  }
  __syncthreads();
  return s_ok != 0;
}

struct Refl3 {
  double beta, tau, scale;
};

// Reflector of column c from its entries, computed by the whole CTA.
__device__ Refl3 refl_from_column(const PersistParams& P, int c, double* red) {
  const int n = P.n;
  const double* col = P.A + (int64_t)c * P.lda;
  double part = 0.0;
  for (int r = c + 2 + threadIdx.x; r < n; r += P_NT) {
    const double x = ldg2(col + r);
    part = fma(x, x, part);
  }
  const double ss = block_sum<P_NW>(part, red);
  double xn = -1.0;
  if (ss_needs_scaling(ss)) {
    double mx = 0.0;
    for (int r = c + 2 + threadIdx.x; r < n; r += P_NT) mx = fmax(mx, fabs(ldg2(col + r)));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __shared__ double rm[P_NW];
    if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = 0.0;
    for (int q = 0; q < P_NW; q++) mx = fmax(mx, rm[q]);
    double qq = 0.0;
    if (mx > 0.0)
      for (int r = c + 2 + threadIdx.x; r < n; r += P_NT) {
        const double x = ldg2(col + r) / mx;
        qq = fma(x, x, qq);
      }
    qq = block_sum<P_NW>(qq, red);
    xn = mx * sqrt(qq);
  }
  __shared__ Refl3 s_R;
  if (threadIdx.x == 0) {
    const Reflector R = make_reflector(ldg2(col + c + 1), ss, xn);
    s_R = Refl3{R.beta, R.tau, R.scale};
  }
  __syncthreads();
  const Refl3 R = s_R;
  __syncthreads();
  return R;
}

// One 64 x 64 lower tile of the trailing update (same arithmetic as upd_kernel).
__device__ void upd_tile(double* __restrict__ A, int64_t lda, int n, int p, int nbp, int q, const double* Wb, int t,
                         double* sbuf) {
  constexpr int KC = 16;
  double (*sVR)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf);
  double (*sWR)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + KC * UPD_T);
  double (*sVC)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + 2 * KC * UPD_T);
  double (*sWC)[UPD_T] = reinterpret_cast<double (*)[UPD_T]>(sbuf + 3 * KC * UPD_T);
  double (*sT)[UPD_T + 1] = reinterpret_cast<double (*)[UPD_T + 1]>(sbuf);
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
    __syncthreads();
    for (int idx = threadIdx.x; idx < KC * UPD_T; idx += P_NT) {
      const int kk = idx / UPD_T, rr = idx - kk * UPD_T;
      double vr = 0.0, wr = 0.0, vc = 0.0, wc = 0.0;
      if (kk < kc) {
        const int l = k0 + kk;
        const int gr = R0 + rr, gc = C0 + rr;
        if (gr < n) {
          vr = ldg2(A + gr + (int64_t)(p + l) * lda);
          wr = ldg2(Wb + (size_t)l * n + gr);
        }
        if (gc < n) {
          vc = ldg2(A + gc + (int64_t)(p + l) * lda);
          wc = ldg2(Wb + (size_t)l * n + gc);
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
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int rr = tx + 16 * a, cc = ty + 16 * b;
      const int gr = R0 + rr, gc = C0 + cc;
      double val = 0.0;
      if (gr < n && gc < n && gr > gc) {
        double* pa = A + gr + (int64_t)gc * lda;
        val = ldg2(pa) + acc[a][b];
        *pa = val;
      }
      sT[rr][cc] = val;
    }
  __syncthreads();
  for (int idx = threadIdx.x; idx < UPD_T * UPD_T; idx += P_NT) {
    const int rr = idx / UPD_T, cc = idx - rr * UPD_T;
    const int gr = R0 + rr, gc = C0 + cc;
    if (gr < n && gc < n && gr > gc) A[gc + (int64_t)gr * lda] = neg(sT[rr][cc]);
  }
  __syncthreads();
}

// Phase B rows: W[:, i], v into column c, the deferred update of column c+1 and the
// norm partials of its rows below the subdiagonal.  Blocks of 256 / TPR rows, TPR
// threads per row; a thread's panel terms j = g + TPR t are loaded once and used
// both for W and for the column update.
template <int TPR, int NBC>
__device__ void rows_phase(const PersistParams& P, double* A, int64_t lda, int n, int p, int c, int i, int nck,
                           bool last, const Refl3& R, const double* psm, const double* su, const double* sWrow,
                           const double* sArow, double* red) {
  constexpr int ROWS = P_NT / TPR;
  constexpr int NJ = NBC / TPR;
  const int tid = threadIdx.x;
  const int m = n - c - 1;
  const int nfb = (m + ROWS - 1) / ROWS;
  for (int fb = blockIdx.x; fb < nfb; fb += gridDim.x) {
    const int row = c + 1 + fb * ROWS + tid / TPR;
    const int g = tid % TPR;
    const bool valid = row < n;
    double aj[NJ], wj[NJ];
#pragma unroll
    for (int t = 0; t < NJ; t++) {
      const int j = g + TPR * t;
      aj[t] = 0.0;
      wj[t] = 0.0;
      if (valid && j < i) {
        aj[t] = ldg2(A + row + (int64_t)(p + j) * lda);
        wj[t] = ldg2(P.W + (size_t)j * n + row);
      }
    }
    double vr = 0.0, acc = 0.0;
    if (valid) {
      vr = psm[row];
      double y0 = 0.0, y1 = 0.0;
      int q = g;
      for (; q + TPR < nck; q += 2 * TPR) {
        y0 += ldg2(P.ypart + (size_t)q * n + row);
        y1 += ldg2(P.ypart + (size_t)(q + TPR) * n + row);
      }
      if (q < nck) y0 += ldg2(P.ypart + (size_t)q * n + row);
      acc = y0 + y1;
#pragma unroll
      for (int t = 0; t < NJ; t++) {
        const int j = g + TPR * t;
        if (j < i) acc = fma(aj[t], su[j], fma(-wj[t], su[NBC + j], acc));
      }
    }
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    double wri = R.tau * acc;
    if (row == c + 1) wri = sWrow[i];
    if (valid && g == 0) {
      P.W[(size_t)i * n + row] = wri;
      A[row + (int64_t)c * lda] = vr;
    }
    double ssp = 0.0, uu = 0.0;
    const bool doupd = valid && !last && row >= c + 2;
    if (doupd) {
#pragma unroll
      for (int t = 0; t < NJ; t++) {
        const int j = g + TPR * t;
        if (j < i) uu = fma(aj[t], sWrow[j], fma(-wj[t], sArow[j], uu));
      }
      if (i % TPR == g) uu = fma(vr, sWrow[i], fma(-wri, sArow[i], uu));
    }
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) uu += __shfl_xor_sync(0xffffffffu, uu, o);
    if (doupd && g == 0) {
      const double anew = ldg2(A + row + (int64_t)(c + 1) * lda) + uu;
      A[row + (int64_t)(c + 1) * lda] = anew;
      if (row >= c + 3) ssp = anew * anew;
    }
    const double sb = block_sum<P_NW>(ssp, red);
    if (tid == 0) P.sspart[fb] = sb;
  }
}

// NBC: compiled panel-width bound (64 or 128); the panels are P.nb <= NBC wide.
template <int NBC>
__global__ void __launch_bounds__(P_NT, 2) persist_kernel(PersistParams P) {
  extern __shared__ __align__(16) double psm[];  // v stage (n doubles) | update tile buffers
  __shared__ double red[P_NW];
  __shared__ double su[2 * NBC];
  __shared__ double sWrow[NBC + 1], sArow[NBC + 1];
  __shared__ int s_item, s_scal;
  __shared__ Refl3 s_R3;
  const int n = P.n;
  const int64_t lda = P.lda;
  double* A = P.A;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int nwarps = gridDim.x * P_NW;
  unsigned item_base = 0;  // running base of the shared item counter

  Refl3 R = refl_from_column(P, 0, red);
  if (blockIdx.x == 0 && tid == 0) {
    P.ev[0] = R.beta;
    P.tau[0] = R.tau;
  }
  int p = 0;
  while (p < P.pend) {
    const int nbp = min(P.nb, P.pend - p);
    for (int i = 0; i < nbp; i++) {
      const int c = p + i, m = n - c - 1;
      // ---- A: stage v, then items from the shared counter
      for (int j = c + 1 + tid; j < n; j += P_NT)
        psm[j] = (R.tau == 0.0) ? 0.0 : (j == c + 1 ? 1.0 : ldg2(A + j + (int64_t)c * lda) * R.scale);
      __syncthreads();
      const int nrt = (m + 31) >> 5;
      int nck = max(1, min((P.items_per_warp * nwarps + nrt - 1) / nrt, (m + 31) >> 5));
      nck = min(nck, P.maxck);
      const int chunk = (m + nck - 1) / nck;
      nck = (m + chunk - 1) / chunk;
      const int ndots = 2 * i;
      const unsigned nitems = (unsigned)(ndots + nrt * nck);
      for (;;) {
        unsigned it = 0;
        if (lane == 0) it = atomicAdd(P.sync + 2, 1u) - item_base;
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= nitems) break;
        if ((int)it < ndots) {
          const int d = (int)it;
          const int j = d < i ? d : d - i;
          const double* col = (d < i) ? (P.W + (size_t)j * n) : (A + (int64_t)(p + j) * lda);
          double a0 = 0.0, a1 = 0.0;
          int r = c + 1 + lane;
          for (; r + 32 < n; r += 64) {
            a0 = fma(ldg2(col + r), psm[r], a0);
            a1 = fma(ldg2(col + r + 32), psm[r + 32], a1);
          }
          if (r < n) a0 = fma(ldg2(col + r), psm[r], a0);
          const double s = warp_sum(a0 + a1);
          if (lane == 0) P.u[d < i ? d : NBC + j] = s;
        } else {
          const int qq = (int)it - ndots;
          const int rt = qq / nck, ck = qq - rt * nck;
          const int r = c + 1 + rt * 32 + lane;
          const int cb = c + 1 + ck * chunk, ce = min(n, cb + chunk);
          if (r < n) {
            const double* row = A + r;
            double a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, a5 = 0, a6 = 0, a7 = 0;
            int j = cb;
            for (; j + 7 < ce; j += 8) {
              const double w0 = ldg2(row + (int64_t)j * lda), w1 = ldg2(row + (int64_t)(j + 1) * lda),
                           w2 = ldg2(row + (int64_t)(j + 2) * lda), w3 = ldg2(row + (int64_t)(j + 3) * lda),
                           w4 = ldg2(row + (int64_t)(j + 4) * lda), w5 = ldg2(row + (int64_t)(j + 5) * lda),
                           w6 = ldg2(row + (int64_t)(j + 6) * lda), w7 = ldg2(row + (int64_t)(j + 7) * lda);
              a0 = fma(w0, psm[j], a0);
              a1 = fma(w1, psm[j + 1], a1);
              a2 = fma(w2, psm[j + 2], a2);
              a3 = fma(w3, psm[j + 3], a3);
              a4 = fma(w4, psm[j + 4], a4);
              a5 = fma(w5, psm[j + 5], a5);
              a6 = fma(w6, psm[j + 6], a6);
              a7 = fma(w7, psm[j + 7], a7);
            }
            for (; j < ce; j++) a0 = fma(ldg2(row + (int64_t)j * lda), psm[j], a0);
            P.ypart[(size_t)ck * n + r] = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
          }
        }
      }
      item_base += nitems + (unsigned)nwarps;  // every warp took exactly one failing ticket
      if (!gsync(P)) return;
      // ---- B: rows
      const bool last = (i == nbp - 1);
      for (int d = tid; d < 2 * i; d += P_NT) su[d < i ? d : NBC + d - i] = ldg2(P.u + (d < i ? d : NBC + d - i));
      __syncthreads();
      if (w == 0) {
        const int r0 = c + 1;
        double acc = 0.0;
        for (int j = lane; j < i; j += 32)
          acc = fma(ldg2(A + r0 + (int64_t)(p + j) * lda), su[j], fma(-ldg2(P.W + (size_t)j * n + r0), su[NBC + j], acc));
        for (int q = lane; q < nck; q += 32) acc += ldg2(P.ypart + (size_t)q * n + r0);
        acc = warp_sum(acc);
        if (lane == 0) sWrow[i] = R.tau * acc;
        for (int j = lane; j < i; j += 32) {
          sWrow[j] = ldg2(P.W + (size_t)j * n + r0);
          sArow[j] = ldg2(A + r0 + (int64_t)(p + j) * lda);
        }
        if (lane == 0) sArow[i] = (R.tau == 0.0) ? 0.0 : 1.0;
      }
      __syncthreads();
      // rows in blocks, TPR threads per row: as many threads per row as keeps every
      // block in one round of CTAs (16 at small m, fewer at large m; at least 8 for
      // 128-wide panels, whose 4-thread rows would hold 32 panel terms per thread)
      int nfb;
      {
        const int G = gridDim.x;
        if ((m + 15) / 16 <= G) {
          nfb = (m + 15) / 16;
          rows_phase<16, NBC>(P, A, lda, n, p, c, i, nck, last, R, psm, su, sWrow, sArow, red);
        } else if ((m + 31) / 32 <= G || NBC > 64) {
          nfb = (m + 31) / 32;
          rows_phase<8, NBC>(P, A, lda, n, p, c, i, nck, last, R, psm, su, sWrow, sArow, red);
        } else {
          nfb = (m + 63) / 64;
          rows_phase<4, NBC>(P, A, lda, n, p, c, i, nck, last, R, psm, su, sWrow, sArow, red);
        }
      }
      if (!gsync(P)) return;
      if (!last) {
        // reflector c+1, identically in every CTA
        const int c1 = c + 1;
        // one lane forms it (a warp-wide FP64 instruction costs the pipe the same
        // with one lane as with 32); the others read it from shared memory
        if (w == 0) {
          double ss = 0.0;
          for (int t = lane; t < nfb; t += 32) ss += ldg2(P.sspart + t);
          ss = warp_sum(ss);
          if (lane == 0) {
            s_scal = ss_needs_scaling(ss) ? 1 : 0;
            if (!s_scal) {
              const Reflector Rf = make_reflector(ldg2(A + (c1 + 1) + (int64_t)c1 * lda), ss, -1.0);
              s_R3 = Refl3{Rf.beta, Rf.tau, Rf.scale};
            }
          }
        }
        __syncthreads();
        if (s_scal)
          R = refl_from_column(P, c1, red);
        else
          R = s_R3;
        __syncthreads();
        if (blockIdx.x == 0 && tid == 0) {
          P.ev[c1] = R.beta;
          P.tau[c1] = R.tau;
        }
      }
    }
    // ---- D: trailing update, tiles from the shared counter
    const int q = p + nbp;
    const int mt = (n - q + UPD_T - 1) / UPD_T;
    const unsigned ntiles = (unsigned)(mt * (mt + 1) / 2);
    for (;;) {
      if (tid == 0) s_item = (int)(atomicAdd(P.sync + 2, 1u) - item_base);
      __syncthreads();
      const unsigned t = (unsigned)s_item;
      __syncthreads();
      if (t >= ntiles) break;
      upd_tile(A, lda, n, p, nbp, q, P.W, (int)t, psm);
    }
    item_base += ntiles + gridDim.x;  // one failing ticket per CTA
    if (!gsync(P)) return;
    p = q;
    if (p < P.pend) {
      R = refl_from_column(P, p, red);
      if (blockIdx.x == 0 && tid == 0) {
        P.ev[p] = R.beta;
        P.tau[p] = R.tau;
      }
    }
  }
}

size_t persist_ws_extra_doubles() { return 2 * PNB_MAX + 8; }

// info <- SKEW_TIMEOUT if a grid barrier of the persistent kernel gave up.
__global__ void merge_err_kernel(const int* err, int* info) {
  if (*err && info) *info = SKEW_TIMEOUT;
}

// Persistent driver; returns cudaErrorNotSupported when the device cannot
// co-schedule one CTA per SM (the caller then uses the multi-launch path).
cudaError_t blocked_hessenberg_persistent(double* A, int64_t lda, int n, double* tau, double* ev, int* info,
                                          double* wsbase, int sms, int* err_dev, const Tuning& T, cudaStream_t st) {
  BlockedWs ws = carve_ws(wsbase, n);
  double* extra = wsbase + blocked_ws_doubles(n);  // u (2*PNB_MAX), 4 sync words, error flag
  int* err_dev_local = (int*)(extra + 2 * PNB_MAX + 4);
  if (!err_dev) err_dev = err_dev_local;
  // panel width: the tuning key persist_nb (setnb, hessenberg.jl:133-142, decides it
  // by rule); widths above 64 run the instantiation with 128-entry panel arrays
  const int nb = std::max(8, std::min(PNB_MAX, T.persist_nb));
  const void* kern = nb <= 64 ? (const void*)persist_kernel<64> : (const void*)persist_kernel<128>;
  const size_t smem = max((size_t)n * sizeof(double), (size_t)UPD_T * (UPD_T + 1) * sizeof(double));
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, P_NT, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorNotSupported;
  // Two CTAs per SM hide more load latency on large matrices; below that, the two
  // grid barriers per column cost more than the extra CTAs bring.
  // The tuning keys persist_ctas / persist_tail replace the grid and the columns
  // left to the one-CTA kernel.
  // measured on GB300: one CTA per SM is 14-22 % faster for n <= 2048, two per
  // SM break even at n = 4096
  int grid = sms * ((occ >= 2 && n > 3072) ? 2 : 1);
  int tail = TAIL;
  if (T.persist_ctas > 0) grid = std::max(1, std::min(sms * occ, T.persist_ctas));
  if (T.persist_tail > 0) tail = std::max(32, std::min(TAIL, T.persist_tail));
  PersistParams P;
  P.A = A;
  P.lda = lda;
  P.n = n;
  P.pend = n - tail;
  P.nb = nb;
  P.tau = tau;
  P.ev = ev;
  P.W = ws.W;
  P.ypart = ws.ypart;
  P.u = extra;
  P.sspart = ws.sspart;
  P.sync = (unsigned*)(extra + 2 * PNB_MAX);
  P.err = err_dev;
  P.maxck = ws.max_chunks;
  // matvec tiles per warp and column: measured on GB300 at n = 8192, 8 gives 932 ms,
  // 4 945 ms, 2 981 ms (more, smaller tiles shorten the wait for the last ones)
  P.items_per_warp = std::max(1, std::min(16, T.persist_items));
  P.poll_limit = T.wait_polls > 0 ? T.wait_polls : BAR_POLL_LIMIT;
  P.skip_cta = T.wait_skip_cta;
  e = cudaMemsetAsync(P.sync, 0, 4 * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(err_dev, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (P.pend > 0) {
    void* args[] = {&P};
    e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(P_NT), args, smem, st);
    if (e != cudaSuccess) return e;
  }
  SingleParams S;
  const int p = P.pend > 0 ? P.pend : 0;
  S.A = A + p + (int64_t)p * lda;
  S.lda = lda;
  S.n = n - p;
  S.G = nullptr;
  S.ldg = 0;
  S.logpf = nullptr;
  S.sign = nullptr;
  S.ev = ev + p;
  S.tau = tau + p;
  S.info = info;
  S.check = 0;
  S.want_pf = 0;
  e = launch_single(S, st);
  if (e != cudaSuccess) return e;
  merge_err_kernel<<<1, 1, 0, st>>>(err_dev, info);
  return cudaGetLastError();
}

}  // namespace skew
