// Blocked ComplexF64 skew-Hermitian tridiagonalisation of one large matrix in one
// cooperative launch: the complex skewlatrd! panel (hessenberg.jl:92-131, with the
// alpha correction of :123-126) and the trailing update of skewblockedhess!
// (:158-166), A22 += V W^H - W V^H on the lower triangle, mirrored as -conj.
//
// Per panel column c (panel step i, panel start p):
//   A  v staged in shared memory.  Each warp takes a static share of the items: the
//      2i panel dots u1 = W^H v and u2 = V^H v (one warp per dot over all rows), and
//      (32-row, column-chunk) tiles of A22 v whose partial sums go to ypart; each
//      warp also writes its share of v^H (A22 v) to dpart.
//   B  every CTA sums dpart in a fixed order and forms the alpha correction without
//      a further reduction: with y = A22 v + V u1 - W u2,
//        v^H y = v^H (A22 v) + u2^H u1 - u1^H u2,   alpha = |tau|^2 conj(v^H y) / 2,
//      which equals tau (W^H v) / 2 for W = tau y (the reference's
//      tau * dot(W, v) / 2).  Row blocks then form W[:, i] = tau y + alpha v, store
//      v into column c, apply the deferred rank-2(i+1) update to column c+1 and
//      write the norm partials of its rows below the subdiagonal.
//   then every CTA builds reflector c+1 from the same partials in the same order.
// After a panel, D applies the trailing update on 64 x 64 lower tiles (complex
// register tiles), with the diagonal receiving only the imaginary part, as
// Omega - Omega^H does in the reference.
// Two grid barriers per column and one per panel, each a monotonic arrival
// counter polled with acquire loads and a bounded number of polls (error flag,
// every CTA returns, the call reports SKEW_TIMEOUT).  Data written by other CTAs
// during the launch is read through L2 (__ldcg).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_complex.cuh"
#include "skew_internal.h"

namespace skew {

namespace {

constexpr int ZP_NT = 256;
constexpr int ZP_NW = ZP_NT / 32;
constexpr int ZBNB = 32;   // largest panel width
constexpr int ZUT = 64;    // trailing-update tile edge
constexpr int ZKC = 8;     // panel columns per shared-memory stage of the update
constexpr int ZFIN = 16;   // smallest row block of phase B (sizes sspart)
constexpr int ZTAILP = 128;  // trailing columns left to the one-CTA kernel
constexpr long long ZP_POLL = 1LL << 24;  // default polls before a grid barrier gives up
constexpr int ZP_MAXWARPS = 16384;  // dpart slots: grid x 8 warps at most

struct ZRef {
  zc tau, scale;
  double beta;
};

// Reflector of (alpha, |x[2:]|), hessenberg.jl:26-44 complex branch (as zrefl).
__device__ ZRef zp_refl(zc alpha, double xnorm) {
  ZRef R;
  if (xnorm == 0.0 && alpha.re == 0.0 && alpha.im == 0.0) {
    R.tau = zc{0.0, 0.0};
    R.scale = zc{0.0, 0.0};
    R.beta = 0.0;
    return R;
  }
  const double h = hypot(hypot(alpha.re, alpha.im), xnorm);
  const double beta = (alpha.re > 0.0) ? neg(h) : h;
  const double rb = 1.0 / beta;
  R.beta = beta;
  R.tau = zc{1.0 - alpha.re * rb, neg(alpha.im * rb)};
  R.scale = zinv(zc{alpha.re - beta, alpha.im});
  return R;
}

__device__ __forceinline__ zc ldz(const zc* p) {
  const double2 v = __ldcg((const double2*)p);
  return zc{v.x, v.y};
}
__device__ __forceinline__ void stz(zc* p, zc x) { __stcg((double2*)p, make_double2(x.re, x.im)); }
__device__ __forceinline__ bool zzero(zc z) { return z.re == 0.0 && z.im == 0.0; }

__device__ __forceinline__ double zp_block_max(double x, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < ZP_NW; i++) s = fmax(s, red[i]);
  __syncthreads();
  return s;
}

}  // namespace

struct ZPersistParams {
  zc* A;
  int64_t lda;
  int n, pend;  // panels cover reflector columns [0, pend)
  int nb;       // panel width (<= ZBNB)
  zc* tau;
  double* ev;
  zc* W;          // n x ZBNB, column j at W + j * n
  zc* ypart;      // maxck x n
  zc* dpart;      // maxitems
  zc* u;          // 2 * ZBNB: u1 then u2
  double* sspart; // row-block norm partials
  unsigned* sync; // [0] barrier arrivals, [1] work items
  int* err;
  int maxck;
  int items_per_warp;  // matvec tiles per warp and column (chunk count)
  long long poll_limit;  // polls before a grid barrier gives up
  int skip_cta;          // >= 0: this CTA never arrives (a test of the timeout path)
};

namespace {

__device__ bool zp_gsync(const ZPersistParams& P) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && (int)blockIdx.x == P.skip_cta) {
    // no arrival: the others give up after poll_limit polls; wait (bounded) for that
    volatile int* verr = P.err;
    long long it = 0;
    while (!*verr && ++it <= P.poll_limit) __nanosleep(32);
    s_ok = 0;
  } else if (threadIdx.x == 0) {
    volatile int* verr = P.err;
    __threadfence();
    const unsigned old = atomicAdd(P.sync, 1u);
    const unsigned target = (old / gridDim.x + 1) * gridDim.x;
    int ok = 1;
    long long it = 0;
    for (;;) {
      unsigned cur;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(P.sync) : "memory");
      if ((int)(cur - target) >= 0) break;
      if ((++it & 63) == 0) {
        if (*verr) {
          ok = 0;
          break;
        }
        if (it > P.poll_limit) {
          atomicExch(P.err, 1);
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

// Reflector of column c from its entries, by the whole CTA (identical in every CTA).
__device__ ZRef zp_refl_from_column(const ZPersistParams& P, int c, double* red) {
  const int n = P.n;
  const zc* col = P.A + (int64_t)c * P.lda;
  double part = 0.0;
  for (int r = c + 2 + threadIdx.x; r < n; r += ZP_NT) {
    const zc x = ldz(col + r);
    part = fma(x.re, x.re, fma(x.im, x.im, part));
  }
  const double ss = block_sum<ZP_NW>(part, red);
  double xn = sqrt(ss);
  if (ss_needs_scaling(ss)) {
    double mx = 0.0;
    for (int r = c + 2 + threadIdx.x; r < n; r += ZP_NT) {
      const zc x = ldz(col + r);
      mx = fmax(mx, fmax(fabs(x.re), fabs(x.im)));
    }
    mx = zp_block_max(mx, red);
    double qq = 0.0;
    if (mx > 0.0) {
      const double inv = 1.0 / mx;
      for (int r = c + 2 + threadIdx.x; r < n; r += ZP_NT) {
        const zc x = ldz(col + r);
        const double a = x.re * inv, b = x.im * inv;
        qq = fma(a, a, fma(b, b, qq));
      }
    }
    qq = block_sum<ZP_NW>(qq, red);
    xn = mx * sqrt(qq);
  }
  // one thread forms the reflector (a warp-wide FP64 instruction costs the same
  // with one lane as with 32), the others read it from shared memory
  __shared__ ZRef s_R;
  if (threadIdx.x == 0) s_R = zp_refl(ldz(col + c + 1), xn);
  __syncthreads();
  const ZRef R = s_R;
  __syncthreads();
  return R;
}

// One 64 x 64 lower tile t of the trailing update A[q:, q:] += V W^H - W V^H,
// V = A[:, p : p + nbp], W = P.W.  16 x 16 threads, 4 x 4 complex entries each.
__device__ void zp_upd_tile(const ZPersistParams& P, int p, int nbp, int q, int t, zc* sbuf) {
  const int n = P.n;
  const int64_t lda = P.lda;
  zc* A = P.A;
  zc (*sVR)[ZUT] = reinterpret_cast<zc (*)[ZUT]>(sbuf);
  zc (*sWR)[ZUT] = reinterpret_cast<zc (*)[ZUT]>(sbuf + ZKC * ZUT);
  zc (*sVC)[ZUT] = reinterpret_cast<zc (*)[ZUT]>(sbuf + 2 * ZKC * ZUT);
  zc (*sWC)[ZUT] = reinterpret_cast<zc (*)[ZUT]>(sbuf + 3 * ZKC * ZUT);
  zc (*sT)[ZUT + 1] = reinterpret_cast<zc (*)[ZUT + 1]>(sbuf);
  int ti = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= t) ti++;
  while (ti * (ti + 1) / 2 > t) ti--;
  const int tj = t - ti * (ti + 1) / 2;
  const int R0 = q + ti * ZUT, C0 = q + tj * ZUT;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double ar[4][4], ai[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) ar[a][b] = ai[a][b] = 0.0;
  for (int k0 = 0; k0 < nbp; k0 += ZKC) {
    const int kc = min(ZKC, nbp - k0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < ZKC * ZUT; idx += ZP_NT) {
      const int kk = idx / ZUT, rr = idx - kk * ZUT;
      zc vr{0.0, 0.0}, wr{0.0, 0.0}, vc{0.0, 0.0}, wc{0.0, 0.0};
      if (kk < kc) {
        const int l = k0 + kk;
        const int gr = R0 + rr, gc = C0 + rr;
        if (gr < n) {
          vr = ldz(A + gr + (int64_t)(p + l) * lda);
          wr = ldz(P.W + (size_t)l * n + gr);
        }
        if (gc < n) {
          vc = ldz(A + gc + (int64_t)(p + l) * lda);
          wc = ldz(P.W + (size_t)l * n + gc);
        }
      }
      sVR[kk][rr] = vr;
      sWR[kk][rr] = wr;
      sVC[kk][rr] = vc;
      sWC[kk][rr] = wc;
    }
    __syncthreads();
    for (int kk = 0; kk < kc; kk++) {
      zc vR[4], wR[4], vC[4], wC[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        vR[a] = sVR[kk][tx + 16 * a];
        wR[a] = sWR[kk][tx + 16 * a];
        vC[a] = sVC[kk][ty + 16 * a];
        wC[a] = sWC[kk][ty + 16 * a];
      }
      // acc += vR conj(wC) - wR conj(vC)
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          ar[a][b] = fma(vR[a].re, wC[b].re, fma(vR[a].im, wC[b].im, fma(-wR[a].re, vC[b].re,
                                                                           fma(-wR[a].im, vC[b].im, ar[a][b]))));
          ai[a][b] = fma(vR[a].im, wC[b].re, fma(-vR[a].re, wC[b].im, fma(-wR[a].im, vC[b].re,
                                                                            fma(wR[a].re, vC[b].im, ai[a][b]))));
        }
    }
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int rr = tx + 16 * a, cc = ty + 16 * b;
      const int gr = R0 + rr, gc = C0 + cc;
      zc val{0.0, 0.0};
      if (gr < n && gc < n && gr >= gc) {
        zc* pa = A + gr + (int64_t)gc * lda;
        val = ldz(pa);
        if (gr == gc) {
          val.im += ai[a][b];  // Omega - Omega^H on the diagonal: imaginary only
        } else {
          val.re += ar[a][b];
          val.im += ai[a][b];
        }
        stz(pa, val);
      }
      sT[rr][cc] = val;
    }
  __syncthreads();
  for (int idx = threadIdx.x; idx < ZUT * ZUT; idx += ZP_NT) {
    const int rr = idx / ZUT, cc = idx - rr * ZUT;
    const int gr = R0 + rr, gc = C0 + cc;
    if (gr < n && gc < n && gr > gc) {
      const zc x = sT[rr][cc];
      stz(A + gc + (int64_t)gr * lda, zc{neg(x.re), x.im});
    }
  }
  __syncthreads();
}

}  // namespace

// Phase B rows: blocks of ZP_NT / TPR rows, TPR threads per row (see the kernel).
template <int TPR>
__device__ void zp_rows_phase(const ZPersistParams& P, zc* A, int64_t lda, int n, int p, int c, int i, int nck,
                              bool last, const ZRef& R, const zc alpha, const zc* vs, const zc* su, const zc* sWrow,
                              const zc* sArow, double* red) {
  constexpr int ROWS = ZP_NT / TPR;
  const int tid = threadIdx.x;
  const int m = n - c - 1;
  const int nfb = (m + ROWS - 1) / ROWS;
  for (int fb = blockIdx.x; fb < nfb; fb += gridDim.x) {
    const int row = c + 1 + fb * ROWS + tid / TPR;
    const int g = tid % TPR;
    const bool valid = row < n;
    // this thread's panel terms j = g + TPR t: loaded once, used for y and for
    // the deferred update of column c+1
    constexpr int NJ = ZBNB / TPR;
    zc aj[NJ], wj[NJ];
#pragma unroll
    for (int t = 0; t < NJ; t++) {
      const int j = g + TPR * t;
      aj[t] = zc{0.0, 0.0};
      wj[t] = zc{0.0, 0.0};
      if (valid && j < i) {
        aj[t] = ldz(A + row + (int64_t)(p + j) * lda);
        wj[t] = ldz(P.W + (size_t)j * n + row);
      }
    }
    zc vr{0.0, 0.0}, acc{0.0, 0.0};
    if (valid) {
      vr = vs[row];
      zc y0{0.0, 0.0}, y1{0.0, 0.0};
      int q2 = g;
      for (; q2 + TPR < nck; q2 += 2 * TPR) {
        y0 = zadd(y0, ldz(P.ypart + (size_t)q2 * n + row));
        y1 = zadd(y1, ldz(P.ypart + (size_t)(q2 + TPR) * n + row));
      }
      if (q2 < nck) y0 = zadd(y0, ldz(P.ypart + (size_t)q2 * n + row));
      acc = zadd(y0, y1);
#pragma unroll
      for (int t = 0; t < NJ; t++) {
        const int j = g + TPR * t;
        if (j < i) acc = zsub(zfma(aj[t], su[j], acc), zmul(wj[t], su[ZBNB + j]));
      }
    }
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) {
      acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
      acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
    }
    zc wri = zfma(alpha, vr, zmul(R.tau, acc));
    if (row == c + 1) wri = sWrow[i];
    if (valid && g == 0) {
      stz(P.W + (size_t)i * n + row, wri);
      stz(A + row + (int64_t)c * lda, vr);
    }
    // deferred update of column c+1 (rows c+1.., the diagonal included):
    // A[row, c+1] += sum_{j <= i} V[row, j] conj(W[c+1, j]) - W[row, j] conj(V[c+1, j])
    double ssp = 0.0;
    zc uu{0.0, 0.0};
    const bool doupd = valid && !last;
    if (doupd) {
#pragma unroll
      for (int t = 0; t < NJ; t++) {
        const int j = g + TPR * t;
        if (j < i) uu = zsub(zadd(uu, zmulc(aj[t], sWrow[j])), zmulc(wj[t], sArow[j]));
      }
      if (i % TPR == g) uu = zsub(zadd(uu, zmulc(vr, sWrow[i])), zmulc(wri, sArow[i]));
    }
#pragma unroll
    for (int o = 1; o < TPR; o <<= 1) {
      uu.re += __shfl_xor_sync(0xffffffffu, uu.re, o);
      uu.im += __shfl_xor_sync(0xffffffffu, uu.im, o);
    }
    if (doupd && g == 0) {
      zc* pa = A + row + (int64_t)(c + 1) * lda;
      zc anew = ldz(pa);
      if (row == c + 1) {
        anew.im += uu.im;  // the diagonal receives the imaginary part only
      } else {
        anew = zadd(anew, uu);
      }
      stz(pa, anew);
      if (row >= c + 3) ssp = fma(anew.re, anew.re, anew.im * anew.im);
    }
    const double sb = block_sum<ZP_NW>(ssp, red);
    if (tid == 0) P.sspart[fb] = sb;
  }
}

__global__ void __launch_bounds__(ZP_NT, 1) zpersist_kernel(ZPersistParams P) {
  extern __shared__ __align__(16) double zpsm_raw[];
  zc* vs = reinterpret_cast<zc*>(zpsm_raw);  // v stage (n complex) | update tile buffers
  __shared__ double red[ZP_NW];
  __shared__ zc su[2 * ZBNB];
  __shared__ zc sWrow[ZBNB + 1], sArow[ZBNB + 1];
  __shared__ double s_dot[2 * ZP_NW];
  __shared__ zc s_alpha, s_y1;
  __shared__ ZRef s_R;
  __shared__ int s_scal;
  __shared__ unsigned s_item;
  const int n = P.n;
  const int64_t lda = P.lda;
  zc* A = P.A;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int nwarps = gridDim.x * ZP_NW;
  const bool lead = blockIdx.x == 0 && tid == 0;
  unsigned item_base = 0;

  ZRef R = zp_refl_from_column(P, 0, red);
  if (lead) {
    P.ev[0] = R.beta;
    P.tau[0] = R.tau;
  }
  int p = 0;
  while (p < P.pend) {
    const int nbp = min(P.nb, P.pend - p);
    for (int i = 0; i < nbp; i++) {
      const int c = p + i, m = n - c - 1;
      const bool zero = zzero(R.tau);
      // ---- A: stage v, then a static share of the items per warp.  Warps are
      // numbered CTA-minor (consecutive items on different SMs); matvec tile q goes
      // to warp q mod nwarps, panel dot d to warp nwarps - 1 - d.  Each warp sums its
      // share of v^H (A22 v) over its tiles in order (deterministic).
      for (int j = c + 1 + tid; j < n; j += ZP_NT)
        vs[j] = zero ? zc{0.0, 0.0} : (j == c + 1 ? zc{1.0, 0.0} : zmul(ldz(A + j + (int64_t)c * lda), R.scale));
      __syncthreads();
      const int nrt = (m + 31) >> 5;
      int nck = max(1, min((P.items_per_warp * nwarps + nrt - 1) / nrt, (m + 31) >> 5));
      nck = min(nck, P.maxck);
      const int chunk = (m + nck - 1) / nck;
      nck = (m + chunk - 1) / chunk;
      const int ndots = 2 * i;
      const int nmv = nrt * nck;
      const int gw = w * gridDim.x + blockIdx.x;
      if (nwarps - 1 - gw < ndots) {  // u1_j = W[:, j]^H v, u2_j = V[:, j]^H v over rows c+1..
        const int d = nwarps - 1 - gw;
        const int j = d < i ? d : d - i;
        const zc* col = (d < i) ? (P.W + (size_t)j * n) : (A + (int64_t)(p + j) * lda);
        zc a0{0.0, 0.0}, a1{0.0, 0.0};
        int r = c + 1 + lane;
        for (; r + 32 < n; r += 64) {
          a0 = zfma(zconj(ldz(col + r)), vs[r], a0);
          a1 = zfma(zconj(ldz(col + r + 32)), vs[r + 32], a1);
        }
        if (r < n) a0 = zfma(zconj(ldz(col + r)), vs[r], a0);
        const double sr = warp_sum(a0.re + a1.re), si = warp_sum(a0.im + a1.im);
        if (lane == 0) P.u[d < i ? d : ZBNB + j] = zc{sr, si};
      }
      zc dl{0.0, 0.0};  // this lane's share of v^H (A22 v)
      for (int qq = gw; qq < nmv; qq += nwarps) {  // partial y = A22 v over (32 rows, column chunk)
        const int rt = qq / nck, ck = qq - rt * nck;
        const int r = c + 1 + rt * 32 + lane;
        const int cb = c + 1 + ck * chunk, ce = min(n, cb + chunk);
        if (r < n) {
          const zc* row = A + r;
          zc a0{0.0, 0.0}, a1{0.0, 0.0}, a2{0.0, 0.0}, a3{0.0, 0.0};
          int j = cb;
          for (; j + 3 < ce; j += 4) {
            const zc w0 = ldz(row + (int64_t)j * lda), w1 = ldz(row + (int64_t)(j + 1) * lda),
                     w2 = ldz(row + (int64_t)(j + 2) * lda), w3 = ldz(row + (int64_t)(j + 3) * lda);
            a0 = zfma(w0, vs[j], a0);
            a1 = zfma(w1, vs[j + 1], a1);
            a2 = zfma(w2, vs[j + 2], a2);
            a3 = zfma(w3, vs[j + 3], a3);
          }
          for (; j < ce; j++) a0 = zfma(ldz(row + (int64_t)j * lda), vs[j], a0);
          const zc acc = zadd(zadd(a0, a1), zadd(a2, a3));
          stz(P.ypart + (size_t)ck * n + r, acc);
          dl = zadd(dl, zcmul(vs[r], acc));  // conj(v_r) y_r
        }
      }
      {
        const double dr = warp_sum(dl.re), di = warp_sum(dl.im);
        if (lane == 0) P.dpart[gw] = zc{dr, di};
      }
      if (!zp_gsync(P)) return;

      // ---- B head: every CTA loads u, sums the warps' shares of v^H (A22 v) in a
      // fixed order, and warp 0 gathers row c+1 of V, W and y in the same round trip
      const bool last = (i == nbp - 1);
      for (int d = tid; d < 2 * i; d += ZP_NT) {
        const int slot = d < i ? d : ZBNB + d - i;
        su[slot] = ldz(P.u + slot);
      }
      {
        double dr = 0.0, di = 0.0;
        for (int q2 = tid; q2 < nwarps; q2 += ZP_NT) {
          const zc x = ldz(P.dpart + q2);
          dr += x.re;
          di += x.im;
        }
        dr = warp_sum(dr);
        di = warp_sum(di);
        if (lane == 0) {
          s_dot[w] = dr;
          s_dot[ZP_NW + w] = di;
        }
      }
      if (w == 0) {
        const int r0 = c + 1;
        for (int j = lane; j < i; j += 32) {
          sWrow[j] = ldz(P.W + (size_t)j * n + r0);
          sArow[j] = ldz(A + r0 + (int64_t)(p + j) * lda);
        }
        zc y1{0.0, 0.0};
        for (int q2 = lane; q2 < nck; q2 += 32) y1 = zadd(y1, ldz(P.ypart + (size_t)q2 * n + r0));
        y1.re = warp_sum(y1.re);
        y1.im = warp_sum(y1.im);
        if (lane == 0) s_y1 = y1;
      }
      __syncthreads();
      if (w == 0) {
        // v^H y = v^H (A22 v) + u2^H u1 - u1^H u2;  alpha = |tau|^2 conj(v^H y) / 2;
        // y_{c+1} = (A22 v)_{c+1} + sum_j (V[c+1, j] u1_j - W[c+1, j] u2_j)
        double hr = 0.0, hi = 0.0, er = 0.0, ei = 0.0;
        for (int j = lane; j < i; j += 32) {
          const zc u1 = su[j], u2 = su[ZBNB + j];
          const zc d = zsub(zcmul(u2, u1), zcmul(u1, u2));
          hr += d.re;
          hi += d.im;
          const zc e = zsub(zmul(sArow[j], u1), zmul(sWrow[j], u2));
          er += e.re;
          ei += e.im;
        }
        hr = warp_sum(hr);
        hi = warp_sum(hi);
        er = warp_sum(er);
        ei = warp_sum(ei);
        if (lane == 0) {
          for (int k = 0; k < ZP_NW; k++) {
            hr += s_dot[k];
            hi += s_dot[ZP_NW + k];
          }
          const double t2 = R.tau.re * R.tau.re + R.tau.im * R.tau.im;
          const zc alpha = zc{0.5 * t2 * hr, -0.5 * t2 * hi};
          s_alpha = alpha;
          const zc y1 = zadd(s_y1, zc{er, ei});
          sWrow[i] = zfma(alpha, vs[c + 1], zmul(R.tau, y1));
          sArow[i] = vs[c + 1];
        }
      }
      __syncthreads();
      const zc alpha = s_alpha;
      // rows: as many threads per row as keeps every block in one round of CTAs
      int nfb;
      if ((m + 15) / 16 <= (int)gridDim.x) {
        nfb = (m + 15) / 16;
        zp_rows_phase<16>(P, A, lda, n, p, c, i, nck, last, R, alpha, vs, su, sWrow, sArow, red);
      } else if ((m + 31) / 32 <= (int)gridDim.x) {
        nfb = (m + 31) / 32;
        zp_rows_phase<8>(P, A, lda, n, p, c, i, nck, last, R, alpha, vs, su, sWrow, sArow, red);
      } else {
        nfb = (m + 63) / 64;
        zp_rows_phase<4>(P, A, lda, n, p, c, i, nck, last, R, alpha, vs, su, sWrow, sArow, red);
      }
      if (!zp_gsync(P)) return;
      if (!last) {  // reflector c+1, identically in every CTA (one thread forms it)
        const int c1 = c + 1;
        if (w == 0) {
          double ss = 0.0;
          for (int t = lane; t < nfb; t += 32) ss += __ldcg(P.sspart + t);
          ss = warp_sum(ss);
          if (lane == 0) {
            s_scal = ss_needs_scaling(ss) ? 1 : 0;
            if (!s_scal) s_R = zp_refl(ldz(A + (c1 + 1) + (int64_t)c1 * lda), sqrt(ss));
          }
        }
        __syncthreads();
        if (s_scal)
          R = zp_refl_from_column(P, c1, red);
        else
          R = s_R;
        __syncthreads();
        if (lead) {
          P.ev[c1] = R.beta;
          P.tau[c1] = R.tau;
        }
      }
    }
    // ---- D: trailing update, tiles from the shared counter
    const int q = p + nbp;
    const int mt = (n - q + ZUT - 1) / ZUT;
    const unsigned ntiles = (unsigned)(mt * (mt + 1) / 2);
    for (;;) {
      if (tid == 0) s_item = atomicAdd(P.sync + 1, 1u) - item_base;
      __syncthreads();
      const unsigned t = s_item;
      __syncthreads();
      if (t >= ntiles) break;
      zp_upd_tile(P, p, nbp, q, (int)t, vs);
    }
    item_base += ntiles + gridDim.x;  // one failing ticket per CTA
    if (!zp_gsync(P)) return;
    p = q;
    if (p < P.pend) {
      R = zp_refl_from_column(P, p, red);
      if (lead) {
        P.ev[p] = R.beta;
        P.tau[p] = R.tau;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int zp_maxck(int n) { return std::max(1, (n + 31) / 32); }

size_t zhess_persist_ws_doubles(int n) {
  const size_t nn = (size_t)n;
  const size_t maxck = (size_t)zp_maxck(n);
  return 2 * nn * ZBNB      // W
         + 2 * maxck * nn   // ypart
         + 2 * ZP_MAXWARPS  // dpart (one per warp)
         + 2 * 2 * ZBNB     // u
         + (nn + ZFIN - 1) / ZFIN + 1  // sspart
         + 8;               // sync words, error flag
}

__global__ void zp_merge_err_kernel(const int* err, int* info) {
  if (*err && info) *info = SKEW_TIMEOUT;
}

// Runs the panels of columns [0, n - 1 - ZTAILP) in one cooperative launch and the
// rest with the one-CTA kernel.  cudaErrorNotSupported when the device cannot
// co-schedule the grid or n is outside the staged range (the caller then uses the
// per-column path).
cudaError_t zhess_persistent(double* Ad, int64_t lda, int n, double* taud, double* ev, double* dvim, double* wsd,
                             int sms, int* info, const Tuning& tune, cudaStream_t st) {
  const size_t smem = std::max((size_t)n * sizeof(zc), (size_t)ZUT * (ZUT + 1) * sizeof(zc));
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (smem + 2048 > (size_t)optin || n <= ZTAILP + 2) return cudaErrorNotSupported;
  e = cudaFuncSetAttribute(zpersist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, zpersist_kernel, ZP_NT, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorNotSupported;
  int grid = sms;
  if (tune.zpersist_ctas > 0) grid = std::max(1, std::min(sms * occ, tune.zpersist_ctas));
  grid = std::min(grid, ZP_MAXWARPS / ZP_NW);
  zc* A = reinterpret_cast<zc*>(Ad);
  zc* tau = reinterpret_cast<zc*>(taud);
  ZPersistParams P;
  P.A = A;
  P.lda = lda;
  P.n = n;
  P.pend = n - 1 - ZTAILP;
  P.nb = std::max(4, std::min(ZBNB, tune.zpersist_nb));
  P.tau = tau;
  P.ev = ev;
  const size_t nn = (size_t)n, maxck = (size_t)zp_maxck(n);
  double* wp = wsd;
  P.W = reinterpret_cast<zc*>(wp);
  wp += 2 * nn * ZBNB;
  P.ypart = reinterpret_cast<zc*>(wp);
  wp += 2 * maxck * nn;
  P.dpart = reinterpret_cast<zc*>(wp);
  wp += 2 * ZP_MAXWARPS;
  P.u = reinterpret_cast<zc*>(wp);
  wp += 2 * 2 * ZBNB;
  P.sspart = wp;
  wp += (nn + ZFIN - 1) / ZFIN + 1;
  P.sync = reinterpret_cast<unsigned*>(wp);  // 2 words
  P.err = reinterpret_cast<int*>(wp + 1);
  P.maxck = (int)maxck;
  P.items_per_warp = std::max(1, std::min(8, tune.zpersist_items));
  P.poll_limit = tune.wait_polls > 0 ? tune.wait_polls : ZP_POLL;
  P.skip_cta = tune.wait_skip_cta;
  e = cudaMemsetAsync(wp, 0, 2 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  void* args[] = {&P};
  e = cudaLaunchCooperativeKernel((const void*)zpersist_kernel, dim3(grid), dim3(ZP_NT), args, smem, st);
  if (e != cudaSuccess) return e;
  // tail: the trailing block with the one-CTA kernel, in place
  const int c0 = P.pend;
  ZHessParams T;
  T.W = nullptr;
  T.W1 = reinterpret_cast<double*>(A + c0 + (int64_t)c0 * lda);
  T.n1 = n - c0;
  T.ld1 = lda;
  T.stride = 0;
  T.n = nullptr;
  T.off = nullptr;
  T.order = nullptr;
  T.count = 1;
  T.nmax = n - c0;
  T.counter = nullptr;
  T.tau = reinterpret_cast<double*>(tau + c0);
  T.ev = ev + c0;
  T.dvim = nullptr;
  e = launch_zhess_cta(T, 1, st);
  if (e != cudaSuccess) return e;
  e = launch_zdiag_im(Ad, lda, n, dvim, st);
  if (e != cudaSuccess) return e;
  zp_merge_err_kernel<<<1, 1, 0, st>>>(P.err, info);
  return cudaGetLastError();
}

}  // namespace skew
