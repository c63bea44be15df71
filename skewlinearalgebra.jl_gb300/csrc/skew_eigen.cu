// Eigenvectors, exp, cis and the exp adjoint for real skew matrices (n <= 1024),
// batched; single matrices run as a batch of one.
//
// Pipeline (after the batched reduction of skew_batch.cu has left the
// reflectors, tau and ev of every matrix in the plan's workspace):
//   chain   one thread per matrix runs the implicit QR of skewtrieigen_divided!
//           (skeweigen.jl:322-377): same tolerance (10 eps), shift, deflation
//           order, the |ev[n-1] - mem| < tol deflation (:355) and the stagnation
//           counter.  The iteration on ev never depends on the eigenvectors, so
//           every Givens rotation is logged instead of applied.
//   vectors one CTA per matrix replays the log on Qodd / Qeven (lanes are rows:
//           every row is rotated independently), applies the odd-size rotations
//           of reducetozero (getoddvectors, :49-62) and assembles the real and
//           imaginary eigenvector parts with the reference's +-1/sqrt(2) pairing
//           (:378-449).  If the QR stagnated, the eigenvectors of the symmetric
//           tridiagonal SymTridiagonal(0, ev) come from a cyclic Jacobi solver
//           in the same CTA and are laid out as skewtrieigen_backup! does
//           (:470-489).
//   back    V <- Q V for both parts (eigen.jl:85-89) by compact-WY blocks of 8
//           reflectors: Y = V_b^T X, Z = T_b Y, X -= V_b Z.
//   exp     E = Qr P^T + Qi R^T with P = Qr C + Qi S, R = Qi C - Qr S
//           (C, S = cos, sin of the eigenvalues; exp.jl:3-35 reassociated).
//   cis     V diag(exp(-Im lambda)) V^H (exp.jl:99-110), two real products.
//   vjp     d<Gbar, exp(A)>/dA = Re(V (conj(Phi) o (V^H Gbar V)) V^H) with the
//           Daleckii-Krein divided differences Phi_jk of exp on the i*mu
//           spectrum, evaluated as exp(i(mu_j+mu_k)/2) sinc((mu_j-mu_k)/2);
//           computed in the real Schur basis (four real products, see below),
//           the complex form only for matrices whose spectrum does not split
//           into conjugate pairs cleanly.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "skew_common.cuh"
#include "skew_internal.h"
#include "skew_twisted.cuh"
#include "skew_funcs.cuh"

namespace skew {

constexpr int ENT = 256;  // threads per CTA of the per-matrix kernels
constexpr int ENW = ENT / 32;
constexpr int EB = 8;     // reflectors per back-transformation block

// ---------------------------------------------------------------------------
// chain: the QR iteration of skewtrieigen_divided!, rotations logged
// ---------------------------------------------------------------------------
// getgivens (skeweigen.jl:3-7): nm = hypot(a, b); (1, 0) if nm == 0, else
// (a/nm, b/nm).  Every product and sum of the chain is rounded separately (no
// fused multiply-add), as in the reference's Float64 code, so that the GPU takes
// the reference's deflation decisions, which hinge on the last bits of ev.
__device__ __forceinline__ void givens_e(double a, double b, double& c, double& s) {
  const double nm = hypot(a, b);
  if (nm == 0.0) {
    c = 1.0;
    s = 0.0;
    return;
  }
  c = __ddiv_rn(a, nm);
  s = __ddiv_rn(b, nm);
}

// reducetozero (skeweigen.jl:11-47) recording G (c, -s pairs); n = N-1 (even).
__device__ void reducetozero_g(double* ev, double* G, int n) {
  if (n == 0) return;
  double bulge = 0.0, c, s;
  if (n > 2) {
    const double a = ev[n - 3], b = ev[n - 2], g = ev[n - 1];
    givens_e(-b, g, c, s);
    G[n - 2] = c;
    G[n - 1] = neg(s);
    ev[n - 3] = __dmul_rn(ev[n - 3], c);
    ev[n - 2] = __dsub_rn(__dmul_rn(c, b), __dmul_rn(s, g));
    ev[n - 1] = 0.0;
    bulge = __dmul_rn(neg(s), a);
    for (int i = n - 2; i >= 4; i -= 2) {
      const double a2 = ev[i - 3], b2 = ev[i - 2];
      givens_e(-b2, bulge, c, s);
      G[i - 2] = c;
      G[i - 1] = neg(s);
      ev[i - 3] = __dmul_rn(ev[i - 3], c);
      ev[i - 2] = __dsub_rn(__dmul_rn(c, b2), __dmul_rn(s, bulge));
      bulge = __dmul_rn(neg(s), a2);
    }
  }
  const double b = (n == 2 ? ev[1] : bulge);
  const double a = ev[0];
  givens_e(-a, b, c, s);
  G[0] = c;
  G[1] = neg(s);
  ev[0] = __dsub_rn(__dmul_rn(c, a), __dmul_rn(s, b));
  if (n == 2) ev[1] = __dadd_rn(__dmul_rn(s, a), __dmul_rn(b, c));
}

// implicitstep_vec! (skeweigen.jl:158-193) without the vector update: the
// rotations (c, s) of steps i = start..n-1 are appended to log after a header
// (start, n).  Returns the new start, or -1 if the log is full.  As in the
// reference, a split found mid-sweep moves `start` at once, so the next step
// restarts the shifted rotation from there (the replay needs only i, not start).
__device__ int implicitstep_log(double* ev, int n, int start, double* log, int64_t& len, int64_t cap) {
  if (len + 2 + 2 * (int64_t)(n - start) > cap) return -1;
  log[len++] = (double)start;
  log[len++] = (double)n;
  double bulge = 0.0;
  const double shift = __dmul_rn(ev[n - 1], ev[n - 1]);
  const double tol = 10.0 * 2.220446049250313e-16;
  const int first = start;
  // ev[i-2], ev[i-1], ev[i] of step i are what step i-1 wrote: carried in
  // registers; ev[i+1] (untouched this sweep) is loaded one step ahead.  Every
  // store of the reference's step is still made.
  double pa = 0.0;            // ev[i-2] as left by the previous step
  double b = ev[first - 1];   // ev[i-1]
  double g = ev[first];       // ev[i]
  double z = (first < n - 1) ? ev[first + 1] : 0.0;
  for (int i = first; i <= n - 1; i++) {
    const double zn = (i + 2 <= n - 1) ? ev[i + 2] : 0.0;
    const double a = (i > start ? pa : 0.0);
    double c, s;
    if (i > start) {
      givens_e(a, bulge, c, s);
    } else {
      const double x1 = __dadd_rn(__dsub_rn(neg(__dmul_rn(a, a)), __dmul_rn(b, b)), shift);
      const double x2 = __dadd_rn(neg(__dmul_rn(a, bulge)), __dmul_rn(b, g));
      givens_e(x1, x2, c, s);
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
      if (fabs(bulge) < tol && fabs(nb) < tol) start = i + 1;
      pa = nb;
      b = ng;
      g = nz;
      z = zn;
    }
    log[len++] = c;
    log[len++] = s;
  }
  return start;
}

__global__ void eigen_chain_kernel(EigenBatch E) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= E.count) return;
  const int b = E.order[t];
  const int N = E.n[b];
  if (N > E.chain_nmax) {  // eigenpairs from bisection and twisted vectors instead
    E.status[b] = SKEW_OK;
    return;
  }
  double* ev = E.ev + E.off_n[b];
  double* evb = E.evb + E.off_n[b];
  double* G = E.G + E.off_n[b];
  double* vals = E.vals[b];
  double* log = E.log + E.off_log[b];
  const int64_t cap = E.cap_log[b];
  int64_t len = 0;
  for (int i = 0; i + 1 < N; i++) evb[i] = ev[i];
  for (int i = 0; i < N; i++) vals[i] = 0.0;
  int status = SKEW_OK;
  int n = N;
  if (N >= 2) {
    if (n & 1) {
      n -= 1;
      reducetozero_g(ev, G, n);
    }
    const double tol = 10.0 * 2.220446049250313e-16;
    const int max_iter = E.max_iter > 0 ? E.max_iter : 30 * n;
    int iter = 0, count_static = 0, start = 1;
    double mem = 1.0;
    while (n > 2 && iter < max_iter) {
      start = implicitstep_log(ev, n - 1, start, log, len, cap);
      if (start < 0) {
        status = SKEW_NO_CONVERGENCE;
        break;
      }
      while (n > 2 && fabs(ev[n - 2]) <= tol) {
        vals[n - 1] = 0.0;
        n -= 1;
      }
      while (n > 2 && fabs(ev[n - 3]) <= tol * fabs(ev[n - 2])) {
        vals[n - 2] = ev[n - 2];
        vals[n - 1] = neg(ev[n - 2]);
        n -= 2;
      }
      if (!E.merged && n > 2 && fabs(ev[n - 2] - mem) < tol) {  // skeweigen.jl:355-358 (divided only)
        vals[n - 2] = ev[n - 2];
        vals[n - 1] = neg(ev[n - 2]);
        n -= 2;
      }
      if (start > n - 2) start = 1;
      if (n > 1 && fabs(mem - ev[n - 2]) < 0.0001 * fabs(ev[n - 2])) {
        count_static += 1;
        if (count_static > 4) {
          status = SKEW_FALLBACK_USED;
          break;
        }
      } else {
        count_static = 0;
      }
      mem = (n > 1 ? ev[n - 2] : 0.0);
      iter += 1;
    }
    if (status == SKEW_OK) {
      if (n > 2) {
        status = SKEW_NO_CONVERGENCE;
      } else if (n == 2) {
        vals[0] = ev[0];
        vals[1] = neg(ev[0]);
      } else if (n == 1) {
        vals[0] = 0.0;
      }
    }
  } else if (N == 1) {
    vals[0] = 0.0;
  }
  E.log_len[b] = len;
  E.status[b] = status;
}

// ---------------------------------------------------------------------------
// vectors: replay the rotations, assemble Qr / Qim
// ---------------------------------------------------------------------------

// The stagnation fallback (skewtrieigen_backup!, skeweigen.jl:470-489) for one
// matrix, by the CTA: all N eigenpairs (lambda_j ascending, w_j) of
// SymTridiagonal(0, e) (the reference calls LAPACK there), written as the
// fallback does: vals_j = -lambda_j (descending) and column j real on odd (1-based)
// rows and imaginary on even rows, sign flipped every pair.
//   - eigenvalues by bisection to relative precision (the zero-diagonal Sturm
//     count resolves tiny singular values of the bidiagonal coupling);
//   - one twisted-factorisation vector per eigenvalue (skew_twisted.cuh), each
//     copy of a repeated eigenvalue confined to its own block where the
//     tridiagonal splits (several odd blocks give several zero eigenvalues);
//   - three passes of the banded symmetric correction over whole vectors, which
//     settle clusters of nearly equal eigenvalues.
// work: fallback_ws_doubles(N).
constexpr int FB_LW = 16;

__host__ __device__ inline int fallback_kp(int N) { return (N + 31) / 32 * 32; }
__host__ __device__ inline int64_t fallback_ws_doubles(int N) {
  const int64_t KP = fallback_kp(N);
  return 3 * (int64_t)N * KP + 2 * KP + KP * (FB_LW + 1) + 64;
}

__device__ void cta_fallback(const double* __restrict__ e, int N, double* __restrict__ vals, double* __restrict__ Vr,
                             double* __restrict__ Vi, int64_t ldv, double* __restrict__ work) {
  __shared__ double red[2][ENW];
  const int tid = threadIdx.x;
  const int KP = fallback_kp(N);
  double* dp = work;
  double* dm = dp + (int64_t)N * KP;
  double* z = dm + (int64_t)N * KP;
  double* nrm2 = z + (int64_t)N * KP;
  double* lam = nrm2 + KP;   // ascending eigenvalues
  double* band = lam + KP;   // [k][d]
  // Gershgorin bound and pivmin
  double bound = 0.0, e2 = 0.0;
  for (int i = tid; i < N; i += ENT) {
    const double l = (i > 0) ? fabs(e[i - 1]) : 0.0, r = (i + 1 < N) ? fabs(e[i]) : 0.0;
    bound = fmax(bound, l + r);
    if (i + 1 < N) e2 = fmax(e2, r * r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    bound = fmax(bound, __shfl_xor_sync(0xffffffffu, bound, o));
    e2 = fmax(e2, __shfl_xor_sync(0xffffffffu, e2, o));
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = bound;
    red[1][tid >> 5] = e2;
  }
  __syncthreads();
  bound = 0.0;
  e2 = 0.0;
  for (int w = 0; w < ENW; w++) {
    bound = fmax(bound, red[0][w]);
    e2 = fmax(e2, red[1][w]);
  }
  __syncthreads();
  const double pivmin = 2.2250738585072014e-308 * fmax(1.0, e2);
  bound = bound * (1.0 + 1e-14) + 1e-300;
  // all eigenvalues, ascending, to relative precision (the spectrum is symmetric:
  // the k-th smallest for k < N/2 is minus the k-th largest)
  const int h = N / 2;
  for (int k = tid; k < h; k += ENT) {
    double lo = 0.0, hi = bound;  // the k-th largest, positive
    for (int it = 0; it < 1100 && hi - lo > fmax(2.220446049250313e-16 * hi, 4.0 * pivmin); it++) {
      const double mid = 0.5 * (lo + hi);
      if (block_sturm(e, nullptr, 0, N, mid, pivmin) <= N - 1 - k)
        lo = mid;
      else
        hi = mid;
    }
    const double x = 0.5 * (lo + hi);
    lam[N - 1 - k] = x;
    lam[k] = neg(x);
  }
  if ((N & 1) && tid == 0) lam[h] = 0.0;
  __syncthreads();
  // one twisted vector per eigenvalue (whole warps: KP and ENT are multiples of 32)
  for (int kb = 0; kb < KP; kb += ENT) {
    if (kb + (tid & ~31) >= KP) continue;
    const int k = kb + tid;
    const double sig = lam[min(k, N - 1)];
    int lo = 0, hi = N;
    if (k < N) {
      const double delta = fmax(16.0 * 2.220446049250313e-16 * fabs(sig), 4.0 * pivmin);
      int j = 0;
      for (int q = k - 1; q >= 0 && fabs(lam[q] - sig) <= delta; q--) j++;
      tdvec_block(e, nullptr, N, sig, delta, j, pivmin, &lo, &hi);
    }
    nrm2[k] = twisted_vector(e, nullptr, N, sig, pivmin, KP, k, lo, hi, dp, dm, z);
  }
  __syncthreads();
  // unit vectors X = z / |z|, then X <- X - 1/2 X E (E = X^T X - I over the band), three passes
  double* X = dp;
  double* Y = z;
  for (int64_t q = tid; q < (int64_t)N * KP; q += ENT) {
    const int k = (int)(q % KP);
    X[q] = (k < N) ? z[q] * rsqrt(nrm2[k]) : 0.0;
  }
  __syncthreads();
  for (int pass = 0; pass < 3; pass++) {
    for (int q = tid; q < N * (FB_LW + 1); q += ENT) {
      const int k = q / (FB_LW + 1), d = q - k * (FB_LW + 1), j = k + d;
      double sum = 0.0;
      if (j < N)
        for (int i = 0; i < N; i++) sum = fma(X[(int64_t)i * KP + k], X[(int64_t)i * KP + j], sum);
      band[q] = sum - (d == 0 ? 1.0 : 0.0);
    }
    __syncthreads();
    for (int64_t q = tid; q < (int64_t)N * KP; q += ENT) {
      const int i = (int)(q / KP), k = (int)(q - (int64_t)i * KP);
      double acc = X[q];
      if (k < N)
        for (int d = -FB_LW; d <= FB_LW; d++) {
          const int j = k + d;
          if (j < 0 || j >= N) continue;
          const int lo = min(k, j), off = abs(d);
          acc = fma(-0.5 * band[lo * (FB_LW + 1) + off], X[(int64_t)i * KP + j], acc);
        }
      Y[q] = acc;
    }
    __syncthreads();
    double* t = X;
    X = Y;
    Y = t;
  }
  // the fallback's layout: column j from w_j, vals_j = -lambda_j
  for (int j = tid; j < N; j += ENT) vals[j] = neg(lam[j]);
  for (int64_t q = tid; q < (int64_t)N * N; q += ENT) {
    const int j = (int)(q / N), i = (int)(q - (int64_t)j * N);
    double o = X[(int64_t)i * KP + j];
    if ((i >> 1) & 1) o = neg(o);
    if ((i & 1) == 0 || ((N & 1) && i == N - 1)) {
      Vr[i + (int64_t)j * ldv] = o;
      Vi[i + (int64_t)j * ldv] = 0.0;
    } else {
      Vr[i + (int64_t)j * ldv] = 0.0;
      Vi[i + (int64_t)j * ldv] = o;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(ENT) eigen_vectors_kernel(EigenBatch E) {
  __shared__ int s_next;
  __shared__ int s_type[1024 + 1];  // per output column: -1 none, 0..3 kinds (see below)
  __shared__ int s_src[1024 + 1];
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(E.counter, 1u);
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= E.count) break;
    const int b = E.order[t];
    const int N = E.n[b];
    if (N > E.chain_nmax) continue;  // vectors from the twisted path
    double* Vr = E.Vr[b];
    double* Vi = E.Vi[b];
    const int64_t ldv = E.n[b];
    double* work = E.work + E.off_w[b];
    const int st = E.status[b];
    // zero the outputs (the reference starts from zeros: tridiag.jl:175)
    for (int64_t k = threadIdx.x; k < (int64_t)N * N; k += ENT) {
      const int j = (int)(k / N), i = (int)(k - (int64_t)j * N);
      Vr[i + (int64_t)j * ldv] = 0.0;
      Vi[i + (int64_t)j * ldv] = 0.0;
    }
    __syncthreads();
    if (N == 1) {
      if (threadIdx.x == 0) Vr[0] = 1.0;
      __syncthreads();
      continue;
    }
    if (st == SKEW_NO_CONVERGENCE) continue;
    if (st == SKEW_FALLBACK_USED) {
      cta_fallback(E.evb + E.off_n[b], N, E.vals[b], Vr, Vi, ldv, work);
      continue;
    }
    // Qodd (ho x ho) and Qeven (he x he), column-major, identity
    const int halfN = (N & 1) ? (N - 1) / 2 : N / 2;
    const int ho = (N + 1) / 2, he = N / 2;
    double* Qo = work;
    double* Qe = work + (int64_t)ho * ho;
    for (int64_t k = threadIdx.x; k < (int64_t)ho * ho; k += ENT) Qo[k] = (k % (ho + 1) == 0) ? 1.0 : 0.0;
    for (int64_t k = threadIdx.x; k < (int64_t)he * he; k += ENT) Qe[k] = (k % (he + 1) == 0) ? 1.0 : 0.0;
    __syncthreads();
    // replay: thread r owns row r of both (rows 0..halfN-1 are rotated)
    const double* log = E.log + E.off_log[b];
    const int64_t len = E.log_len[b];
    for (int r = threadIdx.x; r < halfN; r += ENT) {
      int64_t pos = 0;
      while (pos < len) {
        const int s0 = (int)log[pos], np = (int)log[pos + 1];
        pos += 2;
        for (int i = s0; i <= np - 1; i++) {
          const double c = log[pos], s = log[pos + 1];
          pos += 2;
          const int k = (i + 1) / 2;  // 1-based column pair (k, k+1)
          double* Q = (i & 1) ? Qo : Qe;
          const int ld = (i & 1) ? ho : he;
          double* q0 = Q + r + (int64_t)(k - 1) * ld;
          double* q1 = Q + r + (int64_t)k * ld;
          const double sg = *q0, om = *q1;
          *q0 = fma(c, sg, s * om);
          *q1 = fma(-s, sg, c * om);
        }
      }
    }
    __syncthreads();
    if (N & 1) {  // getoddvectors (:49-62): row rotations (ii, nn) for all columns
      const double* G = E.G + E.off_n[b];
      const int n1 = N - 1, nn = n1 / 2 + 1;
      for (int i = 1; i <= n1 - 1; i += 2) {
        const double c = G[i - 1], s = G[i];
        const int ii = (i + 1) / 2;
        for (int j = threadIdx.x; j < nn; j += ENT) {
          double* a = Qo + (ii - 1) + (int64_t)j * ho;
          double* z = Qo + (nn - 1) + (int64_t)j * ho;
          const double sg = *a, om = *z;
          *a = c * sg + s * om;
          *z = -s * sg + c * om;
        }
        __syncthreads();
      }
    }
    // assembly (:389-449): column descriptors by one thread, then a parallel fill
    if (threadIdx.x == 0) {
      const double* vals = E.vals[b];
      int i = 1, countzeros = 0;
      for (int q = 0; q <= N; q++) s_type[q] = -1;
      while (i <= N) {
        const int ii = (i + 1) / 2;
        if (vals[i - 1] == 0.0) {
          s_type[i] = (countzeros & 1) ? 1 : 0;  // 0: Qodd -> real odd rows; 1: Qeven -> real even rows
          s_src[i] = ii;
          countzeros++;
          i += 1;
        } else {
          s_type[i] = (countzeros & 1) ? 3 : 2;  // pair (i, i+1)
          s_src[i] = ii;
          i += 2;
        }
      }
    }
    __syncthreads();
    const double s2 = 0.7071067811865476;  // 1/sqrt(2)
    for (int i = 1; i <= N; i++) {
      const int ty = s_type[i];
      if (ty < 0) continue;
      const int ii = s_src[i];
      // column ranges implied by the zero-count parity of the reference's
      // assembly; checked so that an inconsistent pattern cannot read past Q
      if ((ty == 0 && ii > ho) || (ty == 1 && ii > he) || (ty == 2 && (ii > ho || ii > he || i + 1 > N)) ||
          (ty == 3 && (ii + 1 > ho || ii > he || i + 1 > N)))
        continue;
      double* vr0 = Vr + (int64_t)(i - 1) * ldv;
      double* vi0 = Vi + (int64_t)(i - 1) * ldv;
      double* vr1 = Vr + (int64_t)i * ldv;
      double* vi1 = Vi + (int64_t)i * ldv;
      for (int jj = 1 + threadIdx.x; jj <= halfN; jj += ENT) {
        const int j = 2 * jj - 1;  // odd 1-based row; rows j-1 and j are 0-based j-1, j
        if (ty == 0) {
          vr0[j - 1] = Qo[(jj - 1) + (int64_t)(ii - 1) * ho];
        } else if (ty == 1) {
          vr0[j] = Qe[(jj - 1) + (int64_t)(ii - 1) * he];
        } else if (ty == 3) {
          const double qo = Qo[(jj - 1) + (int64_t)ii * ho], qe = Qe[(jj - 1) + (int64_t)(ii - 1) * he];
          vi0[j - 1] = -s2 * qo;
          vr0[j] = s2 * qe;
          vr1[j - 1] = -s2 * qo;
          vi1[j] = s2 * qe;
        } else {
          const double qo = Qo[(jj - 1) + (int64_t)(ii - 1) * ho], qe = Qe[(jj - 1) + (int64_t)(ii - 1) * he];
          vr0[j - 1] = s2 * qo;
          vi0[j] = -s2 * qe;
          vi1[j - 1] = s2 * qo;
          vr1[j] = -s2 * qe;
        }
      }
      if ((N & 1) && threadIdx.x == 0) {
        if (ty == 0) {
          vr0[N - 1] = Qo[halfN + (int64_t)(ii - 1) * ho];
        } else if (ty == 3) {
          const double qo = Qo[halfN + (int64_t)ii * ho];
          vr0[N - 1] = -s2 * qo;
          vi1[N - 1] = -s2 * qo;
        } else if (ty == 2) {
          const double qo = Qo[halfN + (int64_t)(ii - 1) * ho];
          vr0[N - 1] = s2 * qo;
          vi1[N - 1] = s2 * qo;
        }
      }
    }
    __syncthreads();
    if (N & 1) {  // last column from Qodd's last column (:444-448)
      for (int j = 1 + 2 * threadIdx.x; j <= N; j += 2 * ENT) {
        const int jj = (j + 1) / 2;
        Vr[(j - 1) + (int64_t)(N - 1) * ldv] = Qo[(jj - 1) + (int64_t)halfN * ho];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// back: V <- Q V for V = Vr and Vi, Q from the stored reflectors
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(ENT) eigen_back_kernel(EigenBatch E) {
  __shared__ int s_next;
  __shared__ double T[EB * EB], P[32], scratch[ENW * 32];
  extern __shared__ __align__(16) double esm[];  // Vs (nmax x EB, row-major) | Zs (EB x 2 nmax)
  double* Vs = esm;
  double* Zs = esm + (size_t)E.nmax * EB;
  __shared__ int s_chunk;
  for (;;) {
    // work item: (matrix in the processing order, chunk of kBackCols columns), the
    // largest matrices first; without back_off, one item per matrix
    if (threadIdx.x == 0) {
      const int item = (int)atomicAdd(E.counter, 1u);
      if (!E.back_off) {
        s_next = item;
        s_chunk = -1;
      } else if (item >= E.back_items) {
        s_next = E.count;
      } else {
        int lo = 0, hi = E.count;  // back_off[lo] <= item < back_off[hi]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (E.back_off[mid] <= item) lo = mid; else hi = mid;
        }
        s_next = lo;
        s_chunk = item - E.back_off[lo];
      }
    }
    __syncthreads();
    const int t = s_next, chunk = s_chunk;
    __syncthreads();
    if (t >= E.count) break;
    const int b = E.order[t];
    const int n = E.n[b];
    const int64_t ldv = E.n[b];
    const double* R = E.refl[b];  // n x n, ld n
    const double* tau = E.tau + E.off_n[b];
    if (E.status[b] == SKEW_NO_CONVERGENCE || n < 3) continue;
    // the columns to transform: Vr and Vi, or the real Schur basis Q (work block 0) alone;
    // this item takes [c0, c1) of them
    const bool qonly = E.back_q && E.fsel && E.fsel[b] == 1;
    const int ncol_all = qonly ? n : 2 * n;
    const int c0 = chunk < 0 ? 0 : chunk * kBackCols;
    const int c1 = chunk < 0 ? ncol_all : min(ncol_all, c0 + kBackCols);
    if (c0 >= c1) continue;
    double* const Xq = E.pwork[b];
    auto colp = [&](int col) -> double* {
      if (qonly) return Xq + (int64_t)col * n;
      return (col < n) ? (E.Vr[b] + (int64_t)col * ldv) : (E.Vi[b] + (int64_t)(col - n) * ldv);
    };
    const int nref = n - 2;
    for (int kend = nref; kend > 0; kend -= EB) {
      const int k0 = max(0, kend - EB), nb = kend - k0;
      const int r0 = k0 + 1, m = n - r0;
      for (int idx = threadIdx.x; idx < m * EB; idx += ENT) {
        const int rr = idx / EB, l = idx - rr * EB;
        const int r = r0 + rr, kk = k0 + l;
        double val = 0.0;
        if (l < nb) val = (r < kk + 1) ? 0.0 : (r == kk + 1 ? 1.0 : R[r + (int64_t)kk * n]);
        Vs[idx] = val;
      }
      __syncthreads();
      {  // Gram and T (forward, columnwise), as in the gradient
        double part[32];
#pragma unroll
        for (int q = 0; q < 32; q++) part[q] = 0.0;
        for (int rr = threadIdx.x; rr < m; rr += ENT) {
          double vr[EB];
#pragma unroll
          for (int l = 0; l < EB; l++) vr[l] = Vs[rr * EB + l];
#pragma unroll
          for (int l1 = 0; l1 < EB; l1++)
#pragma unroll
            for (int l2 = l1 + 1; l2 < EB; l2++) part[pair_slot(l1, l2)] = fma(vr[l1], vr[l2], part[pair_slot(l1, l2)]);
        }
        block_reduce_pairs<ENT>(part, 28, scratch, P);
        if (threadIdx.x < 32) {
          const int lane = threadIdx.x;
          for (int q = lane; q < EB * EB; q += 32) T[q] = 0.0;
          __syncwarp();
          for (int l = 0; l < nb; l++) {
            const double tl = tau[k0 + l];
            double acc = 0.0;
            if (lane < l)
              for (int j = lane; j < l; j++) acc = fma(T[lane * EB + j], P[pair_slot(j, l)], acc);
            __syncwarp();
            if (lane < l) T[lane * EB + l] = neg(tl * acc);
            if (lane == l) T[l * EB + l] = tl;
            __syncwarp();
          }
        }
        __syncthreads();
      }
      // Y = V^T X (EB x the item's columns), then Z = T Y; thread per column of X
      for (int col = c0 + (int)threadIdx.x; col < c1; col += ENT) {
        const double* x = colp(col);
        double y[EB];
#pragma unroll
        for (int l = 0; l < EB; l++) y[l] = 0.0;
        for (int rr = 0; rr < m; rr++) {
          const double xv = x[r0 + rr];
#pragma unroll
          for (int l = 0; l < EB; l++) y[l] = fma(Vs[rr * EB + l], xv, y[l]);
        }
#pragma unroll
        for (int l = 0; l < EB; l++) {
          double z = 0.0;
#pragma unroll
          for (int c = l; c < EB; c++) z = fma(T[l * EB + c], y[c], z);
          Zs[l * 2 * n + col] = z;
        }
      }
      __syncthreads();
      // X[r, col] -= sum_l V[r, l] Z[l, col] for r >= r0; lanes are rows.  Each lane
      // holds its row of V in registers across the warp's columns (read from shared
      // memory once per 32-row chunk: the rows are EB doubles apart, so a warp-wide
      // read of them conflicts), and Z[., col] is a broadcast.
      for (int rr0 = 0; rr0 < m; rr0 += 32) {
        const int rr = rr0 + (threadIdx.x & 31);
        if (rr < m) {
          double vr[EB];
#pragma unroll
          for (int l = 0; l < EB; l++) vr[l] = Vs[rr * EB + l];
          for (int col = c0 + (int)(threadIdx.x >> 5); col < c1; col += ENW) {
            double* x = colp(col);
            double acc = x[r0 + rr];
#pragma unroll
            for (int l = 0; l < EB; l++) acc = fma(-vr[l], Zs[l * 2 * n + col], acc);
            x[r0 + rr] = acc;
          }
        }
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// exp / cis / exp adjoint from (vals, Vr, Vi): tiled batched products
// ---------------------------------------------------------------------------
// Operand of a batched product: matrix b is p[b] + add_sq * n_b^2 (n_b x n_b, ld n_b),
// used transposed if trans.
struct BOperand {
  const double* const* p;
  int add_sq;
  int trans;
};

struct BGemm {
  const int32_t* n;
  const int* status;  // matrices with SKEW_NO_CONVERGENCE are skipped
  const int* sel;     // non-null: only matrices with sel[b] == sel_val
  int sel_val;
  int nterms;         // C_b = sum_t s_t op(A_t,b) op(B_t,b)
  BOperand A[2], B[2];
  double s[2];
  double* const* C;
  int c_add_sq;
  int c_add;   // extra offset in doubles (1: imaginary parts of an interleaved output)
  int c_step;  // 1, or 2 for a ComplexF64 output
};

constexpr int BG_T = 64, BG_K = 16;

// One 64 x 64 tile of one matrix per CTA: grid (tiles^2 of the largest matrix, count);
// tiles outside a smaller matrix return at once.
__global__ void __launch_bounds__(256) bgemm_kernel(BGemm P) {
  __shared__ double As[BG_K][BG_T + 1];
  __shared__ double Bs[BG_K][BG_T + 1];
  const int b = blockIdx.y;
  const int n = P.n[b];
  if (P.status && P.status[b] == SKEW_NO_CONVERGENCE) return;
  if (P.sel && P.sel[b] != P.sel_val) return;
  const int nt = (n + BG_T - 1) / BG_T;
  if ((int)blockIdx.x >= nt * nt) return;
  const int i0 = (blockIdx.x % nt) * BG_T, j0 = (blockIdx.x / nt) * BG_T;
  const int64_t nn = (int64_t)n * n;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[a][q] = 0.0;
  for (int t = 0; t < P.nterms; t++) {
    const double* A = P.A[t].p[b] + (int64_t)P.A[t].add_sq * nn;
    const double* B = P.B[t].p[b] + (int64_t)P.B[t].add_sq * nn;
    const int ta = P.A[t].trans, tb = P.B[t].trans;
    const double sg = P.s[t];
    for (int k0 = 0; k0 < n; k0 += BG_K) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < BG_T * BG_K; idx += 256) {
        int ii, kk;
        if (!ta) {
          ii = idx & 63;
          kk = idx >> 6;
        } else {
          kk = idx & 15;
          ii = idx >> 4;
        }
        const int i = i0 + ii, k = k0 + kk;
        double av = 0.0;
        if (i < n && k < n) av = ta ? A[k + (int64_t)i * n] : A[i + (int64_t)k * n];
        As[kk][ii] = sg * av;
        int jj, kb;
        if (!tb) {
          kb = idx & 15;
          jj = idx >> 4;
        } else {
          jj = idx & 63;
          kb = idx >> 6;
        }
        const int j = j0 + jj, k2 = k0 + kb;
        double bv = 0.0;
        if (j < n && k2 < n) bv = tb ? B[j + (int64_t)k2 * n] : B[k2 + (int64_t)j * n];
        Bs[kb][jj] = bv;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BG_K; kk++) {
        double a4[4], b4[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
          a4[a] = As[kk][tx + 16 * a];
          b4[a] = Bs[kk][ty + 16 * a];
        }
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
          for (int q = 0; q < 4; q++) acc[a][q] = fma(a4[a], b4[q], acc[a][q]);
      }
    }
  }
  double* C = P.C[b] + (int64_t)P.c_add_sq * nn + P.c_add;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int i = i0 + tx + 16 * a, j = j0 + ty + 16 * q;
      if (i < n && j < n) C[(int64_t)P.c_step * (i + (int64_t)j * n)] = acc[a][q];
    }
}

// Elementwise steps, grid (chunks, count):
//   mode 0 (exp): P = Qr C + Qi S, R = Qi C - Qr S with C, S = cos, sin of mu_j per column;
//   mode 1 (cis): P = Qr D, R = Qi D with D = exp(-mu_j);
//   mode 2 (adjoint): M <- conj(Phi) o M on (Mr, Mi) = work blocks 2, 3, with
//   Phi_jk = exp(i(mu_j + mu_k)/2) sinc((mu_j - mu_k)/2).
__global__ void func_elem_kernel(EigenBatch E, int mode) {
  const int b = blockIdx.y;
  if (E.status[b] == SKEW_NO_CONVERGENCE) return;
  if (E.fsel && E.fsel[b] != 0) return;  // real Schur-basis path
  const int n = E.n[b];
  const int64_t nn = (int64_t)n * n;
  const double* mu = E.vals[b];
  double* w = E.pwork[b];
  const double* Qr = E.Vr[b];
  const double* Qi = E.Vi[b];
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / n), r = (int)(k - (int64_t)j * n);
    if (mode == 0) {  // P = Qr a + Qi b, R = Qi a - Qr b for f(i mu_j) = a + i b
      double fa, fb;
      bool sing = false;
      skew_scalar_func(E.func, mu[j], &fa, &fb, &sing);
      if (sing && r == 0) E.status[b] = SKEW_SINGULAR;
      const double qr = Qr[k], qi = Qi[k];
      w[k] = fma(qr, fa, qi * fb);
      w[nn + k] = fma(qi, fa, -(qr * fb));
    } else if (mode == 1) {
      const double d = exp(neg(mu[j]));
      w[k] = Qr[k] * d;
      w[nn + k] = Qi[k] * d;
    } else {
      const double a = mu[r], bb = mu[j];
      const double dlt = 0.5 * (a - bb);
      const double sc = (fabs(dlt) < 1e-8) ? fma(-dlt * dlt, 1.0 / 6.0, 1.0) : sin(dlt) / dlt;
      double sn, cs;
      sincos(0.5 * (a + bb), &sn, &cs);
      const double pr = cs * sc, pi = -sn * sc;  // conj(Phi)
      const double mr = w[2 * nn + k], mi = w[3 * nn + k];
      w[2 * nn + k] = fma(mr, pr, -(mi * pi));
      w[3 * nn + k] = fma(mr, pi, mi * pr);
    }
  }
}

// F <- (F + s F^T) / 2 in place (s = +1 symmetric part, -1 skew part), grid (chunks, count)
__global__ void symmetrize_kernel(const int32_t* __restrict__ nn_, const int* __restrict__ status,
                                  double* const* F, int s) {
  const int b = blockIdx.y;
  if (status && status[b] == SKEW_NO_CONVERGENCE) return;
  const int n = nn_[b];
  double* A = F[b];
  const int64_t tot = (int64_t)n * n;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(q / n), i = (int)(q - (int64_t)j * n);
    if (i < j) continue;
    if (i == j) {
      if (s < 0) A[q] = 0.0;
      continue;
    }
    const double x = A[i + (int64_t)j * n], y = A[j + (int64_t)i * n];
    const double u = 0.5 * (x + s * y);
    A[i + (int64_t)j * n] = u;
    A[j + (int64_t)i * n] = s * u;
  }
}

static BOperand bop(const double* const* p, int add_sq, int trans) {
  BOperand o;
  o.p = p;
  o.add_sq = add_sq;
  o.trans = trans;
  return o;
}

static cudaError_t bgemm(const EigenBatch& E, int nterms, BOperand A0, BOperand B0, double s0, BOperand A1,
                         BOperand B1, double s1, double* const* C, int c_add_sq, int c_add, int c_step,
                         cudaStream_t st, int sel_val = -1) {
  BGemm P;
  P.n = E.n;
  P.status = E.status;
  P.sel = (sel_val >= 0) ? E.fsel : nullptr;
  P.sel_val = sel_val;
  P.nterms = nterms;
  P.A[0] = A0;
  P.B[0] = B0;
  P.s[0] = s0;
  P.A[1] = A1;
  P.B[1] = B1;
  P.s[1] = s1;
  P.C = C;
  P.c_add_sq = c_add_sq;
  P.c_add = c_add;
  P.c_step = c_step;
  const int nt = (E.nmax + BG_T - 1) / BG_T;
  bgemm_kernel<<<dim3(nt * nt, E.count), 256, 0, st>>>(P);
  return cudaGetLastError();
}

__global__ void copy_ev_kernel(const double* const* ev_in, const int32_t* n, const int64_t* off, int count,
                               double* ev) {
  const int b = blockIdx.y;
  if (b >= count) return;
  const int m = n[b] - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) ev[off[b] + i] = ev_in[b][i];
}

cudaError_t launch_copy_ev(const double* const* ev_in, const int32_t* n, const int64_t* off, int count, double* ev,
                           cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  copy_ev_kernel<<<dim3(4, count), 256, 0, st>>>(ev_in, n, off, count, ev);
  return cudaGetLastError();
}

size_t eigen_work_doubles(int n) {
  return (size_t)std::max<int64_t>(4 * (int64_t)n * n, fallback_ws_doubles(n));
}

__global__ void gather_ev_kernel(const double* __restrict__ ev, const int64_t* __restrict__ off_n,
                                 const int32_t* __restrict__ idx, int n, double* __restrict__ e_g) {
  const int mb = blockIdx.y;
  const double* src = ev + off_n[idx[mb]];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    e_g[(size_t)mb * n + i] = (i + 1 < n) ? src[i] : 0.0;
}

cudaError_t launch_gather_ev(const double* ev, const int64_t* off_n, const int32_t* idx, int n, int G, double* e_g,
                             cudaStream_t st) {
  if (n <= 0 || G <= 0) return cudaSuccess;
  gather_ev_kernel<<<dim3((n + 255) / 256, G), 256, 0, st>>>(ev, off_n, idx, n, e_g);
  return cudaGetLastError();
}

cudaError_t launch_eigen_chain(const EigenBatch& E, cudaStream_t st) {
  if (E.count <= 0) return cudaSuccess;
  eigen_chain_kernel<<<(E.count + 31) / 32, 32, 0, st>>>(E);
  return cudaGetLastError();
}

cudaError_t launch_eigen_vectors(const EigenBatch& E, int grid, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(E.counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  eigen_vectors_kernel<<<grid, ENT, 0, st>>>(E);
  return cudaGetLastError();
}

cudaError_t launch_eigen_back(const EigenBatch& E, int grid, int nmax, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(E.counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  const size_t smem = sizeof(double) * (size_t)EB * 3 * (size_t)nmax;
  static std::atomic<uint64_t> raised{0};
  e = raise_smem_limit_once((const void*)eigen_back_kernel, raised);
  if (e != cudaSuccess) return e;
  eigen_back_kernel<<<grid, ENT, smem, st>>>(E);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Matrix functions and the exp adjoint in the real Schur basis
// ---------------------------------------------------------------------------
// The eigenvectors of a real skew matrix come in conjugate pairs.  For mu > 0 the
// column u = (x + i y)/sqrt(2) gives the orthonormal pair (x, y) = sqrt(2) (Re u,
// Im u) with A x = -mu y and A y = mu x; its partner conj(u) adds nothing.  A zero
// eigenvalue's column is real up to its layout (Re u + Im u).  With Q = [x_1, y_1,
// ..., z_1, ...], A = Q S Q^T (S: blocks mu J, J = [[0, 1], [-1, 0]], and zeros), and
// the adjoint of the Frechet derivative of exp at A is
//   G = Q T' Q^T,  T' = int_0^1 e^{-(1-s) S} (Q^T C Q) e^{-s S} ds,
// block by block in closed form.  A 2 x 2 block M splits into P = aI + bJ, which
// commutes with J, and N = cK + dL (K = diag(1, -1), L = [[0, 1], [1, 0]]), which
// anticommutes with it; rotations pass through P and flip through N, so
//   T'_ab = P (c1 I + s1 J) + N (c2 I + s2 J),
// where (c, s) = sinc(delta) (cos m, sin m) for a rotation angle running linearly
// from phi0 to phi1 (m the mean, delta half the difference): -mu_a -> -mu_b for P,
// mu_a -> -mu_b for N.  A 1 x 2, 2 x 1 or 1 x 1 block (zero eigenvalue) takes the
// same with mu = 0.  Four real n x n products instead of the twelve of the complex
// form.  With tol = 64 eps max|mu|, the columns with mu > tol give two Q columns,
// |mu| <= tol one and mu < -tol none.  A zero eigenvalue that a full tridiagonal
// solve returns as a few ulps (several odd blocks, the Jacobi fallback) is then a
// real single column, not half of a pair; its function value is f(0) (singular for
// log, cot and coth).  If the columns do not number n (+-values that are not
// partners), and for n < 4, the matrix takes the complex form.  The other matrix
// functions use the same basis: for a real function f (f(conj z) = conj f(z)),
// f(mu J) = Re f(i mu) I + Im f(i mu) J, so f(A) = (Q f(S)) Q^T is one product, and
// cis(A) = exp(i A) = Q (cosh(mu) I + i sinh(mu) J) Q^T two.
//
// Workspace per matrix (pwork, 4 n^2): Q | T' (and C Q, Q f(S)) | T (and Q T', Q i sinh)
// | metadata: per eigenvector column and per block a code, 2 p + 1 for a pair starting
// at Q column p and 2 p for a single column (-1: a skipped partner column), per block
// its mu, and the block count.

constexpr int SB_NT = 256;

__device__ __forceinline__ void rot_mean(double phi0, double phi1, double* c, double* s) {
  const double d = 0.5 * (phi1 - phi0);
  const double sc = (fabs(d) < 1e-8) ? fma(-d * d, 1.0 / 6.0, 1.0) : sin(d) / d;
  double sn, cs;
  sincos(0.5 * (phi0 + phi1), &sn, &cs);
  *c = cs * sc;
  *s = sn * sc;
}

// One CTA per matrix: the column map (block-wide scans of the widths 2 / 1 / 0).
// colp[j] = 2 p + 1 for a pair starting at Q column p, 2 p for a single column,
// -1 for a skipped partner.
__global__ void __launch_bounds__(SB_NT) schur_scan_kernel(EigenBatch E) {
  const int b = blockIdx.x;
  const int n = E.n[b];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (E.status[b] == SKEW_NO_CONVERGENCE || n < 4) {
    if (tid == 0) E.fsel[b] = 0;
    return;
  }
  __shared__ double red[SB_NT / 32];
  __shared__ long long wsum[SB_NT / 32];
  const double* mu = E.vals[b];
  const int64_t nn = (int64_t)n * n;
  double* meta = E.pwork[b] + 3 * nn;
  double* colp = meta;       // per eigenvector column
  double* bmu = meta + n;    // per block
  double* bst = meta + 2 * n;
  double mx = 0.0;
  for (int j = tid; j < n; j += SB_NT) mx = fmax(mx, fabs(mu[j]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[w] = mx;
  __syncthreads();
  mx = 0.0;
  for (int q = 0; q < SB_NT / 32; q++) mx = fmax(mx, red[q]);
  const double tol = 64.0 * 2.220446049250313e-16 * mx;
  long long base = 0, nblk = 0;
  for (int j0 = 0; j0 < n; j0 += SB_NT) {
    const int j = j0 + tid;
    int wdt = 0;
    if (j < n) wdt = (mu[j] > tol) ? 2 : ((mu[j] < -tol) ? 0 : 1);
    // inclusive scan of (width, is-block) packed as width + 2^32 is-block
    const long long v = (long long)wdt + ((long long)(wdt > 0) << 32);
    long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    __syncthreads();  // the previous chunk's wsum has been read
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    long long before = 0, total = 0;
    for (int q = 0; q < SB_NT / 32; q++) {
      if (q < w) before += wsum[q];
      total += wsum[q];
    }
    const long long excl = before + incl - v;
    if (j < n) {
      const long long p = base + (excl & 0xffffffffLL), a = nblk + (excl >> 32);
      colp[j] = (wdt == 0) ? -1.0 : (double)(2 * p + (wdt == 2 ? 1 : 0));
      if (wdt > 0) {
        bmu[a] = (wdt == 2) ? mu[j] : 0.0;
        bst[a] = (double)(2 * p + (wdt == 2 ? 1 : 0));
      }
    }
    base += total & 0xffffffffLL;
    nblk += total >> 32;
  }
  if (tid == 0) {
    meta[3 * n] = (double)nblk;
    E.fsel[b] = (base == n) ? 1 : 0;
  }
}

// Q from the eigenvectors, grid (chunks, count): a pair column j gives Q columns
// p, p + 1 = sqrt(2) Re u_j, sqrt(2) Im u_j; a single one gives Re u_j + Im u_j.
__global__ void schur_fill_kernel(EigenBatch E) {
  const int b = blockIdx.y;
  if (E.fsel[b] != 1) return;
  const int n = E.n[b];
  const int64_t nn = (int64_t)n * n;
  double* Q = E.pwork[b];
  const double* colp = Q + 3 * nn;
  const double* Vr = E.Vr[b];
  const double* Vi = E.Vi[b];
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / n), r = (int)(k - (int64_t)j * n);
    const double c = colp[j];
    if (c < 0.0) continue;
    const int64_t code = (int64_t)c, p = code >> 1;
    const double xr = Vr[k], xi = Vi[k];
    if (code & 1) {
      Q[r + p * n] = 1.4142135623730951 * xr;
      Q[r + (p + 1) * n] = 1.4142135623730951 * xi;
    } else {
      Q[r + p * n] = xr + xi;
    }
  }
}

// T' from T block by block, grid (chunks, count): one thread per block pair (a, b).
// T in work block 2, T' into work block 1.
__global__ void schur_map_kernel(EigenBatch E) {
  const int bm = blockIdx.y;
  if (E.fsel[bm] != 1) return;
  const int n = E.n[bm];
  const int64_t nn = (int64_t)n * n;
  const double* meta = E.pwork[bm] + 3 * nn;
  const double* bmu = meta + n;
  const double* bst = meta + 2 * n;
  const int64_t nb = (int64_t)meta[3 * n];
  const double* T = E.pwork[bm] + 2 * nn;
  double* Tp = E.pwork[bm] + nn;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nb * nb; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ia = q % nb, ib = q / nb;  // consecutive threads: consecutive block rows
    const int64_t ca = (int64_t)bst[ia], cb = (int64_t)bst[ib];
    const int64_t ra = ca >> 1, rb = cb >> 1;  // first row (column) of each block
    const bool pa = ca & 1, pb = cb & 1;
    const double ma = bmu[ia], mb = bmu[ib];
    auto t = [&](int64_t i, int64_t j) -> double { return T[i + j * n]; };
    auto o = [&](int64_t i, int64_t j) -> double& { return Tp[i + j * n]; };
    if (pa && pb) {
      const double m00 = t(ra, rb), m01 = t(ra, rb + 1), m10 = t(ra + 1, rb), m11 = t(ra + 1, rb + 1);
      const double al = 0.5 * (m00 + m11), be = 0.5 * (m01 - m10);
      const double ga = 0.5 * (m00 - m11), ep = 0.5 * (m01 + m10);
      double c1, s1, c2, s2;
      rot_mean(-ma, -mb, &c1, &s1);
      rot_mean(ma, -mb, &c2, &s2);
      const double A = fma(al, c1, -(be * s1)), B = fma(al, s1, be * c1);
      const double Gm = fma(ga, c2, -(ep * s2)), Ep = fma(ga, s2, ep * c2);
      o(ra, rb) = A + Gm;
      o(ra, rb + 1) = B + Ep;
      o(ra + 1, rb) = Ep - B;
      o(ra + 1, rb + 1) = A - Gm;
    } else if (pb) {  // single row a, pair b
      double c1, s1;
      rot_mean(0.0, -mb, &c1, &s1);
      const double m0 = t(ra, rb), m1 = t(ra, rb + 1);
      o(ra, rb) = fma(m0, c1, -(m1 * s1));
      o(ra, rb + 1) = fma(m0, s1, m1 * c1);
    } else if (pa) {  // pair a, single column b
      double c1, s1;
      rot_mean(-ma, 0.0, &c1, &s1);
      const double m0 = t(ra, rb), m1 = t(ra + 1, rb);
      o(ra, rb) = fma(c1, m0, s1 * m1);
      o(ra + 1, rb) = fma(c1, m1, -(s1 * m0));
    } else {
      o(ra, rb) = t(ra, rb);
    }
  }
}

// Q f(S) (mode 0: f = E.func, into work block 1) or Q cosh(S) and Q i sinh(S) (mode 1:
// blocks 1 and 2), grid (chunks, count); one thread per (row, block).
__global__ void schur_func_kernel(EigenBatch E, int mode) {
  const int bm = blockIdx.y;
  if (E.fsel[bm] != 1) return;
  const int n = E.n[bm];
  const int64_t nn = (int64_t)n * n;
  const double* Q = E.pwork[bm];
  double* P1 = E.pwork[bm] + nn;
  double* P2 = E.pwork[bm] + 2 * nn;
  const double* meta = Q + 3 * nn;
  const double* bmu = meta + n;
  const double* bst = meta + 2 * n;
  const int64_t nb = (int64_t)meta[3 * n];
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nb * n; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = q / n, r = q - a * n;  // consecutive threads: consecutive rows
    const int64_t code = (int64_t)bst[a], p = code >> 1;
    const bool pair = code & 1;
    const double mu = bmu[a];
    const double x = Q[r + p * n];
    const double y = pair ? Q[r + (p + 1) * n] : 0.0;
    if (mode == 0) {  // [x, y] (a I + b J) = [a x - b y, b x + a y] with f(i mu) = a + i b
      double fa, fb;
      bool sing = false;
      skew_scalar_func(E.func, mu, &fa, &fb, &sing);
      if (sing && r == 0) E.status[bm] = SKEW_SINGULAR;
      if (pair) {
        P1[r + p * n] = fma(fa, x, -(fb * y));
        P1[r + (p + 1) * n] = fma(fb, x, fa * y);
      } else {
        P1[r + p * n] = fa * x;
      }
    } else {  // cosh(mu) [x, y] and sinh(mu) [x, y] J = sinh(mu) [-y, x]
      const double ch = cosh(mu), sh = sinh(mu);
      P1[r + p * n] = ch * x;
      P2[r + p * n] = -(sh * y);
      if (pair) {
        P1[r + (p + 1) * n] = ch * y;
        P2[r + (p + 1) * n] = sh * x;
      }
    }
  }
}

cudaError_t launch_schur_basis(const EigenBatch& E, cudaStream_t st) {
  if (E.count <= 0 || !E.fsel) return cudaSuccess;
  const int64_t nn = (int64_t)E.nmax * E.nmax;
  const int chunks = (int)std::min<int64_t>((nn + 255) / 256, 512);
  schur_scan_kernel<<<E.count, SB_NT, 0, st>>>(E);
  schur_fill_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E);
  return cudaGetLastError();
}

cudaError_t launch_eigen_func(const EigenBatch& E, int mode, cudaStream_t st) {
  if (E.count <= 0) return cudaSuccess;
  const int64_t nn = (int64_t)E.nmax * E.nmax;
  const int chunks = (int)std::min<int64_t>((nn + 255) / 256, 512);
  const double* const* Vr = E.Vr;
  const double* const* Vi = E.Vi;
  const double* const* W = E.pwork;
  cudaError_t e;
  const int cx = E.fsel ? 0 : -1;  // the complex form runs for fsel = 0 (every matrix without fsel)
  if (E.fsel && mode != 2) {  // real Schur basis: F = (Q f(S)) Q^T, cis = Q (cosh S + i sinh(S) J) Q^T
    if (!E.back_q && (e = launch_schur_basis(E, st))) return e;
    schur_func_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E, mode);
    if ((e = cudaGetLastError())) return e;
    const int step = mode == 0 ? 1 : 2;
    if ((e = bgemm(E, 1, bop(W, 1, 0), bop(W, 0, 1), 1.0, bop(W, 1, 0), bop(W, 0, 1), 0.0, E.out, 0, 0, step, st, 1)))
      return e;
    if (mode == 1 &&
        (e = bgemm(E, 1, bop(W, 2, 0), bop(W, 0, 1), 1.0, bop(W, 2, 0), bop(W, 0, 1), 0.0, E.out, 0, 1, 2, st, 1)))
      return e;
  }
  if (mode == 0) {  // F = Qr P^T + Qi R^T = Re(V f V^H), then its (skew-)symmetric part
    func_elem_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E, 0);
    e = bgemm(E, 2, bop(Vr, 0, 0), bop(W, 0, 1), 1.0, bop(Vi, 0, 0), bop(W, 1, 1), 1.0, E.out, 0, 0, 1, st, cx);
    if (e != cudaSuccess) return e;
    const int sym = skew_func_symmetry(E.func);
    if (sym != 0) {
      symmetrize_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E.n, E.status, E.out, sym);
      e = cudaGetLastError();
    }
    return e;
  }
  if (mode == 1) {  // Re = Qr P^T + Qi R^T, Im = Qi P^T - Qr R^T, interleaved
    func_elem_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E, 1);
    e = bgemm(E, 2, bop(Vr, 0, 0), bop(W, 0, 1), 1.0, bop(Vi, 0, 0), bop(W, 1, 1), 1.0, E.out, 0, 0, 2, st, cx);
    if (e != cudaSuccess) return e;
    return bgemm(E, 2, bop(Vi, 0, 0), bop(W, 0, 1), 1.0, bop(Vr, 0, 0), bop(W, 1, 1), -1.0, E.out, 0, 1, 2, st, cx);
  }
  const double* const* C = E.cot;
  double* const* Wm = E.pwork;
  // real Schur basis (matrices with fsel = 1): Q, T = Q^T (C Q), T', G = (Q T') Q^T
  if (E.fsel) {
    if (!E.back_q && (e = launch_schur_basis(E, st))) return e;
    if ((e = bgemm(E, 1, bop(C, 0, 0), bop(W, 0, 0), 1.0, bop(C, 0, 0), bop(W, 0, 0), 0.0, Wm, 1, 0, 1, st, 1)))
      return e;  // C Q
    if ((e = bgemm(E, 1, bop(W, 0, 1), bop(W, 1, 0), 1.0, bop(W, 0, 1), bop(W, 1, 0), 0.0, Wm, 2, 0, 1, st, 1)))
      return e;  // T = Q^T (C Q)
    schur_map_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E);
    if ((e = cudaGetLastError())) return e;
    if ((e = bgemm(E, 1, bop(W, 0, 0), bop(W, 1, 0), 1.0, bop(W, 0, 0), bop(W, 1, 0), 0.0, Wm, 2, 0, 1, st, 1)))
      return e;  // Q T'
    if ((e = bgemm(E, 1, bop(W, 2, 0), bop(W, 0, 1), 1.0, bop(W, 2, 0), bop(W, 0, 1), 0.0, E.out, 0, 0, 1, st, 1)))
      return e;  // G = (Q T') Q^T
  }
  // complex form: Y = Cbar V, M = V^H Y, M <- conj(Phi) o M, Z = V M, G = Re(Z V^H)
  if ((e = bgemm(E, 1, bop(C, 0, 0), bop(Vr, 0, 0), 1.0, bop(C, 0, 0), bop(Vr, 0, 0), 0.0, Wm, 0, 0, 1, st, cx)))
    return e;  // Yr
  if ((e = bgemm(E, 1, bop(C, 0, 0), bop(Vi, 0, 0), 1.0, bop(C, 0, 0), bop(Vi, 0, 0), 0.0, Wm, 1, 0, 1, st, cx)))
    return e;  // Yi
  if ((e = bgemm(E, 2, bop(Vr, 0, 1), bop(W, 0, 0), 1.0, bop(Vi, 0, 1), bop(W, 1, 0), 1.0, Wm, 2, 0, 1, st, cx)))
    return e;  // Mr = Qr^T Yr + Qi^T Yi
  if ((e = bgemm(E, 2, bop(Vr, 0, 1), bop(W, 1, 0), 1.0, bop(Vi, 0, 1), bop(W, 0, 0), -1.0, Wm, 3, 0, 1, st, cx)))
    return e;  // Mi = Qr^T Yi - Qi^T Yr
  func_elem_kernel<<<dim3(chunks, E.count), 256, 0, st>>>(E, 2);
  if ((e = cudaGetLastError())) return e;
  if ((e = bgemm(E, 2, bop(Vr, 0, 0), bop(W, 2, 0), 1.0, bop(Vi, 0, 0), bop(W, 3, 0), -1.0, Wm, 0, 0, 1, st, cx)))
    return e;  // Zr = Qr Mr - Qi Mi
  if ((e = bgemm(E, 2, bop(Vr, 0, 0), bop(W, 3, 0), 1.0, bop(Vi, 0, 0), bop(W, 2, 0), 1.0, Wm, 1, 0, 1, st, cx)))
    return e;  // Zi = Qr Mi + Qi Mr
  return bgemm(E, 2, bop(W, 0, 0), bop(Vr, 0, 1), 1.0, bop(W, 1, 0), bop(Vi, 0, 1), 1.0, E.out, 0, 0, 1, st, cx);
}

}  // namespace skew
