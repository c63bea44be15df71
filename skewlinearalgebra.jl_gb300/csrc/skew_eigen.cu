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
//   back    V <- Q V for both parts (eigen.jl:348-352) by compact-WY blocks of 8
//           reflectors: Y = V_b^T X, Z = T_b Y, X -= V_b Z.
//   exp     E = Qr P^T + Qi R^T with P = Qr C + Qi S, R = Qi C - Qr S
//           (C, S = cos, sin of the eigenvalues; exp.jl:3-35 reassociated).
//   cis     V diag(exp(-Im lambda)) V^H (exp.jl:99-110), two real products.
//   vjp     d<Gbar, exp(A)>/dA = Re(V (conj(Phi) o (V^H Gbar V)) V^H) with the
//           Daleckii-Krein divided differences Phi_jk of exp on the i*mu
//           spectrum, evaluated as exp(i(mu_j+mu_k)/2) sinc((mu_j-mu_k)/2).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"
#include "skew_internal.h"

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
  for (int i = first; i <= n - 1; i++) {
    const double a = (i > start ? ev[i - 2] : 0.0);
    const double b = ev[i - 1];
    const double g = ev[i];
    double c, s;
    if (i > start) {
      givens_e(a, bulge, c, s);
    } else {
      const double x1 = __dadd_rn(__dsub_rn(neg(__dmul_rn(a, a)), __dmul_rn(b, b)), shift);
      const double x2 = __dadd_rn(neg(__dmul_rn(a, bulge)), __dmul_rn(b, g));
      givens_e(x1, x2, c, s);
    }
    if (i > 1) ev[i - 2] = __dadd_rn(__dmul_rn(c, a), __dmul_rn(s, bulge));
    ev[i - 1] = __dsub_rn(__dmul_rn(c, b), __dmul_rn(s, g));
    ev[i] = __dadd_rn(__dmul_rn(s, b), __dmul_rn(c, g));
    if (i < n - 1) {
      const double z = ev[i + 1];
      ev[i + 1] = __dmul_rn(z, c);
      bulge = __dmul_rn(s, z);
      if (fabs(bulge) < tol && fabs(ev[i - 1]) < tol) start = i + 1;
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
    const int max_iter = 30 * n;
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
      if (n > 2 && fabs(ev[n - 2] - mem) < tol) {  // skeweigen.jl:355-358
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

// Cyclic Jacobi on the dense symmetric tridiagonal SymTridiagonal(0, e) (size
// n <= 1024) in S (n x n, ld n); eigenvectors accumulate in Z.  Round-robin
// pairing makes the rotations of one round disjoint.  Eigenvalues returned
// ascending in w with Z's columns permuted to match.  The stagnation fallback
// of the QR (rare).
__device__ void jacobi_symtri(const double* e, int n, double* S, double* Z, double* w, int* perm, double* rc,
                              double* rs, int* pp, int* pq) {
  const int tid = threadIdx.x;
  for (int64_t k = tid; k < (int64_t)n * n; k += ENT) {
    const int j = (int)(k / n), i = (int)(k - (int64_t)j * n);
    S[k] = (i == j + 1) ? e[j] : ((j == i + 1) ? e[i] : 0.0);
    Z[k] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  const int m = n + (n & 1);  // players, one dummy when n is odd
  __shared__ double s_off, s_tot;
  if (tid == 0) {
    double t2 = 0.0;
    for (int i = 0; i + 1 < n; i++) t2 = fma(e[i], e[i], t2);
    s_tot = 2.0 * t2;
  }
  __syncthreads();
  for (int sweep = 0; sweep < 60; sweep++) {
    if (tid == 0) s_off = 0.0;
    __syncthreads();
    double part = 0.0;
    for (int64_t k = tid; k < (int64_t)n * n; k += ENT) {
      const int j = (int)(k / n), i = (int)(k - (int64_t)j * n);
      if (i != j) part = fma(S[k], S[k], part);
    }
    part = warp_sum(part);
    if ((tid & 31) == 0) atomicAdd(&s_off, part);
    __syncthreads();
    if (s_off <= 1e-30 * s_tot) break;
    for (int round = 0; round < m - 1; round++) {
      // pairs of the round: (0, round+1) rotated schedule
      for (int k = tid; k < m / 2; k += ENT) {
        int a = (k == 0) ? 0 : ((round + k) % (m - 1)) + 1;
        int b = ((round + m - 1 - k) % (m - 1)) + 1;
        if (k == 0) b = ((round) % (m - 1)) + 1;
        int p = min(a, b), q = max(a, b);
        double c = 1.0, s = 0.0;
        if (q < n && p != q) {
          const double apq = S[p + (int64_t)q * n];
          if (apq != 0.0) {
            const double app = S[p + (int64_t)p * n], aqq = S[q + (int64_t)q * n];
            const double theta = (aqq - app) / (2.0 * apq);
            double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
            c = 1.0 / sqrt(fma(t, t, 1.0));
            s = t * c;
          }
        } else {
          p = q = -1;
        }
        pp[k] = p;
        pq[k] = q;
        rc[k] = c;
        rs[k] = s;
      }
      __syncthreads();
      // columns p, q of S and Z:  [x_p, x_q] <- [c x_p - s x_q, s x_p + c x_q]
      for (int64_t idx = tid; idx < (int64_t)(m / 2) * n; idx += ENT) {
        const int k = (int)(idx / n), r = (int)(idx - (int64_t)k * n);
        const int p = pp[k], q = pq[k];
        if (p < 0) continue;
        const double c = rc[k], s = rs[k];
        double* sp = S + (int64_t)p * n + r;
        double* sq = S + (int64_t)q * n + r;
        const double x = *sp, y = *sq;
        *sp = c * x - s * y;
        *sq = s * x + c * y;
        double* zp = Z + (int64_t)p * n + r;
        double* zq = Z + (int64_t)q * n + r;
        const double u = *zp, v = *zq;
        *zp = c * u - s * v;
        *zq = s * u + c * v;
      }
      __syncthreads();
      // rows p, q of S
      for (int64_t idx = tid; idx < (int64_t)(m / 2) * n; idx += ENT) {
        const int k = (int)(idx / n), col = (int)(idx - (int64_t)k * n);
        const int p = pp[k], q = pq[k];
        if (p < 0) continue;
        const double c = rc[k], s = rs[k];
        double* sp = S + p + (int64_t)col * n;
        double* sq = S + q + (int64_t)col * n;
        const double x = *sp, y = *sq;
        *sp = c * x - s * y;
        *sq = s * x + c * y;
      }
      __syncthreads();
    }
  }
  // sort eigenvalues ascending (selection by rank; n <= 1024)
  for (int i = tid; i < n; i += ENT) {
    const double di = S[i + (int64_t)i * n];
    int rank = 0;
    for (int j = 0; j < n; j++) {
      const double dj = S[j + (int64_t)j * n];
      rank += (dj < di) || (dj == di && j < i);
    }
    perm[rank] = i;
  }
  __syncthreads();
  for (int i = tid; i < n; i += ENT) w[i] = S[perm[i] + (int64_t)perm[i] * n];
  __syncthreads();
}

__global__ void __launch_bounds__(ENT) eigen_vectors_kernel(EigenBatch E) {
  __shared__ int s_next;
  __shared__ int s_type[1024 + 1];  // per output column: -1 none, 0..3 kinds (see below)
  __shared__ int s_src[1024 + 1];
  __shared__ double rc[512], rs[512];
  __shared__ int pp[512], pq[512];
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(E.counter, 1u);
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= E.count) break;
    const int b = E.order[t];
    const int N = E.n[b];
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
      // skewtrieigen_backup! (:470-489) from the original ev
      double* S = work;
      double* Z = work + (int64_t)N * N;
      double* w = E.ev + E.off_n[b];  // reuse: the QR's ev copy is no longer needed
      int* perm = (int*)(E.G + E.off_n[b]);
      jacobi_symtri(E.evb + E.off_n[b], N, S, Z, w, perm, rc, rs, pp, pq);
      double* vals = E.vals[b];
      for (int j = threadIdx.x; j < N; j += ENT) vals[j] = neg(w[j]);
      for (int64_t k = threadIdx.x; k < (int64_t)N * N; k += ENT) {
        const int j = (int)(k / N), i = (int)(k - (int64_t)j * N);
        const double z = Z[i + (int64_t)perm[j] * N];
        const int pair = i >> 1;
        const double c = (pair & 1) ? -1.0 : 1.0;  // c flips after every (odd, even) pair
        if ((N & 1) && i == N - 1) {
          Vr[i + (int64_t)j * ldv] = c * z;
        } else if ((i & 1) == 0) {
          Vr[i + (int64_t)j * ldv] = c * z;
        } else {
          Vi[i + (int64_t)j * ldv] = c * z;
        }
      }
      __syncthreads();
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
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(E.counter, 1u);
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= E.count) break;
    const int b = E.order[t];
    const int n = E.n[b];
    const int64_t ldv = E.n[b];
    const double* R = E.refl[b];  // n x n, ld n
    const double* tau = E.tau + E.off_n[b];
    if (E.status[b] == SKEW_NO_CONVERGENCE || n < 3) continue;
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
      // Y = V^T X (EB x 2n), then Z = T Y; thread per column of X = [Vr | Vi]
      for (int col = threadIdx.x; col < 2 * n; col += ENT) {
        const double* x = (col < n) ? (E.Vr[b] + (int64_t)col * ldv) : (E.Vi[b] + (int64_t)(col - n) * ldv);
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
      // X[r, col] -= sum_l V[r, l] Z[l, col] for r >= r0; lanes are rows
      for (int col = threadIdx.x >> 5; col < 2 * n; col += ENW) {
        double* x = (col < n) ? (E.Vr[b] + (int64_t)col * ldv) : (E.Vi[b] + (int64_t)(col - n) * ldv);
        double z[EB];
#pragma unroll
        for (int l = 0; l < EB; l++) z[l] = Zs[l * 2 * n + col];
        for (int rr = threadIdx.x & 31; rr < m; rr += 32) {
          double acc = x[r0 + rr];
#pragma unroll
          for (int l = 0; l < EB; l++) acc = fma(-Vs[rr * EB + l], z[l], acc);
          x[r0 + rr] = acc;
        }
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Per-CTA product  C[i,j] = sum_s sgn_s sum_k L_s(i,k) R_s(k,j)  over 64 x 64
// tiles; operands are strided views (transposes are stride swaps).
// ---------------------------------------------------------------------------
struct Opnd {
  const double* p;
  int64_t rs, cs;  // element (i, k) at p[i*rs + k*cs]
  __device__ __forceinline__ double at(int i, int k) const { return p[i * rs + k * cs]; }
};

__device__ void cta_product(int n, int K, int ns, const Opnd* L, const Opnd* R, const double* sgn, double* C,
                            int64_t crs, int64_t ccs, double* sbuf) {
  constexpr int TT = 64, KC = 16;
  double (*sL)[TT] = reinterpret_cast<double (*)[TT]>(sbuf);
  double (*sR)[TT] = reinterpret_cast<double (*)[TT]>(sbuf + KC * TT);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int nt = (n + TT - 1) / TT;
  for (int tile = 0; tile < nt * nt; tile++) {
    const int ti = tile % nt, tj = tile / nt;
    const int R0 = ti * TT, C0 = tj * TT;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[a][q] = 0.0;
    for (int sidx = 0; sidx < ns; sidx++) {
      const double sg = sgn[sidx];
      for (int k0 = 0; k0 < K; k0 += KC) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < KC * TT; idx += ENT) {
          const int kk = idx / TT, rr = idx - kk * TT;
          const int k = k0 + kk;
          const int gi = R0 + rr, gj = C0 + rr;
          sL[kk][rr] = (k < K && gi < n) ? sg * L[sidx].at(gi, k) : 0.0;
          sR[kk][rr] = (k < K && gj < n) ? R[sidx].at(k, gj) : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < KC; kk++) {
          double l4[4], r4[4];
#pragma unroll
          for (int a = 0; a < 4; a++) {
            l4[a] = sL[kk][tx + 16 * a];
            r4[a] = sR[kk][ty + 16 * a];
          }
#pragma unroll
          for (int a = 0; a < 4; a++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[a][q] = fma(l4[a], r4[q], acc[a][q]);
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int gi = R0 + tx + 16 * a, gj = C0 + ty + 16 * q;
        if (gi < n && gj < n) C[gi * crs + gj * ccs] = acc[a][q];
      }
  }
  __syncthreads();
}

// exp / cis / exp-vjp assembly from (vals, Vr, Vi).  mode 0: exp -> E (real, lde);
// mode 1: cis -> Cz (complex interleaved, ldc complex); mode 2: vjp of exp with
// cotangent Gbar -> G (real).
__global__ void __launch_bounds__(ENT) eigen_func_kernel(EigenBatch E, int mode) {
  __shared__ int s_next;
  __shared__ double sbuf[2 * 16 * 64];
  for (;;) {
    if (threadIdx.x == 0) s_next = (int)atomicAdd(E.counter, 1u);
    __syncthreads();
    const int t = s_next;
    __syncthreads();
    if (t >= E.count) break;
    const int b = E.order[t];
    const int n = E.n[b];
    const int64_t ldv = E.n[b];
    const double* Qr = E.Vr[b];
    const double* Qi = E.Vi[b];
    const double* mu = E.vals[b];
    double* work = E.work + E.off_w[b];  // >= 4 n^2 doubles
    if (E.status[b] == SKEW_NO_CONVERGENCE) continue;
    const int64_t nn = (int64_t)n * n;
    if (mode == 0) {
      // P = Qr C + Qi S, R = Qi C - Qr S (column scalings); E = Qr P^T + Qi R^T
      double* P = work;
      double* R = work + nn;
      for (int64_t k = threadIdx.x; k < nn; k += ENT) {
        const int j = (int)(k / n), i = (int)(k - (int64_t)j * n);
        double sn, cs;
        sincos(mu[j], &sn, &cs);
        const double qr = Qr[i + (int64_t)j * ldv], qi = Qi[i + (int64_t)j * ldv];
        P[k] = fma(qr, cs, qi * sn);
        R[k] = fma(qi, cs, -(qr * sn));
      }
      __syncthreads();
      Opnd L[2] = {{Qr, 1, ldv}, {Qi, 1, ldv}};
      Opnd Rt[2] = {{P, n, 1}, {R, n, 1}};  // (k, j) -> P[j, k]
      const double sg[2] = {1.0, 1.0};
      cta_product(n, n, 2, L, Rt, sg, E.out[b], 1, n, sbuf);
    } else if (mode == 1) {
      // D = exp(-mu); Re = Qr D Qr^T + Qi D Qi^T, Im = Qi D Qr^T - Qr D Qi^T
      double* P = work;       // Qr D
      double* R = work + nn;  // Qi D
      for (int64_t k = threadIdx.x; k < nn; k += ENT) {
        const int j = (int)(k / n), i = (int)(k - (int64_t)j * n);
        const double d = exp(neg(mu[j]));
        P[k] = Qr[i + (int64_t)j * ldv] * d;
        R[k] = Qi[i + (int64_t)j * ldv] * d;
      }
      __syncthreads();
      double* Cz = E.out[b];
      const int64_t ldc = n;  // in complex elements
      Opnd L[2] = {{Qr, 1, ldv}, {Qi, 1, ldv}};
      Opnd Rt[2] = {{P, n, 1}, {R, n, 1}};
      const double sg[2] = {1.0, 1.0};
      cta_product(n, n, 2, L, Rt, sg, Cz, 2, 2 * ldc, sbuf);
      Opnd L2[2] = {{Qi, 1, ldv}, {Qr, 1, ldv}};
      const double sg2[2] = {1.0, -1.0};
      cta_product(n, n, 2, L2, Rt, sg2, Cz + 1, 2, 2 * ldc, sbuf);
    } else {
      // Y = Gbar V, M = V^H Y, M <- conj(Phi) o M, Z = V M, G = Re(Z V^H)
      const double* Gb = E.cot[b];  // n x n, ld n
      double* Yr = work;
      double* Yi = work + nn;
      double* Mr = work + 2 * nn;
      double* Mi = work + 3 * nn;
      {
        Opnd L[1] = {{Gb, 1, n}};
        Opnd R1[1] = {{Qr, 1, ldv}};
        const double one[1] = {1.0};
        cta_product(n, n, 1, L, R1, one, Yr, 1, n, sbuf);
        Opnd R2[1] = {{Qi, 1, ldv}};
        cta_product(n, n, 1, L, R2, one, Yi, 1, n, sbuf);
      }
      {  // M = (Qr^T - i Qi^T)(Yr + i Yi): Mr = Qr^T Yr + Qi^T Yi, Mi = Qr^T Yi - Qi^T Yr
        Opnd L[2] = {{Qr, ldv, 1}, {Qi, ldv, 1}};
        Opnd R1[2] = {{Yr, 1, n}, {Yi, 1, n}};
        const double pp2[2] = {1.0, 1.0};
        cta_product(n, n, 2, L, R1, pp2, Mr, 1, n, sbuf);
        Opnd R2[2] = {{Yi, 1, n}, {Yr, 1, n}};
        const double pm[2] = {1.0, -1.0};
        cta_product(n, n, 2, L, R2, pm, Mi, 1, n, sbuf);
      }
      // M_jk *= conj(Phi_jk), Phi_jk = exp(i(mu_j+mu_k)/2) sinc((mu_j-mu_k)/2)
      for (int64_t k = threadIdx.x; k < nn; k += ENT) {
        const int c = (int)(k / n), r = (int)(k - (int64_t)c * n);
        const double a = mu[r], bb = mu[c];
        const double d = 0.5 * (a - bb);
        const double sc = (fabs(d) < 1e-8) ? fma(-d * d, 1.0 / 6.0, 1.0) : sin(d) / d;
        double sn, cs;
        sincos(0.5 * (a + bb), &sn, &cs);
        const double pr = cs * sc, pi = -sn * sc;  // conj(Phi)
        const double mr = Mr[k], mi = Mi[k];
        Mr[k] = fma(mr, pr, -(mi * pi));
        Mi[k] = fma(mr, pi, mi * pr);
      }
      __syncthreads();
      {  // Z = (Qr + i Qi)(Mr + i Mi): Zr = Qr Mr - Qi Mi, Zi = Qr Mi + Qi Mr  (into Yr, Yi)
        Opnd L[2] = {{Qr, 1, ldv}, {Qi, 1, ldv}};
        Opnd R1[2] = {{Mr, 1, n}, {Mi, 1, n}};
        const double pm[2] = {1.0, -1.0};
        cta_product(n, n, 2, L, R1, pm, Yr, 1, n, sbuf);
        Opnd R2[2] = {{Mi, 1, n}, {Mr, 1, n}};
        const double pp2[2] = {1.0, 1.0};
        cta_product(n, n, 2, L, R2, pp2, Yi, 1, n, sbuf);
      }
      {  // G = Re((Zr + i Zi)(Qr^T - i Qi^T)) = Zr Qr^T + Zi Qi^T
        Opnd L[2] = {{Yr, 1, n}, {Yi, 1, n}};
        Opnd R1[2] = {{Qr, ldv, 1}, {Qi, ldv, 1}};  // (k, j) -> Q[j, k]
        const double pp2[2] = {1.0, 1.0};
        cta_product(n, n, 2, L, R1, pp2, E.out[b], 1, n, sbuf);
      }
    }
  }
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

cudaError_t launch_eigen_func(const EigenBatch& E, int grid, int mode, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(E.counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  eigen_func_kernel<<<grid, ENT, 0, st>>>(E, mode);
  return cudaGetLastError();
}

}  // namespace skew
