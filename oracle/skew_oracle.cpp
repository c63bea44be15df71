// ORACLE -- test infrastructure only.
//
// A CPU restatement of SkewLinearAlgebra.jl's skew-Householder pipeline, used as
// the checker for the CUDA library: tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py may load it; the product never does.
//
// Every routine is templated on the real type T and instantiated twice:
//   * T = double : the FP64 restatement, following the reference's operation order
//                  (same blocking, same reflector convention, same QR tolerances);
//   * T = quad   : the same algorithm in IEEE binary128 (__float128 on x86-64,
//                  long double on aarch64).  This is the stand-in for the
//                  reference's BigFloat runs: ~34 significant digits.
// Extra independent checks that do not follow the reference's algorithm:
//   * Gauss-Jordan inverse in quad (for the log|Pf| gradient 1/2 A^-T),
//   * Taylor/scaling-squaring exp in quad of the 2n x 2n block matrix
//     [[A^T, C], [0, A^T]] (for the exp adjoint),
//   * cyclic Jacobi for the symmetric tridiagonal eigenproblem used by the
//     reference's LAPACK-backed stagnation fallback (skeweigen.jl:463-489).
//
// Layout: column-major, leading dimension n, 0-based indices (the reference is
// 1-based; each routine cites the lines it follows).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <vector>
#include <algorithm>
#include <limits>

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 quad;
static inline quad qsqrt(quad x) { return sqrtq(x); }
static inline quad qlog(quad x) { return logq(x); }
static inline quad qabs(quad x) { return fabsq(x); }
static inline quad qhypot(quad a, quad b) { return hypotq(a, b); }
static inline quad qsin(quad x) { return sinq(x); }
static inline quad qcos(quad x) { return cosq(x); }
static inline quad qexp(quad x) { return expq(x); }
static inline quad qatan2(quad y, quad x) { return atan2q(y, x); }
static const quad QEPS = (quad)1 / ((quad)(1ULL << 56) * (quad)(1ULL << 56));  // 2^-112
#else
typedef long double quad;  // IEEE binary128 on aarch64 Linux
static inline quad qsqrt(quad x) { return sqrtl(x); }
static inline quad qlog(quad x) { return logl(x); }
static inline quad qabs(quad x) { return fabsl(x); }
static inline quad qhypot(quad a, quad b) { return hypotl(a, b); }
static inline quad qsin(quad x) { return sinl(x); }
static inline quad qcos(quad x) { return cosl(x); }
static inline quad qexp(quad x) { return expl(x); }
static inline quad qatan2(quad y, quad x) { return atan2l(y, x); }
static const quad QEPS = (quad)1 / ((quad)(1ULL << 56) * (quad)(1ULL << 56));  // 2^-112
#endif

template <typename T> struct M;
template <> struct M<double> {
  static double sqrt(double x) { return std::sqrt(x); }
  static double log(double x) { return std::log(x); }
  static double abs(double x) { return std::fabs(x); }
  static double hypot(double a, double b) { return std::hypot(a, b); }
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double exp(double x) { return std::exp(x); }
  static double atan2(double y, double x) { return std::atan2(y, x); }
  static double pi() { return 3.141592653589793; }
  static double eps() { return std::numeric_limits<double>::epsilon(); }
};
template <> struct M<quad> {
  static quad sqrt(quad x) { return qsqrt(x); }
  static quad log(quad x) { return qlog(x); }
  static quad abs(quad x) { return qabs(x); }
  static quad hypot(quad a, quad b) { return qhypot(a, b); }
  static quad sin(quad x) { return qsin(x); }
  static quad cos(quad x) { return qcos(x); }
  static quad exp(quad x) { return qexp(x); }
  static quad atan2(quad y, quad x) { return qatan2(y, x); }
  static quad pi() { return qatan2((quad)0, (quad)-1); }
  static quad eps() { return QEPS; }
};

// Minimal complex type usable with both double and quad.
template <typename T> struct cx {
  T re, im;
  cx() : re(0), im(0) {}
  cx(T r) : re(r), im(0) {}
  cx(T r, T i) : re(r), im(i) {}
};
template <typename T> static inline cx<T> operator+(cx<T> a, cx<T> b) { return cx<T>(a.re + b.re, a.im + b.im); }
template <typename T> static inline cx<T> operator-(cx<T> a, cx<T> b) { return cx<T>(a.re - b.re, a.im - b.im); }
template <typename T> static inline cx<T> operator-(cx<T> a) { return cx<T>(-a.re, -a.im); }
template <typename T> static inline cx<T> operator*(cx<T> a, cx<T> b) {
  return cx<T>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> static inline cx<T> operator/(cx<T> a, cx<T> b) {
  T d = b.re * b.re + b.im * b.im;
  return cx<T>((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
template <typename T> static inline cx<T> conj(cx<T> a) { return cx<T>(a.re, -a.im); }
template <typename T> static inline T cabs(cx<T> a) { return M<T>::hypot(a.re, a.im); }
template <typename T> static inline bool is_zero(cx<T> a) { return a.re == 0 && a.im == 0; }
template <typename T> static inline T realpart(cx<T> a) { return a.re; }
template <typename T> static inline T realpart(T a) { return a; }
template <typename T> static inline T cj(T a) { return a; }
template <typename T> static inline cx<T> cj(cx<T> a) { return conj(a); }
template <typename T> static inline bool is_zero(T a) { return a == 0; }
template <typename T> static inline T absval(T a) { return M<T>::abs(a); }
template <typename T> static inline T absval(cx<T> a) { return cabs(a); }

template <typename S> struct RealOf { typedef S type; };
template <typename T> struct RealOf<cx<T>> { typedef T type; };

// ---------------------------------------------------------------------------
// Tridiagonalisation.  Matrices are views (pointer + leading dimension).
// ---------------------------------------------------------------------------
template <typename S> struct View {
  S* p;
  int64_t ld;
  S& operator()(int64_t i, int64_t j) const { return p[i + j * ld]; }
  View sub(int64_t i, int64_t j) const { return View{p + i + j * ld, ld}; }
};

// 2-norm of x[0:n) with a scaled fallback for overflow/underflow (the
// reference calls LinearAlgebra.norm, which scales the same way).
template <typename S> static typename RealOf<S>::type norm2(const S* x, int64_t n) {
  typedef typename RealOf<S>::type T;
  T s = 0;
  for (int64_t i = 0; i < n; i++) {
    T a = absval(x[i]);
    s += a * a;
  }
  T r = M<T>::sqrt(s);
  if (!(r < std::numeric_limits<double>::max()) || r < T(1e-150)) {
    T mx = 0;
    for (int64_t i = 0; i < n; i++) mx = std::max(mx, absval(x[i]));
    if (mx == 0) return 0;
    s = 0;
    for (int64_t i = 0; i < n; i++) {
      T a = absval(x[i]) / mx;
      s += a * a;
    }
    r = mx * M<T>::sqrt(s);
  }
  return r;
}

// householder!  hessenberg.jl:26-44.  x[0:n) becomes v (v[0] = 1); returns tau, beta.
template <typename S>
static void householder(S* x, int64_t n, S* tau_out, typename RealOf<S>::type* beta_out, bool is_complex) {
  typedef typename RealOf<S>::type T;
  if (n == 1 && !is_complex) {  // :27-29 no final 1x1 reflection for the real case
    *tau_out = S(0);
    *beta_out = realpart(x[0]);
    return;
  }
  T xnorm = norm2(x + 1, n - 1);  // :30
  S alpha = x[0];
  if (xnorm != 0 || !is_zero(alpha)) {  // :32
    T ar = realpart(alpha);
    T h = M<T>::hypot(absval(alpha), xnorm);
    T beta = (ar > 0 ? T(-1) : T(1)) * h;  // :33
    S tau = S(1) - alpha / S(beta);        // :34
    S sc = S(1) / (alpha - S(beta));       // :35
    x[0] = S(1);
    for (int64_t i = 1; i < n; i++) x[i] = x[i] * sc;
    *tau_out = tau;
    *beta_out = beta;
  } else {  // :38-41
    for (int64_t i = 0; i < n; i++) x[i] = S(0);
    *tau_out = S(0);
    *beta_out = 0;
  }
}

// skewhess!  hessenberg.jl:70-90 (unblocked, used for the trailing block).
template <typename S>
static void skewhess(View<S> A, int64_t n, S* tau, typename RealOf<S>::type* eta, bool is_complex) {
  std::vector<S> s(n + 1);
  for (int64_t i = 0; i < n - 1; i++) {
    int64_t m = n - i - 1;  // length of v
    S ts;
    typename RealOf<S>::type al;
    S* v = &A(i + 1, i);
    householder(v, m, &ts, &al, is_complex);  // :74
    eta[i] = al;                              // :76
    View<S> B = A.sub(i + 1, i + 1);
    // lefthouseholder!  :64-68: s = B^H v ; B += (-tau') v s^H
    for (int64_t j = 0; j < m; j++) {
      S acc = S(0);
      for (int64_t r = 0; r < m; r++) acc = acc + cj(B(r, j)) * v[r];
      s[j] = acc;
    }
    S mt = -cj(ts);
    if (!is_zero(mt)) {
      for (int64_t j = 0; j < m; j++) {
        S temp = mt * cj(s[j]);
        for (int64_t r = 0; r < m; r++) B(r, j) = B(r, j) + v[r] * temp;
      }
    }
    // s = B v  :78
    for (int64_t r = 0; r < m; r++) s[r] = S(0);
    for (int64_t j = 0; j < m; j++) {
      S vj = v[j];
      for (int64_t r = 0; r < m; r++) s[r] = s[r] + B(r, j) * vj;
    }
    // :80-86
    for (int64_t j = 0; j < m; j++) {
      B(j, j) = B(j, j) - ts * s[j] * cj(v[j]);
      for (int64_t k = j + 1; k < m; k++) {
        B(k, j) = B(k, j) - ts * s[k] * cj(v[j]);
        B(j, k) = -cj(B(k, j));
      }
    }
    tau[i] = ts;  // :87
  }
}

// skewlatrd!  hessenberg.jl:92-131.  A is the view A[i:n, i:n] of size n.
template <typename S>
static void skewlatrd(View<S> A, typename RealOf<S>::type* eta, View<S> W, S* tau, int64_t n, int64_t nb,
                      bool is_complex) {
  std::vector<S> tmp(nb + 1);
  for (int64_t i = 0; i < nb; i++) {
    if (i > 0) {
      // :100 / :106  A[i:n,i] += A[i:n,0:i] * conj(W[i,0:i])
      for (int64_t j = 0; j < i; j++) tmp[j] = cj(W(i, j));
      for (int64_t j = 0; j < i; j++)
        for (int64_t r = i; r < n; r++) A(r, i) = A(r, i) + A(r, j) * tmp[j];
      // :104 / :107  A[i:n,i] -= W[i:n,0:i] * conj(A[i,0:i])
      for (int64_t j = 0; j < i; j++) tmp[j] = cj(A(i, j));
      for (int64_t j = 0; j < i; j++)
        for (int64_t r = i; r < n; r++) A(r, i) = A(r, i) - W(r, j) * tmp[j];
    }
    int64_t m = n - i - 1;
    S ts;
    typename RealOf<S>::type al;
    householder(&A(i + 1, i), m, &ts, &al, is_complex);  // :112
    eta[i] = al;
    S* v = &A(i + 1, i);
    // :114  W[i+1:n,i] = A[i+1:n,i+1:n] * v
    for (int64_t r = i + 1; r < n; r++) W(r, i) = S(0);
    for (int64_t j = 0; j < m; j++) {
      S vj = v[j];
      for (int64_t r = 0; r < m; r++) W(i + 1 + r, i) = W(i + 1 + r, i) + A(i + 1 + r, i + 1 + j) * vj;
    }
    if (i > 0) {
      // :116  W[0:i,i] = W[i+1:n,0:i]^H v
      for (int64_t j = 0; j < i; j++) {
        S acc = S(0);
        for (int64_t r = 0; r < m; r++) acc = acc + cj(W(i + 1 + r, j)) * v[r];
        W(j, i) = acc;
      }
      // :117  W[i+1:n,i] += A[i+1:n,0:i] * W[0:i,i]
      for (int64_t j = 0; j < i; j++) {
        S wj = W(j, i);
        for (int64_t r = 0; r < m; r++) W(i + 1 + r, i) = W(i + 1 + r, i) + A(i + 1 + r, j) * wj;
      }
      // :118  W[0:i,i] = A[i+1:n,0:i]^H v
      for (int64_t j = 0; j < i; j++) {
        S acc = S(0);
        for (int64_t r = 0; r < m; r++) acc = acc + cj(A(i + 1 + r, j)) * v[r];
        W(j, i) = acc;
      }
      // :119  W[i+1:n,i] -= W[i+1:n,0:i] * W[0:i,i]
      for (int64_t j = 0; j < i; j++) {
        S wj = W(j, i);
        for (int64_t r = 0; r < m; r++) W(i + 1 + r, i) = W(i + 1 + r, i) - W(i + 1 + r, j) * wj;
      }
    }
    for (int64_t r = 0; r < m; r++) W(i + 1 + r, i) = W(i + 1 + r, i) * ts;  // :121
    if (is_complex) {                                                         // :123-126
      S d = S(0);
      for (int64_t r = 0; r < m; r++) d = d + cj(W(i + 1 + r, i)) * v[r];
      S a2 = ts * d / S(2);
      for (int64_t r = 0; r < m; r++) W(i + 1 + r, i) = W(i + 1 + r, i) + a2 * v[r];
    }
    tau[i] = ts;
  }
}

// setnb  hessenberg.jl:133-142
static int64_t setnb(int64_t n) {
  if (n <= 12) return std::max<int64_t>(n - 4, 1);
  if (n <= 100) return 10;
  return 60;
}

// skewblockedhess!  hessenberg.jl:144-173.  A (n x n, ld n) is overwritten:
// reflectors below the subdiagonal, v[0] = 1 on the subdiagonal.
template <typename S>
static void skewblockedhess(S* Ap, int64_t n, int64_t lda, S* tau, typename RealOf<S>::type* eta,
                            bool is_complex) {
  if (n <= 0) return;
  View<S> A{Ap, lda};
  int64_t nb = setnb(n);
  std::vector<S> Wb((size_t)n * nb);
  View<S> W{Wb.data(), n};
  int64_t no = std::max<int64_t>(n - nb, 0);
  std::vector<S> Om((size_t)std::max<int64_t>(no * no, 1));
  View<S> Omega{Om.data(), std::max<int64_t>(no, 1)};
  int64_t oldi = 0;  // 1-based as in the reference
  for (int64_t i = 1; i <= n - nb - 1; i += nb) {
    int64_t size = n - i + 1;
    skewlatrd(A.sub(i - 1, i - 1), eta + (i - 1), W, tau + (i - 1), size, nb, is_complex);  // :157
    // :158  Omega = A[i+nb:n, i:i+nb-1] * W[nb+1:size, :]^H
    int64_t mo = n - nb - i + 1;
    for (int64_t c = 0; c < mo; c++)
      for (int64_t r = 0; r < mo; r++) Omega(r, c) = S(0);
    for (int64_t k = 0; k < nb; k++)
      for (int64_t c = 0; c < mo; c++) {
        S w = cj(W(nb + c, k));
        for (int64_t r = 0; r < mo; r++) Omega(r, c) = Omega(r, c) + A(i + nb - 1 + r, i - 1 + k) * w;
      }
    int64_t s = i + nb - 1;  // :159 (1-based)
    for (int64_t k = 1; k <= n - s; k++) {  // :160-166
      S& akk = A(s + k - 1, s + k - 1);
      akk = akk + (Omega(k - 1, k - 1) - cj(Omega(k - 1, k - 1)));
      for (int64_t j = k + 1; j <= n - s; j++) {
        S& ajk = A(s + j - 1, s + k - 1);
        ajk = ajk + (Omega(j - 1, k - 1) - cj(Omega(k - 1, j - 1)));
        A(s + k - 1, s + j - 1) = -cj(ajk);
      }
    }
    oldi = i;
  }
  oldi += nb;
  if (oldi < n) {  // :169-172
    int64_t o = oldi - 1;
    skewhess(A.sub(o, o), n - o, tau + o, eta + o, is_complex);
  }
}

// Q = H_1 ... H_{n-1} from the reflectors stored below the subdiagonal (what
// LinearAlgebra's Matrix(::HessenbergQ) produces via LAPACK orgtr, uplo 'L').
template <typename S> static void formq(const S* Ap, int64_t n, int64_t lda, const S* tau, S* Q) {
  View<const S> A{Ap, lda};
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) Q[i + j * n] = S(i == j ? 1 : 0);
  std::vector<S> v(n), w(n);
  for (int64_t k = n - 2; k >= 0; k--) {  // H_k acts on rows/cols k+1..n-1
    S t = tau[k];
    if (is_zero(t)) continue;
    int64_t m = n - k - 1;
    v[0] = S(1);
    for (int64_t r = 1; r < m; r++) v[r] = A.p[(k + 1 + r) + k * lda];
    // Q[k+1:, k+1:] = (I - t v v^H) Q[k+1:, k+1:]
    for (int64_t j = k + 1; j < n; j++) {
      S acc = S(0);
      for (int64_t r = 0; r < m; r++) acc = acc + cj(v[r]) * Q[(k + 1 + r) + j * n];
      acc = t * acc;
      for (int64_t r = 0; r < m; r++) Q[(k + 1 + r) + j * n] = Q[(k + 1 + r) + j * n] - v[r] * acc;
    }
  }
}

// ---------------------------------------------------------------------------
// Pfaffian.  pfaffian.jl:167-179 (real SkewHermitian).
// sign(det(H.Q)) is (-1)^(number of nonzero tau) for real reflectors with
// tau*|v|^2 = 2, which is what LinearAlgebra computes for a HessenbergQ.
// ---------------------------------------------------------------------------
template <typename T> static T sgn(T x) { return x > 0 ? T(1) : (x < 0 ? T(-1) : T(0)); }

template <typename T> static void logabspf(const double* Ain, int64_t n, double* logpf, double* sign) {
  if (n % 2 == 1) {  // :169
    *logpf = -std::numeric_limits<double>::infinity();
    *sign = 0;
    return;
  }
  if (n == 0) {
    *logpf = 0;
    *sign = 1;
    return;
  }
  std::vector<T> A((size_t)n * n), tau(n), eta(n);
  for (int64_t i = 0; i < n * n; i++) A[i] = T(Ain[i]);
  skewblockedhess<T>(A.data(), n, n, tau.data(), eta.data(), false);
  T lp = 0, sg = 1;
  for (int64_t i = 0; i < n - 1; i += 2) {  // :174-177
    lp += M<T>::log(M<T>::abs(eta[i]));
    sg *= sgn(-eta[i]);
  }
  int64_t nz = 0;
  for (int64_t i = 0; i < n - 1; i++) nz += (tau[i] != 0);
  if (nz & 1) sg = -sg;
  *logpf = (double)lp;
  *sign = (double)sg;
}

// log|Pf| of A + h (e_i e_j^T - e_j e_i^T) in the working type T, returned in T, so
// that a central difference of two such values keeps T's precision (a difference
// of values already rounded to double would lose about 1e-16 |log|Pf|| / h).
template <typename T>
static T logabspf_pair(const double* Ain, int64_t n, int64_t i, int64_t j, T h) {
  std::vector<T> A((size_t)n * n), tau(n), eta(n);
  for (int64_t k = 0; k < n * n; k++) A[k] = T(Ain[k]);
  A[i + j * n] = A[i + j * n] + h;  // column-major A(i, j)
  A[j + i * n] = A[j + i * n] - h;
  skewblockedhess<T>(A.data(), n, n, tau.data(), eta.data(), false);
  T lp = 0;
  for (int64_t k = 0; k < n - 1; k += 2) lp += M<T>::log(M<T>::abs(eta[k]));
  return lp;
}

// ---------------------------------------------------------------------------
// Complex skew-symmetric Pfaffian by Parlett-Reid elimination with pivoting,
// pfaffian.jl:98-137 (_pfaffian!, the running product) and :193-233
// (_logabspfaffian!, log|Pf| and the accumulated phase).  The whole matrix is
// updated, both triangles, as the reference does.  A is n x n ComplexF64
// (interleaved re, im; column-major).  Outputs: logpf, ph = cis(phase) (2 doubles),
// pf (2 doubles).  Odd n: (-Inf, 0, 0); a zero pivot column: the same.
// ---------------------------------------------------------------------------
template <typename T> static void pfaffian_z(const double* Ain, int64_t n, double* logpf, double* ph, double* pf) {
  typedef cx<T> C;
  const double ninf = -std::numeric_limits<double>::infinity();
  if (n % 2 == 1) {  // :97, :195
    *logpf = ninf;
    ph[0] = ph[1] = pf[0] = pf[1] = 0;
    return;
  }
  std::vector<C> A((size_t)n * n);
  for (int64_t i = 0; i < n * n; i++) A[i] = C(T(Ain[2 * i]), T(Ain[2 * i + 1]));
  auto at = [&](int64_t i, int64_t j) -> C& { return A[i + j * n]; };
  std::vector<C> tau(std::max<int64_t>(n, 1));
  T lp = 0, phase = 0;
  C prod(T(1), T(0));
  for (int64_t k = 0; k + 1 < n; k += 2) {
    // :102 / :201  kp = k + argmaxabs(A[k+1:end, k]) (first maximum)
    int64_t kp = k + 1;
    T best = cabs(at(k + 1, k));
    for (int64_t i = k + 2; i < n; i++) {
      const T v = cabs(at(i, k));
      if (v > best) {
        best = v;
        kp = i;
      }
    }
    if (kp != k + 1) {  // :103-111 / :202-210
      for (int64_t l = k; l < n; l++) std::swap(at(k + 1, l), at(kp, l));
      for (int64_t l = k; l < n; l++) std::swap(at(l, k + 1), at(l, kp));
      prod = -prod;
      phase += M<T>::pi();
    }
    if (is_zero(at(k + 1, k))) {  // :127-129 / :226-228
      *logpf = ninf;
      ph[0] = ph[1] = pf[0] = pf[1] = 0;
      return;
    }
    const C piv = at(k, k + 1);  // :115-117 / :214-216
    for (int64_t j = k + 2; j < n; j++) tau[j] = at(k, j) / piv;
    prod = prod * piv;
    lp += M<T>::log(cabs(piv));
    phase += M<T>::atan2(piv.im, piv.re);
    for (int64_t c = k + 2; c < n; c++)  // :118-125 / :217-224
      for (int64_t r = k + 2; r < n; r++) at(r, c) = at(r, c) + (tau[r] * at(c, k + 1) - tau[c] * at(r, k + 1));
  }
  *logpf = (double)lp;
  ph[0] = (double)M<T>::cos(phase);
  ph[1] = (double)M<T>::sin(phase);
  pf[0] = (double)prod.re;
  pf[1] = (double)prod.im;
}

// ---------------------------------------------------------------------------
// Skew tridiagonal implicit QR.  skeweigen.jl
// ---------------------------------------------------------------------------
template <typename T> static void getgivens(T a, T b, T* c, T* s) {  // :3-7
  T nm = M<T>::hypot(a, b);
  if (nm == 0) {
    *c = 1;
    *s = 0;
    return;
  }
  *c = a / nm;
  *s = b / nm;
}

// reducetozero :11-47 ; ev is 0-based, n is the reference's n (= N-1).
template <typename T> static void reducetozero(T* ev, T* G, int64_t n) {
  if (n == 0) return;
  T bulge = 0;
  if (n > 2) {
    T a = ev[n - 3], b = ev[n - 2], g = ev[n - 1], c, s;
    getgivens(-b, g, &c, &s);
    G[n - 2] = c;
    G[n - 1] = -s;
    ev[n - 3] *= c;
    ev[n - 2] = c * b - s * g;
    ev[n - 1] = 0;
    bulge = -s * a;
    for (int64_t i = n - 2; i >= 4; i -= 2) {  // 1-based i
      a = ev[i - 3];
      b = ev[i - 2];
      getgivens(-b, bulge, &c, &s);
      G[i - 2] = c;
      G[i - 1] = -s;
      ev[i - 3] *= c;
      ev[i - 2] = c * b - s * bulge;
      bulge = -s * a;
    }
  }
  T b = (n == 2 ? ev[1] : bulge);
  T a = ev[0], c, s;
  getgivens(-a, b, &c, &s);
  G[0] = c;
  G[1] = -s;
  ev[0] = c * a - s * b;
  if (n == 2) ev[1] = s * a + b * c;
}

// getoddvectors :49-62.  Qodd is nn x nn column-major (nn = n/2 + 1), n = N-1.
template <typename T> static void getoddvectors(T* Qodd, const T* G, int64_t n) {
  int64_t nn = n / 2 + 1;
  for (int64_t i = 1; i <= n - 1; i += 2) {
    T c = G[i - 1], s = G[i];
    int64_t ii = (i + 1) / 2;
    for (int64_t j = 1; j <= nn; j++) {
      T sig = Qodd[(ii - 1) + (j - 1) * nn];
      T om = Qodd[(nn - 1) + (j - 1) * nn];
      Qodd[(ii - 1) + (j - 1) * nn] = c * sig + s * om;
      Qodd[(nn - 1) + (j - 1) * nn] = -s * sig + c * om;
    }
  }
}

// implicitstep_novec :73-103 (n = active size; ev 0-based; start 1-based)
template <typename T> static int64_t implicitstep_novec(T* ev, int64_t n, int64_t start) {
  T bulge = 0;
  T shift = ev[n - 1] * ev[n - 1];  // getshift(ev[n-1:n]) = ev[n]^2
  T tol = M<T>::eps();
  for (int64_t i = start; i <= n - 1; i++) {
    T a = (i > start ? ev[i - 2] : T(0));
    T b = ev[i - 1];
    T g = ev[i];
    T x1 = -a * a - b * b + shift;
    T x2 = -a * bulge + b * g;
    T c, s;
    if (i > start)
      getgivens(a, bulge, &c, &s);
    else
      getgivens(x1, x2, &c, &s);
    if (i > 1) ev[i - 2] = c * a + s * bulge;
    ev[i - 1] = c * b - s * g;
    ev[i] = s * b + c * g;
    if (i < n - 1) {
      T z = ev[i + 1];
      ev[i + 1] *= c;
      bulge = s * z;
      if (M<T>::abs(bulge) < tol && M<T>::abs(ev[i - 1]) < tol) return i + 1;
    }
  }
  return start;
}

// Symmetric tridiagonal eigenproblem (zero diagonal or given diagonal) by
// cyclic Jacobi on the dense matrix; eigenvalues ascending, vectors in Z.
// Stands in for LAPACK's SymTridiagonal solvers used by the reference's
// fallback (skeweigen.jl:463-489) and complex path (tridiag.jl:506-515).
template <typename T>
static void symtri_eigen(const T* d, const T* e, int64_t n, T* w, T* Z /* n x n or null */) {
  std::vector<T> A((size_t)n * n, T(0)), V((size_t)n * n, T(0));
  for (int64_t i = 0; i < n; i++) {
    A[i + i * n] = d ? d[i] : T(0);
    V[i + i * n] = 1;
  }
  for (int64_t i = 0; i + 1 < n; i++) A[(i + 1) + i * n] = A[i + (i + 1) * n] = e[i];
  for (int sweep = 0; sweep < 100; sweep++) {
    T off = 0, tot = 0;
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) {
        T a = A[i + j * n] * A[i + j * n];
        tot += a;
        if (i != j) off += a;
      }
    if (off <= tot * M<T>::eps() * M<T>::eps() || off == 0) break;
    for (int64_t p = 0; p < n - 1; p++)
      for (int64_t q = p + 1; q < n; q++) {
        T apq = A[p + q * n];
        if (apq == 0) continue;
        T app = A[p + p * n], aqq = A[q + q * n];
        T theta = (aqq - app) / (2 * apq);
        T t = sgn(theta) / (M<T>::abs(theta) + M<T>::sqrt(theta * theta + 1));
        if (theta == 0) t = 1;
        T c = 1 / M<T>::sqrt(t * t + 1), s = t * c;
        for (int64_t k = 0; k < n; k++) {  // columns p,q
          T akp = A[k + p * n], akq = A[k + q * n];
          A[k + p * n] = c * akp - s * akq;
          A[k + q * n] = s * akp + c * akq;
        }
        for (int64_t k = 0; k < n; k++) {  // rows p,q
          T apk = A[p + k * n], aqk = A[q + k * n];
          A[p + k * n] = c * apk - s * aqk;
          A[q + k * n] = s * apk + c * aqk;
        }
        for (int64_t k = 0; k < n; k++) {
          T vkp = V[k + p * n], vkq = V[k + q * n];
          V[k + p * n] = c * vkp - s * vkq;
          V[k + q * n] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int64_t> idx(n);
  for (int64_t i = 0; i < n; i++) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return A[a + a * n] < A[b + b * n]; });
  for (int64_t i = 0; i < n; i++) {
    w[i] = A[idx[i] + idx[i] * n];
    if (Z)
      for (int64_t k = 0; k < n; k++) Z[k + i * n] = V[k + idx[i] * n];
  }
}

// skewtrieigvals! :105-156.  ev (N-1) is destroyed; vals_im[N] receives the
// imaginary parts of the eigenvalues in the reference's order.  Returns 0 on
// success, 1 if the fallback was used, -1 on non-convergence (:154).
template <typename T> static int skewtrieigvals(T* ev, int64_t N, T* vals) {
  int64_t n = N;
  for (int64_t i = 0; i < N; i++) vals[i] = 0;
  std::vector<T> G(std::max<int64_t>(N, 1));
  if (n % 2 == 1) {
    n -= 1;
    reducetozero(ev, G.data(), n);
  }
  T tol = M<T>::eps() * T(10);
  int64_t max_iter = 30 * n, iter = 0;
  T mem = 1;
  int count_static = 0;
  int64_t start = 1;
  while (n > 2 && iter < max_iter) {
    start = implicitstep_novec(ev, n - 1, start);
    while (n > 2 && M<T>::abs(ev[n - 2]) <= tol) {
      vals[n - 1] = 0;
      n -= 1;
    }
    while (n > 2 && M<T>::abs(ev[n - 3]) <= tol * M<T>::abs(ev[n - 2])) {
      vals[n - 2] = ev[n - 2];
      vals[n - 1] = -ev[n - 2];
      n -= 2;
    }
    if (start > n - 2) start = 1;
    if (n > 1 && M<T>::abs(mem - ev[n - 2]) < T(0.0001) * M<T>::abs(ev[n - 2])) {
      count_static += 1;
      if (count_static > 4) {  // :134-137 fallback
        std::vector<T> w(n);
        symtri_eigen<T>(nullptr, ev, n, w.data(), nullptr);
        for (int64_t i = 0; i < n; i++) vals[i] = -w[i];
        return 1;
      }
    } else {
      count_static = 0;
    }
    mem = (n > 1 ? ev[n - 2] : T(0));
    iter += 1;
  }
  if (n == 2) {
    vals[0] = ev[0];
    vals[1] = -ev[0];
    return 0;
  } else if (n == 1) {
    vals[0] = 0;
    return 0;
  } else if (n == 0) {
    return 0;
  }
  return -1;
}

// implicitstep_vec! :158-193.  Qodd (ho x ho), Qeven (he x he), column-major;
// rotations act on columns k, k+1 of rows 1..Nrows.
template <typename T>
static int64_t implicitstep_vec(T* ev, T* Qeven, int64_t lde, T* Qodd, int64_t ldo, int64_t n, int64_t Nrows,
                                int64_t start) {
  T bulge = 0;
  T shift = ev[n - 1] * ev[n - 1];
  T tol = 10 * M<T>::eps();
  for (int64_t i = start; i <= n - 1; i++) {
    T a = (i > start ? ev[i - 2] : T(0));
    T b = ev[i - 1];
    T g = ev[i];
    T x1 = -a * a - b * b + shift;
    T x2 = -a * bulge + b * g;
    T c, s;
    if (i > start)
      getgivens(a, bulge, &c, &s);
    else
      getgivens(x1, x2, &c, &s);
    if (i > 1) ev[i - 2] = c * a + s * bulge;
    ev[i - 1] = c * b - s * g;
    ev[i] = s * b + c * g;
    if (i < n - 1) {
      T z = ev[i + 1];
      ev[i + 1] *= c;
      bulge = s * z;
      if (M<T>::abs(bulge) < tol && M<T>::abs(ev[i - 1]) < tol) start = i + 1;
    }
    T* Q = (i % 2 == 1) ? Qodd : Qeven;
    int64_t ld = (i % 2 == 1) ? ldo : lde;
    int64_t k = (i + 1) / 2;
    for (int64_t j = 1; j <= Nrows; j++) {
      T sig = Q[(j - 1) + (k - 1) * ld];
      T om = Q[(j - 1) + k * ld];
      Q[(j - 1) + (k - 1) * ld] = c * sig + s * om;
      Q[(j - 1) + k * ld] = -s * sig + c * om;
    }
  }
  return start;
}

// skewtrieigen_backup! :470-489 -> vals_im, Qr, Qim (N x N)
template <typename T> static void skewtrieigen_backup(const T* ev, int64_t N, T* vals, T* Qr, T* Qim) {
  std::vector<T> w(N), Z((size_t)N * N);
  symtri_eigen<T>(nullptr, ev, N, w.data(), Z.data());
  for (int64_t j = 0; j < N; j++) {
    vals[j] = -w[j];
    T c = 1;
    for (int64_t i = 0; i + 1 < N; i += 2) {
      Qr[i + j * N] = Z[i + j * N] * c;
      Qim[i + j * N] = 0;
      Qr[(i + 1) + j * N] = 0;
      Qim[(i + 1) + j * N] = Z[(i + 1) + j * N] * c;
      c = -c;
    }
    if (N % 2 == 1) {
      Qr[(N - 1) + j * N] = Z[(N - 1) + j * N] * c;
      Qim[(N - 1) + j * N] = 0;
    }
  }
}

// skewtrieigen_divided! :322-457.  ev (N-1) destroyed; outputs vals_im (N),
// Qr, Qim (N x N column-major).  Returns 0 / 1 (fallback) / -1 (no convergence).
template <typename T> static int skewtrieigen_divided(T* ev, int64_t N, T* vals, T* Qr, T* Qim) {
  std::vector<T> backup(ev, ev + std::max<int64_t>(N - 1, 0));
  int64_t n = N;
  for (int64_t i = 0; i < N; i++) vals[i] = 0;
  for (int64_t i = 0; i < N * N; i++) Qr[i] = Qim[i] = 0;
  int64_t ho = (N + 1) / 2, he = N / 2;
  std::vector<T> Qodd((size_t)ho * ho, T(0)), Qeven((size_t)std::max<int64_t>(he * he, 1), T(0));
  for (int64_t i = 0; i < ho; i++) Qodd[i + i * ho] = 1;
  for (int64_t i = 0; i < he; i++) Qeven[i + i * he] = 1;
  std::vector<T> G(std::max<int64_t>(N, 1));
  if (n % 2 == 1) {
    n -= 1;
    reducetozero(ev, G.data(), n);
  }
  T tol = M<T>::eps() * T(10);
  int64_t max_iter = 30 * n, iter = 0;
  int64_t halfN = n / 2;
  T mem = 1;
  int count_static = 0;
  int64_t start = 1;
  while (n > 2 && iter < max_iter) {
    start = implicitstep_vec(ev, Qeven.data(), std::max<int64_t>(he, 1), Qodd.data(), ho, n - 1, halfN, start);
    while (n > 2 && M<T>::abs(ev[n - 2]) <= tol) {
      vals[n - 1] = 0;
      n -= 1;
    }
    while (n > 2 && M<T>::abs(ev[n - 3]) <= tol * M<T>::abs(ev[n - 2])) {
      vals[n - 2] = ev[n - 2];
      vals[n - 1] = -ev[n - 2];
      n -= 2;
    }
    if (n > 2 && M<T>::abs(ev[n - 2] - mem) < tol) {  // :355-358
      vals[n - 2] = ev[n - 2];
      vals[n - 1] = -ev[n - 2];
      n -= 2;
    }
    if (start > n - 2) start = 1;
    if (n > 1 && M<T>::abs(mem - ev[n - 2]) < T(0.0001) * M<T>::abs(ev[n - 2])) {
      count_static += 1;
      if (count_static > 4) {  // :364-371
        skewtrieigen_backup<T>(backup.data(), N, vals, Qr, Qim);
        return 1;
      }
    } else {
      count_static = 0;
    }
    mem = (n > 1 ? ev[n - 2] : T(0));
    iter += 1;
  }
  if (n > 0) {
    if (n == 2) {
      vals[0] = ev[0];
      vals[1] = -ev[0];
    } else {
      vals[0] = 0;
    }
    if (N % 2 == 1) getoddvectors(Qodd.data(), G.data(), N - 1);
    T s2 = T(1) / M<T>::sqrt(T(2));
    auto QO = [&](int64_t r, int64_t c) -> T { return Qodd[(r - 1) + (c - 1) * ho]; };
    auto QE = [&](int64_t r, int64_t c) -> T { return Qeven[(r - 1) + (c - 1) * std::max<int64_t>(he, 1)]; };
    auto VR = [&](int64_t r, int64_t c) -> T& { return Qr[(r - 1) + (c - 1) * N]; };
    auto VI = [&](int64_t r, int64_t c) -> T& { return Qim[(r - 1) + (c - 1) * N]; };
    int64_t i = 1, countzeros = 0;
    while (i <= N) {
      int64_t ii = (i + 1) / 2;
      if (vals[i - 1] == 0) {
        if (countzeros % 2 == 0) {
          for (int64_t j = 1; j <= N - 1; j += 2) VR(j, i) = QO((j + 1) / 2, ii);
          if (N % 2 == 1) VR(N, i) = QO(halfN + 1, ii);
        } else {
          for (int64_t j = 1; j <= N - 1; j += 2) VR(j + 1, i) = QE((j + 1) / 2, ii);
        }
        countzeros += 1;
        i += 1;
      } else {
        if (countzeros % 2 == 1) {
          for (int64_t j = 1; j <= N - 1; j += 2) {
            int64_t jj = (j + 1) / 2;
            VI(j, i) = -s2 * QO(jj, ii + 1);
            VR(j + 1, i) = s2 * QE(jj, ii);
            VR(j, i + 1) = -s2 * QO(jj, ii + 1);
            VI(j + 1, i + 1) = s2 * QE(jj, ii);
          }
          if (N % 2 == 1) {
            VR(N, i) = -s2 * QO(halfN + 1, ii + 1);
            VI(N, i + 1) = -s2 * QO(halfN + 1, ii + 1);
          }
        } else {
          for (int64_t j = 1; j <= N - 1; j += 2) {
            int64_t jj = (j + 1) / 2;
            VR(j, i) = s2 * QO(jj, ii);
            VI(j + 1, i) = -s2 * QE(jj, ii);
            VI(j, i + 1) = s2 * QO(jj, ii);
            VR(j + 1, i + 1) = -s2 * QE(jj, ii);
          }
          if (N % 2 == 1) {
            VR(N, i) = s2 * QO(halfN + 1, ii);
            VI(N, i + 1) = s2 * QO(halfN + 1, ii);
          }
        }
        i += 2;
      }
    }
    if (N % 2 == 1)
      for (int64_t j = 1; j <= N; j += 2) VR(j, N) = QO((j + 1) / 2, halfN + 1);
    return 0;
  } else if (n == 0) {
    return 0;
  }
  return -1;
}

// skeweigen!  eigen.jl:75-91 (real).  A (n x n) is consumed.
template <typename T>
static int skeweigen(const double* Ain, int64_t n, T* vals, T* Vr, T* Vi, T* ev_out = nullptr) {
  if (n == 1) {  // :340-342
    vals[0] = T(Ain[0]);
    Vr[0] = 1;
    Vi[0] = 0;
    return 0;
  }
  std::vector<T> A((size_t)n * n), tau(n), eta(n), Q((size_t)n * n), Qr((size_t)n * n), Qi((size_t)n * n);
  for (int64_t i = 0; i < n * n; i++) A[i] = T(Ain[i]);
  skewblockedhess<T>(A.data(), n, n, tau.data(), eta.data(), false);
  if (ev_out)
    for (int64_t i = 0; i < n - 1; i++) ev_out[i] = eta[i];
  formq<T>(A.data(), n, n, tau.data(), Q.data());
  int st = skewtrieigen_divided<T>(eta.data(), n, vals, Qr.data(), Qi.data());
  if (st < 0) return st;
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) {
      T ar = 0, ai = 0;
      for (int64_t k = 0; k < n; k++) {
        ar += Q[i + k * n] * Qr[k + j * n];
        ai += Q[i + k * n] * Qi[k + j * n];
      }
      Vr[i + j * n] = ar;
      Vi[i + j * n] = ai;
    }
  return st;
}

// skewexp!  exp.jl:3-35 (real):  (Qr C - Qi S) Qr^T + (Qr S + Qi C) Qi^T
template <typename T> static int skewexp(const double* Ain, int64_t n, T* out) {
  std::vector<T> vals(n), Qr((size_t)n * n), Qi((size_t)n * n);
  int st = skeweigen<T>(Ain, n, vals.data(), Qr.data(), Qi.data());
  if (st < 0) return st;
  std::vector<T> C(n), S(n);
  for (int64_t i = 0; i < n; i++) {
    S[i] = M<T>::sin(vals[i]);
    C[i] = M<T>::cos(vals[i]);
  }
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) {
      T acc = 0;
      for (int64_t k = 0; k < n; k++) {
        T q1 = Qr[i + k * n] * C[k] - Qi[i + k * n] * S[k];
        T q2 = Qr[i + k * n] * S[k] + Qi[i + k * n] * C[k];
        acc += q1 * Qr[j + k * n] + q2 * Qi[j + k * n];
      }
      out[i + j * n] = acc;
    }
  return st;
}

// skewcis!  exp.jl:99-110 (real): V diag(exp(-Im lambda)) V^H, V = Qr + i Qi.
template <typename T> static int skewcis(const double* Ain, int64_t n, T* ore, T* oim) {
  std::vector<T> vals(n), Qr((size_t)n * n), Qi((size_t)n * n);
  int st = skeweigen<T>(Ain, n, vals.data(), Qr.data(), Qi.data());
  if (st < 0) return st;
  std::vector<T> e(n);
  for (int64_t i = 0; i < n; i++) e[i] = M<T>::exp(-vals[i]);
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) {
      T re = 0, im = 0;
      for (int64_t k = 0; k < n; k++) {
        // (a + ib) e (c - id) = e[(ac + bd) + i(bc - ad)]
        T a = Qr[i + k * n], b = Qi[i + k * n], c = Qr[j + k * n], d = Qi[j + k * n];
        re += e[k] * (a * c + b * d);
        im += e[k] * (b * c - a * d);
      }
      ore[i + j * n] = re;
      oim[i + j * n] = im;
    }
  return st;
}

// Independent checks (not reference algorithms) --------------------------------

// Gauss-Jordan inverse with partial pivoting; returns 0 on success.
template <typename T> static int gj_inverse(std::vector<T>& A, int64_t n, std::vector<T>& X) {
  X.assign((size_t)n * n, T(0));
  for (int64_t i = 0; i < n; i++) X[i + i * n] = 1;
  for (int64_t c = 0; c < n; c++) {
    int64_t p = c;
    for (int64_t r = c + 1; r < n; r++)
      if (M<T>::abs(A[r + c * n]) > M<T>::abs(A[p + c * n])) p = r;
    if (A[p + c * n] == 0) return -1;
    if (p != c)
      for (int64_t k = 0; k < n; k++) {
        std::swap(A[c + k * n], A[p + k * n]);
        std::swap(X[c + k * n], X[p + k * n]);
      }
    T d = A[c + c * n];
    for (int64_t k = 0; k < n; k++) {
      A[c + k * n] /= d;
      X[c + k * n] /= d;
    }
    for (int64_t r = 0; r < n; r++) {
      if (r == c) continue;
      T f = A[r + c * n];
      if (f == 0) continue;
      for (int64_t k = 0; k < n; k++) {
        A[r + k * n] -= f * A[c + k * n];
        X[r + k * n] -= f * X[c + k * n];
      }
    }
  }
  return 0;
}

// exp of a dense real matrix by scaling and squaring with a long Taylor series.
template <typename T> static void dense_expm(const std::vector<T>& A, int64_t n, std::vector<T>& E) {
  T nrm = 0;
  for (int64_t j = 0; j < n; j++) {
    T s = 0;
    for (int64_t i = 0; i < n; i++) s += M<T>::abs(A[i + j * n]);
    nrm = std::max(nrm, s);
  }
  int sq = 0;
  T scale = 1;
  while (nrm * scale > T(0.25)) {
    scale /= 2;
    sq++;
  }
  std::vector<T> B(A.size()), term((size_t)n * n), nt((size_t)n * n);
  for (size_t i = 0; i < A.size(); i++) B[i] = A[i] * scale;
  E.assign((size_t)n * n, T(0));
  for (int64_t i = 0; i < n; i++) E[i + i * n] = 1;
  term = E;
  for (int k = 1; k <= 40; k++) {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) {
        T acc = 0;
        for (int64_t l = 0; l < n; l++) acc += term[i + l * n] * B[l + j * n];
        nt[i + j * n] = acc / T(k);
      }
    term.swap(nt);
    for (size_t i = 0; i < E.size(); i++) E[i] += term[i];
  }
  for (int s = 0; s < sq; s++) {
    for (int64_t j = 0; j < n; j++)
      for (int64_t i = 0; i < n; i++) {
        T acc = 0;
        for (int64_t l = 0; l < n; l++) acc += E[i + l * n] * E[l + j * n];
        nt[i + j * n] = acc;
      }
    E.swap(nt);
  }
}

// ---------------------------------------------------------------------------
// C entry points for ctypes.  Suffix _d: FP64 restatement; _q: binary128.
// All matrices column-major with leading dimension n.
// ---------------------------------------------------------------------------
extern "C" {

int orc_quad_digits() { return std::numeric_limits<double>::digits10 + (sizeof(quad) > 8 ? 18 : 0); }

void orc_hessenberg_d(double* A, int64_t n, double* tau, double* ev) {
  std::vector<double> t(std::max<int64_t>(n, 1)), e(std::max<int64_t>(n, 1));
  skewblockedhess<double>(A, n, n, t.data(), e.data(), false);
  for (int64_t i = 0; i + 1 < n; i++) {
    tau[i] = t[i];
    ev[i] = e[i];
  }
}

void orc_hessenberg_q(double* A, int64_t n, double* tau, double* ev) {
  std::vector<quad> Aq((size_t)n * n), t(std::max<int64_t>(n, 1)), e(std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n * n; i++) Aq[i] = A[i];
  skewblockedhess<quad>(Aq.data(), n, n, t.data(), e.data(), false);
  for (int64_t i = 0; i < n * n; i++) A[i] = (double)Aq[i];
  for (int64_t i = 0; i + 1 < n; i++) {
    tau[i] = (double)t[i];
    ev[i] = (double)e[i];
  }
}

// Complex (interleaved re,im) hessenberg: A n x n complex; tau complex (n-1);
// ev real (n-1); dvim = imag(diag(A)) after the reduction (hessenberg.jl:7-9).
void orc_hessenberg_z(double* A, int64_t n, double* tau, double* ev, double* dvim) {
  std::vector<cx<double>> t(std::max<int64_t>(n, 1));
  std::vector<double> e(std::max<int64_t>(n, 1));
  skewblockedhess<cx<double>>(reinterpret_cast<cx<double>*>(A), n, n, t.data(), e.data(), true);
  for (int64_t i = 0; i + 1 < n; i++) {
    tau[2 * i] = t[i].re;
    tau[2 * i + 1] = t[i].im;
    ev[i] = e[i];
  }
  for (int64_t i = 0; i < n; i++) dvim[i] = A[2 * (i + i * n) + 1];
}

void orc_hessenberg_zq(double* A, int64_t n, double* tau, double* ev, double* dvim) {
  std::vector<cx<quad>> Aq((size_t)n * n), t(std::max<int64_t>(n, 1));
  std::vector<quad> e(std::max<int64_t>(n, 1));
  for (int64_t i = 0; i < n * n; i++) Aq[i] = cx<quad>(A[2 * i], A[2 * i + 1]);
  skewblockedhess<cx<quad>>(Aq.data(), n, n, t.data(), e.data(), true);
  for (int64_t i = 0; i < n * n; i++) {
    A[2 * i] = (double)Aq[i].re;
    A[2 * i + 1] = (double)Aq[i].im;
  }
  for (int64_t i = 0; i + 1 < n; i++) {
    tau[2 * i] = (double)t[i].re;
    tau[2 * i + 1] = (double)t[i].im;
    ev[i] = (double)e[i];
  }
  for (int64_t i = 0; i < n; i++) dvim[i] = (double)Aq[i + i * n].im;
}

void orc_formq_d(const double* A, int64_t n, const double* tau, double* Q) { formq<double>(A, n, n, tau, Q); }

void orc_logabspf_d(const double* A, int64_t n, double* logpf, double* sign) { logabspf<double>(A, n, logpf, sign); }
void orc_logabspf_q(const double* A, int64_t n, double* logpf, double* sign) { logabspf<quad>(A, n, logpf, sign); }

void orc_pfaffian_z(const double* A, int64_t n, double* logpf, double* ph, double* pf) {
  pfaffian_z<double>(A, n, logpf, ph, pf);
}
void orc_pfaffian_zq(const double* A, int64_t n, double* logpf, double* ph, double* pf) {
  pfaffian_z<quad>(A, n, logpf, ph, pf);
}

int orc_skewtrieigvals_d(double* ev, int64_t N, double* vals) { return skewtrieigvals<double>(ev, N, vals); }
int orc_skewtrieigvals_q(double* ev, int64_t N, double* vals) {
  std::vector<quad> e(std::max<int64_t>(N, 1)), v(std::max<int64_t>(N, 1));
  for (int64_t i = 0; i + 1 < N; i++) e[i] = ev[i];
  int st = skewtrieigvals<quad>(e.data(), N, v.data());
  for (int64_t i = 0; i < N; i++) vals[i] = (double)v[i];
  return st;
}

int orc_eigvals_d(const double* A, int64_t n, double* vals) {
  // skeweigvals!  eigen.jl:49-55
  if (n == 1) {
    vals[0] = A[0];
    return 0;
  }
  std::vector<double> B(A, A + n * n), t(n), e(n);
  skewblockedhess<double>(B.data(), n, n, t.data(), e.data(), false);
  return skewtrieigvals<double>(e.data(), n, vals);
}
int orc_eigvals_q(const double* A, int64_t n, double* vals) {
  if (n == 1) {
    vals[0] = A[0];
    return 0;
  }
  std::vector<quad> B((size_t)n * n), t(n), e(n), v(n);
  for (int64_t i = 0; i < n * n; i++) B[i] = A[i];
  skewblockedhess<quad>(B.data(), n, n, t.data(), e.data(), false);
  int st = skewtrieigvals<quad>(e.data(), n, v.data());
  for (int64_t i = 0; i < n; i++) vals[i] = (double)v[i];
  return st;
}

int orc_skewtrieigen_d(double* ev, int64_t N, double* vals, double* Qr, double* Qi) {
  return skewtrieigen_divided<double>(ev, N, vals, Qr, Qi);
}

int orc_eigen_d(const double* A, int64_t n, double* vals, double* Vr, double* Vi) {
  return skeweigen<double>(A, n, vals, Vr, Vi);
}
int orc_eigen_q(const double* A, int64_t n, double* vals, double* Vr, double* Vi) {
  std::vector<quad> v(n), r((size_t)n * n), i((size_t)n * n);
  int st = skeweigen<quad>(A, n, v.data(), r.data(), i.data());
  for (int64_t k = 0; k < n; k++) vals[k] = (double)v[k];
  for (int64_t k = 0; k < n * n; k++) {
    Vr[k] = (double)r[k];
    Vi[k] = (double)i[k];
  }
  return st;
}

int orc_exp_d(const double* A, int64_t n, double* out) { return skewexp<double>(A, n, out); }
int orc_exp_q(const double* A, int64_t n, double* out) {
  std::vector<quad> o((size_t)n * n);
  int st = skewexp<quad>(A, n, o.data());
  for (int64_t k = 0; k < n * n; k++) out[k] = (double)o[k];
  return st;
}
int orc_cis_d(const double* A, int64_t n, double* re, double* im) { return skewcis<double>(A, n, re, im); }
int orc_cis_q(const double* A, int64_t n, double* re, double* im) {
  std::vector<quad> r((size_t)n * n), i((size_t)n * n);
  int st = skewcis<quad>(A, n, r.data(), i.data());
  for (int64_t k = 0; k < n * n; k++) {
    re[k] = (double)r[k];
    im[k] = (double)i[k];
  }
  return st;
}

// d log|Pf(A)| / dA = 1/2 A^{-T}, by a quad Gauss-Jordan inverse (independent of
// the Householder path).  Returns -1 if A is singular.
int orc_logabspf_grad_q(const double* A, int64_t n, double* grad) {
  std::vector<quad> B((size_t)n * n), X;
  for (int64_t i = 0; i < n * n; i++) B[i] = A[i];
  if (gj_inverse<quad>(B, n, X) != 0) return -1;
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) grad[i + j * n] = (double)(X[j + i * n] / 2);
  return 0;
}

// Adjoint of exp for the real loss <C, exp(A)>: the gradient is L(A^T, C), the
// Frechet derivative of exp at A^T in direction C, read off the top-right block
// of exp([[A^T, C], [0, A^T]]) in quad precision.
void orc_exp_vjp_q(const double* A, const double* C, int64_t n, double* grad) {
  int64_t m = 2 * n;
  std::vector<quad> B((size_t)m * m, quad(0)), E;
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) {
      B[i + j * m] = A[j + i * n];
      B[(n + i) + (n + j) * m] = A[j + i * n];
      B[i + (n + j) * m] = C[i + j * n];
    }
  dense_expm<quad>(B, m, E);
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) grad[i + j * n] = (double)E[i + (n + j) * m];
}

// Dense exp in quad (independent check of the eigen-based exp).
void orc_expm_dense_q(const double* A, int64_t n, double* out) {
  std::vector<quad> B((size_t)n * n), E;
  for (int64_t i = 0; i < n * n; i++) B[i] = A[i];
  dense_expm<quad>(B, n, E);
  for (int64_t i = 0; i < n * n; i++) out[i] = (double)E[i];
}

// Symmetric tridiagonal eigenvalues (ascending), quad Jacobi.
void orc_symtri_eigvals_q(const double* d, const double* e, int64_t n, double* w) {
  std::vector<quad> dq(n), eq(std::max<int64_t>(n, 1)), wq(n);
  for (int64_t i = 0; i < n; i++) dq[i] = d ? d[i] : 0.0;
  for (int64_t i = 0; i + 1 < n; i++) eq[i] = e[i];
  symtri_eigen<quad>(dq.data(), eq.data(), n, wq.data(), nullptr);
  for (int64_t i = 0; i < n; i++) w[i] = (double)wq[i];
}

// Batched FP64 logabspfaffian over a packed batch (the CPU baseline for the
// batched workload).  Matrices are stored back to back, matrix b at offset
// off[b] (in doubles) with size n[b].  Parallel over matrices with OpenMP when
// the library is built with it.
void orc_batch_logabspf_d(const double* A, const int64_t* off, const int64_t* n, int64_t count, double* logpf,
                          double* sign, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int64_t b = 0; b < count; b++) logabspf<double>(A + off[b], n[b], logpf + b, sign + b);
  (void)nthreads;
}

// Batched FP64 log|Pf| + gradient (the CPU baseline for the batched adjoint
// workload): the restated logabspfaffian plus 1/2 A^{-T} from an FP64
// Gauss-Jordan inverse, OpenMP across matrices.  grad has the same packing as A.
void orc_batch_logabspf_grad_d(const double* A, const int64_t* off, const int64_t* n, int64_t count, double* logpf,
                               double* sign, double* grad, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int64_t b = 0; b < count; b++) {
    const int64_t m = n[b];
    logabspf<double>(A + off[b], m, logpf + b, sign + b);
    std::vector<double> B(A + off[b], A + off[b] + m * m), X;
    if (gj_inverse<double>(B, m, X) == 0) {
      for (int64_t j = 0; j < m; j++)
        for (int64_t i = 0; i < m; i++) grad[off[b] + i + j * m] = 0.5 * X[j + i * m];
    } else {
      for (int64_t k = 0; k < m * m; k++) grad[off[b] + k] = std::numeric_limits<double>::quiet_NaN();
    }
  }
  (void)nthreads;
}

// Central finite differences of log|Pf| along skew pairs (the check of the
// rrule gradient: d/dh log|Pf(A + h (e_i e_j^T - e_j e_i^T))| = G_ij - G_ji for
// G = 1/2 A^{-T}).  pairs holds k (i, j) index pairs per matrix (count * k * 2
// entries, 0-based); fd[b * k + p] receives the difference quotient with step h.
// quad != 0 runs the restated reduction and the difference in binary128, so
// the quotient carries only the O(h^2) truncation error.  OpenMP over pairs.
void orc_batch_logabspf_fd(const double* A, const int64_t* off, const int64_t* n, int64_t count,
                           const int64_t* pairs, int64_t k, double h, int quad_prec, double* fd, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int64_t t = 0; t < count * k; t++) {
    const int64_t b = t / k, i = pairs[2 * t], j = pairs[2 * t + 1];
    if (quad_prec) {
      const quad hq = (quad)h;
      const quad d = logabspf_pair<quad>(A + off[b], n[b], i, j, hq) - logabspf_pair<quad>(A + off[b], n[b], i, j, -hq);
      fd[t] = (double)(d / (2 * hq));
    } else {
      const double d = logabspf_pair<double>(A + off[b], n[b], i, j, h) - logabspf_pair<double>(A + off[b], n[b], i, j, -h);
      fd[t] = d / (2 * h);
    }
  }
  (void)nthreads;
}

}  // extern "C"
