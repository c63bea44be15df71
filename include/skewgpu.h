/*
 * skewgpu.h -- C ABI of libskewgpu.so, the GB300 (sm_103a) FP64 implementation of
 * SkewLinearAlgebra.jl's skew-Householder pipeline.
 *
 * Every pointer argument that refers to matrix or vector data is a DEVICE pointer
 * owned by the caller (e.g. pointer(A.data) of a CuArray).  Matrices are
 * column-major (Julia layout) with a leading dimension.  Calls are asynchronous
 * with respect to the host and ordered on the handle's stream.  Each entry point
 * returns a skew_status_t for argument/launch errors; conditions that are only
 * known on the device (non-convergence, a singular matrix, a matrix that is not
 * skew) are written to the caller's device-side `info`/`status` integers.
 *
 * Reference interfaces each entry point replaces are cited by file:line of
 * SkewLinearAlgebra.jl (v1.1.0).
 */
#ifndef SKEWGPU_H
#define SKEWGPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define SKEW_API __attribute__((visibility("default")))
#else
#define SKEW_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* skew_stream_t; /* == cudaStream_t */

typedef enum {
  SKEW_OK = 0,
  SKEW_NOT_SKEW = 1,        /* ArgumentError("Pfaffian requires a skew-Hermitian matrix"), pfaffian.jl:255 */
  SKEW_NO_CONVERGENCE = 2,  /* error("Maximum number of iterations reached"), skeweigen.jl:154 */
  SKEW_BAD_ARG = 3,
  SKEW_CUDA_ERROR = 4,
  SKEW_SINGULAR = 5,        /* Pf(A) == 0: log|Pf| = -Inf, gradient not finite (odd n, pfaffian.jl:169) */
  SKEW_UNSUPPORTED = 6,
  SKEW_NO_MEMORY = 7,
  SKEW_FALLBACK_USED = 8,   /* QR stagnated; values from the symmetric-tridiagonal fallback (skeweigen.jl:132-137) */
  SKEW_TIMEOUT = 9          /* a bounded device-side wait gave up; outputs are not valid */
} skew_status_t;

/* Matrix functions of a skew matrix from its eigendecomposition (exp.jl:3-283):
 * F = V diag(f(lambda)) V^H; cos/cosh are returned Hermitian (symmetric), sin, sinh,
 * tan, tanh, cot, coth skew(-Hermitian), as the reference's Hermitian / skewhermitian!
 * wrappers.  sincos is SKEW_FUNC_SIN and SKEW_FUNC_COS.  log, cot, coth of a matrix
 * with a zero eigenvalue (every odd n) report SKEW_SINGULAR (the reference's
 * DomainError / singular solve). */
typedef enum {
  SKEW_FUNC_EXP = 0,
  SKEW_FUNC_COS = 1,
  SKEW_FUNC_SIN = 2,
  SKEW_FUNC_COSH = 3,
  SKEW_FUNC_SINH = 4,
  SKEW_FUNC_TAN = 5,
  SKEW_FUNC_TANH = 6,
  SKEW_FUNC_COT = 7,
  SKEW_FUNC_COTH = 8,
  SKEW_FUNC_LOG = 9
} skew_func_t;

typedef struct skew_handle_st* skew_handle_t;
typedef struct skew_batch_plan_st* skew_batch_plan_t;

/* Library handle: owns the stream binding and cached workspaces (one per stream). */
SKEW_API int skew_create(skew_handle_t* handle);
SKEW_API int skew_destroy(skew_handle_t handle);
SKEW_API int skew_set_stream(skew_handle_t handle, skew_stream_t stream);
SKEW_API const char* skew_status_string(int status);
SKEW_API int skew_version(void);

/* ---------------------------------------------------------------------------
 * Single-matrix entry points (real Float64).
 * ------------------------------------------------------------------------- */

/* LA.hessenberg!(A::SkewHermitian{Float64})  hessenberg.jl:5-13 (skewblockedhess! :144-173).
 * In place: on exit A holds the reflectors below the subdiagonal (v[1] = 1 stored on
 * the subdiagonal, as the reference stores them), tau[n-1] the reflector scalars and
 * ev[n-1] the subdiagonal of H = SkewHermTridiagonal(ev). */
SKEW_API int skew_hessenberg_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* tau, double* ev, int* info);

/* logabspfaffian!(A::SkewHermitian{Float64})  pfaffian.jl:167-179, :235.
 * In place.  logpf[0] = log|Pf(A)|, sign[0] = sign of Pf(A) (odd n: -Inf, 0).
 * check != 0 verifies A == -A^T exactly first (pfaffian.jl:254-256) -> info = SKEW_NOT_SKEW. */
SKEW_API int skew_logabspf_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* sign, int check,
                    int* info);

/* rrule(logabspfaffian) forward + pullback seed 1: as skew_logabspf_d, and
 * G = d log|Pf(A)| / dA = 1/2 A^{-T}, formed as Q (1/2 T^{-T}) Q^T from the reflectors.
 * (No reference counterpart: the reference defines no rrule for logabspfaffian.) */
SKEW_API int skew_logabspf_grad_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* sign,
                         double* G, int64_t ldg, int* info);

/* LA.eigvals!(A::SkewHermitian{Float64})  eigen.jl:2-6 -> skeweigvals! :49-55.
 * vals_im[n] = imaginary parts of the eigenvalues (eigenvalue k is i*vals_im[k]).
 * n <= 1024: in the reference's order, the deflation order of skewtrieigvals!
 * (skeweigen.jl:105-156), run on one GPU thread after the reduction; info receives
 * SKEW_OK, SKEW_FALLBACK_USED (the shifts stagnated and the values come from the
 * reference's fallback, sorted descending, skeweigen.jl:132-137) or
 * SKEW_NO_CONVERGENCE (skeweigen.jl:154).  n > 1024: sorted descending by bisection
 * over the whole GPU (the fallback's order).  For the values sorted descending at any
 * n, at bisection speed, use skew_eigvals_irange_d(1, n), which is eigvals(A, 1:n).
 * A is destroyed. */
SKEW_API int skew_eigvals_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, int* info);

/* LA.eigvals!(A::SkewHermitian{Float64}, irange)  eigen.jl:8-11, :57-64: vals_im[0 .. iu-il] =
 * -lambda_{il..iu} for the ascending eigenvalues lambda of SymTridiagonal(0, ev), i.e. the
 * imaginary parts in descending order from the il-th largest; 1 <= il <= iu <= n.  A destroyed. */
SKEW_API int skew_eigvals_irange_d(skew_handle_t h, double* A, int64_t n, int64_t lda, int64_t il, int64_t iu,
                                   double* vals_im, int* info);

/* LA.eigvals!(A::SkewHermitian{Float64}, vl, vh)  eigen.jl:13-16, :66-73: the eigenvalues whose
 * imaginary part lies in [vl, vh), descending, in vals_im (room for n); *count (device int)
 * receives how many.  A destroyed. */
SKEW_API int skew_eigvals_interval_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double vl, double vh,
                                     double* vals_im, int* count, int* info);

/* eigvals without any device allocation.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc (a host that owns all device memory
 * through its own pool, or a path where an allocation's synchronisation or
 * failure is not acceptable): the eigenvalues of skew_eigvals_d, sorted
 * descending (as eigvals(A, 1:n)), equal to them to rounding; its scratch
 * (n+1 doubles) is a fixed array inside the library instead of the handle's
 * workspace, and the stream is passed directly (no handle).  n <= 1024, else
 * SKEW_UNSUPPORTED.  The first call on each device (and again after a device
 * reset) looks up the array's device address, so make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller. */
SKEW_API int skew_eigvals_noalloc_d(double* A, int64_t n, int64_t lda, double* vals_im, int* info,
                                    skew_stream_t stream);

/* LA.eigen!(A::SkewHermitian{Float64})  eigen.jl:75-97 (skeweigen! + skewtrieigen_divided!).
 * vals_im[n] in the reference's order; eigenvectors V = Vr + i*Vi (n x n each).  A is
 * destroyed.  n <= 1024: lda == ldv == n.  n > 1024 (up to 32768): blocked reduction,
 * bisection and twisted-factorisation vectors, values sorted descending (the reference's
 * own fallback formulation, skeweigen.jl:470-489); lda, ldv >= n. */
SKEW_API int skew_eigen_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* Vr, double* Vi,
                 int64_t ldv, int* info);

/* Base.exp(A::SkewHermitian{Float64})  exp.jl:3-35, :48.  E (n x n) = exp(A). A destroyed.
 * Requires lda == lde == n.  Above n = 1024 the eigenpairs come from the large-matrix path
 * of skew_eigen_d (their order does not change the function). */
SKEW_API int skew_exp_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* E, int64_t lde, int* info);

/* Base.cis(A::SkewHermitian{Float64})  exp.jl:99-110, :204.  C = cis(A) = exp(iA), Hermitian,
 * ComplexF64 interleaved (re, im).  A destroyed.  Requires lda == ldc == n (any n, as skew_exp_d). */
SKEW_API int skew_cis_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* C, int64_t ldc, int* info);

/* ---------------------------------------------------------------------------
 * Batched entry points: many independent real skew matrices of uneven size.
 * A plan fixes the sizes (host array n[count]), sorts them largest first, picks a
 * kernel configuration per size bucket and owns the device workspace.
 * ------------------------------------------------------------------------- */
SKEW_API int skew_batch_plan_create(skew_handle_t h, const int64_t* n, int64_t count, skew_batch_plan_t* plan);
SKEW_API int skew_batch_plan_destroy(skew_batch_plan_t plan);

/* logabspfaffian for every matrix; A[b] (device array of device pointers) is read only,
 * leading dimension n[b].  grad may be NULL; otherwise grad[b] receives 1/2 A_b^{-T}
 * (leading dimension n[b]).  status[b] is a skew_status_t per matrix. */
SKEW_API int skew_batch_logabspf_d(skew_batch_plan_t plan, const double* const* A, double* logpf, double* sign,
                          double* const* grad, int* status);

/* The same on host buffers (pfaffian.jl:236-246 called on host matrices, one call
 * for the batch): A holds the matrices back to back in the order of n[] given to
 * the plan, each column-major with leading dimension n[b]; grad (or NULL) receives
 * 1/2 A_b^{-T} in the same layout; logpf, sign, status are host arrays [count].
 * A and grad must be page-locked (cudaHostAlloc / cudaHostRegister), else
 * SKEW_BAD_ARG: every CTA reads its matrix from host memory and writes its
 * gradient back itself, so the transfers overlap the compute.  Returns when the
 * results are in host memory (synchronises the handle's stream). */
SKEW_API int skew_batch_logabspf_host_d(skew_batch_plan_t plan, const double* A, double* grad, double* logpf,
                               double* sign, int* status);

/* eigvals for every matrix: vals_im[b] (device pointers) receives n[b] values. */
SKEW_API int skew_batch_eigvals_d(skew_batch_plan_t plan, const double* const* A, double* const* vals_im, int* status);

/* eigen for every matrix (skeweigen! + skewtrieigen_divided!, eigen.jl:75-97): vals_im[b] (n),
 * Vr[b], Vi[b] (n x n, leading dimension n) device pointers; eigenvectors are Vr + i*Vi.
 * status[b]: SKEW_OK, SKEW_FALLBACK_USED (the reference's LAPACK fallback path,
 * skeweigen.jl:364-371, taken on the GPU) or SKEW_NO_CONVERGENCE.  n <= 1024. */
SKEW_API int skew_batch_eigen_d(skew_batch_plan_t plan, const double* const* A, double* const* vals_im,
                                double* const* Vr, double* const* Vi, int* status);

/* exp(A_b) for every matrix (skewexp!, exp.jl:3-35): E[b] n x n real, leading dimension n. */
SKEW_API int skew_batch_exp_d(skew_batch_plan_t plan, const double* const* A, double* const* E, int* status);

/* cis(A_b) = exp(i A_b) for every matrix (skewcis!, exp.jl:99-110): C[b] n x n ComplexF64
 * interleaved, leading dimension n (complex elements). */
SKEW_API int skew_batch_cis_d(skew_batch_plan_t plan, const double* const* A, double* const* C, int* status);

/* Adjoint of exp (no reference counterpart): G[b] = d<Cbar_b, exp(A_b)>/dA_b, by
 * Daleckii-Krein divided differences on the eigendecomposition.  Cbar[b], G[b] n x n real. */
SKEW_API int skew_batch_exp_vjp_d(skew_batch_plan_t plan, const double* const* A, const double* const* Cbar,
                                  double* const* G, int* status);

/* Single-matrix adjoint of exp (no reference counterpart): G = d<Cbar, exp(A)>/dA.
 * A is destroyed; lda, ldg must equal n (any n, as skew_exp_d). */
SKEW_API int skew_exp_vjp_d(skew_handle_t h, double* A, int64_t n, int64_t lda, const double* Cbar, double* G,
                            int64_t ldg, int* info);

/* ---------------------------------------------------------------------------
 * ComplexF64 skew-Hermitian matrices (A^H = -A).  Complex arrays are ComplexF64
 * interleaved (re, im), column-major, leading dimensions in complex elements.
 * ------------------------------------------------------------------------- */

/* LA.hessenberg!(A::SkewHermitian{ComplexF64})  hessenberg.jl:5-13 with the complex
 * branches of householder! :26-44, skewlatrd! :92-131 and skewblockedhess! :144-173.
 * In place: reflectors below the subdiagonal (v[1] = 1 on the subdiagonal), tau[n-1]
 * complex, ev[n-1] the real subdiagonal and dvim[n] = imag(diag) of
 * H = SkewHermTridiagonal(ev, dvim).  dvim may be NULL. */
SKEW_API int skew_hessenberg_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* tau, double* ev,
                               double* dvim, int* info);

/* LA.eigvals!(A::SkewHermitian{ComplexF64})  eigen.jl:18-27: vals_im[n] = imaginary parts,
 * descending (the reference returns -eigvals(Hermitian(i A)), eigenvalues ascending).
 * A is destroyed. */
SKEW_API int skew_eigvals_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, int* info);

/* LA.eigvals!(A::SkewHermitian{ComplexF64}, vl, vh)  eigen.jl:36-41: imaginary parts in [vl, vh),
 * descending, *count (device int) of them (vals_im room for n).  A destroyed.  (The reference's
 * complex irange method passes a negated range to LAPACK and fails; it has no counterpart.) */
SKEW_API int skew_eigvals_interval_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double vl, double vh,
                                     double* vals_im, int* count, int* info);

/* LA.eigen!(A::SkewHermitian{ComplexF64})  eigen.jl:101-106: vals_im[n] (descending) and
 * the eigenvectors V (n x n ComplexF64, ldv).  Eigenvectors are defined up to a
 * phase per column (LAPACK's choice in the reference).  A is destroyed. */
SKEW_API int skew_eigen_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* V,
                          int64_t ldv, int* info);

/* Base.exp(A::SkewHermitian{ComplexF64})  exp.jl:37-46: E = V diag(exp(lambda)) V^H
 * (ComplexF64, lde).  A is destroyed. */
SKEW_API int skew_exp_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* E, int64_t lde, int* info);

/* Adjoint of exp for ComplexF64 (no reference counterpart): G = V (conj(Phi) o (V^H Cbar V)) V^H
 * with Phi the divided differences of exp on the spectrum, i.e. dL = Re tr(G^H dA) for
 * L = Re tr(Cbar^H exp(A)).  Cbar (n x n, leading dimension n), G (ldg) ComplexF64. */
SKEW_API int skew_exp_vjp_z(skew_handle_t h, double* A, int64_t n, int64_t lda, const double* Cbar, double* G,
                            int64_t ldg, int* info);

/* Batched ComplexF64 of one size: `count` skew-Hermitian n x n matrices stored back to
 * back (matrix b at A + 2 n^2 b doubles, column-major, leading dimension n), read only;
 * outputs laid out the same way.  n <= 1024 (else SKEW_UNSUPPORTED).  status[count]
 * (may be NULL) receives SKEW_OK per matrix.
 * eigen: vals_im (count x n, descending per matrix) and V (count x n x n). */
SKEW_API int skew_batch_eigen_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* vals_im,
                                double* V, int* status);
/* exp for every matrix (exp.jl:37-46): E (count x n x n ComplexF64). */
SKEW_API int skew_batch_exp_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* E, int* status);
/* Adjoint of exp for every matrix: G_b = V_b (conj(Phi_b) o (V_b^H Cbar_b V_b)) V_b^H. */
SKEW_API int skew_batch_exp_vjp_z(skew_handle_t h, const double* A, int64_t n, int64_t count, const double* Cbar,
                                  double* G, int* status);

/* Base.cos/sin/sinh/cosh/tan/tanh/cot/coth/log(A::SkewHermitian{Float64})  exp.jl:50-283
 * (and exp): F = f(A) (real n x n, ldf).  A is destroyed; lda == ldf == n (any n, as skew_exp_d). */
SKEW_API int skew_func_d(skew_handle_t h, double* A, int64_t n, int64_t lda, int func, double* F, int64_t ldf,
                         int* info);
/* The same for every matrix of a batch plan: F[b] (n[b] x n[b], leading dimension n[b]). */
SKEW_API int skew_batch_func_d(skew_batch_plan_t plan, const double* const* A, int func, double* const* F,
                               int* status);
/* ComplexF64: F = f(A) (ComplexF64, ldf).  A is destroyed. */
SKEW_API int skew_func_z(skew_handle_t h, double* A, int64_t n, int64_t lda, int func, double* F, int64_t ldf,
                         int* info);
/* ComplexF64 batches of one size (matrices back to back, as skew_batch_exp_z). */
SKEW_API int skew_batch_func_z(skew_handle_t h, const double* A, int64_t n, int64_t count, int func, double* F,
                               int* status);

/* ---------------------------------------------------------------------------
 * Singular values and vectors from the eigenpairs (eigen.jl:110-144): the eigenvalues'
 * imaginary parts lambda stably sorted by |lambda| descending (sortperm(vals; by = abs,
 * rev = true)); S = |lambda|; U = the eigenvectors in that order; V = -i U with the
 * columns of negative lambda negated, so that A = U diag(S) V^H (the reference returns
 * SVD(U, S, adjoint(V))).  A is destroyed.
 * ------------------------------------------------------------------------- */
/* LA.svdvals!(A::SkewHermitian{Float64})  eigen.jl:110-114: S[n] descending. */
SKEW_API int skew_svdvals_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, int* info);
/* LA.svd!(A::SkewHermitian{Float64})  eigen.jl:119-136: S[n], U = Ur + i Ui, V = Vr + i Vi (n x n,
 * ldu; ldu == lda == n for n <= 1024, as skew_eigen_d). */
SKEW_API int skew_svd_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, double* Ur, double* Ui,
                        double* Vr, double* Vi, int64_t ldu, int* info);
/* LA.svdvals!(A::SkewHermitian{ComplexF64})  eigen.jl:116 (svdvals of Hermitian(i A)): S[n] descending. */
SKEW_API int skew_svdvals_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, int* info);
/* LA.svd(A::SkewHermitian{ComplexF64})  eigen.jl:138-142 (svd of Hermitian(i A), which LinearAlgebra
 * forms from its eigenpairs by the same rule): S[n], U, V ComplexF64 (n x n, ldu).  Singular
 * vectors are defined up to a phase per column (LAPACK's choice in the reference). */
SKEW_API int skew_svd_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, double* U, double* V,
                        int64_t ldu, int* info);

/* ---------------------------------------------------------------------------
 * Complex skew-symmetric matrices (A == -transpose(A), ComplexF64): the Pfaffian by
 * Parlett-Reid elimination with pivoting (pfaffian.jl:98-137 and :193-233).
 * check != 0 verifies A == -transpose(A) exactly first (pfaffian.jl:162, :261; isskewsymmetric,
 * skewhermitian.jl:101-110)
 * -> info / status = SKEW_NOT_SKEW and NaN outputs.  A zero Pfaffian (odd n, or a zero
 * pivot column) gives log|Pf| = -Inf, phase 0, Pf 0 and info = SKEW_SINGULAR.
 * ------------------------------------------------------------------------- */
/* logabspfaffian!(A::AbstractMatrix{ComplexF64})  pfaffian.jl:193-233, :259-263:
 * logpf[0] = log|Pf(A)|, phase[0..1] = cis(phase) (re, im) with Pf(A) = cis(phase) exp(logpf).
 * A (n x n, lda) is overwritten (its strictly lower triangle) for n above one CTA's size. */
SKEW_API int skew_logabspf_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* phase,
                             int check, int* info);
/* pfaffian!(A::AbstractMatrix{ComplexF64})  pfaffian.jl:98-137, :160-164: pf[0..1] = Pf(A),
 * the running product of the pivots (overflows where the reference's does). */
SKEW_API int skew_pfaffian_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* pf, int check, int* info);
/* Batches of one size (matrices back to back, leading dimension n, read only): logpf[count],
 * phase[2 count], pf[2 count] (each nullable, not all), status[count] (nullable). */
SKEW_API int skew_batch_logabspf_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* logpf,
                                   double* phase, double* pf, int check, int* status);
/* The same on host buffers: A in page-locked host memory (else SKEW_BAD_ARG), read by
 * the kernels over the host link; logpf, phase, pf, status are host arrays, filled when
 * the call returns (it synchronises the handle's stream). */
SKEW_API int skew_batch_logabspf_host_z(skew_handle_t h, const double* A, int64_t n, int64_t count,
                                        double* logpf, double* phase, double* pf, int check, int* status);

/* ---------------------------------------------------------------------------
 * SkewHermTridiagonal inputs (tridiag.jl): ev[n-1] the subdiagonal on the device, no
 * reduction (Q = I).
 * ------------------------------------------------------------------------- */
/* LA.eigvals!(::SkewHermTridiagonal{Float64})  tridiag.jl:446-450 (skewtrieigvals!): the
 * reference's QR order for n <= 1024; larger n sorted descending (bisection).  ev unchanged. */
SKEW_API int skew_tridiag_eigvals_d(skew_handle_t h, const double* ev, int64_t n, double* vals_im, int* info);
/* LA.eigen!(::SkewHermTridiagonal{Float64})  tridiag.jl:506 (skewtrieigen_merged!): vals_im, Vr + i Vi
 * (ldv == n for n <= 1024); larger n: bisection and twisted vectors, values descending. */
SKEW_API int skew_tridiag_eigen_d(skew_handle_t h, const double* ev, int64_t n, double* vals_im, double* Vr,
                                  double* Vi, int64_t ldv, int* info);
/* exp.jl functions of a SkewHermTridiagonal{Float64}: F = f(T), ldf == n (above n = 1024 the
 * eigenpairs come from bisection and twisted vectors, as skew_tridiag_eigen_d). */
SKEW_API int skew_tridiag_func_d(skew_handle_t h, const double* ev, int64_t n, int func, double* F, int64_t ldf,
                                 int* info);
/* LA.eigvals! / LA.eigen!(::SkewHermTridiagonal{ComplexF64})  tridiag.jl:462-468, :508-515: ev[n-1]
 * ComplexF64 subdiagonal, dvim[n] the imaginary diagonal (or NULL); through to_symtridiagonal
 * (:558-583): values descending, V = D Y (V may be NULL for eigvals). */
SKEW_API int skew_tridiag_eigvals_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n,
                                    double* vals_im, int* info);
SKEW_API int skew_tridiag_eigen_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n,
                                  double* vals_im, double* V, int64_t ldv, int* info);
/* LA.svdvals! / LA.svd! of a SkewHermTridiagonal  tridiag.jl:526-555: as skew_svdvals_d /
 * skew_svd_d on its eigenpairs (Float64: ev[n-1]; ComplexF64: ev[n-1] complex and dvim[n] or NULL). */
SKEW_API int skew_tridiag_svdvals_d(skew_handle_t h, const double* ev, int64_t n, double* S, int* info);
SKEW_API int skew_tridiag_svd_d(skew_handle_t h, const double* ev, int64_t n, double* S, double* Ur, double* Ui,
                                double* Vr, double* Vi, int64_t ldu, int* info);
SKEW_API int skew_tridiag_svdvals_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* S,
                                    int* info);
SKEW_API int skew_tridiag_svd_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* S,
                                double* U, double* V, int64_t ldu, int* info);

/* ---------------------------------------------------------------------------
 * Tuning: the launch shapes and limits of the kernels, one table per handle.  The
 * reference fixes its one shape by rule (setnb, hessenberg.jl:133-142, the panel
 * width from n); here each shape that a measurement decides is a key.  A new handle
 * starts from the compiled-in defaults (measured on GB300) and then loads the
 * device's entry (matched by the CUDA device name) from the JSON table that the
 * environment variable SKEW_TUNING_FILE names, or else from skew_tuning.json beside
 * libskewgpu.so, written by the autotuner (skewgpu/autotune.py).  Keys
 * (skew_tuning_key lists them): bucket_edges (list), batch_smem_nmax,
 * batch_smem_nt_small, batch_smem_nt_large, batch_global_nt,
 * batch_global_ctas_per_sm, batch_graph, batch_merge_global (the global-memory size
 * buckets as one launch), batch_split_pct (that launch in two regions, the first with
 * this share of the work), func_chain_nmax, func_real_schur (functions of real
 * matrices in the real Schur basis), blocked_min_n,
 * blocked_persistent, cluster_max_n, persist_ctas, persist_tail, persist_items,
 * persist_nb (panel width of the blocked reduction, 8..128; 64 at most on the
 * multi-launch path), zpersist_min_n, zpersist_ctas, zpersist_items, zpersist_nb (the
 * complex panel width, 4..32), pfz_cta_max, pfz_nt, pfz_ctas, and the limits
 * wait_polls (grid-barrier polls before SKEW_TIMEOUT; 0: the default, seconds),
 * wait_skip_cta (>= 0: that CTA of a cooperative kernel skips its arrivals, so the
 * bounded waits run out: a test of the timeout path; -1: off) and qr_max_iter (QR
 * sweeps before SKEW_NO_CONVERGENCE; 0: the reference's 30 n, skeweigen.jl:115).
 * Batch plans take the bucket keys when they are created.  No reference counterpart.
 * ------------------------------------------------------------------------- */
/* One integer key; SKEW_BAD_ARG for an unknown key or a value out of its range. */
SKEW_API int skew_tuning_set(skew_handle_t h, const char* key, int64_t value);
/* A list key (bucket_edges: 1..8 ascending sizes). */
SKEW_API int skew_tuning_set_list(skew_handle_t h, const char* key, const int64_t* values, int count);
/* values[0 .. *count) <- the key's value(s) (cap: room in values). */
SKEW_API int skew_tuning_get(skew_handle_t h, const char* key, int64_t* values, int cap, int* count);
/* Back to the compiled-in defaults. */
SKEW_API int skew_tuning_reset(skew_handle_t h);
/* Load the device's entry from a table file; SKEW_UNSUPPORTED if it has none (no change),
 * SKEW_BAD_ARG if the file cannot be read or a value is out of range (no change). */
SKEW_API int skew_tuning_load(skew_handle_t h, const char* path);
/* Where the handle's table came from ("defaults", or the file and device name, then
 * " +key" for each key set since). */
SKEW_API const char* skew_tuning_source(skew_handle_t h);
/* The i-th key name (0-based), NULL past the last. */
SKEW_API const char* skew_tuning_key(int i);
/* What a table file holds for a device name, without a handle or a GPU: the key's
 * value(s) after loading the device's entry over the defaults.  SKEW_OK if the file
 * has an entry for the device, SKEW_UNSUPPORTED if not (values are the defaults),
 * SKEW_BAD_ARG if it cannot be read, a value is out of range or the key is unknown. */
SKEW_API int skew_tuning_file_get(const char* path, const char* device, const char* key, int64_t* values, int cap,
                                  int* count);

/* Diagnostics: measured FP64 DFMA throughput of the current device in TFLOP/s
 * (runs a short microbenchmark on the handle's stream and synchronizes). */
SKEW_API int skew_measure_fp64_peak(skew_handle_t h, double* tflops);
/* Diagnostics: the FP64 tensor instruction (mma.sync f64) against DFMA, in TFLOP/s:
 * tflops[0] DFMA, [1] mma m8n8k4, [2] mma m16n8k16, [3] half the warps DFMA and half
 * m8n8k4 in one kernel, [4] half DFMA and half m16n8k16 (equal flops per warp).  If
 * [3] and [4] are about [0], the two share one FP64 pipe (synchronises the stream). */
SKEW_API int skew_measure_fp64_pipes(skew_handle_t h, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* SKEWGPU_H */
