// Internal declarations shared by the libskewgpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace skew {

// Raises a kernel's dynamic shared-memory limit to the most the device allows
// beside the kernel's static shared memory (opt-in maximum minus static bytes),
// once per device (bit `device` of `done`), so that later launches, which may be
// recorded into a CUDA graph, issue no attribute calls.
inline cudaError_t raise_smem_limit_once(const void* kernel, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  const int dyn = optin - (int)fa.sharedSizeBytes;
  if (dyn <= 0) return cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
  if (e != cudaSuccess) return e;
  done.fetch_or(bit, std::memory_order_release);
  return cudaSuccess;
}

// Launch shapes and limits of the kernels, one table per handle (skew_tuning.cu):
// compiled-in defaults measured on GB300, replaced per device by a table the
// autotuner writes, or key by key through skew_tuning_set.
constexpr int kMaxBucketEdges = 8;
struct Tuning {
  // batched plans (fixed when a plan is created)
  int bucket_edges[kMaxBucketEdges];  // a bucket holds the matrices with n <= edge (ascending)
  int nedges;
  int batch_smem_nmax;           // working copy in shared memory up to this n (and if it fits)
  int batch_smem_nt_small;       // threads per CTA of shared-memory buckets with nmax <= 96
  int batch_smem_nt_large;       // ... above 96
  int batch_global_nt;           // threads per CTA of global-memory buckets
  int batch_global_ctas_per_sm;  // resident CTAs per SM for global-memory buckets
  int batch_graph;               // 1: batched calls record and replay CUDA graphs
  int batch_merge_global;        // 1: consecutive global-memory buckets run as one launch
  int batch_split_pct;           // global-memory launches: first region holds this % of the work (0: one)
  int func_chain_nmax;           // function paths: the QR chain up to this n, bisection above
  int func_real_schur;           // 1: functions of real matrices in the real Schur basis
  // one large real matrix
  int blocked_min_n;             // the blocked multi-CTA reduction from this n
  int blocked_persistent;        // 1: one cooperative launch for all panels
  int cluster_max_n;             // up to this n, one 16-CTA cluster with the matrix in shared memory
  int persist_ctas;              // grid of the persistent reduction (0: chosen by n)
  int persist_tail;              // columns left to the one-CTA kernel (0: the default)
  int persist_items;             // matvec tiles per warp and column
  int persist_nb;                // panel width of the blocked reduction (setnb's role)
  // ComplexF64
  int zpersist_min_n;            // the persistent complex reduction from this n
  int zpersist_ctas;             // its grid (0: one CTA per SM)
  int zpersist_items;            // its matvec tiles per warp and column
  int zpersist_nb;               // its panel width
  int pfz_cta_max;               // complex Pfaffian: one CTA per matrix up to this n, a grid above
  int pfz_nt;                    // threads per CTA of the one-CTA Pfaffian (0: chosen by n)
  int pfz_ctas;                  // grid of the cooperative Pfaffian (0: chosen by n)
  // bounded waits and iteration limits
  long long wait_polls;          // grid-barrier polls before SKEW_TIMEOUT (0: the kernel's default)
  int wait_skip_cta;             // >= 0: this CTA skips its arrivals, so the barrier waits run out
  int qr_max_iter;               // > 0: QR sweeps before SKEW_NO_CONVERGENCE (0: 30 n, the reference's)
};
void tuning_defaults(Tuning* T);
int tuning_set(Tuning* T, const char* key, const long long* values, int count);
int tuning_get(const Tuning* T, const char* key, long long* values, int cap, int* count);
const char* tuning_key_name(int i);
int tuning_load_file(Tuning* T, const char* path, const char* device, bool* found);

// Batched one-CTA-per-matrix launches (skew_batch.cu).
struct BatchParams {
  const double* const* A;  // [count] device pointers, original order
  const int32_t* n;        // [count] sizes, original order
  const int32_t* order;    // processing order -> original index (largest first)
  int32_t begin, end;      // slice of `order` handled by this launch
  int32_t nmax;            // largest n in the slice
  int32_t smem_matrix;     // 1: working copy in shared memory; 0: global slot
  int32_t check;           // verify A == -A^T
  double* gws;             // global workspace (one slot per CTA) when !smem_matrix
  int64_t gws_slot;        // doubles per slot
  unsigned* counter;       // work counter (two words, 8-byte aligned), zero before the launch
  double* logpf;           // [count] or null
  double* sign;            // [count] or null
  double* const* grad;     // [count] device pointers or null
  double* ev_out;          // packed ev (n-1 per matrix) or null
  const int64_t* ev_off;   // offsets into ev_out (and tau_out)
  double* tau_out;         // packed tau, same offsets, or null
  double* const* refl_out; // [count] n x n buffers receiving the reduced matrix (reflectors) or null
  int* status;             // [count] or null
  int32_t nt = 0;          // threads per CTA (0: the default for the copy's location)
  int32_t host_in = 0;     // A[] point into page-locked host memory (read with more loads in flight)
  double* const* grad_host = nullptr;  // [count] page-locked host destinations: the finished
                                       // gradient is copied there by the CTA that formed it
  int32_t split = 0;       // > begin: two regions [begin, split) and [split, end) with a
                           // counter each (counter[0], counter[1]); the first half of the CTAs
                           // starts in the first, the second half in the second
};

struct SingleParams {
  double* A;
  int64_t lda;
  int n;
  double* G;
  int64_t ldg;
  double* logpf;
  double* sign;
  double* ev;
  double* tau;
  int* info;
  int check;
  int want_pf;
};

size_t batch_smem_bytes(int nmax, bool smem_matrix, int nt);
cudaError_t launch_batch_pf(const BatchParams& P, int grid, cudaStream_t st, bool tridiag_only);
cudaError_t launch_single(const SingleParams& P, cudaStream_t st);
int batch_threads();
int batch_occupancy(int nmax, bool smem_matrix, int nt);  // resident CTAs per SM

// Skew tridiagonal eigenvalues (skew_qr.cu).
struct TrieigParams {
  const double* ev_all;    // packed subdiagonals (n-1 per matrix)
  const int64_t* ev_off;   // [count]
  const int32_t* n;        // [count]
  const int32_t* order;    // [count] processing order
  int32_t count;
  double* evwork;          // packed scratch, same layout as ev_all
  double* const* vals;     // [count] device pointers (n[b] each)
  int* status;             // [count] or null
  unsigned* fallback;      // [2 + 2 count]: number of stagnated matrices, work counter,
                           // then their indices and active sizes (solved by a second kernel)
  int grid;                // CTAs of the fallback kernel
  int max_iter = 0;        // QR sweeps before SKEW_NO_CONVERGENCE (0: 30 n, skeweigen.jl:115)
};
cudaError_t launch_batch_trieig(const TrieigParams& P, cudaStream_t st);

// Eigenvalues of one skew tridiagonal by bisection on the equivalent zero-diagonal
// symmetric tridiagonal; vals_im sorted descending.
cudaError_t launch_tridiag_bisect(const double* ev, int n, double* vals_im, double* scratch2, cudaStream_t st);
// selected eigenvalues (by 1-based index range or by the interval [vl, vh) of the
// imaginary parts), negated eigenvalues of the symmetric tridiagonal (dg or zero, e);
// bnd: sym_bound ? {bound, pivmin} : {lo, pivmin, hi}; *count (device) = how many
cudaError_t launch_select(const double* e, const double* dg, int n, const double* bnd, int sym_bound, int by_index,
                          int il, int iu, double vl, double vh, double* out, int* count, cudaStream_t st);
cudaError_t launch_tridiag_bounds(const double* ev, int n, double* bnd, cudaStream_t st);
// complex: the real symmetric tridiagonal of i T (diagonal -dvim, off-diagonal |ev|) and
// its bounds {lo, pivmin, hi} (plus the phases, unused here)
cudaError_t zsymtri_prep(const double* ev, const double* dvim, int n, double* dg, double* off, double* ph,
                         double* bnd, cudaStream_t st);
// eigen of a SkewHermTridiagonal{ComplexF64} (complex ev, dvim or null): vals_im, V = D Y
cudaError_t zeigen_tridiag(const double* ev, const double* dvim, int n, double* vals_im, double* V, int64_t ldv,
                           double* ws, cudaStream_t st);

// ComplexF64 Householder tridiagonalisation (skew_complex.cu).  Complex values are
// interleaved (re, im).  Batched: W[b] (in place, ld n[b]), tau/ev/dvim at off[b];
// single: W == nullptr and W1/n1/ld1 (off 0).  counter == nullptr: CTA b takes
// matrix b (grid = count), else matrices come from the counter (largest first via order).
struct ZHessParams {
  double* const* W;
  double* W1;
  int n1;
  int64_t ld1;
  const int32_t* n;
  const int32_t* order;
  const int64_t* off;
  int32_t count;
  int nmax;
  unsigned* counter;
  int64_t stride;  // W == nullptr: matrix b at W1 + b * stride (complex elements)
  double* tau;   // complex
  double* ev;    // real subdiagonal
  double* dvim;  // imag(diag) after the reduction, or null
};
size_t zhess_cta_smem_bytes(int nmax);
cudaError_t launch_zhess_cta(const ZHessParams& P, int grid, cudaStream_t st);
size_t zhess_large_ws_doubles(int n);
// imag(diag(A)) of a reduced matrix into dvim
cudaError_t launch_zdiag_im(const double* A, int64_t lda, int n, double* dvim, cudaStream_t st);
// One cooperative launch for all panels of one large matrix (skew_zblocked.cu), then the
// tail with the one-CTA kernel.  cudaErrorNotSupported where it cannot run (the caller
// falls back to zhess_large); info <- SKEW_TIMEOUT if a grid barrier gave up.
size_t zhess_persist_ws_doubles(int n);
cudaError_t zhess_persistent(double* A, int64_t lda, int n, double* tau, double* ev, double* dvim, double* ws,
                             int sms, int* info, const Tuning& T, cudaStream_t st);
cudaError_t zhess_large(double* A, int64_t lda, int n, double* tau, double* ev, double* dvim, double* ws,
                        cudaStream_t st);
// complex eigen from `batch` reduced matrices of size n (arrays per matrix: A lda*n,
// tau/ev/dvim/vals n, V ldv*n apart); values descending (-mu, mu ascending), vectors Q D Y
size_t zeigen_ws_doubles(int n, int batch);
cudaError_t zeigen_from_tridiag(const double* A, int64_t lda, int n, const double* tau, const double* ev,
                                const double* dvim, double* vals_im, double* V, int64_t ldv, double* ws, int batch,
                                cudaStream_t st);
// mode 0: O = V f(i mu) V^H for the matrix function `func` (skew_func_t), projected on
// the Hermitian / skew-Hermitian part where the function's result has that symmetry;
// mode 1: the adjoint of exp, O = V (conj(Phi) o (V^H C V)) V^H.  `batch` problems with
// operands ld*n apart; status (count, or null) gets SKEW_SINGULAR where f has no value.
size_t zfunc_ws_doubles(int n, int batch);
cudaError_t zfunc_from_eigen(int mode, int func, int n, const double* vals_im, const double* V, int64_t ldv,
                             const double* C, int64_t ldc, double* O, int64_t ldo, double* ws, int batch, int* status,
                             cudaStream_t st);

// Eigenvectors of one large skew matrix after the blocked reduction (skew_tdvec.cu):
// vals (descending, from launch_tridiag_bisect) and its scratch bp (bound, pivmin);
// A holds the reflectors, tau their scalars, ev the subdiagonal.  Vr, Vi (n x n, ldv).
size_t large_eigen_ws_doubles(int n);
cudaError_t symtri_vectors(const double* dg, const double* e, int n, const double* mu, const double* bp, double* Y,
                           double* ws, int batch, cudaStream_t st);
// gate: a device int of scratch; aux: large_eigen_aux_doubles(n) doubles of scratch.
// A tridiagonal that splits exactly into more odd-size blocks than n mod 2 (several
// zero eigenvalues) is solved in full mode, as the reference's fallback does.
size_t large_eigen_aux_doubles(int n);
cudaError_t large_eigen_vectors(const double* A, int64_t lda, int n, const double* tau, const double* ev,
                                const double* vals, const double* bp, double* Vr, double* Vi, int64_t ldv, double* ws,
                                int* gate, double* aux, cudaStream_t st);

// Eigenvectors / exp / cis / exp adjoint for batches of real skew matrices (skew_eigen.cu).
// Leading dimensions of every per-matrix n x n buffer are n.
struct EigenBatch {
  int32_t count;
  int32_t nmax;
  const int32_t* order;      // processing order (largest first)
  const int32_t* n;          // sizes
  const int64_t* off_n;      // packed offsets (>= max(n,1) apart) of ev, evb, tau, G
  double* ev;                // subdiagonals from the reduction (consumed by the QR)
  double* evb;               // copy kept for the stagnation fallback
  double* tau;               // reflector scalars
  double* G;                 // reducetozero rotations (odd n)
  double* const* vals;       // [count] -> n (imaginary parts of the eigenvalues)
  double* log;               // rotation logs
  const int64_t* off_log;    // per-matrix log offsets
  const int64_t* cap_log;    // per-matrix log capacity (doubles)
  int64_t* log_len;          // per-matrix log length
  int* status;               // per-matrix skew_status_t
  unsigned* counter;         // work counter of the per-matrix kernels
  double* const* Vr;         // [count] n x n real parts of the eigenvectors
  double* const* Vi;         // [count] n x n imaginary parts
  double* const* refl;       // [count] n x n reduced matrices (reflectors)
  double* work;              // 4 n^2 per matrix
  const int64_t* off_w;
  double* const* out;        // [count] exp (real) / cis (complex interleaved) / adjoint (real)
  const double* const* cot;  // [count] cotangents for the adjoint
  double* const* pwork;      // [count] work + off_w (pointer array for the tiled products)
  int func;                  // skew_func_t of mode 0 (exp and the other matrix functions)
  int merged;                // 1: skewtrieigen_merged! (tridiagonal input; no mem deflation of :355)
  int chain_nmax;            // matrices with n > chain_nmax skip the QR chain and its vectors
                             // (their eigenpairs come from bisection and twisted vectors)
  int max_iter = 0;          // QR sweeps before SKEW_NO_CONVERGENCE (0: 30 n, skeweigen.jl:340)
  int* fsel = nullptr;       // [count] exp adjoint: 1 real Schur-basis path, 0 complex path
                             // (null: the complex path for every matrix)
  const int32_t* back_off = nullptr;  // [count + 1] back-transformation items before each matrix
                             // of the processing order (null: one item per matrix)
  int32_t back_items = 0;    // total items (chunks of kBackCols columns)
  int back_q = 0;            // 1: the real Schur basis Q was built in the tridiagonal basis
                             // (pwork block 0): the back-transformation takes Q alone for the
                             // matrices with fsel = 1, and the adjoint starts from it
};
// Eigenpairs of G skew tridiagonals of one size n (subdiagonals e_g, n apart) by
// bisection (values descending, exact +-pairs, also into vals_out[idx[mb]]) and
// twisted-factorisation vectors with the banded orthogonal correction, written in
// the tridiagonal basis to Vr[idx[mb]], Vi[idx[mb]] (n x n, leading dimension n).
// ws: G x skew_vectors_batch_ws_doubles(n); bp_g: 8 G; vals_g: n G.
cudaError_t launch_tridiag_bisect_batch(const double* e_g, int n, int G, double* bp_g, double* vals_g,
                                        double* const* vals_out, const int32_t* idx, cudaStream_t st);
size_t skew_vectors_batch_ws_doubles(int n);
cudaError_t skew_vectors_batch(const double* e_g, int n, int G, const double* vals_g, const double* bp_g,
                               double* const* Vr, double* const* Vi, const int32_t* idx, double* ws,
                               cudaStream_t st);
// e_g[mb n + i] = ev[off_n[idx[mb]] + i] (i < n - 1), 0 at i = n - 1
cudaError_t launch_gather_ev(const double* ev, const int64_t* off_n, const int32_t* idx, int n, int G, double* e_g,
                             cudaStream_t st);
// copies n[b] - 1 subdiagonal entries from ev_in[b] to ev + off[b] for every matrix
cudaError_t launch_copy_ev(const double* const* ev_in, const int32_t* n, const int64_t* off, int count, double* ev,
                           cudaStream_t st);
// doubles of per-matrix work the eigen kernels need (4 n^2, or more for the fallback of small n)
size_t eigen_work_doubles(int n);
// Columns per work item of the batched back-transformation (of [Vr | Vi], 2n columns).
constexpr int kBackCols = 64;
inline int back_items_of(int n) { return n < 3 ? 0 : (2 * n + kBackCols - 1) / kBackCols; }
cudaError_t launch_eigen_chain(const EigenBatch& E, cudaStream_t st);
cudaError_t launch_eigen_vectors(const EigenBatch& E, int grid, cudaStream_t st);
cudaError_t launch_eigen_back(const EigenBatch& E, int grid, int nmax, cudaStream_t st);
// exp / cis / exp adjoint from (vals, Vr, Vi): elementwise kernels and tiled
// batched products over the whole GPU (tiles of every matrix in one launch).
cudaError_t launch_eigen_func(const EigenBatch& E, int mode, cudaStream_t st);
// exp adjoint: the real Schur basis Q (and fsel) from vals, Vr, Vi into pwork
cudaError_t launch_schur_basis(const EigenBatch& E, cudaStream_t st);

// Multi-CTA blocked reduction of one large matrix (skew_blocked.cu).
size_t blocked_ws_doubles(int n);
cudaError_t blocked_hessenberg(double* A, int64_t lda, int n, double* tau, double* ev, int* info, double* ws, int sms,
                               int nb, cudaStream_t st);
size_t persist_ws_extra_doubles();
// One moderate-size matrix (3 <= n, 16 x its shared memory per CTA) in one 16-CTA
// thread-block cluster, the matrix in distributed shared memory (skew_cluster.cu);
// cudaErrorNotSupported if the device cannot run that cluster.
cudaError_t cluster_hessenberg(double* A, int64_t lda, int n, double* tau, double* ev, int* info, cudaStream_t st);
// One cooperative launch for all panels (grid barriers with bounded waits); then the tail.
cudaError_t blocked_hessenberg_persistent(double* A, int64_t lda, int n, double* tau, double* ev, int* info,
                                          double* ws, int sms, int* err_dev, const Tuning& T, cudaStream_t st);
cudaError_t launch_pf_from_tridiag(const double* ev, const double* tau, int n, double* logpf, double* sign, int* info,
                                   const double* notskew, cudaStream_t st);
cudaError_t launch_check_skew(const double* A, int64_t lda, int n, double* flag, int sms, cudaStream_t st);

// Complex skew-symmetric Pfaffian, Parlett-Reid with pivoting (skew_pfz.cu).
struct zc;
struct PfzParams {
  const zc* A;  // matrix b at A + b * stride, column-major, leading dimension lda; read only
  int64_t lda, stride;
  int n, count, check;
  int smem_matrix;  // 1: packed triangle in shared memory, 0: in the per-CTA slot of gws
  zc* gws;
  int64_t slot;  // complex entries per slot (n (n - 1) / 2)
  double* logpf;  // [count] (nullable)
  double* phase;  // [2 count] cis(phase) (nullable)
  double* pf;     // [2 count] the product (nullable)
  int* status;    // [count] (nullable)
  int nt;         // threads per CTA of the shared-memory kernel (0: chosen by n)
};
struct PfzGridParams {
  zc* A;  // in place on the strictly lower triangle
  int64_t lda;
  int n;
  zc* tau;
  zc* cc;
  zc* piv;  // n/2 recorded pivots
  unsigned long long* part_v;  // argmax keys
  int* part_i;
  unsigned* sync;
  int* err;
  const double* notskew;
  double* logpf;
  double* phase;
  double* pf;
  int* info;
  long long poll_limit;  // polls before a grid barrier gives up
  int skip_cta;          // >= 0: this CTA never arrives (a test of the timeout path)
};
size_t pfz_cta_smem(int n, bool smem_matrix);
bool pfz_smem_fits(int n);
int pfz_cta_occupancy(int n, bool smem_matrix, int nt);
cudaError_t launch_pfz_cta(const PfzParams& P, int grid, cudaStream_t st);
size_t pfz_grid_ws_doubles(int n);
// n >= 1 (odd n: Pf = 0); check != 0 tests A == -transpose(A) first (info = SKEW_NOT_SKEW).
cudaError_t launch_pfz_grid(zc* A, int64_t lda, int n, int check, double* logpf, double* phase, double* pf,
                            int* info, double* ws, int sms, const Tuning& T, cudaStream_t st);

// svdvals / svd from the eigenpairs (skew_svd.cu).  Stable rank sort of each problem's
// values by |v| descending: perm (batch x n, nullable), S (sstride apart, nullable),
// sgn (batch x n, -1 for negative values, nullable).
cudaError_t launch_svd_rank(const double* vals, int n, int64_t vstride, int batch, int* perm, double* S,
                            int64_t sstride, double* sgn, cudaStream_t st);
// U[:, k] = W[:, perm[k]], V[:, k] = -i sgn[k] U[:, k]; W may share storage with V.
cudaError_t launch_svd_vectors_d(const double* Wr, const double* Wi, int n, int64_t ld, const int* perm,
                                 const double* sgn, double* Ur, double* Ui, double* Vr, double* Vi, cudaStream_t st);
cudaError_t launch_svd_vectors_z(const double* W, int n, int64_t ld, const int* perm, const double* sgn, double* U,
                                 double* V, cudaStream_t st);

// FP64 DFMA microbenchmark kernel (skew_api.cu).
cudaError_t launch_dfma_probe(double* out, int blocks, int iters, cudaStream_t st);

}  // namespace skew
