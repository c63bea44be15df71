// C ABI of libskewgpu (declared in include/skewgpu.h): handles, batch plans and
// the single-matrix entry points.  Host code only dispatches and owns
// workspaces; every numerical step runs in the kernels of the other units.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/skewgpu.h"
#include "skew_internal.h"

using namespace skew;

namespace skew {
std::string tuning_default_path();
}

struct skew_handle_st {
  cudaStream_t stream = nullptr;
  int device = 0;
  int sms = 0;
  void* ws = nullptr;  // grow-only workspace, stream ordered
  size_t ws_bytes = 0;
  void* aux = nullptr;  // small grow-only scratch kept across calls that use ws themselves
  size_t aux_bytes = 0;
  struct skew_batch_plan_st* plan1 = nullptr;  // batch-of-one plan for single-matrix eigen/exp/cis
  int64_t plan1_n = 0;
  Tuning tune;              // launch shapes and limits (compiled defaults, then the device's table)
  std::string tune_source;  // where tune came from
};

struct Bucket {
  int begin, end, nmax, smem_matrix, grid, nt;
  int64_t gws_slot;  // doubles per CTA slot (global bucket)
  int split = 0;     // > begin: the work median of the slice (two regions, see batch_kernel)
  size_t gws_off;    // offset of the bucket's slots in the plan workspace (doubles)
};

struct skew_batch_plan_st {
  skew_handle_t h = nullptr;
  Tuning tune;  // the handle's table when the plan was created (bucket shapes)
  int64_t count = 0;
  std::vector<int32_t> n_host;
  std::vector<Bucket> buckets;
  int32_t* d_n = nullptr;
  int32_t* d_order = nullptr;
  int64_t* d_ev_off = nullptr;
  unsigned* d_counters = nullptr;
  unsigned* d_fallback = nullptr;  // eigvals: stagnated matrices for the fallback kernel
  double* d_ev = nullptr;
  double* d_gws = nullptr;
  int64_t ev_total = 0;
  size_t gws_total = 0;
  // eigen / exp workspace, allocated on first use
  bool eig_ready = false;
  int nmax = 0;
  double* e_refl = nullptr;   // sum n^2
  double* e_tau = nullptr;    // ev_total (ev offsets)
  double* e_evb = nullptr;
  double* e_G = nullptr;
  double* e_log = nullptr;
  double* e_work = nullptr;   // 4 sum n^2
  double* e_vr = nullptr;     // internal eigenvectors (exp, cis, vjp)
  double* e_vi = nullptr;
  double* e_vals = nullptr;   // internal eigenvalues (ev offsets)
  int64_t* e_off_log = nullptr;
  int64_t* e_cap_log = nullptr;
  int64_t* e_log_len = nullptr;
  int64_t* e_off_w = nullptr;
  double** e_p_refl = nullptr;  // device pointer arrays
  double** e_p_vr = nullptr;
  double** e_p_vi = nullptr;
  double** e_p_vals = nullptr;
  double** e_p_scratch = nullptr;  // 8 x count: single-call pointer arrays
  double** e_p_work = nullptr;     // work + off_w per matrix
  int* e_status = nullptr;
  unsigned* e_counter = nullptr;
  int* e_fsel = nullptr;  // exp adjoint: per matrix, real Schur-basis (1) or complex (0) form
  int32_t* e_back_off = nullptr;  // back-transformation items before each matrix (processing order)
  int32_t back_items = 0;
  // one instantiated CUDA graph per batched operation, keyed on its arguments
  struct GraphSlot {
    bool valid = false;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
    std::array<const void*, 6> key{};
  };
  GraphSlot graphs[6];
  bool graphs_off = false;              // capture failed once (or disabled): launch directly
  // host-buffer logabspfaffian (skew_batch_logabspf_host_d), allocated on first use
  int64_t hio_total = 0;       // sum n^2
  int64_t* hio_off = nullptr;  // packed offsets (creation order)
  double** hio_a = nullptr;    // [count] host-mapped input addresses
  double** hio_gh = nullptr;   // [count] host-mapped gradient destinations
  double** hio_g = nullptr;    // [count] device gradient slots
  double* hio_grad = nullptr;  // sum n^2 doubles
  double* hio_out = nullptr;   // logpf, sign (2 x count)
  int* hio_status = nullptr;
  // function paths (exp, cis, the exp adjoint, matrix functions): matrices with
  // n > fv_thresh take bisection and twisted vectors instead of the QR chain,
  // by size group; built once per plan and threshold (outside any capture)
  struct FvGroup {
    int n, start, count, chunk;
  };
  int fv_thresh = -1;
  std::vector<FvGroup> fv_groups;
  int32_t* fv_idx = nullptr;  // matrix indices, grouped by size
  double* fv_ws = nullptr;    // e_g | bp_g | vals_g | vector workspace of one chunk
  size_t fv_ws_doubles = 0;
  cudaStream_t capture_stream = nullptr;  // graphs are recorded here, launched on the caller's stream
};

#define CK(x)                                  \
  do {                                         \
    cudaError_t e_ = (x);                      \
    if (e_ != cudaSuccess) return SKEW_CUDA_ERROR; \
  } while (0)

static int ensure_ws(skew_handle_t h, size_t bytes) {
  if (bytes <= h->ws_bytes) return SKEW_OK;
  if (h->ws) CK(cudaFreeAsync(h->ws, h->stream));
  h->ws = nullptr;
  h->ws_bytes = 0;
  CK(cudaMallocAsync(&h->ws, bytes, h->stream));
  h->ws_bytes = bytes;
  return SKEW_OK;
}

static int ensure_aux(skew_handle_t h, size_t bytes) {
  if (bytes <= h->aux_bytes) return SKEW_OK;
  if (h->aux) CK(cudaFreeAsync(h->aux, h->stream));
  h->aux = nullptr;
  h->aux_bytes = 0;
  CK(cudaMallocAsync(&h->aux, bytes, h->stream));
  h->aux_bytes = bytes;
  return SKEW_OK;
}

extern "C" {

int skew_version(void) { return 100; }

const char* skew_status_string(int s) {
  switch (s) {
    case SKEW_OK: return "ok";
    case SKEW_NOT_SKEW: return "matrix is not skew-symmetric";
    case SKEW_NO_CONVERGENCE: return "maximum number of iterations reached, the algorithm didn't converge";
    case SKEW_BAD_ARG: return "bad argument";
    case SKEW_CUDA_ERROR: return "CUDA error";
    case SKEW_SINGULAR: return "singular (Pfaffian is zero)";
    case SKEW_UNSUPPORTED: return "unsupported";
    case SKEW_NO_MEMORY: return "out of memory";
    case SKEW_FALLBACK_USED: return "QR stagnated; symmetric tridiagonal fallback used";
    case SKEW_TIMEOUT: return "a bounded device-side wait gave up (timeout)";
    default: return "unknown status";
  }
}

int skew_create(skew_handle_t* handle) {
  if (!handle) return SKEW_BAD_ARG;
  skew_handle_st* h = new (std::nothrow) skew_handle_st();
  if (!h) return SKEW_NO_MEMORY;
  cudaDeviceProp prop;
  if (cudaGetDevice(&h->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess ||
      cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) {
    delete h;
    return SKEW_CUDA_ERROR;
  }
  // the compiled-in defaults, then the table for this device's name, if there is one
  tuning_defaults(&h->tune);
  h->tune_source = "defaults";
  const std::string path = tuning_default_path();
  bool found = false;
  if (FILE* f = std::fopen(path.c_str(), "rb")) {
    std::fclose(f);
    if (tuning_load_file(&h->tune, path.c_str(), prop.name, &found) != SKEW_OK)
      h->tune_source = "defaults (unreadable table: " + path + ")";
    else if (found)
      h->tune_source = path + " [" + prop.name + "]";
  }
  *handle = h;
  return SKEW_OK;
}

int skew_tuning_set(skew_handle_t h, const char* key, int64_t value) {
  if (!h) return SKEW_BAD_ARG;
  const long long v = value;
  const int s = tuning_set(&h->tune, key, &v, 1);
  if (s == SKEW_OK) h->tune_source += std::string(" +") + key;
  return s;
}

int skew_tuning_set_list(skew_handle_t h, const char* key, const int64_t* values, int count) {
  if (!h || !values || count < 1 || count > kMaxBucketEdges) return SKEW_BAD_ARG;
  long long v[kMaxBucketEdges];
  for (int i = 0; i < count; i++) v[i] = values[i];
  const int s = tuning_set(&h->tune, key, v, count);
  if (s == SKEW_OK) h->tune_source += std::string(" +") + key;
  return s;
}

static int tuning_get_i64(const Tuning* T, const char* key, int64_t* values, int cap, int* count) {
  if (!values || cap < 1) return SKEW_BAD_ARG;
  long long v[kMaxBucketEdges];
  int c = 0;
  const int s = tuning_get(T, key, v, kMaxBucketEdges, &c);
  if (s != SKEW_OK) return s;
  for (int i = 0; i < c && i < cap; i++) values[i] = v[i];
  if (count) *count = c;
  return SKEW_OK;
}

int skew_tuning_get(skew_handle_t h, const char* key, int64_t* values, int cap, int* count) {
  if (!h) return SKEW_BAD_ARG;
  return tuning_get_i64(&h->tune, key, values, cap, count);
}

int skew_tuning_reset(skew_handle_t h) {
  if (!h) return SKEW_BAD_ARG;
  tuning_defaults(&h->tune);
  h->tune_source = "defaults";
  return SKEW_OK;
}

int skew_tuning_load(skew_handle_t h, const char* path) {
  if (!h || !path) return SKEW_BAD_ARG;
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, h->device));
  bool found = false;
  const int s = tuning_load_file(&h->tune, path, prop.name, &found);
  if (s != SKEW_OK) return s;
  if (!found) return SKEW_UNSUPPORTED;  // no entry for this device: nothing changed
  h->tune_source = std::string(path) + " [" + prop.name + "]";
  return SKEW_OK;
}

const char* skew_tuning_source(skew_handle_t h) { return h ? h->tune_source.c_str() : nullptr; }

const char* skew_tuning_key(int i) { return tuning_key_name(i); }

int skew_tuning_file_get(const char* path, const char* device, const char* key, int64_t* values, int cap,
                         int* count) {
  if (!path || !device || !key || !values || cap < 1) return SKEW_BAD_ARG;
  Tuning T;
  tuning_defaults(&T);
  bool found = false;
  int s = tuning_load_file(&T, path, device, &found);
  if (s != SKEW_OK) return s;
  s = tuning_get_i64(&T, key, values, cap, count);
  if (s != SKEW_OK) return s;
  return found ? SKEW_OK : SKEW_UNSUPPORTED;
}

int skew_destroy(skew_handle_t h) {
  if (!h) return SKEW_BAD_ARG;
  if (h->plan1) skew_batch_plan_destroy(h->plan1);
  if (h->ws) cudaFreeAsync(h->ws, h->stream);
  if (h->aux) cudaFreeAsync(h->aux, h->stream);
  if (h->ws || h->aux) cudaStreamSynchronize(h->stream);
  delete h;
  return SKEW_OK;
}

int skew_set_stream(skew_handle_t h, skew_stream_t s) {
  if (!h) return SKEW_BAD_ARG;
  if ((h->ws || h->aux) && (cudaStream_t)s != h->stream) {  // keep the workspaces ordered on the new stream
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, h->stream));
    CK(cudaStreamWaitEvent((cudaStream_t)s, ev, 0));
    CK(cudaEventDestroy(ev));
  }
  h->stream = (cudaStream_t)s;
  return SKEW_OK;
}

// Largest n handled by the one-CTA single-matrix kernel, and the size above
// which single-matrix calls use the multi-CTA blocked reduction instead (the
// tuning key blocked_min_n).
static const int64_t kSingleMax = 1024;
static int64_t blocked_min_n(skew_handle_t h) { return h->tune.blocked_min_n; }

static int single(skew_handle_t h, double* A, int64_t n, int64_t lda, double* G, int64_t ldg, double* logpf,
                  double* sign, double* ev, double* tau, int* info, int check, int want_pf) {
  if (!h || n < 0 || (n > 0 && (!A || lda < n))) return SKEW_BAD_ARG;
  if (n > kSingleMax) return SKEW_UNSUPPORTED;
  SingleParams P;
  P.A = A;
  P.lda = lda;
  P.n = (int)n;
  P.G = G;
  P.ldg = ldg;
  P.logpf = logpf;
  P.sign = sign;
  P.ev = ev;
  P.tau = tau;
  P.info = info;
  P.check = check;
  P.want_pf = want_pf;
  CK(launch_single(P, h->stream));
  return SKEW_OK;
}

// Blocked reduction of a large matrix into tau/ev (device); A in place.
static int blocked(skew_handle_t h, double* A, int64_t n, int64_t lda, double* tau, double* ev, int* info,
                   size_t extra_doubles, double** extra) {
  if (!h || !A || lda < n || n > (1LL << 15)) return n > (1LL << 15) ? SKEW_UNSUPPORTED : SKEW_BAD_ARG;
  const size_t wsd = blocked_ws_doubles((int)n) + persist_ws_extra_doubles();
  int st = ensure_ws(h, sizeof(double) * (wsd + extra_doubles));
  if (st) return st;
  double* ws = (double*)h->ws;
  if (extra) *extra = ws + wsd;
  if (!tau || !ev) {  // caller wants only the tridiagonal: use the extra area
    if (!extra || extra_doubles < 2 * (size_t)n) return SKEW_BAD_ARG;
    ev = ws + wsd;
    tau = ws + wsd + n;
  }
  // up to cluster_max_n: one 16-CTA cluster with the matrix in distributed shared
  // memory (no device-wide barriers)
  if (n >= 3 && n <= h->tune.cluster_max_n) {
    if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
    cudaError_t e = cluster_hessenberg(A, lda, (int)n, tau, ev, info, h->stream);
    if (e == cudaSuccess) return SKEW_OK;
    if (e != cudaErrorNotSupported) return SKEW_CUDA_ERROR;
    cudaGetLastError();
  }
  // one cooperative launch for all panels when v fits in shared memory; the
  // multi-launch path otherwise (or with the tuning key blocked_persistent = 0)
  const bool persistent = n <= 24576 && h->tune.blocked_persistent != 0;
  if (persistent) {
    cudaError_t e =
        blocked_hessenberg_persistent(A, lda, (int)n, tau, ev, info, ws, h->sms, nullptr, h->tune, h->stream);
    if (e == cudaSuccess) return SKEW_OK;
    if (e != cudaErrorNotSupported && e != cudaErrorCooperativeLaunchTooLarge) return SKEW_CUDA_ERROR;
    cudaGetLastError();
  }
  CK(blocked_hessenberg(A, lda, (int)n, tau, ev, info, ws, h->sms, h->tune.persist_nb, h->stream));
  return SKEW_OK;
}

int skew_hessenberg_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* tau, double* ev, int* info) {
  if (n > 1 && (!tau || !ev)) return SKEW_BAD_ARG;
  if (n >= blocked_min_n(h)) return blocked(h, A, n, lda, tau, ev, info, 0, nullptr);
  return single(h, A, n, lda, nullptr, 0, nullptr, nullptr, n > 1 ? ev : nullptr, n > 1 ? tau : nullptr, info, 0,
                0);
}

int skew_logabspf_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* sign, int check,
                    int* info) {
  if (!logpf || !sign) return SKEW_BAD_ARG;
  if (n >= blocked_min_n(h) && (n % 2) == 0) {
    double* extra = nullptr;
    // workspace layout: [blocked ws][ev (n)][tau (n)][not-skew flag]; size it before the check
    const size_t wsd = blocked_ws_doubles((int)n) + persist_ws_extra_doubles();
    int st = ensure_ws(h, sizeof(double) * (wsd + 2 * (size_t)n + 1));
    if (st) return st;
    double* flag = (double*)h->ws + wsd + 2 * (size_t)n;  // after blocked()'s ev/tau extra area
    if (check) CK(launch_check_skew(A, lda, (int)n, flag, h->sms, h->stream));
    st = blocked(h, A, n, lda, nullptr, nullptr, info, 2 * (size_t)n + 1, &extra);
    if (st) return st;
    CK(launch_pf_from_tridiag(extra, extra + n, (int)n, logpf, sign, info, check ? flag : nullptr, h->stream));
    return SKEW_OK;
  }
  return single(h, A, n, lda, nullptr, 0, logpf, sign, nullptr, nullptr, info, check, 1);
}

int skew_logabspf_grad_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* sign, double* G,
                         int64_t ldg, int* info) {
  if (!logpf || !sign || (n > 0 && (!G || ldg < n))) return SKEW_BAD_ARG;
  return single(h, A, n, lda, G, ldg, logpf, sign, nullptr, nullptr, info, 0, 1);
}

static int single_plan(skew_handle_t h, int64_t n, skew_batch_plan_t* out);
static int tridiag_qr_vals(skew_handle_t h, const double* ev, int64_t n, double* vals_im, int* status);

// info <- the QR's status unless the reduction already reported an error.
__global__ void merge_qr_status_kernel(const int* qr, int* info) {
  if (*info == SKEW_OK) *info = *qr;
}

// Eigenvalues sorted descending by bisection on SymTridiagonal(0, ev) after the
// reduction (the values of skew_eigvals_d without the reference's QR order): the
// large-matrix path of skew_eigvals_d, and the values under svdvals, which sorts them.
static int eigvals_bisect_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !vals_im))) return SKEW_BAD_ARG;
  if (n == 0) return SKEW_OK;
  if (n == 1) {  // skeweigvals! n == 1 returns [A[1,1]] (eigen.jl:51)
    CK(cudaMemcpyAsync(vals_im, A, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
    if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
    return SKEW_OK;
  }
  if (n >= blocked_min_n(h)) {
    double* extra = nullptr;
    int st = blocked(h, A, n, lda, nullptr, nullptr, info, 2 * (size_t)n + 2, &extra);
    if (st) return st;
    CK(launch_tridiag_bisect(extra, (int)n, vals_im, extra + 2 * n, h->stream));
    return SKEW_OK;
  }
  int st = ensure_ws(h, sizeof(double) * (size_t)(n + 2));
  if (st) return st;
  double* ev = (double*)h->ws;
  st = single(h, A, n, lda, nullptr, 0, nullptr, nullptr, ev, nullptr, info, 0, 0);
  if (st) return st;
  CK(launch_tridiag_bisect(ev, (int)n, vals_im, ev + n, h->stream));
  return SKEW_OK;
}

int skew_eigvals_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !vals_im))) return SKEW_BAD_ARG;
  if (n <= 1 || n > kSingleMax) return eigvals_bisect_d(h, A, n, lda, vals_im, info);
  // n <= 1024: the reduction, then skewtrieigvals! (skeweigen.jl:105-156) on one lane,
  // which gives the values in the reference's deflation order (eigen.jl:49-55).
  skew_batch_plan_t P = nullptr;
  int st = single_plan(h, n, &P);
  if (st) return st;
  double* ev = nullptr;
  if (n >= blocked_min_n(h)) {
    double* extra = nullptr;
    st = blocked(h, A, n, lda, nullptr, nullptr, info, 2 * (size_t)n + 2, &extra);
    if (st) return st;
    ev = extra;
  } else {
    st = ensure_ws(h, sizeof(double) * (size_t)(n + 2));
    if (st) return st;
    ev = (double*)h->ws;
    st = single(h, A, n, lda, nullptr, 0, nullptr, nullptr, ev, nullptr, info, 0, 0);
    if (st) return st;
  }
  st = tridiag_qr_vals(h, ev, n, vals_im, info ? P->e_status : nullptr);
  if (st) return st;
  if (info) {
    merge_qr_status_kernel<<<1, 1, 0, h->stream>>>(P->e_status, info);
    CK(cudaGetLastError());
  }
  return SKEW_OK;
}


// Selected eigenvalues (eigvals(A, irange) / eigvals(A, vl, vh)): the reduction,
// then multisection on the selected indices only.
static int eigvals_select_d(skew_handle_t h, double* A, int64_t n, int64_t lda, int by_index, int64_t il, int64_t iu,
                            double vl, double vh, double* vals_im, int* count, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !vals_im || lda < n))) return SKEW_BAD_ARG;
  if (by_index && (il < 1 || iu < il || iu > n)) return SKEW_BAD_ARG;
  if (!by_index && !(vl < vh)) return SKEW_BAD_ARG;
  if (n == 0) {
    if (count) CK(cudaMemsetAsync(count, 0, sizeof(int), h->stream));
    return SKEW_OK;
  }
  double* ev = nullptr;
  double* bnd = nullptr;
  if (n >= blocked_min_n(h)) {
    double* extra = nullptr;
    int st = blocked(h, A, n, lda, nullptr, nullptr, info, 2 * (size_t)n + 8, &extra);
    if (st) return st;
    ev = extra;
    bnd = extra + 2 * n;
  } else {
    int st = ensure_ws(h, sizeof(double) * (size_t)(n + 8));
    if (st) return st;
    ev = (double*)h->ws;
    bnd = ev + n;
    st = single(h, A, n, lda, nullptr, 0, nullptr, nullptr, n > 1 ? ev : nullptr, nullptr, info, 0, 0);
    if (st) return st;
  }
  CK(launch_tridiag_bounds(ev, (int)n, bnd, h->stream));
  CK(launch_select(ev, nullptr, (int)n, bnd, 1, by_index, (int)il, (int)iu, vl, vh, vals_im, count, h->stream));
  return SKEW_OK;
}

int skew_eigvals_irange_d(skew_handle_t h, double* A, int64_t n, int64_t lda, int64_t il, int64_t iu, double* vals_im,
                          int* info) {
  return eigvals_select_d(h, A, n, lda, 1, il, iu, 0.0, 0.0, vals_im, nullptr, info);
}

int skew_eigvals_interval_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double vl, double vh,
                            double* vals_im, int* count, int* info) {
  if (!count) return SKEW_BAD_ARG;
  return eigvals_select_d(h, A, n, lda, 0, 0, 0, vl, vh, vals_im, count, info);
}

// ---------------------------------------------------------------------------
// Batched plans
// ---------------------------------------------------------------------------

// Size buckets (the tuning key bucket_edges; by default 32, 64, 96, 128, 152, and one
// bucket above the last edge): the working copy may stay in shared memory up to
// n = 152 (227 KB with the vectors and gradient scratch); larger matrices work in a
// per-CTA global slot (L2 resident).  The keys batch_smem_nmax and
// batch_global_ctas_per_sm pick the copy's location and the resident CTAs per SM of
// the global-memory buckets (each CTA holds an n x n working copy; 2 per SM keeps
// 152 * 2 * 0.5 MB in L2), batch_smem_nt_* / batch_global_nt the threads per CTA.
static int bucket_threads(const Tuning& T, int nmax, bool smem_matrix) {
  if (!smem_matrix) return T.batch_global_nt;
  return nmax <= 96 ? T.batch_smem_nt_small : T.batch_smem_nt_large;
}

int skew_batch_plan_create(skew_handle_t h, const int64_t* n, int64_t count, skew_batch_plan_t* plan) {
  if (!h || !plan || count < 0 || (count > 0 && !n)) return SKEW_BAD_ARG;
  for (int64_t b = 0; b < count; b++)
    if (n[b] < 0 || n[b] > kSingleMax) return SKEW_BAD_ARG;
  skew_batch_plan_st* P = new (std::nothrow) skew_batch_plan_st();
  if (!P) return SKEW_NO_MEMORY;
  P->h = h;
  P->tune = h->tune;
  P->count = count;
  P->n_host.resize(count);
  for (int64_t b = 0; b < count; b++) P->n_host[b] = (int32_t)n[b];
  std::vector<int32_t> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return P->n_host[a] > P->n_host[b]; });
  std::vector<int64_t> ev_off(count);
  int64_t acc = 0;
  for (int64_t b = 0; b < count; b++) {
    ev_off[b] = acc;
    acc += std::max<int32_t>(P->n_host[b], 1);
  }
  P->ev_total = acc;
  // buckets over the sorted order
  const Tuning& T = P->tune;
  auto edge_of = [&T](int nn) {
    for (int i = 0; i < T.nedges; i++)
      if (nn <= T.bucket_edges[i]) return T.bucket_edges[i];
    return 1 << 30;
  };
  size_t gws_total = 0;
  for (int64_t t = 0; t < count;) {
    const int e = edge_of(P->n_host[order[t]]);
    int64_t u = t;
    while (u < count && edge_of(P->n_host[order[u]]) == e) u++;
    Bucket B;
    B.begin = (int)t;
    B.end = (int)u;
    B.nmax = std::max<int32_t>(P->n_host[order[t]], 1);
    const size_t smem_full = batch_smem_bytes(B.nmax, true, bucket_threads(T, B.nmax, true));
    // Working copies in shared memory up to n = 96 (several CTAs per SM).  Above that a
    // copy takes most of an SM's shared memory, one CTA per SM stalls at every step's
    // barriers, and two CTAs per SM on L2-resident global copies are faster (measured
    // on GB300: 1024 x n = 128 with gradient 12.8 ms against 15.3 ms; the mixed
    // 16..256 workload +1.5 %).  The tuning key batch_smem_nmax moves the limit.
    B.smem_matrix = (smem_full <= 227 * 1024 && B.nmax <= T.batch_smem_nmax) ? 1 : 0;
    B.nt = bucket_threads(T, B.nmax, B.smem_matrix != 0);
    // Consecutive global-memory buckets with the same threads per CTA run as one launch
    // (tuning key batch_merge_global): the CTAs take matrices largest first from one
    // counter, so the smaller sizes fill the tail of the larger ones instead of each
    // bucket ending on a partly empty round of CTAs.  The slots keep the first (largest)
    // size.
    if (T.batch_merge_global && !B.smem_matrix) {
      while (u < count) {
        const int e2 = edge_of(P->n_host[order[u]]);
        int64_t u2 = u;
        while (u2 < count && edge_of(P->n_host[order[u2]]) == e2) u2++;
        const int nm2 = std::max<int32_t>(P->n_host[order[u]], 1);
        const size_t sf2 = batch_smem_bytes(nm2, true, bucket_threads(T, nm2, true));
        const bool sm2 = sf2 <= 227 * 1024 && nm2 <= T.batch_smem_nmax;
        if (sm2 || bucket_threads(T, nm2, false) != B.nt) break;
        u = u2;
      }
      B.end = (int)u;
    }
    int occ = batch_occupancy(B.nmax, B.smem_matrix != 0, B.nt);
    if (!B.smem_matrix) occ = std::max(1, std::min(occ, T.batch_global_ctas_per_sm));
    // Global-memory slices with two CTAs per SM: two regions, the first holding the
    // largest matrices with batch_split_pct % of the work (sum of n^3), see
    // batch_kernel.  Measured on GB300 (4096 matrices, even n in [16, 256]): 71.3 ms
    // per step at 50 % against 73.3 ms with one region, DRAM traffic 20.8 GB against
    // 34.5 GB; taking from the two ends of one region instead cut the traffic to
    // 14.4 GB but ended on mid-size matrices (74.1 ms).
    if (!B.smem_matrix && T.batch_split_pct > 0 && occ >= 2 && u - t >= 2) {
      double total = 0.0, run = 0.0;
      for (int64_t q = t; q < u; q++) total += std::pow((double)P->n_host[order[q]], 3.0);
      const double first = 0.01 * T.batch_split_pct * total;
      int64_t q = t;
      while (q < u - 1 && run + std::pow((double)P->n_host[order[q]], 3.0) <= first) {
        run += std::pow((double)P->n_host[order[q]], 3.0);
        q++;
      }
      B.split = (int)std::max<int64_t>(q, t + 1);
    }
    B.grid = (int)std::min<int64_t>((int64_t)h->sms * occ, u - t);
    B.gws_slot = B.smem_matrix ? 0 : (int64_t)B.nmax * (B.nmax | 1);
    B.gws_off = gws_total;
    gws_total += (size_t)B.gws_slot * B.grid;
    P->buckets.push_back(B);
    t = u;
  }
  P->gws_total = gws_total;
  cudaStream_t st = h->stream;
  bool ok = true;
  ok &= cudaMallocAsync(&P->d_n, sizeof(int32_t) * std::max<int64_t>(count, 1), st) == cudaSuccess;
  ok &= cudaMallocAsync(&P->d_order, sizeof(int32_t) * std::max<int64_t>(count, 1), st) == cudaSuccess;
  ok &= cudaMallocAsync(&P->d_ev_off, sizeof(int64_t) * std::max<int64_t>(count, 1), st) == cudaSuccess;
  ok &= cudaMallocAsync(&P->d_counters, 2 * sizeof(unsigned) * std::max<size_t>(P->buckets.size(), 1), st) ==
        cudaSuccess;
  ok &= cudaMallocAsync(&P->d_ev, sizeof(double) * std::max<int64_t>(P->ev_total, 1), st) == cudaSuccess;
  ok &= cudaMallocAsync(&P->d_fallback, sizeof(unsigned) * (2 + 2 * (size_t)std::max<int64_t>(count, 1)), st) ==
        cudaSuccess;
  if (gws_total) ok &= cudaMallocAsync(&P->d_gws, sizeof(double) * gws_total, st) == cudaSuccess;
  if (ok && count) {
    ok &= cudaMemcpyAsync(P->d_n, P->n_host.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice, st) ==
          cudaSuccess;
    ok &= cudaMemcpyAsync(P->d_order, order.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice, st) ==
          cudaSuccess;
    ok &= cudaMemcpyAsync(P->d_ev_off, ev_off.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st) ==
          cudaSuccess;
    ok &= cudaStreamSynchronize(st) == cudaSuccess;  // host vectors go out of scope
  }
  if (!ok) {
    skew_batch_plan_destroy(P);
    return SKEW_CUDA_ERROR;
  }
  *plan = P;
  return SKEW_OK;
}

int skew_batch_plan_destroy(skew_batch_plan_t P) {
  if (!P) return SKEW_BAD_ARG;
  for (auto& g : P->graphs)
    if (g.valid) cudaGraphExecDestroy(g.exec);
  if (P->capture_stream) cudaStreamDestroy(P->capture_stream);
  cudaStream_t st = P->h ? P->h->stream : nullptr;
  if (P->d_n) cudaFreeAsync(P->d_n, st);
  if (P->d_order) cudaFreeAsync(P->d_order, st);
  if (P->d_ev_off) cudaFreeAsync(P->d_ev_off, st);
  if (P->d_counters) cudaFreeAsync(P->d_counters, st);
  if (P->d_fallback) cudaFreeAsync(P->d_fallback, st);
  if (P->d_ev) cudaFreeAsync(P->d_ev, st);
  if (P->d_gws) cudaFreeAsync(P->d_gws, st);
  void* eig[] = {P->e_refl, P->e_tau, P->e_evb, P->e_G, P->e_log, P->e_work, P->e_vr, P->e_vi, P->e_vals,
                 P->e_off_log, P->e_cap_log, P->e_log_len, P->e_off_w, P->e_p_refl, P->e_p_vr, P->e_p_vi,
                 P->e_p_vals, P->e_p_scratch, P->e_p_work, P->e_status, P->e_fsel, P->e_back_off,
                 P->e_counter};
  for (void* q : eig)
    if (q) cudaFreeAsync(q, st);
  if (P->fv_idx) cudaFreeAsync(P->fv_idx, st);
  if (P->fv_ws) cudaFreeAsync(P->fv_ws, st);
  void* hio[] = {P->hio_off, P->hio_a, P->hio_gh, P->hio_g, P->hio_grad, P->hio_out, P->hio_status};
  for (void* q : hio)
    if (q) cudaFreeAsync(q, st);
  cudaStreamSynchronize(st);
  delete P;
  return SKEW_OK;
}

static int run_buckets(skew_batch_plan_t P, const double* const* A, double* logpf, double* sign,
                       double* const* grad, int* status, bool tridiag_only, double* tau_out = nullptr,
                       double* const* refl_out = nullptr, bool host_in = false,
                       double* const* grad_host = nullptr) {
  cudaStream_t st = P->h->stream;
  CK(cudaMemsetAsync(P->d_counters, 0, 2 * sizeof(unsigned) * std::max<size_t>(P->buckets.size(), 1), st));
  for (size_t i = 0; i < P->buckets.size(); i++) {
    const Bucket& B = P->buckets[i];
    BatchParams bp;
    bp.A = A;
    bp.n = P->d_n;
    bp.order = P->d_order;
    bp.begin = B.begin;
    bp.end = B.end;
    bp.nmax = B.nmax;
    bp.smem_matrix = B.smem_matrix;
    bp.nt = B.nt;
    bp.check = 0;
    bp.gws = P->d_gws ? P->d_gws + B.gws_off : nullptr;
    bp.gws_slot = B.gws_slot;
    bp.counter = P->d_counters + 2 * i;
    bp.split = B.split;
    bp.logpf = logpf;
    bp.sign = sign;
    bp.grad = grad;
    bp.ev_out = tridiag_only ? P->d_ev : nullptr;
    bp.ev_off = P->d_ev_off;
    bp.tau_out = tau_out;
    bp.refl_out = refl_out;
    bp.status = status;
    bp.host_in = host_in ? 1 : 0;
    bp.grad_host = grad_host;
    CK(launch_batch_pf(bp, B.grid, st, tridiag_only));
  }
  return SKEW_OK;
}

}  // extern "C"

// Batched operations run as CUDA graphs: the first call with a given set of
// argument pointers records the plan's launch sequence on a plan-owned stream
// (the legacy default stream cannot be captured) and instantiates it; every
// call then launches the graph on the handle's stream.  Kernels read the
// per-matrix pointer arrays at run time, so new contents behind the same arrays
// need no re-capture.  A stream that the caller is already capturing,
// the tuning key batch_graph = 0, or a capture that fails falls back to plain
// launches of the same kernels on the handle's stream.
enum GraphOp { G_LOGPF = 0, G_EIGVALS, G_EIGEN, G_EXP, G_CIS, G_EXPVJP };

template <class Issue>
static int graph_issue(skew_batch_plan_t P, GraphOp op, const std::array<const void*, 6>& key, Issue&& issue) {
  cudaStream_t user = P->h->stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (P->graphs_off || !P->tune.batch_graph || cudaStreamIsCapturing(user, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone) {
    (void)cudaGetLastError();
    return issue();
  }
  auto& g = P->graphs[op];
  if (g.valid && g.key == key) {
    CK(cudaGraphLaunch(g.exec, user));
    return SKEW_OK;
  }
  if (g.valid) {
    cudaGraphExecDestroy(g.exec);
    g.valid = false;
    g.exec = nullptr;
  }
  if (!P->capture_stream && cudaStreamCreateWithFlags(&P->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    (void)cudaGetLastError();
    P->capture_stream = nullptr;
    P->graphs_off = true;
    return issue();
  }
  if (cudaStreamBeginCapture(P->capture_stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    (void)cudaGetLastError();
    P->graphs_off = true;
    return issue();
  }
  P->h->stream = P->capture_stream;  // issue() launches on the handle's stream
  const int s = issue();
  P->h->stream = user;
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(P->capture_stream, &graph);
  cudaGraphExec_t exec = nullptr;
  const bool ok = s == SKEW_OK && ec == cudaSuccess && graph &&
                  cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  if (!ok) {
    (void)cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    P->graphs_off = true;
    return issue();
  }
  g.valid = true;
  g.exec = exec;
  g.stream = user;
  g.key = key;
  CK(cudaGraphLaunch(exec, user));
  return SKEW_OK;
}

extern "C" {

int skew_batch_logabspf_d(skew_batch_plan_t P, const double* const* A, double* logpf, double* sign,
                          double* const* grad, int* status) {
  if (!P || (P->count > 0 && (!A || !logpf || !sign || !status))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return graph_issue(P, G_LOGPF, {A, logpf, sign, grad, status, nullptr},
                     [&] { return run_buckets(P, A, logpf, sign, grad, status, false); });
}

int skew_batch_eigvals_d(skew_batch_plan_t P, const double* const* A, double* const* vals_im, int* status) {
  if (!P || (P->count > 0 && (!A || !vals_im))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return graph_issue(P, G_EIGVALS, {A, vals_im, status, nullptr, nullptr, nullptr}, [&]() -> int {
    int s = run_buckets(P, A, nullptr, nullptr, nullptr, nullptr, true);
    if (s) return s;
    TrieigParams tp;
    tp.ev_all = P->d_ev;
    tp.ev_off = P->d_ev_off;
    tp.n = P->d_n;
    tp.order = P->d_order;
    tp.count = (int32_t)P->count;
    tp.evwork = P->d_ev;
    tp.vals = vals_im;
    tp.status = status;
    tp.fallback = P->d_fallback;
    tp.grid = (int)std::min<int64_t>(2 * (int64_t)P->h->sms, P->count);
    tp.max_iter = P->h->tune.qr_max_iter;
    CK(launch_batch_trieig(tp, P->h->stream));
    return SKEW_OK;
  });
}

// ---------------------------------------------------------------------------
// Eigenvectors / exp / cis / exp adjoint (skew_eigen.cu)
// ---------------------------------------------------------------------------
namespace {
__global__ void fill_ptrs_kernel(double** dst, double* base, const int64_t* off, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = base + off[i];
}
}  // namespace

// ---------------------------------------------------------------------------
// logabspfaffian + gradient on host buffers.  Each CTA reads its matrix from
// page-locked host memory over the host link and writes its finished gradient
// back the same way, so the transfers of one matrix overlap the compute of the
// others instead of running as whole-batch copies before and after the launch.
// ---------------------------------------------------------------------------

// The device address of a page-locked host buffer [h, h + bytes), or an error
// when any part of it is pageable or the range is not one mapping.
static int host_mapped(const void* h, size_t bytes, void** d) {
  cudaPointerAttributes a0, a1;
  if (cudaPointerGetAttributes(&a0, h) != cudaSuccess ||
      cudaPointerGetAttributes(&a1, (const char*)h + bytes - 1) != cudaSuccess) {
    (void)cudaGetLastError();
    return SKEW_BAD_ARG;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return SKEW_BAD_ARG;
  if ((const char*)a1.devicePointer - (const char*)a0.devicePointer != (ptrdiff_t)(bytes - 1)) return SKEW_BAD_ARG;
  *d = a0.devicePointer;
  return SKEW_OK;
}

static int hio_ws(skew_batch_plan_t P) {
  if (P->hio_off) return SKEW_OK;
  cudaStream_t st = P->h->stream;
  const int64_t count = P->count;
  std::vector<int64_t> off(count);
  int64_t sq = 0;
  for (int64_t b = 0; b < count; b++) {
    off[b] = sq;
    sq += (int64_t)P->n_host[b] * P->n_host[b];
  }
  bool ok = true;
  auto alloc = [&](void** p, size_t bytes) { ok &= cudaMallocAsync(p, std::max<size_t>(bytes, 8), st) == cudaSuccess; };
  alloc((void**)&P->hio_off, sizeof(int64_t) * count);
  alloc((void**)&P->hio_a, sizeof(double*) * count);
  alloc((void**)&P->hio_gh, sizeof(double*) * count);
  alloc((void**)&P->hio_g, sizeof(double*) * count);
  alloc((void**)&P->hio_grad, sizeof(double) * sq);
  alloc((void**)&P->hio_out, sizeof(double) * 2 * count);
  alloc((void**)&P->hio_status, sizeof(int) * count);
  if (!ok) return SKEW_NO_MEMORY;
  CK(cudaMemcpyAsync(P->hio_off, off.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st));
  fill_ptrs_kernel<<<(int)((count + 255) / 256), 256, 0, st>>>(P->hio_g, P->hio_grad, P->hio_off, (int)count);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));  // `off` goes out of scope
  P->hio_total = sq;
  return SKEW_OK;
}

extern "C" int skew_batch_logabspf_host_d(skew_batch_plan_t P, const double* hA, double* hG, double* h_logpf,
                                          double* h_sign, int* h_status) {
  if (!P || (P->count > 0 && (!hA || !h_logpf || !h_sign || !h_status))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  int s = hio_ws(P);
  if (s) return s;
  const int64_t count = P->count;
  cudaStream_t st = P->h->stream;
  const int g = (int)((count + 255) / 256);
  if (P->hio_total > 0) {
    const size_t bytes = sizeof(double) * (size_t)P->hio_total;
    void *dA = nullptr, *dG = nullptr;
    if ((s = host_mapped(hA, bytes, &dA))) return s;
    if (hG && (s = host_mapped(hG, bytes, &dG))) return s;
    fill_ptrs_kernel<<<g, 256, 0, st>>>(P->hio_a, (double*)dA, P->hio_off, (int)count);
    if (dG) fill_ptrs_kernel<<<g, 256, 0, st>>>(P->hio_gh, (double*)dG, P->hio_off, (int)count);
    CK(cudaGetLastError());
    s = run_buckets(P, P->hio_a, P->hio_out, P->hio_out + count, dG ? P->hio_g : nullptr, P->hio_status, false,
                    nullptr, nullptr, true, dG ? P->hio_gh : nullptr);
  } else {  // every matrix is 0 x 0: nothing to read
    s = run_buckets(P, P->hio_g, P->hio_out, P->hio_out + count, nullptr, P->hio_status, false);
  }
  if (s) return s;
  CK(cudaMemcpyAsync(h_logpf, P->hio_out, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h_sign, P->hio_out + count, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h_status, P->hio_status, sizeof(int) * count, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return SKEW_OK;
}

namespace {
__global__ void set8_kernel(double** dst, double* a, double* b, double* c, double* d, double* e, double* f,
                            double* g, double* h) {
  dst[0] = a;
  dst[1] = b;
  dst[2] = c;
  dst[3] = d;
  dst[4] = e;
  dst[5] = f;
  dst[6] = g;
  dst[7] = h;
}
__global__ void copy_status_kernel(const int* src, int* dst) { *dst = *src; }
}  // namespace

static int eigen_ws(skew_batch_plan_t P) {
  if (P->eig_ready) return SKEW_OK;
  cudaStream_t st = P->h->stream;
  const int64_t count = P->count;
  std::vector<int64_t> off_sq(count), off_log(count), cap_log(count), off_w(count);
  int64_t sq = 0, lg = 0, w = 0;
  int nmax = 1;
  for (int64_t b = 0; b < count; b++) {
    const int64_t n = std::max<int32_t>(P->n_host[b], 1);
    nmax = std::max<int>(nmax, (int)n);
    off_sq[b] = sq;
    sq += n * n;
    off_log[b] = lg;
    cap_log[b] = 3 * n * n + 64;
    lg += cap_log[b];
    off_w[b] = w;
    w += (int64_t)eigen_work_doubles((int)n);
  }
  P->nmax = nmax;
  bool ok = true;
  auto alloc = [&](void** p, size_t bytes) { ok &= cudaMallocAsync(p, std::max<size_t>(bytes, 8), st) == cudaSuccess; };
  alloc((void**)&P->e_refl, sizeof(double) * sq);
  alloc((void**)&P->e_tau, sizeof(double) * P->ev_total);
  alloc((void**)&P->e_evb, sizeof(double) * P->ev_total);
  alloc((void**)&P->e_G, sizeof(double) * P->ev_total);
  alloc((void**)&P->e_vals, sizeof(double) * P->ev_total);
  alloc((void**)&P->e_log, sizeof(double) * lg);
  alloc((void**)&P->e_work, sizeof(double) * w);
  alloc((void**)&P->e_vr, sizeof(double) * sq);
  alloc((void**)&P->e_vi, sizeof(double) * sq);
  alloc((void**)&P->e_off_log, sizeof(int64_t) * count);
  alloc((void**)&P->e_cap_log, sizeof(int64_t) * count);
  alloc((void**)&P->e_log_len, sizeof(int64_t) * count);
  alloc((void**)&P->e_off_w, sizeof(int64_t) * count);
  alloc((void**)&P->e_p_refl, sizeof(double*) * count);
  alloc((void**)&P->e_p_vr, sizeof(double*) * count);
  alloc((void**)&P->e_p_vi, sizeof(double*) * count);
  alloc((void**)&P->e_p_vals, sizeof(double*) * count);
  alloc((void**)&P->e_p_scratch, sizeof(double*) * 8);
  alloc((void**)&P->e_p_work, sizeof(double*) * count);
  alloc((void**)&P->e_status, sizeof(int) * count);
  alloc((void**)&P->e_fsel, sizeof(int) * count);
  alloc((void**)&P->e_back_off, sizeof(int32_t) * (count + 1));
  alloc((void**)&P->e_counter, sizeof(unsigned));
  if (!ok) return SKEW_NO_MEMORY;
  int64_t* d_off_sq = nullptr;
  ok &= cudaMallocAsync(&d_off_sq, sizeof(int64_t) * count, st) == cudaSuccess;
  ok &= cudaMemcpyAsync(d_off_sq, off_sq.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st) == cudaSuccess;
  ok &= cudaMemcpyAsync(P->e_off_log, off_log.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st) ==
        cudaSuccess;
  ok &= cudaMemcpyAsync(P->e_cap_log, cap_log.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st) ==
        cudaSuccess;
  ok &= cudaMemcpyAsync(P->e_off_w, off_w.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, st) ==
        cudaSuccess;
  // back-transformation items in the processing order (the plan's largest-first order)
  std::vector<int32_t> ord(count), boff(count + 1, 0);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int32_t a, int32_t c) { return P->n_host[a] > P->n_host[c]; });
  for (int64_t t = 0; t < count; t++) boff[t + 1] = boff[t] + back_items_of(P->n_host[ord[t]]);
  P->back_items = boff[count];
  ok &= cudaMemcpyAsync(P->e_back_off, boff.data(), sizeof(int32_t) * (count + 1), cudaMemcpyHostToDevice, st) ==
        cudaSuccess;
  if (!ok) return SKEW_CUDA_ERROR;
  const int g = (int)((count + 255) / 256);
  fill_ptrs_kernel<<<g, 256, 0, st>>>(P->e_p_refl, P->e_refl, d_off_sq, (int)count);
  fill_ptrs_kernel<<<g, 256, 0, st>>>(P->e_p_vr, P->e_vr, d_off_sq, (int)count);
  fill_ptrs_kernel<<<g, 256, 0, st>>>(P->e_p_vi, P->e_vi, d_off_sq, (int)count);
  fill_ptrs_kernel<<<g, 256, 0, st>>>(P->e_p_vals, P->e_vals, P->d_ev_off, (int)count);
  fill_ptrs_kernel<<<g, 256, 0, st>>>(P->e_p_work, P->e_work, P->e_off_w, (int)count);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(st));  // host vectors go out of scope
  cudaFree(d_off_sq);
  P->eig_ready = true;
  return SKEW_OK;
}

// Reduction, QR with logged rotations, vectors, back-transformation.
// A != null: dense matrices (reduction, QR of skewtrieigen_divided!, vectors,
// back-transformation).  ev_in != null instead: the subdiagonals of
// SkewHermTridiagonal matrices (skewtrieigen_merged!, no reduction, Q = I).
// Above this size (the tuning key func_chain_nmax) the batched function paths take
// bisection and twisted vectors; the eigenvalue order does not matter there.
// The QR chain runs one matrix per thread, O(n^2) with a long dependency chain:
// for n = 512 it takes 0.30 s on GB300, where bisection and twisted vectors take
// a few milliseconds.  Measured on the 512-matrix exp-adjoint workload (n in
// {32, ..., 512}, complex form of the adjoint): 745 ms per step with 64, 768 with
// 160, 813 with 256, 1013 with the chain for every size.
static int func_chain_nmax(skew_batch_plan_t P) { return P->h->tune.func_chain_nmax; }

// Size groups of the matrices above thr, their device index list and the workspace
// of one chunk (problems per chunk bounded so one chunk's workspace stays within
// 64 M doubles).
static int fv_setup(skew_batch_plan_t P, int thr) {
  if (P->fv_thresh == thr) return SKEW_OK;
  cudaStream_t st = P->h->stream;
  // recorded graphs reference the old workspace: drop them (they re-record)
  for (auto& g : P->graphs)
    if (g.valid) {
      CK(cudaGraphExecDestroy(g.exec));
      g.valid = false;
      g.exec = nullptr;
    }
  if (P->fv_idx) CK(cudaFreeAsync(P->fv_idx, st));
  if (P->fv_ws) CK(cudaFreeAsync(P->fv_ws, st));
  P->fv_idx = nullptr;
  P->fv_ws = nullptr;
  P->fv_groups.clear();
  P->fv_ws_doubles = 0;
  std::vector<int32_t> idx;
  std::vector<int32_t> bysize(P->count);
  std::iota(bysize.begin(), bysize.end(), 0);
  std::stable_sort(bysize.begin(), bysize.end(), [&](int32_t a, int32_t b) { return P->n_host[a] > P->n_host[b]; });
  for (size_t t = 0; t < bysize.size();) {
    const int n = P->n_host[bysize[t]];
    size_t u = t;
    while (u < bysize.size() && P->n_host[bysize[u]] == n) u++;
    if (n > thr && n >= 3) {
      skew_batch_plan_st::FvGroup g;
      g.n = n;
      g.start = (int)idx.size();
      g.count = (int)(u - t);
      const size_t per = skew_vectors_batch_ws_doubles(n) + 2 * (size_t)n + 8;
      g.chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)g.count, (64u << 20) / per));
      P->fv_ws_doubles = std::max(P->fv_ws_doubles, per * (size_t)g.chunk);
      for (size_t q = t; q < u; q++) idx.push_back(bysize[q]);
      P->fv_groups.push_back(g);
    }
    t = u;
  }
  if (!idx.empty()) {
    CK(cudaMallocAsync(&P->fv_idx, sizeof(int32_t) * idx.size(), st));
    CK(cudaMemcpyAsync(P->fv_idx, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMallocAsync(&P->fv_ws, sizeof(double) * P->fv_ws_doubles, st));
    CK(cudaStreamSynchronize(st));  // idx goes out of scope
  }
  P->fv_thresh = thr;
  return SKEW_OK;
}

// Bisection and twisted vectors for the groups above the chain threshold.
static int fv_issue(skew_batch_plan_t P, const EigenBatch& E) {
  cudaStream_t st = P->h->stream;
  for (const auto& g : P->fv_groups) {
    for (int c0 = 0; c0 < g.count; c0 += g.chunk) {
      const int G = std::min(g.chunk, g.count - c0);
      const int32_t* ix = P->fv_idx + g.start + c0;
      double* e_g = P->fv_ws;
      double* vals_g = e_g + (size_t)G * g.n;
      double* bp_g = vals_g + (size_t)G * g.n;
      double* ws = bp_g + (size_t)G * 8;
      CK(launch_gather_ev(P->d_ev, P->d_ev_off, ix, g.n, G, e_g, st));
      CK(launch_tridiag_bisect_batch(e_g, g.n, G, bp_g, vals_g, E.vals, ix, st));
      CK(skew_vectors_batch(e_g, g.n, G, vals_g, bp_g, E.Vr, E.Vi, ix, ws, st));
    }
  }
  return SKEW_OK;
}

// back_q: the exp adjoint's path, which needs only the real Schur basis: Q is built in
// the tridiagonal basis before the back-transformation, which then takes Q (n columns)
// instead of Vr and Vi (2n) for the matrices that split into pairs.
static int eigen_run(skew_batch_plan_t P, const double* const* A, double* const* vals, double* const* Vr,
                     double* const* Vi, EigenBatch* Eout, const double* const* ev_in = nullptr,
                     int chain_nmax = 1 << 30, bool back_q = false) {
  int s = eigen_ws(P);
  if (s) return s;
  cudaStream_t st = P->h->stream;
  if (ev_in)
    CK(launch_copy_ev(ev_in, P->d_n, P->d_ev_off, (int)P->count, P->d_ev, st));
  else
    s = run_buckets(P, A, nullptr, nullptr, nullptr, nullptr, true, P->e_tau, P->e_p_refl);
  if (s) return s;
  EigenBatch E;
  E.count = (int32_t)P->count;
  E.nmax = P->nmax;
  E.order = P->d_order;
  E.n = P->d_n;
  E.off_n = P->d_ev_off;
  E.ev = P->d_ev;
  E.evb = P->e_evb;
  E.tau = P->e_tau;
  E.G = P->e_G;
  E.vals = vals ? vals : P->e_p_vals;
  E.log = P->e_log;
  E.off_log = P->e_off_log;
  E.cap_log = P->e_cap_log;
  E.log_len = P->e_log_len;
  E.status = P->e_status;
  E.counter = P->e_counter;
  E.Vr = Vr ? Vr : P->e_p_vr;
  E.Vi = Vi ? Vi : P->e_p_vi;
  E.refl = P->e_p_refl;
  E.work = P->e_work;
  E.off_w = P->e_off_w;
  E.out = nullptr;
  E.cot = nullptr;
  E.pwork = P->e_p_work;
  E.func = SKEW_FUNC_EXP;
  E.merged = ev_in ? 1 : 0;
  E.chain_nmax = (ev_in || chain_nmax >= P->nmax) ? (1 << 30) : chain_nmax;
  E.max_iter = P->h->tune.qr_max_iter;
  const int grid = (int)std::min<int64_t>(2 * (int64_t)P->h->sms, P->count);
  CK(launch_eigen_chain(E, st));
  CK(launch_eigen_vectors(E, grid, st));
  if (E.chain_nmax < P->nmax) {
    s = fv_issue(P, E);
    if (s) return s;
  }
  if (back_q && !ev_in) {
    E.fsel = P->e_fsel;
    E.back_q = 1;
    CK(launch_schur_basis(E, st));
  }
  if (!ev_in) {
    // back-transformation: column chunks of every matrix, so the largest matrices do not
    // leave most of the GPU idle at the end
    E.back_off = P->e_back_off;
    E.back_items = P->back_items;
    const int bgrid = (int)std::max<int64_t>(1, std::min<int64_t>(2 * (int64_t)P->h->sms, P->back_items));
    CK(launch_eigen_back(E, bgrid, P->nmax, st));
  }
  *Eout = E;
  return SKEW_OK;
}

static int finish_status(skew_batch_plan_t P, int* status) {
  if (status)
    CK(cudaMemcpyAsync(status, P->e_status, sizeof(int) * P->count, cudaMemcpyDeviceToDevice, P->h->stream));
  return SKEW_OK;
}

int skew_batch_eigen_d(skew_batch_plan_t P, const double* const* A, double* const* vals_im, double* const* Vr,
                       double* const* Vi, int* status) {
  if (!P || (P->count > 0 && (!A || !vals_im || !Vr || !Vi))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  int s = eigen_ws(P);
  if (s) return s;
  return graph_issue(P, G_EIGEN, {A, vals_im, Vr, Vi, status, nullptr}, [&]() -> int {
    EigenBatch E;
    int s2 = eigen_run(P, A, vals_im, Vr, Vi, &E);
    if (s2) return s2;
    return finish_status(P, status);
  });
}

static int func_issue(skew_batch_plan_t P, const double* const* A, double* const* out, const double* const* cot,
                      int mode, int func, int* status);

// matrix functions / cis / exp adjoint as one graph per mode (batched entry points);
// the function id is part of the key, so another function re-captures
static int func_run_graph(skew_batch_plan_t P, const double* const* A, double* const* out,
                          const double* const* cot, int mode, int func, int* status) {
  int s = eigen_ws(P);
  if (s) return s;
  s = fv_setup(P, func_chain_nmax(P));
  if (s) return s;
  const GraphOp op = mode == 0 ? G_EXP : (mode == 1 ? G_CIS : G_EXPVJP);
  return graph_issue(P, op, {A, out, cot, status, reinterpret_cast<const void*>((intptr_t)func), nullptr},
                     [&] { return func_issue(P, A, out, cot, mode, func, status); });
}

static int func_run(skew_batch_plan_t P, const double* const* A, double* const* out, const double* const* cot,
                    int mode, int func, int* status) {
  return func_issue(P, A, out, cot, mode, func, status);
}

static int func_issue(skew_batch_plan_t P, const double* const* A, double* const* out, const double* const* cot,
                      int mode, int func, int* status) {
  EigenBatch E;
  int s = fv_setup(P, func_chain_nmax(P));
  if (s) return s;
  const bool schur = P->h->tune.func_real_schur != 0;
  s = eigen_run(P, A, nullptr, nullptr, nullptr, &E, nullptr, func_chain_nmax(P), schur);
  if (s) return s;
  E.out = out;
  E.cot = cot;
  E.func = func;
  E.fsel = schur ? P->e_fsel : nullptr;
  CK(launch_eigen_func(E, mode, P->h->stream));
  return finish_status(P, status);
}

int skew_batch_exp_d(skew_batch_plan_t P, const double* const* A, double* const* E, int* status) {
  if (!P || (P->count > 0 && (!A || !E))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return func_run_graph(P, A, E, nullptr, 0, SKEW_FUNC_EXP, status);
}

int skew_batch_func_d(skew_batch_plan_t P, const double* const* A, int func, double* const* F, int* status) {
  if (!P || (P->count > 0 && (!A || !F)) || func < SKEW_FUNC_EXP || func > SKEW_FUNC_LOG) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return func_run_graph(P, A, F, nullptr, 0, func, status);
}

int skew_batch_cis_d(skew_batch_plan_t P, const double* const* A, double* const* C, int* status) {
  if (!P || (P->count > 0 && (!A || !C))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return func_run_graph(P, A, C, nullptr, 1, SKEW_FUNC_EXP, status);
}

int skew_batch_exp_vjp_d(skew_batch_plan_t P, const double* const* A, const double* const* Cbar, double* const* G,
                         int* status) {
  if (!P || (P->count > 0 && (!A || !Cbar || !G))) return SKEW_BAD_ARG;
  if (P->count == 0) return SKEW_OK;
  return func_run_graph(P, A, G, Cbar, 2, SKEW_FUNC_EXP, status);
}

// Single matrices run as a batch of one through a plan cached on the handle.
static int single_plan(skew_handle_t h, int64_t n, skew_batch_plan_t* out) {
  if (h->plan1 && h->plan1_n == n) {
    *out = h->plan1;
    return SKEW_OK;
  }
  if (h->plan1) skew_batch_plan_destroy(h->plan1);
  h->plan1 = nullptr;
  skew_batch_plan_t p = nullptr;
  int s = skew_batch_plan_create(h, &n, 1, &p);
  if (s) return s;
  s = eigen_ws(p);
  if (s) {
    skew_batch_plan_destroy(p);
    return s;
  }
  h->plan1 = p;
  h->plan1_n = n;
  *out = p;
  return SKEW_OK;
}

static int func_large(skew_handle_t h, double* A, const double* ev, int64_t n, double* out, const double* cot,
                      int mode, int func, int* info);

static int single_func(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* Vr, double* Vi,
                       int64_t ldv, double* out, int64_t ldo, const double* cot, int mode, int* info,
                       int func = SKEW_FUNC_EXP) {
  if (!h || n < 1 || !A || lda != n || (ldv && ldv != n) || (ldo && ldo != n)) return n < 1 ? SKEW_BAD_ARG
                                                                                            : SKEW_UNSUPPORTED;
  if (n > kSingleMax) {
    if (mode < 0) return SKEW_UNSUPPORTED;  // eigen of large matrices: eigen_large
    return func_large(h, A, nullptr, n, out, cot, mode, func, info);
  }
  skew_batch_plan_t P = nullptr;
  int s = single_plan(h, n, &P);
  if (s) return s;
  double** arr = P->e_p_scratch;  // [0] A, [1] vals, [2] Vr, [3] Vi, [4] out, [5] cot
  set8_kernel<<<1, 1, 0, h->stream>>>(arr, A, vals_im, Vr, Vi, out, (double*)cot, nullptr, nullptr);
  CK(cudaGetLastError());
  if (mode < 0) {
    EigenBatch E;
    s = eigen_run(P, (const double* const*)arr, arr + 1, arr + 2, arr + 3, &E);
  } else {
    s = func_run(P, (const double* const*)arr, arr + 4, (const double* const*)(arr + 5), mode, func, nullptr);
  }
  if (s) return s;
  if (info) {
    copy_status_kernel<<<1, 1, 0, h->stream>>>(P->e_status, info);
    CK(cudaGetLastError());
  }
  return SKEW_OK;
}

// Large single matrices (n > 1024): blocked reduction, bisection and the
// twisted-factorisation eigenvectors of skew_tdvec.cu (the reference's fallback
// formulation, values sorted descending).
static int eigen_large(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* Vr, double* Vi,
                       int64_t ldv, int* info) {
  if (lda < n || ldv < n || n > (1LL << 15)) return n > (1LL << 15) ? SKEW_UNSUPPORTED : SKEW_BAD_ARG;
  const size_t wsd = blocked_ws_doubles((int)n) + persist_ws_extra_doubles();
  const size_t lwsd = large_eigen_ws_doubles((int)n), auxd = large_eigen_aux_doubles((int)n);
  const size_t extra = 2 * (size_t)n + 8 + lwsd + auxd + 1;
  int st = ensure_ws(h, sizeof(double) * (wsd + extra));
  if (st) return st;
  // [ev (n)][tau (n)][bisection scratch (8)][eigenvector workspace][aux][gate]
  double* base = (double*)h->ws + wsd;
  double* ev = base;
  double* tau = base + n;
  double* bp = base + 2 * n;
  double* lws = base + 2 * n + 8;
  double* aux = lws + lwsd;
  int* gate = (int*)(aux + auxd);
  st = blocked(h, A, n, lda, tau, ev, info, extra, nullptr);
  if (st) return st;
  CK(launch_tridiag_bisect(ev, (int)n, vals_im, bp, h->stream));
  CK(large_eigen_vectors(A, lda, (int)n, tau, ev, vals_im, bp, Vr, Vi, ldv, lws, gate, aux, h->stream));
  return SKEW_OK;
}

// exp, cis, the other matrix functions and the exp adjoint of one large matrix
// (n > 1024): the eigenpairs come from eigen_large (dense A, destroyed) or from
// bisection and twisted vectors of the tridiagonal ev; then the element-wise step
// and the tiled products of the batched path run on them as a batch of one.  The
// eigenvalue order (descending here) does not change these functions.
// Handle aux layout (doubles): [Vr n^2][Vi n^2][work 4 n^2][vals n][8 pointers][n, status].
static int func_large(skew_handle_t h, double* A, const double* ev, int64_t n, double* out, const double* cot,
                      int mode, int func, int* info) {
  if (!h || !out || (mode == 2 && !cot)) return SKEW_BAD_ARG;
  if (n > (1LL << 15)) return SKEW_UNSUPPORTED;
  const size_t nn = (size_t)n * (size_t)n;
  int st = ensure_aux(h, sizeof(double) * (6 * nn + (size_t)n + 8 + 2));
  if (st) return st;
  cudaStream_t s = h->stream;
  double* Vr = (double*)h->aux;
  double* Vi = Vr + nn;
  double* work = Vi + nn;
  double* vals = work + 4 * nn;
  double** ptrs = (double**)(vals + n);  // [0] Vr, [1] Vi, [2] vals, [3] work, [4] out, [5] cot
  int32_t* dn = (int32_t*)(ptrs + 8);
  int* status = (int*)(dn + 1);
  const int32_t n32 = (int32_t)n;
  CK(cudaMemcpyAsync(dn, &n32, sizeof(int32_t), cudaMemcpyHostToDevice, s));  // pageable: staged before return
  CK(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (A) {
    st = eigen_large(h, A, n, n, vals, Vr, Vi, n, status);
  } else {
    st = skew_tridiag_eigen_d(h, ev, n, vals, Vr, Vi, n, status);
  }
  if (st) return st;
  set8_kernel<<<1, 1, 0, s>>>(ptrs, Vr, Vi, vals, work, out, const_cast<double*>(cot), nullptr, nullptr);
  CK(cudaGetLastError());
  EigenBatch E{};
  E.count = 1;
  E.nmax = (int32_t)n;
  E.n = dn;
  E.status = status;
  E.vals = ptrs + 2;
  E.Vr = ptrs;
  E.Vi = ptrs + 1;
  E.pwork = ptrs + 3;
  E.out = ptrs + 4;
  E.cot = (const double* const*)(ptrs + 5);
  E.func = func;
  E.fsel = h->tune.func_real_schur ? status + 1 : nullptr;  // aux tail after status: n, status, fsel
  CK(launch_eigen_func(E, mode, s));
  if (info) {
    copy_status_kernel<<<1, 1, 0, s>>>(status, info);
    CK(cudaGetLastError());
  }
  return SKEW_OK;
}

int skew_eigen_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* Vr, double* Vi,
                 int64_t ldv, int* info) {
  if (!vals_im || !Vr || !Vi) return SKEW_BAD_ARG;
  if (h && n > kSingleMax) return eigen_large(h, A, n, lda, vals_im, Vr, Vi, ldv, info);
  return single_func(h, A, n, lda, vals_im, Vr, Vi, ldv, nullptr, 0, nullptr, -1, info);
}
int skew_exp_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* E, int64_t lde, int* info) {
  if (!E) return SKEW_BAD_ARG;
  return single_func(h, A, n, lda, nullptr, nullptr, nullptr, 0, E, lde, nullptr, 0, info);
}
int skew_func_d(skew_handle_t h, double* A, int64_t n, int64_t lda, int func, double* F, int64_t ldf, int* info) {
  if (!F || func < SKEW_FUNC_EXP || func > SKEW_FUNC_LOG) return SKEW_BAD_ARG;
  return single_func(h, A, n, lda, nullptr, nullptr, nullptr, 0, F, ldf, nullptr, 0, info, func);
}
int skew_cis_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* C, int64_t ldc, int* info) {
  if (!C) return SKEW_BAD_ARG;
  return single_func(h, A, n, lda, nullptr, nullptr, nullptr, 0, C, ldc, nullptr, 1, info);
}
int skew_exp_vjp_d(skew_handle_t h, double* A, int64_t n, int64_t lda, const double* Cbar, double* G, int64_t ldg,
                   int* info) {
  if (!Cbar || !G) return SKEW_BAD_ARG;
  return single_func(h, A, n, lda, nullptr, nullptr, nullptr, 0, G, ldg, Cbar, 2, info);
}

// ---------------------------------------------------------------------------
// ComplexF64 skew-Hermitian matrices (skew_complex.cu)
// ---------------------------------------------------------------------------
// Workspace of the complex calls (B matrices of size n): [reduction ws][working
// copy (batched: 2 B n^2)][ev (B n)][tau (2 B n)][dvim (B n)][vals (B n + 8)]
// [V (2 B n^2, exp / adjoint)][eigen ws][function ws].
struct ZLayout {
  double *zws, *W, *ev, *tau, *dvim, *vals, *V, *ews, *fws;
};

static int zlayout(skew_handle_t h, int64_t n, int64_t B, bool copy, bool vecs, bool func, ZLayout* L) {
  // every segment a multiple of 32 doubles: complex arrays stay 16-byte aligned
  auto seg = [](size_t d) { return (d + 31) & ~(size_t)31; };
  const size_t zr =
      B == 1 ? seg(std::max(zhess_large_ws_doubles((int)n), zhess_persist_ws_doubles((int)n))) : 0;
  const size_t zw = copy ? seg(2 * (size_t)B * n * n) : 0;
  const size_t ze = seg(zeigen_ws_doubles((int)n, (int)B));
  const size_t zf = func ? seg(zfunc_ws_doubles((int)n, (int)B)) : 0;
  const size_t nv = vecs ? seg(2 * (size_t)B * n * n) : 0;
  const size_t sn = seg((size_t)B * n), s2n = seg(2 * (size_t)B * n), sv = seg((size_t)B * n + 8);
  const size_t total = zr + zw + sn + s2n + sn + sv + nv + ze + zf + 64;
  int st = ensure_ws(h, sizeof(double) * total);
  if (st) return st;
  double* p = (double*)h->ws;
  L->zws = p;
  p += zr;
  L->W = copy ? p : nullptr;
  p += zw;
  L->ev = p;
  p += sn;
  L->tau = p;
  p += s2n;
  L->dvim = p;
  p += sn;
  L->vals = p;
  p += sv;
  L->V = vecs ? p : nullptr;
  p += nv;
  L->ews = p;
  p += ze;
  L->fws = func ? p : nullptr;
  return SKEW_OK;
}

// complex reduction in place.  One matrix: one CTA for n <= 128, the persistent
// blocked kernel from the tuning key zpersist_min_n, per-column multi-CTA
// kernels between (and where the persistent kernel cannot run).  B > 1 matrices of
// size n, n^2 apart: one CTA each.
static int64_t zpersist_min_n(skew_handle_t h) { return h->tune.zpersist_min_n; }

static int zreduce(skew_handle_t h, double* A, int64_t n, int64_t lda, int64_t B, double* tau, double* ev,
                   double* dvim, double* zws, int* info = nullptr) {
  if (B > 1 || n <= 128) {
    ZHessParams P;
    P.W = nullptr;
    P.W1 = A;
    P.n1 = (int)n;
    P.ld1 = lda;
    P.stride = lda * n;
    P.n = nullptr;
    P.order = nullptr;
    P.off = nullptr;
    P.count = (int32_t)B;
    P.nmax = (int)n;
    P.counter = nullptr;
    P.tau = tau;
    P.ev = ev;
    P.dvim = dvim;
    CK(launch_zhess_cta(P, (int)B, h->stream));
    return SKEW_OK;
  }
  if (n >= zpersist_min_n(h)) {
    const cudaError_t e = zhess_persistent(A, lda, (int)n, tau, ev, dvim, zws, h->sms, info, h->tune, h->stream);
    if (e == cudaSuccess) return SKEW_OK;
    if (e != cudaErrorNotSupported) return SKEW_CUDA_ERROR;
    cudaGetLastError();
  }
  CK(zhess_large(A, lda, (int)n, tau, ev, dvim, zws, h->stream));
  return SKEW_OK;
}

static int zcheck(skew_handle_t h, const double* A, int64_t n, int64_t lda) {
  if (!h || n < 0 || (n > 0 && (!A || lda < n))) return SKEW_BAD_ARG;
  if (n > (1LL << 15)) return SKEW_UNSUPPORTED;
  return SKEW_OK;
}

int skew_hessenberg_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* tau, double* ev, double* dvim,
                      int* info) {
  int st = zcheck(h, A, n, lda);
  if (st) return st;
  if (n > 1 && (!tau || !ev)) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return SKEW_OK;
  ZLayout L;
  st = zlayout(h, n, 1, false, false, false, &L);
  if (st) return st;
  return zreduce(h, A, n, lda, 1, n > 1 ? tau : L.tau, n > 1 ? ev : L.ev, dvim ? dvim : L.dvim, L.zws, info);
}

int skew_eigvals_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, int* info) {
  int st = zcheck(h, A, n, lda);
  if (st) return st;
  if (n > 0 && !vals_im) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return SKEW_OK;
  ZLayout L;
  st = zlayout(h, n, 1, false, false, false, &L);
  if (st) return st;
  st = zreduce(h, A, n, lda, 1, L.tau, L.ev, L.dvim, L.zws, info);
  if (st) return st;
  CK(zeigen_from_tridiag(A, lda, (int)n, L.tau, L.ev, L.dvim, vals_im, nullptr, 0, L.ews, 1, h->stream));
  return SKEW_OK;
}

int skew_eigen_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* vals_im, double* V, int64_t ldv,
                 int* info) {
  int st = zcheck(h, A, n, lda);
  if (st) return st;
  if (n > 0 && (!vals_im || !V || ldv < n)) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return SKEW_OK;
  ZLayout L;
  st = zlayout(h, n, 1, false, false, false, &L);
  if (st) return st;
  st = zreduce(h, A, n, lda, 1, L.tau, L.ev, L.dvim, L.zws, info);
  if (st) return st;
  CK(zeigen_from_tridiag(A, lda, (int)n, L.tau, L.ev, L.dvim, vals_im, V, ldv, L.ews, 1, h->stream));
  return SKEW_OK;
}

static int zfunc(skew_handle_t h, double* A, int64_t n, int64_t lda, const double* C, double* O, int64_t ldo,
                 int mode, int func, int* info) {
  int st = zcheck(h, A, n, lda);
  if (st) return st;
  if (n > 0 && (!O || ldo < n || (mode == 1 && !C))) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return SKEW_OK;
  ZLayout L;
  st = zlayout(h, n, 1, false, true, true, &L);
  if (st) return st;
  st = zreduce(h, A, n, lda, 1, L.tau, L.ev, L.dvim, L.zws, info);
  if (st) return st;
  CK(zeigen_from_tridiag(A, lda, (int)n, L.tau, L.ev, L.dvim, L.vals, L.V, n, L.ews, 1, h->stream));
  CK(zfunc_from_eigen(mode, func, (int)n, L.vals, L.V, n, C, n, O, ldo, L.fws, 1, info, h->stream));
  return SKEW_OK;
}

int skew_exp_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* E, int64_t lde, int* info) {
  return zfunc(h, A, n, lda, nullptr, E, lde, 0, SKEW_FUNC_EXP, info);
}

int skew_exp_vjp_z(skew_handle_t h, double* A, int64_t n, int64_t lda, const double* Cbar, double* G, int64_t ldg,
                   int* info) {
  return zfunc(h, A, n, lda, Cbar, G, ldg, 1, SKEW_FUNC_EXP, info);
}

// Batched ComplexF64 of one size: count matrices n^2 apart (inputs read only).
static int zbatch(skew_handle_t h, const double* A, int64_t n, int64_t count, double* vals_im, double* V,
                  const double* C, double* O, int mode, int func, int* status) {
  if (!h || n < 0 || count < 0 || (count > 0 && n > 0 && !A)) return SKEW_BAD_ARG;
  if (n > 1024) return SKEW_UNSUPPORTED;
  if (count == 0 || n == 0) return SKEW_OK;
  if (mode < 0 && (!vals_im || !V)) return SKEW_BAD_ARG;
  if (mode >= 0 && (!O || (mode == 1 && !C))) return SKEW_BAD_ARG;
  if (status) CK(cudaMemsetAsync(status, 0, sizeof(int) * count, h->stream));
  ZLayout L;
  int st = zlayout(h, n, count, true, mode >= 0, mode >= 0, &L);
  if (st) return st;
  CK(cudaMemcpyAsync(L.W, A, sizeof(double) * 2 * (size_t)count * n * n, cudaMemcpyDeviceToDevice, h->stream));
  st = zreduce(h, L.W, n, n, count, L.tau, L.ev, L.dvim, L.zws);
  if (st) return st;
  double* vv = mode < 0 ? vals_im : L.vals;
  double* VV = mode < 0 ? V : L.V;
  CK(zeigen_from_tridiag(L.W, n, (int)n, L.tau, L.ev, L.dvim, vv, VV, n, L.ews, (int)count, h->stream));
  if (mode >= 0) CK(zfunc_from_eigen(mode, func, (int)n, vv, VV, n, C, n, O, n, L.fws, (int)count, status, h->stream));
  return SKEW_OK;
}

int skew_batch_eigen_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* vals_im, double* V,
                       int* status) {
  return zbatch(h, A, n, count, vals_im, V, nullptr, nullptr, -1, 0, status);
}

int skew_batch_exp_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* E, int* status) {
  return zbatch(h, A, n, count, nullptr, nullptr, nullptr, E, 0, SKEW_FUNC_EXP, status);
}

int skew_batch_exp_vjp_z(skew_handle_t h, const double* A, int64_t n, int64_t count, const double* Cbar, double* G,
                         int* status) {
  return zbatch(h, A, n, count, nullptr, nullptr, Cbar, G, 1, SKEW_FUNC_EXP, status);
}

int skew_eigvals_interval_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double vl, double vh,
                            double* vals_im, int* count, int* info) {
  int st = zcheck(h, A, n, lda);
  if (st) return st;
  if (n > 0 && (!vals_im || !count)) return SKEW_BAD_ARG;
  if (!(vl < vh)) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return count ? (cudaMemsetAsync(count, 0, sizeof(int), h->stream) == cudaSuccess ? SKEW_OK
                                                                                              : SKEW_CUDA_ERROR)
                           : SKEW_OK;
  ZLayout L;
  st = zlayout(h, n, 1, false, false, false, &L);
  if (st) return st;
  st = zreduce(h, A, n, lda, 1, L.tau, L.ev, L.dvim, L.zws, info);
  if (st) return st;
  double* dg = L.ews;
  double* off = dg + ((n + 31) & ~(int64_t)31);
  double* ph = off + ((n + 31) & ~(int64_t)31);
  double* bnd = ph + 2 * ((n + 31) & ~(int64_t)31);
  CK(zsymtri_prep(L.ev, L.dvim, (int)n, dg, off, ph, bnd, h->stream));
  CK(launch_select(off, dg, (int)n, bnd, 0, 0, 0, 0, vl, vh, vals_im, count, h->stream));
  return SKEW_OK;
}

int skew_func_z(skew_handle_t h, double* A, int64_t n, int64_t lda, int func, double* F, int64_t ldf, int* info) {
  if (func < SKEW_FUNC_EXP || func > SKEW_FUNC_LOG) return SKEW_BAD_ARG;
  return zfunc(h, A, n, lda, nullptr, F, ldf, 0, func, info);
}

int skew_batch_func_z(skew_handle_t h, const double* A, int64_t n, int64_t count, int func, double* F,
                      int* status) {
  if (func < SKEW_FUNC_EXP || func > SKEW_FUNC_LOG) return SKEW_BAD_ARG;
  return zbatch(h, A, n, count, nullptr, nullptr, nullptr, F, 0, func, status);
}

// ---------------------------------------------------------------------------
// Complex skew-symmetric Pfaffian (pfaffian.jl:98-137, :193-233): one CTA per
// matrix up to the tuning key pfz_cta_max, above that one cooperative grid per matrix.
// ---------------------------------------------------------------------------
static int pfz_cta_max(skew_handle_t h) { return h->tune.pfz_cta_max; }

static int pfz_run(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* phase, double* pf,
                   int check, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || lda < n))) return SKEW_BAD_ARG;
  if (n > (1LL << 15)) return SKEW_UNSUPPORTED;
  if (n > pfz_cta_max(h)) {
    int st = ensure_ws(h, sizeof(double) * pfz_grid_ws_doubles((int)n));
    if (st) return st;
    if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
    CK(launch_pfz_grid((zc*)A, lda, (int)n, check, logpf, phase, pf, info, (double*)h->ws, h->sms, h->tune,
                       h->stream));
    return SKEW_OK;
  }
  PfzParams P{};
  P.A = (const zc*)A;
  P.lda = lda;
  P.stride = 0;
  P.n = (int)n;
  P.count = 1;
  P.check = check;
  P.smem_matrix = 1;
  P.logpf = logpf;
  P.phase = phase;
  P.pf = pf;
  P.status = info;
  P.nt = h->tune.pfz_nt;
  CK(launch_pfz_cta(P, 1, h->stream));
  return SKEW_OK;
}

int skew_logabspf_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* logpf, double* phase, int check,
                    int* info) {
  if (!logpf || !phase) return SKEW_BAD_ARG;
  return pfz_run(h, A, n, lda, logpf, phase, nullptr, check, info);
}

int skew_pfaffian_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* pf, int check, int* info) {
  if (!pf) return SKEW_BAD_ARG;
  return pfz_run(h, A, n, lda, nullptr, nullptr, pf, check, info);
}

int skew_batch_logabspf_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* logpf, double* phase,
                          double* pf, int check, int* status) {
  if (!h || n < 0 || count < 0 || (count > 0 && n > 0 && !A)) return SKEW_BAD_ARG;
  if (!logpf && !phase && !pf) return SKEW_BAD_ARG;
  if (n > (1LL << 15) || count > INT32_MAX) return SKEW_UNSUPPORTED;
  if (count == 0) return SKEW_OK;
  const int nn = (int)n;
  const bool even = nn % 2 == 0 && nn > 0;
  const bool sm = !even || pfz_smem_fits(nn);
  if (even && !sm && nn > pfz_cta_max(h) && count < h->sms) {
    // few large matrices: one grid per matrix, on a copy (the input is read only)
    const size_t mat = 2 * (size_t)n * n, gw = pfz_grid_ws_doubles(nn);
    int st = ensure_ws(h, sizeof(double) * (mat + gw));
    if (st) return st;
    double* W = (double*)h->ws;
    if (status) CK(cudaMemsetAsync(status, 0, sizeof(int) * count, h->stream));
    for (int64_t b = 0; b < count; b++) {
      CK(cudaMemcpyAsync(W, A + b * mat, sizeof(double) * mat, cudaMemcpyDefault, h->stream));
      CK(launch_pfz_grid((zc*)W, n, nn, check, logpf ? logpf + b : nullptr, phase ? phase + 2 * b : nullptr,
                         pf ? pf + 2 * b : nullptr, status ? status + b : nullptr, W + mat, h->sms, h->tune,
                         h->stream));
    }
    return SKEW_OK;
  }
  PfzParams P{};
  P.A = (const zc*)A;
  P.lda = n;
  P.stride = n * n;
  P.n = nn;
  P.count = (int)count;
  P.check = check;
  P.smem_matrix = (sm && even) ? 1 : 0;
  P.logpf = logpf;
  P.phase = phase;
  P.pf = pf;
  P.status = status;
  P.nt = h->tune.pfz_nt;
  const int occ = pfz_cta_occupancy(nn, P.smem_matrix != 0, P.nt);
  int64_t grid = std::min<int64_t>(count, (int64_t)h->sms * (P.smem_matrix || !even ? occ : std::min(occ, 2)));
  if (even && !P.smem_matrix) {
    P.slot = n * (n - 1) / 2;
    int st = ensure_ws(h, sizeof(double) * 2 * (size_t)P.slot * grid);
    if (st) return st;
    P.gws = (zc*)h->ws;
  }
  CK(launch_pfz_cta(P, (int)grid, h->stream));
  return SKEW_OK;
}

// The same on host buffers: A (count x n x n ComplexF64, column-major, back to back)
// in page-locked host memory, read by the kernels over the host link; the results
// are copied to the host arrays given (any of logpf, phase, pf, status may be NULL,
// not all of the first three) and the call returns when they are there.
int skew_batch_logabspf_host_z(skew_handle_t h, const double* A, int64_t n, int64_t count, double* logpf,
                               double* phase, double* pf, int check, int* status) {
  if (!h || n < 0 || count < 0 || (count > 0 && n > 0 && !A)) return SKEW_BAD_ARG;
  if (!logpf && !phase && !pf) return SKEW_BAD_ARG;
  if (n > (1LL << 15) || count > INT32_MAX) return SKEW_UNSUPPORTED;
  if (count == 0) return SKEW_OK;
  void* dA = nullptr;
  if (n > 0) {
    const int st = host_mapped(A, sizeof(double) * 2 * (size_t)n * (size_t)n * (size_t)count, &dA);
    if (st) return st;
  }
  int st = ensure_aux(h, sizeof(double) * 5 * (size_t)count + sizeof(int) * (size_t)count);
  if (st) return st;
  double* d_lp = (double*)h->aux;
  double* d_ph = d_lp + count;
  double* d_pf = d_ph + 2 * count;
  int* d_st = (int*)(d_pf + 2 * count);
  st = skew_batch_logabspf_z(h, (const double*)dA, n, count, logpf ? d_lp : nullptr, phase ? d_ph : nullptr,
                             pf ? d_pf : nullptr, check, d_st);
  if (st) return st;
  cudaStream_t s = h->stream;
  if (logpf) CK(cudaMemcpyAsync(logpf, d_lp, sizeof(double) * count, cudaMemcpyDeviceToHost, s));
  if (phase) CK(cudaMemcpyAsync(phase, d_ph, sizeof(double) * 2 * count, cudaMemcpyDeviceToHost, s));
  if (pf) CK(cudaMemcpyAsync(pf, d_pf, sizeof(double) * 2 * count, cudaMemcpyDeviceToHost, s));
  if (status) CK(cudaMemcpyAsync(status, d_st, sizeof(int) * count, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return SKEW_OK;
}

// ---------------------------------------------------------------------------
// svdvals / svd from the eigenpairs (eigen.jl:110-144, tridiag.jl:526-555)
// ---------------------------------------------------------------------------
// aux layout: vals (n doubles), signs (n doubles), perm (n ints)
static int svd_aux(skew_handle_t h, int64_t n, double** vals, double** sgn, int** perm) {
  const size_t nn = (size_t)std::max<int64_t>(n, 1);
  int st = ensure_aux(h, nn * (2 * sizeof(double) + sizeof(int)));
  if (st) return st;
  *vals = (double*)h->aux;
  *sgn = *vals + nn;
  *perm = (int*)(*sgn + nn);
  return SKEW_OK;
}

// S from eigenvalue imaginary parts already in aux
static int svdvals_finish(skew_handle_t h, int64_t n, const double* vals, double* S) {
  CK(launch_svd_rank(vals, (int)n, n, 1, nullptr, S, n, nullptr, h->stream));
  return SKEW_OK;
}

int skew_svdvals_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !S || lda < n))) return SKEW_BAD_ARG;
  if (n == 0) return info ? (cudaMemsetAsync(info, 0, sizeof(int), h->stream) == cudaSuccess ? SKEW_OK
                                                                                          : SKEW_CUDA_ERROR)
                          : SKEW_OK;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = eigvals_bisect_d(h, A, n, lda, vals, info);
  if (st) return st;
  return svdvals_finish(h, n, vals, S);
}

int skew_svd_d(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, double* Ur, double* Ui, double* Vr,
               double* Vi, int64_t ldu, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !S || !Ur || !Ui || !Vr || !Vi || lda < n || ldu < n))) return SKEW_BAD_ARG;
  if (n == 0) return info ? (cudaMemsetAsync(info, 0, sizeof(int), h->stream) == cudaSuccess ? SKEW_OK
                                                                                          : SKEW_CUDA_ERROR)
                          : SKEW_OK;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_eigen_d(h, A, n, lda, vals, Vr, Vi, ldu, info);  // eigenvectors W in the V planes
  if (st) return st;
  CK(launch_svd_rank(vals, (int)n, n, 1, perm, S, n, sgn, h->stream));
  CK(launch_svd_vectors_d(Vr, Vi, (int)n, ldu, perm, sgn, Ur, Ui, Vr, Vi, h->stream));
  return SKEW_OK;
}

int skew_svdvals_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !S || lda < n))) return SKEW_BAD_ARG;
  if (n == 0) return info ? (cudaMemsetAsync(info, 0, sizeof(int), h->stream) == cudaSuccess ? SKEW_OK
                                                                                          : SKEW_CUDA_ERROR)
                          : SKEW_OK;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_eigvals_z(h, A, n, lda, vals, info);
  if (st) return st;
  return svdvals_finish(h, n, vals, S);
}

int skew_svd_z(skew_handle_t h, double* A, int64_t n, int64_t lda, double* S, double* U, double* V, int64_t ldu,
               int* info) {
  if (!h || n < 0 || (n > 0 && (!A || !S || !U || !V || lda < n || ldu < n))) return SKEW_BAD_ARG;
  if (n == 0) return info ? (cudaMemsetAsync(info, 0, sizeof(int), h->stream) == cudaSuccess ? SKEW_OK
                                                                                          : SKEW_CUDA_ERROR)
                          : SKEW_OK;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_eigen_z(h, A, n, lda, vals, V, ldu, info);
  if (st) return st;
  CK(launch_svd_rank(vals, (int)n, n, 1, perm, S, n, sgn, h->stream));
  CK(launch_svd_vectors_z(V, (int)n, ldu, perm, sgn, U, V, h->stream));
  return SKEW_OK;
}

// ---------------------------------------------------------------------------
// SkewHermTridiagonal entry points (tridiag.jl): no reduction, Q = I
// ---------------------------------------------------------------------------
int skew_tridiag_eigvals_d(skew_handle_t h, const double* ev, int64_t n, double* vals_im, int* info) {
  if (!h || n < 0 || (n > 1 && !ev) || (n > 0 && !vals_im)) return SKEW_BAD_ARG;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  if (n == 0) return SKEW_OK;
  if (n > kSingleMax) {  // bisection, values sorted descending
    int st = ensure_ws(h, sizeof(double) * 8);
    if (st) return st;
    CK(launch_tridiag_bisect(ev, (int)n, vals_im, (double*)h->ws, h->stream));
    return SKEW_OK;
  }
  // skewtrieigvals! (tridiag.jl:446-450): the QR in the reference's order, batch of one
  return tridiag_qr_vals(h, ev, n, vals_im, info);
}

// skewtrieigvals! on one subdiagonal ev (device, n-1 entries, read only) through the
// handle's batch-of-one plan: vals_im in the reference's order, status <- SKEW_OK,
// SKEW_FALLBACK_USED or SKEW_NO_CONVERGENCE (status may be NULL).  2 <= n <= 1024.
static int tridiag_qr_vals(skew_handle_t h, const double* ev, int64_t n, double* vals_im, int* status) {
  skew_batch_plan_t P = nullptr;
  int st = single_plan(h, n, &P);
  if (st) return st;
  double** arr = P->e_p_scratch;
  set8_kernel<<<1, 1, 0, h->stream>>>(arr, const_cast<double*>(ev), vals_im, nullptr, nullptr, nullptr, nullptr,
                                      nullptr, nullptr);
  CK(cudaGetLastError());
  CK(launch_copy_ev((const double* const*)arr, P->d_n, P->d_ev_off, 1, P->d_ev, h->stream));
  TrieigParams tp;
  tp.ev_all = P->d_ev;
  tp.ev_off = P->d_ev_off;
  tp.n = P->d_n;
  tp.order = P->d_order;
  tp.count = 1;
  tp.evwork = P->d_ev;
  tp.vals = arr + 1;
  tp.status = status;
  tp.fallback = P->d_fallback;
  tp.grid = 1;
  tp.max_iter = h->tune.qr_max_iter;
  CK(launch_batch_trieig(tp, h->stream));
  return SKEW_OK;
}

int skew_tridiag_eigen_d(skew_handle_t h, const double* ev, int64_t n, double* vals_im, double* Vr, double* Vi,
                         int64_t ldv, int* info) {
  if (!h || n < 1 || (n > 1 && !ev) || !vals_im || !Vr || !Vi || ldv < n) return SKEW_BAD_ARG;
  if (n > kSingleMax) {  // bisection + twisted vectors, Q = I (values sorted descending)
    if (n > (1LL << 15)) return SKEW_UNSUPPORTED;
    const size_t lwsd = large_eigen_ws_doubles((int)n), auxd = large_eigen_aux_doubles((int)n);
    int st = ensure_ws(h, sizeof(double) * (8 + lwsd + auxd + 1));
    if (st) return st;
    double* bp = (double*)h->ws;  // [bisection scratch (8)][eigenvector workspace][aux][gate]
    double* aux = bp + 8 + lwsd;
    if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
    CK(launch_tridiag_bisect(ev, (int)n, vals_im, bp, h->stream));
    CK(large_eigen_vectors(nullptr, 0, (int)n, nullptr, ev, vals_im, bp, Vr, Vi, ldv, bp + 8, (int*)(aux + auxd),
                           aux, h->stream));
    return SKEW_OK;
  }
  if (ldv != n) return SKEW_UNSUPPORTED;
  // skewtrieigen_merged! (tridiag.jl:506), batch of one
  skew_batch_plan_t P = nullptr;
  int st = single_plan(h, n, &P);
  if (st) return st;
  double** arr = P->e_p_scratch;  // [0] ev, [1] vals, [2] Vr, [3] Vi
  set8_kernel<<<1, 1, 0, h->stream>>>(arr, const_cast<double*>(ev), vals_im, Vr, Vi, nullptr, nullptr, nullptr,
                                      nullptr);
  CK(cudaGetLastError());
  EigenBatch E;
  st = eigen_run(P, nullptr, arr + 1, arr + 2, arr + 3, &E, (const double* const*)arr);
  if (st) return st;
  if (info) {
    copy_status_kernel<<<1, 1, 0, h->stream>>>(P->e_status, info);
    CK(cudaGetLastError());
  }
  return SKEW_OK;
}

int skew_tridiag_func_d(skew_handle_t h, const double* ev, int64_t n, int func, double* F, int64_t ldf, int* info) {
  if (!h || n < 1 || (n > 1 && !ev) || !F || ldf != n || func < SKEW_FUNC_EXP || func > SKEW_FUNC_LOG)
    return SKEW_BAD_ARG;
  if (n > kSingleMax) return func_large(h, nullptr, ev, n, F, nullptr, 0, func, info);
  skew_batch_plan_t P = nullptr;
  int st = single_plan(h, n, &P);
  if (st) return st;
  double** arr = P->e_p_scratch;  // [0] ev, [4] out
  set8_kernel<<<1, 1, 0, h->stream>>>(arr, const_cast<double*>(ev), nullptr, nullptr, nullptr, F, nullptr, nullptr,
                                      nullptr);
  CK(cudaGetLastError());
  EigenBatch E;
  st = eigen_run(P, nullptr, nullptr, nullptr, nullptr, &E, (const double* const*)arr);
  if (st) return st;
  E.out = arr + 4;
  E.cot = nullptr;
  E.func = func;
  CK(launch_eigen_func(E, 0, h->stream));
  if (info) {
    copy_status_kernel<<<1, 1, 0, h->stream>>>(P->e_status, info);
    CK(cudaGetLastError());
  }
  return SKEW_OK;
}

int skew_tridiag_eigen_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* vals_im,
                         double* V, int64_t ldv, int* info) {
  if (!h || n < 1 || (n > 1 && !ev) || !vals_im || (V && ldv < n)) return SKEW_BAD_ARG;
  if (n > (1LL << 15)) return SKEW_UNSUPPORTED;
  int st = ensure_ws(h, sizeof(double) * (zeigen_ws_doubles((int)n, 1) + 64));
  if (st) return st;
  if (info) CK(cudaMemsetAsync(info, 0, sizeof(int), h->stream));
  CK(zeigen_tridiag(ev, dvim, (int)n, vals_im, V, ldv, (double*)h->ws, h->stream));
  return SKEW_OK;
}

int skew_tridiag_eigvals_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* vals_im,
                           int* info) {
  return skew_tridiag_eigen_z(h, ev, dvim, n, vals_im, nullptr, 0, info);
}

// svdvals! / svd! of a SkewHermTridiagonal (tridiag.jl:526-555): the same sort on its eigenpairs
int skew_tridiag_svdvals_d(skew_handle_t h, const double* ev, int64_t n, double* S, int* info) {
  if (!h || n < 1 || !S) return SKEW_BAD_ARG;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_tridiag_eigvals_d(h, ev, n, vals, info);
  if (st) return st;
  return svdvals_finish(h, n, vals, S);
}

int skew_tridiag_svd_d(skew_handle_t h, const double* ev, int64_t n, double* S, double* Ur, double* Ui, double* Vr,
                       double* Vi, int64_t ldu, int* info) {
  if (!h || n < 1 || !S || !Ur || !Ui || !Vr || !Vi || ldu < n) return SKEW_BAD_ARG;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_tridiag_eigen_d(h, ev, n, vals, Vr, Vi, ldu, info);
  if (st) return st;
  CK(launch_svd_rank(vals, (int)n, n, 1, perm, S, n, sgn, h->stream));
  CK(launch_svd_vectors_d(Vr, Vi, (int)n, ldu, perm, sgn, Ur, Ui, Vr, Vi, h->stream));
  return SKEW_OK;
}

int skew_tridiag_svdvals_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* S, int* info) {
  if (!h || n < 1 || !S) return SKEW_BAD_ARG;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_tridiag_eigvals_z(h, ev, dvim, n, vals, info);
  if (st) return st;
  return svdvals_finish(h, n, vals, S);
}

int skew_tridiag_svd_z(skew_handle_t h, const double* ev, const double* dvim, int64_t n, double* S, double* U,
                       double* V, int64_t ldu, int* info) {
  if (!h || n < 1 || !S || !U || !V || ldu < n) return SKEW_BAD_ARG;
  double *vals, *sgn;
  int* perm;
  int st = svd_aux(h, n, &vals, &sgn, &perm);
  if (st) return st;
  st = skew_tridiag_eigen_z(h, ev, dvim, n, vals, V, ldu, info);
  if (st) return st;
  CK(launch_svd_rank(vals, (int)n, n, 1, perm, S, n, sgn, h->stream));
  CK(launch_svd_vectors_z(V, (int)n, ldu, perm, sgn, U, V, h->stream));
  return SKEW_OK;
}

// ---------------------------------------------------------------------------
// FP64 peak probe
// ---------------------------------------------------------------------------
int skew_measure_fp64_peak(skew_handle_t h, double* tflops) {
  if (!h || !tflops) return SKEW_BAD_ARG;
  const int blocks = h->sms * 4, iters = 4096;
  int st = ensure_ws(h, sizeof(double) * (size_t)blocks * 128);
  if (st) return st;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(launch_dfma_probe((double*)h->ws, blocks, iters, h->stream));  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    CK(cudaEventRecord(e0, h->stream));
    CK(launch_dfma_probe((double*)h->ws, blocks, iters, h->stream));
    CK(cudaEventRecord(e1, h->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * 128.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SKEW_OK;
}

}  // extern "C"

namespace skew {
// Eight independent FMA chains per thread keep the FP64 pipe of every
// sub-partition busy; the result is stored so nothing is optimised away.
__global__ void dfma_probe_kernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
cudaError_t launch_dfma_probe(double* out, int blocks, int iters, cudaStream_t st) {
  dfma_probe_kernel<<<blocks, 128, 0, st>>>(out, iters, 1.0000001, 1e-9);
  return cudaGetLastError();
}

// The FP64 tensor instruction (mma.sync f64) against DFMA, alone and mixed in one
// kernel.  mode 0: DFMA (eight chains per thread); 1: mma m8n8k4 (four
// accumulators per warp); 2: mma m16n8k16 (two); 3: even warps DFMA, odd warps
// m8n8k4; 4: even warps DFMA, odd warps m16n8k16.  it_f / it_m are the iterations
// of the DFMA and mma loops (chosen so both halves of a mixed launch do the same flops).
__global__ void fp64_pipe_probe_kernel(double* out, int it_f, int it_m, int mode, double a, double b) {
  const int warp = threadIdx.x >> 5;
  double x[8];
#pragma unroll
  for (int q = 0; q < 8; q++) x[q] = threadIdx.x * 1e-3 + q;
  const bool mma = mode == 1 || mode == 2 || (mode >= 3 && (warp & 1));
  if (!mma) {
    for (int it = 0; it < it_f; it++) {
#pragma unroll
      for (int q = 0; q < 8; q++) x[q] = fma(x[q], a, b);
    }
  } else if (mode == 1 || mode == 3) {
    for (int it = 0; it < it_m; it++) {
#pragma unroll
      for (int q = 0; q < 4; q++)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(x[2 * q]), "+d"(x[2 * q + 1])
                     : "d"(a), "d"(b));
    }
  } else {
    for (int it = 0; it < it_m; it++) {
#pragma unroll
      for (int q = 0; q < 2; q++)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%4,%4,%4,%4,%4,%4,%4}, "
            "{%5,%5,%5,%5}, {%0,%1,%2,%3};"
            : "+d"(x[4 * q]), "+d"(x[4 * q + 1]), "+d"(x[4 * q + 2]), "+d"(x[4 * q + 3])
            : "d"(a), "d"(b));
    }
  }
  double s = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace skew

extern "C" int skew_measure_fp64_pipes(skew_handle_t h, double* tflops) {
  if (!h || !tflops) return SKEW_BAD_ARG;
  const int blocks = h->sms * 4, nt = 128, it_f = 4096;
  int st = ensure_ws(h, sizeof(double) * (size_t)blocks * nt);
  if (st) return st;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  // flops per warp and iteration: DFMA 8 x 32 x 2 = 512, m8n8k4 4 x 512 = 2048,
  // m16n8k16 2 x 4096 = 8192; the mma loops run it_f / 4 and it_f / 16 iterations
  const double warps = (double)blocks * nt / 32, fl_f = 512.0 * it_f;
  const int it_m[5] = {0, it_f / 4, it_f / 16, it_f / 4, it_f / 16};
  for (int mode = 0; mode < 5; mode++) {
    float best = 1e30f;
    for (int r = 0; r < 6; r++) {  // the first launch warms up
      CK(cudaEventRecord(e0, h->stream));
      fp64_pipe_probe_kernel<<<blocks, nt, 0, h->stream>>>((double*)h->ws, it_f, it_m[mode], mode, 1.0000001, 1e-9);
      CK(cudaGetLastError());
      CK(cudaEventRecord(e1, h->stream));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (r) best = std::min(best, ms);
    }
    tflops[mode] = warps * fl_f / (best * 1e-3) / 1e12;  // every warp does fl_f flops
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return SKEW_OK;
}
