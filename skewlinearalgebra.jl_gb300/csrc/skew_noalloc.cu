// eigvals for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host that owns every
// device byte through its own pool and forbids foreign allocations (CUDA.jl's
// allocator, an inference server running under a fixed memory cap), or code on
// a path where an allocation's implicit synchronisation or possible failure is
// not acceptable.  skew_eigvals_d needs n+1 doubles of device scratch (the
// tridiagonal's subdiagonal and two bisection bounds) from the handle's
// workspace; this entry point keeps that scratch in a fixed array compiled
// into the library instead, so it allocates nothing.
//
// Limits and behaviour:
//   * n <= SKEW_NOALLOC_EIGVALS_NMAX (1024, the one-CTA reduction's limit);
//     larger n returns SKEW_UNSUPPORTED before anything is launched.
//   * The array (1026 doubles, about 8 KB) lives on every GPU that loads the
//     library until the process exits.
//   * The device address of the array is looked up with cudaGetSymbolAddress
//     on the first call made on each device (with that device current); make
//     that first call before any stream capture.  The address is kept per
//     device and per CUDA context: after a device reset (a new primary
//     context), the next call looks it up again.
//   * All calls share the one array.  Each call writes every entry it reads
//     before reading it, so nothing has to start at zero, but calls that
//     overlap on the GPU (different streams, or threads) race on it and give
//     wrong results: serialise them.
//   * Values come out sorted descending (bisection on the tridiagonal form),
//     the order of the reference's own fallback and of eigvals(A, 1:n); they
//     are the eigenvalues skew_eigvals_d returns in the QR's order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/skewgpu.h"
#include "skew_internal.h"

#define SKEW_NOALLOC_EIGVALS_NMAX 1024

namespace {

static __device__ __align__(256) double g_eigvals_scratch[SKEW_NOALLOC_EIGVALS_NMAX + 2];

constexpr int kMaxDevices = 64;

// Cached device address of g_eigvals_scratch per device, with the id of the CUDA
// context it belongs to (a device reset destroys the context and the module with it).
struct ScratchSlot {
  double* addr = nullptr;
  unsigned long long ctx = 0;
};
ScratchSlot g_slot[kMaxDevices];
std::mutex g_slot_mu;

// Id of the calling thread's current CUDA context (unique for the process's
// lifetime), or 0 if there is none; through the CUDA driver-API entry points that
// the runtime hands out, so the library does not link libcuda itself.
unsigned long long current_context_id() {
  typedef int (*GetCurrentFn)(void**);
  typedef int (*GetIdFn)(void*, unsigned long long*);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetIdFn)f;
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of g_eigvals_scratch on the current device and context.
int scratch_address(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return SKEW_CUDA_ERROR;
  if (dev < 0 || dev >= kMaxDevices) return SKEW_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_slot_mu);
  ScratchSlot& slot = g_slot[dev];
  const unsigned long long ctx = current_context_id();
  if (!slot.addr || ctx == 0 || ctx != slot.ctx) {
    double* p = nullptr;
    // also makes the device's primary context current if no context is yet
    if (cudaGetSymbolAddress((void**)&p, g_eigvals_scratch) != cudaSuccess || !p) return SKEW_CUDA_ERROR;
    slot.addr = p;
    slot.ctx = current_context_id();
  }
  *out = slot.addr;
  return SKEW_OK;
}

}  // namespace

extern "C" SKEW_API int skew_eigvals_noalloc_d(double* A, int64_t n, int64_t lda, double* vals_im, int* info,
                                               skew_stream_t stream) {
  if (n < 0 || (n > 0 && (!A || !vals_im || lda < n))) return SKEW_BAD_ARG;
  if (n > SKEW_NOALLOC_EIGVALS_NMAX) return SKEW_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  if (n == 0) return SKEW_OK;
  if (n == 1) {  // skeweigvals! returns [A[1,1]] for n == 1 (eigen.jl:51)
    if (cudaMemcpyAsync(vals_im, A, sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return SKEW_CUDA_ERROR;
    if (info && cudaMemsetAsync(info, 0, sizeof(int), st) != cudaSuccess) return SKEW_CUDA_ERROR;
    return SKEW_OK;
  }
  double* scratch = nullptr;
  const int s = scratch_address(&scratch);
  if (s != SKEW_OK) return s;
  skew::SingleParams P;
  P.A = A;
  P.lda = lda;
  P.n = (int)n;
  P.G = nullptr;
  P.ldg = 0;
  P.logpf = nullptr;
  P.sign = nullptr;
  P.ev = scratch;  // subdiagonal of the tridiagonal form: n-1 doubles
  P.tau = nullptr;
  P.info = info;
  P.check = 0;
  P.want_pf = 0;
  if (skew::launch_single(P, st) != cudaSuccess) return SKEW_CUDA_ERROR;
  // bisection bounds in the two doubles after the subdiagonal
  if (skew::launch_tridiag_bisect(scratch, (int)n, vals_im, scratch + n, st) != cudaSuccess) return SKEW_CUDA_ERROR;
  return SKEW_OK;
}
