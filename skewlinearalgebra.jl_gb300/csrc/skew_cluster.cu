// Householder tridiagonalisation of one moderate-size real skew matrix
// (skewhess!, hessenberg.jl:70-90, with the reflectors of householder!,
// :26-44) inside one thread-block cluster of 16 CTAs.
//
// The whole matrix lives in the cluster's distributed shared memory: CTA r
// holds the columns j = r, r + 16, r + 32, ... in full (all n rows), so n <=
// 640 fits (16 x 227 KB).  Dealing the columns cyclically keeps every CTA
// busy as the trailing block shrinks.  Step k (reflector v_k on rows k+1..n-1)
// is the unblocked two-sided update of the batched kernel, spread over the
// cluster:
//   a. every CTA forms the partial row products of its own columns,
//      P_r[i] = sum_{own j > k} W[i,j] v_j, and stores each into the shared memory
//      of the CTA that owns row i's slice (the m active rows cut into 16 slices);
//   b. cluster barrier;
//   c. each CTA sums the 16 partials of its slice by a fixed pairwise tree,
//      p_i = tau_k sum_r P_r[i], and stores p_i into every CTA; cluster barrier.
//      Every row is summed once, so all CTAs hold the same p bit for bit, and each
//      CTA moves 2 m values instead of reading 16 m;
//   d. the CTA owning column k+1 updates that column with warp 0 and builds
//      reflector k+1 from it (look-ahead), while every other warp of the
//      cluster applies W += v p^T - p v^T to its own columns j > k+1;
//   e. cluster barrier; every CTA copies v_{k+1} and tau_{k+1} from the owner.
// The hardware cluster barrier replaces the two grid barriers per column of the
// persistent multi-CTA reduction, whose L2 round trips bound it at 15-20 us per
// column on this size.
//
// Skew-symmetry is kept exactly although the two triangles live in different
// CTAs: an element below the diagonal takes fma(v_i, p_j, fma(-p_i, v_j, a)),
// one above it fma(-v_j, p_i, fma(p_j, v_i, a)), which is the exact negation of
// its partner's value (round-to-nearest is symmetric under negation).  The
// diagonal stays zero.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "skew_common.cuh"
#include "skew_internal.h"

namespace cg = cooperative_groups;

namespace skew {

constexpr int CL = 16;       // CTAs per cluster
constexpr int CL_NT = 512;   // threads per CTA
constexpr int CL_NW = CL_NT / 32;

struct ClusterParams {
  double* A;
  int64_t lda;
  int n;
  double* tau;
  double* ev;
  int* info;
};

// rows per slice of the partial-product exchange (the m <= n - 1 active rows in CL slices)
__host__ __device__ inline int cluster_slice_max(int n) { return (n + CL - 1) / CL; }

// shared memory of one CTA, in doubles: own columns, then the vectors and the
// receive buffer of the partial row products (CL x slice)
__host__ __device__ inline size_t cluster_smem_doubles(int n) {
  const int nq = (n + CL - 1) / CL;
  return (size_t)nq * n + 3 * (size_t)n + (size_t)CL * cluster_slice_max(n) + CL_NT + 64 + 8;
}

// The reflector of a column held by this CTA (col: its n entries), computed by
// one warp: alpha = col[c+1], x = col[c+2:n].  Writes v (v[c+1] = 1) into the
// column and into vout, beta and tau into ev[c] and tau[c] (global) and tau into
// *tau_out.  householder! (hessenberg.jl:26-44) via make_reflector.  part is this
// lane's share of |x|^2 (the lanes together covering rows c+2..n-1 once), or
// negative to have it formed here.
__device__ void cluster_reflector_warp(double* col, int n, int c, double* vout, double* tau_out, double* ev,
                                       double* tau, double part = -1.0) {
  const int lane = threadIdx.x & 31;
  if (part < 0.0) {
    part = 0.0;
    for (int r = c + 2 + lane; r < n; r += 32) part = fma(col[r], col[r], part);
  }
  const double ss = warp_sum(part);
  double xn = -1.0;
  if (ss_needs_scaling(ss)) {  // warp-uniform rare path: the norm with scaling
    double mx = 0.0;
    for (int r = c + 2 + lane; r < n; r += 32) mx = fmax(mx, fabs(col[r]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    double q = 0.0;
    if (mx > 0.0)
      for (int r = c + 2 + lane; r < n; r += 32) {
        const double x = col[r] / mx;
        q = fma(x, x, q);
      }
    xn = mx * sqrt(warp_sum(q));
  }
  const Reflector R = make_reflector(col[c + 1], ss, xn);
  if (lane == 0) {
    ev[c] = R.beta;
    tau[c] = R.tau;
    *tau_out = R.tau;
  }
  for (int r = c + 1 + lane; r < n; r += 32) {
    const double vr = (R.tau == 0.0) ? 0.0 : (r == c + 1 ? 1.0 : col[r] * R.scale);
    vout[r] = vr;
    col[r] = vr;
  }
}

__global__ void __launch_bounds__(CL_NT, 1) cluster_hess_kernel(ClusterParams P) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int n = P.n, nq = (n + CL - 1) / CL;
  const int tid = threadIdx.x, w = tid >> 5;
  extern __shared__ __align__(16) double sm[];
  double* Wl = sm;                     // own column q (global j = rank + CL q) at Wl + q n
  double* v = Wl + (size_t)nq * n;     // current reflector v_k
  double* p = v + n;                   // tau_k W v_k
  double* vnext = p + n;               // reflector built here (owner of its column)
  const int smax = cluster_slice_max(n);
  double* Pin = vnext + n;             // [CL][smax] partial row products of this CTA's slice
  double* part = Pin + (size_t)CL * smax;  // [CL_NT] split-column partials
  double* scal = part + CL_NT + 64;    // [0] tau_k, [1] tau of the reflector built here
  const int ncl = (n - rank + CL - 1) / CL;  // own columns

  for (int64_t e = tid; e < (int64_t)ncl * n; e += CL_NT) {
    const int q = (int)(e / n), i = (int)(e - (int64_t)q * n);
    Wl[e] = P.A[i + (int64_t)(rank + CL * q) * P.lda];
  }
  for (int i = tid; i < n; i += CL_NT) v[i] = 0.0;
  __syncthreads();
  // reflector 0 from column 0 (rank 0, warp 0)
  if (rank == 0 && w == 0) cluster_reflector_warp(Wl, n, 0, vnext, scal + 1, P.ev, P.tau);
  cl.sync();
  {
    const double* src = cl.map_shared_rank(vnext, 0);
    for (int i = 1 + tid; i < n; i += CL_NT) v[i] = src[i];
    if (tid == 0) scal[0] = *cl.map_shared_rank(scal + 1, 0);
  }
  __syncthreads();

  for (int k = 0; k + 2 < n; k++) {
    const double tauk = scal[0];
    const int m = n - (k + 1);  // active rows k+1 .. n-1
    const int L = (m + CL - 1) / CL;  // rows per slice: slice s holds rows k+1+sL ..
    // partial of active row i (offset t = i - k - 1) into its slice owner's buffer
    auto put_partial = [&](int t, double val) {
      const int s = t / L;
      cl.map_shared_rank(Pin, s)[rank * smax + (t - s * L)] = val;
    };
    // first own column >= k+1 and >= k+2
    const int qa = (k + 1 > rank) ? (k + 1 - rank + CL - 1) / CL : 0;
    const int qb = (k + 2 > rank) ? (k + 2 - rank + CL - 1) / CL : 0;
    // a. partial row products over own columns j >= k+1; with few rows the
    //    columns are split between thread groups and combined through `part`
    {
      const int rows_pp = min(CL_NT, (m + 31) & ~31);
      const int cs = CL_NT / rows_pp;
      const int ri = tid % rows_pp, c = tid / rows_pp;
      for (int i0 = 0; i0 < m; i0 += rows_pp) {
        const int i = k + 1 + i0 + ri;
        if (c < cs && i < n) {
          double a0 = 0.0, a1 = 0.0;
          int q = qa + c;
          for (; q + cs < ncl; q += 2 * cs) {
            a0 = fma(Wl[(size_t)q * n + i], v[rank + CL * q], a0);
            a1 = fma(Wl[(size_t)(q + cs) * n + i], v[rank + CL * (q + cs)], a1);
          }
          if (q < ncl) a0 = fma(Wl[(size_t)q * n + i], v[rank + CL * q], a0);
          if (cs == 1)
            put_partial(i - k - 1, (tauk != 0.0) ? a0 + a1 : 0.0);
          else
            part[c * rows_pp + ri] = a0 + a1;
        }
      }
      if (cs > 1) {  // then m <= rows_pp: one pass
        __syncthreads();
        for (int i = k + 1 + tid; i < n; i += CL_NT) {
          double s = 0.0;
          for (int cc = 0; cc < cs; cc++) s += part[cc * rows_pp + (i - k - 1)];
          put_partial(i - k - 1, (tauk != 0.0) ? s : 0.0);
        }
      }
    }
    cl.sync();  // b
    // c. this CTA's slice: p = tau_k sum_r P_r by a fixed pairwise tree (four
    //    dependent adds instead of sixteen), then p_i into every CTA
    {
      const int t0 = rank * L, nl = max(0, min(m, t0 + L) - t0);
      if (tid < nl) {
        double t[CL];
#pragma unroll
        for (int r = 0; r < CL; r++) t[r] = Pin[r * smax + tid];
#pragma unroll
        for (int h = CL / 2; h >= 1; h >>= 1)
#pragma unroll
          for (int r = 0; r < h; r++) t[r] = t[r] + t[r + h];
        part[tid] = tauk * t[0];  // part is free after a
      }
      __syncthreads();
      for (int e = tid; e < nl * CL; e += CL_NT) {
        const int tt = e / CL, d = e - tt * CL;  // row of the slice, destination CTA
        cl.map_shared_rank(p, d)[k + 1 + t0 + tt] = part[tt];
      }
    }
    cl.sync();  // c
    // d. look-ahead on column k+1 (its owner's warp 0), bulk update of own columns j >= k+2
    const int c1 = k + 1;
    const int owner = c1 % CL;
    const bool look = (rank == owner);
    if (look && w == 0) {
      double* col = Wl + (size_t)(c1 / CL) * n;
      double part = 0.0;  // this lane's share of |x|^2 of the updated column, formed on the way
      if (tauk != 0.0) {
        const double vc = v[c1], pc = p[c1];
        for (int i = c1 + 1 + (tid & 31); i < n; i += 32) {
          const double a = fma(v[i], pc, fma(neg(p[i]), vc, col[i]));
          col[i] = a;
          if (i >= c1 + 2) part = fma(a, a, part);
        }
        __syncwarp();
      } else {
        for (int i = c1 + 2 + (tid & 31); i < n; i += 32) part = fma(col[i], col[i], part);
      }
      if (c1 + 2 < n) {
        cluster_reflector_warp(col, n, c1, vnext, scal + 1, P.ev, P.tau, part);
      } else if ((tid & 31) == 0) {  // the last step: the real 1 x 1 tail (hessenberg.jl:27-29)
        P.ev[c1] = col[c1 + 1];
        P.tau[c1] = 0.0;
      }
    } else if (tauk != 0.0 && qb < ncl) {
      // elements e = t0, t0 + T, ... of the own block (column qb + e / m, row
      // k + 1 + e % m), four per pass; the quotient and remainder are stepped, not
      // divided
      const int t0 = look ? tid - 32 : tid, T = look ? CL_NT - 32 : CL_NT;
      const int cols = ncl - qb;
      const int Tq = T / m, Tr = T - Tq * m;
      int qd = t0 / m, ir = t0 - qd * m;
      while (qd < cols) {
        double a[4];
        int ii[4], jj[4];
        size_t at[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          ii[u] = -1;
          if (qd < cols) {
            const int qq = qb + qd;
            ii[u] = k + 1 + ir;
            jj[u] = rank + CL * qq;
            at[u] = (size_t)qq * n + ii[u];
            a[u] = Wl[at[u]];
            qd += Tq;
            ir += Tr;
            if (ir >= m) {
              ir -= m;
              qd++;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int i = ii[u], j = jj[u];
          if (i < 0 || i == j) continue;
          double x;
          if (i > j)
            x = fma(v[i], p[j], fma(neg(p[i]), v[j], a[u]));
          else
            x = fma(neg(v[j]), p[i], fma(p[j], v[i], a[u]));
          Wl[at[u]] = x;
        }
      }
    }
    cl.sync();  // e
    if (c1 + 2 < n) {
      const double* src = cl.map_shared_rank(vnext, owner);
      for (int i = c1 + 1 + tid; i < n; i += CL_NT) v[i] = src[i];
      if (tid == 0) scal[0] = *cl.map_shared_rank(scal + 1, owner);
    }
    __syncthreads();
  }
  if (n == 2 && rank == 0 && tid == 0) {  // no step: the 1 x 1 tail only
    P.ev[0] = Wl[1];
    P.tau[0] = 0.0;
  }
  // the reduced matrix back in place (reflectors below the subdiagonal)
  for (int64_t e = tid; e < (int64_t)ncl * n; e += CL_NT) {
    const int q = (int)(e / n), i = (int)(e - (int64_t)q * n);
    P.A[i + (int64_t)(rank + CL * q) * P.lda] = Wl[e];
  }
  if (rank == 0 && tid == 0 && P.info) *P.info = SKEW_OK;
  cl.sync();  // no CTA leaves while another may still read its shared memory
}

size_t cluster_hess_smem_bytes(int n) { return sizeof(double) * cluster_smem_doubles(n); }

// One cluster of 16 CTAs.  cudaErrorNotSupported (the caller then takes the
// grid-wide reduction) if the device cannot run a 16-CTA cluster with this
// much shared memory per CTA.
cudaError_t cluster_hessenberg(double* A, int64_t lda, int n, double* tau, double* ev, int* info, cudaStream_t st) {
  if (n < 3) return cudaErrorInvalidValue;
  const size_t smem = cluster_hess_smem_bytes(n);
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  if (smem > (size_t)optin) return cudaErrorNotSupported;
  static std::atomic<uint64_t> configured{0};
  const uint64_t bit = 1ull << (dev & 63);
  if (!(configured.load(std::memory_order_acquire) & bit)) {
    e = cudaFuncSetAttribute(cluster_hess_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(cluster_hess_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
    configured.fetch_or(bit, std::memory_order_release);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(CL_NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&clusters, (void*)cluster_hess_kernel, &cfg);
  if (e != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return cudaErrorNotSupported;
  }
  ClusterParams P{A, lda, n, tau, ev, info};
  return cudaLaunchKernelEx(&cfg, cluster_hess_kernel, P);
}

}  // namespace skew
