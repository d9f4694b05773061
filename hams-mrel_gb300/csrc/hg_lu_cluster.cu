// LU panel factorisation on a 16-CTA thread-block cluster, and the
// column-parallel triangular solves used by getrs.
//
// Panel (rows k..n-1, 32 columns): the 16 CTAs of one cluster each keep a
// contiguous slice of the panel's rows in shared memory, so the whole panel
// (up to ~3.5 MB) stays on chip in distributed shared memory for all 32
// column steps.  Per column: every CTA finds its local pivot candidate
// (max |re|+|im|, the IZAMAX rule, first row on ties), a cluster barrier
// publishes the candidates, every CTA reads the 16 candidates and the pivot
// row straight out of the owners' shared memory, a second cluster barrier
// orders those reads before the row interchange is written, and each CTA
// scales and rank-1 updates its own rows.
#include <climits>
#include <cooperative_groups.h>

#include "hg_linalg.cuh"

namespace cg = cooperative_groups;

namespace hg {

template <typename T> __device__ __forceinline__ T c_mul(T a, T b) {
  T r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename T> __device__ __forceinline__ T c_sub(T a, T b) { T r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename T> __device__ __forceinline__ T c_recip(T a) {
  T r;
  if (fabs((double)a.x) >= fabs((double)a.y)) {
    auto q = a.y / a.x, d = a.x + a.y * q;
    r.x = 1 / d; r.y = -q / d;
  } else {
    auto q = a.x / a.y, d = a.y + a.x * q;
    r.x = q / d; r.y = -1 / d;
  }
  return r;
}
template <typename T> __device__ __forceinline__ T c_div(T a, T b) {
  T r;
  if (fabs((double)b.x) >= fabs((double)b.y)) {
    auto q = b.y / b.x, d = b.x + b.y * q;
    r.x = (a.x + a.y * q) / d; r.y = (a.y - a.x * q) / d;
  } else {
    auto q = b.x / b.y, d = b.y + b.x * q;
    r.x = (a.x * q + a.y) / d; r.y = (a.y * q - a.x) / d;
  }
  return r;
}

constexpr int kClusterCTAs = 16;
constexpr int kClusterNB = 32;
constexpr int kClusterThreads = 512;

template <typename R>
__global__ void __launch_bounds__(kClusterThreads)
k_getf2_cluster(typename cx<R>::T* __restrict__ P, long lda, int m, int jb, int rpc, int* __restrict__ ipiv, int k0,
                int* __restrict__ info) {
  typedef typename cx<R>::T T;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // [jb][rpc], row index fastest
  __shared__ R s_cval;
  __shared__ int s_cidx;
  __shared__ R red_v[kClusterThreads / 32];
  __shared__ int red_i[kClusterThreads / 32];
  __shared__ T s_prow[kClusterNB];
  __shared__ T s_tmp[kClusterNB];
  __shared__ int s_p;
  __shared__ R s_pmax;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = rank * rpc;
  const int rl = max(0, min(rpc, m - r0));

  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    tile[c * rpc + r] = P[(r0 + r) + (long)c * lda];
  }
  __syncthreads();

  for (int jj = 0; jj < jb; ++jj) {
    // (a) local pivot candidate among rows >= jj
    R best = -1;
    int bidx = INT_MAX;
    for (int r = tid; r < rl; r += blockDim.x) {
      if (r0 + r >= jj) {
        const T a = tile[jj * rpc + r];
        const R v = fabs(a.x) + fabs(a.y);
        if (v > best) { best = v; bidx = r0 + r; }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const R ov = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
    }
    if (lane == 0) { red_v[warp] = best; red_i[warp] = bidx; }
    __syncthreads();
    if (tid == 0) {
      R b = -1;
      int bi = INT_MAX;
      for (int w = 0; w < kClusterThreads / 32; ++w)
        if (red_v[w] > b || (red_v[w] == b && red_i[w] < bi)) { b = red_v[w]; bi = red_i[w]; }
      s_cval = b;
      s_cidx = bi;
    }
    cluster.sync();  // (1) candidates visible cluster-wide

    // (b) the pivot: same decision in every CTA
    if (warp == 0) {
      R v = -1;
      int i = INT_MAX;
      if (lane < kClusterCTAs) {
        v = *cluster.map_shared_rank(&s_cval, lane);
        i = *cluster.map_shared_rank(&s_cidx, lane);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const R ov = __shfl_down_sync(0xffffffffu, v, off);
        const int oi = __shfl_down_sync(0xffffffffu, i, off);
        if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
      }
      if (lane == 0) {
        s_p = (i == INT_MAX) ? jj : i;
        s_pmax = v;
      }
    }
    __syncthreads();
    const int p = s_p;
    const R pmax = s_pmax;
    const int op = p / rpc, lp = p - op * rpc;
    const int oj = jj / rpc, lj = jj - oj * rpc;
    // (c) read the old pivot row; the owner of row p also reads the old row jj
    if (tid < jb) {
      s_prow[tid] = *cluster.map_shared_rank(&tile[tid * rpc + lp], op);
      if (rank == op && p != jj) s_tmp[tid] = *cluster.map_shared_rank(&tile[tid * rpc + lj], oj);
    }
    cluster.sync();  // (2) every read of the old rows precedes the interchange
    if (tid < jb) {
      if (rank == oj) tile[tid * rpc + lj] = s_prow[tid];
      if (rank == op && p != jj) tile[tid * rpc + lp] = s_tmp[tid];
    }
    if (rank == 0 && tid == 0) {
      ipiv[k0 + jj] = k0 + p + 1;
      if (!(pmax > 0) && *info == 0) *info = k0 + jj + 1;
    }
    __syncthreads();
    // (d) scale the column below the pivot and update this CTA's rows
    if (pmax > 0) {
      const T rp = c_recip(s_prow[jj]);
      for (int r = tid; r < rl; r += blockDim.x) {
        if (r0 + r > jj) {
          const T l = c_mul(tile[jj * rpc + r], rp);
          tile[jj * rpc + r] = l;
          for (int c = jj + 1; c < jb; ++c) tile[c * rpc + r] = c_sub(tile[c * rpc + r], c_mul(l, s_prow[c]));
        }
      }
    }
    __syncthreads();
  }
  cluster.sync();  // no CTA leaves while another could still read its shared memory
  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    P[(r0 + r) + (long)c * lda] = tile[c * rpc + r];
  }
}

template <typename R>
cudaError_t panel_cluster(cudaStream_t st, typename cx<R>::T* P, long lda, int m, int jb, int* ipiv, int k0,
                          int* info) {
  typedef typename cx<R>::T T;
  if (jb > kClusterNB) return cudaErrorNotSupported;
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  const size_t smem = (size_t)rpc * jb * sizeof(T);
  static int attr_done[2] = {0, 0};
  const int idx = sizeof(R) == 8 ? 1 : 0;
  if (smem > 220 * 1024) return cudaErrorNotSupported;
  auto kern = k_getf2_cluster<R>;
  if (!attr_done[idx]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e != cudaSuccess) return e;
    attr_done[idx] = 1;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCTAs, 1, 1);
  cfg.blockDim = dim3(kClusterThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kClusterCTAs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, P, lda, m, jb, rpc, ipiv, k0, info);
}

template cudaError_t panel_cluster<float>(cudaStream_t, float2*, long, int, int, int*, int, int*);
template cudaError_t panel_cluster<double>(cudaStream_t, double2*, long, int, int, int*, int, int*);

// Whether a 16-CTA cluster with the given dynamic shared memory can run here.
template <typename R>
bool panel_cluster_supported(int m) {
  typedef typename cx<R>::T T;
  static int cached[2] = {-1, -1};
  const int idx = sizeof(R) == 8 ? 1 : 0;
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  if ((size_t)rpc * kClusterNB * sizeof(T) > 220 * 1024) return false;
  if (cached[idx] < 0) {
    auto kern = k_getf2_cluster<R>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    int ncl = 0;
    if (e == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kClusterCTAs, 1, 1);
      cfg.blockDim = dim3(kClusterThreads, 1, 1);
      cfg.dynamicSmemBytes = 220 * 1024;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = kClusterCTAs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      e = cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg);
    }
    cudaGetLastError();
    cached[idx] = (e == cudaSuccess && ncl >= 1) ? 1 : 0;
  }
  return cached[idx] == 1;
}
template bool panel_cluster_supported<float>(int);
template bool panel_cluster_supported<double>(int);

// ---------------------------------------------------------------------------
// Triangular solves, one CTA per right-hand-side column, rows across threads
// (jb <= 256): X = L^{-1} X (unit lower) or X = U^{-1} X (upper, divides by
// the diagonal as ZTRSM does).
// ---------------------------------------------------------------------------
constexpr int kTrsmBlock = 256;

template <typename T, bool UPPER>
__global__ void __launch_bounds__(kTrsmBlock)
k_trsm_col(const T* __restrict__ A, long lda, int jb, T* __restrict__ X, long ldx) {
  __shared__ T x[kTrsmBlock];
  const int col = blockIdx.x, tid = threadIdx.x;
  T* xc = X + (long)col * ldx;
  if (tid < jb) x[tid] = xc[tid];
  __syncthreads();
  if (!UPPER) {
    for (int c = 0; c < jb; ++c) {
      if (tid > c && tid < jb) x[tid] = c_sub(x[tid], c_mul(A[tid + (long)c * lda], x[c]));
      __syncthreads();
    }
  } else {
    for (int c = jb - 1; c >= 0; --c) {
      if (tid == c) x[c] = c_div(x[c], A[c + (long)c * lda]);
      __syncthreads();
      if (tid < c) x[tid] = c_sub(x[tid], c_mul(A[tid + (long)c * lda], x[c]));
      __syncthreads();
    }
  }
  if (tid < jb) xc[tid] = x[tid];
}

template <typename R>
cudaError_t trsm_cols(cudaStream_t st, bool upper, const typename cx<R>::T* A, long lda, int jb,
                      typename cx<R>::T* X, long ldx, int ncols) {
  typedef typename cx<R>::T T;
  if (jb > kTrsmBlock) return cudaErrorInvalidValue;
  if (ncols <= 0) return cudaSuccess;
  if (upper) k_trsm_col<T, true><<<ncols, kTrsmBlock, 0, st>>>(A, lda, jb, X, ldx);
  else k_trsm_col<T, false><<<ncols, kTrsmBlock, 0, st>>>(A, lda, jb, X, ldx);
  return cudaGetLastError();
}
template cudaError_t trsm_cols<float>(cudaStream_t, bool, const float2*, long, int, float2*, long, int);
template cudaError_t trsm_cols<double>(cudaStream_t, bool, const double2*, long, int, double2*, long, int);

}  // namespace hg
