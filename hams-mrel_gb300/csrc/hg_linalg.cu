// Blocked complex LU with partial pivoting and triangular solves.
//
// getrf: right-looking, panel width NB = 32.  Per panel: the panel
// factorisation (16-CTA cluster kernel, or one CTA when a cluster does not
// fit: pivot = max |re|+|im| as LAPACK's IZAMAX, row swaps, reciprocal
// scaling, rank-1 updates), the row interchanges applied to the columns
// outside the panel, a unit-lower triangular solve for the U12 block and the
// trailing update A22 -= L21 U12, the only O(n^3) step.  Complex64 with
// tensor cores: two levels, 256-wide outer panels factorised by that loop
// and their trailing updates on tcgen05 (hg_tc.cu).
#include <climits>
#include "hg_linalg.cuh"

namespace hg {

template <typename R> struct ops;
template <> struct ops<double> {
  typedef double2 T;
  static __device__ __forceinline__ T mk(double a, double b) { return make_double2(a, b); }
};
template <> struct ops<float> {
  typedef float2 T;
  static __device__ __forceinline__ T mk(float a, float b) { return make_float2(a, b); }
};

template <typename T> __device__ __forceinline__ T cmul(T a, T b) {
  T r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename T> __device__ __forceinline__ T csub(T a, T b) { T r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename T> __device__ __forceinline__ T crecip(T a) {
  // 1/a with Smith's scaling, compared in the element type
  T r;
  if (fabs(a.x) >= fabs(a.y)) {
    auto q = a.y / a.x, d = a.x + a.y * q;
    r.x = 1 / d; r.y = -q / d;
  } else {
    auto q = a.x / a.y, d = a.y + a.x * q;
    r.x = q / d; r.y = -1 / d;
  }
  return r;
}
template <typename T> __device__ __forceinline__ T cdiv_(T a, T b) { return cmul(a, crecip(b)); }

// ------------------------------------------------------------------------
// GEMM
// ------------------------------------------------------------------------
template <typename R, int BM, int BN, int BK, int TM, int TN, bool TA>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
k_gemm(int m, int n, int k, typename cx<R>::T alpha, const typename cx<R>::T* __restrict__ A, long lda,
       const typename cx<R>::T* __restrict__ B, long ldb, typename cx<R>::T beta,
       typename cx<R>::T* __restrict__ C, long ldc, int kchunk, typename cx<R>::T* __restrict__ ws) {
  // Split-K when gridDim.z > 1: this CTA sums k in [z*kchunk, (z+1)*kchunk)
  // and writes alpha * partial into the z-th m x n slice of ws (no beta).
  typedef typename cx<R>::T T;
  constexpr int TX = BM / TM, TY = BN / TN, NT = TX * TY;
  __shared__ R as_re[BK][BM], as_im[BK][BM], bs_re[BK][BN], bs_im[BK][BN];
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const bool split = gridDim.z > 1;
  const int kbeg = split ? blockIdx.z * kchunk : 0;
  const int kend = split ? min(k, kbeg + kchunk) : k;
  if (split) {
    C = ws + (long)blockIdx.z * m * n;
    ldc = m;
    beta.x = 0; beta.y = 0;
  }
  R acr[TM][TN], aci[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) { acr[i][j] = 0; aci[i][j] = 0; }

  for (int kk = kbeg; kk < kend; kk += BK) {
#pragma unroll
    for (int e = tid; e < BM * BK; e += NT) {
      int i, l;
      if (!TA) { i = e % BM; l = e / BM; } else { l = e % BK; i = e / BK; }
      const int gm = m0 + i, gk = kk + l;
      T v;
      v.x = 0; v.y = 0;
      if (gm < m && gk < kend) v = TA ? A[gk + (long)gm * lda] : A[gm + (long)gk * lda];
      as_re[l][i] = v.x; as_im[l][i] = v.y;
    }
#pragma unroll
    for (int e = tid; e < BN * BK; e += NT) {
      const int l = e % BK, j = e / BK, gk = kk + l, gn = n0 + j;
      T v;
      v.x = 0; v.y = 0;
      if (gn < n && gk < kend) v = B[gk + (long)gn * ldb];
      bs_re[l][j] = v.x; bs_im[l][j] = v.y;
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < BK; ++l) {
      R ar[TM], ai[TM], br[TN], bi[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) { ar[i] = as_re[l][tx + i * TX]; ai[i] = as_im[l][tx + i * TX]; }
#pragma unroll
      for (int j = 0; j < TN; ++j) { br[j] = bs_re[l][ty + j * TY]; bi[j] = bs_im[l][ty + j * TY]; }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) {
          acr[i][j] = fma(ar[i], br[j], acr[i][j]);
          acr[i][j] = fma(-ai[i], bi[j], acr[i][j]);
          aci[i][j] = fma(ar[i], bi[j], aci[i][j]);
          aci[i][j] = fma(ai[i], br[j], aci[i][j]);
        }
    }
    __syncthreads();
  }
  const bool zb = (beta.x == 0 && beta.y == 0);
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int gn = n0 + ty + j * TY;
    if (gn >= n) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int gm = m0 + tx + i * TX;
      if (gm >= m) continue;
      T r;
      r.x = alpha.x * acr[i][j] - alpha.y * aci[i][j];
      r.y = alpha.x * aci[i][j] + alpha.y * acr[i][j];
      T* c = C + gm + (long)gn * ldc;
      if (!zb) {
        const T o = *c;
        r.x += beta.x * o.x - beta.y * o.y;
        r.y += beta.x * o.y + beta.y * o.x;
      }
      *c = r;
    }
  }
}

// C = sum over slices of the split-K partials + beta * C
template <typename T>
__global__ void k_splitk_reduce(int m, int n, int slices, const T* __restrict__ ws, T beta, T* __restrict__ C,
                                long ldc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= m) return;
  T acc;
  acc.x = 0; acc.y = 0;
  for (int z = 0; z < slices; ++z) {
    const T v = ws[(long)z * m * n + i + (long)j * m];
    acc.x += v.x; acc.y += v.y;
  }
  T* c = C + i + (long)j * ldc;
  if (beta.x != 0 || beta.y != 0) {
    const T o = *c;
    acc.x += beta.x * o.x - beta.y * o.y;
    acc.y += beta.x * o.y + beta.y * o.x;
  }
  *c = acc;
}

constexpr int kNumSMs = 152;

template <typename R, int BM, int BN, int BK, int TM, int TN>
static cudaError_t launch_gemm(cudaStream_t st, bool transa, int m, int n, int k, typename cx<R>::T alpha,
                               const typename cx<R>::T* A, long lda, const typename cx<R>::T* B, long ldb,
                               typename cx<R>::T beta, typename cx<R>::T* C, long ldc, void* ws, size_t ws_bytes) {
  typedef typename cx<R>::T T;
  if (m <= 0 || n <= 0) return cudaSuccess;
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN, 1);
  const int nt = (BM / TM) * (BN / TN);
  // Tall-skinny products (the refinement residuals, the normal-equation
  // right-hand sides) have too few output tiles to fill the GPU: split K.
  int slices = 1;
  const int tiles = grid.x * grid.y;
  if (ws && k >= 4 * 256 && tiles < 2 * kNumSMs) {
    slices = (2 * kNumSMs + tiles - 1) / tiles;
    slices = min(slices, k / 256);
    while (slices > 1 && (size_t)slices * m * n * sizeof(T) > ws_bytes) --slices;
  }
  int kchunk = k;
  if (slices > 1) {
    kchunk = ((k + slices - 1) / slices + BK - 1) / BK * BK;
    slices = (k + kchunk - 1) / kchunk;
    grid.z = slices;
  }
  T* w = static_cast<T*>(ws);
  if (transa)
    k_gemm<R, BM, BN, BK, TM, TN, true><<<grid, nt, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, w);
  else
    k_gemm<R, BM, BN, BK, TM, TN, false><<<grid, nt, 0, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, w);
  if (slices > 1) k_splitk_reduce<T><<<dim3((m + 255) / 256, n), 256, 0, st>>>(m, n, slices, w, beta, C, ldc);
  return cudaGetLastError();
}

template <>
cudaError_t gemm<double>(cudaStream_t st, bool transa, int m, int n, int k, double2 alpha, const double2* A,
                         long lda, const double2* B, long ldb, double2 beta, double2* C, long ldc, void* ws,
                         size_t ws_bytes) {
  if (n <= 32)
    return launch_gemm<double, 64, 32, 8, 4, 2>(st, transa, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes);
  return launch_gemm<double, 64, 64, 8, 4, 4>(st, transa, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes);
}
template <>
cudaError_t gemm<float>(cudaStream_t st, bool transa, int m, int n, int k, float2 alpha, const float2* A,
                        long lda, const float2* B, long ldb, float2 beta, float2* C, long ldc, void* ws,
                        size_t ws_bytes) {
  // Split-K (a workspace and a deep K) keeps the older kernel; otherwise
  // the cp.async kernels: skinny (N <= 48) or wide.
  const bool splitk = ws && k >= 1024;
  if (!transa && n <= 48 && !splitk) return cgemm_skinny(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  if (n <= 64)
    return launch_gemm<float, 64, 32, 8, 4, 2>(st, transa, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, ws, ws_bytes);
  return cgemm_wide(st, transa, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ------------------------------------------------------------------------
// Panel factorisation: one CTA, rows [0, m) x columns [0, jb) of P.
// ------------------------------------------------------------------------
constexpr int kNB = 32;
constexpr int kPanelThreads = 1024;

template <typename R>
__global__ void __launch_bounds__(kPanelThreads)
k_getf2(typename cx<R>::T* P, long lda, int m, int jb, int* ipiv, int k0, int* info) {
  typedef typename cx<R>::T T;
  __shared__ R s_v[32];
  __shared__ int s_i[32];
  __shared__ T s_row[kNB];
  __shared__ int s_p;
  __shared__ R s_max;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int jj = 0; jj < jb; ++jj) {
    R best = -1;
    int bidx = INT_MAX;
    for (int r = jj + tid; r < m; r += kPanelThreads) {
      const T a = P[r + (long)jj * lda];
      const R v = fabs(a.x) + fabs(a.y);
      if (v > best) { best = v; bidx = r; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const R ov = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
    }
    if (lane == 0) { s_v[warp] = best; s_i[warp] = bidx; }
    __syncthreads();
    if (warp == 0) {
      best = (lane < kPanelThreads / 32) ? s_v[lane] : (R)-1;
      bidx = (lane < kPanelThreads / 32) ? s_i[lane] : INT_MAX;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const R ov = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
        if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
      }
      if (lane == 0) {
        if (bidx == INT_MAX) bidx = jj;
        s_p = bidx;
        s_max = best;
        ipiv[k0 + jj] = k0 + bidx + 1;
        if (!(best > 0) && *info == 0) *info = k0 + jj + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    if (s_max > 0) {
      if (p != jj && tid < jb) {
        const T t = P[jj + (long)tid * lda];
        P[jj + (long)tid * lda] = P[p + (long)tid * lda];
        P[p + (long)tid * lda] = t;
      }
      __syncthreads();
      if (tid < jb) s_row[tid] = P[jj + (long)tid * lda];
      __syncthreads();
      const T rp = crecip(s_row[jj]);
      for (int r = jj + 1 + tid; r < m; r += kPanelThreads) {
        const T l = cmul(P[r + (long)jj * lda], rp);
        P[r + (long)jj * lda] = l;
        for (int c = jj + 1; c < jb; ++c) {
          T* a = P + r + (long)c * lda;
          *a = csub(*a, cmul(l, s_row[c]));
        }
      }
    }
    __syncthreads();
  }
}

// Apply the pivots ipiv[r0..r1) (1-based global rows) to every column of A
// outside [skip0, skip1).
template <typename T>
__global__ void k_laswp(T* A, long lda, int ncols, const int* ipiv, int r0, int r1, int skip0, int skip1) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols || (c >= skip0 && c < skip1)) return;
  T* col = A + (long)c * lda;
  for (int r = r0; r < r1; ++r) {
    const int p = ipiv[r] - 1;
    if (p != r) {
      const T t = col[r];
      col[r] = col[p];
      col[p] = t;
    }
  }
}

template <typename T> __device__ __forceinline__ T shfl_c(T v, int src) {
  v.x = __shfl_sync(0xffffffffu, v.x, src);
  v.y = __shfl_sync(0xffffffffu, v.y, src);
  return v;
}

// After the panel at rows/columns [k, k + jb): the row interchanges
// ipiv[k..k+jb) on the other columns of [c0, c1), and X = L11^-1 X on the
// columns right of the panel (L11 the panel's unit-lower jb x jb block), in
// one pass: one warp per column.  The jb interchanges (in LAPACK's order)
// are first composed into labels: lane r learns which row's value ends up in
// block row k + r, and up to jb "outside" slots (rows below the block that
// an interchange touched) learn theirs; every warp composes them for itself
// (jb shuffle steps).  A column's values are then read once (all reads
// before any write) and written to their final rows, and lanes r > c
// subtract L(r, c) x_c for c = 0 .. jb - 2 with x_c shuffled from lane c.
// perm (optional): the running row permutation of the factorisation, one
// more column (of row numbers) that takes the same interchanges.
template <typename T>
__global__ void __launch_bounds__(256)
k_swap_trsm(T* __restrict__ A, long lda, int c0, int c1, int k, int jb, const int* __restrict__ ipiv,
            int* __restrict__ perm) {
  __shared__ T Ls[kNB][kNB + 1];  // Ls[c][r] = L(r, c)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (c1 > k + jb) {
    for (int e = tid; e < jb * jb; e += blockDim.x) {
      const int r = e % jb, c = e / jb;
      Ls[c][r] = A[(k + r) + (long)(k + c) * lda];
    }
  }
  const int tl = (lane < jb) ? ipiv[k + lane] - 1 - k : lane;  // relative target of interchange `lane`
  int blab = lane;          // row (relative to k) whose value ends in block row lane
  int opos = -1, olab = 0;  // outside slot of this lane: its row and the row whose value ends there
  int nused = 0;
  for (int r = 0; r < jb; ++r) {
    const int t = __shfl_sync(0xffffffffu, tl, r);
    if (t == r) continue;
    int s;
    int b;
    if (t < jb) {
      s = -1;
      b = __shfl_sync(0xffffffffu, blab, t);
    } else {
      const unsigned m = __ballot_sync(0xffffffffu, opos == t);
      if (m) {
        s = __ffs(m) - 1;
      } else {
        s = nused++;
        if (lane == s) { opos = t; olab = t; }
      }
      b = __shfl_sync(0xffffffffu, olab, s);
    }
    const int a = __shfl_sync(0xffffffffu, blab, r);
    if (lane == r) blab = b;
    if (s < 0) {
      if (lane == t) blab = a;
    } else if (lane == s) {
      olab = a;
    }
  }
  __syncthreads();  // Ls
  const int ncols = c1 - c0 - jb;
  const int q = blockIdx.x * (blockDim.x >> 5) + warp;
  if (perm && q == ncols) {
    int* x = perm + k;
    const int v = (lane < jb) ? x[blab] : 0;
    const int ov = (lane < nused) ? x[olab] : 0;
    __syncwarp();
    if (lane < jb) x[lane] = v;
    if (lane < nused) x[opos] = ov;
    return;
  }
  if (q >= ncols) return;
  const int col = (c0 + q < k) ? c0 + q : c0 + q + jb;
  T* x = A + (long)col * lda + k;
  T v, ov;
  v.x = 0; v.y = 0; ov = v;
  if (lane < jb) v = x[blab];
  if (lane < nused) ov = x[olab];
  __syncwarp();
  if (col > k) {
    for (int c = 0; c + 1 < jb; ++c) {
      const T xc = shfl_c(v, c);
      if (lane > c && lane < jb) v = csub(v, cmul(Ls[c][lane], xc));
    }
  }
  if (lane < jb) x[lane] = v;
  if (lane < nused) x[opos] = ov;
}

__global__ void k_iota(int n, int* __restrict__ perm) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) perm[r] = r;
}

// dst[r, c] = src[perm[r], c]
__global__ void k_gather_rows(int n, int nc, const int* __restrict__ perm, const float2* __restrict__ src, long lds,
                              float2* __restrict__ dst, long ldd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < n && c < nc) dst[r + (long)c * ldd] = src[perm[r] + (long)c * lds];
}

__global__ void k_copy_cols(int n, int nc, const float2* __restrict__ src, long lds, float2* __restrict__ dst,
                            long ldd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < n && c < nc) dst[r + (long)c * ldd] = src[r + (long)c * lds];
}

// X = U^{-1} X for the non-unit upper jb x jb block U.
template <typename T>
__global__ void k_trsm_upper(const T* U, long lda, int jb, T* X, long ldx, int ncols) {
  __shared__ T su[kNB][kNB + 1];
  __shared__ T sd[kNB];
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int r = e % jb, c = e / jb;
    su[r][c] = U[r + (long)c * lda];
  }
  __syncthreads();
  if (threadIdx.x < jb) sd[threadIdx.x] = crecip(su[threadIdx.x][threadIdx.x]);
  __syncthreads();
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncols) return;
  T x[kNB];
  T* xc = X + (long)col * ldx;
#pragma unroll
  for (int r = 0; r < kNB; ++r)
    if (r < jb) x[r] = xc[r];
#pragma unroll
  for (int rr = kNB - 1; rr >= 0; --rr) {
    if (rr >= jb) continue;
#pragma unroll
    for (int c = 0; c < kNB; ++c)
      if (c > rr && c < jb) x[rr] = csub(x[rr], cmul(su[rr][c], x[c]));
    x[rr] = cmul(x[rr], sd[rr]);
  }
#pragma unroll
  for (int r = 0; r < kNB; ++r)
    if (r < jb) xc[r] = x[r];
}

// Outer panel width of the two-level LU whose trailing updates run on the
// tensor cores: the inner dimension of the update GEMM (512 real), wide
// enough that its C tile read and write amortise over the multiply.
constexpr int kOuterNB = 256;
// Below this order the one-level loop is used (few outer panels to amortise).
constexpr int kTcMinN = 1024;

// Workspace of the two-level LU (complex64, tensor cores), in order:
//   tc    the tensor-core GEMM's packed operands
//   minv  I - L11^-1 of the current outer panel (256 x 256), to form U12 by a GEMM
//   linv  L_kk^-1 of every 256-wide diagonal block (256 x 256 each, kept for getrs_inv)
//   uinv  U_kk^-1 of every diagonal block
//   y     the intermediate solution of getrs_inv (n x kSolveChunk)
//   perm  the row permutation of the pivots (n ints, for getrs_inv): perm[r]
//         is the original row that the interchanges bring to row r
constexpr int kSolveChunk = 64;
struct LuWork {
  size_t tc, minv, linv, uinv, y, perm, total;
  explicit LuWork(int n) {
    const size_t blk = (size_t)kOuterNB * kOuterNB * sizeof(float2);
    const size_t nblk = (size_t)((n + kOuterNB - 1) / kOuterNB);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    tc = 0;
    minv = up(cgemm_tc_work_bytes(n, n, kOuterNB));
    linv = minv + blk;
    uinv = linv + nblk * blk;
    y = uinv + nblk * blk;
    perm = y + up((size_t)n * kSolveChunk * sizeof(float2));
    total = perm + up((size_t)n * sizeof(int));
  }
};

size_t lu_work_bytes(int n, int tc_passes) {
  if (tc_passes == 0 || n < kTcMinN) return 0;
  return LuWork(n).total;
}

// Workspace of the two-level complex128 LU (tensor cores): the sliced GEMM's
// digits; then for the current outer panel X = L11^-1, M = I - X, Xn = -X and
// Lf = L11 with its unit diagonal and zeros above (256 x 256 each), and W, a
// copy of A12 (256 x n) for the refinement of U12.
struct LuWorkZ {
  size_t zg, x, m, xn, lf, w, total;
  explicit LuWorkZ(int n) {
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t blk = up((size_t)kOuterNB * kOuterNB * sizeof(double2));
    zg = up(zgemm_tc_work_bytes(n, n, kOuterNB));
    x = zg;
    m = x + blk;
    xn = m + blk;
    lf = xn + blk;
    w = lf + blk;
    total = w + up((size_t)kOuterNB * n * sizeof(double2));
  }
};

size_t lu_work_bytes_z(int n) { return n < kTcMinN ? 0 : LuWorkZ(n).total; }

namespace {

// LU of the panel rows [k0, n) x columns [k0, k0 + jb) (jb <= 32), pivots
// written 1-based as global rows.
template <typename R>
cudaError_t panel(cudaStream_t st, bool use_cluster, int n, typename cx<R>::T* A, long lda, int k0, int jb, int* ipiv,
                  int* info) {
  if (use_cluster) return panel_cluster<R>(st, A + k0 + (long)k0 * lda, lda, n - k0, jb, ipiv, k0, info);
  k_getf2<R><<<1, kPanelThreads, 0, st>>>(A + k0 + (long)k0 * lda, lda, n - k0, jb, ipiv, k0, info);
  return cudaGetLastError();
}

// Columns [c0, c1) of A through one level of right-looking blocking with
// 32-wide panels (pivots applied only inside [c0, c1)).  With aux, the
// update of the columns beyond the next panel runs on aux->side (see getrf).
// Complex128 with zws (zgemm_tc_work_bytes of the update): each update is one
// sliced product on the tensor cores, on st.
template <typename R>
cudaError_t factor_columns(cudaStream_t st, bool use_cluster, int n, typename cx<R>::T* A, long lda, int c0, int c1,
                           int* ipiv, int* info, int* perm = nullptr, const LuAux* aux = nullptr, void* zws = nullptr,
                           size_t zws_bytes = 0) {
  typedef typename cx<R>::T T;
  T mone, one;
  mone.x = -1; mone.y = 0; one.x = 1; one.y = 0;
  bool side_pending = false;
  cudaError_t e = cudaSuccess;
  // complex128 on the tensor cores: 16-wide panels (their FP64 rank-1
  // updates, the panel's bound, are half those of 32-wide ones; the updates
  // between panels are tensor-core products either way)
  const int nbp = (sizeof(R) == 8 && zws) ? kNB / 2 : kNB;
  for (int k = c0; k < c1; k += nbp) {
    const int jb = (c1 - k < nbp) ? c1 - k : nbp;
    e = panel<R>(st, use_cluster, n, A, lda, k, jb, ipiv, info);
    if (e != cudaSuccess) return e;
    // the interchanges touch every other column of [c0, c1): the side update must be done
    if (side_pending) {
      e = cudaStreamWaitEvent(st, aux->ev_side, 0);
      if (e != cudaSuccess) return e;
      side_pending = false;
    }
    const int other = c1 - c0 - jb + (perm ? 1 : 0);
    if (other > 0) k_swap_trsm<T><<<(other + 7) / 8, 256, 0, st>>>(A, lda, c0, c1, k, jb, ipiv, perm);
    const int rest = c1 - k - jb;
    if (rest <= 0) continue;
    const int m = n - k - jb;
    const T* L21 = A + (k + jb) + (long)k * lda;
    const T* U12 = A + k + (long)(k + jb) * lda;
    T* A22 = A + (k + jb) + (long)(k + jb) * lda;
    if (sizeof(R) == 8 && zws) {
      e = zgemm_tc(st, m, rest, jb, reinterpret_cast<const double2*>(L21), lda, reinterpret_cast<const double2*>(U12), lda,
                   reinterpret_cast<double2*>(A22), lda, zws, zws_bytes, info);
      if (e != cudaSuccess) return e;
    } else if (aux && rest > kNB) {
      // the next panel's columns here, the others on the side stream
      e = gemm<R>(st, false, m, kNB, jb, mone, L21, lda, U12, lda, one, A22, lda);
      if (e == cudaSuccess) e = cudaEventRecord(aux->ev_main, st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(aux->side, aux->ev_main, 0);
      if (e == cudaSuccess)
        e = gemm<R>(aux->side, false, m, rest - kNB, jb, mone, L21, lda, U12 + (long)kNB * lda, lda, one,
                    A22 + (long)kNB * lda, lda);
      if (e == cudaSuccess) e = cudaEventRecord(aux->ev_side, aux->side);
      if (e != cudaSuccess) return e;
      side_pending = true;
    } else {
      e = gemm<R>(st, false, m, rest, jb, mone, L21, lda, U12, lda, one, A22, lda);
      if (e != cudaSuccess) return e;
    }
  }
  if (side_pending) {
    e = cudaStreamWaitEvent(st, aux->ev_side, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// Y <- I - X
__global__ void k_eye_minus(int nb, const float2* X, int ldx, float2* Y, int ldy) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < nb) {
    float2 v = X[r + (long)c * ldx];
    v.x = (r == c ? 1.f : 0.f) - v.x;
    v.y = -v.y;
    Y[r + (long)c * ldy] = v;
  }
}

// Y[0:jb, 0:nc] = M[0:jb, 0:jb] X[0:jb, 0:nc] for one diagonal block's
// inverse M (leading dimension 256).  It sits on the serial chain of the
// blocked solve, so it is cut into many short CTAs: a 32 x 8 output tile per
// CTA, the 256-deep inner dimension split over the 8 warps (lane = row, 32
// independent loads of M per thread in flight), X's 256 x 8 slice staged in
// shared memory, and the 8 partial tiles added in shared memory.
__global__ void __launch_bounds__(256)
k_apply_inv(int jb, int nc, const float2* __restrict__ M, const float2* __restrict__ X, long ldx,
            float2* __restrict__ Y, long ldy) {
  __shared__ float2 xs[kOuterNB][8];
  __shared__ float2 red[8][32][9];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 8;
  for (int e = threadIdx.x; e < kOuterNB * 8; e += 256) {
    const int p = e % kOuterNB, c = e / kOuterNB;
    xs[p][c] = (p < jb && c0 + c < nc) ? X[p + (long)(c0 + c) * ldx] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int r = r0 + lane;
  float ar[8], ai[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) { ar[j] = 0.f; ai[j] = 0.f; }
  const int p0 = w * 32;
  if (r < jb) {
    float2 mv[32];  // all 32 loads of M in flight at once
#pragma unroll
    for (int q = 0; q < 32; ++q) mv[q] = (p0 + q < jb) ? M[r + (long)(p0 + q) * kOuterNB] : make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 32; ++q) {
      const int p = p0 + q;
      const float2 m = mv[q];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 x = xs[p][j];
        ar[j] = fmaf(m.x, x.x, fmaf(-m.y, x.y, ar[j]));
        ai[j] = fmaf(m.x, x.y, fmaf(m.y, x.x, ai[j]));
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) red[w][lane][j] = make_float2(ar[j], ai[j]);
  __syncthreads();
  const int rr = threadIdx.x & 31, cc = threadIdx.x >> 5;  // one output per thread
  float2 acc = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    acc.x += red[k][rr][cc].x;
    acc.y += red[k][rr][cc].y;
  }
  if (r0 + rr < jb && c0 + cc < nc) Y[(r0 + rr) + (long)(c0 + cc) * ldy] = acc;
}

// X <- I (nb x nb, complex128)
__global__ void k_eye_z(int nb, double2* X, int ldx) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < nb) X[r + (long)c * ldx] = make_double2(r == c ? 1.0 : 0.0, 0.0);
}

// From X = L11^-1: M = I - X, Xn = -X, and Lf = the unit-lower L11 of the
// factor A11 with zeros above its diagonal (all nb x nb, leading dimension ld).
__global__ void k_u12_operands(int nb, const double2* __restrict__ X, const double2* __restrict__ A11, long lda,
                               double2* __restrict__ M, double2* __restrict__ Xn, double2* __restrict__ Lf, int ld) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= nb) return;
  const long o = r + (long)c * ld;
  const double2 x = X[o];
  M[o] = make_double2((r == c ? 1.0 : 0.0) - x.x, -x.y);
  Xn[o] = make_double2(-x.x, -x.y);
  Lf[o] = r > c ? A11[r + (long)c * lda] : make_double2(r == c ? 1.0 : 0.0, 0.0);
}

// Two-level complex128 LU: 256-wide outer panels by the 32-wide loop (panels
// on the FP64 pipes, their updates inside the outer panel on the tensor
// cores), then U12 = L11^-1 A12 and A22 -= L21 U12, all products as exact
// BF16 digit products (zgemm_tc).  U12 from the explicit inverse
// (X = L11^-1, a column-parallel triangular solve of the identity) with one
// refinement step, U0 = A12 - (I - X) A12, U12 = U0 + X (A12 - L11 U0): the
// inverse alone would leave a backward error of cond(L11) eps in U12, the
// step brings the factorisation's back to that of a triangular solve.
cudaError_t getrf_z_tc(cudaStream_t st, bool use_cluster, int n, double2* A, long lda, int* ipiv, int* info, void* work,
                       const LuAux* aux) {
  const LuWorkZ lw(n);
  char* wb = static_cast<char*>(work);
  double2* X = reinterpret_cast<double2*>(wb + lw.x);
  double2* M = reinterpret_cast<double2*>(wb + lw.m);
  double2* Xn = reinterpret_cast<double2*>(wb + lw.xn);
  double2* Lf = reinterpret_cast<double2*>(wb + lw.lf);
  double2* W = reinterpret_cast<double2*>(wb + lw.w);
  cudaError_t e = cudaSuccess;
  for (int K = 0; K < n; K += kOuterNB) {
    const int jbo = (n - K < kOuterNB) ? n - K : kOuterNB;
    e = factor_columns<double>(st, use_cluster, n, A, lda, K, K + jbo, ipiv, info, nullptr, aux, work, lw.zg);
    if (e != cudaSuccess) return e;
    k_laswp<double2><<<(n + 127) / 128, 128, 0, st>>>(A, lda, n, ipiv, K, K + jbo, K, K + jbo);
    const int rest = n - K - jbo;
    if (rest <= 0) continue;
    const dim3 eg((jbo + 127) / 128, jbo);
    double2* A11 = A + K + (long)K * lda;
    double2* A12 = A + K + (long)(K + jbo) * lda;
    k_eye_z<<<eg, 128, 0, st>>>(jbo, X, kOuterNB);
    e = trsm_cols<double>(st, false, A11, lda, jbo, X, kOuterNB, jbo);
    if (e != cudaSuccess) return e;
    k_u12_operands<<<eg, 128, 0, st>>>(jbo, X, A11, lda, M, Xn, Lf, kOuterNB);
    e = cudaMemcpy2DAsync(W, (size_t)kOuterNB * sizeof(double2), A12, (size_t)lda * sizeof(double2),
                          (size_t)jbo * sizeof(double2), rest, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    e = zgemm_tc(st, jbo, rest, jbo, M, kOuterNB, A12, lda, A12, lda, work, lw.zg, info);  // A12 <- U0
    if (e == cudaSuccess) e = zgemm_tc(st, jbo, rest, jbo, Lf, kOuterNB, A12, lda, W, kOuterNB, work, lw.zg, info);
    if (e == cudaSuccess) e = zgemm_tc(st, jbo, rest, jbo, Xn, kOuterNB, W, kOuterNB, A12, lda, work, lw.zg, info);
    if (e != cudaSuccess) return e;
    e = zgemm_tc(st, rest, rest, jbo, A + (K + jbo) + (long)K * lda, lda, A12, lda, A + (K + jbo) + (long)(K + jbo) * lda,
                 lda, work, lw.zg, info);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace

template <typename R>
cudaError_t getrf(cudaStream_t st, int n, typename cx<R>::T* A, long lda, int* ipiv, int* info, void* work,
                  size_t work_bytes, int tc_passes, const LuAux* aux) {
  if (aux && (!aux->side || !aux->ev_main || !aux->ev_side)) aux = nullptr;
  cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (sizeof(R) == 8 && tc_passes != 0 && n >= kTcMinN && work && work_bytes >= lu_work_bytes_z(n) &&
      zgemm_tc_supported())
    return getrf_z_tc(st, panel_cluster_supported<R>(n, kNB / 2), n, reinterpret_cast<double2*>(A), lda, ipiv, info,
                      work, aux);
  const bool use_cluster = panel_cluster_supported<R>(n);
  const bool tc = sizeof(R) == 4 && tc_passes != 0 && n >= kTcMinN && work &&
                  work_bytes >= lu_work_bytes(n, tc_passes) && cgemm_tc_supported();
  if (!tc) return factor_columns<R>(st, use_cluster, n, A, lda, 0, n, ipiv, info, nullptr, aux);
  // Two levels: 256-wide outer panels factorised by the 32-wide loop above,
  // then U12 = L11^-1 A12 and the tensor-core update A22 -= L21 U12.  U12
  // is formed as A12 - (I - L11^-1) A12 on the tensor cores too, with
  // L11^-1 from one column-parallel triangular solve of the identity (the
  // GEMM packs its B operand, here A12, before it overwrites A12).
  typedef typename cx<R>::T T;
  const LuWork lw(n);
  const size_t tcb = lw.minv;
  char* wb = static_cast<char*>(work);
  float2* Minv = reinterpret_cast<float2*>(wb + lw.minv);
  int* perm = reinterpret_cast<int*>(wb + lw.perm);
  k_iota<<<(n + 255) / 256, 256, 0, st>>>(n, perm);
  const size_t blk = (size_t)kOuterNB * kOuterNB;
  for (int K = 0; K < n; K += kOuterNB) {
    const int jbo = (n - K < kOuterNB) ? n - K : kOuterNB;
    e = factor_columns<R>(st, use_cluster, n, A, lda, K, K + jbo, ipiv, info, perm, aux);
    if (e != cudaSuccess) return e;
    k_laswp<T><<<(n + 127) / 128, 128, 0, st>>>(A, lda, n, ipiv, K, K + jbo, K, K + jbo);
    // inverse of this diagonal block's unit-lower triangle (for U12 here and
    // for getrs_inv); the upper triangles' inverses follow after the loop
    float2* Linv_all = reinterpret_cast<float2*>(wb + lw.linv);
    const float2* Linv = Linv_all + (size_t)(K / kOuterNB) * blk;
    e = trsm_inverse_blocks<float>(st, false, reinterpret_cast<const float2*>(A), lda, n, kOuterNB, Linv_all, kOuterNB,
                                   K / kOuterNB, 1);
    if (e != cudaSuccess) return e;
    const dim3 eg((jbo + 127) / 128, jbo);
    const int rest = n - K - jbo;
    if (rest > 0) {
      k_eye_minus<<<eg, 128, 0, st>>>(jbo, Linv, kOuterNB, Minv, jbo);
      float2* A12 = reinterpret_cast<float2*>(A + K + (long)(K + jbo) * lda);
      e = cgemm_tc(st, tc_passes, jbo, rest, jbo, Minv, jbo, A12, lda, A12, lda, work, tcb, info);
      if (e != cudaSuccess) return e;
      e = cgemm_tc(st, tc_passes, rest, rest, jbo, reinterpret_cast<const float2*>(A + (K + jbo) + (long)K * lda), lda,
                   A12, lda, reinterpret_cast<float2*>(A + (K + jbo) + (long)(K + jbo) * lda), lda, work, tcb, info);
      if (e != cudaSuccess) return e;
    }
  }
  // U_kk^-1 of every diagonal block, in one launch
  return trsm_inverse_blocks<float>(st, true, reinterpret_cast<const float2*>(A), lda, n, kOuterNB,
                                    reinterpret_cast<float2*>(wb + lw.uinv), kOuterNB, 0, (n + kOuterNB - 1) / kOuterNB);
}

constexpr int kSolveNB = 256;

bool lu_has_inverses(int n, int tc_passes, size_t work_bytes) {
  return tc_passes != 0 && n >= kTcMinN && work_bytes >= lu_work_bytes(n, tc_passes) && cgemm_tc_supported();
}

// Triangular solves with the diagonal-block inverses getrf kept: per 256-row
// block one small GEMM by the block inverse and one update GEMM of the rows
// below (above), instead of a row-by-row substitution inside each block.
//   forward:  Y_k = L_kk^-1 B_k;  B_(k+1:) -= L_(k+1:),k Y_k
//   backward: X_k = U_kk^-1 Y_k;  Y_(:k)   -= U_(:k),k X_k   (X written into B)
cudaError_t getrs_inv(cudaStream_t st, int n, int nrhs, const float2* LU, long lda, const int* ipiv, float2* B,
                      long ldb, void* work) {
  const LuWork lw(n);
  char* wb = static_cast<char*>(work);
  const float2* Linv = reinterpret_cast<const float2*>(wb + lw.linv);
  const float2* Uinv = reinterpret_cast<const float2*>(wb + lw.uinv);
  float2* Y = reinterpret_cast<float2*>(wb + lw.y);
  const size_t blk = (size_t)kOuterNB * kOuterNB;
  const float2 mone = make_float2(-1.f, 0.f), one = make_float2(1.f, 0.f);
  const int nblk = (n + kOuterNB - 1) / kOuterNB;
  const int* perm = reinterpret_cast<const int*>(wb + lw.perm);
  for (int c0 = 0; c0 < nrhs; c0 += kSolveChunk) {
    const int nc = (nrhs - c0 < kSolveChunk) ? nrhs - c0 : kSolveChunk;
    float2* Bc = B + (long)c0 * ldb;
    {  // Bc = P Bc through Y
      const dim3 g((n + 255) / 256, nc);
      k_gather_rows<<<g, 256, 0, st>>>(n, nc, perm, Bc, ldb, Y, n);
      k_copy_cols<<<g, 256, 0, st>>>(n, nc, Y, n, Bc, ldb);
    }
    for (int b = 0; b < nblk; ++b) {
      const int K = b * kOuterNB, jb = (n - K < kOuterNB) ? n - K : kOuterNB;
      k_apply_inv<<<dim3((jb + 31) / 32, (nc + 7) / 8), 256, 0, st>>>(jb, nc, Linv + b * blk, Bc + K, ldb, Y + K, n);
      const int rest = n - K - jb;
      if (rest > 0) {
        cudaError_t e = gemm<float>(st, false, rest, nc, jb, mone, LU + (K + jb) + (long)K * lda, lda, Y + K, n, one,
                                    Bc + K + jb, ldb);
        if (e != cudaSuccess) return e;
      }
    }
    for (int b = nblk - 1; b >= 0; --b) {
      const int K = b * kOuterNB, jb = (n - K < kOuterNB) ? n - K : kOuterNB;
      k_apply_inv<<<dim3((jb + 31) / 32, (nc + 7) / 8), 256, 0, st>>>(jb, nc, Uinv + b * blk, Y + K, n, Bc + K, ldb);
      if (K > 0) {
        cudaError_t e = gemm<float>(st, false, K, nc, jb, mone, LU + (long)K * lda, lda, Bc + K, ldb, one, Y, n);
        if (e != cudaSuccess) return e;
      }
    }
  }
  return cudaGetLastError();
}

template <typename R>
cudaError_t getrs(cudaStream_t st, int n, int nrhs, const typename cx<R>::T* LU, long lda, const int* ipiv,
                  typename cx<R>::T* B, long ldb, void* work, size_t work_bytes, int* status) {
  typedef typename cx<R>::T T;
  T mone, one;
  mone.x = -1; mone.y = 0; one.x = 1; one.y = 0;
  // complex128 block updates as exact digit products on the tensor cores
  const bool ztc = sizeof(R) == 8 && work && status && n > kSolveNB &&
                   work_bytes >= zgemm_tc_work_bytes(n, nrhs, kSolveNB) && zgemm_tc_supported();
  auto update = [&](int m, int kk, const T* A_, const T* X_, T* C_) -> cudaError_t {
    if (ztc)
      return zgemm_tc(st, m, nrhs, kk, reinterpret_cast<const double2*>(A_), lda, reinterpret_cast<const double2*>(X_),
                      ldb, reinterpret_cast<double2*>(C_), ldb, work, work_bytes, status);
    return gemm<R>(st, false, m, nrhs, kk, mone, A_, lda, X_, ldb, one, C_, ldb);
  };
  k_laswp<T><<<(nrhs + 127) / 128, 128, 0, st>>>(B, ldb, nrhs, ipiv, 0, n, 0, 0);
  for (int k = 0; k < n; k += kSolveNB) {
    const int jb = (n - k < kSolveNB) ? n - k : kSolveNB;
    cudaError_t e = trsm_cols<R>(st, false, LU + k + (long)k * lda, lda, jb, B + k, ldb, nrhs);
    if (e != cudaSuccess) return e;
    const int rest = n - k - jb;
    if (rest > 0) {
      e = update(rest, jb, LU + (k + jb) + (long)k * lda, B + k, B + k + jb);
      if (e != cudaSuccess) return e;
    }
  }
  const int last = ((n - 1) / kSolveNB) * kSolveNB;
  for (int k = last; k >= 0; k -= kSolveNB) {
    const int jb = (n - k < kSolveNB) ? n - k : kSolveNB;
    cudaError_t e = trsm_cols<R>(st, true, LU + k + (long)k * lda, lda, jb, B + k, ldb, nrhs);
    if (e != cudaSuccess) return e;
    if (k > 0) {
      e = update(k, jb, LU + (long)k * lda, B + k, B);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}

template cudaError_t getrf<double>(cudaStream_t, int, double2*, long, int*, int*, void*, size_t, int, const LuAux*);
template cudaError_t getrf<float>(cudaStream_t, int, float2*, long, int*, int*, void*, size_t, int, const LuAux*);
template cudaError_t getrs<double>(cudaStream_t, int, int, const double2*, long, const int*, double2*, long, void*,
                                   size_t, int*);
template cudaError_t getrs<float>(cudaStream_t, int, int, const float2*, long, const int*, float2*, long, void*,
                                  size_t, int*);

// ------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------
__global__ void k_z2c(long count, const double2* s, float2* d) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x)
    d[i] = make_float2((float)s[i].x, (float)s[i].y);
}
__global__ void k_c2z(long count, const float2* s, double2* d) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < count; i += (long)gridDim.x * blockDim.x)
    d[i] = make_double2(s[i].x, s[i].y);
}
__global__ void k_z2c_2d(int rows, int cols, const double2* s, long lds, float2* d, long ldd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < rows) {
    const double2 v = s[r + (long)c * lds];
    d[r + (long)c * ldd] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_add_c2z_2d(int rows, int cols, const float2* s, long lds, double2* d, long ldd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < rows) {
    const float2 v = s[r + (long)c * lds];
    double2* o = d + r + (long)c * ldd;
    o->x += v.x;
    o->y += v.y;
  }
}
cudaError_t convert_z2c(cudaStream_t st, long count, const double2* src, float2* dst) {
  k_z2c<<<1216, 256, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}
cudaError_t convert_c2z(cudaStream_t st, long count, const float2* src, double2* dst) {
  k_c2z<<<1216, 256, 0, st>>>(count, src, dst);
  return cudaGetLastError();
}
cudaError_t convert_z2c_2d(cudaStream_t st, int rows, int cols, const double2* src, long lds, float2* dst, long ldd) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  k_z2c_2d<<<dim3((rows + 255) / 256, cols), 256, 0, st>>>(rows, cols, src, lds, dst, ldd);
  return cudaGetLastError();
}
cudaError_t add_c2z_2d(cudaStream_t st, int rows, int cols, const float2* src, long lds, double2* dst, long ldd) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  k_add_c2z_2d<<<dim3((rows + 255) / 256, cols), 256, 0, st>>>(rows, cols, src, lds, dst, ldd);
  return cudaGetLastError();
}

}  // namespace hg
