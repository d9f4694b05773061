// LU panel factorisation on a 16-CTA thread-block cluster, and the
// column-parallel triangular solves used by getrs.
//
// Panel (rows k..n-1, 32 columns): the 16 CTAs of one cluster each keep a
// contiguous slice of the panel's rows in shared memory, so the whole panel
// (up to ~3.5 MB) stays on chip in distributed shared memory for all 32
// column steps.  Per column: every CTA finds its local pivot candidate
// (max |re|+|im|, the IZAMAX rule, first row on ties) and publishes it with
// its row, one cluster barrier, every CTA reads the 16 candidates and rows
// out of the other CTAs' shared memory, takes the same pivot, and scales and
// rank-1 updates its own rows.
//
// Complex64 panels of up to 16 x 512 rows take a register-resident form
// (k_getf2_cluster_reg): one panel row per thread for all 32 column steps,
// the steps unrolled so that every register index is a compile-time
// constant, and per column one 528-byte message (candidate row, row jj,
// the candidate's reciprocal) pushed to every CTA by bulk copy.  Taller
// complex64 panels keep the rows in shared memory (k_getf2_cluster_push).
// FP64 panels of at most 16 columns take the same pushed exchange
// (k_getf2_cluster_push_z), wider or taller ones the loading form
// (k_getf2_cluster).  The two complex64 forms give bitwise-equal factors and
// pivots.
#include <mutex>
#include <climits>
#include <cooperative_groups.h>

#include "hg_linalg.cuh"
#include "hg_tma.cuh"

namespace cg = cooperative_groups;

namespace hg {

template <typename T> __device__ __forceinline__ T c_mul(T a, T b) {
  T r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename T> __device__ __forceinline__ T c_sub(T a, T b) { T r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// Smith's algorithm; the comparisons stay in the element type (a double
// conversion would run on the FP64 pipes, 1/64 of the FP32 rate here).
template <typename T> __device__ __forceinline__ T c_recip(T a) {
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
constexpr int kClusterCTAs = 16;
constexpr int kClusterNB = 32;
constexpr int kClusterThreads = 512;
// Dynamic shared memory of one panel CTA (its rows of the panel); with the
// kernel's static buffers (< 11 KB) it stays under the 227 KB per-CTA limit.
constexpr int kPanelSmemMax = 208 * 1024;

// Per column jj (q = jj & 1 selects one of two publication slots):
//  (a) each thread scans its own rows (fixed thread-to-row map, so no
//      barrier is needed after its own updates of the previous column); the
//      CTA reduces to one candidate, and publishes the candidate's value,
//      index and whole row in pub_*[q]; the owner of row jj publishes row jj.
//  cluster barrier (the only one per column)
//  (b) every CTA reads all 16 published candidates and candidate rows and
//      the published row jj (one round trip of distributed shared memory),
//      and makes the same pivot decision.
//  (c) row interchange and (d) scaling and rank-1 update of local rows.
// Only the pub_* slots are read remotely, never the tile, so the tile can be
// updated without a second barrier.  A slot written at column jj + 2 cannot
// race a remote read of it at column jj: the writer has passed the barrier
// of column jj + 1, which the reader only reaches after that read.
template <typename R>
__global__ void __launch_bounds__(kClusterThreads)
k_getf2_cluster(typename cx<R>::T* __restrict__ P, long lda, int m, int jb, int rpc, int* __restrict__ ipiv, int k0,
                int* __restrict__ info) {
  typedef typename cx<R>::T T;
  constexpr int kWarps = kClusterThreads / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // [jb][rpc], row index fastest
  __shared__ R pub_val[2];
  __shared__ int pub_idx[2];
  __shared__ T pub_row[2][kClusterNB];
  __shared__ T pub_jrow[2][kClusterNB];
  __shared__ R red_v[kWarps];
  __shared__ int red_i[kWarps];
  __shared__ T s_cand[kClusterCTAs][kClusterNB];
  __shared__ T s_jrow[kClusterNB];
  __shared__ T s_rp;  // the pivot's reciprocal, computed once per column
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = rank * rpc;
  const int rl = max(0, min(rpc, m - r0));

  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    tile[c * rpc + r] = P[(r0 + r) + (long)c * lda];
  }
  __syncthreads();  // the tile is complete before any thread reads another thread's elements
  // row 0 of the panel for column 0's publication (read remotely after the first cluster barrier)
  if (rank == 0 && tid < jb) pub_jrow[0][tid] = tile[tid * rpc];

  for (int jj = 0; jj < jb; ++jj) {
    const int q = jj & 1;
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
    if (warp == 0) {
      R v = (lane < kWarps) ? red_v[lane] : (R)-1;
      int i = (lane < kWarps) ? red_i[lane] : INT_MAX;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const R ov = __shfl_down_sync(0xffffffffu, v, off);
        const int oi = __shfl_down_sync(0xffffffffu, i, off);
        if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
      }
      v = __shfl_sync(0xffffffffu, v, 0);
      i = __shfl_sync(0xffffffffu, i, 0);
      if (lane == 0) { pub_val[q] = v; pub_idx[q] = i; }
      if (i != INT_MAX && lane < jb) pub_row[q][lane] = tile[lane * rpc + (i - r0)];
    }
    cluster.sync();

    // (b) all candidates, their rows and row jj from the cluster
    const int oj = jj / rpc, lj = jj - oj * rpc;
    {
      const int src = tid / kClusterNB, c = tid % kClusterNB;  // 512 threads = 16 CTAs x 32 columns
      if (c < jb) s_cand[src][c] = *cluster.map_shared_rank(&pub_row[q][c], src);
      if (tid < jb) s_jrow[tid] = *cluster.map_shared_rank(&pub_jrow[q][tid], oj);
    }
    R pmax = -1;
    int p = INT_MAX;
    if (lane < kClusterCTAs) {
      pmax = *cluster.map_shared_rank(&pub_val[q], lane);
      p = *cluster.map_shared_rank(&pub_idx[q], lane);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const R ov = __shfl_down_sync(0xffffffffu, pmax, off);
      const int oi = __shfl_down_sync(0xffffffffu, p, off);
      if (ov > pmax || (ov == pmax && oi < p)) { pmax = ov; p = oi; }
    }
    pmax = __shfl_sync(0xffffffffu, pmax, 0);
    p = __shfl_sync(0xffffffffu, p, 0);
    if (p == INT_MAX) p = jj;
    const int op = p / rpc;
    // one thread forms the pivot's reciprocal (in double precision three
    // divisions, each a long FP64-pipe sequence, so not once per thread)
    if (tid == 0 && pmax > 0) s_rp = c_recip(*cluster.map_shared_rank(&pub_row[q][jj], op));
    __syncthreads();  // s_cand, s_jrow and s_rp complete
    const bool swap = pmax > 0 && p != jj;
    const T* prow = s_cand[op];
    if (rank == 0 && tid == 0) {
      ipiv[k0 + jj] = k0 + p + 1;
      if (!(pmax > 0) && *info == 0) *info = k0 + jj + 1;
    }
    // (c) row jj becomes the pivot row (U row of this column)
    if (swap && rank == oj && tid < jb) tile[tid * rpc + lj] = prow[tid];
    // (d) scale below the pivot and update; the owner of row p takes old row jj
    if (pmax > 0) {
      const T rp = s_rp;
      for (int r = tid; r < rl; r += blockDim.x) {
        const int gr = r0 + r;
        if (gr <= jj) continue;
        if (swap && gr == p)
          for (int c = 0; c < jb; ++c) tile[c * rpc + r] = s_jrow[c];
        const T l = c_mul(tile[jj * rpc + r], rp);
        tile[jj * rpc + r] = l;
        // the rank-1 update in chunks of 8 columns with compile-time indices,
        // the chunk's loads issued back to back
#pragma unroll
        for (int c0 = 0; c0 < kClusterNB; c0 += 8) {
          if (c0 + 8 <= jj + 1 || c0 >= jb) continue;
          T u[8], a[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) {
              u[t] = prow[c];
              a[t] = tile[c * rpc + r];
            }
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) tile[c * rpc + r] = c_sub(a[t], c_mul(l, u[t]));
          }
        }
      }
    }
    // publish row jj + 1 for the next column (its owner thread updated it)
    if (jj + 1 < jb) {
      const int gr = jj + 1;
      if (gr >= r0 && gr < r0 + rl && ((gr - r0) % blockDim.x) == tid) {
        for (int c = 0; c < jb; ++c) pub_jrow[q ^ 1][c] = tile[c * rpc + (gr - r0)];
      }
    }
  }
  cluster.sync();  // no CTA leaves while another could still read its shared memory
  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    P[(r0 + r) + (long)c * lda] = tile[c * rpc + r];
  }
}

// Single-precision panel with pushed candidates.  The per-column exchange is
// the latency-critical step of the whole LU (n column steps in sequence), so
// it is done with the cluster's asynchronous copy engine instead of loads:
// every CTA packs one message (its candidate's value, index and row, and, if
// it owns row jj, row jj) and sends it with 16 bulk copies into slot [rank]
// of every CTA's receive buffer, each copy completing on the receiver's
// mbarrier.  A CTA then waits on its own mbarrier (bounded) and finds the
// pivot among 16 local messages: no cluster barrier and no remote loads per
// column, 16 bulk transfers instead of thousands of small DSMEM requests.
//
// Buffers alternate by column parity q.  Reuse is safe one step ahead: a CTA
// sends column jj + 2's message only after receiving everyone's column jj + 1
// message, which each CTA sends only after it has finished reading the
// column-jj slots (and its own column-jj copies have landed everywhere).  For
// the same reason a copy can only reach an mbarrier whose previous phase has
// completed.  The mbarrier of parity q is re-armed (one arrival with the
// expected bytes) right after its phase completes.
struct __align__(16) PanelMsg {
  float val;
  int idx;
  int pad[2];
  float2 cand[kClusterNB];  // the candidate row
  float2 jrow[kClusterNB];  // row jj, from its owner only
};
static_assert(sizeof(PanelMsg) % 16 == 0, "bulk copies move multiples of 16 bytes");
constexpr uint64_t kPanelWaitNs = 2000000000ull;  // 2 s
constexpr int kPanelTimeout = -1000;  // info value of a wait that ran out

__device__ __forceinline__ bool better(float v, int i, float bv, int bi) {
  return v > bv || (v == bv && i < bi);
}

// The warp's best candidate under `better` (largest value, smallest row on
// ties; values < 0 or NaN mean no candidate) in two redux instructions
// instead of ten dependent shuffles: non-negative floats order as their bit
// patterns, so the largest value is the largest key bits + 1 (0 = none), and
// the row is the smallest among the lanes holding that key.
__device__ __forceinline__ void warp_best(float& v, int& idx) {
  const unsigned key = (v >= 0.f) ? __float_as_uint(v) + 1u : 0u;
  const unsigned km = __reduce_max_sync(0xffffffffu, key);
  const unsigned im = __reduce_min_sync(0xffffffffu, key == km ? (unsigned)idx : 0xffffffffu);
  idx = (km == 0u) ? INT_MAX : (int)im;
  v = (km == 0u) ? -1.f : __uint_as_float(km - 1u);
}

__global__ void __launch_bounds__(kClusterThreads, 1)
k_getf2_cluster_push(float2* __restrict__ P, long lda, int m, int jb, int rpc, int* __restrict__ ipiv, int k0,
                     int* __restrict__ info) {
  constexpr int kWarps = kClusterThreads / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tile = reinterpret_cast<float2*>(smem_raw);  // [jb][rpc], row index fastest
  __shared__ PanelMsg sendbuf[2];
  __shared__ PanelMsg recv[2][kClusterCTAs];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ float red_v[kWarps];
  __shared__ int red_i[kWarps];
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = rank * rpc;
  const int rl = max(0, min(rpc, m - r0));
  constexpr uint32_t kMsgBytes = sizeof(PanelMsg);

  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    tile[c * rpc + r] = P[(r0 + r) + (long)c * lda];
  }
  if (tid == 0) {
    s_bad = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_expect_tx(&mbar[0], kClusterCTAs * kMsgBytes);
    if (jb > 1) mbar_expect_tx(&mbar[1], kClusterCTAs * kMsgBytes);
  }
  cluster.sync();  // barriers initialised and armed everywhere before any copy

  bool bad = false;
  for (int jj = 0; jj < jb; ++jj) {
    const int q = jj & 1;
    const int oj = jj / rpc, lj = jj - oj * rpc;
    // (a) this CTA's candidate for column jj (rows >= jj)
    float v = -1.f;
    int idx = INT_MAX;
    for (int r = tid; r < rl; r += blockDim.x) {
      if (r0 + r >= jj) {
        const float2 a = tile[jj * rpc + r];
        const float av = fabsf(a.x) + fabsf(a.y);
        if (better(av, r0 + r, v, idx)) { v = av; idx = r0 + r; }
      }
    }
    warp_best(v, idx);
    if (lane == 0) { red_v[warp] = v; red_i[warp] = idx; }
    __syncthreads();  // also orders every thread's column jj - 1 updates before the copies below
    if (warp == 0) {
      v = (lane < kWarps) ? red_v[lane] : -1.f;
      idx = (lane < kWarps) ? red_i[lane] : INT_MAX;
      warp_best(v, idx);
      // (b) pack and push the message
      PanelMsg& msg = sendbuf[q];
      if (lane == 0) { msg.val = v; msg.idx = idx; }
      if (lane < jb) {
        if (idx != INT_MAX) msg.cand[lane] = tile[lane * rpc + (idx - r0)];
        if (rank == oj) msg.jrow[lane] = tile[lane * rpc + lj];
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane < kClusterCTAs) {
        const uint32_t dst = mapa_shared(smem_addr(&recv[q][rank]), lane);
        const uint32_t bar = mapa_shared(smem_addr(&mbar[q]), lane);
        bulk_s2s_cluster(dst, smem_addr(&msg), kMsgBytes, bar);
      }
    }
    // (c) wait for the 16 messages of this column
    if (!mbar_wait_timed(&mbar[q], (jj >> 1) & 1, kPanelWaitNs)) bad = true;
    if (__syncthreads_or(bad)) {
      if (tid == 0) s_bad = 1;
      break;
    }
    if (tid == 0 && jj + 2 < jb) mbar_expect_tx(&mbar[q], kClusterCTAs * kMsgBytes);
    // (d) the pivot: every warp reduces the 16 local messages
    float pmax = (lane < kClusterCTAs) ? recv[q][lane].val : -1.f;
    int p = (lane < kClusterCTAs) ? recv[q][lane].idx : INT_MAX;
    warp_best(pmax, p);
    if (p == INT_MAX) p = jj;
    const int op = p / rpc;
    const float2* prow = recv[q][op].cand;
    const float2* jrow = recv[q][oj].jrow;
    const bool swap = pmax > 0.f && p != jj;
    if (rank == 0 && tid == 0) {
      ipiv[k0 + jj] = k0 + p + 1;
      if (!(pmax > 0.f) && *info == 0) *info = k0 + jj + 1;
    }
    // (e) row jj becomes the pivot row; the owner of row p takes old row jj
    if (swap && rank == oj && tid < jb) tile[tid * rpc + lj] = prow[tid];
    if (pmax > 0.f) {
      const float2 rp = c_recip(prow[jj]);
      for (int r = tid; r < rl; r += blockDim.x) {
        const int gr = r0 + r;
        if (gr <= jj) continue;
        if (swap && gr == p) {
          for (int c = 0; c < jb; ++c) tile[c * rpc + r] = jrow[c];
        }
        const float2 l = c_mul(tile[jj * rpc + r], rp);
        tile[jj * rpc + r] = l;
        // the rank-1 update in chunks of 8 columns with compile-time indices:
        // the chunk's 8 pivot-row and 8 own-row loads issue back to back (a
        // column-by-column loop waits on each load, the stores in between
        // keeping the compiler from hoisting the next loads)
#pragma unroll
        for (int c0 = 0; c0 < kClusterNB; c0 += 8) {
          if (c0 + 8 <= jj + 1 || c0 >= jb) continue;
          float2 u[8], a[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) {
              u[t] = prow[c];
              a[t] = tile[c * rpc + r];
            }
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) {
              a[t].x = fmaf(-l.x, u[t].x, fmaf(l.y, u[t].y, a[t].x));
              a[t].y = fmaf(-l.x, u[t].y, fmaf(-l.y, u[t].x, a[t].y));
              tile[c * rpc + r] = a[t];
            }
          }
        }
      }
    }
  }
  __syncthreads();
  if (s_bad) {
    if (rank == 0 && tid == 0) *info = kPanelTimeout;
  } else {
    for (int e = tid; e < rl * jb; e += blockDim.x) {
      const int r = e % rl, c = e / rl;
      P[(r0 + r) + (long)c * lda] = tile[c * rpc + r];
    }
  }
  cluster.sync();  // no CTA leaves while a copy into its shared memory could be pending
}

// Complex128 panel with pushed candidates, at most 16 columns (the width of
// the complex128 LU's panels when its updates run on the tensor cores): the
// exchange of k_getf2_cluster_push (per column one message per CTA, sent by
// 16 bulk copies, a bounded mbarrier wait; no cluster barrier and no remote
// loads per column) with the arithmetic of k_getf2_cluster<double>.  The
// message also carries the reciprocal of the candidate's entry in column jj,
// formed once by its sender (three FP64 divisions).  Reuse of the two message
// slots is safe for the reasons given above.
constexpr int kPanelNBZ = 16;
struct __align__(16) PanelMsgZ {
  double val;
  int idx;
  int pad;
  double2 rcp;
  double2 cand[kPanelNBZ];
  double2 jrow[kPanelNBZ];
};
static_assert(sizeof(PanelMsgZ) % 16 == 0, "bulk copies move multiples of 16 bytes");

// warp_best for double values: the non-negative doubles' 64-bit patterns
// (plus one, 0 = none) reduced as two 32-bit halves, then the smallest row
// among the lanes holding the largest key.
__device__ __forceinline__ void warp_best_z(double& v, int& idx) {
  const unsigned long long key = (v >= 0.0) ? (unsigned long long)__double_as_longlong(v) + 1ull : 0ull;
  const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)(key & 0xffffffffull);
  const unsigned hm = __reduce_max_sync(0xffffffffu, hi);
  const unsigned lm = __reduce_max_sync(0xffffffffu, hi == hm ? lo : 0u);
  const unsigned im = __reduce_min_sync(0xffffffffu, (hi == hm && lo == lm) ? (unsigned)idx : 0xffffffffu);
  const unsigned long long km = ((unsigned long long)hm << 32) | lm;
  idx = (km == 0ull) ? INT_MAX : (int)im;
  v = (km == 0ull) ? -1.0 : __longlong_as_double((long long)(km - 1ull));
}

__global__ void __launch_bounds__(kClusterThreads, 1)
k_getf2_cluster_push_z(double2* __restrict__ P, long lda, int m, int jb, int rpc, int* __restrict__ ipiv, int k0,
                       int* __restrict__ info) {
  constexpr int kWarps = kClusterThreads / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tile = reinterpret_cast<double2*>(smem_raw);  // [jb][rpc], row index fastest
  __shared__ PanelMsgZ sendbuf[2];
  __shared__ PanelMsgZ recv[2][kClusterCTAs];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ double red_v[kWarps];
  __shared__ int red_i[kWarps];
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = rank * rpc;
  const int rl = max(0, min(rpc, m - r0));
  constexpr uint32_t kMsgBytes = sizeof(PanelMsgZ);

  for (int e = tid; e < rl * jb; e += blockDim.x) {
    const int r = e % rl, c = e / rl;
    tile[c * rpc + r] = P[(r0 + r) + (long)c * lda];
  }
  if (tid == 0) {
    s_bad = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_expect_tx(&mbar[0], kClusterCTAs * kMsgBytes);
    if (jb > 1) mbar_expect_tx(&mbar[1], kClusterCTAs * kMsgBytes);
  }
  cluster.sync();  // barriers initialised and armed everywhere before any copy

  bool bad = false;
  for (int jj = 0; jj < jb; ++jj) {
    const int q = jj & 1;
    const int oj = jj / rpc, lj = jj - oj * rpc;
    // (a) this CTA's candidate for column jj (rows >= jj): |re| + |im|, first row on ties
    double v = -1.0;
    int idx = INT_MAX;
    for (int r = tid; r < rl; r += blockDim.x) {
      if (r0 + r >= jj) {
        const double2 a = tile[jj * rpc + r];
        const double av = fabs(a.x) + fabs(a.y);
        if (av > v || (av == v && r0 + r < idx)) { v = av; idx = r0 + r; }
      }
    }
    warp_best_z(v, idx);
    if (lane == 0) { red_v[warp] = v; red_i[warp] = idx; }
    __syncthreads();  // also orders every thread's column jj - 1 updates before the copies below
    if (warp == 0) {
      v = (lane < kWarps) ? red_v[lane] : -1.0;
      idx = (lane < kWarps) ? red_i[lane] : INT_MAX;
      warp_best_z(v, idx);
      // (b) pack and push the message
      PanelMsgZ& msg = sendbuf[q];
      if (lane == 0) {
        msg.val = v;
        msg.idx = idx;
        if (v > 0.0) msg.rcp = c_recip(tile[jj * rpc + (idx - r0)]);
      }
      if (lane < jb) {
        if (idx != INT_MAX) msg.cand[lane] = tile[lane * rpc + (idx - r0)];
        if (rank == oj) msg.jrow[lane] = tile[lane * rpc + lj];
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane < kClusterCTAs) {
        const uint32_t dst = mapa_shared(smem_addr(&recv[q][rank]), lane);
        const uint32_t bar = mapa_shared(smem_addr(&mbar[q]), lane);
        bulk_s2s_cluster(dst, smem_addr(&msg), kMsgBytes, bar);
      }
    }
    // (c) wait for the 16 messages of this column
    if (!mbar_wait_timed(&mbar[q], (jj >> 1) & 1, kPanelWaitNs)) bad = true;
    if (__syncthreads_or(bad)) {
      if (tid == 0) s_bad = 1;
      break;
    }
    if (tid == 0 && jj + 2 < jb) mbar_expect_tx(&mbar[q], kClusterCTAs * kMsgBytes);
    // (d) the pivot: every warp reduces the 16 local messages
    double pmax = (lane < kClusterCTAs) ? recv[q][lane].val : -1.0;
    int p = (lane < kClusterCTAs) ? recv[q][lane].idx : INT_MAX;
    warp_best_z(pmax, p);
    if (p == INT_MAX) p = jj;
    const int op = p / rpc;
    const double2* prow = recv[q][op].cand;
    const double2* jrow = recv[q][oj].jrow;
    const bool swap = pmax > 0.0 && p != jj;
    if (rank == 0 && tid == 0) {
      ipiv[k0 + jj] = k0 + p + 1;
      if (!(pmax > 0.0) && *info == 0) *info = k0 + jj + 1;
    }
    // (e) row jj becomes the pivot row; the owner of row p takes old row jj
    if (swap && rank == oj && tid < jb) tile[tid * rpc + lj] = prow[tid];
    if (pmax > 0.0) {
      const double2 rp = recv[q][op].rcp;
      for (int r = tid; r < rl; r += blockDim.x) {
        const int gr = r0 + r;
        if (gr <= jj) continue;
        if (swap && gr == p)
          for (int c = 0; c < jb; ++c) tile[c * rpc + r] = jrow[c];
        const double2 l = c_mul(tile[jj * rpc + r], rp);
        tile[jj * rpc + r] = l;
#pragma unroll
        for (int c0 = 0; c0 < kPanelNBZ; c0 += 8) {
          if (c0 + 8 <= jj + 1 || c0 >= jb) continue;
          double2 u[8], a[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) {
              u[t] = prow[c];
              a[t] = tile[c * rpc + r];
            }
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const int c = c0 + t;
            if (c > jj && c < jb) tile[c * rpc + r] = c_sub(a[t], c_mul(l, u[t]));
          }
        }
      }
    }
  }
  __syncthreads();
  if (s_bad) {
    if (rank == 0 && tid == 0) *info = kPanelTimeout;
  } else {
    for (int e = tid; e < rl * jb; e += blockDim.x) {
      const int r = e % rl, c = e / rl;
      P[(r0 + r) + (long)c * lda] = tile[c * rpc + r];
    }
  }
  cluster.sync();  // no CTA leaves while a copy into its shared memory could be pending
}

// Register-resident form of the pushed-candidate panel, for panels of at
// most 512 rows per CTA: each thread keeps its one row of the panel (32
// complex values) in registers for all 32 column steps.  The shared-memory
// form loads and stores every element of the trailing panel through shared
// memory at every column (about 60 shared-memory wavefronts per column per
// SM, the bound of its update); here the update is register FMAs with the
// pivot row read as broadcast 16-byte loads, and the owners of the candidate
// row and of row jj write their rows into the message themselves.  The
// candidate's owner also sends the reciprocal of its pivot value, so the
// other threads do no division.  Same pivot rule, message protocol and
// bounded waits as k_getf2_cluster_push.
struct __align__(16) PanelMsgR {
  float val;
  int idx;
  float2 rcp;               // 1 / candidate[jj] (from the candidate's owner)
  float2 cand[kClusterNB];  // the candidate row
  float2 jrow[kClusterNB];  // row jj, from its owner only
};
static_assert(sizeof(PanelMsgR) % 16 == 0, "bulk copies move multiples of 16 bytes");

__device__ __forceinline__ float2 pick32(const float2 (&a)[kClusterNB], int j) {
  float2 x = a[0];
#pragma unroll
  for (int c = 1; c < kClusterNB; ++c)
    if (c == j) x = a[c];
  return x;
}

// A panel row between registers and a 16-byte aligned message row, two
// complex values per 16-byte access.
__device__ __forceinline__ void store_row(float2* dst, const float2 (&a)[kClusterNB]) {
  float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int c = 0; c < kClusterNB / 2; ++c) d4[c] = make_float4(a[2 * c].x, a[2 * c].y, a[2 * c + 1].x, a[2 * c + 1].y);
}
__device__ __forceinline__ void load_row(float2 (&a)[kClusterNB], const float2* src) {
  const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
  for (int c = 0; c < kClusterNB / 2; ++c) {
    const float4 v = s4[c];
    a[2 * c] = make_float2(v.x, v.y);
    a[2 * c + 1] = make_float2(v.z, v.w);
  }
}

// The cluster has as many CTAs (up to 16) as the panel needs at one row per
// thread: ncta = ceil(m / 512), rpc = ceil(m / ncta).
__global__ void __launch_bounds__(kClusterThreads, 1)
k_getf2_cluster_reg(float2* __restrict__ P, long lda, int m, int jb, int rpc, int* __restrict__ ipiv, int k0,
                    int* __restrict__ info) {
  constexpr int kWarps = kClusterThreads / 32;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int ncta = (int)cluster.num_blocks();
  __shared__ PanelMsgR sendbuf[2];
  __shared__ PanelMsgR recv[2][kClusterCTAs];  // ncta <= 16 slots used
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ float red_v[kWarps];
  __shared__ int red_i[kWarps];
  __shared__ int s_bad;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r0 = rank * rpc;
  const int rl = max(0, min(rpc, m - r0));
  const bool own = tid < rl;
  const int gr = r0 + tid;
  constexpr uint32_t kMsgBytes = sizeof(PanelMsgR);
  float2 a[kClusterNB];
  {
    const float2* q = P + gr;  // a running pointer: no column address stays live through the steps
#pragma unroll
    for (int c = 0; c < kClusterNB; ++c, q += lda) a[c] = (own && c < jb) ? *q : make_float2(0.f, 0.f);
  }
  if (tid == 0) {
    s_bad = 0;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_expect_tx(&mbar[0], ncta * kMsgBytes);
    if (jb > 1) mbar_expect_tx(&mbar[1], ncta * kMsgBytes);
  }
  cluster.sync();  // barriers initialised and armed everywhere before any copy

  bool bad = false;
  // Fully unrolled: every column index below is a compile-time constant, so
  // the row stays in registers without selects and the update touches only
  // the columns right of jj.
#pragma unroll
  for (int jj = 0; jj < kClusterNB; ++jj) {
    if (jj >= jb) break;
    const int q = jj & 1;
    const int oj = jj / rpc;
    // (a) this CTA's candidate for column jj (rows >= jj), reduced by every warp
    const float2 x = pick32(a, jj);
    float v = (own && gr >= jj) ? fabsf(x.x) + fabsf(x.y) : -1.f;
    int idx = (own && gr >= jj) ? gr : INT_MAX;
    warp_best(v, idx);
    if (lane == 0) { red_v[warp] = v; red_i[warp] = idx; }
    __syncthreads();  // (the previous column's message slots were read before this barrier too)
    v = (lane < kWarps) ? red_v[lane] : -1.f;
    idx = (lane < kWarps) ? red_i[lane] : INT_MAX;
    warp_best(v, idx);
    // (b) the owners write the message: header and candidate row, row jj
    PanelMsgR& msg = sendbuf[q];
    if (idx == INT_MAX) {
      if (tid == 0) { msg.val = -1.f; msg.idx = INT_MAX; }
    } else if (own && gr == idx) {
      msg.val = v;
      msg.idx = idx;
      msg.rcp = (x.x != 0.f || x.y != 0.f) ? c_recip(x) : make_float2(0.f, 0.f);
      store_row(msg.cand, a);
    }
    if (own && gr == jj) {
      store_row(msg.jrow, a);
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (warp == 0 && lane < ncta) {
      const uint32_t dst = mapa_shared(smem_addr(&recv[q][rank]), lane);
      const uint32_t bar = mapa_shared(smem_addr(&mbar[q]), lane);
      bulk_s2s_cluster(dst, smem_addr(&msg), kMsgBytes, bar);
    }
    // (c) wait for the ncta messages of this column
    if (!mbar_wait_timed(&mbar[q], (jj >> 1) & 1, kPanelWaitNs)) bad = true;
    if (__syncthreads_or(bad)) {
      if (tid == 0) s_bad = 1;
      break;
    }
    if (tid == 0 && jj + 2 < jb) mbar_expect_tx(&mbar[q], ncta * kMsgBytes);
    // (d) the pivot: every warp reduces the ncta local messages
    float pmax = (lane < ncta) ? recv[q][lane].val : -1.f;
    int p = (lane < ncta) ? recv[q][lane].idx : INT_MAX;
    warp_best(pmax, p);
    if (p == INT_MAX) p = jj;
    const int op = p / rpc;
    const PanelMsgR& pm = recv[q][op];
    const bool swap = pmax > 0.f && p != jj;
    if (rank == 0 && tid == 0) {
      ipiv[k0 + jj] = k0 + p + 1;
      if (!(pmax > 0.f) && *info == 0) *info = k0 + jj + 1;
    }
    // (e) row jj becomes the pivot row; the owner of row p takes old row jj; update below jj
    if (own && swap && gr == jj) {
      load_row(a, pm.cand);
    } else if (own && swap && gr == p) {
      load_row(a, recv[q][oj].jrow);
    }
    if (pmax > 0.f && own && gr > jj) {
      const float2 rp = pm.rcp;
      const float2 l = c_mul(pick32(a, jj), rp);
#pragma unroll
      for (int c = 0; c < kClusterNB; ++c)
        if (c == jj) a[c] = l;
      // columns >= jb hold zeros in every row and in the pivot row and are never stored
      const float4* u4 = reinterpret_cast<const float4*>(pm.cand);
#pragma unroll
      for (int c2 = 0; c2 < kClusterNB / 2; ++c2) {
        if (2 * c2 + 1 > jj) {
          const float4 uu = u4[c2];
          if (2 * c2 > jj) {
            a[2 * c2].x = fmaf(-l.x, uu.x, fmaf(l.y, uu.y, a[2 * c2].x));
            a[2 * c2].y = fmaf(-l.x, uu.y, fmaf(-l.y, uu.x, a[2 * c2].y));
          }
          a[2 * c2 + 1].x = fmaf(-l.x, uu.z, fmaf(l.y, uu.w, a[2 * c2 + 1].x));
          a[2 * c2 + 1].y = fmaf(-l.x, uu.w, fmaf(-l.y, uu.z, a[2 * c2 + 1].y));
        }
        if ((c2 & 3) == 3) asm volatile("" ::: "memory");  // keep at most 8 columns of loads in flight
      }
    }
  }
  __syncthreads();
  if (s_bad) {
    if (rank == 0 && tid == 0) *info = kPanelTimeout;
  } else if (own) {
    float2* q = P + gr;
#pragma unroll
    for (int c = 0; c < kClusterNB; ++c, q += lda) {
      asm volatile("" : "+l"(q));  // computed here, not kept from the loads
      if (c < jb) *q = a[c];
    }
  }
  cluster.sync();  // no CTA leaves while a copy into its shared memory could be pending
}

template <typename R>
cudaError_t panel_cluster_smem(cudaStream_t st, typename cx<R>::T* P, long lda, int m, int jb, int* ipiv, int k0,
                               int* info) {
  typedef typename cx<R>::T T;
  if (jb > kClusterNB) return cudaErrorNotSupported;
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  const size_t smem = (size_t)rpc * jb * sizeof(T);
  static int attr_done[2] = {0, 0};
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  const int idx = sizeof(R) == 8 ? 1 : 0;
  if (smem > (size_t)kPanelSmemMax) return cudaErrorNotSupported;
  auto kern = k_getf2_cluster<R>;
  if (!attr_done[idx]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kPanelSmemMax);
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

// Single precision: the pushed-candidate panel (its tile plus the message
// buffers must fit one CTA's shared memory), else the loading panel.
constexpr int kPushStaticSmem = 20 * 1024;  // message buffers, barriers, reductions

template <>
cudaError_t panel_cluster<float>(cudaStream_t st, float2* P, long lda, int m, int jb, int* ipiv, int k0, int* info) {
  if (jb > kClusterNB) return cudaErrorNotSupported;
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  if (rpc <= kClusterThreads) {  // one row per thread: the register-resident panel
    cudaError_t e = cudaFuncSetAttribute(k_getf2_cluster_reg, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    // as few CTAs as hold the panel at one row per thread: shorter panels
    // (later in the factorisation) occupy fewer SMs and exchange fewer messages
    const int ncta = (m + kClusterThreads - 1) / kClusterThreads;
    const int rpcr = (m + ncta - 1) / ncta;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ncta, 1, 1);
    cfg.blockDim = dim3(kClusterThreads, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ncta;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_getf2_cluster_reg, P, lda, m, jb, rpcr, ipiv, k0, info);
  }
  const size_t smem = (size_t)rpc * jb * sizeof(float2);
  if (smem > (size_t)(kPanelSmemMax - kPushStaticSmem)) return panel_cluster_smem<float>(st, P, lda, m, jb, ipiv, k0, info);
  cudaError_t e = cudaFuncSetAttribute(k_getf2_cluster_push, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_getf2_cluster_push, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kPanelSmemMax - kPushStaticSmem);
  if (e != cudaSuccess) return e;
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
  return cudaLaunchKernelEx(&cfg, k_getf2_cluster_push, P, lda, m, jb, rpc, ipiv, k0, info);
}
// Double precision: the pushed-candidate panel for panels of at most 16
// columns whose tile fits beside its message buffers, else the loading panel.
template <>
cudaError_t panel_cluster<double>(cudaStream_t st, double2* P, long lda, int m, int jb, int* ipiv, int k0,
                                  int* info) {
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  const size_t smem = (size_t)rpc * jb * sizeof(double2);
  if (jb > kPanelNBZ || smem > (size_t)(kPanelSmemMax - kPushStaticSmem))
    return panel_cluster_smem<double>(st, P, lda, m, jb, ipiv, k0, info);
  cudaError_t e = cudaFuncSetAttribute(k_getf2_cluster_push_z, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_getf2_cluster_push_z, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kPanelSmemMax - kPushStaticSmem);
  if (e != cudaSuccess) return e;
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
  return cudaLaunchKernelEx(&cfg, k_getf2_cluster_push_z, P, lda, m, jb, rpc, ipiv, k0, info);
}


// Whether a 16-CTA cluster with the given dynamic shared memory can run here.
template <typename R>
bool panel_cluster_supported(int m, int jb) {
  typedef typename cx<R>::T T;
  static int cached[2] = {-1, -1};
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  const int idx = sizeof(R) == 8 ? 1 : 0;
  const int rpc = (m + kClusterCTAs - 1) / kClusterCTAs;
  if ((size_t)rpc * jb * sizeof(T) > (size_t)kPanelSmemMax) return false;
  if (cached[idx] < 0) {
    auto kern = k_getf2_cluster<R>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kPanelSmemMax);
    int ncl = 0;
    if (e == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kClusterCTAs, 1, 1);
      cfg.blockDim = dim3(kClusterThreads, 1, 1);
      cfg.dynamicSmemBytes = kPanelSmemMax;
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
template bool panel_cluster_supported<float>(int, int);
template bool panel_cluster_supported<double>(int, int);

// ---------------------------------------------------------------------------
// Triangular solves, one CTA per right-hand-side column (jb <= 256 rows):
// X = L^{-1} X (unit lower) or X = U^{-1} X (upper; multiplies by the
// reciprocal of each diagonal entry, computed for a whole sub-block at once).  The block is walked in sub-blocks of SB columns staged in
// shared memory by cp.async, the next sub-block in flight while the current
// one is used.  One warp solves the SB x SB diagonal part with shuffles (no
// CTA barrier per row), then every thread updates its own row with the SB
// new unknowns: two CTA barriers per sub-block instead of one or two per row.
// ---------------------------------------------------------------------------
constexpr int kTrsmBlock = 256;

template <typename T> struct TrsmSub;
template <> struct TrsmSub<float2> { static constexpr int SB = 32; };
template <> struct TrsmSub<double2> { static constexpr int SB = 16; };

template <typename T>
__device__ __forceinline__ void cp_elem(T* dst, const T* src, bool pred);
template <> __device__ __forceinline__ void cp_elem<float2>(float2* dst, const float2* src, bool pred) {
  cp_async8(dst, src, pred);
}
template <> __device__ __forceinline__ void cp_elem<double2>(double2* dst, const double2* src, bool pred) {
  cp_async16(dst, src, pred ? 16 : 0);
}

template <typename T>
__device__ __forceinline__ T shfl_c(T v, int src) {
  v.x = __shfl_sync(0xffffffffu, v.x, src);
  v.y = __shfl_sync(0xffffffffu, v.y, src);
  return v;
}

template <typename T, bool UPPER>
__device__ __forceinline__ void trsm_stage(T* buf, const T* __restrict__ A, long lda, int jb, int s, int tid) {
  constexpr int SB = TrsmSub<T>::SB;
  const int c0 = s * SB, w = min(SB, jb - c0);
  // lower: rows >= c0 are used; upper: rows < c0 + w
#pragma unroll 4
  for (int e = tid; e < SB * kTrsmBlock; e += kTrsmBlock) {
    const int r = e % kTrsmBlock, j = e / kTrsmBlock;
    const bool need = j < w && r < jb && (UPPER ? r < c0 + w : r >= c0);
    cp_elem<T>(buf + j * kTrsmBlock + r, need ? A + r + (long)(c0 + j) * lda : A, need);
  }
}

template <typename T, bool UPPER>
__global__ void __launch_bounds__(kTrsmBlock)
k_trsm_col(const T* __restrict__ A, long lda, int jb, T* __restrict__ X, long ldx) {
  constexpr int SB = TrsmSub<T>::SB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* bufs = reinterpret_cast<T*>(smem_raw);  // 2 x [SB][kTrsmBlock]
  __shared__ T x[kTrsmBlock];
  const int col = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* xc = X + (long)col * ldx;
  T zero;
  zero.x = 0; zero.y = 0;
  const int nsb = (jb + SB - 1) / SB;
  if (tid < jb) x[tid] = xc[tid];
  int s = UPPER ? nsb - 1 : 0;
  const int iters = UPPER ? s + 1 : nsb - s;
  trsm_stage<T, UPPER>(bufs, A, lda, jb, s, tid);
  cp_async_commit();
  for (int it = 0; it < iters; ++it, s += (UPPER ? -1 : 1)) {
    T* cur = bufs + (it & 1) * SB * kTrsmBlock;
    cp_async_wait<0>();
    __syncthreads();  // sub-block landed; x and the other buffer are free
    if (it + 1 < iters)
      trsm_stage<T, UPPER>(bufs + ((it + 1) & 1) * SB * kTrsmBlock, A, lda, jb, s + (UPPER ? -1 : 1), tid);
    cp_async_commit();
    const int c0 = s * SB, w = min(SB, jb - c0);
    if (warp == 0) {
      T xr = (lane < w) ? x[c0 + lane] : zero;
      if (!UPPER) {
        for (int j = 0; j < w; ++j) {
          const T xj = shfl_c(xr, j);
          if (lane > j && lane < w) xr = c_sub(xr, c_mul(cur[j * kTrsmBlock + c0 + lane], xj));
        }
      } else {
        // reciprocals of the diagonal, all lanes at once, off the serial chain
        T rd = zero;
        if (lane < w) rd = c_recip(cur[lane * kTrsmBlock + c0 + lane]);
        for (int j = w - 1; j >= 0; --j) {
          if (lane == j) xr = c_mul(xr, rd);
          const T xj = shfl_c(xr, j);
          if (lane < j) xr = c_sub(xr, c_mul(cur[j * kTrsmBlock + c0 + lane], xj));
        }
      }
      if (lane < w) x[c0 + lane] = xr;
    }
    __syncthreads();
    const bool mine = UPPER ? (tid < c0) : (tid >= c0 + w && tid < jb);
    if (mine) {
      T acc = x[tid];
      for (int j = 0; j < w; ++j) acc = c_sub(acc, c_mul(cur[j * kTrsmBlock + tid], x[c0 + j]));
      x[tid] = acc;
    }
  }
  __syncthreads();
  if (tid < jb) xc[tid] = x[tid];
}

template <typename R>
cudaError_t trsm_cols(cudaStream_t st, bool upper, const typename cx<R>::T* A, long lda, int jb,
                      typename cx<R>::T* X, long ldx, int ncols) {
  typedef typename cx<R>::T T;
  if (jb > kTrsmBlock) return cudaErrorInvalidValue;
  if (ncols <= 0 || jb <= 0) return cudaSuccess;
  const int smem = 2 * TrsmSub<T>::SB * kTrsmBlock * (int)sizeof(T);
  auto kern = upper ? k_trsm_col<T, true> : k_trsm_col<T, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  kern<<<ncols, kTrsmBlock, smem, st>>>(A, lda, jb, X, ldx);
  return cudaGetLastError();
}
template cudaError_t trsm_cols<float>(cudaStream_t, bool, const float2*, long, int, float2*, long, int);
template cudaError_t trsm_cols<double>(cudaStream_t, bool, const double2*, long, int, double2*, long, int);

// ---------------------------------------------------------------------------
// Inverses of the diagonal blocks (order <= 256) of the complex64 factors:
// the unit-lower L_bb or the upper U_bb.  One CTA per (8 columns of the
// inverse, block): thread r holds row r of those 8 columns in registers and
// the block is walked in 32-wide sub-blocks (forward for L, backward for U):
//  1. the warp holding the sub-block's rows solves with its 32 x 32 diagonal
//     triangle (staged in shared memory; the new rows broadcast by shuffles);
//  2. the solved rows go to shared memory and every thread below (L) or
//     above (U) them subtracts their product with its own row segment of the
//     triangle, all threads at once.
// Eight columns per CTA keep the walk short (the lower inverses sit on the
// LU's critical path, one block after each outer panel) while every CTA
// still reads its part of the triangle once for eight columns.
// ---------------------------------------------------------------------------
constexpr int kInvRows = 256, kInvSub = 32, kInvW = 8;

template <bool UPPER>
__global__ void __launch_bounds__(kInvRows)
k_trinv(const float2* __restrict__ A, long lda, int nb, int ntot, float2* __restrict__ X, long ldx) {
  __shared__ __align__(16) float2 Ts[kInvSub][kInvSub];  // the diagonal triangle, Ts[j][i] = T(c0 + i, c0 + j)
  __shared__ __align__(16) float2 Xs[kInvSub][kInvW];    // the sub-block's solved rows
  const int q = blockIdx.x, b = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int jbb = min(nb, ntot - b * nb);
  const int qc = q * kInvW;
  if (qc >= jbb) return;
  A += (long)b * nb * (1 + lda);
  X += (long)b * nb * ldx;
  const int r = tid;
  float2 x[kInvW];
#pragma unroll
  for (int c = 0; c < kInvW; ++c) x[c] = make_float2(r == qc + c ? 1.f : 0.f, 0.f);
  const int ns = (jbb + kInvSub - 1) / kInvSub, sq = qc / kInvSub;
  for (int it = 0; it < (UPPER ? sq + 1 : ns - sq); ++it) {
    const int s = UPPER ? sq - it : sq + it;
    const int c0 = s * kInvSub, w = min(kInvSub, jbb - c0);
    __syncthreads();  // the previous sub-block's Ts and Xs are no longer read
    for (int e = tid; e < kInvSub * kInvSub; e += kInvRows) {
      const int i = e % kInvSub, j = e / kInvSub;
      Ts[j][i] = (i < w && j < w) ? A[(c0 + i) + (long)(c0 + j) * lda] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (warp == s) {
      if (!UPPER) {
        for (int j = 0; j < w; ++j) {
          const float2 l = Ts[j][lane];
          const bool upd = lane > j && lane < w;
#pragma unroll
          for (int c = 0; c < kInvW; ++c) {
            const float2 xj = make_float2(__shfl_sync(0xffffffffu, x[c].x, j), __shfl_sync(0xffffffffu, x[c].y, j));
            if (upd) x[c] = c_sub(x[c], c_mul(l, xj));
          }
        }
      } else {
        const float2 rd = (lane < w) ? c_recip(Ts[lane][lane]) : make_float2(0.f, 0.f);
        for (int j = w - 1; j >= 0; --j) {
          if (lane == j) {
#pragma unroll
            for (int c = 0; c < kInvW; ++c) x[c] = c_mul(x[c], rd);
          }
          const float2 u = Ts[j][lane];
          const bool upd = lane < j;
#pragma unroll
          for (int c = 0; c < kInvW; ++c) {
            const float2 xj = make_float2(__shfl_sync(0xffffffffu, x[c].x, j), __shfl_sync(0xffffffffu, x[c].y, j));
            if (upd) x[c] = c_sub(x[c], c_mul(u, xj));
          }
        }
      }
      float4* d4 = reinterpret_cast<float4*>(&Xs[lane][0]);
#pragma unroll
      for (int c2 = 0; c2 < kInvW / 2; ++c2) d4[c2] = make_float4(x[2 * c2].x, x[2 * c2].y, x[2 * c2 + 1].x, x[2 * c2 + 1].y);
    }
    __syncthreads();
    const bool mine = UPPER ? r < c0 : (r >= c0 + w && r < jbb);
    if (mine) {
      const float2* trow = A + r + (long)c0 * lda;
#pragma unroll 8
      for (int j = 0; j < w; ++j) {
        const float2 t = trow[(long)j * lda];
        const float4* xs4 = reinterpret_cast<const float4*>(&Xs[j][0]);
#pragma unroll
        for (int c2 = 0; c2 < kInvW / 2; ++c2) {
          const float4 v = xs4[c2];
          x[2 * c2].x = fmaf(-t.x, v.x, fmaf(t.y, v.y, x[2 * c2].x));
          x[2 * c2].y = fmaf(-t.x, v.y, fmaf(-t.y, v.x, x[2 * c2].y));
          x[2 * c2 + 1].x = fmaf(-t.x, v.z, fmaf(t.y, v.w, x[2 * c2 + 1].x));
          x[2 * c2 + 1].y = fmaf(-t.x, v.w, fmaf(-t.y, v.z, x[2 * c2 + 1].y));
        }
      }
    }
  }
  if (r < jbb) {
    float2* o = X + r + (long)qc * ldx;
#pragma unroll
    for (int c = 0; c < kInvW; ++c)
      if (qc + c < jbb) o[(long)c * ldx] = x[c];
  }
}

template <typename R>
cudaError_t trsm_inverse_blocks(cudaStream_t st, bool upper, const typename cx<R>::T* A, long lda, int n, int nb,
                                typename cx<R>::T* X, long ldx, int nblk_first, int nblk) {
  static_assert(sizeof(R) == 4, "the diagonal-block inverses serve the complex64 LU");
  if (nb > kInvRows) return cudaErrorInvalidValue;
  if (nblk <= 0) return cudaSuccess;
  const long k0 = (long)nblk_first * nb;
  const dim3 grid((nb + kInvW - 1) / kInvW, nblk);
  if (upper)
    k_trinv<true><<<grid, kInvRows, 0, st>>>(A + k0 + k0 * lda, lda, nb, n - (int)k0, X + (long)nblk_first * nb * ldx, ldx);
  else
    k_trinv<false><<<grid, kInvRows, 0, st>>>(A + k0 + k0 * lda, lda, nb, n - (int)k0, X + (long)nblk_first * nb * ldx, ldx);
  return cudaGetLastError();
}

template cudaError_t trsm_inverse_blocks<float>(cudaStream_t, bool, const float2*, long, int, int, float2*, long, int,
                                                int);

}  // namespace hg
