// Complex single-precision GEMM for wide products: the LU trailing update
// A22 -= L21 U12 (inner dimension 32, the panel width) and the normal-equation
// product A^T A of the irregular-frequency form.
//
// Tile 128 x 64 outputs per CTA, 256 threads (8 warps): warp w owns columns
// 8w..8w+7 and lane l rows {2l, 2l+1, 64+2l, 65+2l}, 32 complex accumulators
// per thread.  Operand tiles (32 deep) arrive in shared memory by cp.async,
// two stages in flight when K > 32.  When K <= 32 (the LU update) there is a
// single stage and the CTA also prefetches its C tile into shared memory
// together with A and B, so the read of C overlaps the multiply; two CTAs
// share an SM so that one CTA's stores overlap the other's arithmetic.
#include <mutex>
#include "hg_linalg.cuh"
#include "hg_tma.cuh"

namespace hg {
namespace {

constexpr int kBM = 128, kBN = 64, kBK = 32, kThreads = 256;
constexpr int kBPitch = 33;  // B tile stored [column][k], padded row
constexpr size_t kATileBytes = (size_t)kBK * kBM * sizeof(float2);
constexpr size_t kBTileBytes = (size_t)kBN * kBPitch * sizeof(float2);
constexpr size_t kStageBytes = kATileBytes + kBTileBytes;
constexpr size_t kCTileBytes = (size_t)kBN * kBM * sizeof(float2);
constexpr size_t kSmemSmallK = kStageBytes + kCTileBytes;  // 115200
constexpr size_t kSmemLargeK = 2 * kStageBytes;            // 99328

// One 32-deep stage: As[l][i] (i fastest) for op(A) rows m0.., Bs[j][l].
template <bool TA, bool VEC>
__device__ __forceinline__ void load_stage(float2* As, float2* Bs, const float2* __restrict__ A, long lda,
                                           const float2* __restrict__ B, long ldb, int m, int n, int k, int m0,
                                           int n0, int k0, int tid) {
  if (!TA) {
    if (VEC) {
#pragma unroll
      for (int it = 0; it < kBK * kBM / 2 / kThreads; ++it) {
        const int e = tid + it * kThreads;
        const int i = (e % (kBM / 2)) * 2, l = e / (kBM / 2);
        const int gm = m0 + i, gk = k0 + l;
        int bytes = 0;
        if (gk < k) bytes = (gm + 1 < m) ? 16 : (gm < m ? 8 : 0);
        cp_async16(As + l * kBM + i, bytes ? A + gm + (long)gk * lda : A, bytes);
      }
    } else {
#pragma unroll
      for (int it = 0; it < kBK * kBM / kThreads; ++it) {
        const int e = tid + it * kThreads;
        const int i = e % kBM, l = e / kBM;
        const int gm = m0 + i, gk = k0 + l;
        const bool ok = gm < m && gk < k;
        cp_async8(As + l * kBM + i, ok ? A + gm + (long)gk * lda : A, ok);
      }
    }
  } else {
#pragma unroll
    for (int it = 0; it < kBK * kBM / kThreads; ++it) {
      const int e = tid + it * kThreads;
      const int l = e % kBK, i = e / kBK;
      const int gm = m0 + i, gk = k0 + l;
      const bool ok = gm < m && gk < k;
      cp_async8(As + l * kBM + i, ok ? A + gk + (long)gm * lda : A, ok);
    }
  }
#pragma unroll
  for (int it = 0; it < kBK * kBN / kThreads; ++it) {
    const int e = tid + it * kThreads;
    const int l = e % kBK, j = e / kBK;
    const int gk = k0 + l, gn = n0 + j;
    const bool ok = gn < n && gk < k;
    cp_async8(Bs + j * kBPitch + l, ok ? B + gk + (long)gn * ldb : B, ok);
  }
}

template <bool VEC>
__device__ __forceinline__ void load_ctile(float2* Cs, const float2* __restrict__ C, long ldc, int m, int n, int m0,
                                           int n0, int tid) {
  if (VEC) {
#pragma unroll 4
    for (int it = 0; it < kBM * kBN / 2 / kThreads; ++it) {
      const int e = tid + it * kThreads;
      const int i = (e % (kBM / 2)) * 2, j = e / (kBM / 2);
      const int gm = m0 + i, gn = n0 + j;
      int bytes = 0;
      if (gn < n) bytes = (gm + 1 < m) ? 16 : (gm < m ? 8 : 0);
      cp_async16(Cs + j * kBM + i, bytes ? C + gm + (long)gn * ldc : C, bytes);
    }
  } else {
#pragma unroll 4
    for (int it = 0; it < kBM * kBN / kThreads; ++it) {
      const int e = tid + it * kThreads;
      const int i = e % kBM, j = e / kBM;
      const int gm = m0 + i, gn = n0 + j;
      const bool ok = gm < m && gn < n;
      cp_async8(Cs + j * kBM + i, ok ? C + gm + (long)gn * ldc : C, ok);
    }
  }
}

// acc[r][c] += sum_l As[l][row r] * Bs[col c][l]; rows r = 2*lane + (r & 1) +
// 64 * (r >> 1), columns 8 * warp + c.
__device__ __forceinline__ void compute_stage(const float2* As, const float2* Bs, int lane, int warp,
                                              float (&acr)[4][8], float (&aci)[4][8]) {
  const float2* bcol = Bs + warp * 8 * kBPitch;
#pragma unroll 2
  for (int l = 0; l < kBK; ++l) {
    float ar[4], ai[4], br[8], bi[8];
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const float4 v = *reinterpret_cast<const float4*>(As + l * kBM + g * 64 + lane * 2);
      ar[2 * g] = v.x; ai[2 * g] = v.y; ar[2 * g + 1] = v.z; ai[2 * g + 1] = v.w;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const float2 b = bcol[c * kBPitch + l];
      br[c] = b.x; bi[c] = b.y;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        acr[r][c] = fmaf(ar[r], br[c], acr[r][c]);
        acr[r][c] = fmaf(-ai[r], bi[c], acr[r][c]);
        aci[r][c] = fmaf(ar[r], bi[c], aci[r][c]);
        aci[r][c] = fmaf(ai[r], br[c], aci[r][c]);
      }
  }
}

__device__ __forceinline__ float2 axpby(float2 alpha, float re, float im, float2 beta, float2 o) {
  float2 r;
  r.x = alpha.x * re - alpha.y * im + (beta.x * o.x - beta.y * o.y);
  r.y = alpha.x * im + alpha.y * re + (beta.x * o.y + beta.y * o.x);
  return r;
}

template <bool TA, bool VEC, bool KSMALL>
__global__ void __launch_bounds__(kThreads, 2)
k_cgemm_wide(int m, int n, int k, float2 alpha, const float2* __restrict__ A, long lda,
             const float2* __restrict__ B, long ldb, float2 beta, float2* __restrict__ C, long ldc) {
  extern __shared__ __align__(16) unsigned char smem[];
  float2* As0 = reinterpret_cast<float2*>(smem);
  float2* Bs0 = reinterpret_cast<float2*>(smem + kATileBytes);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const bool zb = (beta.x == 0.f && beta.y == 0.f);
  float acr[4][8], aci[4][8];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 8; ++c) { acr[r][c] = 0.f; aci[r][c] = 0.f; }

  const float2* Cs = nullptr;
  if (KSMALL) {
    float2* Cw = reinterpret_cast<float2*>(smem + kStageBytes);
    load_stage<TA, VEC>(As0, Bs0, A, lda, B, ldb, m, n, k, m0, n0, 0, tid);
    cp_async_commit();
    if (!zb) load_ctile<VEC>(Cw, C, ldc, m, n, m0, n0, tid);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    compute_stage(As0, Bs0, lane, warp, acr, aci);
    cp_async_wait<0>();
    __syncthreads();
    Cs = Cw;
  } else {
    float2* As1 = reinterpret_cast<float2*>(smem + kStageBytes);
    float2* Bs1 = reinterpret_cast<float2*>(smem + kStageBytes + kATileBytes);
    const int nk = (k + kBK - 1) / kBK;
    load_stage<TA, VEC>(As0, Bs0, A, lda, B, ldb, m, n, k, m0, n0, 0, tid);
    cp_async_commit();
    for (int s = 0; s < nk; ++s) {
      const bool odd = (s & 1) != 0;
      if (s + 1 < nk)
        load_stage<TA, VEC>(odd ? As0 : As1, odd ? Bs0 : Bs1, A, lda, B, ldb, m, n, k, m0, n0, (s + 1) * kBK, tid);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      compute_stage(odd ? As1 : As0, odd ? Bs1 : Bs0, lane, warp, acr, aci);
      __syncthreads();
    }
  }

  // Epilogue: C = alpha * acc + beta * C.
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int col = warp * 8 + c, gn = n0 + col;
    if (gn >= n) continue;
    float2* ccol = C + (long)gn * ldc;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      const int row = g * 64 + lane * 2, gm = m0 + row;
      float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
      if (!zb) {
        if (KSMALL) {
          o = *reinterpret_cast<const float4*>(Cs + col * kBM + row);
        } else if (VEC && gm + 1 < m) {
          o = *reinterpret_cast<const float4*>(ccol + gm);
        } else {
          if (gm < m) { const float2 t = ccol[gm]; o.x = t.x; o.y = t.y; }
          if (gm + 1 < m) { const float2 t = ccol[gm + 1]; o.z = t.x; o.w = t.y; }
        }
      }
      const float2 r0 = axpby(alpha, acr[2 * g][c], aci[2 * g][c], beta, make_float2(o.x, o.y));
      const float2 r1 = axpby(alpha, acr[2 * g + 1][c], aci[2 * g + 1][c], beta, make_float2(o.z, o.w));
      if (VEC && gm + 1 < m) {
        *reinterpret_cast<float4*>(ccol + gm) = make_float4(r0.x, r0.y, r1.x, r1.y);
      } else {
        if (gm < m) ccol[gm] = r0;
        if (gm + 1 < m) ccol[gm + 1] = r1;
      }
    }
  }
}

template <bool TA, bool VEC, bool KSMALL>
cudaError_t launch_wide(cudaStream_t st, int m, int n, int k, float2 alpha, const float2* A, long lda,
                        const float2* B, long ldb, float2 beta, float2* C, long ldc) {
  auto kern = k_cgemm_wide<TA, VEC, KSMALL>;
  const size_t smem = KSMALL ? kSmemSmallK : kSmemLargeK;
  // Set on every call: the attribute belongs to the current device.
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((m + kBM - 1) / kBM, (n + kBN - 1) / kBN, 1);
  kern<<<grid, kThreads, smem, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Skinny products, N <= 48 (the blocked triangular solves' updates
// B2 -= L21 X1 with all right-hand sides at once): 32 rows x CW = 8*CPT
// columns per CTA, 512 threads: one row x CPT columns each, the two halves
// of the CTA taking the two halves of every 32-deep stage and adding their
// sums in shared memory at the end.  The triangular solves' updates give
// at most ~190 such tiles, so an SM holds one CTA and its time is the
// solve's latency: sixteen warps instead of eight halve the instructions
// each warp issues.  Small tiles give enough CTAs to fill the GPU without
// splitting K across CTAs.
// ---------------------------------------------------------------------------
// Four stages in flight (80 KB of dynamic shared memory at 48 columns): the
// products this kernel serves (a 256-deep block of L or U times the
// right-hand sides) read their A block once from HBM, so the copies in
// flight per SM, not the FMAs, set their speed.
constexpr int kSRows = 32, kSK = 32, kSThreads = 512, kSMaxCW = 48, kSStages = 4;
// Row stride of the B stage in shared memory: CW + 2 complex, so that the
// 32 consecutive k of one column that a warp copies land on 8 bank pairs
// (4-way) instead of one (32-way at the bare 48-column stride), and rows
// stay 16-byte aligned for the paired reads.
template <int CPT> constexpr int skinny_bstride() { return 8 * CPT + 2; }

template <int CPT, bool VEC>
__device__ __forceinline__ void skinny_stage(float2* As, float2* Bs, const float2* __restrict__ A, long lda,
                                             const float2* __restrict__ B, long ldb, int m, int n, int k, int m0,
                                             int k0, int tid) {
  constexpr int CW = 8 * CPT;
  if (VEC) {
#pragma unroll
    for (int it = 0; it < kSK * kSRows / 2 / kSThreads; ++it) {
      const int e = tid + it * kSThreads;
      const int i = (e % (kSRows / 2)) * 2, l = e / (kSRows / 2);
      const int gm = m0 + i, gk = k0 + l;
      int bytes = 0;
      if (gk < k) bytes = (gm + 1 < m) ? 16 : (gm < m ? 8 : 0);
      cp_async16(As + l * kSRows + i, bytes ? A + gm + (long)gk * lda : A, bytes);
    }
  } else {
#pragma unroll
    for (int it = 0; it < kSK * kSRows / kSThreads; ++it) {
      const int e = tid + it * kSThreads;
      const int i = e % kSRows, l = e / kSRows;
      const int gm = m0 + i, gk = k0 + l;
      const bool ok = gm < m && gk < k;
      cp_async8(As + l * kSRows + i, ok ? A + gm + (long)gk * lda : A, ok);
    }
  }
  for (int e = tid; e < kSK * CW; e += kSThreads) {
    const int l = e % kSK, c = e / kSK;
    const int gk = k0 + l;
    const bool ok = c < n && gk < k;
    cp_async8(Bs + l * skinny_bstride<CPT>() + c, ok ? B + gk + (long)c * ldb : B, ok);
  }
}

template <int CPT, bool VEC>
__global__ void __launch_bounds__(kSThreads)
k_cgemm_skinny(int m, int n, int k, float2 alpha, const float2* __restrict__ A, long lda,
               const float2* __restrict__ B, long ldb, float2 beta, float2* __restrict__ C, long ldc) {
  constexpr int BST = skinny_bstride<CPT>();
  extern __shared__ __align__(16) float2 s_skinny[];
  float2* As = s_skinny;                            // [kSStages][kSK * kSRows]
  float2* Bs = s_skinny + kSStages * kSK * kSRows;  // [kSStages][kSK * BST]
  const int tid = threadIdx.x, tx = tid & 31, cg = (tid >> 5) & 7, kh = tid >> 8;
  const int m0 = blockIdx.x * kSRows;
  float ar[CPT], ai[CPT];
#pragma unroll
  for (int j = 0; j < CPT; ++j) { ar[j] = 0.f; ai[j] = 0.f; }
  const int nst = (k + kSK - 1) / kSK;
#pragma unroll
  for (int s = 0; s < kSStages - 1; ++s) {
    if (s < nst)
      skinny_stage<CPT, VEC>(As + s * kSK * kSRows, Bs + s * kSK * BST, A, lda, B, ldb, m, n, k, m0, s * kSK, tid);
    cp_async_commit();
  }
  for (int s = 0; s < nst; ++s) {
    const int b = s % kSStages;
    cp_async_wait<kSStages - 2>();
    __syncthreads();  // stage s landed; the buffer of stage s - 1 is free again
    const int sn = s + kSStages - 1;
    if (sn < nst)
      skinny_stage<CPT, VEC>(As + (sn % kSStages) * kSK * kSRows, Bs + (sn % kSStages) * kSK * BST, A, lda, B, ldb,
                             m, n, k, m0, sn * kSK, tid);
    cp_async_commit();
    const float2* as = As + b * kSK * kSRows;
    const float2* bs = Bs + b * kSK * BST + cg * CPT;
#pragma unroll 4
    for (int l = kh * (kSK / 2); l < (kh + 1) * (kSK / 2); ++l) {
      const float2 a = as[l * kSRows + tx];
#pragma unroll
      for (int j = 0; j < CPT; j += 2) {
        const float4 bb = *reinterpret_cast<const float4*>(bs + l * BST + j);
        ar[j] = fmaf(a.x, bb.x, ar[j]);
        ar[j] = fmaf(-a.y, bb.y, ar[j]);
        ai[j] = fmaf(a.x, bb.y, ai[j]);
        ai[j] = fmaf(a.y, bb.x, ai[j]);
        ar[j + 1] = fmaf(a.x, bb.z, ar[j + 1]);
        ar[j + 1] = fmaf(-a.y, bb.w, ar[j + 1]);
        ai[j + 1] = fmaf(a.x, bb.w, ai[j + 1]);
        ai[j + 1] = fmaf(a.y, bb.z, ai[j + 1]);
      }
    }
  }
  // the upper half's sums join the lower half's (the stage buffers are free
  // once every copy has landed and every thread has left the loop)
  cp_async_wait<0>();
  __syncthreads();
  float2* red = s_skinny;  // [CPT][8 column groups][32 rows]
  if (kh == 1) {
#pragma unroll
    for (int j = 0; j < CPT; ++j) red[(j * 8 + cg) * 32 + tx] = make_float2(ar[j], ai[j]);
  }
  __syncthreads();
  if (kh == 1) return;
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    const float2 o = red[(j * 8 + cg) * 32 + tx];
    ar[j] += o.x;
    ai[j] += o.y;
  }
  const int row = m0 + tx;
  if (row >= m) return;
  const bool zb = (beta.x == 0.f && beta.y == 0.f);
#pragma unroll
  for (int j = 0; j < CPT; ++j) {
    const int col = cg * CPT + j;
    if (col < n) {
      float2* c = C + row + (long)col * ldc;
      const float2 o = zb ? make_float2(0.f, 0.f) : *c;
      *c = axpby(alpha, ar[j], ai[j], beta, o);
    }
  }
}

template <int CPT, bool VEC>
cudaError_t launch_skinny_v(cudaStream_t st, int m, int n, int k, float2 alpha, const float2* A, long lda,
                            const float2* B, long ldb, float2 beta, float2* C, long ldc) {
  constexpr size_t smem = (size_t)kSStages * kSK * (kSRows + skinny_bstride<CPT>()) * sizeof(float2);
  static bool done[64] = {false};
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64 || !done[dev]) {
      e = cudaFuncSetAttribute(k_cgemm_skinny<CPT, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      if (dev >= 0 && dev < 64) done[dev] = true;
    }
  }
  const dim3 grid((m + kSRows - 1) / kSRows);
  k_cgemm_skinny<CPT, VEC><<<grid, kSThreads, smem, st>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return cudaGetLastError();
}

template <int CPT>
cudaError_t launch_skinny(cudaStream_t st, bool vec, int m, int n, int k, float2 alpha, const float2* A, long lda,
                          const float2* B, long ldb, float2 beta, float2* C, long ldc) {
  if (vec) return launch_skinny_v<CPT, true>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return launch_skinny_v<CPT, false>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

}  // namespace

cudaError_t cgemm_skinny(cudaStream_t st, int m, int n, int k, float2 alpha, const float2* A, long lda,
                         const float2* B, long ldb, float2 beta, float2* C, long ldc) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (n > kSMaxCW) return cudaErrorInvalidValue;
  const bool vec = (reinterpret_cast<uintptr_t>(A) % 16 == 0) && (lda % 2 == 0);
  const int per = (n + 7) / 8;
  if (per <= 2) return launch_skinny<2>(st, vec, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  if (per <= 4) return launch_skinny<4>(st, vec, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return launch_skinny<6>(st, vec, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

cudaError_t cgemm_wide(cudaStream_t st, bool transa, int m, int n, int k, float2 alpha, const float2* A, long lda,
                       const float2* B, long ldb, float2 beta, float2* C, long ldc) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  // 16-byte accesses to A (untransposed) and C need 16-byte aligned columns.
  const bool vec = (reinterpret_cast<uintptr_t>(C) % 16 == 0) && (ldc % 2 == 0) &&
                   (transa || ((reinterpret_cast<uintptr_t>(A) % 16 == 0) && (lda % 2 == 0)));
  const bool small = k <= kBK;
#define HG_WIDE(TA, V, KS) return launch_wide<TA, V, KS>(st, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)
  if (transa) {
    if (vec) { if (small) HG_WIDE(true, true, true); HG_WIDE(true, true, false); }
    if (small) HG_WIDE(true, false, true);
    HG_WIDE(true, false, false);
  }
  if (vec) { if (small) HG_WIDE(false, true, true); HG_WIDE(false, true, false); }
  if (small) HG_WIDE(false, false, true);
  HG_WIDE(false, false, false);
#undef HG_WIDE
}

}  // namespace hg
