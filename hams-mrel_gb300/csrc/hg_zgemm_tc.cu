// Complex128 products C -= A B on the tensor cores, FP64-accurate, by exact
// operand slicing: the plain form's LU updates (U12 = L11^-1 A12 and
// A22 -= L21 U12 of ZGETRF, AssbMatx.f90:111), its blocked solves and its
// field-point sums, which otherwise run on GB300's thin FP64 pipes.
//
// The scheme (Ozaki, Ogita, Oishi and Rump, Numer. Algorithms 59 (2012)
// 95-118), as in hg_resid_tc.cu but with both operands in double precision:
//  - complex as real: [Ar | Ai] (m x 2k) times, per complex column j of B, the
//    real output column 2j = [Br_j ; -Bi_j] and the imaginary one 2j + 1 =
//    [Bi_j ; Br_j]; the two outputs of a complex column sit side by side, so
//    a 64-column output tile is 32 complex columns of C;
//  - row i of A is scaled by 2^-e_i (|entries| < 1/2) and written as eight
//    balanced 7-bit digits, a = 2^e_i sum_s d_s 2^-7s, |d_s| <= 64, to 2^-57
//    of twice the row's largest entry; complex column j of B the same with
//    2^f_j.  The digits come from the 53-bit significand by integer shifts
//    and masks, not FP64 arithmetic;
//  - the 36 digit pairs with s + t <= 9 (dropped terms below 2^-63 each) go
//    into eight level accumulators (L = s + t) in TMEM.  Every partial sum of
//    one level over the 512 real K of one pass (k <= 256) stays within
//    8 * 64^2 * 512 = 2^24, so the FP32 accumulation of BF16 digit products
//    (kind::f16) is exact;
//  - after the pass the drains fold the eight exact level sums into two
//    64-bit integers (levels 2..5 and 6..9, by Horner in base 2^7), release
//    TMEM, and update C with one rounding of the product into double
//    precision and one of the subtraction.
// Error: per term the digits' truncation, 2^-57 of the row's and the
// column's largest entries, plus the two roundings: 2.6e-16 .. 5.7e-16 of
// |c| + sum |a||b| measured, the accuracy of a double-precision product.
//
// Kernel (k_zoz_gemm): persistent, one CTA per SM, output tiles of 128 rows x
// 64 real columns in M-fastest order (the CTAs working at one time share B's
// digit tiles and all of A's in L2).  576 threads: warp 0 the TMA producer
// (eight A digit tiles 128 x 32 and eight B digit tiles 64 x 32 per 32-deep
// stage, 64-byte rows, 64-byte swizzle; two stages of 96 KB), warp 1 the MMA
// issuer (72 instructions M = 128, N = 64, K = 16 per stage), warps 2..17 the
// drains (four per TMEM lane quarter, 16 columns each).  A tile's double
// precision update of C runs while the MMAs of the next tile fill the
// accumulators.  Every wait is bounded in time.
#include <algorithm>
#include <mutex>
#include <cuda_bf16.h>

#include "hg_common.cuh"
#include "hg_linalg.cuh"
#include "hg_oz.cuh"

namespace hg {
namespace {

constexpr int kZD = 8;          // digits per operand
constexpr int kZTM = 128;       // rows of a tile
constexpr int kZTN = 64;        // real output columns of a tile (32 complex)
constexpr int kZStages = 2;
constexpr int kZMaxK = 256;     // complex K of one slicing pass: 512 real, one drain
constexpr uint32_t kZATile = kZTM * kOzKS * 2;  // 8 KB
constexpr uint32_t kZBTile = kZTN * kOzKS * 2;  // 4 KB
constexpr uint32_t kZStageBytes = kZD * (kZATile + kZBTile);
constexpr int kZEpiWarps = 16;
constexpr int kZThreads = 64 + 32 * kZEpiWarps;
constexpr int kZEpiCols = kZTN / (kZEpiWarps / 4);  // 16 real = 8 complex columns per thread
constexpr uint32_t kZTmemCols = 512;                // 8 levels x 64 columns
constexpr int kZTimeout = -1000;
constexpr size_t kZSmem = (size_t)kZStages * kZStageBytes + 1024;
constexpr uint32_t kZIdesc = oz_idesc(kZTM, kZTN);
static_assert(kZD * kZTN <= (int)kZTmemCols, "level accumulators exceed TMEM");

// BF16 bits of a small integer (|d| <= 128): exact through the FP32 magic
// constant 1.5 * 2^23, whose low 16 bits are zero for such values.
__device__ __forceinline__ uint16_t oz_bf16_int(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return (uint16_t)(__float_as_uint(f) >> 16);
}

// Largest |v| of a set as the bit pattern of a non-negative double (bit
// patterns of non-negative doubles order as their values).
__device__ __forceinline__ unsigned long long oz_abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// Scale exponent from the bit pattern of the largest |v|: e with
// max * 2^-e in [0.25, 0.5); 0 for zero; subnormal maxima take the smallest
// normal exponent.
__device__ __forceinline__ int oz_exp_bits(unsigned long long amax) {
  if (amax == 0) return 0;
  const int ef = (int)(amax >> 52);
  return (ef == 0 ? 1 : ef) - 1021;
}

// Eight balanced 7-bit digits of v 2^-e (|v| 2^-e < 1/2) as BF16 bits, d[0]
// the leading one: X = v 2^(56-e) rounded to an integer from v's
// significand, then d_8 .. d_2 in [-64, 63] from the bottom and d_1 the rest
// (|d_1| <= 64), X = sum_s d_s 2^(56-7s).
__device__ __forceinline__ void oz_digits_d(double v, int e, uint16_t (&d)[kZD]) {
  const long long b = __double_as_longlong(v);
  const int ef = (int)((b >> 52) & 0x7FF);
  long long X = 0;
  if (ef != 0) {
    const long long mant = (b & 0xFFFFFFFFFFFFFll) | (1ll << 52);
    const int sh = ef - 1075 + 56 - e;  // X = mant 2^sh, sh <= 2 since |v| 2^-e < 1/2
    if (sh >= 0)
      X = mant << sh;
    else if (sh > -62)
      X = (mant + (1ll << (-sh - 1))) >> (-sh);
    if (b < 0) X = -X;
  }
#pragma unroll
  for (int s = kZD - 1; s >= 1; --s) {
    const int r = (int)(X & 127);
    const int dd = r >= 64 ? r - 128 : r;
    d[s] = oz_bf16_int(dd);
    X = (X - dd) >> 7;
  }
  d[0] = oz_bf16_int((int)X);
}

// v 2^sc for a double v: the exponent field moved by integer addition while
// the result stays normal (exact), ldexp otherwise.
__device__ __forceinline__ double oz_scale2(double v, int sc) {
  const long long b = __double_as_longlong(v);
  const int ef = (int)((b >> 52) & 0x7FF);
  if (ef != 0 && ef + sc > 0 && ef + sc < 0x7FF) return __longlong_as_double(b + ((long long)sc << 52));
  return ldexp(v, sc);
}

// A's digits: [kZD][mp][kp] BF16 rows (K fastest), row i holding Ar(i, :) at
// 0..k-1 and Ai(i, :) at k..2k-1, zero beyond (rows m..mp-1, K 2k..kp-1);
// ex[i] the row's exponent.  The operand is A (m x k, A[i + p lda]) or, with
// TRANS, the transpose of the k x m matrix A (A[p + i lda]: its rows are A's
// columns).  One CTA per 32 rows: their largest entries first, then 32 x 32
// tiles through shared memory (transposed for A, direct for TRANS), so that
// the reads of A and the digit writes are both coalesced.
template <bool TRANS>
__global__ void __launch_bounds__(256) k_zoz_slice_a(int m, int k, int mp, int kp, const double2* __restrict__ A,
                                                     long lda, int* __restrict__ ex, uint16_t* __restrict__ D) {
  __shared__ double2 t[32][33];
  __shared__ unsigned long long red[8][32];
  __shared__ int es[32];
  const int i0 = blockIdx.x * 32, tx = threadIdx.x, ty = threadIdx.y;
  if (TRANS) {  // a warp per row, lanes along its contiguous entries
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + r;
      unsigned long long amax = 0;
      if (i < m)
        for (int p = tx; p < k; p += 32) {
          const double2 a = A[p + (long)i * lda];
          amax = max(amax, max(oz_abs_bits(a.x), oz_abs_bits(a.y)));
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) amax = max(amax, __shfl_xor_sync(0xffffffffu, amax, o));
      if (tx == 0) {
        const int e = oz_exp_bits(amax);
        es[r] = e;
        if (i < mp) ex[i] = e;
      }
    }
    __syncthreads();
  } else {
    unsigned long long amax = 0;
    const int i = i0 + tx;
    if (i < m)
      for (int p = ty; p < k; p += 8) {
        const double2 a = A[i + (long)p * lda];
        amax = max(amax, max(oz_abs_bits(a.x), oz_abs_bits(a.y)));
      }
    red[ty][tx] = amax;
    __syncthreads();
    if (ty == 0) {
      for (int r = 1; r < 8; ++r) amax = max(amax, red[r][tx]);
      const int e = oz_exp_bits(amax);
      es[tx] = e;
      if (i < mp) ex[i] = e;
    }
    __syncthreads();
  }
  const size_t slice = (size_t)mp * kp;
  for (int p0 = 0; p0 < k; p0 += 32) {
    for (int r = ty; r < 32; r += 8) {
      if (TRANS) {  // t[r][tx] = op(i0 + r, p0 + tx)
        const int i = i0 + r, p = p0 + tx;
        t[r][tx] = (i < m && p < k) ? A[p + (long)i * lda] : make_double2(0.0, 0.0);
      } else {  // t[r][tx] = op(i0 + tx, p0 + r)
        const int i = i0 + tx, p = p0 + r;
        t[r][tx] = (i < m && p < k) ? A[i + (long)p * lda] : make_double2(0.0, 0.0);
      }
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + r, p = p0 + tx;
      if (i >= mp || p >= k) continue;
      const double2 a = TRANS ? t[r][tx] : t[tx][r];
      uint16_t dr[kZD], di[kZD];
      oz_digits_d(a.x, es[r], dr);
      oz_digits_d(a.y, es[r], di);
      uint16_t* row = D + (size_t)i * kp;
#pragma unroll
      for (int s = 0; s < kZD; ++s) {
        row[s * slice + p] = dr[s];
        row[s * slice + k + p] = di[s];
      }
    }
    __syncthreads();
  }
  const int w = kp - 2 * k;
  if (w > 0)
    for (int e = ty * 32 + tx; e < kZD * 32 * w; e += 256) {
      const int c = e % w, r = (e / w) % 32, s = e / (w * 32);
      if (i0 + r < mp) D[s * slice + (size_t)(i0 + r) * kp + 2 * k + c] = 0;
    }
}

// B's digits: [kZD][np][kp] BF16 rows, row 2j the real output column of
// complex column j ([Br_j ; -Bi_j]), row 2j + 1 the imaginary one
// ([Bi_j ; Br_j]), zero beyond; fx[j] the column's exponent.  One warp per
// complex column (B's columns are contiguous).
__global__ void __launch_bounds__(256) k_zoz_slice_b(int k, int n, int np, int kp, const double2* __restrict__ B,
                                                     long ldb, int* __restrict__ fx, uint16_t* __restrict__ G) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (2 * j >= np) return;
  const bool live = j < n;
  const double2* col = B + (long)j * ldb;
  unsigned long long amax = 0;
  if (live)
    for (int p = lane; p < k; p += 32) {
      const double2 y = col[p];
      amax = max(amax, max(oz_abs_bits(y.x), oz_abs_bits(y.y)));
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = max(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  const int f = oz_exp_bits(amax);
  if (lane == 0) fx[j] = f;
  const size_t slice = (size_t)np * kp;
  uint16_t* re = G + (size_t)(2 * j) * kp;
  uint16_t* im = re + kp;
  for (int p = lane; p < k; p += 32) {
    uint16_t dr[kZD], di[kZD];
    const double2 y = live ? col[p] : make_double2(0.0, 0.0);
    oz_digits_d(y.x, f, dr);
    oz_digits_d(y.y, f, di);
#pragma unroll
    for (int s = 0; s < kZD; ++s) {
      re[s * slice + p] = dr[s];
      re[s * slice + k + p] = (uint16_t)(di[s] ^ 0x8000u);
      im[s * slice + p] = di[s];
      im[s * slice + k + p] = dr[s];
    }
  }
  for (int q = 2 * k + lane; q < kp; q += 32)
#pragma unroll
    for (int s = 0; s < kZD; ++s) {
      re[s * slice + q] = 0;
      im[s * slice + q] = 0;
    }
}

__global__ void __launch_bounds__(kZThreads, 1)
k_zoz_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int m, int n, int mp,
           int np, int kp, const int* __restrict__ ex, const int* __restrict__ fx, double2* __restrict__ C, long ldc,
           int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kZStages], empty[kZStages], tfull, tempty, drain;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  unsigned char* smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = mp / kZTM, ntiles = mt * (np / kZTN);
  const int nst = kp / kOzKS;  // kp <= 512: one drain per tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < kZStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&tfull, 1);
    mbar_init(&tempty, kZEpiWarps);
    mbar_init(&drain, 1);
    s_abort = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                 "r"(kZTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  oz_fence_before();
  __syncthreads();
  oz_fence_after();
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: per stage eight A digit tiles and eight B digit tiles ----
      int s = 0;
      uint32_t ph = 0;
      int issued[kZStages];
      uint32_t last_ph[kZStages];
      for (int i = 0; i < kZStages; ++i) { issued[i] = 0; last_ph[i] = 0; }
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int row0 = (tile % mt) * kZTM, col0 = (tile / mt) * kZTN;
        for (int kt = 0; kt < nst; ++kt) {
          if (!oz_wait(&empty[s], ph ^ 1, &s_abort)) { ok = false; break; }
          unsigned char* st = smem + (size_t)s * kZStageBytes;
          mbar_expect_tx(&full[s], kZStageBytes);
          const int kx = kt * kOzKS;
          for (int d = 0; d < kZD; ++d) {
            oz_tma_2d(st + d * kZATile, &ta, kx, d * mp + row0, &full[s]);
            oz_tma_2d(st + kZD * kZATile + d * kZBTile, &tb, kx, d * np + col0, &full[s]);
          }
          issued[s] = 1;
          last_ph[s] = ph;
          if (++s == kZStages) { s = 0; ph ^= 1; }
        }
      }
      if (!ok) {
        for (int i = 0; i < kZStages; ++i) {
          if (!issued[i]) continue;
          const uint64_t t0 = global_ns();
          while (!mbar_try_wait(&full[i], last_ph[i]) && global_ns() - t0 < kOzWaitNs) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: the 36 digit pairs of levels 2..9 into eight accumulators ----
      int s = 0;
      uint32_t ph = 0, tph = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        if (!oz_wait(&tempty, tph ^ 1, &s_abort)) break;  // the previous tile is drained
        tph ^= 1;
        oz_fence_after();
        for (int q = 0; q < nst; ++q) {
          if (!oz_wait(&full[s], ph, &s_abort)) { ok = false; break; }
          oz_fence_after();
          const uint32_t abase = smem_addr(smem + (size_t)s * kZStageBytes);
          const uint32_t bbase = abase + kZD * kZATile;
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 of K = 32 bytes of the 64-byte row
#pragma unroll
            for (int L = 2; L <= kZD + 1; ++L) {
              const uint32_t d = tmem + (uint32_t)((L - 2) * kZTN);
#pragma unroll
              for (int sa = 1; sa <= kZD; ++sa) {
                const int tb_ = L - sa;
                if (tb_ < 1 || tb_ > kZD) continue;
                const uint32_t acc = (q == 0 && kk == 0 && sa == 1) ? 0u : 1u;
                oz_mma(d, sw64_desc(abase + (sa - 1) * kZATile + off), sw64_desc(bbase + (tb_ - 1) * kZBTile + off),
                       kZIdesc, acc);
              }
            }
          }
          oz_commit(&empty[s]);
          if (++s == kZStages) { s = 0; ph ^= 1; }
        }
        if (ok) oz_commit(&tfull);
      }
      oz_commit(&drain);
      const uint64_t t0 = global_ns();
      while (!mbar_try_wait(&drain, 0) && global_ns() - t0 < kOzWaitNs) {
      }
    }
  } else {
    // ---- drains: warps 2..17, TMEM lane quarter q = warp % 4, 16 columns each ----
    const int qd = warp & 3, cb = (warp - 2) >> 2;
    const uint32_t tq = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(cb * kZEpiCols);
    uint32_t tph = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      const int row0 = (tile % mt) * kZTM, col0 = (tile / mt) * kZTN;
      const bool w = oz_wait(&tfull, tph, &s_abort);
      tph ^= 1;
      if (!__all_sync(0xffffffffu, w)) break;
      oz_fence_after();
      // the exact level sums a_L (integers, |a_L| <= 2^24) folded into
      // T_hi = sum_{L=2..5} a_L 2^(7(5-L)) and T_lo = sum_{L=6..9} a_L 2^(7(9-L))
      long long th[kZEpiCols], tl[kZEpiCols];
#pragma unroll
      for (int c = 0; c < kZEpiCols; ++c) { th[c] = 0; tl[c] = 0; }
#pragma unroll
      for (int L = 2; L <= kZD + 1; ++L) {
        uint32_t v[16];
        oz_ld16(tq + (uint32_t)((L - 2) * kZTN), v);
        oz_ld_wait();
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const long long a = (long long)__float2int_rn(__uint_as_float(v[c]));
          if (L <= 5)
            th[c] = th[c] * 128 + a;
          else
            tl[c] = tl[c] * 128 + a;
        }
      }
      oz_fence_before();
      __syncwarp();
      if (lane == 0) oz_arrive(&tempty);  // the next tile's MMAs may start
      // C -= 2^(e_i + f_j - 35) (T_hi + T_lo 2^-28): both words exact in double
      // precision (|T| < 2^46), one rounding of their sum by an FMA, the power
      // of two by the exponent field, one rounding of the subtraction
      const int row = row0 + qd * 32 + lane;
      if (row < m) {
        const int e = ex[row];
        const int jc0 = (col0 >> 1) + cb * (kZEpiCols / 2);
#pragma unroll
        for (int c = 0; c < kZEpiCols / 2; ++c) {
          const int jc = jc0 + c;
          if (jc >= n) break;
          const int sc = e + fx[jc] - 35;
          double2* p = C + row + (long)jc * ldc;
          double2 cv = *p;
          cv.x -= oz_scale2(fma((double)tl[2 * c], 0x1p-28, (double)th[2 * c]), sc);
          cv.y -= oz_scale2(fma((double)tl[2 * c + 1], 0x1p-28, (double)th[2 * c + 1]), sc);
          *p = cv;
        }
      }
    }
  }
  oz_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    oz_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kZTmemCols) : "memory");
  }
  if (threadIdx.x == 0 && s_abort) atomicExch(status, kZTimeout);
}

struct ZozLayout {
  int mp, np, kp;
  size_t a_off, b_off, ex_off, fx_off, total;
  ZozLayout(int m, int n, int k) {
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    mp = (m + kZTM - 1) / kZTM * kZTM;
    np = (2 * n + kZTN - 1) / kZTN * kZTN;
    kp = (2 * k + kOzKS - 1) / kOzKS * kOzKS;
    a_off = 0;
    b_off = a_off + up((size_t)kZD * mp * kp * 2);
    ex_off = b_off + up((size_t)kZD * np * kp * 2);
    fx_off = ex_off + up((size_t)mp * sizeof(int));
    total = fx_off + up((size_t)(np / 2) * sizeof(int));
  }
};

int g_z_sms = 0;

}  // namespace

bool zgemm_tc_supported() {
  static int cached = -1;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (cached < 0) cached = oz_device_supported(&g_z_sms) ? 1 : 0;
  return cached == 1;
}

size_t zgemm_tc_work_bytes(int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  return ZozLayout(m, n, std::min(k, kZMaxK)).total;
}

cudaError_t zgemm_tc(cudaStream_t st, int m, int n, int k, const double2* A, long lda, const double2* B, long ldb,
                     double2* C, long ldc, void* ws, size_t ws_bytes, int* status, bool transa) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if (!zgemm_tc_supported()) return cudaErrorNotSupported;
  if (!ws || ws_bytes < zgemm_tc_work_bytes(m, n, k) || (reinterpret_cast<uintptr_t>(ws) & 255u))
    return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_zoz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZSmem);
  if (e != cudaSuccess) return e;
  char* w = static_cast<char*>(ws);
  // inner dimension in passes of at most 256 (the exactness bound of one
  // drain group holds per pass; each pass is a complete update of C)
  for (int k0 = 0; k0 < k; k0 += kZMaxK) {
    const int kc = std::min(kZMaxK, k - k0);
    const ZozLayout lw(m, n, kc);
    uint16_t* Ad = reinterpret_cast<uint16_t*>(w + lw.a_off);
    uint16_t* Bd = reinterpret_cast<uint16_t*>(w + lw.b_off);
    int* ex = reinterpret_cast<int*>(w + lw.ex_off);
    int* fx = reinterpret_cast<int*>(w + lw.fx_off);
    if (transa)
      k_zoz_slice_a<true><<<lw.mp / 32, dim3(32, 8), 0, st>>>(m, kc, lw.mp, lw.kp, A + k0, lda, ex, Ad);
    else
      k_zoz_slice_a<false><<<lw.mp / 32, dim3(32, 8), 0, st>>>(m, kc, lw.mp, lw.kp, A + (long)k0 * lda, lda, ex, Ad);
    k_zoz_slice_b<<<(lw.np / 2 + 7) / 8, 256, 0, st>>>(kc, n, lw.np, lw.kp, B + k0, ldb, fx, Bd);
    CUtensorMap ma, mb;
    if (!oz_map(&ma, Ad, lw.kp, kZD * lw.mp, kZTM) || !oz_map(&mb, Bd, lw.kp, kZD * lw.np, kZTN))
      return cudaErrorNotSupported;
    const int ntiles = (lw.mp / kZTM) * (lw.np / kZTN);
    const int grid = std::min(ntiles, g_z_sms > 0 ? g_z_sms : 152);
    k_zoz_gemm<<<grid, kZThreads, kZSmem, st>>>(ma, mb, m, n, lw.mp, lw.np, lw.kp, ex, fx, C, ldc, status);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace hg
