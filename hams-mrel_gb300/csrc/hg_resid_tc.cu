// FP64-accurate residual products on the tensor cores by exact operand
// slicing: out = b + sign * A y for the mixed form's complex64 matrix A
// (m x k, exact in single precision) and complex128 y, b (k x nc, m x nc),
// the refinement residual r = b - A x of hg_resid.cu's exact mode.
//
// The scheme is that of Ozaki, Ogita, Oishi and Rump ("Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012) 95-118):
//  - complex as real: out_re = [Ar | Ai] [yr; -yi], out_im = [Ar | Ai] [yi; yr],
//    one real product of m x 2k by 2k x 2nc;
//  - each row i of [Ar | Ai] is scaled by 2^-e_i (|entries| < 1) and cut into
//    six balanced 7-bit digits, a = 2^e_i sum_s d_s 2^-7s with integers
//    |d_s| <= 128, to 2^-43 of the row's largest entry; each column pair j of
//    y the same with 2^f_j (y's 53 bits to 2^-43 of the column's largest);
//  - the digit products sum_k d_s g_t are integers, and every partial sum of
//    one level L = s + t (at most six pairs) over 128 real K stays below
//    6 * 128^2 * 128 < 2^24, so the tensor cores' FP32 accumulation of BF16
//    digits (kind::f16) is exact; the 21 pairs with s + t <= 7 (dropped
//    terms below 2^-49) go into six level accumulators in TMEM;
//  - every 128 K the levels are drained: each exact integer times 2^-7L is
//    added into a double-float (two FP32 words, TwoSum) per output, and the
//    K-range's sum times 2^(e_i + f_j) is written in double precision; a last
//    kernel adds the K ranges and b in double precision.
// Error: the digits' remainders, below 2^-43 of a row's (column's) largest
// entry each, summed over the inner dimension: ~1e-12 of sum |a||y| on rows
// whose entries fall off over five orders of magnitude (measured), against
// ~1e-14 for the double-float SIMT kernel; below the refinement's 1e-10.
//
// Kernel layout (k_oz_gemm): one CTA per (128 rows
// of A, range of K), 576 threads: warp 0 one TMA producer (six A digit tiles
// 128 x 32 and six y digit tiles 80 x 32, 64-byte rows, 64-byte swizzle, per
// 32-deep stage, two stages of 78 KB), warp 1 one MMA issuer (42 instructions
// M = 128, N = 80, K = 16 per stage), warps 2..17 the drains (four per TMEM
// lane quarter, 20 columns each).  Every wait is bounded in time.
#include <algorithm>
#include <mutex>
#include <cuda_bf16.h>

#include "hg_common.cuh"
#include "hg_linalg.cuh"
#include "hg_oz.cuh"

namespace hg {
namespace {

constexpr int kOzD = 6;                  // digits per operand
constexpr int kOzTM = 128;               // rows of A per CTA
constexpr int kOzTN = 80;                // output columns: 2 nc <= 80
constexpr int kOzGroup = 4;              // stages between drains: 128 real K
constexpr int kOzKUnit = kOzKS * kOzGroup;
constexpr int kOzStages = 2;
constexpr uint32_t kOzATile = kOzTM * kOzKS * 2;  // 8 KB
constexpr uint32_t kOzBTile = kOzTN * kOzKS * 2;  // 5 KB
constexpr uint32_t kOzStageBytes = kOzD * (kOzATile + kOzBTile);
constexpr int kOzEpiWarps = 16;
constexpr int kOzThreads = 64 + 32 * kOzEpiWarps;
constexpr int kOzEpiCols = kOzTN / (kOzEpiWarps / 4);  // 20
constexpr uint32_t kOzTmemCols = 512;                  // 6 levels x 80 columns used
constexpr int kOzTimeout = -1000;
constexpr size_t kOzSmem = (size_t)kOzStages * kOzStageBytes + 1024;
constexpr uint32_t kOzIdesc = oz_idesc(kOzTM, kOzTN);

// Largest |re|, |im| of each row of A: a thread per row over 128 columns
// (coalesced across the warp's consecutive rows), the column ranges combined
// by atomicMax on the bits (non-negative floats order as their bit patterns;
// rmax zeroed beforehand).
constexpr int kOzMaxCols = 128;
__global__ void k_oz_row_max(int m, int k, const float2* __restrict__ A, long lda, unsigned* __restrict__ rmax) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, p0 = blockIdx.y * kOzMaxCols;
  if (i >= m) return;
  float amax = 0.f;
  const int p1 = min(k, p0 + kOzMaxCols);
  for (int p = p0; p < p1; ++p) {
    const float2 a = A[i + (long)p * lda];
    amax = fmaxf(amax, fmaxf(fabsf(a.x), fabsf(a.y)));
  }
  atomicMax(rmax + i, __float_as_uint(amax));
}

__global__ void k_oz_row_exp(int m, const unsigned* __restrict__ rmax, int* __restrict__ ex) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) ex[i] = oz_exp((double)__uint_as_float(rmax[i]));
}

// Balanced digits of x (|x| < 1, exact in FP32 after the power-of-two
// scaling): d_s = rint(128 x_(s-1)), x_s = 128 x_(s-1) - d_s in [-1/2, 1/2],
// all steps exact; |d_1| <= 128, |d_s| <= 64 after it (BF16-exact integers),
// the remainder below 2^-43 and unbiased.
__device__ __forceinline__ void oz_digits_f(float x, __nv_bfloat16 (&d)[kOzD]) {
#pragma unroll
  for (int s = 0; s < kOzD; ++s) {
    x *= 128.f;
    const float t = rintf(x);
    d[s] = __float2bfloat16_rn(t);
    x -= t;
  }
}

// A's digits: [kOzD][mp][kp] BF16 rows (K fastest), row i of digit s holding
// Ar(i, :) at 0..k-1 and Ai(i, :) at k..2k-1; rows m..mp-1 and K 2k..kp-1 are
// zero.  A 32 x 32 complex tile per CTA, transposed in shared memory so that
// both the reads of A and the digit writes are coalesced.
__global__ void k_oz_slice_a(int m, int k, int mp, int kp, const float2* __restrict__ A, long lda,
                             const int* __restrict__ ex, __nv_bfloat16* __restrict__ D) {
  __shared__ float2 t[32][33];
  const int i0 = blockIdx.x * 32, p0 = blockIdx.y * 32, tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, p = p0 + r;
    t[r][tx] = (i < m && p < k) ? A[i + (long)p * lda] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  const size_t slice = (size_t)mp * kp;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, p = p0 + tx;
    if (i >= mp || p >= k) continue;
    const float2 a = t[tx][r];
    const float sc = (i < m) ? ldexpf(1.f, -ex[i]) : 0.f;
    __nv_bfloat16 dr[kOzD], di[kOzD];
    oz_digits_f(a.x * sc, dr);
    oz_digits_f(a.y * sc, di);
    __nv_bfloat16* row = D + (size_t)i * kp;
#pragma unroll
    for (int s = 0; s < kOzD; ++s) {
      row[s * slice + p] = dr[s];
      row[s * slice + k + p] = di[s];
    }
  }
}

// Zero the K padding 2k..kp-1 of every row of every digit of A.
__global__ void k_oz_zero_kpad(int mp, int k, int kp, __nv_bfloat16* __restrict__ D) {
  const int w = kp - 2 * k;
  const long total = (long)kOzD * mp * w;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e % w);
    const long r = e / w;  // digit * mp + row
    D[r * kp + 2 * k + c] = __float2bfloat16_rn(0.f);
  }
}

// y's digits: [kOzD][kOzTN][kp] BF16 rows: row j < nc the real output column
// j ([yr_j ; -yi_j]), row nc + j the imaginary one ([yi_j ; yr_j]), the other
// rows zero.  One CTA per output row; the column exponent f_j from the
// largest |re|, |im| of y_j (the same for rows j and nc + j).
__global__ void k_oz_slice_y(int k, int nc, int kp, const double2* __restrict__ Y, long ldy, int* __restrict__ fx,
                             __nv_bfloat16* __restrict__ G) {
  const int r = blockIdx.x;  // 0 .. kOzTN - 1
  const int j = r < nc ? r : r - nc;
  const bool im = r >= nc;
  const bool live = r < 2 * nc;
  __shared__ double red[32];
  double amax = 0.0;
  if (live)
    for (int p = threadIdx.x; p < k; p += blockDim.x) {
      const double2 y = Y[p + (long)j * ldy];
      amax = fmax(amax, fmax(fabs(y.x), fabs(y.y)));
    }
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = amax;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const int f = oz_exp(red[0]);
  if (threadIdx.x == 0) fx[r] = live ? f : 0;
  const double sc = ldexp(1.0, -f);
  const size_t slice = (size_t)kOzTN * kp;
  __nv_bfloat16* row = G + (size_t)r * kp;
  for (int q = threadIdx.x; q < kp; q += blockDim.x) {
    double x = 0.0;
    if (live && q < 2 * k) {
      const int p = q < k ? q : q - k;
      const double2 y = Y[p + (long)j * ldy];
      // real row: [yr ; -yi], imaginary row: [yi ; yr]
      x = (q < k) ? (im ? y.y : y.x) : (im ? y.x : -y.y);
      x *= sc;
    }
#pragma unroll
    for (int s = 0; s < kOzD; ++s) {  // balanced digits as for A
      x *= 128.0;
      const double t = rint(x);
      row[s * slice + q] = __float2bfloat16_rn((float)t);
      x -= t;
    }
  }
}

__global__ void __launch_bounds__(kOzThreads, 1)
k_oz_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tg, int m, int mp, int kchunk,
          int kp, const int* __restrict__ ex, const int* __restrict__ fx, double* __restrict__ part, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kOzStages], empty[kOzStages], tfull, tempty, drain;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  unsigned char* smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = blockIdx.x * kOzTM, z = blockIdx.y;
  const int kbeg = z * kchunk, kend = min(kp, kbeg + kchunk);
  const int nst = (kend - kbeg) / kOzKS;  // kchunk and kp are multiples of kOzKUnit
  const int ngroups = nst / kOzGroup;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kOzStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&tfull, 1);
    mbar_init(&tempty, kOzEpiWarps);
    mbar_init(&drain, 1);
    s_abort = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                 "r"(kOzTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  oz_fence_before();
  __syncthreads();
  oz_fence_after();
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: per stage six A digit tiles and six y digit tiles ----
      int s = 0;
      uint32_t ph = 0;
      int issued[kOzStages];
      uint32_t last_ph[kOzStages];
      for (int i = 0; i < kOzStages; ++i) { issued[i] = 0; last_ph[i] = 0; }
      bool ok = true;
      for (int kt = 0; kt < nst && ok; ++kt) {
        if (!oz_wait(&empty[s], ph ^ 1, &s_abort)) { ok = false; break; }
        unsigned char* st = smem + (size_t)s * kOzStageBytes;
        mbar_expect_tx(&full[s], kOzStageBytes);
        const int kx = kbeg + kt * kOzKS;
        for (int d = 0; d < kOzD; ++d) {
          oz_tma_2d(st + d * kOzATile, &ta, kx, d * mp + row0, &full[s]);
          oz_tma_2d(st + kOzD * kOzATile + d * kOzBTile, &tg, kx, d * kOzTN, &full[s]);
        }
        issued[s] = 1;
        last_ph[s] = ph;
        if (++s == kOzStages) { s = 0; ph ^= 1; }
      }
      if (!ok) {
        for (int i = 0; i < kOzStages; ++i) {
          if (!issued[i]) continue;
          const uint64_t t0 = global_ns();
          while (!mbar_try_wait(&full[i], last_ph[i]) && global_ns() - t0 < kOzWaitNs) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: the 21 digit pairs of levels 2..7 into six accumulators ----
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int g = 0; g < ngroups && ok; ++g) {
        if (!oz_wait(&tempty, (g & 1) ^ 1, &s_abort)) break;  // the previous group is drained
        oz_fence_after();
        for (int q = 0; q < kOzGroup; ++q) {
          if (!oz_wait(&full[s], ph, &s_abort)) { ok = false; break; }
          oz_fence_after();
          const uint32_t abase = smem_addr(smem + (size_t)s * kOzStageBytes);
          const uint32_t gbase = abase + kOzD * kOzATile;
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            const uint32_t off = kk * 32;  // 16 bf16 of K = 32 bytes of the 64-byte row
#pragma unroll
            for (int L = 2; L <= kOzD + 1; ++L) {
              const uint32_t d = tmem + (uint32_t)((L - 2) * kOzTN);
#pragma unroll
              for (int sa = 1; sa <= kOzD; ++sa) {
                const int tb = L - sa;
                if (tb < 1 || tb > kOzD) continue;
                const uint32_t acc = (q == 0 && kk == 0 && sa == 1) ? 0u : 1u;
                oz_mma(d, sw64_desc(abase + (sa - 1) * kOzATile + off), sw64_desc(gbase + (tb - 1) * kOzBTile + off),
                       kOzIdesc, acc);
              }
            }
          }
          oz_commit(&empty[s]);
          if (++s == kOzStages) { s = 0; ph ^= 1; }
        }
        if (ok) oz_commit(&tfull);
      }
      oz_commit(&drain);
      const uint64_t t0 = global_ns();
      while (!mbar_try_wait(&drain, 0) && global_ns() - t0 < kOzWaitNs) {
      }
    }
  } else {
    // ---- drains: warps 2..17, TMEM lane quarter q = warp % 4, 20 columns each ----
    const int qd = warp & 3, cb = (warp - 2) >> 2;
    float hi[kOzEpiCols], lo[kOzEpiCols];
#pragma unroll
    for (int c = 0; c < kOzEpiCols; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
    const uint32_t tq = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(cb * kOzEpiCols);
    bool ok = true;
    for (int g = 0; g < ngroups; ++g) {
      const bool w = oz_wait(&tfull, g & 1, &s_abort);
      if (!__all_sync(0xffffffffu, w)) { ok = false; break; }
      oz_fence_after();
#pragma unroll 1
      for (int L = 2; L <= kOzD + 1; ++L) {
        uint32_t v16[16], v4[4];
        const uint32_t ta_ = tq + (uint32_t)((L - 2) * kOzTN);
        oz_ld16(ta_, v16);
        oz_ld4(ta_ + 16, v4);
        oz_ld_wait();
        const float sc = __int_as_float((127 - 7 * L) << 23);  // 2^-7L
#pragma unroll
        for (int c = 0; c < 16; ++c) oz_two_sum(hi[c], lo[c], __uint_as_float(v16[c]) * sc);
#pragma unroll
        for (int c = 0; c < 4; ++c) oz_two_sum(hi[16 + c], lo[16 + c], __uint_as_float(v4[c]) * sc);
      }
      oz_fence_before();
      __syncwarp();
      if (lane == 0) oz_arrive(&tempty);
    }
    const int row = row0 + qd * 32 + lane;
    if (ok && row < m) {
      const int e = ex[row];
      double* pz = part + (size_t)z * kOzTN * m;
#pragma unroll
      for (int c = 0; c < kOzEpiCols; ++c) {
        const int col = cb * kOzEpiCols + c;
        pz[(size_t)col * m + row] = ldexp((double)hi[c] + (double)lo[c], e + fx[col]);
      }
    }
  }
  oz_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    oz_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOzTmemCols) : "memory");
  }
  if (threadIdx.x == 0 && s_abort) atomicExch(status, kOzTimeout);
}

// out = b + sign * (the K ranges' sums), complex columns from the real and
// imaginary output rows.
__global__ void k_oz_reduce(int m, int nc, int zs, const double* __restrict__ part, const double2* __restrict__ Bin,
                            long ldb, double sign, double2* __restrict__ out, long ldo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= m) return;
  double re = 0.0, im = 0.0;
  for (int z = 0; z < zs; ++z) {
    const double* pz = part + (size_t)z * kOzTN * m;
    re += pz[(size_t)j * m + i];
    im += pz[(size_t)(nc + j) * m + i];
  }
  double2 r = make_double2(sign * re, sign * im);
  if (Bin) {
    const double2 b = Bin[i + (long)j * ldb];
    r.x += b.x;
    r.y += b.y;
  }
  out[i + (long)j * ldo] = r;
}

struct OzLayout {
  int mp, kp, zs, kchunk;
  size_t a_off, g_off, ex_off, fx_off, part_off, total;
  OzLayout(int m, int nc, int k, int nsm) {
    (void)nc;
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    mp = (m + kOzTM - 1) / kOzTM * kOzTM;
    kp = (2 * k + kOzKUnit - 1) / kOzKUnit * kOzKUnit;
    // K ranges: enough CTAs for about one per SM
    const int tiles = mp / kOzTM;
    const int units = kp / kOzKUnit;
    zs = std::max(1, std::min(units, nsm / tiles));
    kchunk = (units + zs - 1) / zs * kOzKUnit;
    zs = (kp + kchunk - 1) / kchunk;
    a_off = 0;
    g_off = a_off + up((size_t)kOzD * mp * kp * 2);
    ex_off = g_off + up((size_t)kOzD * kOzTN * kp * 2);
    fx_off = ex_off + up((size_t)mp * sizeof(int));
    part_off = fx_off + up((size_t)kOzTN * sizeof(int));
    total = part_off + up((size_t)zs * kOzTN * m * sizeof(double));
  }
};

int g_oz_sms = 0;

}  // namespace

size_t resid_tc_work_bytes(int m, int nc, int k) {
  if (2 * nc > kOzTN || m <= 0 || k <= 0) return 0;
  return OzLayout(m, nc, k, 152).total;
}

bool resid_tc_supported() {
  static int cached = -1;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (cached < 0) cached = oz_device_supported(&g_oz_sms) ? 1 : 0;
  return cached == 1;
}

cudaError_t resid_tc(cudaStream_t st, int m, int nc, int k, const float2* A, long lda, const double2* Y, long ldy,
                     const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws, size_t ws_bytes,
                     int* status) {
  if (m <= 0 || nc <= 0) return cudaSuccess;
  if (k <= 0 || 2 * nc > kOzTN) return cudaErrorInvalidValue;
  if (!resid_tc_supported()) return cudaErrorNotSupported;
  const OzLayout lw(m, nc, k, 152);  // the same layout resid_tc_work_bytes sized
  if (!ws || ws_bytes < lw.total || (reinterpret_cast<uintptr_t>(ws) & 255u)) return cudaErrorInvalidValue;
  char* w = static_cast<char*>(ws);
  __nv_bfloat16* Ad = reinterpret_cast<__nv_bfloat16*>(w + lw.a_off);
  __nv_bfloat16* Gd = reinterpret_cast<__nv_bfloat16*>(w + lw.g_off);
  int* ex = reinterpret_cast<int*>(w + lw.ex_off);
  int* fx = reinterpret_cast<int*>(w + lw.fx_off);
  double* part = reinterpret_cast<double*>(w + lw.part_off);
  unsigned* rmax = reinterpret_cast<unsigned*>(part);  // the K ranges' sums are written later
  cudaError_t e = cudaMemsetAsync(rmax, 0, (size_t)m * sizeof(unsigned), st);
  if (e != cudaSuccess) return e;
  k_oz_row_max<<<dim3((m + 255) / 256, (k + kOzMaxCols - 1) / kOzMaxCols), 256, 0, st>>>(m, k, A, lda, rmax);
  k_oz_row_exp<<<(m + 255) / 256, 256, 0, st>>>(m, rmax, ex);
  k_oz_slice_a<<<dim3(lw.mp / 32, (k + 31) / 32), dim3(32, 8), 0, st>>>(m, k, lw.mp, lw.kp, A, lda, ex, Ad);
  if (lw.kp > 2 * k) k_oz_zero_kpad<<<4 * 152, 256, 0, st>>>(lw.mp, k, lw.kp, Ad);
  k_oz_slice_y<<<kOzTN, 256, 0, st>>>(k, nc, lw.kp, Y, ldy, fx, Gd);
  CUtensorMap ma, mg;
  if (!oz_map(&ma, Ad, lw.kp, kOzD * lw.mp, kOzTM) || !oz_map(&mg, Gd, lw.kp, kOzD * kOzTN, kOzTN))
    return cudaErrorNotSupported;
  e = cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOzSmem);
  if (e != cudaSuccess) return e;
  k_oz_gemm<<<dim3(lw.mp / kOzTM, lw.zs), kOzThreads, kOzSmem, st>>>(ma, mg, m, lw.mp, lw.kchunk, lw.kp, ex, fx, part,
                                                                     status);
  k_oz_reduce<<<dim3((m + 255) / 256, nc), 256, 0, st>>>(m, nc, lw.zs, part, Bin, ldb, sign, out, ldo);
  return cudaGetLastError();
}

}  // namespace hg
