// Complex single-precision GEMM on the fifth-generation tensor cores
// (tcgen05.mma kind::tf32, accumulators in tensor memory): C -= A B, the
// trailing update A22 -= L21 U12 of the blocked LU (CGETRF step of
// AssbMatx.f90:111) with the panel width as inner dimension.
//
// Complex as real.  With a = ar + i ai, the product c = a b is the real 2x2
// block [[ar, -ai], [ai, ar]] times the real pair [br; bi].  So the complex
// m x n x k product is one real (2m) x n x (2k) product:
//   A_r (2m x 2k): rows 2i, 2i+1 and columns 2p, 2p+1 hold that 2x2 block of A(i,p)
//   B_r (2k x n):  B's interleaved (re, im) columns as they lie in memory
//   C_r (2m x n):  C's interleaved (re, im) columns as they lie in memory
// and the real product does exactly the 4mnk real multiply-adds of the
// complex one.  A_r and B_r are packed K-major (each row of A_r and each
// column of B_r contiguous) by two small kernels, which also split every
// value into TF32 parts: hi = rna_tf32(x), lo = rna_tf32(x - hi).
//   passes = 3: C -= A_hi B_hi + A_lo B_hi + A_hi B_lo, the three products
//               accumulated in the same tensor-memory tile.  The split makes
//               the products as accurate as single-precision ones; what
//               remains is the tensor cores' FP32 accumulation, which
//               truncates at every 8-deep step: measured 1.5e-5 of |C| at
//               k = 256 (the FP32 SIMT kernel 1e-6), enough for one
//               refinement sweep of the mixed-form solve.
//   passes = 1: C -= A_hi B_hi (TF32 products, measured 1e-3 of |C|).
//   passes = 2: the three products of passes = 3 with BF16 parts
//               (kind::f16, twice the TF32 rate): hi = rn_bf16(x),
//               lo = rn_bf16(x - hi) keep 16 of x's 24 bits, so the products
//               carry ~2^-16 relative error, of the order of the FP32
//               accumulation's own.  Each 128-byte row of a packed operand
//               holds 32 real K as [32 hi | 32 lo], so one tensor copy per
//               operand brings both parts and a stage is 48 KB: four stages
//               in flight instead of two.
//
// Kernel: persistent, one CTA per SM, 576 threads in three roles:
//   warp 0 (one thread)  TMA producer: per stage one 2-D tensor copy per
//                         operand tile (128 B rows, 128-byte swizzle) into a
//                         ring of shared-memory stages, completing on the
//                         stage's full barrier;
//   warp 1 (one thread)  MMA issuer: 4 K-steps of 8 per 32-wide stage,
//                         M = 128 real rows, N = 256 columns per instruction,
//                         tcgen05.commit frees the stage and, after the last
//                         stage, publishes the accumulator;
//   warps 2..17          epilogue: tcgen05.ld of the accumulator (warp w
//                         reads TMEM lanes 32 (w % 4) .., and the (w - 2) / 4-th
//                         quarter of the tile's columns, 16 at a time), C -= D
//                         with coalesced column loads and stores: sixteen
//                         warps keep the C loads of a tile in flight, which
//                         four could not (the update then waited on them).
// Two accumulators (2 x 256 TMEM columns) let the epilogue of one tile run
// under the main loop of the next.  Every wait is bounded in time: a wait
// that runs out raises an abort flag that ends every role, and the kernel
// records the timeout in the caller's status word.
#include <mutex>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "hg_common.cuh"
#include "hg_linalg.cuh"
#include "hg_tma.cuh"

namespace hg {
namespace {

constexpr int kTM = 128;         // real output rows per tile (64 complex rows)
constexpr int kTN = 256;         // output columns per tile
constexpr int kTK = 32;          // real inner extent per stage: one 128-byte swizzle row of fp32
constexpr int kEpiWarps = 16;                   // four per TMEM lane quarter, each a quarter of the tile's columns
constexpr int kThreads = 64 + 32 * kEpiWarps;    // + the producer and MMA warps
constexpr int kEpiCols = kTN / (kEpiWarps / 4);  // columns of one epilogue warp
constexpr int kEpiChunk = 16;                    // accumulator columns per tcgen05.ld
constexpr uint32_t kATile = kTM * kTK * 4;  // 16 KB
constexpr uint32_t kBTile = kTN * kTK * 4;  // 32 KB
constexpr uint32_t kTmemCols = 2 * kTN;     // two accumulators
constexpr uint64_t kTcWaitNs = 2000000000ull;
constexpr int kTcTimeout = -1000;           // value written to the status word on a wait that ran out

template <int P> struct TcCfg;
template <> struct TcCfg<3> {
  static constexpr int kStages = 2;
  static constexpr uint32_t kStageBytes = 2 * (kATile + kBTile);  // A_hi B_hi A_lo B_lo
  static constexpr int kEB = 4;                                    // bytes per packed element
};
template <> struct TcCfg<2> {
  static constexpr int kStages = 4;
  static constexpr uint32_t kStageBytes = kATile + kBTile;  // [hi | lo] rows of A and B
  static constexpr int kEB = 2;
};
template <> struct TcCfg<1> {
  static constexpr int kStages = 4;
  static constexpr uint32_t kStageBytes = kATile + kBTile;
  static constexpr int kEB = 4;
};
// real K per stage: one 128-byte swizzle row of packed elements (BF16: 32 hi + 32 lo)
template <int P> constexpr int tc_kstage() { return P == 2 ? 32 : 128 / TcCfg<P>::kEB; }
template <int P> constexpr size_t tc_smem_bytes() {
  return (size_t)TcCfg<P>::kStages * TcCfg<P>::kStageBytes + 1024;  // + slack for 1024-byte alignment
}

// Instruction descriptor of kind::tf32: F32 accumulator (bits 4-5 = 1), A and
// B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at
// bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);
// kind::f16 with A and B both BF16 (bits 7-9, 10-12 = 1), F32 accumulator.
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                                ((uint32_t)(kTM >> 4) << 24);

// Shared-memory matrix descriptor, K-major with 128-byte swizzle: start
// address >> 4 (bits 0-13), leading offset unused for this layout (1),
// stride between 8-row core groups 1024 B (bits 32-45), descriptor version 1
// (bit 46), base offset 0 (atoms 1024-byte aligned), swizzle mode 2 =
// 128-byte (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

template <bool BF>
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accum) {
  if (BF)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdescBf16), "r"(accum)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accum)
        : "memory");
}

// Arrive on bar once every tcgen05 operation this thread issued so far has completed.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// 16 consecutive accumulator columns of this warp's 32 TMEM lanes, one lane per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 32 consecutive accumulator columns of this warp's 32 TMEM lanes, one lane per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Bounded wait: false if the phase did not complete within the time limit
// (this thread then raises the abort flag) or another role already aborted.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (global_ns() - t0 > kTcWaitNs) {
      *abort_flag = 1;
      return false;
    }
  }
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1)
k_cgemm_tc(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap tb_hi,
           const __grid_constant__ CUtensorMap ta_lo, const __grid_constant__ CUtensorMap tb_lo,
           float* __restrict__ C, long ldcf, int mr, int n, int nkt, int tiles_m, int ntiles, int* status) {
  constexpr int S = TcCfg<P>::kStages;
  constexpr uint32_t SB = TcCfg<P>::kStageBytes;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2], drain;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  unsigned char* smem = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&tfull[0], 1);
    mbar_init(&tfull[1], 1);
    mbar_init(&tempty[0], kEpiWarps);
    mbar_init(&tempty[1], kEpiWarps);
    mbar_init(&drain, 1);
    s_abort = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      int s = 0;
      uint32_t ph = 0;
      int issued[S];
      uint32_t last_ph[S];
      for (int i = 0; i < S; ++i) { issued[i] = 0; last_ph[i] = 0; }
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int ym = (t % tiles_m) * kTM, yn = (t / tiles_m) * kTN;
        for (int kt = 0; kt < nkt; ++kt) {
          if (!tc_wait(&empty[s], ph ^ 1, &s_abort)) { ok = false; break; }
          unsigned char* st = smem + (size_t)s * SB;
          mbar_expect_tx(&full[s], SB);
          const int kx = kt * (P == 2 ? 64 : tc_kstage<P>());  // x in packed elements
          tma_load_2d(st, &ta_hi, kx, ym, &full[s]);
          tma_load_2d(st + kATile, &tb_hi, kx, yn, &full[s]);
          if (P == 3) {
            tma_load_2d(st + kATile + kBTile, &ta_lo, kx, ym, &full[s]);
            tma_load_2d(st + 2 * kATile + kBTile, &tb_lo, kx, yn, &full[s]);
          }
          issued[s] = 1;
          last_ph[s] = ph;
          if (++s == S) { s = 0; ph ^= 1; }
        }
      }
      if (!ok) {
        // let the copies already issued land before the CTA can exit
        for (int i = 0; i < S; ++i) {
          if (!issued[i]) continue;
          const uint64_t t0 = global_ns();
          while (!mbar_try_wait(&full[i], last_ph[i]) && global_ns() - t0 < kTcWaitNs) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      int s = 0;
      uint32_t ph = 0;
      int it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++it) {
        const int acc = it & 1;
        if (!tc_wait(&tempty[acc], ((it >> 1) & 1) ^ 1, &s_abort)) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * kTN);
        for (int kt = 0; kt < nkt; ++kt) {
          if (!tc_wait(&full[s], ph, &s_abort)) { ok = false; break; }
          tc_fence_after();
          const uint32_t a_hi = smem_addr(smem + (size_t)s * SB), b_hi = a_hi + kATile;
          const uint32_t a_lo = b_hi + kBTile, b_lo = a_lo + kATile;
          if (P == 2) {
            // [hi | lo] rows: K-steps of 16 bf16 (32 bytes) at 0 and 32, their lo parts 64 bytes on
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
              const uint32_t off = kk * 32;
              tc_mma<true>(d, sw128_desc(a_hi + 64 + off), sw128_desc(b_hi + off), (kt | kk) != 0);
              tc_mma<true>(d, sw128_desc(a_hi + off), sw128_desc(b_hi + 64 + off), 1u);
              tc_mma<true>(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), 1u);
            }
          } else {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint32_t off = kk * 32;  // one instruction's K (8 tf32) = 32 bytes of the swizzle row
              if (P == 3) {
                tc_mma<false>(d, sw128_desc(a_lo + off), sw128_desc(b_hi + off), (kt | kk) != 0);
                tc_mma<false>(d, sw128_desc(a_hi + off), sw128_desc(b_lo + off), 1u);
                tc_mma<false>(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), 1u);
              } else {
                tc_mma<false>(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), (kt | kk) != 0);
              }
            }
          }
          tc_commit(&empty[s]);
          if (++s == S) { s = 0; ph ^= 1; }
        }
        if (ok) tc_commit(&tfull[acc]);
      }
      // no MMA may still be running when the accumulators are freed
      tc_commit(&drain);
      const uint64_t t0 = global_ns();
      while (!mbar_try_wait(&drain, 0) && global_ns() - t0 < kTcWaitNs) {
      }
    }
  } else {
    // ---- epilogue: warps 2..17, TMEM lane quarter q = warp % 4, column quarter (warp - 2) / 4 ----
    const int q = warp & 3, part = (warp - 2) >> 2;
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
      const int acc = it & 1;
      const bool ok = tc_wait(&tfull[acc], (it >> 1) & 1, &s_abort);
      if (!__all_sync(0xffffffffu, ok)) break;
      tc_fence_after();
      const int row = (t % tiles_m) * kTM + q * 32 + lane;
      const int col_base = (t / tiles_m) * kTN;
      const bool rok = row < mr;
      float* crow = C + row;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * kTN);
      for (int c0 = part * kEpiCols; c0 < (part + 1) * kEpiCols; c0 += kEpiChunk) {
        const int col0 = col_base + c0;
        if (col0 >= n) break;  // uniform over the warp
        float cv[kEpiChunk];
#pragma unroll
        for (int j = 0; j < kEpiChunk; ++j) cv[j] = (rok && col0 + j < n) ? crow[(long)(col0 + j) * ldcf] : 0.f;
        uint32_t dv[kEpiChunk];
        tmem_ld16(tbase + (uint32_t)c0, dv);
#pragma unroll
        for (int j = 0; j < kEpiChunk; ++j)
          if (rok && col0 + j < n) crow[(long)(col0 + j) * ldcf] = cv[j] - __uint_as_float(dv[j]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
  if (threadIdx.x == 0 && s_abort) atomicExch(status, kTcTimeout);
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// off: the packed element offset row * kr + k of a pair (k even).  BF16 rows
// hold [32 hi | 32 lo] per 32 values of k, so row r's k lands at
// r * 2 kr + (k / 32) * 64 + k % 32 (hi) and 32 further on (lo); lo is unused.
template <int P>
__device__ __forceinline__ void split_store(void* hi, void* lo, long off, float x0, float x1) {
  if (P == 2) {
    const long e = 2 * off - (off & 31);  // r * 2 kr + (k / 32) * 64 + k % 32, kr a multiple of 32
    const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
    __nv_bfloat162 hv, lv;
    hv.x = h0; hv.y = h1;
    lv.x = __float2bfloat16_rn(x0 - __bfloat162float(h0));
    lv.y = __float2bfloat16_rn(x1 - __bfloat162float(h1));
    __nv_bfloat16* base = static_cast<__nv_bfloat16*>(hi);
    *reinterpret_cast<__nv_bfloat162*>(base + e) = hv;
    *reinterpret_cast<__nv_bfloat162*>(base + e + 32) = lv;
    (void)lo;
    return;
  }
  const float h0 = tf32_rna(x0), h1 = tf32_rna(x1);
  *reinterpret_cast<float2*>(static_cast<float*>(hi) + off) = make_float2(h0, h1);
  if (P == 3)
    *reinterpret_cast<float2*>(static_cast<float*>(lo) + off) = make_float2(tf32_rna(x0 - h0), tf32_rna(x1 - h1));
}

// A (m x k complex, column-major) -> A_r hi/lo (2m rows x kr floats, row-major),
// through a 32 x 32 shared-memory transpose so that both sides are coalesced.
template <int P>
__global__ void k_pack_a(int m, int k, int kr, const float2* __restrict__ A, long lda, void* __restrict__ hi,
                         void* __restrict__ lo) {
  __shared__ float2 t[32][33];
  const int i0 = blockIdx.x * 32, p0 = blockIdx.y * 32, tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, p = p0 + r;
    t[r][tx] = (i < m && p < k) ? A[i + (long)p * lda] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, p = p0 + tx;
    if (i >= m || 2 * p >= kr) continue;
    const float2 a = t[tx][r];
    split_store<P>(hi, lo, (long)(2 * i) * kr + 2 * p, a.x, -a.y);
    split_store<P>(hi, lo, (long)(2 * i + 1) * kr + 2 * p, a.y, a.x);
  }
}

// B (k x n complex, column-major) -> B_r hi/lo (n rows x kr floats): column j of B
// as floats, zero-padded from 2k to kr.
template <int P>
__global__ void k_pack_b(int k, int n, int kr, const float2* __restrict__ B, long ldb, void* __restrict__ hi,
                         void* __restrict__ lo) {
  const int kp = kr / 2;
  const long total = (long)kp * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int p = (int)(e % kp), j = (int)(e / kp);
    const float2 b = p < k ? B[p + (long)j * ldb] : make_float2(0.f, 0.f);
    split_store<P>(hi, lo, (long)j * kr + 2 * p, b.x, b.y);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  }
  return fn;
}

// 2-D tensor map over rows x kr packed elements (fp32, or bf16 when eb = 2;
// row-major, kr a multiple of one 128-byte row), box 128 bytes x box_rows,
// 128-byte swizzle, zero fill beyond the last row.
bool make_map(CUtensorMap* m, const void* base, int kr, int rows, int box_rows, int eb) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)kr, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kr * eb};
  const cuuint32_t box[2] = {(cuuint32_t)(128 / eb), (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, eb == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base),
            dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int g_num_sms = 0;

template <int P>
cudaError_t launch_tc(cudaStream_t st, int m, int n, int k, const float2* A, long lda, const float2* B, long ldb,
                      float2* C, long ldc, void* ws, int* status) {
  constexpr int EB = TcCfg<P>::kEB, KS = tc_kstage<P>();
  const int kr = ((2 * k + KS - 1) / KS) * KS;
  const size_t abytes = (size_t)2 * m * kr * EB, bbytes = (size_t)n * kr * EB;
  char* w = static_cast<char*>(ws);
  void* a_hi = w;
  void* a_lo = w + abytes;
  void* b_hi = w + 2 * abytes;
  void* b_lo = w + 2 * abytes + bbytes;
  k_pack_a<P><<<dim3((m + 31) / 32, (kr / 2 + 31) / 32), dim3(32, 8), 0, st>>>(m, k, kr, A, lda, a_hi, a_lo);
  k_pack_b<P><<<1216, 256, 0, st>>>(k, n, kr, B, ldb, b_hi, b_lo);
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  const int kx = (P == 2) ? 2 * kr : kr;  // BF16: [hi | lo] rows twice as long, one map per operand
  if (!make_map(&ma_hi, a_hi, kx, 2 * m, kTM, EB) || !make_map(&mb_hi, b_hi, kx, n, kTN, EB))
    return cudaErrorNotSupported;
  if (P == 3) {
    if (!make_map(&ma_lo, a_lo, kr, 2 * m, kTM, EB) || !make_map(&mb_lo, b_lo, kr, n, kTN, EB))
      return cudaErrorNotSupported;
  } else {
    ma_lo = ma_hi;
    mb_lo = mb_hi;
  }
  const int tiles_m = (2 * m + kTM - 1) / kTM, tiles_n = (n + kTN - 1) / kTN;
  const int ntiles = tiles_m * tiles_n;
  const int grid = ntiles < g_num_sms ? ntiles : g_num_sms;
  const size_t smem = tc_smem_bytes<P>();
  cudaError_t e = cudaFuncSetAttribute(k_cgemm_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_cgemm_tc<P><<<grid, kThreads, smem, st>>>(ma_hi, mb_hi, ma_lo, mb_lo, reinterpret_cast<float*>(C), 2 * ldc,
                                              2 * m, n, kr / KS, tiles_m, ntiles, status);
  return cudaGetLastError();
}

}  // namespace

bool cgemm_tc_supported() {
  static int cached = -1;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  if (cached < 0) {
    int dev = 0, major = 0, minor = 0;
    cached = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess) {
      // the kernels are built for sm_103a only
      cached = (major == 10 && minor == 3 && encode_fn() != nullptr) ? 1 : 0;
    }
    cudaGetLastError();
  }
  return cached == 1;
}

size_t cgemm_tc_work_bytes(int m, int n, int k) {
  const size_t kr = (size_t)((2 * k + kTK - 1) / kTK) * kTK;
  return 2 * ((size_t)2 * m * kr + (size_t)n * kr) * sizeof(float) + 256;
}

cudaError_t cgemm_tc(cudaStream_t st, int passes, int m, int n, int k, const float2* A, long lda, const float2* B,
                     long ldb, float2* C, long ldc, void* ws, size_t ws_bytes, int* status) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if (!cgemm_tc_supported()) return cudaErrorNotSupported;
  if (!ws || ws_bytes < cgemm_tc_work_bytes(m, n, k) || (reinterpret_cast<uintptr_t>(ws) & 255u)) return cudaErrorInvalidValue;
  if (passes == 3) return launch_tc<3>(st, m, n, k, A, lda, B, ldb, C, ldc, ws, status);
  if (passes == 2) return launch_tc<2>(st, m, n, k, A, lda, B, ldb, C, ldc, ws, status);
  if (passes == 1) return launch_tc<1>(st, m, n, k, A, lda, B, ldb, C, ldc, ws, status);
  return cudaErrorInvalidValue;
}

}  // namespace hg
