// Device and host helpers of the exact-slicing tensor-core products
// (hg_resid_tc.cu: the refinement residual; hg_zgemm_tc.cu: the complex128
// LU updates): 64-byte-swizzled K-major BF16 digit tiles moved by TMA,
// kind::f16 MMAs into FP32 TMEM accumulators, bounded mbarrier waits, TMEM
// loads, and the tensor-map encoder.
#pragma once
#include <mutex>
#include <cuda.h>
#include <cudaTypedefs.h>

#include "hg_tma.cuh"

namespace hg {
namespace {

constexpr uint64_t kOzWaitNs = 2000000000ull;  // a wait on an mbarrier gives up after 2 s
constexpr int kOzKS = 32;                       // real K per stage: one 64-byte row of BF16 digits

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator,
// both K-major, N x M = n x m.
__host__ __device__ constexpr uint32_t oz_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Shared-memory descriptor, K-major, 64-byte swizzle: start >> 4, leading
// offset unused (1), 512 bytes between 8-row groups, version 1, layout 4.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(512 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)4 << 61);
}

__device__ __forceinline__ void oz_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void oz_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void oz_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void oz_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void oz_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void oz_tma_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// 16 and 4 consecutive accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void oz_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
__device__ __forceinline__ void oz_ld4(uint32_t taddr, uint32_t (&v)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
               : "r"(taddr));
}
__device__ __forceinline__ void oz_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Bounded wait on an mbarrier phase; on running out it raises the CTA's abort
// flag (which ends the other roles' waits too) and returns false.
__device__ __forceinline__ bool oz_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (global_ns() - t0 > kOzWaitNs) {
      *abort_flag = 1;
      return false;
    }
  }
}

// (S, s) += p exactly: S <- fl(S + p), s collects the rounding error.
__device__ __forceinline__ void oz_two_sum(float& S, float& s, float p) {
  const float t = __fadd_rn(S, p);
  const float z = __fsub_rn(t, S);
  s = __fadd_rn(s, __fadd_rn(__fsub_rn(S, __fsub_rn(t, z)), __fsub_rn(p, z)));
  S = t;
}

// Exponent e with max |x| * 2^-e in [0.5, 1) (0 for an all-zero set).
__device__ __forceinline__ int oz_exp(double amax) { return amax > 0.0 ? ilogb(amax) + 1 : 0; }

PFN_cuTensorMapEncodeTiled_v12000 oz_encode_fn() {
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

// BF16 rows x kp (kp a multiple of kOzKS), box kOzKS x box_rows (64 bytes
// wide), 64-byte swizzle.
bool oz_map(CUtensorMap* mp_, const void* base, int kp, int rows, int box_rows) {
  auto fn = oz_encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kOzKS, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(mp_, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// True on a compute capability 10.3 device with the tensor-map encoder; sets
// *nsm to its multiprocessor count.
bool oz_device_supported(int* nsm) {
  int dev = 0, major = 0, minor = 0;
  bool ok = cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess;
  cudaGetLastError();
  return ok && major == 10 && minor == 3 && oz_encode_fn() != nullptr;
}

}  // namespace
}  // namespace hg
