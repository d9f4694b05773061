// Refinement residual of the mixed form: out = b + sign * op(A) y, where A is
// the complex64 matrix that was factorised (its entries are exact in single
// precision) and y, b are complex128.
//
// GB300's FP64 pipes run at a small fraction of its FP32 pipes, and a
// complex128 GEMM of this shape (n x n times n x ~40) is FP64-bound.  This
// kernel keeps double-precision accuracy on the FP32 pipes instead:
//  - y is split once into two floats, y = yh + yl (|y - yh - yl| <= 2^-48 |y|);
//  - a * yh is formed exactly as p + e (p = fl(a yh), e = fma(a, yh, -p),
//    Dekker's TwoProduct with a fused multiply-add);
//  - p is accumulated with Knuth's TwoSum into a float pair (S, s), the
//    rounding error of every addition going into s together with e and the
//    small products a * yl (Ogita, Rump and Oishi's compensated dot product).
// The result has the accuracy of a dot product in ~2x single precision
// (about 1e-14 relative to sum |a||y| in practice), far below the 1e-10
// refinement tolerance.  The explicit _rn intrinsics keep the compiler from
// contracting the TwoSum steps into fused operations, which would break the
// error-free transformations.
//
// A cheaper mode (exact = false) serves products whose operands carry single
// precision anyway (the mixed form's right-hand sides, B = S W with S from the
// single-precision fill, and the refinement's updated residual r - A d): products
// a * yh in FP32, summed in FP32 within each 32-deep stage, and the stage sums
// accumulated with TwoSum as above, so the error is that of a 32-term
// single-precision sum (~1e-7 of sum |a||y|), not of an n-term one.  With four
// FMAs per complex product this mode would be bound by its shared-memory reads
// at one row per thread, so it has its own kernel (k_resid_sp): two rows per
// thread and y's high parts only, 7 reads per 80 FMAs instead of 11 per 40.
//
// Tiling: 64 rows x CW = 4*CPT columns per CTA, 256 threads (64 rows x 4
// column groups of CPT), 32-deep stages of A (complex64) and of the split y
// (float4 = yh.re, yl.re, yh.im, yl.im) double-buffered by cp.async.  The
// inner dimension is split across CTAs (gridDim.z) so that a tall-skinny
// product fills the GPU; each slice writes a complex128 partial and a second
// kernel adds the slices and b in double precision.
#include "hg_linalg.cuh"
#include "hg_tma.cuh"

namespace hg {
namespace {

constexpr int kRRows = 64, kRK = 32, kRThreads = 256, kRMaxCW = 40, kRMaxSlices = 16;
constexpr size_t kRATile = (size_t)kRK * kRRows * sizeof(float2);   // 16 KB
constexpr size_t kRYTile = (size_t)kRK * kRMaxCW * sizeof(float4);  // 20 KB
constexpr size_t kRStage = kRATile + kRYTile;
constexpr size_t kRSmem = 2 * kRStage;

__global__ void k_split_y(int k, int nc, int cw, int ncb, const double2* __restrict__ Y, long ldy,
                          float4* __restrict__ Ys) {
  const long total = (long)ncb * k * cw;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e % cw);
    const long rest = e / cw;
    const int l = (int)(rest % k), cb = (int)(rest / k);
    const int col = cb * cw + c;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
    if (col < nc) {
      const double2 y = Y[l + (long)col * ldy];
      o.x = (float)y.x;
      o.y = (float)(y.x - (double)o.x);
      o.z = (float)y.y;
      o.w = (float)(y.y - (double)o.z);
    }
    Ys[e] = o;
  }
}

// (S, s) += p exactly: S <- fl(S + p), s collects the rounding error.
__device__ __forceinline__ void two_sum_acc(float& S, float& s, float p) {
  const float t = __fadd_rn(S, p);
  const float z = __fsub_rn(t, S);
  s = __fadd_rn(s, __fadd_rn(__fsub_rn(S, __fsub_rn(t, z)), __fsub_rn(p, z)));
  S = t;
}

// One complex multiply-accumulate a * y into (Sr, sr) + i (Si, si);
// y = (yh.re, yl.re, yh.im, yl.im).
__device__ __forceinline__ void mac_df(float ar, float ai, const float4& y, float& Sr, float& sr, float& Si,
                                       float& si) {
  float p, e;
  p = __fmul_rn(ar, y.x); e = fmaf(ar, y.x, -p); two_sum_acc(Sr, sr, p); sr = __fadd_rn(sr, e);
  p = __fmul_rn(-ai, y.z); e = fmaf(-ai, y.z, -p); two_sum_acc(Sr, sr, p); sr = __fadd_rn(sr, e);
  sr = fmaf(ar, y.y, sr);
  sr = fmaf(-ai, y.w, sr);
  p = __fmul_rn(ar, y.z); e = fmaf(ar, y.z, -p); two_sum_acc(Si, si, p); si = __fadd_rn(si, e);
  p = __fmul_rn(ai, y.x); e = fmaf(ai, y.x, -p); two_sum_acc(Si, si, p); si = __fadd_rn(si, e);
  si = fmaf(ar, y.w, si);
  si = fmaf(ai, y.y, si);
}

template <int CPT, bool TA, bool VEC>
__device__ __forceinline__ void resid_stage(float2* As, float4* Yt, const float2* __restrict__ A, long lda,
                                            const float4* __restrict__ Ycb, int m, int m0, int k0, int kend, int tid) {
  constexpr int CW = 4 * CPT;
  if (!TA) {
    if (VEC) {
#pragma unroll
      for (int it = 0; it < kRK * kRRows / 2 / kRThreads; ++it) {
        const int e = tid + it * kRThreads;
        const int i = (e % (kRRows / 2)) * 2, l = e / (kRRows / 2);
        const int gm = m0 + i, gk = k0 + l;
        int bytes = 0;
        if (gk < kend) bytes = (gm + 1 < m) ? 16 : (gm < m ? 8 : 0);
        cp_async16(As + l * kRRows + i, bytes ? A + gm + (long)gk * lda : A, bytes);
      }
    } else {
#pragma unroll
      for (int it = 0; it < kRK * kRRows / kRThreads; ++it) {
        const int e = tid + it * kRThreads;
        const int i = e % kRRows, l = e / kRRows;
        const int gm = m0 + i, gk = k0 + l;
        const bool ok = gm < m && gk < kend;
        cp_async8(As + l * kRRows + i, ok ? A + gm + (long)gk * lda : A, ok);
      }
    }
  } else {
#pragma unroll
    for (int it = 0; it < kRK * kRRows / kRThreads; ++it) {
      const int e = tid + it * kRThreads;
      const int l = e % kRK, i = e / kRK;
      const int gm = m0 + i, gk = k0 + l;
      const bool ok = gm < m && gk < kend;
      cp_async8(As + l * kRRows + i, ok ? A + gk + (long)gm * lda : A, ok);
    }
  }
  for (int e = tid; e < kRK * CW; e += kRThreads) {
    const int l = e / CW, c = e % CW;
    const int gk = k0 + l;
    const bool ok = gk < kend;
    cp_async16(Yt + l * CW + c, ok ? Ycb + (long)gk * CW + c : Ycb, ok ? 16 : 0);
  }
}

template <int CPT, bool TA, bool VEC, bool EXACT>
__global__ void __launch_bounds__(kRThreads, 2)
k_resid_df(int m, int nc, int k, int kchunk, const float2* __restrict__ A, long lda, const float4* __restrict__ Ys,
           double2* __restrict__ part) {
  constexpr int CW = 4 * CPT;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, tx = tid & 63, cg = tid >> 6;
  const int m0 = blockIdx.x * kRRows, cb = blockIdx.y, z = blockIdx.z;
  const int kbeg = z * kchunk, kend = min(k, kbeg + kchunk);
  const float4* Ycb = Ys + (size_t)cb * k * CW;
  float Sr[CPT], sr[CPT], Si[CPT], si[CPT];
#pragma unroll
  for (int j = 0; j < CPT; ++j) { Sr[j] = 0.f; sr[j] = 0.f; Si[j] = 0.f; si[j] = 0.f; }

  const int nst = (kend - kbeg + kRK - 1) / kRK;
  if (nst > 0)
    resid_stage<CPT, TA, VEC>(reinterpret_cast<float2*>(smem), reinterpret_cast<float4*>(smem + kRATile), A, lda, Ycb,
                              m, m0, kbeg, kend, tid);
  cp_async_commit();
  for (int s = 0; s < nst; ++s) {
    unsigned char* cur = smem + (s & 1) * kRStage;
    if (s + 1 < nst) {
      unsigned char* nxt = smem + ((s + 1) & 1) * kRStage;
      resid_stage<CPT, TA, VEC>(reinterpret_cast<float2*>(nxt), reinterpret_cast<float4*>(nxt + kRATile), A, lda, Ycb,
                                m, m0, kbeg + (s + 1) * kRK, kend, tid);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float2* as = reinterpret_cast<const float2*>(cur);
    const float4* yt = reinterpret_cast<const float4*>(cur + kRATile) + cg * CPT;
    if (EXACT) {
#pragma unroll 4
      for (int l = 0; l < kRK; ++l) {
        const float2 a = as[l * kRRows + tx];
#pragma unroll
        for (int j = 0; j < CPT; ++j) mac_df(a.x, a.y, yt[l * CW + j], Sr[j], sr[j], Si[j], si[j]);
      }
    } else {
      float pr[CPT], pi[CPT];
#pragma unroll
      for (int j = 0; j < CPT; ++j) { pr[j] = 0.f; pi[j] = 0.f; }
#pragma unroll 4
      for (int l = 0; l < kRK; ++l) {
        const float2 a = as[l * kRRows + tx];
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
          const float4 y = yt[l * CW + j];
          pr[j] = fmaf(a.x, y.x, pr[j]);
          pr[j] = fmaf(-a.y, y.z, pr[j]);
          pi[j] = fmaf(a.x, y.z, pi[j]);
          pi[j] = fmaf(a.y, y.x, pi[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < CPT; ++j) {
        two_sum_acc(Sr[j], sr[j], pr[j]);
        two_sum_acc(Si[j], si[j], pi[j]);
      }
    }
    __syncthreads();
  }
  const int row = m0 + tx;
  if (row < m) {
    double2* pz = part + (size_t)z * m * nc;
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
      const int col = cb * CW + cg * CPT + j;
      if (col < nc) pz[row + (size_t)col * m] = make_double2((double)Sr[j] + (double)sr[j], (double)Si[j] + (double)si[j]);
    }
  }
}

// The single-product mode: 64 rows x CW = 4*CPT columns per CTA, 128
// threads (32 lanes x 4 column groups), each thread rows lane and lane + 32
// of the tile and CPT columns; y's high parts as complex64 [cb][k][CW].
constexpr int kSpThreads = 128;
constexpr size_t kSpYTile = (size_t)kRK * kRMaxCW * sizeof(float2);  // 10 KB
constexpr size_t kSpStage = kRATile + kSpYTile;
constexpr size_t kSpSmem = 2 * kSpStage;

__global__ void k_split_yh(int k, int nc, int cw, int ncb, const double2* __restrict__ Y, long ldy,
                           float2* __restrict__ Ys) {
  const long total = (long)ncb * k * cw;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e % cw);
    const long rest = e / cw;
    const int l = (int)(rest % k), cb = (int)(rest / k);
    const int col = cb * cw + c;
    float2 o = make_float2(0.f, 0.f);
    if (col < nc) {
      const double2 y = Y[l + (long)col * ldy];
      o = make_float2((float)y.x, (float)y.y);
    }
    Ys[e] = o;
  }
}

template <int CPT, bool VEC>
__device__ __forceinline__ void sp_stage(float2* As, float2* Yt, const float2* __restrict__ A, long lda,
                                         const float2* __restrict__ Ycb, int m, int m0, int k0, int kend, int tid) {
  constexpr int CW = 4 * CPT;
  if (VEC) {
#pragma unroll
    for (int it = 0; it < kRK * kRRows / 2 / kSpThreads; ++it) {
      const int e = tid + it * kSpThreads;
      const int i = (e % (kRRows / 2)) * 2, l = e / (kRRows / 2);
      const int gm = m0 + i, gk = k0 + l;
      int bytes = 0;
      if (gk < kend) bytes = (gm + 1 < m) ? 16 : (gm < m ? 8 : 0);
      cp_async16(As + l * kRRows + i, bytes ? A + gm + (long)gk * lda : A, bytes);
    }
  } else {
#pragma unroll
    for (int it = 0; it < kRK * kRRows / kSpThreads; ++it) {
      const int e = tid + it * kSpThreads;
      const int i = e % kRRows, l = e / kRRows;
      const int gm = m0 + i, gk = k0 + l;
      const bool ok = gm < m && gk < kend;
      cp_async8(As + l * kRRows + i, ok ? A + gm + (long)gk * lda : A, ok);
    }
  }
  // CW complex per k row: CW / 2 16-byte pieces
  for (int e = tid; e < kRK * CW / 2; e += kSpThreads) {
    const int l = e / (CW / 2), c2 = e % (CW / 2);
    const int gk = k0 + l;
    const bool ok = gk < kend;
    cp_async16(Yt + l * CW + 2 * c2, ok ? Ycb + (long)gk * CW + 2 * c2 : Ycb, ok ? 16 : 0);
  }
}

template <int CPT, bool VEC>
__global__ void __launch_bounds__(kSpThreads, 3)
k_resid_sp(int m, int nc, int k, int kchunk, const float2* __restrict__ A, long lda, const float2* __restrict__ Ys,
           double2* __restrict__ part) {
  constexpr int CW = 4 * CPT;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, cg = tid >> 5;
  const int m0 = blockIdx.x * kRRows, cb = blockIdx.y, z = blockIdx.z;
  const int kbeg = z * kchunk, kend = min(k, kbeg + kchunk);
  const float2* Ycb = Ys + (size_t)cb * k * CW;
  float Sr[2][CPT], sr[2][CPT], Si[2][CPT], si[2][CPT];
#pragma unroll
  for (int h = 0; h < 2; ++h)
#pragma unroll
    for (int j = 0; j < CPT; ++j) { Sr[h][j] = 0.f; sr[h][j] = 0.f; Si[h][j] = 0.f; si[h][j] = 0.f; }
  const int nst = (kend - kbeg + kRK - 1) / kRK;
  if (nst > 0)
    sp_stage<CPT, VEC>(reinterpret_cast<float2*>(smem), reinterpret_cast<float2*>(smem + kRATile), A, lda, Ycb, m, m0,
                       kbeg, kend, tid);
  cp_async_commit();
  for (int s = 0; s < nst; ++s) {
    unsigned char* cur = smem + (s & 1) * kSpStage;
    if (s + 1 < nst) {
      unsigned char* nxt = smem + ((s + 1) & 1) * kSpStage;
      sp_stage<CPT, VEC>(reinterpret_cast<float2*>(nxt), reinterpret_cast<float2*>(nxt + kRATile), A, lda, Ycb, m, m0,
                         kbeg + (s + 1) * kRK, kend, tid);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float2* as = reinterpret_cast<const float2*>(cur);
    const float4* yt = reinterpret_cast<const float4*>(cur + kRATile);
    float pr[2][CPT], pi[2][CPT];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int j = 0; j < CPT; ++j) { pr[h][j] = 0.f; pi[h][j] = 0.f; }
#pragma unroll 2
    for (int l = 0; l < kRK; ++l) {
      const float2 a0 = as[l * kRRows + lane], a1 = as[l * kRRows + lane + 32];
#pragma unroll
      for (int j2 = 0; j2 < CPT / 2; ++j2) {
        const float4 y = yt[(l * CW + cg * CPT) / 2 + j2];  // (yh_re, yh_im) of two columns
        pr[0][2 * j2] = fmaf(-a0.y, y.y, fmaf(a0.x, y.x, pr[0][2 * j2]));
        pi[0][2 * j2] = fmaf(a0.y, y.x, fmaf(a0.x, y.y, pi[0][2 * j2]));
        pr[0][2 * j2 + 1] = fmaf(-a0.y, y.w, fmaf(a0.x, y.z, pr[0][2 * j2 + 1]));
        pi[0][2 * j2 + 1] = fmaf(a0.y, y.z, fmaf(a0.x, y.w, pi[0][2 * j2 + 1]));
        pr[1][2 * j2] = fmaf(-a1.y, y.y, fmaf(a1.x, y.x, pr[1][2 * j2]));
        pi[1][2 * j2] = fmaf(a1.y, y.x, fmaf(a1.x, y.y, pi[1][2 * j2]));
        pr[1][2 * j2 + 1] = fmaf(-a1.y, y.w, fmaf(a1.x, y.z, pr[1][2 * j2 + 1]));
        pi[1][2 * j2 + 1] = fmaf(a1.y, y.z, fmaf(a1.x, y.w, pi[1][2 * j2 + 1]));
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int j = 0; j < CPT; ++j) {
        two_sum_acc(Sr[h][j], sr[h][j], pr[h][j]);
        two_sum_acc(Si[h][j], si[h][j], pi[h][j]);
      }
    __syncthreads();
  }
  double2* pz = part + (size_t)z * m * nc;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int row = m0 + lane + 32 * h;
    if (row >= m) continue;
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
      const int col = cb * CW + cg * CPT + j;
      if (col < nc)
        pz[row + (size_t)col * m] = make_double2((double)Sr[h][j] + (double)sr[h][j], (double)Si[h][j] + (double)si[h][j]);
    }
  }
}

__global__ void k_resid_reduce(int m, int nc, int slices, const double2* __restrict__ part,
                               const double2* __restrict__ Bin, long ldb, double sign, double2* __restrict__ out,
                               long ldo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i >= m) return;
  double sx = 0.0, sy = 0.0;
  for (int z = 0; z < slices; ++z) {
    const double2 v = part[(size_t)z * m * nc + i + (size_t)c * m];
    sx += v.x;
    sy += v.y;
  }
  double2 r = make_double2(sign * sx, sign * sy);
  if (Bin) {
    const double2 b = Bin[i + (long)c * ldb];
    r.x += b.x;
    r.y += b.y;
  }
  out[i + (long)c * ldo] = r;
}

int pick_cpt(int nc) {
  const int per = (nc + 3) / 4;  // columns per group for one column block
  if (per <= 2) return 2;
  if (per <= 4) return 4;
  if (per <= 6) return 6;
  if (per <= 8) return 8;
  return 10;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

template <int CPT, bool TA, bool VEC, bool EXACT>
cudaError_t launch_resid(cudaStream_t st, int m, int nc, int k, const float2* A, long lda, const double2* Y, long ldy,
                         const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws, size_t ws_bytes) {
  constexpr int CW = 4 * CPT;
  const int ncb = (nc + CW - 1) / CW;
  const int gx = (m + kRRows - 1) / kRRows;
  const size_t ys_bytes = align256((size_t)ncb * k * CW * sizeof(float4));
  // Slices of the inner dimension: at least enough CTAs for two per SM, then
  // the count (up to 16) whose CTAs fill their last wave best (95 row blocks
  // x 4 slices would run 1.25 waves of 304 CTAs; x 16 slices, 5 full ones).
  const int kmax = min(kRMaxSlices, (k + kRK - 1) / kRK);
  int slices = max(1, min((2 * 152 + gx * ncb - 1) / (gx * ncb), kmax));
  {
    double best = 0.0;
    for (int s = slices; s <= kmax; ++s) {
      const long ctas = (long)gx * ncb * s;
      const double fill = (double)ctas / (double)(((ctas + 303) / 304) * 304);
      if (fill > best + 1e-9) { best = fill; slices = s; }
    }
  }
  while (slices > 1 && ys_bytes + (size_t)slices * m * nc * sizeof(double2) > ws_bytes) --slices;
  if (ys_bytes + (size_t)slices * m * nc * sizeof(double2) > ws_bytes) return cudaErrorInvalidValue;
  int kchunk = ((k + slices - 1) / slices + kRK - 1) / kRK * kRK;
  slices = (k + kchunk - 1) / kchunk;
  float4* Ys = static_cast<float4*>(ws);
  double2* part = reinterpret_cast<double2*>(static_cast<unsigned char*>(ws) + ys_bytes);
  k_split_y<<<4 * 152, 256, 0, st>>>(k, nc, CW, ncb, Y, ldy, Ys);
  auto kern = k_resid_df<CPT, TA, VEC, EXACT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRSmem);
  if (e != cudaSuccess) return e;
  kern<<<dim3(gx, ncb, slices), kRThreads, kRSmem, st>>>(m, nc, k, kchunk, A, lda, Ys, part);
  k_resid_reduce<<<dim3((m + 255) / 256, nc), 256, 0, st>>>(m, nc, slices, part, Bin, ldb, sign, out, ldo);
  return cudaGetLastError();
}

template <int CPT, bool VEC>
cudaError_t launch_sp(cudaStream_t st, int m, int nc, int k, const float2* A, long lda, const double2* Y, long ldy,
                      const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws, size_t ws_bytes) {
  constexpr int CW = 4 * CPT;
  const int ncb = (nc + CW - 1) / CW;
  const int gx = (m + kRRows - 1) / kRRows;
  const size_t ys_bytes = align256((size_t)ncb * k * CW * sizeof(float4));  // the exact mode's layout size
  // slices of the inner dimension as in launch_resid, for three CTAs per SM
  const int kmax = min(kRMaxSlices, (k + kRK - 1) / kRK);
  int slices = max(1, min((3 * 152 + gx * ncb - 1) / (gx * ncb), kmax));
  {
    double best = 0.0;
    for (int s = slices; s <= kmax; ++s) {
      const long ctas = (long)gx * ncb * s;
      const double fill = (double)ctas / (double)(((ctas + 455) / 456) * 456);
      if (fill > best + 1e-9) { best = fill; slices = s; }
    }
  }
  while (slices > 1 && ys_bytes + (size_t)slices * m * nc * sizeof(double2) > ws_bytes) --slices;
  if (ys_bytes + (size_t)slices * m * nc * sizeof(double2) > ws_bytes) return cudaErrorInvalidValue;
  int kchunk = ((k + slices - 1) / slices + kRK - 1) / kRK * kRK;
  slices = (k + kchunk - 1) / kchunk;
  float2* Ys = static_cast<float2*>(ws);
  double2* part = reinterpret_cast<double2*>(static_cast<unsigned char*>(ws) + ys_bytes);
  k_split_yh<<<4 * 152, 256, 0, st>>>(k, nc, CW, ncb, Y, ldy, Ys);
  auto kern = k_resid_sp<CPT, VEC>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSpSmem);
  if (e != cudaSuccess) return e;
  kern<<<dim3(gx, ncb, slices), kSpThreads, kSpSmem, st>>>(m, nc, k, kchunk, A, lda, Ys, part);
  k_resid_reduce<<<dim3((m + 255) / 256, nc), 256, 0, st>>>(m, nc, slices, part, Bin, ldb, sign, out, ldo);
  return cudaGetLastError();
}

template <int CPT>
cudaError_t dispatch(cudaStream_t st, bool transa, bool vec, bool exact, int m, int nc, int k, const float2* A,
                     long lda, const double2* Y, long ldy, const double2* Bin, long ldb, double sign, double2* out,
                     long ldo, void* ws, size_t ws_bytes) {
#define HG_RES(TA, V, EX) \
  return launch_resid<CPT, TA, V, EX>(st, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes)
  if (!exact) {
    if (transa) return cudaErrorNotSupported;
    if (vec) return launch_sp<CPT, true>(st, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
    return launch_sp<CPT, false>(st, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
  }
  if (transa) HG_RES(true, false, true);
  if (vec) HG_RES(false, true, true);
  HG_RES(false, false, true);
#undef HG_RES
}

}  // namespace

size_t resid_work_bytes(int m, int nc, int k) {
  const int cw = 4 * pick_cpt(nc);
  const int ncb = (nc + cw - 1) / cw;
  return align256((size_t)ncb * k * cw * sizeof(float4)) + (size_t)kRMaxSlices * m * nc * sizeof(double2);
}

cudaError_t resid_df(cudaStream_t st, bool transa, int m, int nc, int k, const float2* A, long lda, const double2* Y,
                     long ldy, const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws,
                     size_t ws_bytes, bool exact) {
  if (m <= 0 || nc <= 0) return cudaSuccess;
  if (k <= 0) return cudaErrorInvalidValue;
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0) return cudaErrorInvalidValue;
  const bool vec = !transa && reinterpret_cast<uintptr_t>(A) % 16 == 0 && lda % 2 == 0;
  switch (pick_cpt(nc)) {
    case 2: return dispatch<2>(st, transa, vec, exact, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
    case 4: return dispatch<4>(st, transa, vec, exact, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
    case 6: return dispatch<6>(st, transa, vec, exact, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
    case 8: return dispatch<8>(st, transa, vec, exact, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
    default: return dispatch<10>(st, transa, vec, exact, m, nc, k, A, lda, Y, ldy, Bin, ldb, sign, out, ldo, ws, ws_bytes);
  }
}

}  // namespace hg
