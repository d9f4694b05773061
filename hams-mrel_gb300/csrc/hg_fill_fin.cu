// Finite-depth instantiations of the pair kernel.  This translation unit
// is compiled with -fmad=false: the Wynn epsilon extrapolation of the
// finite-depth series (Limes, src/FinGrnExtSubs.f90:370-503) divides by
// differences of nearly converged partial sums, so a fused multiply-add
// anywhere upstream changes its result far beyond one rounding; with
// separately rounded products the series reproduce the reference's
// arithmetic.  The mixed form, whose matrices are single precision, uses the
// instantiation of hg_fill_fin_fma.cu instead (same code, contracted).
#include "hg_fill_kernel.cuh"

namespace hg {

// bins: device scratch of fin_bins_ints(n, tn) ints (pairs binned by cost,
// hg_fill_kernel.cuh); without it the tiled kernel runs.
template <typename OUT>
cudaError_t launch_green_fill_fin(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                  const FinState& fs, int grn_kind, OUT* A, OUT* S, long lda, int* status, int* bins,
                                  int ndiag) {
  if (bins) return launch_fin_binned<OUT, 0>(st, rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, bins, ndiag);
  dim3 grid((tn + FILL_ROWS - 1) / FILL_ROWS, (n + FILL_COLS - 1) / FILL_COLS);
  k_green_fill<false, OUT><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, status, ndiag);
  return cudaGetLastError();
}
template cudaError_t launch_green_fill_fin<double2>(cudaStream_t, const double*, const double*, int, int, int,
                                                    const FinState&, int, double2*, double2*, long, int*, int*, int);
template cudaError_t launch_green_fill_fin<float2>(cudaStream_t, const double*, const double*, int, int, int,
                                                   const FinState&, int, float2*, float2*, long, int*, int*, int);

// The pairs below R/h = 0.05 (FINGREEN3D's LINTON and PIDCOCK methods,
// FinGreen3D.f90:182-191) evaluated per pair with the reference's
// arithmetic and written over what A and S hold; the other pairs are left
// alone.  The mixed form's tabulated fill calls this after the tables:
// LINTON's adaptive quadrature and PIDCOCK's epsilon-extrapolated series
// make the reference's values in those bands jump with R and depth by far
// more than a smooth interpolation can follow, so only a per-pair
// evaluation reproduces them.
cudaError_t launch_fin_near(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                            const FinState& fs, int grn_kind, float2* A, float2* S, long lda, int* bins, int ndiag) {
  return launch_fin_binned<float2, 0>(st, rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, bins, ndiag, kFinNearBins);
}

// ---------------------------------------------------------------------------
// The same near pairs with their region-method values de-duplicated.  A
// pair's FINGREEN3D_R value depends only on (R, zq, zp); meshes with
// symmetries repeat these triples bit for bit (all the vertically stacked
// pairs at R = 0, mirror-image pairs, equal bodies at offsets that round
// alike), so the near pairs are keyed by (the bits of R as the pair kernel
// computes it, the index of zq and of zp among the mesh's distinct depths)
// once per mesh and depth, the region methods run once per key per
// frequency, and each pair assembles its A and S entries from its key's
// values (fill_pair with the values given; the Newman integral, the
// Rankine pair and the assembly stay per pair).  Keys are exact: two pairs
// share values only where the reference computes the same function of the
// same three numbers.  (Rounding R to share more keys is not an option: the
// epsilon-extrapolated series turn last-bit changes of R into changes of
// the value that average out over the many pairs of a matrix only while each
// pair keeps its own.)  Two hash tables of 64-bit keys: R's bits -> slot r,
// then (r, zq index, zp index) -> slot of the key.
// ---------------------------------------------------------------------------
namespace {

constexpr unsigned long long kNearEmpty = ~0ull;

__device__ __forceinline__ unsigned near_hash(unsigned long long k, unsigned mask) {
  k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
  return (unsigned)k & mask;
}

// Slot of key in an open-addressing table of mask + 1 slots (inserted if
// absent); the table holds fewer keys than half its slots, so one is found.
__device__ __forceinline__ unsigned near_insert(unsigned long long* tab, unsigned mask, unsigned long long key) {
  unsigned s = near_hash(key, mask);
  for (unsigned probe = 0; probe <= mask; ++probe) {
    const unsigned long long prev = atomicCAS(&tab[s], kNearEmpty, key);
    if (prev == kNearEmpty || prev == key) break;
    s = (s + 1) & mask;
  }
  return s;
}

// R/h < 0.05 band (bins 0..7 of fin_bin for a non-special frequency)
__device__ __forceinline__ int near_bin(double rhp) {
  if (rhp < 0.0005) return 0;
  const int nt = (int)(SPD(-1010.10) * rhp + SPD(100.50));
  return 1 + min(6, max(0, (100 - nt) / 8));
}

// INSERT = false: count the near pairs; true: insert their keys and list
// them as (pair index i + j tn, key slot).  R as fin_green computes it.
template <bool INSERT>
__global__ void k_near_pairs(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int n, int tn,
                             double h, const short* __restrict__ zsrc, const short* __restrict__ zfld,
                             unsigned long long* __restrict__ tabr, unsigned long long* __restrict__ tabk,
                             unsigned mask, int* __restrict__ counter, int2* __restrict__ pairs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  bool near = false;
  double rr = 0.0;
  if (i < tn) {
    const double* pr = rec + (size_t)j * PR_SIZE;
    const double xpq = pr[PR_XQ] - fx[i], ypq = pr[PR_XQ + 1] - fx[i + ldf];
    rr = sqrt(xpq * xpq + ypq * ypq);
    near = fabs(rr / h) < 0.05;
  }
  const unsigned act = __ballot_sync(0xffffffffu, near);
  if (!act) return;
  const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(act));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!INSERT || !near) return;
  const unsigned sr = near_insert(tabr, mask, (unsigned long long)__double_as_longlong(rr));
  const unsigned long long key = ((unsigned long long)sr << 22) | ((unsigned long long)zsrc[j] << 11) |
                                 (unsigned long long)zfld[i];
  const unsigned sk = near_insert(tabk, mask, key);
  pairs[base + __popc(act & ((1u << lane) - 1u))] = make_int2(i + j * tn, (int)sk);
}

// Occupied key slots -> keys (R's bits, depth indices), grouped by the
// near_bin of their R (pass 1 counts, pass 2 scatters at the bins'
// cursors); slot2u[slot] = key index.
template <bool SCATTER>
__global__ void k_near_unique(const unsigned long long* __restrict__ tabr, const unsigned long long* __restrict__ tabk,
                              unsigned cap, double h, int* __restrict__ cursor, int* __restrict__ slot2u,
                              longlong2* __restrict__ ukeys) {
  const unsigned s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  const unsigned long long key = tabk[s];
  if (key == kNearEmpty) return;
  const unsigned long long rbits = tabr[key >> 22];
  const int b = near_bin(fabs(__longlong_as_double((long long)rbits) / h));
  if (!SCATTER) {
    atomicAdd(&cursor[b], 1);
  } else {
    const int u = atomicAdd(&cursor[b], 1);
    slot2u[s] = u;
    ukeys[u] = make_longlong2((long long)rbits, (long long)(key & 0x3FFFFFull));
  }
}

__global__ void k_near_map(int np, int2* __restrict__ pairs, const int* __restrict__ slot2u) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < np) pairs[k].y = slot2u[pairs[k].y];
}

// Region-method values per key (FINGREEN3D_R, FinGreen3D.f90:160-226).
__global__ void k_near_eval(int nu, const longlong2* __restrict__ ukeys, const double* __restrict__ zlev, FinState fs,
                            double* __restrict__ F) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nu) return;
  const longlong2 key = ukeys[u];
  double f[6];
  fin_regions(fs, __longlong_as_double(key.x), zlev[(key.y >> 11) & 2047], zlev[key.y & 2047], f);
  for (int q = 0; q < 6; ++q) F[6 * (size_t)u + q] = f[q];
}

__global__ void __launch_bounds__(128)
k_near_fill(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int tn, int np,
            const int2* __restrict__ pairs, const double* __restrict__ F, FinState fs, int grn_kind,
            float2* __restrict__ A, float2* __restrict__ S, long lda, int ndiag) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    const int2 pu = pairs[k];
    const int i = pu.x % tn, j = pu.x / tn;
    fill_pair<false, float2>(rec + (size_t)j * PR_SIZE, fx[i], fx[i + ldf], fx[i + 2 * (size_t)ldf], i, j, fs,
                             grn_kind, A, S, lda, ndiag, F + 6 * (size_t)pu.y);
  }
}

}  // namespace

int near_count(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double h,
               const short* zsrc, const short* zfld, int* counter) {
  if (cudaMemsetAsync(counter, 0, sizeof(int), st) != cudaSuccess) return -1;
  const dim3 g((tn + 127) / 128, n);
  k_near_pairs<false><<<g, 128, 0, st>>>(rec, fx, ldf, n, tn, h, zsrc, zfld, nullptr, nullptr, 0, counter, nullptr);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

unsigned near_table_size(int npairs) {
  unsigned cap = 4096;
  while (cap < 2u * (unsigned)npairs) cap <<= 1;
  return cap;
}

cudaError_t near_build(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double h,
                       const short* zsrc, const short* zfld, unsigned long long* tabr, unsigned long long* tabk,
                       unsigned cap, int* counters, int* slot2u, int2* pairs, longlong2* ukeys) {
  cudaError_t e = cudaMemsetAsync(tabr, 0xff, (size_t)cap * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(tabk, 0xff, (size_t)cap * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, (1 + kFinBins) * sizeof(int), st);
  if (e != cudaSuccess) return e;
  const dim3 g((tn + 127) / 128, n);
  k_near_pairs<true><<<g, 128, 0, st>>>(rec, fx, ldf, n, tn, h, zsrc, zfld, tabr, tabk, cap - 1, counters, pairs);
  int* cursor = counters + 1;
  k_near_unique<false><<<(cap + 255) / 256, 256, 0, st>>>(tabr, tabk, cap, h, cursor, slot2u, ukeys);
  k_fin_scan<<<1, 32, 0, st>>>(cursor);
  k_near_unique<true><<<(cap + 255) / 256, 256, 0, st>>>(tabr, tabk, cap, h, cursor, slot2u, ukeys);
  return cudaGetLastError();
}

cudaError_t near_map(cudaStream_t st, int np, int2* pairs, const int* slot2u) {
  if (np > 0) k_near_map<<<(np + 255) / 256, 256, 0, st>>>(np, pairs, slot2u);
  return cudaGetLastError();
}

cudaError_t near_fill(cudaStream_t st, const double* rec, const double* fx, int ldf, int tn, int np, int nu,
                      const int2* pairs, const longlong2* ukeys, const double* zlev, double* F, const FinState& fs,
                      int grn_kind, float2* A, float2* S, long lda, int ndiag) {
  if (nu > 0) k_near_eval<<<(nu + 63) / 64, 64, 0, st>>>(nu, ukeys, zlev, fs, F);
  if (np > 0) {
    int blocks = (np + 127) / 128;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_near_fill<<<blocks, 128, 0, st>>>(rec, fx, ldf, tn, np, pairs, F, fs, grn_kind, A, S, lda, ndiag);
  }
  return cudaGetLastError();
}

cudaError_t launch_green_points_fin(cudaStream_t st, int npts, const double* pts, const int* flags, const FinState& fs,
                                    double* out) {
  k_green_points<false><<<(npts + 63) / 64, 64, 0, st>>>(npts, pts, flags, fs, out);
  return cudaGetLastError();
}

}  // namespace hg
