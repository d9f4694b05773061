// Pair kernel of the Green-function fill, shared by the deep-water
// (hg_fill.cu) and finite-depth (hg_fill_fin.cu) translation units.
#pragma once
#include "hg_common.cuh"
#include "hg_green.cuh"
#include "hg_kernels.cuh"
#include "hg_tma.cuh"

namespace hg {

// ---------------------------------------------------------------------------
// Pair kernel.  CTA = FILL_ROWS field rows x FILL_COLS source columns.  The
// source records of the tile are brought into shared memory with one bulk
// async copy; each thread owns one field row and walks the tile's columns,
// so every warp store of A/S is 32 consecutive complex entries of one column.
// ---------------------------------------------------------------------------
constexpr int FILL_ROWS = 128;
constexpr int FILL_COLS = 16;

// One (field i, source j) pair of the fill: FLAG, Newman integral, Green
// function, assembly of A(i, j) and S(i, j) (the loop body of k_green_fill).
// ndiag: rows below it are collocation points (row i is panel i's centroid)
// and get the free term 2 pi on the diagonal; field points (ndiag = 0) none.
// fpre (finite depth): FINGREEN3D's region-method values at this pair when
// already evaluated (fin_green).
template <bool DEEP, typename OUT>
__device__ __forceinline__ void fill_pair(const double* __restrict__ pr, double xp, double yp, double zp, int i, int j,
                                          const FinState& fs, int grn_kind, OUT* __restrict__ A,
                                          OUT* __restrict__ S, long lda, int ndiag, const double* fpre = nullptr) {
  const double xq = pr[PR_XQ], yq = pr[PR_XQ + 1], zq = pr[PR_XQ + 2];
  const double dist = sqrt((xp - xq) * (xp - xq) + (yp - yq) * (yp - yq) + (zp - zq) * (zp - zq));
  const int flag = (dist <= pr[PR_FLAGD]) ? 1 : 0;
  double sij = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0;
  if (flag) newman_pair(pr, xp, yp, zp, sij, d0, d1, d2);
  double2 g[4];
  if (DEEP) inf_green(xq, yq, zq, xp, yp, zp, fs.v, flag, g);
  else fin_green(fs, xq, yq, zq, xp, yp, zp, flag, g, fpre);
  if (grn_kind == 4) {
    sij = (float)sij; d0 = (float)d0; d1 = (float)d1; d2 = (float)d2;
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = make_double2((float)g[k].x, (float)g[k].y);
  }
  const double ear = pr[PR_DS], n0 = pr[PR_N], n1 = pr[PR_N + 1], n2 = pr[PR_N + 2];
  double ar, ai, sr, si;
  if (flag) {
    ar = (d0 + g[1].x * ear) * n0 + (d1 + g[2].x * ear) * n1 + (d2 + g[3].x * ear) * n2;
    ai = (g[1].y * ear) * n0 + (g[2].y * ear) * n1 + (g[3].y * ear) * n2;
    sr = sij + g[0].x * ear;
  } else {
    ar = (g[1].x * n0 + g[2].x * n1 + g[3].x * n2) * ear;
    ai = (g[1].y * n0 + g[2].y * n1 + g[3].y * n2) * ear;
    sr = g[0].x * ear;
  }
  si = g[0].y * ear;
  if (i == j && i < ndiag) ar += 2.0 * HG_PI;
  store_c(A + i + (long)j * lda, ar, ai);
  store_c(S + i + (long)j * lda, sr, si);
}

// FAST distinguishes the instantiation compiled with fused multiply-adds
// (the mixed form's finite-depth fill) from the one compiled without; the
// code is the same.
template <bool DEEP, typename OUT, int FAST = 0>
__global__ void __launch_bounds__(FILL_ROWS)
k_green_fill(const double* __restrict__ rec, const double* __restrict__ fx /* ldf x 3 col-major */, int ldf, int n, int tn,
             FinState fs, int grn_kind, OUT* __restrict__ A, OUT* __restrict__ S, long lda, int* status, int ndiag) {
  __shared__ alignas(128) double tile[FILL_COLS * PR_SIZE];
  __shared__ alignas(8) uint64_t bar;
  const int col0 = blockIdx.y * FILL_COLS;
  const int ncol = min(FILL_COLS, n - col0);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_expect_tx(&bar, (uint32_t)(ncol * PR_SIZE * sizeof(double)));
    bulk_g2s(tile, rec + (size_t)col0 * PR_SIZE, (uint32_t)(ncol * PR_SIZE * sizeof(double)), &bar);
  }
  __syncthreads();
  if (!mbar_wait_timed(&bar, 0, 2000000000ull)) {
    hg_set_status(status, HG_DEV_WAIT_TIMEOUT);
    mbar_wait_timed(&bar, 0, 2000000000ull);  // drain the copy before shared memory goes away
    return;
  }
  const int i = blockIdx.x * FILL_ROWS + threadIdx.x;
  if (i >= tn) return;
  const double xp = fx[i], yp = fx[i + ldf], zp = fx[i + 2 * (size_t)ldf];
  for (int jj = 0; jj < ncol; ++jj)
    fill_pair<DEEP, OUT>(tile + jj * PR_SIZE, xp, yp, zp, i, col0 + jj, fs, grn_kind, A, S, lda, ndiag);
}

// ---------------------------------------------------------------------------
// Finite depth, pairs binned by cost.  FINGREEN3D (FinGreen3D.f90:81-155)
// branches per pair on R/h into methods whose costs differ by orders of
// magnitude (LINTON's adaptive quadrature, PIDCOCK's and EIGENE's 10-100-term
// series with Wynn extrapolation, EIGEN's <= 10 terms).  In the tiled kernel
// one expensive pair holds up the 31 other threads of its warp; here the
// pairs are first sorted into kFinBins bins by method and series length
// (counting pass, scan, scatter pass), and the evaluation kernel then walks
// the bins in order, one pair per thread, so that a warp's pairs cost about
// the same.  Each result goes to its own (i, j), so the order inside a bin
// (set by atomics) does not affect the matrices.
// ---------------------------------------------------------------------------
constexpr int kFinBins = 16;
constexpr int kFinNearBins = 8;  // bins 0..7: LINTON and PIDCOCK (R/h < 0.05)

__device__ __forceinline__ int fin_bin(const FinState& fs, double rr) {
  const double v = fs.v;
  if (fabs(v) < SPD(1.e-8) || fabs(v + 1.0) < SPD(1.e-8)) return kFinBins - 1;  // closed forms
  const double rhp = fabs(rr / fs.h);
  if (rhp < 0.0005) return 0;                                                    // LINTON
  if (rhp < 0.05) {                                                              // PIDCOCK, 50-100 terms
    const int nt = (int)(SPD(-1010.10) * rhp + SPD(100.50));
    return 1 + min(6, max(0, (100 - nt) / 8));
  }
  if (rhp < 0.5) {                                                               // EIGENE, 10-50 terms
    const int nt = (int)(SPD(-88.89) * rhp + SPD(54.45));
    return 8 + min(5, max(0, (54 - nt) / 8));
  }
  return 14;                                                                     // EIGEN
}

// Pass 1 (scatter = false): bin counts; pass 2 (scatter = true): pair index
// i + j * tn appended to its bin at cursor[bin] (warp-aggregated atomics).
// Pairs whose bin is maxbin or above are left out of both passes.
template <bool SCATTER>
__global__ void k_fin_bins(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int n, int tn,
                           FinState fs, int maxbin, int* __restrict__ counts, int* __restrict__ list) {
  __shared__ int hist[kFinBins];
  if (!SCATTER && threadIdx.x < kFinBins) hist[threadIdx.x] = 0;
  if (!SCATTER) __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  int b = kFinBins;
  if (i < tn) {
    const double* pr = rec + (size_t)j * PR_SIZE;
    const double dx = pr[PR_XQ] - fx[i], dy = pr[PR_XQ + 1] - fx[i + ldf];
    b = fin_bin(fs, sqrt(dx * dx + dy * dy));
  }
  const bool ok = b < maxbin;
  const unsigned act = __ballot_sync(0xffffffffu, ok);
  if (ok) {
    const unsigned peers = __match_any_sync(act, b);
    const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (!SCATTER) {
      if (lane == leader) atomicAdd(&hist[b], __popc(peers));
    } else {
      int base = 0;
      if (lane == leader) base = atomicAdd(&counts[b], __popc(peers));
      base = __shfl_sync(peers, base, leader);
      list[base + rank] = i + j * tn;
    }
  }
  if (!SCATTER) {
    __syncthreads();
    if (threadIdx.x < kFinBins && hist[threadIdx.x]) atomicAdd(&counts[threadIdx.x], hist[threadIdx.x]);
  }
}

// counts -> cursors (exclusive prefix sums), one thread.
static __global__ void k_fin_scan(int* __restrict__ counts) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < kFinBins; ++b) {
      const int c = counts[b];
      counts[b] = acc;
      acc += c;
    }
  }
}

// npairs: list length, or (listed != nullptr) read from *listed, the last
// bin's cursor after the scatter pass when only some bins were listed.
template <typename OUT, int FAST>
__global__ void __launch_bounds__(128)
k_green_fill_binned(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int tn, long npairs,
                    const int* __restrict__ listed, const int* __restrict__ list, FinState fs, int grn_kind,
                    OUT* __restrict__ A, OUT* __restrict__ S, long lda, int ndiag) {
  if (listed) npairs = *listed;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < npairs; k += (long)gridDim.x * blockDim.x) {
    const int p = list[k];
    const int i = p % tn, j = p / tn;
    fill_pair<false, OUT>(rec + (size_t)j * PR_SIZE, fx[i], fx[i + ldf], fx[i + 2 * (size_t)ldf], i, j, fs, grn_kind,
                          A, S, lda, ndiag);
  }
}

// maxbin < kFinBins evaluates only the pairs of bins below it (the others
// keep what A and S hold).
template <typename OUT, int FAST>
cudaError_t launch_fin_binned(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                              const FinState& fs, int grn_kind, OUT* A, OUT* S, long lda, int* bins, int ndiag,
                              int maxbin = kFinBins) {
  int* counts = bins;
  int* list = bins + kFinBins;
  cudaError_t e = cudaMemsetAsync(counts, 0, kFinBins * sizeof(int), st);
  if (e != cudaSuccess) return e;
  const dim3 cg((tn + 127) / 128, n);
  k_fin_bins<false><<<cg, 128, 0, st>>>(rec, fx, ldf, n, tn, fs, maxbin, counts, list);
  k_fin_scan<<<1, 32, 0, st>>>(counts);
  k_fin_bins<true><<<cg, 128, 0, st>>>(rec, fx, ldf, n, tn, fs, maxbin, counts, list);
  const long np = (long)tn * n;
  long blocks = (np + 127) / 128;
  if (blocks > 152L * 64) blocks = 152L * 64;
  const int* listed = (maxbin < kFinBins) ? counts + (maxbin - 1) : nullptr;
  k_green_fill_binned<OUT, FAST><<<(unsigned)blocks, 128, 0, st>>>(rec, fx, ldf, tn, np, listed, list, fs, grn_kind, A,
                                                                  S, lda, ndiag);
  return cudaGetLastError();
}

// Green function at arbitrary points (kernel-level parity tests of every
// region): pts[k] = (xq,yq,zq,xp,yp,zp), out[k] = 4 complex.
template <bool DEEP>
__global__ void k_green_points(int npts, const double* __restrict__ pts, const int* __restrict__ flags, FinState fs,
                               double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npts) return;
  const double* p = pts + 6 * (size_t)k;
  double2 g[4];
  if (DEEP) inf_green(p[0], p[1], p[2], p[3], p[4], p[5], fs.v, flags[k], g);
  else fin_green(fs, p[0], p[1], p[2], p[3], p[4], p[5], flags[k], g);
  for (int q = 0; q < 4; ++q) { out[8 * (size_t)k + 2 * q] = g[q].x; out[8 * (size_t)k + 2 * q + 1] = g[q].y; }
}

}  // namespace hg
