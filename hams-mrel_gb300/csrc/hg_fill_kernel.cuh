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

template <bool DEEP, typename OUT>
__global__ void __launch_bounds__(FILL_ROWS)
k_green_fill(const double* __restrict__ rec, const double* __restrict__ fx /* ldf x 3 col-major */, int ldf, int n, int tn,
             FinState fs, int grn_kind, OUT* __restrict__ A, OUT* __restrict__ S, long lda, int* status) {
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
  for (int jj = 0; jj < ncol; ++jj) {
    const double* pr = tile + jj * PR_SIZE;
    const int j = col0 + jj;
    const double xq = pr[PR_XQ], yq = pr[PR_XQ + 1], zq = pr[PR_XQ + 2];
    const double dist = sqrt((xp - xq) * (xp - xq) + (yp - yq) * (yp - yq) + (zp - zq) * (zp - zq));
    const int flag = (dist <= pr[PR_FLAGD]) ? 1 : 0;
    double sij = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0;
    if (flag) newman_pair(pr, xp, yp, zp, sij, d0, d1, d2);
    double2 g[4];
    if (DEEP) inf_green(xq, yq, zq, xp, yp, zp, fs.v, flag, g);
    else fin_green(fs, xq, yq, zq, xp, yp, zp, flag, g);
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
    if (i == j) ar += 2.0 * HG_PI;
    store_c(A + i + (long)j * lda, ar, ai);
    store_c(S + i + (long)j * lda, sr, si);
  }
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
