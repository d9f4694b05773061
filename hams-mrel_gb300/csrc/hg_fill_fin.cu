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

cudaError_t launch_green_points_fin(cudaStream_t st, int npts, const double* pts, const int* flags, const FinState& fs,
                                    double* out) {
  k_green_points<false><<<(npts + 63) / 64, 64, 0, st>>>(npts, pts, flags, fs, out);
  return cudaGetLastError();
}

}  // namespace hg
