// Finite-depth pair kernel for the mixed form, compiled with fused
// multiply-adds.  The same code as hg_fill_fin.cu; contraction changes the
// FP64 results by about 1e-7 of their size (the reference's own spread
// between equally valid builds, through the epsilon extrapolation of
// FinGrnExtSubs.f90:370-503), below the single precision the mixed form
// stores, and saves the separate multiply and add instructions on GB300's
// FP64 pipes, which bound this kernel.
#include "hg_fill_kernel.cuh"

namespace hg {

cudaError_t launch_green_fill_fin_fma(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                      const FinState& fs, int grn_kind, float2* A, float2* S, long lda, int* status,
                                      int* bins) {
  if (bins) return launch_fin_binned<float2, 1>(st, rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, bins, tn);
  dim3 grid((tn + FILL_ROWS - 1) / FILL_ROWS, (n + FILL_COLS - 1) / FILL_COLS);
  k_green_fill<false, float2, 1><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, status, tn);
  return cudaGetLastError();
}

}  // namespace hg
