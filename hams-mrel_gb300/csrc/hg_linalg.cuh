// Dense complex linear algebra for the per-frequency solve: blocked
// right-looking LU with partial pivoting (the ZGETRF/CGETRF of
// AssbMatx.f90:111) and the triangular solves of ZGETRS (AssbMatx.f90:277),
// in complex128 (plain form) and complex64 (mixed form).
#pragma once
#include <cuda_runtime.h>
#include "hg_common.cuh"

namespace hg {

template <typename R> struct cx;
template <> struct cx<double> { typedef double2 T; };
template <> struct cx<float> { typedef float2 T; };

// C = alpha * op(A) * B + beta * C, column-major, op(A) = A or A^T (no
// conjugation: the irregular-frequency normal equations use A^T A,
// AssbMatx_irr.f90:151-169).  M x N result, inner dimension K.
template <typename R>
cudaError_t gemm(cudaStream_t st, bool transa, int m, int n, int k, typename cx<R>::T alpha,
                 const typename cx<R>::T* A, long lda, const typename cx<R>::T* B, long ldb,
                 typename cx<R>::T beta, typename cx<R>::T* C, long ldc, void* ws = nullptr,
                 size_t ws_bytes = 0);

// Complex64 GEMM for wide outputs (hg_gemm32.cu): same contract as gemm<float>
// without split-K; used by gemm<float> when N > 64.
cudaError_t cgemm_wide(cudaStream_t st, bool transa, int m, int n, int k, float2 alpha, const float2* A, long lda,
                       const float2* B, long ldb, float2 beta, float2* C, long ldc);

// out = Bin + sign * op(A) Y (hg_resid.cu): A complex64 (exact entries), Y and
// Bin complex128 (Bin may be null), result complex128 in double-float
// arithmetic on the FP32 pipes.  M x NC result, inner dimension K.  ws: a
// 256-byte aligned device workspace of at least resid_work_bytes(m, nc, k).
// exact = false: single-precision products and 32-term partial sums,
// compensated across partial sums (untransposed A only).
size_t resid_work_bytes(int m, int nc, int k);
cudaError_t resid_df(cudaStream_t st, bool transa, int m, int nc, int k, const float2* A, long lda, const double2* Y,
                     long ldy, const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws,
                     size_t ws_bytes, bool exact = true);

// The same product as resid_df (exact mode, untransposed A) on the tensor
// cores by exact operand slicing (hg_resid_tc.cu): about 2^-42 of sum |a||y|
// per entry.  nc <= 40; ws: 256-byte aligned, at least resid_tc_work_bytes;
// status receives a timeout code if a bounded wait runs out.
bool resid_tc_supported();
size_t resid_tc_work_bytes(int m, int nc, int k);
cudaError_t resid_tc(cudaStream_t st, int m, int nc, int k, const float2* A, long lda, const double2* Y, long ldy,
                     const double2* Bin, long ldb, double sign, double2* out, long ldo, void* ws, size_t ws_bytes,
                     int* status);

// Complex64 GEMM for N <= 48 untransposed (hg_gemm32.cu), without split-K.
cudaError_t cgemm_skinny(cudaStream_t st, int m, int n, int k, float2 alpha, const float2* A, long lda,
                         const float2* B, long ldb, float2 beta, float2* C, long ldc);

// In-place LU with partial pivoting of the n x n matrix A (lda).  ipiv is a
// device array of n 1-based pivot rows, LAPACK style.  info (device int) is
// set to the first zero pivot (1-based) or left at 0 (a negative value: a
// bounded device wait ran out).  Complex64: tc_passes = 3, 2 or 1 runs the
// trailing updates of 256-wide outer panels on the tensor cores (cgemm_tc:
// 3xTF32, split BF16 or TF32) with work a 256-byte aligned device scratch of
// at least lu_work_bytes(n, tc_passes) bytes.  Complex128: any tc_passes != 0
// runs U12 and the trailing updates of 256-wide outer panels as exact BF16
// digit products (zgemm_tc) with work of at least lu_work_bytes_z(n) bytes.
// tc_passes = 0 keeps every update on the SIMT kernels (work unused).
//
// Look-ahead (aux, optional): a second stream of lower priority and two
// events.  After each 32-column panel only the next panel's 32 columns are
// updated on st; the update of the remaining columns runs on aux->side while
// the next panel is factorised on st (the interchanges of that panel wait for
// it).  The arithmetic of every entry is that of the same update in one
// launch split by columns.
struct LuAux {
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_side = nullptr;
};
template <typename R>
cudaError_t getrf(cudaStream_t st, int n, typename cx<R>::T* A, long lda, int* ipiv, int* info, void* work,
                  size_t work_bytes = 0, int tc_passes = 0, const LuAux* aux = nullptr);

// Solve A X = B with the factors of getrf; B is n x nrhs (ldb), overwritten.
// Complex128 with work (256-byte aligned, at least zgemm_tc_work_bytes(n,
// nrhs, 256) bytes) and a device status word: the block updates run as exact
// digit products on the tensor cores (zgemm_tc); otherwise on the SIMT GEMM.
template <typename R>
cudaError_t getrs(cudaStream_t st, int n, int nrhs, const typename cx<R>::T* LU, long lda, const int* ipiv,
                  typename cx<R>::T* B, long ldb, void* work = nullptr, size_t work_bytes = 0, int* status = nullptr);

size_t lu_work_bytes(int n, int tc_passes);
size_t lu_work_bytes_z(int n);

// H-matrix of the iterative solver's matrix (hg_hmatrix.cu; the reference's
// src/HMatrix.f90): cluster and block trees of the panel centres xyz
// (n x 3, column-major), ACA-compressed admissible blocks (1e-4, rank <= 50),
// dense near-field blocks, all in complex128; M (complex128) or Mf
// (complex64) is the assembled n x n matrix (leading dimension ld), read
// only by build.  matvec: W = Bin + sign * H Z for nc columns (Bin may be
// null; leading dimensions ldz, ldb, ldw).
struct HMatrixStats {
  int nblocks = 0, ndense = 0, nlowrank = 0;
  long long rank_sum = 0;
  double bytes = 0.0;  // storage of the blocks
};
// Device bytes of the H-matrix of n panels with centres xyz and of its
// product with nc columns: the ACA factors at their maximum rank, the dense
// near-field blocks and the scratch, from the host trees (admissible blocks
// assumed to compress).
size_t hmatrix_bytes_estimate(int n, const double* xyz, int nc);
// The host trees alone: the cluster permutation (n) and up to max_blocks
// blocks as (row start, rows, column start, columns, admissible); returns
// the block count.
int hmatrix_partition(int n, const double* xyz, int* perm, int* blocks, int max_blocks);
class HMatrix {
 public:
  HMatrix();
  ~HMatrix();
  HMatrix(const HMatrix&) = delete;
  HMatrix& operator=(const HMatrix&) = delete;
  cudaError_t build(cudaStream_t st, int n, const double2* M, const float2* Mf, long ld, const double* xyz);
  cudaError_t matvec(cudaStream_t st, int nc, const double2* Z, long ldz, const double2* Bin, long ldb, double sign,
                     double2* W, long ldw);
  HMatrixStats stats() const;
  struct Impl;

 private:
  Impl* p;
};

// Complex128 C -= op(A) B on the tcgen05 tensor cores, FP64-accurate, by
// exact BF16 digit slicing of both operands (hg_zgemm_tc.cu): op(A) = A
// (m x k, lda) or, with transa, A^T of the k x m matrix A (lda, no
// conjugation); B k x n (ldb), C m x n (ldc), column-major; B may alias C (B
// is sliced before C is written), A may not.  About 2^-48 of each output plus 2^-57 of sum |a||b|.
// ws: 256-byte aligned device scratch of zgemm_tc_work_bytes(m, n, k) bytes.
// status (device int) receives -1000 if a bounded wait ran out.
bool zgemm_tc_supported();
size_t zgemm_tc_work_bytes(int m, int n, int k);
cudaError_t zgemm_tc(cudaStream_t st, int m, int n, int k, const double2* A, long lda, const double2* B, long ldb,
                     double2* C, long ldc, void* ws, size_t ws_bytes, int* status, bool transa = false);

// getrs for the complex64 factors of a two-level getrf (tc_passes != 0):
// uses the inverses of the 256 x 256 diagonal blocks that getrf kept in its
// workspace.  lu_has_inverses tells whether getrf took that path.
bool lu_has_inverses(int n, int tc_passes, size_t work_bytes);
cudaError_t getrs_inv(cudaStream_t st, int n, int nrhs, const float2* LU, long lda, const int* ipiv, float2* B,
                      long ldb, void* work);

// Complex64 C -= A B on the tcgen05 tensor cores (hg_tc.cu): A m x k (lda),
// B k x n (ldb), C m x n (ldc), column-major.  passes 3: split-TF32 products
// (single-precision quality); passes 1: plain TF32.  ws: 256-byte aligned
// device scratch of cgemm_tc_work_bytes(m, n, k) bytes for the packed
// operands.  status (device int) receives -1000 if a bounded wait ran out.
bool cgemm_tc_supported();
size_t cgemm_tc_work_bytes(int m, int n, int k);
cudaError_t cgemm_tc(cudaStream_t st, int passes, int m, int n, int k, const float2* A, long lda, const float2* B,
                     long ldb, float2* C, long ldc, void* ws, size_t ws_bytes, int* status);

// Panel LU on a 16-CTA cluster (hg_lu_cluster.cu): rows [0, m) x columns
// [0, jb <= 32) of P, pivots written 1-based as k0 + row + 1.
template <typename R>
cudaError_t panel_cluster(cudaStream_t st, typename cx<R>::T* P, long lda, int m, int jb, int* ipiv, int k0, int* info);
template <>
cudaError_t panel_cluster<float>(cudaStream_t st, float2* P, long lda, int m, int jb, int* ipiv, int k0, int* info);
template <>
cudaError_t panel_cluster<double>(cudaStream_t st, double2* P, long lda, int m, int jb, int* ipiv, int k0, int* info);
// Whether the cluster panel runs here for m rows and panels of jb columns.
template <typename R>
bool panel_cluster_supported(int m, int jb = 32);
// Column-parallel triangular solve of a jb <= 256 diagonal block for ncols columns.
template <typename R>
cudaError_t trsm_cols(cudaStream_t st, bool upper, const typename cx<R>::T* A, long lda, int jb,
                      typename cx<R>::T* X, long ldx, int ncols);

// Inverses of the diagonal nb x nb blocks nblk_first .. nblk_first + nblk - 1
// of the n x n factor A (unit lower triangle, or upper triangle), in one
// launch: block b's inverse goes to X + b nb ldx (an nb x nb block with
// leading dimension ldx; the last block of order n - b nb if smaller).
template <typename R>
cudaError_t trsm_inverse_blocks(cudaStream_t st, bool upper, const typename cx<R>::T* A, long lda, int n, int nb,
                                typename cx<R>::T* X, long ldx, int nblk_first, int nblk);

// Column-batched FP64 vector kernels of the GMRES refinement (hg_gmres.cu).
// Blocks V_i = V + i vstride are n x nc (leading dimension ldv).
//   col_dots:  H[i + c ldh] = V_i[:, c]^H W[:, c], i < nv
//   col_axpy:  W[:, c] += sign sum_{i < nv} H[i + c ldh] V_i[:, c]
//   col_norm2: out[c] = ||W[:, c]||_2;  col_scale: out[:, c] = W[:, c] / s[c]
cudaError_t col_dots(cudaStream_t st, int n, int nc, int nv, const double2* V, long ldv, long vstride, const double2* W,
                     long ldw, double2* H, int ldh);
cudaError_t col_axpy(cudaStream_t st, int n, int nc, int nv, const double2* V, long ldv, long vstride,
                     const double2* H, int ldh, double2* W, long ldw, double sign);
cudaError_t col_norm2(cudaStream_t st, int n, int nc, const double2* W, long ldw, double* out);
// Jacobi preconditioner of the iterative solver: d = diag(M) (1 where
// |M_ii| < 1e-30), Z = V ./ d column by column.
cudaError_t diag_extract(cudaStream_t st, int n, const double2* M, long ldm, double2* d);
cudaError_t diag_extract(cudaStream_t st, int n, const float2* M, long ldm, double2* d);
cudaError_t jacobi_apply(cudaStream_t st, int n, int nc, const double2* V, long ldv, const double2* d, double2* Z,
                         long ldz);
cudaError_t col_scale(cudaStream_t st, int n, int nc, const double2* W, long ldw, const double* s, double2* out,
                      long ldo);
cudaError_t convert_c2z_2d(cudaStream_t st, int rows, int cols, const float2* src, long lds, double2* dst, long ldd);

// Elementwise conversions between complex128 and complex64 buffers.
cudaError_t convert_z2c(cudaStream_t st, long count, const double2* src, float2* dst);
cudaError_t convert_c2z(cudaStream_t st, long count, const float2* src, double2* dst);
// 2D (column-major) versions with leading dimensions.
cudaError_t convert_z2c_2d(cudaStream_t st, int rows, int cols, const double2* src, long lds, float2* dst,
                           long ldd);
cudaError_t add_c2z_2d(cudaStream_t st, int rows, int cols, const float2* src, long lds, double2* dst, long ldd);

}  // namespace hg
