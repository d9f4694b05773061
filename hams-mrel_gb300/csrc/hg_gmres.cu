// Column-batched vector kernels of the GMRES-based refinement (the restarted
// GMRES of IterativeSolvers.f90:324-488, ZGMRES_SOLVE, run for all right-hand
// sides of a frequency at once, each column with its own Krylov basis).
//
// Krylov vectors are n x nc complex128 blocks (column c = right-hand side c)
// stored one after another: V_i = V + i * vstride, leading dimension ldv.
// Orthogonalisation is classical Gram-Schmidt applied twice (two passes of
// all inner products then one combined update), which keeps the basis as
// orthogonal as modified Gram-Schmidt does while every pass is one launch.
// All reductions are deterministic: one CTA per (column, vector) pair sums
// its column in a fixed order.
#include "hg_linalg.cuh"

namespace hg {
namespace {

constexpr int kVThreads = 256;

__device__ __forceinline__ double2 block_sum2(double2 v) {
  __shared__ double2 sm[kVThreads / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, off);
    v.y += __shfl_down_sync(0xffffffffu, v.y, off);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sm[w] = v;
  __syncthreads();
  double2 t = make_double2(0.0, 0.0);
  if (threadIdx.x == 0) {
    for (int k = 0; k < kVThreads / 32; ++k) { t.x += sm[k].x; t.y += sm[k].y; }
  }
  return t;  // valid in thread 0
}

// H[i + c * ldh] = sum_r conj(V_i[r, c]) W[r, c]; grid (nc, nv).
__global__ void __launch_bounds__(kVThreads)
k_col_dots(int n, const double2* __restrict__ V, long ldv, long vstride, const double2* __restrict__ W, long ldw,
           double2* __restrict__ H, int ldh) {
  const int c = blockIdx.x, i = blockIdx.y;
  const double2* v = V + i * vstride + (long)c * ldv;
  const double2* w = W + (long)c * ldw;
  double2 acc = make_double2(0.0, 0.0);
  for (int r = threadIdx.x; r < n; r += kVThreads) {
    const double2 a = v[r], b = w[r];
    acc.x += a.x * b.x + a.y * b.y;
    acc.y += a.x * b.y - a.y * b.x;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) H[i + (long)c * ldh] = acc;
}

// W[:, c] -= sum_{i < nv} H[i + c ldh] V_i[:, c]; grid (row blocks, nc).
__global__ void k_col_axpy(int n, int nv, const double2* __restrict__ V, long ldv, long vstride,
                           const double2* __restrict__ H, int ldh, double2* __restrict__ W, long ldw, double sign) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= n) return;
  double2 w = W[r + (long)c * ldw];
  for (int i = 0; i < nv; ++i) {
    const double2 h = H[i + (long)c * ldh];
    const double2 v = V[i * vstride + r + (long)c * ldv];
    w.x += sign * (h.x * v.x - h.y * v.y);
    w.y += sign * (h.x * v.y + h.y * v.x);
  }
  W[r + (long)c * ldw] = w;
}

// out[c] = ||W[:, c]||_2; grid nc.
__global__ void __launch_bounds__(kVThreads)
k_col_norm2(int n, const double2* __restrict__ W, long ldw, double* __restrict__ out) {
  const int c = blockIdx.x;
  double2 acc = make_double2(0.0, 0.0);
  for (int r = threadIdx.x; r < n; r += kVThreads) {
    const double2 a = W[r + (long)c * ldw];
    acc.x += a.x * a.x + a.y * a.y;
  }
  acc = block_sum2(acc);
  if (threadIdx.x == 0) out[c] = sqrt(acc.x);
}

// out[:, c] = W[:, c] / s[c] (0 where s[c] is 0).
__global__ void k_col_scale(int n, const double2* __restrict__ W, long ldw, const double* __restrict__ s,
                            double2* __restrict__ out, long ldo) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= n) return;
  const double d = s[c];
  const double inv = d > 0.0 ? 1.0 / d : 0.0;
  const double2 w = W[r + (long)c * ldw];
  out[r + (long)c * ldo] = make_double2(w.x * inv, w.y * inv);
}

__global__ void k_c2z_cols(int rows, const float2* __restrict__ s, long lds, double2* __restrict__ d, long ldd) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r < rows) {
    const float2 v = s[r + (long)c * lds];
    d[r + (long)c * ldd] = make_double2(v.x, v.y);
  }
}

// d[i] = M[i, i] widened to complex128, with 1 where |M[i, i]| < 1e-30:
// the Jacobi preconditioner of the iterative solver (SETUP_PRECONDITIONER,
// IterativeSolvers.f90:156-174).
template <typename T>
__global__ void k_diag(int n, const T* __restrict__ M, long ldm, double2* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T v = M[i + (long)i * ldm];
  double2 r = make_double2((double)v.x, (double)v.y);
  if (sqrt(r.x * r.x + r.y * r.y) < 1.0e-30) r = make_double2(1.0, 0.0);
  d[i] = r;
}

// Z[:, c] = V[:, c] / d, element by element (the Jacobi branch of
// APPLY_PRECONDITIONER, IterativeSolvers.f90:296-304).
__global__ void k_jacobi(int n, const double2* __restrict__ V, long ldv, const double2* __restrict__ d,
                         double2* __restrict__ Z, long ldz) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= n) return;
  const double2 v = V[r + (long)c * ldv], q = d[r];
  const double den = q.x * q.x + q.y * q.y;
  Z[r + (long)c * ldz] = make_double2((v.x * q.x + v.y * q.y) / den, (v.y * q.x - v.x * q.y) / den);
}

}  // namespace

cudaError_t diag_extract(cudaStream_t st, int n, const double2* M, long ldm, double2* d) {
  if (n <= 0) return cudaSuccess;
  k_diag<double2><<<(n + 255) / 256, 256, 0, st>>>(n, M, ldm, d);
  return cudaGetLastError();
}

cudaError_t diag_extract(cudaStream_t st, int n, const float2* M, long ldm, double2* d) {
  if (n <= 0) return cudaSuccess;
  k_diag<float2><<<(n + 255) / 256, 256, 0, st>>>(n, M, ldm, d);
  return cudaGetLastError();
}

cudaError_t jacobi_apply(cudaStream_t st, int n, int nc, const double2* V, long ldv, const double2* d, double2* Z,
                         long ldz) {
  if (n <= 0 || nc <= 0) return cudaSuccess;
  k_jacobi<<<dim3((n + 255) / 256, nc), 256, 0, st>>>(n, V, ldv, d, Z, ldz);
  return cudaGetLastError();
}

cudaError_t col_dots(cudaStream_t st, int n, int nc, int nv, const double2* V, long ldv, long vstride, const double2* W,
                     long ldw, double2* H, int ldh) {
  if (nc <= 0 || nv <= 0) return cudaSuccess;
  k_col_dots<<<dim3(nc, nv), kVThreads, 0, st>>>(n, V, ldv, vstride, W, ldw, H, ldh);
  return cudaGetLastError();
}

cudaError_t col_axpy(cudaStream_t st, int n, int nc, int nv, const double2* V, long ldv, long vstride,
                     const double2* H, int ldh, double2* W, long ldw, double sign) {
  if (nc <= 0 || nv <= 0) return cudaSuccess;
  k_col_axpy<<<dim3((n + 255) / 256, nc), 256, 0, st>>>(n, nv, V, ldv, vstride, H, ldh, W, ldw, sign);
  return cudaGetLastError();
}

cudaError_t col_norm2(cudaStream_t st, int n, int nc, const double2* W, long ldw, double* out) {
  if (nc <= 0) return cudaSuccess;
  k_col_norm2<<<nc, kVThreads, 0, st>>>(n, W, ldw, out);
  return cudaGetLastError();
}

cudaError_t col_scale(cudaStream_t st, int n, int nc, const double2* W, long ldw, const double* s, double2* out,
                      long ldo) {
  if (nc <= 0) return cudaSuccess;
  k_col_scale<<<dim3((n + 255) / 256, nc), 256, 0, st>>>(n, W, ldw, s, out, ldo);
  return cudaGetLastError();
}

cudaError_t convert_c2z_2d(cudaStream_t st, int rows, int cols, const float2* src, long lds, double2* dst, long ldd) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  k_c2z_cols<<<dim3((rows + 255) / 256, cols), 256, 0, st>>>(rows, src, lds, dst, ldd);
  return cudaGetLastError();
}

}  // namespace hg
