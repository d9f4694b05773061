// Potential, pressure and free-surface elevation at field points
// (CalPotential / CalPressure / CalElevation, PressureElevation.f90:53-336, and
// their multi-body forms, PressureElevationMulti.f90:55-360).
//
// The per-point panel sums of the reference,
//     pot(x) = (1/SLD) sum_j [DUM1(x, j) w_j - DUM2(x, j) phi_j] (+ VINP),
// are two dense products once DUM1 and DUM2 are laid out as field-point x
// panel matrices: the Green-function fill kernels produce them (the rows are
// the field points, without the collocation free term) and the products run
// through the complex128 GEMM.  This file holds the two small kernels around
// the products: the on-body test that picks SLD, and the finishing pass.
#include "hg_kernels.cuh"

namespace hg {
namespace {

// One warp per field point: is the point on some panel's surface?  The test
// of PressureElevation.f90:213-260: within TOLP = max(1e-6, 1e-3 PNSZ) of the
// panel plane and inside the polygon, i.e. (edge x (P - vertex)) . n keeps its
// sign (within TOLA = 1e-3 PNSZ^2) around the NCN edges.
__global__ void k_field_on_body(int npts, const double* __restrict__ px, int ldp, int n, int ntnd,
                                const double* __restrict__ nodes, const int* __restrict__ ncon,
                                const int* __restrict__ ncn, const double* __restrict__ dxyz,
                                const double* __restrict__ pnsz, int* __restrict__ onb) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= npts) return;
  const double x = px[p], y = px[p + ldp], z = px[p + 2 * (size_t)ldp];
  int hit = 0;
  for (int j = lane; j < n && !hit; j += 32) {
    const double e0 = dxyz[j], e1 = dxyz[j + n], e2 = dxyz[j + 2 * (size_t)n];
    const double sz = pnsz[j];
    const double tolp = fmax(1.0e-6, 1.0e-3 * sz), tola = 1.0e-3 * sz * sz;
    const int nv = ncn[j];
    const int a0 = ncon[j] - 1;
    const double dpln = (x - nodes[a0]) * e0 + (y - nodes[a0 + ntnd]) * e1 + (z - nodes[a0 + 2 * (size_t)ntnd]) * e2;
    if (fabs(dpln) > tolp) continue;
    double smin = 1.0e30, smax = -1.0e30;
    for (int k = 0; k < nv; ++k) {
      const int ia = ncon[j + (size_t)k * n] - 1;
      const int ib = ncon[j + (size_t)((k + 1 < nv) ? k + 1 : 0) * n] - 1;
      const double ax = nodes[ia], ay = nodes[ia + ntnd], az = nodes[ia + 2 * (size_t)ntnd];
      const double ex = nodes[ib] - ax, ey = nodes[ib + ntnd] - ay, ez = nodes[ib + 2 * (size_t)ntnd] - az;
      const double wx = x - ax, wy = y - ay, wz = z - az;
      const double s = (ey * wz - ez * wy) * e0 + (ez * wx - ex * wz) * e1 + (ex * wy - ey * wx) * e2;
      smin = fmin(smin, s);
      smax = fmax(smax, s);
    }
    if (smin >= -tola || smax <= tola) hit = 1;
  }
  hit = __any_sync(0xffffffffu, hit);
  if (lane == 0) onb[p] = hit;
}

// acc[p, c] / SLD(p), plus VINP for diffraction columns (c >= nrad) when
// isol = 1 away from the zero and infinite frequencies
// (PressureElevation.f90:262-282), then the output scaling of kind:
// 0 potential, 1 pressure (i w rho pot; rho pot at the special frequencies),
// 2 elevation (i w / g pot; pot at the special frequencies).
__global__ void k_field_finish(int npts, int ncol, int nrad, double2* __restrict__ acc, long lda,
                               const int* __restrict__ onb, const double* __restrict__ px, int ldp,
                               const double* __restrict__ betas, double v, double wk, double w1, double h, double g,
                               double rho, int isol, int kind) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (p >= npts) return;
  const bool special = fabs(v) < SPD(1.e-8) || fabs(v + 1.0) < SPD(1.e-8);
  const double sld = onb[p] ? 2.0 * HG_PI : 4.0 * HG_PI;
  double2 r = acc[p + (long)c * lda];
  r.x /= sld;
  r.y /= sld;
  if (c >= nrad && isol == 1 && !special) {
    // VINP (PatclVelct.f90:42-76), deep if H < 0 or H > 500
    const double x = px[p], y = px[p + ldp], z = px[p + 2 * (size_t)ldp];
    double sb, cb;
    sincos(betas[c - nrad], &sb, &cb);
    double s, co;
    sincos(wk * (x * cb + y * sb), &s, &co);
    double amp;
    if (h < 0.0 || h > 500.0) amp = -g / w1 * exp(wk * z);
    else amp = (-w1 / (wk * sinh(wk * h))) * cosh(wk * (z + h));
    r.x += amp * co;
    r.y += amp * s;
  }
  if (kind == 1) {
    r = special ? make_double2(rho * r.x, rho * r.y) : make_double2(-w1 * rho * r.y, w1 * rho * r.x);
  } else if (kind == 2) {
    if (!special) r = make_double2(-w1 / g * r.y, w1 / g * r.x);
  }
  acc[p + (long)c * lda] = r;
}

}  // namespace

cudaError_t launch_field_on_body(cudaStream_t st, int npts, const double* px, int ldp, int n, int ntnd,
                                 const double* nodes, const int* ncon, const int* ncn, const double* dxyz,
                                 const double* pnsz, int* onb) {
  if (npts <= 0) return cudaSuccess;
  k_field_on_body<<<(npts + 7) / 8, 256, 0, st>>>(npts, px, ldp, n, ntnd, nodes, ncon, ncn, dxyz, pnsz, onb);
  return cudaGetLastError();
}

cudaError_t launch_field_finish(cudaStream_t st, int npts, int ncol, int nrad, double2* acc, long lda, const int* onb,
                                const double* px, int ldp, const double* betas, double v, double wk, double w1,
                                double h, double g, double rho, int isol, int kind) {
  if (npts <= 0 || ncol <= 0) return cudaSuccess;
  k_field_finish<<<dim3((npts + 127) / 128, ncol), 128, 0, st>>>(npts, ncol, nrad, acc, lda, onb, px, ldp, betas, v, wk,
                                                                 w1, h, g, rho, isol, kind);
  return cudaGetLastError();
}

}  // namespace hg
