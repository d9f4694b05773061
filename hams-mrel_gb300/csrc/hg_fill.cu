// Green-function influence-matrix fill (CALGREEN* + ASSB_LEFT* +
// BODINT_LEFT, CalGreenFunc.f90:49-252 / AssbMatx.f90:53-116), the
// single-layer matrix that feeds the right-hand sides (RBC_RIGHT /
// DBC_RIGHT DUM, BodyIntgr.f90:83-173), the right-hand-side products
// (ASSB_RBC*, ASSB_DBC*) and the force integration (RFORCE*/EFORCE*,
// PotentWavForce.f90:44-221).
//
// Layout: field rows 0..n-1 are hull panels, n..tn-1 lid panels (IRSP=1);
// source columns are hull panels.  A and S are column-major tn x n with
// lda = tn, one complex entry per (field, source) pair.
#include <mutex>
#include "hg_common.cuh"
#include "hg_green.cuh"
#include "hg_kernels.cuh"
#include "hg_tma.cuh"
#include "hg_fill_kernel.cuh"
#include "hg_green32.cuh"
#include "hg_fintab.cuh"
#include <cmath>

namespace hg {

// ---------------------------------------------------------------------------
// Source-panel records (Newman frame of SingularIntgr.f90:150-179 / :372-427)
// ---------------------------------------------------------------------------
__global__ void k_prep_panels(int n, int ntnd, const double* __restrict__ nodes /* ntnd x 3, col-major */,
                              const int* __restrict__ ncon /* n x 4, col-major, 1-based */,
                              const int* __restrict__ ncn, const double* __restrict__ xyz_p /* n x 3 */,
                              const double* __restrict__ ds, const double* __restrict__ pnsz,
                              const double* __restrict__ dxyz_p /* n x 6 */, double* __restrict__ rec,
                              int* status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double* p = rec + (size_t)j * PR_SIZE;
  for (int k = 0; k < PR_SIZE; ++k) p[k] = 0.0;
  const int nv = ncn[j];
  double xv[4][3];
  for (int c = 0; c < 4; ++c) {
    int id = (c < nv) ? ncon[j + (size_t)c * n] : ncon[j];
    if (id < 1 || id > ntnd) { hg_set_status(status, 64); id = 1; }
    for (int k = 0; k < 3; ++k) xv[c][k] = nodes[(id - 1) + (size_t)k * ntnd];
  }
  for (int k = 0; k < 3; ++k) {
    p[PR_XQ + k] = xyz_p[j + (size_t)k * n];
    p[PR_N + k] = dxyz_p[j + (size_t)k * n];
  }
  p[PR_DS] = ds[j];
  p[PR_FLAGD] = 50.0 * pnsz[j];
  p[PR_NCN] = (double)nv;
  double po[3], ui[3], uj[3], uk[3], ksi[4], eta[4];
  if (nv == 3) {
    double p12[3], p13[3], po3[3], po1[3], po2[3];
    for (int k = 0; k < 3; ++k) { p12[k] = xv[1][k] - xv[0][k]; p13[k] = xv[2][k] - xv[0][k]; }
    const double alfa = (p12[0] * p13[0] + p12[1] * p13[1] + p12[2] * p13[2]) /
                        (p12[0] * p12[0] + p12[1] * p12[1] + p12[2] * p12[2]);
    for (int k = 0; k < 3; ++k) po[k] = xv[0][k] + alfa * p12[k];
    for (int k = 0; k < 3; ++k) po3[k] = xv[2][k] - po[k];
    const double n12 = sqrt(p12[0] * p12[0] + p12[1] * p12[1] + p12[2] * p12[2]);
    const double n3 = sqrt(po3[0] * po3[0] + po3[1] * po3[1] + po3[2] * po3[2]);
    for (int k = 0; k < 3; ++k) { ui[k] = p12[k] / n12; uj[k] = po3[k] / n3; }
    uk[0] = ui[1] * uj[2] - ui[2] * uj[1];
    uk[1] = ui[2] * uj[0] - ui[0] * uj[2];
    uk[2] = ui[0] * uj[1] - ui[1] * uj[0];
    for (int k = 0; k < 3; ++k) { po1[k] = xv[0][k] - po[k]; po2[k] = xv[1][k] - po[k]; }
    ksi[0] = -copysign(1.0, alfa) * sqrt(po1[0] * po1[0] + po1[1] * po1[1] + po1[2] * po1[2]);
    eta[0] = 0.0;
    ksi[1] = 0.0;
    eta[1] = n3;
    ksi[2] = sqrt(po2[0] * po2[0] + po2[1] * po2[1] + po2[2] * po2[2]);
    eta[2] = 0.0;
    ksi[3] = 0.0; eta[3] = 0.0;
  } else {
    double pov[4][3], un[3];
    for (int k = 0; k < 3; ++k) po[k] = (xv[0][k] + xv[1][k] + xv[2][k] + xv[3][k]) / 4.0;
    for (int c = 0; c < 4; ++c)
      for (int k = 0; k < 3; ++k) pov[c][k] = xv[c][k] - po[k];
    un[0] = pov[0][1] * pov[1][2] - pov[0][2] * pov[1][1];
    un[1] = pov[0][2] * pov[1][0] - pov[0][0] * pov[1][2];
    un[2] = pov[0][0] * pov[1][1] - pov[0][1] * pov[1][0];
    double nn = sqrt(pov[0][0] * pov[0][0] + pov[0][1] * pov[0][1] + pov[0][2] * pov[0][2]);
    for (int k = 0; k < 3; ++k) ui[k] = pov[0][k] / nn;
    nn = sqrt(un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
    for (int k = 0; k < 3; ++k) uk[k] = un[k] / nn;
    uj[0] = uk[1] * ui[2] - uk[2] * ui[1];
    uj[1] = uk[2] * ui[0] - uk[0] * ui[2];
    uj[2] = uk[0] * ui[1] - uk[1] * ui[0];
    for (int c = 0; c < 4; ++c) {
      const double d = uk[0] * pov[c][0] + uk[1] * pov[c][1] + uk[2] * pov[c][2];
      double pon[3];
      for (int k = 0; k < 3; ++k) pon[k] = pov[c][k] - d * uk[k];
      ksi[c] = ui[0] * pon[0] + ui[1] * pon[1] + ui[2] * pon[2];
      eta[c] = uj[0] * pon[0] + uj[1] * pon[1] + uj[2] * pon[2];
    }
  }
  for (int k = 0; k < 3; ++k) {
    p[PR_PO + k] = po[k]; p[PR_UI + k] = ui[k]; p[PR_UJ + k] = uj[k]; p[PR_UK + k] = uk[k];
  }
  for (int e = 0; e < 4; ++e) { p[PR_KSI + e] = ksi[e]; p[PR_ETA + e] = eta[e]; }
  for (int e = 0; e < nv; ++e) {
    const int nx = (e + 1 == nv) ? 0 : e + 1;
    const double a = ksi[nx] - ksi[e], b = eta[nx] - eta[e];
    p[PR_L + e] = sqrt(a * a + b * b);
  }
}

// ---------------------------------------------------------------------------
// Deep-water pair kernel instantiations (the finite-depth ones live in
// hg_fill_fin.cu, compiled without FMA contraction, and, for the mixed form,
// hg_fill_fin_fma.cu).
// ---------------------------------------------------------------------------
template <typename OUT>
cudaError_t launch_green_fill(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                              const FinState& fs, bool deep, int grn_kind, OUT* A, OUT* S, long lda, int* status,
                              int* bins, int ndiag) {
  if (ndiag < 0) ndiag = tn;
  if (!deep) return launch_green_fill_fin<OUT>(st, rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, status, bins, ndiag);
  dim3 grid((tn + FILL_ROWS - 1) / FILL_ROWS, (n + FILL_COLS - 1) / FILL_COLS);
  k_green_fill<true, OUT><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, fs, grn_kind, A, S, lda, status, ndiag);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Mixed form, deep water: the pair kernel in single precision (the kernel
// k_green_fill_mixed below says which parts stay in double).
// ---------------------------------------------------------------------------
// Monomial coefficients in rho of the Wu-Noblesse local-flow polynomials
// A, B, C, D (InfGreen_Appr.f90:298-416) and A', B', C' (:494-580).
static const double kWuPoly[7][10] = {
    {1.21, -13.328, 215.896, -1763.96, 8418.94, -24314.21, 42002.57, -41592.9, 21859.0, -4838.6},
    {0.938, 5.373, -67.92, 796.534, -4780.77, 17137.74, -36618.81, 44894.06, -29030.24, 7671.22},
    {1.268, -9.747, 209.653, -1397.89, 5155.67, -9844.35, 9136.4, -3272.62, 0.0, 0.0},
    {0.632, -40.97, 667.16, -6072.07, 31127.39, -96293.05, 181856.75, -205690.43, 128170.2, -33744.6},
    {2.948, -24.53, 249.69, -754.85, -1187.71, 16370.75, -48811.41, 68220.87, -46688.0, 12622.25},
    {1.11, 2.894, -76.765, 1565.35, -11336.19, 44270.15, -97014.11, 118879.26, -76209.82, 19923.28},
    {14.19, -148.24, 847.8, -2318.58, 3168.35, -1590.27, 0.0, 0.0, 0.0, 0.0}};

// Chebyshev coefficients (in x = 2 rho - 1) of a degree-9 polynomial in rho.
static void monomial_to_chebyshev(const double* c, double* t) {
  double q[kChebTerms] = {0};  // coefficients in x: rho = (x + 1) / 2
  for (int i = 0; i < kChebTerms; ++i) {
    // ((x + 1) / 2)^i = 2^-i sum_k binom(i, k) x^k
    double binom = 1.0, scale = std::ldexp(1.0, -i);
    for (int k = 0; k <= i; ++k) {
      q[k] += c[i] * scale * binom;
      binom = binom * (i - k) / (k + 1);
    }
  }
  double r[kChebTerms + 1] = {0};
  for (int i = kChebTerms - 1; i >= 0; --i) {
    // r <- x * r + q_i in the Chebyshev basis: x T0 = T1, x Tn = (T(n+1) + T(n-1)) / 2
    double s[kChebTerms + 1] = {0};
    for (int nn = 0; nn < kChebTerms; ++nn) {
      if (r[nn] == 0.0) continue;
      if (nn == 0) s[1] += r[0];
      else { s[nn + 1] += 0.5 * r[nn]; s[nn - 1] += 0.5 * r[nn]; }
    }
    s[0] += q[i];
    for (int nn = 0; nn <= kChebTerms; ++nn) r[nn] = s[nn];
  }
  for (int nn = 0; nn < kChebTerms; ++nn) t[nn] = r[nn];
}

static cudaError_t upload_cheb_constants() {
  static bool done[64] = {false};
  static std::mutex mu;  // host threads of several contexts may get here at once
  std::lock_guard<std::mutex> lock(mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
  float h[7][kChebTerms];
  for (int p = 0; p < 7; ++p) {
    double t[kChebTerms];
    monomial_to_chebyshev(kWuPoly[p], t);
    for (int k = 0; k < kChebTerms; ++k) h[p][k] = (float)t[k];
  }
  e = cudaMemcpyToSymbol(c_cheb, h, sizeof(h));
  if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
  return e;
}

// Gauss points of one panel for panel_gauss_f, from its record (double):
// the flat panel of the closed form, X = PO + ksi ui + eta uj.
__device__ __forceinline__ void panel_gauss_points(const double* __restrict__ pr, double ox, double oy, float4* q) {
  const int nv = (int)pr[PR_NCN];
  double v[4][3];
  for (int c = 0; c < 4; ++c) {
    const int k = (c < nv) ? c : nv - 1;
    const double ks = pr[PR_KSI + k], et = pr[PR_ETA + k];
    for (int d = 0; d < 3; ++d) v[c][d] = pr[PR_PO + d] + ks * pr[PR_UI + d] + et * pr[PR_UJ + d];
  }
  double a2 = 0.0;
  for (int c = 0; c < nv; ++c) {
    const int e = (c + 1 == nv) ? 0 : c + 1;
    a2 += pr[PR_KSI + c] * pr[PR_ETA + e] - pr[PR_KSI + e] * pr[PR_ETA + c];
  }
  const double sgn = ((a2 > 0.0) == (nv == 4)) ? 1.0 : -1.0;
  // 3 x 3 rule (points 0-8), then 2 x 2 (points 9-12)
  const double gp3[3] = {-0.7745966692414834, 0.0, 0.7745966692414834}, gw3[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  const double gp2[2] = {-0.5773502691896258, 0.5773502691896258}, gw2[2] = {1.0, 1.0};
  for (int t = 0; t < 13; ++t) {
    const bool r3 = t < 9;
    const int a = r3 ? t / 3 : (t - 9) / 2, b = r3 ? t % 3 : (t - 9) % 2;
    const double u = r3 ? gp3[a] : gp2[a], w = r3 ? gp3[b] : gp2[b];
    const double wt = r3 ? gw3[a] * gw3[b] : gw2[a] * gw2[b];
    const double N[4] = {0.25 * (1 - u) * (1 - w), 0.25 * (1 + u) * (1 - w), 0.25 * (1 + u) * (1 + w),
                         0.25 * (1 - u) * (1 + w)};
    const double Nu[4] = {-0.25 * (1 - w), 0.25 * (1 - w), 0.25 * (1 + w), -0.25 * (1 + w)};
    const double Nw[4] = {-0.25 * (1 - u), -0.25 * (1 + u), 0.25 * (1 + u), 0.25 * (1 - u)};
    double X[3] = {0, 0, 0}, Xu[3] = {0, 0, 0}, Xw[3] = {0, 0, 0};
    for (int c = 0; c < 4; ++c)
      for (int d = 0; d < 3; ++d) {
        X[d] += N[c] * v[c][d];
        Xu[d] += Nu[c] * v[c][d];
        Xw[d] += Nw[c] * v[c][d];
      }
    const double cx = Xu[1] * Xw[2] - Xu[2] * Xw[1], cy = Xu[2] * Xw[0] - Xu[0] * Xw[2],
                 cz = Xu[0] * Xw[1] - Xu[1] * Xw[0];
    q[t] = make_float4((float)(X[0] - ox), (float)(X[1] - oy), (float)X[2],
                       (float)(sgn * wt * sqrt(cx * cx + cy * cy + cz * cz)));
  }
}

// Single-precision pair loop of the mixed form.  Per pair only FP32
// arithmetic, except (a) the self and adjacent pairs, within 2 panel sizes
// (0.04 of the 50-panel-size FLAG radius), whose Newman integrals stay in
// FP64 with FP64 coordinates, and (b) the rare pairs whose FP32 squared
// distance lies within
// 1e-3 of the FLAG radius, where FLAG is decided again in FP64 exactly as
// CALGREEN does (dist <= 50 PNSZ).  Horizontal coordinates enter FP32
// relative to the mesh centre (ox, oy) so that their rounding is that of the
// array's size, not of its position; depths stay absolute (the image
// distance zp + zq needs them).  FIN: finite depth, the Green function from
// the tables of hg_fintab.cuh plus FINGREEN3D's Rankine pair (FinGreen3D.f90
// :120-150) in FP32; otherwise deep water (inf_green_f).
// Squared FP32 distance of a pair, with the multiply-adds spelled out so
// that the tile kernel and the near-pair kernel round it alike.
__device__ __forceinline__ float pair_d2f(float dxf, float dyf, float dzf) {
  return fmaf(dzf, dzf, fmaf(dyf, dyf, dxf * dxf));
}

// The self and adjacent pairs (FP32 squared distance within 0.0016 of the
// squared FLAG radius: 2 panel sizes), whose Newman integrals the mixed form
// computes in FP64.
__device__ __forceinline__ bool mixed_near(float d2f, float fl2) { return d2f <= 0.0016f * fl2; }

// SKIPNEAR: leave the mixed_near pairs to k_green_fill_mixed_near (deep
// water), so that no warp of this FP32 kernel runs the FP64 Newman integral.
template <bool FIN, bool SKIPNEAR = false>
__global__ void __launch_bounds__(FILL_ROWS)
k_green_fill_mixed(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int n, int tn, float vf,
                   double ox, double oy, const float4* __restrict__ pg, FinTab tab, const float* __restrict__ diag,
                   float2* __restrict__ A, float2* __restrict__ S, long lda, int* status, int ndiag) {
  __shared__ alignas(128) double tile[FILL_COLS * PR_SIZE];
  __shared__ alignas(8) uint64_t bar;
  __shared__ PanelF pfs[FILL_COLS];
  __shared__ float pds[FILL_COLS][4];  // area, normal
  __shared__ float pxs[FILL_COLS][8];  // xq, yq, zq (relative), FLAG radius squared, Newman origin (relative)
  __shared__ float4 pgs[FILL_COLS][kPanelGauss];  // Gauss points of the panel integrals beyond 4 panel sizes
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
    mbar_wait_timed(&bar, 0, 2000000000ull);
    return;
  }
  if (threadIdx.x < ncol) {
    const double* pr = tile + threadIdx.x * PR_SIZE;
    PanelF& q = pfs[threadIdx.x];
    for (int k = 0; k < 3; ++k) {
      q.ui[k] = (float)pr[PR_UI + k]; q.uj[k] = (float)pr[PR_UJ + k]; q.uk[k] = (float)pr[PR_UK + k];
    }
    for (int k = 0; k < 4; ++k) {
      q.ksi[k] = (float)pr[PR_KSI + k]; q.eta[k] = (float)pr[PR_ETA + k]; q.l[k] = (float)pr[PR_L + k];
    }
    q.nv = (int)pr[PR_NCN];
    pds[threadIdx.x][0] = (float)pr[PR_DS];
    for (int k = 0; k < 3; ++k) pds[threadIdx.x][1 + k] = (float)pr[PR_N + k];
    float* px = pxs[threadIdx.x];
    px[0] = (float)(pr[PR_XQ] - ox);
    px[1] = (float)(pr[PR_XQ + 1] - oy);
    px[2] = (float)pr[PR_XQ + 2];
    px[3] = (float)(pr[PR_FLAGD] * pr[PR_FLAGD]);
    px[4] = (float)(pr[PR_PO] - ox);
    px[5] = (float)(pr[PR_PO + 1] - oy);
    px[6] = (float)pr[PR_PO + 2];
    px[7] = 0.f;
  }
  for (int t = threadIdx.x; t < ncol * kPanelGauss; t += FILL_ROWS)
    pgs[t / kPanelGauss][t % kPanelGauss] = pg[(size_t)col0 * kPanelGauss + t];
  __syncthreads();
  const int i = blockIdx.x * FILL_ROWS + threadIdx.x;
  if (i >= tn) return;
  const double xp = fx[i], yp = fx[i + ldf], zp = fx[i + 2 * (size_t)ldf];
  const float xpf = (float)(xp - ox), ypf = (float)(yp - oy), zpf = (float)zp;
  for (int jj = 0; jj < ncol; ++jj) {
    const float* px = pxs[jj];
    const int j = col0 + jj;
    const float dxf = px[0] - xpf, dyf = px[1] - ypf, zqf = px[2];
    const float dzf = zpf - zqf;
    const float d2f = pair_d2f(dxf, dyf, dzf);
    const float fl2 = px[3];
    if (SKIPNEAR && mixed_near(d2f, fl2)) continue;
    int flag;
    if (fabsf(d2f - fl2) > 1e-3f * fl2) {
      flag = d2f < fl2 ? 1 : 0;
    } else {
      const double* pr = tile + jj * PR_SIZE;
      const double dx = pr[PR_XQ] - xp, dy = pr[PR_XQ + 1] - yp, dz = zp - pr[PR_XQ + 2];
      flag = (sqrt(dx * dx + dy * dy + dz * dz) <= pr[PR_FLAGD]) ? 1 : 0;
    }
    float sij = 0.f, d0 = 0.f, d1 = 0.f, d2 = 0.f;
    if (flag) {
      if (mixed_near(d2f, fl2)) {
        double s64, e0, e1, e2;
        newman_pair(tile + jj * PR_SIZE, xp, yp, zp, s64, e0, e1, e2);
        sij = (float)s64; d0 = (float)e0; d1 = (float)e1; d2 = (float)e2;
      } else if (d2f <= 0.0064f * fl2) {
        newman_pair_f(pfs[jj], xpf - px[4], ypf - px[5], zpf - px[6], sij, d0, d1, d2);
      } else if (d2f <= 0.0576f * fl2) {
        panel_gauss_f<9>(pgs[jj], xpf, ypf, zpf, sij, d0, d1, d2);
      } else {
        panel_gauss_f<4>(pgs[jj] + 9, xpf, ypf, zpf, sij, d0, d1, d2);
      }
    }
    float2 g[4];
    if (!FIN) {
      inf_green_f(dxf, dyf, zpf + zqf, dzf, vf, flag, g);
    } else {
      const float rr = sqrtf(dxf * dxf + dyf * dyf);
      float f[6];
      if (d2f > 1e-10f) {
        fintab_eval(tab, rr, zqf, zpf, f);
      } else {
        // coincident centroids (the diagonal): LINTON drops its direct term at
        // r < 1e-6 (FinGreen3D.f90, Linton's image sums) instead of taking the
        // limit, so these pairs take the reference's FP64 value at
        // (R = 0, zq = zp), computed beforehand per source panel (k_fin_diag)
#pragma unroll
        for (int q = 0; q < 6; ++q) f[q] = diag[6 * j + q];
      }
      g[0] = make_float2(f[0], f[1]);
      g[3] = make_float2(f[4], f[5]);
      if (rr > 1e-6f) {
        const float cx = dxf / rr, cy = dyf / rr;
        g[1] = make_float2(f[2] * cx, f[3] * cx);
        g[2] = make_float2(f[2] * cy, f[3] * cy);
      } else {
        g[1] = make_float2(0.f, 0.f);
        g[2] = g[1];
      }
      const float zs = zqf + zpf;
      const float ir1 = rsqrtf(rr * rr + zs * zs), ir13 = ir1 * ir1 * ir1;
      g[0].x += ir1; g[1].x -= dxf * ir13; g[2].x -= dyf * ir13; g[3].x -= zs * ir13;
      if (flag == 0) {
        const float ir = rsqrtf(d2f), ir3 = ir * ir * ir;
        g[0].x += ir; g[1].x -= dxf * ir3; g[2].x -= dyf * ir3; g[3].x += dzf * ir3;  // (zq - zp) = -dzf
      }
    }
    const float ear = pds[jj][0], n0 = pds[jj][1], n1 = pds[jj][2], n2 = pds[jj][3];
    float ar, ai, sr;
    if (flag) {
      ar = (d0 + g[1].x * ear) * n0 + (d1 + g[2].x * ear) * n1 + (d2 + g[3].x * ear) * n2;
      ai = (g[1].y * ear) * n0 + (g[2].y * ear) * n1 + (g[3].y * ear) * n2;
      sr = sij + g[0].x * ear;
    } else {
      ar = (g[1].x * n0 + g[2].x * n1 + g[3].x * n2) * ear;
      ai = (g[1].y * n0 + g[2].y * n1 + g[3].y * n2) * ear;
      sr = g[0].x * ear;
    }
    if (i == j && i < ndiag) ar += 6.28318530717959f;
    A[i + (long)j * lda] = make_float2(ar, ai);
    S[i + (long)j * lda] = make_float2(sr, g[0].y * ear);
  }
}

// The mixed_near pairs of the deep-water mixed fill, listed once per mesh as
// i + j tn (COUNT = true: counted only).  The FP32 quantities are those of
// k_green_fill_mixed, computed the same way.
template <bool COUNT>
__global__ void k_mixed_near_list(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int n,
                                  int tn, double ox, double oy, int* __restrict__ counter, int* __restrict__ list) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  bool near = false;
  if (i < tn) {
    const double* pr = rec + (size_t)j * PR_SIZE;
    const float xqf = (float)(pr[PR_XQ] - ox), yqf = (float)(pr[PR_XQ + 1] - oy), zqf = (float)pr[PR_XQ + 2];
    const float fl2 = (float)(pr[PR_FLAGD] * pr[PR_FLAGD]);
    const float xpf = (float)(fx[i] - ox), ypf = (float)(fx[i + ldf] - oy), zpf = (float)fx[i + 2 * (size_t)ldf];
    near = mixed_near(pair_d2f(xqf - xpf, yqf - ypf, zpf - zqf), fl2);
  }
  const unsigned act = __ballot_sync(0xffffffffu, near);
  if (!act) return;
  const int lane = threadIdx.x & 31, leader = __ffs(act) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(act));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!COUNT && near) list[base + __popc(act & ((1u << lane) - 1u))] = i + j * tn;
}

// The listed pairs with the arithmetic of k_green_fill_mixed's near branch:
// FLAG = 1, the FP64 Newman integral, the FP32 Green function and assembly.
__global__ void __launch_bounds__(128)
k_green_fill_mixed_near(const double* __restrict__ rec, const double* __restrict__ fx, int ldf, int tn, int np,
                        const int* __restrict__ list, float vf, double ox, double oy, float2* __restrict__ A,
                        float2* __restrict__ S, long lda, int ndiag) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np; k += gridDim.x * blockDim.x) {
    const int p = list[k];
    const int i = p % tn, j = p / tn;
    const double* pr = rec + (size_t)j * PR_SIZE;
    const double xp = fx[i], yp = fx[i + ldf], zp = fx[i + 2 * (size_t)ldf];
    const float xpf = (float)(xp - ox), ypf = (float)(yp - oy), zpf = (float)zp;
    const float dxf = (float)(pr[PR_XQ] - ox) - xpf, dyf = (float)(pr[PR_XQ + 1] - oy) - ypf, zqf = (float)pr[PR_XQ + 2];
    const float dzf = zpf - zqf;
    double s64, e0, e1, e2;
    newman_pair(pr, xp, yp, zp, s64, e0, e1, e2);
    const float sij = (float)s64, d0 = (float)e0, d1 = (float)e1, d2 = (float)e2;
    float2 g[4];
    inf_green_f(dxf, dyf, zpf + zqf, dzf, vf, 1, g);
    const float ear = (float)pr[PR_DS], n0 = (float)pr[PR_N], n1 = (float)pr[PR_N + 1], n2 = (float)pr[PR_N + 2];
    float ar = (d0 + g[1].x * ear) * n0 + (d1 + g[2].x * ear) * n1 + (d2 + g[3].x * ear) * n2;
    const float ai = (g[1].y * ear) * n0 + (g[2].y * ear) * n1 + (g[3].y * ear) * n2;
    const float sr = sij + g[0].x * ear;
    if (i == j && i < ndiag) ar += 6.28318530717959f;
    A[i + (long)j * lda] = make_float2(ar, ai);
    S[i + (long)j * lda] = make_float2(sr, g[0].y * ear);
  }
}

cudaError_t launch_green_fill_mixed(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                    double v, double ox, double oy, const float4* pg, float2* A, float2* S, long lda,
                                    int* status, int ndiag, const int* near_list, int near_np) {
  cudaError_t e = upload_cheb_constants();
  if (e != cudaSuccess) return e;
  dim3 grid((tn + FILL_ROWS - 1) / FILL_ROWS, (n + FILL_COLS - 1) / FILL_COLS);
  FinTab none = {};
  const int nd = ndiag < 0 ? tn : ndiag;
  if (!near_list) {
    k_green_fill_mixed<false><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, (float)v, ox, oy, pg, none, nullptr, A,
                                                           S, lda, status, nd);
    return cudaGetLastError();
  }
  k_green_fill_mixed<false, true><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, (float)v, ox, oy, pg, none, nullptr,
                                                               A, S, lda, status, nd);
  if (near_np > 0) {
    int blocks = (near_np + 127) / 128;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_green_fill_mixed_near<<<blocks, 128, 0, st>>>(rec, fx, ldf, tn, near_np, near_list, (float)v, ox, oy, A, S, lda,
                                                     nd);
  }
  return cudaGetLastError();
}

int mixed_near_count(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double ox,
                     double oy, int* counter) {
  if (cudaMemsetAsync(counter, 0, sizeof(int), st) != cudaSuccess) return -1;
  k_mixed_near_list<true><<<dim3((tn + 127) / 128, n), 128, 0, st>>>(rec, fx, ldf, n, tn, ox, oy, counter, nullptr);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

cudaError_t mixed_near_build(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double ox,
                             double oy, int* counter, int* list) {
  cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_mixed_near_list<false><<<dim3((tn + 127) / 128, n), 128, 0, st>>>(rec, fx, ldf, n, tn, ox, oy, counter, list);
  return cudaGetLastError();
}

// F at R = 0, zq = zp = z_j for every source panel j (the coincident pairs).
__global__ void k_fin_diag(int n, const double* __restrict__ rec, FinState fs, float* __restrict__ diag) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double z = rec[(size_t)j * PR_SIZE + PR_XQ + 2];
  double f[6];
  fin_regions(fs, 0.0, z, z, f);
  for (int q = 0; q < 6; ++q) diag[6 * j + q] = (float)f[q];
}

cudaError_t launch_green_fill_mixed_fin(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                        const FinState& fs, const FinTab& tab, double ox, double oy,
                                        const float4* pg, float* diag, float2* A, float2* S, long lda, int* status) {
  // the coincident pairs' FP64 values; with the per-pair pass below R/h = 0.05
  // (tab.gmin = 2) that pass writes them, and the table fill reads zeros
  if (tab.gmin < 2) {
    k_fin_diag<<<(n + 31) / 32, 32, 0, st>>>(n, rec, fs, diag);
  } else {
    cudaError_t e = cudaMemsetAsync(diag, 0, (size_t)6 * n * sizeof(float), st);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((tn + FILL_ROWS - 1) / FILL_ROWS, (n + FILL_COLS - 1) / FILL_COLS);
  k_green_fill_mixed<true><<<grid, FILL_ROWS, 0, st>>>(rec, fx, ldf, n, tn, (float)fs.v, ox, oy, pg, tab, diag, A, S,
                                                        lda, status, tn);
  return cudaGetLastError();
}
template cudaError_t launch_green_fill<double2>(cudaStream_t, const double*, const double*, int, int, int,
                                                const FinState&, bool, int, double2*, double2*, long, int*, int*,
                                                int);
template cudaError_t launch_green_fill<float2>(cudaStream_t, const double*, const double*, int, int, int,
                                               const FinState&, bool, int, float2*, float2*, long, int*, int*,
                                               int);

__global__ void k_panel_gauss(int n, const double* __restrict__ rec, double ox, double oy, float4* __restrict__ pg) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) panel_gauss_points(rec + (size_t)j * PR_SIZE, ox, oy, pg + (size_t)j * kPanelGauss);
}

cudaError_t launch_panel_gauss(cudaStream_t st, int n, const double* rec, double ox, double oy, float4* pg) {
  k_panel_gauss<<<(n + 63) / 64, 64, 0, st>>>(n, rec, ox, oy, pg);
  return cudaGetLastError();
}

cudaError_t launch_prep_panels(cudaStream_t st, int n, int ntnd, const double* nodes, const int* ncon, const int* ncn,
                               const double* xyz_p, const double* ds, const double* pnsz, const double* dxyz_p,
                               double* rec, int* status) {
  k_prep_panels<<<(n + 127) / 128, 128, 0, st>>>(n, ntnd, nodes, ncon, ncn, xyz_p, ds, pnsz, dxyz_p, rec, status);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Incident-wave weights of the diffraction RHS: w[j, b] = -(grad phi_I(x_j; beta_b) . n_j),
// DINP (PatclVelct.f90:83-123) at the source centroid, XW = 0, AMP = 1.
// ---------------------------------------------------------------------------
__global__ void k_incident(int n, const double* __restrict__ xyz_p, const double* __restrict__ dxyz_p, int nbeta,
                           const double* __restrict__ betas, double v, double wk, double w1, double h,
                           double2* __restrict__ w) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
  if (j >= n || b >= nbeta) return;
  double w0, wk0;
  if (fabs(v) < SPD(1.e-8)) { w0 = SPD(1.e-20); wk0 = SPD(1.e-20); }
  else if (fabs(v + 1.0) < SPD(1.e-8)) { w0 = SPD(1.e+20); wk0 = SPD(1.e+20); }
  else { w0 = w1; wk0 = wk; }
  const double x = xyz_p[j], y = xyz_p[j + n], z = xyz_p[j + 2 * (size_t)n];
  double sb, cb;
  sincos(betas[b], &sb, &cb);
  const double wkx = wk0 * (x * cb + y * sb);
  double s, c;
  sincos(wkx, &s, &c);
  double th, tv;
  if (h < 0.0) { th = exp(wk0 * z); tv = th; }
  else { const double sh = sinh(wk0 * h); th = cosh(wk0 * (z + h)) / sh; tv = sinh(wk0 * (z + h)) / sh; }
  // DPOX = w0 th e^{i wkx} cos(beta) / i ; DPOZ = -i w0 tv e^{i wkx} / i = -w0 tv e^{i wkx}
  const double n1 = dxyz_p[j], n2 = dxyz_p[j + n], n3 = dxyz_p[j + 2 * (size_t)n];
  const double hx = w0 * th * (cb * n1 + sb * n2);
  // (c + i s)/i = s - i c
  const double dre = hx * s - w0 * tv * n3 * c;
  const double dim = -hx * c - w0 * tv * n3 * s;
  w[j + (size_t)b * n] = make_double2(-dre, -dim);
}

cudaError_t launch_incident(cudaStream_t st, int n, const double* xyz_p, const double* dxyz_p, int nbeta,
                            const double* betas, double v, double wk, double w1, double h, double2* w) {
  if (nbeta <= 0) return cudaSuccess;
  k_incident<<<dim3((n + 127) / 128, nbeta), 128, 0, st>>>(n, xyz_p, dxyz_p, nbeta, betas, v, wk, w1, h, w);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Right-hand sides from the single-layer matrix S (tn x n):
//   B[:, 6b+md] = sum_{j in body b} S[:, j] n_j,md        (ASSB_RBC_MULTI)
//   B[:, 6NB+k] = sum_j S[:, j] w[j, k]                   (ASSB_DBC)
// Grid: (row blocks, source chunks, heading groups).  Each thread owns one
// row and writes its chunk's partial sums; k_rhs_reduce adds the chunks.
// ---------------------------------------------------------------------------
constexpr int RHS_ROWS = 128;
constexpr int RHS_CHUNK = 256;
constexpr int RHS_HG = 8;

template <typename IN>
__global__ void __launch_bounds__(RHS_ROWS)
k_rhs_partial(int n, int tn, const IN* __restrict__ S, long lds, const double* __restrict__ dxyz_p,
              const int* __restrict__ body_of, int nbody, int nbeta, const double2* __restrict__ w,
              double2* __restrict__ part /* [nchunk][ncols][tn] */) {
  const int i = blockIdx.x * RHS_ROWS + threadIdx.x;
  const int chunk = blockIdx.y, hg0 = blockIdx.z * RHS_HG;
  const int j0 = chunk * RHS_CHUNK, j1 = min(n, j0 + RHS_CHUNK);
  const int ncols = 6 * nbody + nbeta;
  if (i >= tn) return;
  double2* pc = part + (size_t)chunk * ncols * tn;
  const bool do_modes = (blockIdx.z == 0);
  const int nh = max(0, min(RHS_HG, nbeta - hg0));
  double mr[6] = {0, 0, 0, 0, 0, 0}, mi[6] = {0, 0, 0, 0, 0, 0};
  double hr[RHS_HG], hi[RHS_HG];
#pragma unroll
  for (int k = 0; k < RHS_HG; ++k) { hr[k] = 0; hi[k] = 0; }
  int cur = (j0 < j1) ? body_of[j0] : 0;
  for (int j = j0; j < j1; ++j) {
    const IN sv = S[i + (long)j * lds];
    const double sr = sv.x, si = sv.y;
    if (do_modes) {
      const int b = body_of[j];
      if (b != cur) {
#pragma unroll
        for (int md = 0; md < 6; ++md) {
          pc[(size_t)(6 * cur + md) * tn + i] = make_double2(mr[md], mi[md]);
          mr[md] = 0; mi[md] = 0;
        }
        cur = b;
      }
#pragma unroll
      for (int md = 0; md < 6; ++md) {
        const double nv = dxyz_p[j + (size_t)md * n];
        mr[md] += sr * nv;
        mi[md] += si * nv;
      }
    }
#pragma unroll
    for (int k = 0; k < RHS_HG; ++k) {
      if (k < nh) {
        const double2 ww = w[j + (size_t)(hg0 + k) * n];
        hr[k] += sr * ww.x - si * ww.y;
        hi[k] += sr * ww.y + si * ww.x;
      }
    }
  }
  if (do_modes && j0 < j1) {
#pragma unroll
    for (int md = 0; md < 6; ++md) pc[(size_t)(6 * cur + md) * tn + i] = make_double2(mr[md], mi[md]);
  }
#pragma unroll
  for (int k = 0; k < RHS_HG; ++k)
    if (k < nh) pc[(size_t)(6 * nbody + hg0 + k) * tn + i] = make_double2(hr[k], hi[k]);
}

__global__ void k_rhs_reduce(int tn, int ncols, int nchunk, const double2* __restrict__ part, double2* __restrict__ B,
                             long ldb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i >= tn) return;
  double r = 0, im = 0;
  for (int k = 0; k < nchunk; ++k) {
    const double2 v = part[((size_t)k * ncols + c) * tn + i];
    r += v.x;
    im += v.y;
  }
  B[i + (long)c * ldb] = make_double2(r, im);
}

size_t rhs_work_bytes(int n, int tn, int nbody, int nbeta) {
  const int nchunk = (n + RHS_CHUNK - 1) / RHS_CHUNK;
  return (size_t)nchunk * (6 * nbody + nbeta) * tn * sizeof(double2);
}

template <typename IN>
cudaError_t launch_rhs(cudaStream_t st, int n, int tn, const IN* S, long lds, const double* dxyz_p, const int* body_of,
                       int nbody, int nbeta, const double2* w, double2* part, double2* B, long ldb) {
  const int nchunk = (n + RHS_CHUNK - 1) / RHS_CHUNK;
  const int ncols = 6 * nbody + nbeta;
  cudaError_t e = cudaMemsetAsync(part, 0, rhs_work_bytes(n, tn, nbody, nbeta), st);
  if (e != cudaSuccess) return e;
  const int ngroups = max(1, (nbeta + RHS_HG - 1) / RHS_HG);
  k_rhs_partial<IN><<<dim3((tn + RHS_ROWS - 1) / RHS_ROWS, nchunk, ngroups), RHS_ROWS, 0, st>>>(
      n, tn, S, lds, dxyz_p, body_of, nbody, nbeta, w, part);
  k_rhs_reduce<<<dim3((tn + 255) / 256, ncols), 256, 0, st>>>(tn, ncols, nchunk, part, B, ldb);
  return cudaGetLastError();
}
template cudaError_t launch_rhs<double2>(cudaStream_t, int, int, const double2*, long, const double*, const int*, int,
                                         int, const double2*, double2*, double2*, long);
template cudaError_t launch_rhs<float2>(cudaStream_t, int, int, const float2*, long, const double*, const int*, int,
                                        int, const double2*, double2*, double2*, long);

__global__ void k_rhs_cols(int n, const double* __restrict__ dxyz_p, const int* __restrict__ body_of, int nbody,
                           int nbeta, const double2* __restrict__ w, double2* __restrict__ W, long ldw) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (j >= n) return;
  double2 v = make_double2(0.0, 0.0);
  if (c < 6 * nbody) {
    if (body_of[j] == c / 6) v.x = dxyz_p[j + (size_t)(c % 6) * n];
  } else {
    v = w[j + (size_t)(c - 6 * nbody) * n];
  }
  W[j + (long)c * ldw] = v;
}

cudaError_t launch_rhs_cols(cudaStream_t st, int n, const double* dxyz_p, const int* body_of, int nbody, int nbeta,
                            const double2* w, double2* W, long ldw) {
  k_rhs_cols<<<dim3((n + 255) / 256, 6 * nbody + nbeta), 256, 0, st>>>(n, dxyz_p, body_of, nbody, nbeta, w, W, ldw);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Forces.  One CTA per (body m, potential column c): six direction sums over
// body m's panels, then
//   c < 6NB : AMAS[6m+k][c] = sum Im(i rho phi ds n_k) ,  BDMP = -sum Re(i rho w phi ds n_k)
//   c >= 6NB: EXFC[c-6NB][6m+k] = i w rho sum (phi [+ phi_I]) ds n_k
// (RFORCE_MULTI / EFORCE_MULTI, PotentWavForceMulti.f90:45-226)
// ---------------------------------------------------------------------------
__global__ void k_forces(int n, const double2* __restrict__ X, long ldx, const double* __restrict__ xyz_p,
                         const double* __restrict__ ds, const double* __restrict__ dxyz_p,
                         const int* __restrict__ body_start, const int* __restrict__ body_end, int nbody, int nbeta,
                         const double* __restrict__ betas, double v, double wk, double w1, double h, int isol,
                         double rho, double g, double* __restrict__ amas, double* __restrict__ bdmp,
                         double2* __restrict__ exfc) {
  const int m = blockIdx.x, c = blockIdx.y;
  const int nd = 6 * nbody;
  const bool rad = c < nd;
  const int i0 = body_start[m], i1 = body_end[m];
  double sr[6] = {0, 0, 0, 0, 0, 0}, si[6] = {0, 0, 0, 0, 0, 0};
  double w0 = w1, wk0 = wk;
  if (fabs(v) < SPD(1.e-8)) { w0 = SPD(1.e-20); wk0 = SPD(1.e-20); }
  else if (fabs(v + 1.0) < SPD(1.e-8)) { w0 = SPD(1.e+20); wk0 = SPD(1.e+20); }
  double sb = 0, cb = 1;
  if (!rad) sincos(betas[c - nd], &sb, &cb);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    double2 p = X[i + (long)c * ldx];
    if (!rad && isol == 1) {
      // VINP (PatclVelct.f90:42-76), deep if H < 0 or H > 500
      const double x = xyz_p[i], y = xyz_p[i + n], z = xyz_p[i + 2 * (size_t)n];
      const double wkx = wk0 * (x * cb + y * sb);
      double s, co;
      sincos(wkx, &s, &co);
      double amp;
      if (h < 0.0 || h > 500.0) amp = -g / w0 * exp(wk0 * z);        // VINP = -i g/w0 e^{kz} e^{i kx} / i
      else amp = (-w0 / (wk0 * sinh(wk0 * h))) * cosh(wk0 * (z + h));  // VINP = i dum cosh e^{ikx} / i
      p.x += amp * co;
      p.y += amp * s;
    }
    const double a = ds[i];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const double nk = dxyz_p[i + (size_t)k * n];
      sr[k] += p.x * a * nk;
      si[k] += p.y * a * nk;
    }
  }
  __shared__ double red[2][6][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    for (int off = 16; off > 0; off >>= 1) {
      sr[k] += __shfl_down_sync(0xffffffffu, sr[k], off);
      si[k] += __shfl_down_sync(0xffffffffu, si[k], off);
    }
    if (lane == 0) { red[0][k][warp] = sr[k]; red[1][k][warp] = si[k]; }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int k = threadIdx.x;
    double tr = 0, ti = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { tr += red[0][k][w]; ti += red[1][k][w]; }
    if (rad) {
      // i rho (tr + i ti) = rho (-ti + i tr)
      amas[(size_t)(6 * m + k) * nd + c] = rho * tr;
      bdmp[(size_t)(6 * m + k) * nd + c] = rho * w1 * ti;
    } else {
      // i w rho (tr + i ti) = w rho (-ti + i tr)
      exfc[(size_t)(c - nd) * nd + 6 * m + k] = make_double2(-w1 * rho * ti, w1 * rho * tr);
    }
  }
}

cudaError_t launch_forces(cudaStream_t st, int n, const double2* X, long ldx, const double* xyz_p, const double* ds,
                          const double* dxyz_p, const int* body_start, const int* body_end, int nbody, int nbeta,
                          const double* betas, double v, double wk, double w1, double h, int isol, double rho,
                          double g, double* amas, double* bdmp, double2* exfc) {
  k_forces<<<dim3(nbody, 6 * nbody + nbeta), 256, 0, st>>>(n, X, ldx, xyz_p, ds, dxyz_p, body_start, body_end, nbody,
                                                           nbeta, betas, v, wk, w1, h, isol, rho, g, amas, bdmp, exfc);
  return cudaGetLastError();
}

cudaError_t launch_green_points(cudaStream_t st, int npts, const double* pts, const int* flags, const FinState& fs,
                                bool deep, double* out) {
  if (!deep) return launch_green_points_fin(st, npts, pts, flags, fs, out);
  k_green_points<true><<<(npts + 63) / 64, 64, 0, st>>>(npts, pts, flags, fs, out);
  return cudaGetLastError();
}

}  // namespace hg
