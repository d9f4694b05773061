// Tabulated finite-depth Green function for the mixed form.
//
// FINGREEN3D's value and derivatives at horizontal distance R, source depth
// zq and field depth zp, minus the Rankine pair 1/r + 1/r1 (the quantity its
// region methods return, fin_regions), split exactly into two functions of
// two variables:
//     F(R, zq, zp) = P(R, W) + Q(R, U),   W = zq - zp,  U = zq + zp.
// This holds for every term: the eigenfunction products
// cos(k(zq+h)) cos(k(zp+h)) and cosh(k0(zq+h)) cosh(k0(zp+h)) are half sums
// of functions of U and of W, and the Rankine pair is 1/r(R, W) + 1/r1(R, U);
// d/dzq acts as d/dW + d/dU.  With U0 = -h,
//     TP(R, W) = F(R; W, U0),   TQ(R, U) = F(R; W', U) - F(R; W', U0)
// satisfy F = TP + TQ for any W' with both points inside the fluid; W' =
// min(-U, 2h + U, h) / 2 keeps the reference points off the source point.
// Each table entry is an evaluation of the reference's own methods (FP64,
// FinGreen3D.f90:160-226).  The reference switches method at R/h = 0.0005,
// 0.05 and 0.5, and the methods differ slightly at the switches, so the R
// grid is cut into those four segments, each evaluated by its own method
// up to and including its end points; an interpolation stencil never
// crosses a segment end.  Within a segment the nodes are R = a + (b - a)
// expm1(c u) / expm1(c), u uniform (denser near the short end); the W nodes
// are cell-centred (W = 0 is never a node); the U nodes are uniform in
// t = log(1 + |U|/u0), shifted by half a step (U = 0 is never a node).
// Pairs interpolate both tables bicubically (Catmull-Rom) in single precision.
// Below R/h = 0.05 the fill evaluates the pairs again per pair in FP64
// (launch_fin_near): LINTON's and PIDCOCK's values are not smooth in R.
// The propagating-wave term of F (the k0 mode: p0 (-Y0, J0)(k0 R) with
// p0 = pi/N0 cosh(k0(zq+h)) cosh(k0(zp+h)), and its derivatives; the
// d_prop_part of FinGreen3D.f90:281-362) oscillates on the wavelength scale
// and grows exponentially towards the surface, so it is left out of the
// tables and evaluated per pair in FP32 instead (fintab_prop).  Y0's
// logarithm is kept in the tables near R = 0, where the evanescent modes
// cancel it: the term taken out uses Z = Y0 - chi (2/pi) ln(k0 R) J0 with the
// smooth cut-off chi = exp(-(k0 R / 1.5)^2), so both the term and the
// remainder stay regular; the remainder is smooth on the depth scale.
// Each node holds 8 floats: re/im of F, dF/dR, dF/dzq, and 2 pads.
#pragma once
#include "hg_common.cuh"

namespace hg {

constexpr int kFinSegs = 4;
struct FinTab {
  const float* tp;  // [nr][nw][8]
  const float* tq;  // [nr][nu][8]
  int nr, nw, nu;
  float sa[kFinSegs], sb[kFinSegs], sc[kFinSegs], sx[kFinSegs];  // segment ends, concentration, expm1(c)
  int so[kFinSegs], sn[kFinSegs];                               // first node, node count
  float h;       // W_j = -h + (j + 1/2) 2h / nw
  float u0, dt;  // U_k = -u0 (exp((k + 1/2) dt) - 1)
  float k0;      // wave number WK
  float pk;      // pi e^(2 k0 h) / N0, N0 = h/2 (1 + sinh(2 k0 h) / (2 k0 h))
  double pk_d;   // the same in double (table build)
  int gmin;      // first segment built: 2 when the pairs below R/h = 0.05 are evaluated per pair
};

// Propagating term, T = double (table build) or float (pairs): f = [re, im]
// of the term, its R derivative and its zq derivative.
//   p0 = pk/4 e^(k0 U)(1 + qa)(1 + qb), dp0 = k0 pk/4 e^(k0 U)(1 - qa)(1 + qb),
//   qa = e^(-2 k0 (zq+h)), qb = e^(-2 k0 (zp+h)): pi/N0 cosh(a) cosh(b) and
//   k0 pi/N0 sinh(a) cosh(b) without overflow;
//   Z = Y0(x) - chi L(x) J0(x), L = (2/pi) ln x, x = k0 R; for x < 0.1 from
//   Y0 - L J0 = (2/pi)(gamma - ln 2) J0 + (2/pi)(x^2/4 - 3 x^4/128) (the
//   series of Y0) plus (1 - chi) L J0, free of cancellation.
template <typename T>
__device__ __forceinline__ void fintab_prop(T k0, T pk, T h, T R, T zq, T zp, T f[6]) {
  const T ea = exp(k0 * (zq + zp));
  const T qa = exp(-2 * k0 * (zq + h)), qb = exp(-2 * k0 * (zp + h));
  const T p0 = T(0.25) * pk * ea * (1 + qa) * (1 + qb);
  const T dp0 = T(0.25) * k0 * pk * ea * (1 - qa) * (1 + qb);
  const T x = k0 * R;
  const T tpi = T(0.6366197723675814);        // 2 / pi
  const T c0 = T(-0.07380429510868723);       // (2/pi)(gamma - ln 2)
  const T ixc2 = T(1.0) / T(2.25);            // 1 / 1.5^2
  const T chi = exp(-x * x * ixc2);
  T j0v, j1v, Z, dZ;                          // dZ = dZ/dR
  if (x < T(0.1)) {
    j0v = T(1) - x * x / 4 + x * x * x * x / 64;
    j1v = x / 2 - x * x * x / 16;
    const T x2 = x * x;
    const T ys = c0 * j0v + tpi * (x2 / 4 - 3 * x2 * x2 / 128);
    const T dys = -c0 * j1v + tpi * (x / 2 - 3 * x2 * x / 32);
    const T omc = -expm1(-x2 * ixc2);         // 1 - chi
    if (x > T(0)) {
      const T L = tpi * log(x);
      Z = ys + omc * L * j0v;
      // d/dR[(1 - chi) L J0] = k0 [2 x chi / xc^2 L J0 + ((1 - chi)/x) (2/pi) J0 - (1 - chi) L J1]
      dZ = k0 * (dys + 2 * x * chi * ixc2 * L * j0v + (omc / x) * tpi * j0v - omc * L * j1v);
    } else {
      Z = ys;
      dZ = 0;
    }
  } else {
    T y0v, y1v;
    if (sizeof(T) == 4) {
      j0v = j0f((float)x); j1v = j1f((float)x); y0v = y0f((float)x); y1v = y1f((float)x);
    } else {
      j0v = ::j0((double)x); j1v = ::j1((double)x); y0v = ::y0((double)x); y1v = ::y1((double)x);
    }
    const T L = tpi * log(x);
    Z = y0v - chi * L * j0v;
    // dZ/dR = k0 [ -Y1 + 2 x chi / xc^2 L J0 - chi ((2/pi) J0 / x - L J1) ]
    dZ = k0 * (-y1v + 2 * x * chi * ixc2 * L * j0v - chi * (tpi * j0v / x - L * j1v));
  }
  f[0] = -p0 * Z;
  f[1] = p0 * j0v;
  f[2] = -p0 * dZ;
  f[3] = -(k0 * p0) * j1v;
  f[4] = -dp0 * Z;
  f[5] = dp0 * j0v;
}

__device__ __forceinline__ void cr_weights(float t, float w[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * (-t3 + 2.f * t2 - t);
  w[1] = 0.5f * (3.f * t3 - 5.f * t2 + 2.f);
  w[2] = 0.5f * (-3.f * t3 + 4.f * t2 + t);
  w[3] = 0.5f * (t3 - t2);
}

// Catmull-Rom weights of the end intervals of an axis with nodes lo..hi: the
// stencil's node beyond the end is a ghost extrapolated from the nodes
// inside (quadratically, f(lo-1) = 3 f(lo) - 3 f(lo+1) + f(lo+2), or
// linearly on a 2-node axis), folded into their weights.  A ghost equal to
// the end node instead would make the end intervals first-order accurate
// (an error of about an eighth of the node spacing times the slope).
__device__ __forceinline__ void cr_fold_ends(float w[4], int i0, int lo, int hi) {
  const bool quad = hi - lo >= 2;
  if (i0 == lo) {
    const float g = w[0];
    w[0] = 0.f;
    if (quad) { w[1] += 3.f * g; w[2] -= 3.f * g; w[3] += g; }
    else { w[1] += 2.f * g; w[2] -= g; }
  }
  if (i0 == hi - 1) {
    const float g = w[3];
    w[3] = 0.f;
    if (quad) { w[2] += 3.f * g; w[1] -= 3.f * g; w[0] += g; }
    else { w[2] += 2.f * g; w[1] -= g; }
  }
}

// Bicubic Catmull-Rom interpolation of one table at fractional indices x
// (first axis, nodes lo..hi of one R segment) and y (second axis, size n2);
// the end intervals use extrapolated ghost nodes (cr_fold_ends).
__device__ __forceinline__ void cr_interp(const float* __restrict__ T, int lo, int hi, int n2, float x, float y,
                                          float f[6]) {
  x = fminf(fmaxf(x, (float)lo), (float)hi);
  y = fminf(fmaxf(y, 0.f), (float)(n2 - 1));
  int i0 = min((int)x, hi - 1), j0 = min((int)y, n2 - 2);
  float wx[4], wy[4];
  cr_weights(x - (float)i0, wx);
  cr_weights(y - (float)j0, wy);
  cr_fold_ends(wx, i0, lo, hi);
  cr_fold_ends(wy, j0, 0, n2 - 1);
#pragma unroll
  for (int q = 0; q < 6; ++q) f[q] = 0.f;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = min(max(i0 - 1 + a, lo), hi);
    float row[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = min(max(j0 - 1 + b, 0), n2 - 1);
      const float4* p = reinterpret_cast<const float4*>(T + ((size_t)i * n2 + j) * 8);
      const float4 v0 = __ldg(p), v1 = __ldg(p + 1);
      row[0] = fmaf(wy[b], v0.x, row[0]); row[1] = fmaf(wy[b], v0.y, row[1]);
      row[2] = fmaf(wy[b], v0.z, row[2]); row[3] = fmaf(wy[b], v0.w, row[3]);
      row[4] = fmaf(wy[b], v1.x, row[4]); row[5] = fmaf(wy[b], v1.y, row[5]);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) f[q] = fmaf(wx[a], row[q], f[q]);
  }
}

// F(R, zq, zp) from the tables (see above).
__device__ __forceinline__ void fintab_eval(const FinTab& T, float R, float zq, float zp, float f[6]) {
  const float rh = R / T.h;
  const int g = max(T.gmin, (rh < 0.0005f) ? 0 : (rh < 0.05f) ? 1 : (rh < 0.5f) ? 2 : 3);  // the reference's switches
  const float a = T.sa[g], b = T.sb[g], c = T.sc[g];
  const float v = fminf(fmaxf((R - a) / (b - a), 0.f), 1.f);
  const float u = (c > 0.f) ? log1pf(v * T.sx[g]) / c : v;
  const int lo = T.so[g], hi = T.so[g] + T.sn[g] - 1;
  const float x = (float)lo + u * (float)(T.sn[g] - 1);
  const float w = (zq - zp + T.h) * ((float)T.nw / (2.f * T.h)) - 0.5f;
  const float t = log1pf(fmaxf(-(zq + zp), 0.f) / T.u0) / T.dt - 0.5f;
  float pa[6], pb[6], p[6];
  cr_interp(T.tp, lo, hi, T.nw, x, w, pa);
  cr_interp(T.tq, lo, hi, T.nu, x, t, pb);
  fintab_prop<float>(T.k0, T.pk, T.h, R, zq, zp, p);
#pragma unroll
  for (int q = 0; q < 6; ++q) f[q] = pa[q] + pb[q] + p[q];
}

// Grid sizes: R nodes per segment (LINTON, PIDCOCK, EIGENE, EIGEN), W and U
// nodes; the build costs (sum of R nodes) x (W + 2 U) evaluations.
constexpr int kFinSegN[kFinSegs] = {2, 64, 72, 64};
constexpr int kFinTabR = 2 + 64 + 72 + 64, kFinTabW = 160, kFinTabU = 200;

}  // namespace hg
