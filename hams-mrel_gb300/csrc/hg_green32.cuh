// Single-precision deep-water Green function and Newman integrals for the
// mixed form of the fill.
//
// The Wu-Noblesse polynomials A, B, C, D, A', B', C' of the local flow
// (InfGreen_Appr.f90:298-580) have monomial coefficients up to 2e5 with
// alternating signs: a single-precision Horner evaluation loses ~1e-3 of
// their value.  The same polynomials are evaluated here in the Chebyshev
// basis on rho in [0, 1] (coefficients converted once per device from the
// monomial ones in double precision), where single-precision Clenshaw
// recurrence keeps ~1e-6.  The Newman edge logarithm log((s+L)/(s-L)) is
// evaluated as log1p(2L/(s-L)), which stays accurate when the field point is
// far from the edge; pairs within a few panel sizes use the double-precision
// integral instead.
#pragma once
#include "hg_common.cuh"

namespace hg {

constexpr int kChebTerms = 10;
// 7 polynomials x 10 Chebyshev coefficients (A, B, C, D, dA, dB, dC), set by
// the host once per device.  Only hg_fill.cu includes this header.
__constant__ float c_cheb[7][kChebTerms];

__device__ __forceinline__ float clenshaw(const float* c, float x) {
  float b1 = 0.f, b2 = 0.f;
#pragma unroll
  for (int k = kChebTerms - 1; k >= 1; --k) {
    const float t = fmaf(2.f * x, b1, c[k] - b2);
    b2 = b1;
    b1 = t;
  }
  return fmaf(x, b1, c[0] - b2);
}

__device__ __forceinline__ void havelock_f(float hh, float vv, float2& gf, float2& gfh) {
  const float gama = 0.5772156649f, pi = 3.14159265358979f;
  const float dd = sqrtf(hh * hh + vv * vv);
  const float idd = 1.f / dd;
  const float alpha = -vv * idd, beta = hh * idd, rho = dd / (1.f + dd);
  const float ev = expf(vv), emd = expf(-dd);
  const float dd3 = 1.f + dd * dd * dd;
  const float omr = 1.f - rho, omr3 = omr * omr * omr;
  const float x = 2.f * rho - 1.f;
  const float pa = clenshaw(c_cheb[0], x), pb = clenshaw(c_cheb[1], x), pc = clenshaw(c_cheb[2], x),
              pd = clenshaw(c_cheb[3], x);
  const float pp = (logf(0.5f * (dd - vv)) + gama - 2.f * dd * dd) * ev + dd * dd - vv;
  const float rr = (1.f - beta) * pa - beta * pb - alpha * pc / (1.f + 6.f * alpha * rho * omr) +
                   beta * (1.f - beta) * pd;
  const float l0 = 2.f * pp / dd3 + 2.f * (rho * omr3 * rr);
  float j0, j1, h0, h1;
  if (hh <= 3.f) {
    const float yy = (hh / 3.f) * (hh / 3.f);
    j0 = 0.999999999f + (-2.249999879f + (1.265623060f + (-0.316394552f + (0.044460948f +
         (-0.003954479f + 0.000212950f * yy) * yy) * yy) * yy) * yy) * yy;
    j1 = (0.5f + (-0.562499992f + (0.210937377f + (-0.039550040f + (0.004447331f + (-0.000330547f +
          0.000015525f * yy) * yy) * yy) * yy) * yy) * yy) * hh;
    h0 = (1.909859164f + (-1.909855001f + (0.687514637f + (-0.126164557f + (0.013828813f -
          0.000876918f * yy) * yy) * yy) * yy) * yy) * (hh / 3.f);
    h1 = (1.909859286f + (-1.145914713f + (0.294656958f + (-0.042070508f + (0.003785727f -
          0.000207183f * yy) * yy) * yy) * yy) * yy) * yy;
  } else {
    const float y = 3.f / hh, y2 = y * y, isq = rsqrtf(hh);
    const float f0 = 0.79788454f + (-0.00553897f + (0.00099336f + (-0.00044346f + (0.00020445f -
                     0.00004959f * y2) * y2) * y2) * y2) * y2;
    const float t0 = hh - 0.25f * pi + (-0.04166592f + (0.00239399f + (-0.00073984f + (0.00031099f -
                     0.00007605f * y2) * y2) * y2) * y2) * y;
    const float f1 = 0.79788459f + (0.01662008f + (-0.00187002f + (0.00068519f + (-0.00029440f +
                     0.00006952f * y2) * y2) * y2) * y2) * y2;
    const float t1 = hh - 0.75f * pi + (0.12499895f + (-0.00605240f + (0.00135825f + (-0.00049616f +
                     0.00011531f * y2) * y2) * y2) * y2) * y;
    float s0, c0, s1, c1;
    sincosf(t0, &s0, &c0);
    sincosf(t1, &s1, &c1);
    j0 = f0 * c0 * isq;
    j1 = f1 * c1 * isq;
    const float y0 = f0 * s0 * isq, y1 = f1 * s1 * isq;
    h0 = 2.f * (0.99999906f + (4.77228920f + (3.85542044f + 0.32303607f * y2) * y2) * y2) /
             (pi * hh * (1.f + (4.88331068f + (4.28957333f + 0.52120508f * y2) * y2) * y2)) + y0;
    h1 = 2.f * (1.00000004f + (3.92205313f + (2.64893033f + 0.27450895f * y2) * y2) * y2) /
             (pi * (1.f + (3.81095112f + (2.26216956f + 0.10885141f * y2) * y2) * y2)) + y1;
  }
  const float tpe = 2.f * pi * ev;
  gf = make_float2(l0 + tpe * h0, -tpe * j0);
  const float ps = (beta + hh) / (dd - vv) - 2.f * beta + 2.f * ev * dd - hh;
  const float qs = emd * (1.f - beta) * (1.f + dd / dd3);
  const float da = clenshaw(c_cheb[4], x), db = clenshaw(c_cheb[5], x), dc = clenshaw(c_cheb[6], x);
  const float rs = beta * da - (1.f - alpha) * db + beta * (1.f - beta) * rho * (1.f - 2.f * rho) * dc;
  const float ls = 2.f * ps / dd3 - 4.f * qs + 2.f * (rho * omr3 * rs);
  gfh = make_float2(ls + tpe * (2.f / pi - h1), tpe * j1);
}

// INFGREEN3D in single precision; (dx, dy) = source - field horizontally,
// zpq = zfield + zsource, zdf = zfield - zsource (differences formed in
// double by the caller).
__device__ __forceinline__ void inf_green_f(float dx, float dy, float zpq, float zdf, float v, int flag, float2 g[4]) {
  const float rr2 = dx * dx + dy * dy;
  const float rr = sqrtf(rr2);
  const float ir1 = rsqrtf(rr2 + zpq * zpq), ir13 = ir1 * ir1 * ir1;
  float2 gf, gfh;
  havelock_f(v * rr, v * zpq, gf, gfh);
  const float v2 = v * v;
  if (rr > 1.e-6f) {
    const float cx = -v2 * dx / rr, cy = -v2 * dy / rr;
    g[1] = make_float2(gfh.x * cx, gfh.y * cx);
    g[2] = make_float2(gfh.x * cy, gfh.y * cy);
  } else {
    g[1] = make_float2(0.f, 0.f);
    g[2] = make_float2(0.f, 0.f);
  }
  g[0] = make_float2(-v * gf.x + ir1, -v * gf.y);
  g[3] = make_float2(-v2 * gf.x + 2.f * v * ir1, -v2 * gf.y);
  g[1].x -= dx * ir13;
  g[2].x -= dy * ir13;
  g[3].x -= zpq * ir13;
  if (flag == 0) {
    const float ir = rsqrtf(rr2 + zdf * zdf), ir3 = ir * ir * ir;
    g[0].x += ir;
    g[1].x -= dx * ir3;
    g[2].x -= dy * ir3;
    g[3].x += zdf * ir3;  // -(zsource - zfield)/R^3
  }
}

// Newman integral in single precision; (p0, p1, p2) = field point - panel
// origin (formed in double), record fields converted by the caller.
struct PanelF {
  float ui[3], uj[3], uk[3], ksi[4], eta[4], l[4];
  int nv;
};

__device__ __forceinline__ void newman_pair_f(const PanelF& pf, float p0, float p1, float p2, float& sij, float& d0,
                                              float& d1, float& d2) {
  const float x = pf.ui[0] * p0 + pf.ui[1] * p1 + pf.ui[2] * p2;
  const float y = pf.uj[0] * p0 + pf.uj[1] * p1 + pf.uj[2] * p2;
  const float z = pf.uk[0] * p0 + pf.uk[1] * p1 + pf.uk[2] * p2;
  const bool tri = (pf.nv == 3);
  const float z2 = z * z;
  float st = 0.f, sxt = 0.f, syt = 0.f, szt = 0.f;
  float ksa = pf.ksi[0], eta_a = pf.eta[0];
  const float r_first = sqrtf((ksa - x) * (ksa - x) + (eta_a - y) * (eta_a - y) + z2);
  float r1 = r_first;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if (e >= pf.nv) break;
    const int nx = (e + 1 == pf.nv) ? 0 : e + 1;
    const float ksb = pf.ksi[nx], etb = pf.eta[nx];
    const float r2 = (nx == 0) ? r_first : sqrtf((ksb - x) * (ksb - x) + (etb - y) * (etb - y) + z2);
    const float l = pf.l[e];
    if (!tri && fabsf(l) < 1.0e-8f) { ksa = ksb; eta_a = etb; r1 = r2; continue; }
    const float dksi = ksb - ksa, deta = etb - eta_a;
    const float b1 = deta * ((ksa - x) * (ksa - x) + z2) - dksi * (ksa - x) * (eta_a - y);
    const float a1 = r1 * z * dksi;
    const float b2 = deta * ((ksb - x) * (ksb - x) + z2) - dksi * (ksb - x) * (etb - y);
    const float a2 = r2 * z * dksi;
    if (!(fabsf(z) < 1.0e-6f)) szt += atan2f(b1 * a2 - b2 * a1, a1 * a2 + b1 * b2);
    const float s = r1 + r2;
    if (!(fabsf(s - l) < 1.0e-6f)) {
      const float lg = log1pf(2.f * l / (s - l));
      sxt -= deta / l * lg;
      syt += dksi / l * lg;
      const float t = (deta * (x - ksa) - dksi * (y - eta_a)) / l * lg;
      st = tri ? st + t : st - t;
    }
    ksa = ksb; eta_a = etb; r1 = r2;
  }
  sij = tri ? st - z * szt : st + z * szt;
  const float sg = tri ? 1.f : -1.f;
  d0 = sg * (pf.ui[0] * sxt + pf.uj[0] * syt + pf.uk[0] * szt);
  d1 = sg * (pf.ui[1] * sxt + pf.uj[1] * syt + pf.uk[1] * szt);
  d2 = sg * (pf.ui[2] * sxt + pf.uj[2] * syt + pf.uk[2] * szt);
}

// Gauss rules of the panel integrals for field points 4 or more panel sizes
// away, where the closed form loses accuracy in single precision: its edge
// terms are each of the panel's size while the integral is of size
// area / distance, so rounding grows with distance (2e-6 relative at 4 panel
// sizes, 2.5e-4 at 50), whereas Gauss-Legendre rules on the flat panel
// (bilinear map; triangles as quads with a collapsed edge) hold 3e-7: the
// integrand is smooth there and every term has the sign of the sum.  The
// 3 x 3 rule serves 4 to 12 panel sizes, the 2 x 2 rule (also 3e-7 there)
// the rest.  The points of both rules (the 9, then the 4), each
// (x - ox, y - oy, z, signed weight), are prepared once per mesh
// (launch_panel_gauss); the signed weight is the Gauss weight times |Jacobian|
// times the sign that reproduces the closed form's convention, which follows
// the vertex order (quads: the sign of the panel's signed area in its own
// frame; triangles: the opposite).  Outputs as newman_pair_f: the integral
// of 1/r and sg times the gradient terms, here d = -sum w (X_q - P)/r^3.
template <int NQ>
__device__ __forceinline__ void panel_gauss_f(const float4* __restrict__ q, float xp, float yp, float zp, float& sij,
                                              float& d0, float& d1, float& d2) {
  float s = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    const float4 g = q[k];
    const float dx = g.x - xp, dy = g.y - yp, dz = g.z - zp;
    const float ir = rsqrtf(dx * dx + dy * dy + dz * dz);
    const float wi = g.w * ir, wi3 = wi * ir * ir;
    s += wi;
    gx = fmaf(dx, wi3, gx);
    gy = fmaf(dy, wi3, gy);
    gz = fmaf(dz, wi3, gz);
  }
  sij = s;
  d0 = -gx;
  d1 = -gy;
  d2 = -gz;
}

}  // namespace hg
