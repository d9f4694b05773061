// Device-side free-surface Green functions and Newman panel integrals.
//
// Deep water: the Wu-Noblesse global approximation used by HAMS-MREL
// (src/InfGreen_Appr.f90:104-872).  The GPU form evaluates exp(vv),
// exp(-dd) and log(dd-vv) once per pair and shares one sincos between each
// J/Y Bessel pair: the reference's BesselY0/Y1 (:674-760) use the same
// modulus and phase polynomials as BesselJ0/J1 (:583-671), so
// Y = f*sin(theta)/sqrt(x) and J = f*cos(theta)/sqrt(x) come from one call.
//
// Finite depth: the region-decomposed Green function of src/FinGreen3D.f90
// (Linton / Pidcock / eigenfunction series with Wynn's epsilon algorithm),
// with every convergence loop bounded, the recursive Gauss-Kronrod 7-15
// quadrature turned into an explicit-stack loop, and the E_n(x) upward
// recursion of ENXA (src/FinGrnExtSubs.f90:82-107) advanced incrementally
// instead of restarted from E_1 on every series term.  Loops that hit their
// cap set HG_DEV_SERIES_CAP in the status word.
#pragma once
#include "hg_common.cuh"

#ifdef __CUDACC__
#define HGD __host__ __device__
#else
#define HGD
#endif

namespace hg {

#ifdef __CUDA_ARCH__
#define HGD_TABLE __device__ const
#else
#define HGD_TABLE static const
#endif

// ===================================================================
// Newman (1986) closed-form integral of 1/r and grad(1/r) over a flat
// panel, SingularIntgr.f90:44-244 (triangles) and :252-445 (quads).
// pr = 36-double source-panel record (hg_common.cuh).
// ===================================================================
HGD inline void newman_pair(const double* __restrict__ pr, double xf0, double xf1,
                                            double xf2, double& sij, double& d0, double& d1,
                                            double& d2) {
  const double p0 = xf0 - pr[PR_PO], p1 = xf1 - pr[PR_PO + 1], p2 = xf2 - pr[PR_PO + 2];
  const double x = pr[PR_UI] * p0 + pr[PR_UI + 1] * p1 + pr[PR_UI + 2] * p2;
  const double y = pr[PR_UJ] * p0 + pr[PR_UJ + 1] * p1 + pr[PR_UJ + 2] * p2;
  const double z = pr[PR_UK] * p0 + pr[PR_UK + 1] * p1 + pr[PR_UK + 2] * p2;
  const int nv = (int)pr[PR_NCN];
  const bool tri = (nv == 3);
  double st = 0.0, sxt = 0.0, syt = 0.0, szt = 0.0;
  const double z2 = z * z;
  double ksa = pr[PR_KSI], eta_a = pr[PR_ETA];
  const double r_first = sqrt((ksa - x) * (ksa - x) + (eta_a - y) * (eta_a - y) + z2);
  double r1 = r_first;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if (e >= nv) break;
    const int nx = (e + 1 == nv) ? 0 : e + 1;
    const double ksb = pr[PR_KSI + nx], etb = pr[PR_ETA + nx];
    const double r2 = (nx == 0) ? r_first : sqrt((ksb - x) * (ksb - x) + (etb - y) * (etb - y) + z2);
    const double l = pr[PR_L + e];
    if (!tri && fabs(l) < 1.0e-8) {
      ksa = ksb; eta_a = etb; r1 = r2;
      continue;
    }
    const double dksi = ksb - ksa, deta = etb - eta_a;
    const double b1 = deta * ((ksa - x) * (ksa - x) + z2) - dksi * (ksa - x) * (eta_a - y);
    const double a1 = r1 * z * dksi;
    const double b2 = deta * ((ksb - x) * (ksb - x) + z2) - dksi * (ksb - x) * (etb - y);
    const double a2 = r2 * z * dksi;
    if (!(fabs(z) < 1.0e-6)) szt += atan2(b1 * a2 - b2 * a1, a1 * a2 + b1 * b2);
    const double s = r1 + r2;
    if (!(fabs(s - l) < 1.0e-6)) {
      const double lg = log((s + l) / (s - l));
      sxt -= deta / l * lg;
      syt += dksi / l * lg;
      const double t = (deta * (x - ksa) - dksi * (y - eta_a)) / l * lg;
      st = tri ? st + t : st - t;
    }
    ksa = ksb; eta_a = etb; r1 = r2;
  }
  sij = tri ? st - z * szt : st + z * szt;
  const double sg = tri ? 1.0 : -1.0;
  d0 = sg * (pr[PR_UI] * sxt + pr[PR_UJ] * syt + pr[PR_UK] * szt);
  d1 = sg * (pr[PR_UI + 1] * sxt + pr[PR_UJ + 1] * syt + pr[PR_UK + 1] * szt);
  d2 = sg * (pr[PR_UI + 2] * sxt + pr[PR_UJ + 2] * syt + pr[PR_UK + 2] * szt);
}

// ===================================================================
// Deep water
// ===================================================================
HGD inline double poly_a(double t) {
  double g = (21859.0 + -4838.6 * t) * t;
  g = (-41592.9 + g) * t; g = (42002.57 + g) * t; g = (-24314.21 + g) * t;
  g = (8418.94 + g) * t; g = (-1763.96 + g) * t; g = (215.896 + g) * t;
  g = (-13.328 + g) * t; return 1.21 + g;
}
HGD inline double poly_b(double t) {
  double g = (-29030.24 + 7671.22 * t) * t;
  g = (44894.06 + g) * t; g = (-36618.81 + g) * t; g = (17137.74 + g) * t;
  g = (-4780.77 + g) * t; g = (796.534 + g) * t; g = (-67.92 + g) * t;
  g = (5.373 + g) * t; return 0.938 + g;
}
HGD inline double poly_c(double t) {
  double g = (9136.4 + -3272.62 * t) * t;
  g = (-9844.35 + g) * t; g = (5155.67 + g) * t; g = (-1397.89 + g) * t;
  g = (209.653 + g) * t; g = (-9.747 + g) * t; return 1.268 + g;
}
HGD inline double poly_d(double t) {
  double g = (128170.2 + -33744.6 * t) * t;
  g = (-205690.43 + g) * t; g = (181856.75 + g) * t; g = (-96293.05 + g) * t;
  g = (31127.39 + g) * t; g = (-6072.07 + g) * t; g = (667.16 + g) * t;
  g = (-40.97 + g) * t; return 0.632 + g;
}
HGD inline double poly_da(double t) {
  double g = (-46688.0 + 12622.25 * t) * t;
  g = (68220.87 + g) * t; g = (-48811.41 + g) * t; g = (16370.75 + g) * t;
  g = (-1187.71 + g) * t; g = (-754.85 + g) * t; g = (249.69 + g) * t;
  g = (-24.53 + g) * t; return 2.948 + g;
}
HGD inline double poly_db(double t) {
  double g = (-76209.82 + 19923.28 * t) * t;
  g = (118879.26 + g) * t; g = (-97014.11 + g) * t; g = (44270.15 + g) * t;
  g = (-11336.19 + g) * t; g = (1565.35 + g) * t; g = (-76.765 + g) * t;
  g = (2.894 + g) * t; return 1.11 + g;
}
HGD inline double poly_dc(double t) {
  double g = (3168.35 + -1590.27 * t) * t;
  g = (-2318.58 + g) * t; g = (847.8 + g) * t; g = (-148.24 + g) * t;
  return 14.19 + g;
}

// Havelock wave term GF and its horizontal derivative GFh at the
// non-dimensional horizontal distance hh = v*R and depth vv = v*(z+zeta).
HGD inline void havelock(double hh, double vv, double2& gf, double2& gfh) {
  const double gama = 0.5772156649;
  const double dd = sqrt(hh * hh + vv * vv);
  const double alpha = -vv / dd, beta = hh / dd, rho = dd / (1.0 + dd);
  const double ev = exp(vv), emd = exp(-dd);
  const double dd3 = 1.0 + dd * dd * dd;
  const double omr = 1.0 - rho, omr3 = omr * omr * omr;
  double pp = (log(0.5 * (dd - vv)) + gama - 2.0 * dd * dd) * ev + dd * dd - vv;
  double rr = (1.0 - beta) * poly_a(rho) - beta * poly_b(rho) -
              alpha * poly_c(rho) / (1.0 + 6.0 * alpha * rho * omr) + beta * (1.0 - beta) * poly_d(rho);
  const double l0 = 2.0 * pp / dd3 + 2.0 * (rho * omr3 * rr);
  double j0, j1, h0, h1;
  if (hh <= 3.0) {
    const double yy = (hh / 3.0) * (hh / 3.0);
    j0 = 0.999999999 + (-2.249999879 + (1.265623060 + (-0.316394552 + (0.044460948 +
         (-0.003954479 + 0.000212950 * yy) * yy) * yy) * yy) * yy) * yy;
    j1 = (0.5 + (-0.562499992 + (0.210937377 + (-0.039550040 + (0.004447331 + (-0.000330547 +
          0.000015525 * yy) * yy) * yy) * yy) * yy) * yy) * hh;
    h0 = (1.909859164 + (-1.909855001 + (0.687514637 + (-0.126164557 + (0.013828813 -
          0.000876918 * yy) * yy) * yy) * yy) * yy) * (hh / 3.0);
    h1 = (1.909859286 + (-1.145914713 + (0.294656958 + (-0.042070508 + (0.003785727 -
          0.000207183 * yy) * yy) * yy) * yy) * yy) * yy;
  } else {
    const double y = 3.0 / hh, y2 = y * y, isq = 1.0 / sqrt(hh);
    const double f0 = 0.79788454 + (-0.00553897 + (0.00099336 + (-0.00044346 + (0.00020445 -
                      0.00004959 * y2) * y2) * y2) * y2) * y2;
    const double t0 = hh - 0.25 * HG_PI + (-0.04166592 + (0.00239399 + (-0.00073984 + (0.00031099 -
                      0.00007605 * y2) * y2) * y2) * y2) * y;
    const double f1 = 0.79788459 + (0.01662008 + (-0.00187002 + (0.00068519 + (-0.00029440 +
                      0.00006952 * y2) * y2) * y2) * y2) * y2;
    const double t1 = hh - 0.75 * HG_PI + (0.12499895 + (-0.00605240 + (0.00135825 + (-0.00049616 +
                      0.00011531 * y2) * y2) * y2) * y2) * y;
    double s0, c0, s1, c1;
    sincos(t0, &s0, &c0);
    sincos(t1, &s1, &c1);
    j0 = f0 * c0 * isq;
    j1 = f1 * c1 * isq;
    const double y0 = f0 * s0 * isq, y1 = f1 * s1 * isq;
    h0 = 2.0 * (0.99999906 + (4.77228920 + (3.85542044 + 0.32303607 * y2) * y2) * y2) /
             (HG_PI * hh * (1.0 + (4.88331068 + (4.28957333 + 0.52120508 * y2) * y2) * y2)) + y0;
    h1 = 2.0 * (1.00000004 + (3.92205313 + (2.64893033 + 0.27450895 * y2) * y2) * y2) /
             (HG_PI * (1.0 + (3.81095112 + (2.26216956 + 0.10885141 * y2) * y2) * y2)) + y1;
  }
  const double tpe = 2.0 * HG_PI * ev;
  gf = make_double2(l0 + tpe * h0, -tpe * j0);
  const double ps = (beta + hh) / (dd - vv) - 2.0 * beta + 2.0 * ev * dd - hh;
  const double qs = emd * (1.0 - beta) * (1.0 + dd / dd3);
  rr = beta * poly_da(rho) - (1.0 - alpha) * poly_db(rho) +
       beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * poly_dc(rho);
  const double ls = 2.0 * ps / dd3 - 4.0 * qs + 2.0 * (rho * omr3 * rr);
  gfh = make_double2(ls + tpe * (2.0 / HG_PI - h1), tpe * j1);
}

// INFGREEN3D (InfGreen_Appr.f90:104-186).  Source (xq,yq,zq), field (xp,yp,zp).
HGD inline void inf_green(double xq, double yq, double zq, double xp, double yp,
                                          double zp, double v, int flag, double2 g[4]) {
  const double xpq = xq - xp, ypq = yq - yp, zpq = zp + zq;
  const double rr = sqrt(xpq * xpq + ypq * ypq);
  const double r = sqrt(rr * rr + (zp - zq) * (zp - zq));
  const double r1 = sqrt(rr * rr + zpq * zpq);
  const double ir1 = 1.0 / r1, ir13 = ir1 * ir1 * ir1;
  const double ir = 1.0 / r, ir3 = ir * ir * ir;
  double sgn1 = 1.0;  // sign of the image term: -1 at the infinite-frequency limit
  if (fabs(v) < SPD(1.e-8) || fabs(v + 1.0) < SPD(1.e-8)) {
    if (!(fabs(v) < SPD(1.e-8))) sgn1 = -1.0;
    g[0] = make_double2(0.0, 0.0); g[1] = g[0]; g[2] = g[0]; g[3] = g[0];
  } else {
    double2 gf, gfh;
    havelock(v * rr, v * zpq, gf, gfh);
    const double v2 = v * v;
    if (rr > SPD(1.e-6)) {
      const double cx = -v2 * xpq / rr, cy = -v2 * ypq / rr;
      g[1] = make_double2(gfh.x * cx, gfh.y * cx);
      g[2] = make_double2(gfh.x * cy, gfh.y * cy);
    } else {
      g[1] = make_double2(0.0, 0.0);
      g[2] = make_double2(0.0, 0.0);
    }
    g[0] = make_double2(-v * gf.x, -v * gf.y);
    g[3] = make_double2(-v2 * gf.x + 2.0 * v * ir1, -v2 * gf.y);
  }
  g[0].x += sgn1 * ir1;
  g[1].x -= sgn1 * xpq * ir13;
  g[2].x -= sgn1 * ypq * ir13;
  g[3].x -= sgn1 * zpq * ir13;
  if (flag == 0) {
    g[0].x += ir;
    g[1].x -= xpq * ir3;
    g[2].x -= ypq * ir3;
    g[3].x -= (zq - zp) * ir3;
  }
}

// ===================================================================
// Finite depth: special functions (FinGrnExtSubs.f90)
// ===================================================================
// x**k for an integer k by binary powering, the evaluation order a Fortran
// compiler uses for an integer exponent.
HGD inline double powi(double x, int m) {
  unsigned n = (unsigned)m;
  double y = (n % 2u) ? x : 1.0;
  while (n >>= 1) {
    x = x * x;
    if (n % 2u) y = y * x;
  }
  return y;
}
HGD inline double d_error(double x) {  // ERROR :62-93
  const double x2 = x * x;
  if (fabs(x) < 3.5) {
    double er = 1.0, r = 1.0;
    for (int k = 1; k <= 50; ++k) {
      r = r * x2 / (k + 0.5);
      er += r;
      if (fabs(r) <= fabs(er) * 1.0e-15) break;
    }
    return 2.0 / sqrt(HG_PI) * x * exp(-x2) * er;
  }
  double er = 1.0, r = 1.0;
  for (int k = 1; k <= 12; ++k) {
    r = -r * (k - 0.5) / x2;
    er += r;
  }
  double e = 1.0 - exp(-x2) / (fabs(x) * sqrt(HG_PI)) * er;
  return x < 0.0 ? -e : e;
}
HGD inline double d_erfcc(double x) { return 1.0 - d_error(x); }
HGD inline double d_derfcc(double x) { return -2.0 / sqrt(HG_PI) * exp(-(x * x)); }

HGD inline double d_e1xa(double x) {  // E1XA :119-133
  if (x == 0.0) return 1.0e+300;
  if (x <= 1.0)
    return -log(x) + ((((1.07857e-3 * x - 9.76004e-3) * x + 5.519968e-2) * x - 0.24991055) * x +
                      0.99999193) * x - 0.57721566;
  const double es1 = (((x + 8.5733287401) * x + 18.059016973) * x + 8.6347608925) * x + 0.2677737343;
  const double es2 = (((x + 9.5733223454) * x + 25.6329561486) * x + 21.0996530827) * x + 3.9584969228;
  return exp(-x) / x * es1 / es2;
}

HGD inline double d_eix(double x) {  // EIX :146-172
  if (x == 0.0) return -1.0e+300;
  if (x <= 40.0) {
    double ei = 1.0, r = 1.0;
    for (int k = 1; k <= 100; ++k) {
      r = r * k * x / ((k + 1.0) * (k + 1.0));
      ei += r;
      if (fabs(r / ei) <= 1.0e-15) break;
    }
    return 0.5772156649015328 + log(x) + x * ei;
  }
  double ei = 1.0, r = 1.0;
  for (int k = 1; k <= 20; ++k) {
    r = r * k / x;
    ei += r;
  }
  return exp(x) / x * ei;
}

// IK01A :538-640, returning K0 and K1.
HGD inline void d_ik01a(double x, double& bk0, double& bk1) {
  if (x == 0.0) { bk0 = 1.0e+300; bk1 = 1.0e+300; return; }
  const double x2 = x * x;
  double bi0, bi1;
  if (x <= 18.0) {
    bi0 = 1.0;
    double r = 1.0;
    for (int k = 1; k <= 50; ++k) {
      r = 0.25 * r * x2 / (double)(k * k);
      bi0 += r;
      if (fabs(r / bi0) < 1.0e-15) break;
    }
    bi1 = 1.0;
    r = 1.0;
    for (int k = 1; k <= 50; ++k) {
      r = 0.25 * r * x2 / (double)(k * (k + 1));
      bi1 += r;
      if (fabs(r / bi1) < 1.0e-15) break;
    }
    bi1 = 0.5 * x * bi1;
  } else {
    const double A[12] = {0.125, 7.03125e-2, 7.32421875e-2, 1.1215209960938e-1, 2.2710800170898e-1,
                          5.7250142097473e-1, 1.7277275025845, 6.0740420012735, 2.4380529699556e01,
                          1.1001714026925e02, 5.5133589612202e02, 3.0380905109224e03};
    const double B[12] = {-0.375, -1.171875e-1, -1.025390625e-1, -1.4419555664063e-1,
                          -2.7757644653320e-1, -6.7659258842468e-1, -1.9935317337513,
                          -6.8839142681099, -2.7248827311269e01, -1.2159789187654e02,
                          -6.0384407670507e02, -3.3022722944809e03};
    int k0 = 12;
    if (x >= 35.0) k0 = 9;
    if (x >= 50.0) k0 = 7;
    const double ca = exp(x) / sqrt(2.0 * HG_PI * x), xr = 1.0 / x;
    double s0 = 1.0, s1 = 1.0;
    for (int k = 1; k <= 12; ++k) {
      if (k > k0) break;
      s0 += A[k - 1] * powi(xr, k);
    }
    for (int k = 1; k <= 12; ++k) {
      if (k > k0) break;
      s1 += B[k - 1] * powi(xr, k);
    }
    bi0 = ca * s0;
    bi1 = ca * s1;
  }
  if (x <= 9.0) {
    const double ct = -(log(x / 2.0) + 0.5772156649015329);
    double k0v = 0.0, w0 = 0.0, r = 1.0, ww = 0.0;
    for (int k = 1; k <= 50; ++k) {
      w0 += 1.0 / k;
      r = 0.25 * r / (double)(k * k) * x2;
      k0v += r * (w0 + ct);
      if (fabs((k0v - ww) / k0v) < 1.0e-15) break;
      ww = k0v;
    }
    bk0 = k0v + ct;
  } else {
    const double A1[8] = {0.125, 0.2109375, 1.0986328125, 1.1775970458984e01, 2.1461706161499e02,
                          5.9511522710323e03, 2.3347645606175e05, 1.2312234987631e07};
    const double xr2 = 1.0 / x2;
    double s = 1.0;
    for (int k = 0; k < 8; ++k) s += A1[k] * powi(xr2, k + 1);
    bk0 = 0.5 / x * s / bi0;
  }
  bk1 = (1.0 / x - bi1 * bk0) / bi0;
}

// JY01B :663-736
HGD inline void d_jy01b(double x, double& bj0, double& bj1, double& by0, double& by1) {
  if (x == 0.0) { bj0 = 1.0; bj1 = 0.0; by0 = -1.0e+300; by1 = -1.0e+300; return; }
  if (x <= 4.0) {
    const double t = x / 4.0, t2 = t * t;
    bj0 = ((((((-.5014415e-3 * t2 + .76771853e-2) * t2 - .0709253492) * t2 + .4443584263) * t2 -
             1.7777560599) * t2 + 3.9999973021) * t2 - 3.9999998721) * t2 + 1.0;
    bj1 = t * (((((((-.1289769e-3 * t2 + .22069155e-2) * t2 - .0236616773) * t2 + .1777582922) * t2 -
                  .8888839649) * t2 + 2.6666660544) * t2 - 3.9999999710) * t2 + 1.9999999998);
    const double lg = 2.0 / HG_PI * log(x / 2.0);
    by0 = lg * bj0 + ((((((((-.567433e-4 * t2 + .859977e-3) * t2 - .94855882e-2) * t2 + .0772975809) * t2 -
                         .4261737419) * t2 + 1.4216421221) * t2 - 2.3498519931) * t2 + SPD(1.0766115157)) * t2 +
                      .3674669052);
    by1 = lg * bj1 + (((((((((.6535773e-3 * t2 - .0108175626) * t2 + .107657606) * t2 - .7268945577) * t2 +
                           3.1261399273) * t2 - 7.3980241381) * t2 + 6.8529236342) * t2 + .3932562018) * t2 -
                        .6366197726) / x);
    return;
  }
  const double t = 4.0 / x, t2 = t * t, a0 = sqrt(2.0 / (HG_PI * x));
  const double p0 = ((((-.9285e-5 * t2 + .43506e-4) * t2 - .122226e-3) * t2 + .434725e-3) * t2 - .4394275e-2) * t2 + .999999997;
  const double q0 = t * (((((.8099e-5 * t2 - .35614e-4) * t2 + .85844e-4) * t2 - .218024e-3) * t2 + .1144106e-2) * t2 - .031249995);
  const double p1 = ((((.10632e-4 * t2 - .50363e-4) * t2 + .145575e-3) * t2 - .559487e-3) * t2 + .7323931e-2) * t2 + 1.000000004;
  const double q1 = t * (((((-.9173e-5 * t2 + .40658e-4) * t2 - .99941e-4) * t2 + .266891e-3) * t2 - .1601836e-2) * t2 + .093749994);
  double s0, c0;
  sincos(x - .25 * HG_PI, &s0, &c0);
  // cos(x - 3pi/4) = -sin... computed directly for fidelity with the reference
  double s1, c1;
  sincos(x - .75 * HG_PI, &s1, &c1);
  bj0 = a0 * (p0 * c0 - q0 * s0);
  by0 = a0 * (p0 * s0 + q0 * c0);
  bj1 = a0 * (p1 * c1 - q1 * s1);
  by1 = a0 * (p1 * s1 + q1 * c1);
}

// Wynn epsilon algorithm, Limes FinGrnExtSubs.f90:370-503.  s[0..n] is
// overwritten; a[] is caller scratch of n+1 entries.
HGD inline double d_limes(int n, double* s, double* a) {
  double a_max = 0.0, rl = s[n];
  for (int i = 0; i <= n; ++i) a[i] = 0.0;
  for (int k = 1;; ++k) {
    if (n - 2 * k + 1 < 0) break;
    for (int i = 0; i <= n - 2 * k + 1; ++i)
      a[i] = (s[i + 1] != s[i]) ? a[i + 1] + 1.0 / (s[i + 1] - s[i]) : a[i + 1];
    if (n - 2 * k < 0) break;
    for (int i = 0; i <= n - 2 * k; ++i) {
      s[i] = (a[i + 1] != a[i]) ? s[i + 1] + 1.0 / (a[i + 1] - a[i]) : s[i + 1];
      if (fabs(a[i]) > a_max) {
        a_max = fabs(a[i]);
        rl = s[i];
        if (s[i + 1] == s[i]) return rl;
      }
    }
  }
  return rl;
}

// Pidcock's image-source sums IMGS / DGSR / DGSZ (FinGreen3D.f90:908-1102).
HGD inline void d_imgs_all(double r, double zf, double zp, double h, double& gs, double& gr,
                                  double& gz) {
  // AMN(M,N), M = 0..4 (rows), N = 0..4
  const double AMN[5][5] = {{0.0, 0.05051418, 0.00230838, 0.00012934, 0.00000913},
                            {-0.02525711, -0.00692380, -0.00097875, -0.00010879, -0.00001270},
                            {0.00086546, 0.00073292, 0.00020597, 0.00003965, 0.00000466},
                            {-0.00004063, -0.00006636, -0.00003333, -0.00000891, 0.0},
                            {0.00000193, 0.00000398, 0.00000524, 0.0, 0.0}};
  const double t1 = r / h, t2 = (zf - zp) / h, t3 = (zf + zp + 2.0 * h) / h;
  double s1 = 0.0, s1r = 0.0, s1z = 0.0;
  for (int l = -1; l <= 1; ++l) {
    const double za = t2 + 2.0 * l, zb = t3 + 2.0 * l;
    const double ra = sqrt(t1 * t1 + za * za), rb = sqrt(t1 * t1 + zb * zb);
    const double ra3 = ra * ra * ra, rb3 = rb * rb * rb;
    s1 = s1 + 1.0 / ra + 1.0 / rb;
    s1r = s1r + t1 / ra3 + t1 / rb3;
    s1z = s1z + za / ra3 + zb / rb3;
  }
  // real powers t^(2m), t^(2m-1) as in the reference (pow with a real exponent)
  double p1[5], p2[5], p3[5], q2[5], q3[5], pr1[5];
  for (int k = 0; k < 5; ++k) {
    p1[k] = pow(t1, 2.0 * k); p2[k] = pow(t2, 2.0 * k); p3[k] = pow(t3, 2.0 * k);
    pr1[k] = k ? pow(t1, 2.0 * k - 1.0) : 0.0;
    q2[k] = k ? pow(t2, 2.0 * k - 1.0) : 0.0;
    q3[k] = k ? pow(t3, 2.0 * k - 1.0) : 0.0;
  }
  double s2 = 0.0, s2r = 0.0, s2z = 0.0;
  for (int m = 0; m <= 4; ++m)
    for (int n = 0; n <= 4; ++n) {
      const double a = AMN[m][n];
      s2 += a * p1[m] * (p2[n] + p3[n]);
      if (m >= 1) s2r += 2.0 * m * a * pr1[m] * (p2[n] + p3[n]);
      if (n >= 1) s2z += 2.0 * n * a * p1[m] * (q2[n] + q3[n]);
    }
  gs = (s1 - 2.0 + s2) / h;
  gr = (-s1r + s2r) / (h * h);
  gz = (-s1z + s2z) / (h * h);
}

// Subtraction of the Rankine pair shared by EIGEN / EIGENE / PIDCOCK.
HGD inline void d_sub_rankine(double r, double zf, double zp, double& g0, double& g1,
                                              double& g2) {
  const double sr = sqrt(r * r + (zf - zp) * (zf - zp)), sr1 = sqrt(r * r + (zf + zp) * (zf + zp));
  g0 -= (1.0 / sr + 1.0 / sr1);
  g1 += (r / sr / (sr * sr) + r / sr1 / (sr1 * sr1));
  g2 += ((zf - zp) / sr / (sr * sr) + (zf + zp) / sr1 / (sr1 * sr1));
}

struct FinState {
  double v, wk, h, nm0;  // nm0 = h/2 (1 + sinh(2 wk h)/(2 wk h))
  const double* wvn;     // roots, wvn[0] = wk
  int nk;
  int* status;
};

// Imaginary (propagating) part shared by the three series methods:
// P0 (i J0 - Y0) etc. of EIGEN/EIGENE/PIDCOCK.
HGD inline void d_prop_part(const FinState& s, double r, double zf, double zp, double g[6],
                                            bool pid) {
  const double wk = s.wk, h = s.h;
  const double p0 = HG_PI / s.nm0 * cosh(wk * (zf + h)) * cosh(wk * (zp + h));
  // DP0 carries WK inside (PIDCOCK :601) or outside (EIGEN :317, EIGENE :442);
  // kept in the reference's order so the rounding matches.
  const double dp0 = pid ? wk * HG_PI / s.nm0 * sinh(wk * (zf + h)) * cosh(wk * (zp + h))
                         : wk * (HG_PI / s.nm0 * sinh(wk * (zf + h)) * cosh(wk * (zp + h)));
  double j0, j1, y0, y1;
  d_jy01b(wk * r, j0, j1, y0, y1);
  g[0] = -p0 * y0;  g[1] = p0 * j0;
  g[2] = wk * p0 * y1; g[3] = -(wk * p0) * j1;
  g[4] = -dp0 * y0; g[5] = dp0 * j0;
  if (pid) {
    g[0] += 2.0 / h * (0.5772156649015328 + log(r / 4.0 / h));
    g[2] += 2.0 / (r * h);
  }
}

// EIGEN (R/h >= 0.5), FinGreen3D.f90:281-362.  g = [re0, im0, re1, im1, re2, im2]
HGD inline void d_eigen(const FinState& s, double r, double zf, double zp, double g[6]) {
  d_prop_part(s, r, zf, zp, g, false);
  const double h = s.h;
  for (int i = 2; i <= 10; ++i) {
    const double km = s.wvn[i - 1], tkh = 2.0 * km * h;
    const double pm = 4.0 / (1.0 + sin(tkh) / tkh) / h;
    double k0, k1, skzf, ckzf;
    d_ik01a(km * r, k0, k1);
    sincos(km * (zf + h), &skzf, &ckzf);
    const double ckzp = cos(km * (zp + h));
    const double rm1 = pm * k0 * ckzf * ckzp, rm2 = -(pm * km * k1 * ckzf * ckzp),
                 rm3 = -(pm * km * k0 * skzf * ckzp);
    g[0] += rm1; g[2] += rm2; g[4] += rm3;
    if (fabs(rm1) < SPD(1.e-6) && fabs(rm2) < SPD(1.e-6) && fabs(rm3) < SPD(1.e-6)) break;
  }
  d_sub_rankine(r, zf, zp, g[0], g[2], g[4]);
}

// EIGENE (0.05 <= R/h < 0.5), :413-506, and PIDCOCK (0.0005 <= R/h < 0.05), :558-660.
HGD inline void d_series_eps(const FinState& s, double r, double zf, double zp, double g[6],
                                    bool pid) {
  double gs[101], gr[101], gz[101], scratch[101];
  const double h = s.h, v = s.v, rhp = fabs(r / h);
  int nt = pid ? (int)(SPD(-1010.10) * rhp + SPD(100.50)) : (int)(SPD(-88.89) * rhp + SPD(54.45));
  if (nt > 101) nt = 101;
  if (nt > s.nk) nt = s.nk;
  d_prop_part(s, r, zf, zp, g, pid);
  gs[0] = 0.0; gr[0] = 0.0; gz[0] = 0.0;
  for (int i = 2; i <= nt; ++i) {
    const double um = s.wvn[i - 1];
    double k0, k1;
    d_ik01a(um * r, k0, k1);
    double su, cu;
    sincos(um * (zf + h), &su, &cu);
    const double cp = cos(um * (zp + h));
    if (!pid) {
      const double tkh = 2.0 * um * h, pm = 4.0 / (1.0 + sin(tkh) / tkh) / h;
      gs[i - 1] = gs[i - 2] + pm * k0 * cu * cp;
      gr[i - 1] = gr[i - 2] - pm * um * k1 * cu * cp;
      gz[i - 1] = gz[i - 2] - pm * um * k0 * su * cp;
    } else {
      const double umt = (i - 1) * HG_PI / h;
      double k0t, k1t, st, ct;
      d_ik01a(umt * r, k0t, k1t);
      sincos(umt * (zf + h), &st, &ct);
      const double cpt = cos(umt * (zp + h));
      const double ac = (um * um + v * v) / ((um * um + v * v) * h - v);
      const double am = ac * cu * cp, amt = ct * cpt / h;
      const double dam = -(um * ac * su * cp), damt = -(umt * st * cpt / h);
      gs[i - 1] = gs[i - 2] + (am * k0 - amt * k0t);
      gr[i - 1] = gr[i - 2] + (-(um * am * k1) + umt * amt * k1t);
      gz[i - 1] = gz[i - 2] + (dam * k0 - damt * k0t);
    }
  }
  const double l0 = d_limes(nt - 1, gs, scratch);
  const double l1 = d_limes(nt - 1, gr, scratch);
  const double l2 = d_limes(nt - 1, gz, scratch);
  if (pid) {
    double is, ir, iz;
    d_imgs_all(r, zf, zp, h, is, ir, iz);
    g[0] = g[0] + 4.0 * l0 + is;
    g[2] = g[2] + 4.0 * l1 + ir;
    g[4] = g[4] + 4.0 * l2 + iz;
  } else {
    g[0] += l0; g[2] += l1; g[4] += l2;
  }
  d_sub_rankine(r, zf, zp, g[0], g[2], g[4]);
}

// ---- Linton's method (R/h < 0.0005), FinGreen3D.f90:712-861 ----
struct LintonPar {
  double v, r, zf, zp, h;
};

// Integrands G1/G2/G3 (:1904-2057) of the deep-water-like correction.
HGD inline double d_gfun(const LintonPar& p, double t, int tag) {
  if (fabs(t) < 1.0e-8) return 0.0;
  const double val[4] = {-p.zp - p.zf, 2.0 * p.h - p.zp + p.zf, 2.0 * p.h + p.zp - p.zf,
                         4.0 * p.h + p.zp + p.zf};
  const double dval[4] = {-1.0, 1.0, -1.0, 1.0};
  double sum = 0.0;
  for (int i = 0; i < 4; ++i) {
    const double e = exp(-p.v * val[i]), arg = val[i] / 2.0 / t - p.v * t;
    if (tag == 3)
      sum = sum - p.v * dval[i] * e * d_erfcc(arg) + e * d_derfcc(arg) * dval[i] / 2.0 / t;
    else
      sum += e * d_erfcc(arg);
  }
  const double ex = exp(p.v * p.v * (t * t) - p.r * p.r / 4.0 / (t * t));
  if (tag == 2) return p.r / 2.0 / (t * t * t) * ex * sum;
  return ex * sum / t;
}
// Integrands F1/F2 (:1795-1880) of the expansion coefficients.
HGD inline double d_ffun(double r, double wvn, int no, double t, int tag) {
  if (fabs(t) < 1.0e-8) return 0.0;
  const double e = (no == 1) ? exp(-r * r / 4.0 / t + wvn * wvn * t) : exp(-r * r / 4.0 / t - wvn * wvn * t);
  return tag == 1 ? e / 4.0 / HG_PI / t : -r * e / 8.0 / HG_PI / (t * t);
}

HGD_TABLE double c_xgq[7] = {-0.949107912342759, -0.741531185599394, -0.405845151377397, 0.0,
                                0.405845151377397, 0.741531185599394, 0.949107912342759};
HGD_TABLE double c_wgq[7] = {0.129484966168870, 0.279705391489277, 0.381830050505119,
                                0.417959183673469, 0.381830050505119, 0.279705391489277,
                                0.129484966168870};
HGD_TABLE double c_xkq[15] = {-0.991455371120813, -0.949107912342759, -0.864864423359769,
                                 -0.741531185599394, -0.586087235467691, -0.405845151377397,
                                 -0.207784955007898, 0.0, 0.207784955007898, 0.405845151377397,
                                 0.586087235467691, 0.741531185599394, 0.864864423359769,
                                 0.949107912342759, 0.991455371120813};
HGD_TABLE double c_wkq[15] = {0.022935322010529, 0.063092092629979, 0.104790010322250,
                                 0.140653259715525, 0.169004726639267, 0.190350578064785,
                                 0.204432940075298, 0.209482141084728, 0.204432940075298,
                                 0.190350578064785, 0.169004726639267, 0.140653259715525,
                                 0.104790010322250, 0.063092092629979, 0.022935322010529};

// Adaptive Gauss-Kronrod 7-15 (AQUADF :2387-2532 / AQUAD :2599-2745) with an
// explicit stack: an interval is split while (200|K-G|)^1.5 > eps and it is
// wider than eps.  kind 0 integrates d_gfun(tag), kind 1 d_ffun(no, tag).
template <int KIND>
HGD inline double d_aquad(const LintonPar& lp, double r, double wvn, int no, double a, double b,
                                 double eps, int tag, int* status) {
  const int kMaxStack = 64;
  double sa[kMaxStack], sb[kMaxStack];
  int top = 0;
  sa[0] = a; sb[0] = b; top = 1;
  double total = 0.0;
  int guard = 0;
  while (top > 0) {
    --top;
    const double aa = sa[top], bb = sb[top];
    double stf[7], gi = 0.0, gk = 0.0;
    for (int i = 0; i < 7; ++i) {
      const double t = 0.5 * (bb + aa + (bb - aa) * c_xgq[i]);
      stf[i] = KIND == 0 ? d_gfun(lp, t, tag) : d_ffun(r, wvn, no, t, tag);
      gi += c_wgq[i] * (bb - aa) / 2.0 * stf[i];
    }
    for (int i = 1; i <= 15; ++i) {
      double f;
      if (i % 2 == 0) f = stf[i / 2 - 1];
      else {
        const double t = 0.5 * (bb + aa + (bb - aa) * c_xkq[i - 1]);
        f = KIND == 0 ? d_gfun(lp, t, tag) : d_ffun(r, wvn, no, t, tag);
      }
      gk += c_wkq[i - 1] * (bb - aa) / 2.0 * f;
    }
    const double err = pow(200.0 * fabs(gk - gi), 1.5);
    if (err > eps && fabs(aa - bb) > eps && top + 2 <= kMaxStack && guard < 4096) {
      const double mid = (aa + bb) / 2.0;
      sa[top] = mid; sb[top] = bb; ++top;   // right half, popped second
      sa[top] = aa; sb[top] = mid; ++top;   // left half, popped first
    } else {
      if (err > eps && fabs(aa - bb) > eps) hg_set_status(status, HG_DEV_QUAD_STACK);
      total += gk;
    }
    ++guard;
  }
  return total;
}

// SA0 / DSA0 (:1389-1524): series for the m=0 coefficient and its R-derivative.
HGD inline void d_sa0(double r, double pa, double wk, double& sa, double& dsa, int* status) {
  const double ga = 0.5772156649015328, eps = SPD(1.e-6);
  const double x = (r / pa) * (r / pa), ex = exp(-x), lg = log(wk * r / 2.0);
  // SA0 uses E_{n+1}(x), DSA0 uses E_n(x), n = 1, 2, ...
  double e_n = d_e1xa(x);  // E_1
  double e_np1 = (ex - x * e_n) / 1.0;  // E_2
  double s = -ga - 2.0 * log(wk * pa / 2.0), ds = 0.0, sgn = -1.0, facn = 1.0, psi = 0.0;
  bool sdone = false, ddone = false;
  for (int n = 1; n <= 400; ++n) {
    psi += 1.0 / n;
    if (!sdone) {
      const double rm = sgn * pow(r / pa, 2.0 * n) / facn / n - pow(wk * pa / 2.0, 2.0 * n) / facn * e_np1 -
                        2.0 * sgn / (facn * facn) * pow(wk * r / 2.0, 2.0 * n) * (lg + ga - psi);
      s += rm;
      if (!(fabs(rm) > eps)) sdone = true;
    }
    if (!ddone) {
      const double rm = 2.0 * sgn * pow(r / pa, 2.0 * n - 1.0) / facn / pa +
                        pow(wk * pa / 2.0, 2.0 * n) / facn * e_n * 2.0 * r / (pa * pa) -
                        2.0 * sgn * n * wk / (facn * facn) * pow(wk * r / 2.0, 2.0 * n - 1.0) * (lg + ga - psi) -
                        2.0 * sgn / (facn * facn) * pow(wk * r / 2.0, 2.0 * n) / r;
      ds += rm;
      if (!(fabs(rm) > eps)) ddone = true;
    }
    if (sdone && ddone) break;
    if (n == 400) hg_set_status(status, HG_DEV_SERIES_CAP);
    sgn = -sgn;
    facn *= (n + 1);
    e_n = e_np1;
    e_np1 = (ex - x * e_n) / (double)(n + 1);
  }
  sa = s / 4.0 / HG_PI;
  dsa = ds / 4.0 / HG_PI;
}

// SAM / DSAM (:1575-1693) for m >= 1.
HGD inline void d_sam(double r, double pa, double wvn, double& sa, double& dsa, int* status) {
  const double eps = SPD(1.e-6);
  const double x = (wvn * pa / 2.0) * (wvn * pa / 2.0), ex = exp(-x);
  double e = d_e1xa(x);  // E_{n+1} for n = 0
  double s = 0.0, ds = 0.0, sgn = 1.0, facn = 1.0;
  bool sdone = false, ddone = false;
  // SAM runs n = 0,1,2,... with E_{n+1}; DSAM runs n = 1,2,... with E_{n+1}
  // and the sign/factorial of its own n.
  for (int n = 0; n <= 400; ++n) {
    if (!sdone) {
      const double rm = sgn * pow(r / pa, 2.0 * n) / facn * e;
      s += rm;
      if (!(fabs(rm) > eps)) sdone = true;
    }
    if (n >= 1 && !ddone) {
      const double rm = 2.0 * n * sgn * pow(r / pa, 2.0 * n - 1.0) / facn / pa * e;
      ds += rm;
      if (!(fabs(rm) > eps)) ddone = true;
    }
    if (sdone && ddone) break;
    if (n == 400) hg_set_status(status, HG_DEV_SERIES_CAP);
    sgn = -sgn;
    facn *= (n + 1);
    e = (ex - x * e) / (double)(n + 1);
  }
  sa = s / 4.0 / HG_PI;
  dsa = ds / 4.0 / HG_PI;
}

HGD inline void d_linton(const FinState& st, double r, double zf, double zp, double g[6]) {
  const double eps = SPD(1.e-6), v = st.v, wk = st.wk, h = st.h;
  double a;
  if (v < 0.02) a = 3324.2 * (v * v * v) - 258.89 * (v * v) + 8.3958 * v + 1.3208;
  else if (v < 0.1) a = -30.303 * (v * v * v) - 2.8138 * (v * v) + 2.7740 * v + 0.05052;
  else if (v < 1.0) a = 1.5699 * (v * v * v) - 2.5075 * (v * v) + 1.8316 * v + 0.1077;
  else a = -0.000069641 * (v * v * v) - 0.0017082 * (v * v) + 0.45566 * v + 0.80551;
  a = fabs(a) / (wk * h);
  const double pa = a * h, dnt = pa * pa / 4.0;
  const double sr = sqrt(r * r + (zf - zp) * (zf - zp));
  const double sr1 = sqrt(r * r + (2.0 * h + zf + zp) * (2.0 * h + zf + zp));
  const double sr2 = sqrt(r * r + (zf + zp) * (zf + zp));
  const double p4 = 4.0 * HG_PI;

  // III. evanescent series with coefficients COEF/DCOEF (:1170-1340)
  double re0 = 0.0, re1 = 0.0, re2 = 0.0;
  const double czf = cosh(wk * (zf + h)), czp = cosh(wk * (zp + h)), szf = sinh(wk * (zf + h));
  for (int i = 1; i <= 20; ++i) {
    double cof, dcof;
    const double km = (i == 1) ? wk : st.wvn[i - 1];
    if (i == 1) {
      if (fabs(r) < SPD(1.e-6)) {
        cof = -d_eix(wk * wk * dnt) / 4.0 / HG_PI;
        dcof = 0.0;
      } else if (r / a <= 0.5) {
        d_sa0(r, pa, wk, cof, dcof, st.status);
      } else {
        double j0, j1, y0, y1;
        d_jy01b(wk * r, j0, j1, y0, y1);
        LintonPar dummy{};
        cof = -y0 / 4.0 - d_aquad<1>(dummy, r, wk, 1, 0.0, dnt, eps, 1, st.status);
        dcof = wk * y1 / 4.0 - d_aquad<1>(dummy, r, wk, 1, 0.0, dnt, eps, 2, st.status);
      }
    } else {
      if (fabs(r) < SPD(1.e-6)) {
        cof = d_e1xa(km * km * dnt) / 4.0 / HG_PI;
        dcof = 0.0;
      } else if (r / a <= 1.0) {
        d_sam(r, pa, km, cof, dcof, st.status);
      } else {
        LintonPar dummy{};
        double p1 = dnt + 100.0;
        for (int it = 0; fabs(d_ffun(r, km, i, p1, 1)) > eps; ++it) {
          if (it > 100000) { hg_set_status(st.status, HG_DEV_SERIES_CAP); break; }
          p1 += 100.0;
        }
        cof = d_aquad<1>(dummy, r, km, i, dnt, p1, eps, 1, st.status);
        p1 = dnt + 100.0;
        for (int it = 0; fabs(d_ffun(r, km, i, p1, 2)) > eps; ++it) {
          if (it > 100000) { hg_set_status(st.status, HG_DEV_SERIES_CAP); break; }
          p1 += 100.0;
        }
        dcof = d_aquad<1>(dummy, r, km, i, dnt, p1, eps, 2, st.status);
      }
    }
    double rm1, rm2, rm3;
    if (i == 1) {
      rm1 = -(cof / st.nm0 * czf * czp);
      rm2 = -(dcof / st.nm0 * czf * czp);
      rm3 = -(cof * wk / st.nm0 * szf * czp);
    } else {
      const double nm = h / 2.0 * (1.0 + sin(2.0 * km * h) / (2.0 * km * h));
      double s1, c1;
      sincos(km * (zf + h), &s1, &c1);
      const double c2 = cos(km * (zp + h));
      rm1 = -(cof / nm * c1 * c2);
      rm2 = -(dcof / nm * c1 * c2);
      rm3 = cof * km / nm * s1 * c2;
    }
    re0 += rm1; re1 += rm2; re2 += rm3;
    if (i > 2 && fabs(rm1) < eps && fabs(rm2) < eps && fabs(rm3) < eps) break;
  }

  // IV. error-function image sums
  double e0 = 0.0, e1 = 0.0, e2 = 0.0;
  const double val[4] = {-zp - zf, 2.0 * h - zp + zf, 2.0 * h + zp - zf, 4.0 * h + zp + zf};
  for (int i = 0; i < 4; ++i) {
    const double ro = sqrt(r * r + val[i] * val[i]);
    const double dror = r / ro, droz = val[i] * ((i % 2 == 0) ? -1.0 : 1.0) / ro;
    const double ef = d_erfcc(ro / pa), df = d_derfcc(ro / pa);
    e0 += ef / (p4 * ro);
    e1 += (df / pa * dror * ro - dror * ef) / (p4 * (ro * ro));
    e2 += (df / pa * droz * ro - droz * ef) / (p4 * (ro * ro));
  }
  const double dsr1r = r / sr1, dsr1z = (2.0 * h + zf + zp) / sr1, dsr2r = r / sr2, dsr2z = (zf + zp) / sr2;
  const double ef1 = d_erfcc(sr1 / pa), df1 = d_derfcc(sr1 / pa);
  if (fabs(sr) > SPD(1.e-6)) {
    const double dsrr = r / sr, dsrz = (zf - zp) / sr;
    const double ef = d_erfcc(sr / pa), df = d_derfcc(sr / pa);
    e0 = e0 + (ef - 1.0) / (p4 * sr) + ef1 / (p4 * sr1) - 1.0 / (p4 * sr2);
    e1 = e1 - (ef - 1.0) / (p4 * (sr * sr)) * dsrr + df / (p4 * sr * pa) * dsrr - ef1 / (p4 * (sr1 * sr1)) * dsr1r +
         df1 / (p4 * sr1 * pa) * dsr1r + dsr2r / (p4 * (sr2 * sr2));
    e2 = e2 - (ef - 1.0) / (p4 * (sr * sr)) * dsrz + df / (p4 * sr * pa) * dsrz - ef1 / (p4 * (sr1 * sr1)) * dsr1z +
         df1 / (p4 * sr1 * pa) * dsr1z + dsr2z / (p4 * (sr2 * sr2));
  } else {
    e0 = e0 + ef1 / (p4 * sr1) - 1.0 / (p4 * sr2);
    e1 = e1 - ef1 / (p4 * (sr1 * sr1)) * dsr1r + df1 / (p4 * sr1 * pa) * dsr1r + dsr2r / (p4 * (sr2 * sr2));
    e2 = e2 - ef1 / (p4 * (sr1 * sr1)) * dsr1z + df1 / (p4 * sr1 * pa) * dsr1z + dsr2z / (p4 * (sr2 * sr2));
  }

  // V. integral over [0, PA/2]
  LintonPar lp{v, r, zf, zp, h};
  const double q1 = d_aquad<0>(lp, 0.0, 0.0, 0, 0.0, pa / 2.0, eps, 1, st.status);
  const double q2 = d_aquad<0>(lp, 0.0, 0.0, 0, 0.0, pa / 2.0, eps, 2, st.status);
  const double q3 = d_aquad<0>(lp, 0.0, 0.0, 0, 0.0, pa / 2.0, eps, 3, st.status);
  re0 = re0 - e0 - v / 2.0 / HG_PI * q1;
  re1 = re1 - e1 + v / 2.0 / HG_PI * q2;
  re2 = re2 - e2 - v / 2.0 / HG_PI * q3;

  double bj0, bj1, by0, by1;
  d_jy01b(wk * r, bj0, bj1, by0, by1);
  const double im0 = -(bj0 * czf * czp / 4.0 / st.nm0);
  const double im1 = wk * bj1 * czf * czp / 4.0 / st.nm0;
  const double im2 = -(wk * bj0 * szf * czp / 4.0 / st.nm0);
  g[0] = -p4 * re0; g[1] = -p4 * im0;
  g[2] = -p4 * re1; g[3] = -p4 * im1;
  g[4] = -p4 * re2; g[5] = -p4 * im2;
}

// FINGREEN3D_R dispatch (FinGreen3D.f90:160-226): the Green function minus
// its Rankine pair 1/r + 1/r1 and its derivatives, f = [G, dG/dR, dG/dzq]
// as (re, im) pairs, at horizontal distance rr, source depth zq, field depth zp.
// method: -1 by R/h as the reference; 0 LINTON, 1 PIDCOCK, 2 EIGENE, 3 EIGEN.
HGD inline void fin_regions(const FinState& st, double rr, double zq, double zp, double f[6], int method = -1) {
  if (method < 0) {
    const double rhp = fabs(rr / st.h);
    method = (rhp < 0.0005) ? 0 : (rhp < 0.05) ? 1 : (rhp < 0.5) ? 2 : 3;
  }
  if (method == 0) d_linton(st, rr, zq, zp, f);
  else if (method == 1) d_series_eps(st, rr, zq, zp, f, true);
  else if (method == 2) d_series_eps(st, rr, zq, zp, f, false);
  else d_eigen(st, rr, zq, zp, f);
  if (rr == 0.0) { f[2] = 0.0; f[3] = 0.0; }
}

// FINGREEN3D (FinGreen3D.f90:81-155) for source (xq,yq,zq) and field (xp,yp,zp).
// fpre: the region methods' result f at this pair when already known (the
// de-duplicated near pairs of the mixed form), else nullptr; the arithmetic
// around it is the same either way.
HGD inline void fin_green(const FinState& st, double xq, double yq, double zq, double xp,
                                 double yp, double zp, int flag, double2 g[4], const double* fpre = nullptr) {
  const double xpq = xq - xp, ypq = yq - yp, zpq = zq + zp;
  const double rr = sqrt(xpq * xpq + ypq * ypq);
  const double r = sqrt(rr * rr + (zp - zq) * (zp - zq));
  const double r1 = sqrt(rr * rr + zpq * zpq);
  const double ir1 = 1.0 / r1, ir13 = ir1 * ir1 * ir1, ir = 1.0 / r, ir3 = ir * ir * ir;
  g[0] = make_double2(0.0, 0.0); g[1] = g[0]; g[2] = g[0]; g[3] = g[0];
  const double v = st.v;
  if (!(fabs(v) < SPD(1.e-8)) && fabs(v + 1.0) < SPD(1.e-8)) {
    g[0].x = -ir1; g[1].x = xpq * ir13; g[2].x = ypq * ir13; g[3].x = zpq * ir13;
    if (flag == 0) { g[0].x += ir; g[1].x -= xpq * ir3; g[2].x -= ypq * ir3; g[3].x -= (zq - zp) * ir3; }
    return;
  }
  if (!(fabs(v) < SPD(1.e-8))) {
    double f[6];
    if (fpre) {
      for (int q = 0; q < 6; ++q) f[q] = fpre[q];
    } else {
      fin_regions(st, rr, zq, zp, f);
    }
    if (rr > SPD(1.e-6)) {
      const double cx = xpq / rr, cy = ypq / rr;
      g[1] = make_double2(f[2] * cx, f[3] * cx);
      g[2] = make_double2(f[2] * cy, f[3] * cy);
    }
    g[0] = make_double2(f[0], f[1]);
    g[3] = make_double2(f[4], f[5]);
  }
  g[0].x += ir1; g[1].x -= xpq * ir13; g[2].x -= ypq * ir13; g[3].x -= zpq * ir13;
  if (flag == 0) { g[0].x += ir; g[1].x -= xpq * ir3; g[2].x -= ypq * ir3; g[3].x -= (zq - zp) * ir3; }
}

}  // namespace hg
