// Host-side pieces of the path that run once per frequency or once per
// mesh: the dispersion roots, the wave properties of one frequency-list
// entry and the panel geometry.  FP64 on the CPU: O(200) work per
// frequency and O(N) per mesh.
#include <cmath>

#include "../../include/hamsgpu.h"

extern "C" {

// DISPERSION, src/WavDynSubs.f90:40-126: wvn[0] is the positive root of
// w^2/g = k tanh(kh), wvn[1..nk-1] the roots of -w^2/g = u tan(uh), by the
// third-order (Halley-type) iteration of Newman (1990) from the same
// starting values, with the reference's g = 9.807 and convergence 1e-10.
int hg_dispersion(double w, double h, int nk, double* wvn) {
  if (!(h > 0.0)) return -2;
  if (nk < 1) return -3;
  if (!wvn) return -4;
  const double g = 9.807, pi = 3.141592653589793;
  const double x = w * w * h / g;
  double y, t;
  if (x > 0.0 && x <= 2.0) {
    y = std::sqrt(x) * (0.9994 + 0.1701 * x + (double)0.0305f * x * x);
  } else {
    t = x * std::exp(-2.0 * x);
    y = x + 2.0 * t - 6.0 * t * t;
  }
  if (std::fabs(y - x) < (double)1.e-10f) {
    wvn[0] = x / h;
  } else {
    double exx = 1.0;
    for (int it = 0; exx > 1.0e-10; ++it) {
      if (it > 200) return 1;
      const double trial = y, dnm = trial * trial - x * x;
      const double fun = std::log((trial + x) / (trial - x)) / 2.0 - trial;
      const double dfun = -x / dnm - 1.0, d2fun = 2.0 * x * trial / (dnm * dnm);
      y = trial - fun / dfun * (1.0 + (fun / dfun) * (d2fun / dfun) / 2.0);
      exx = std::fabs(y - trial);
    }
    wvn[0] = y / h;
  }
  const double u = 3.0 * x / (7.0 + 3.0 * x);
  t = 0.0159 + 0.1032 * u + 4.3152 * u * u - 2.8768 * u * u * u;
  for (int i = 2; i <= nk; ++i) {
    double exx = 1.0;
    for (int it = 0; exx > 1.0e-10; ++it) {
      if (it > 200) return i;
      const double trial = t, yy = (i - 1) * pi - trial, dnm = yy * yy + x * x;
      const double fun = std::atan2(x, yy) - trial;
      const double dfun = x / dnm - 1.0, d2fun = 2.0 * x * trial / (dnm * dnm);
      t = trial - fun / dfun * (1.0 + (fun / dfun) * (d2fun / dfun) / 2.0);
      exx = std::fabs(t - trial);
    }
    wvn[i - 1] = ((i - 1) * pi - t) / h;
    t = t - pi * x / (x * x + pi * i * (pi * (i - 1) - t));
  }
  return 0;
}

// CalWaveProperts, src/ImplementSubs.f90:40-151, for one entry of the
// frequency list.  inft: 1 deep-water wave number, 2 finite-depth wave
// number, 3 circular frequency, 4 period, 5 wave length.  Outputs v = w^2/g
// (G = 9.80665), wk, w1 and, for h > 0, nk dispersion roots.
int hg_wave_properties(int inft, double value, double h, int nk, double* v, double* wk, double* w1, double* wvn) {
  if (inft < 1 || inft > 5) return -1;
  if (!v || !wk || !w1) return -5;
  const double G = 9.80665, pi = 3.141592653589793;
  const bool fin = h > 0.0;
  if (fin && (!wvn || nk < 1)) return -8;
  int rc = 0;
  switch (inft) {
    case 1:
      *v = value;
      *w1 = std::sqrt(G * *v);
      if (fin) { rc = hg_dispersion(*w1, h, nk, wvn); *wk = wvn[0]; }
      else *wk = *v;
      break;
    case 2:
      *wk = value;
      *v = fin ? *wk * std::tanh(*wk * h) : *wk;
      *w1 = std::sqrt(G * *v);
      if (fin) rc = hg_dispersion(*w1, h, nk, wvn);
      break;
    case 3:
    case 4:
      *w1 = (inft == 3) ? value : 2.0 * pi / value;
      *v = *w1 * *w1 / G;
      if (fin) { rc = hg_dispersion(*w1, h, nk, wvn); *wk = wvn[0]; }
      else *wk = *v;
      break;
    default:
      *wk = 2.0 * pi / value;
      *v = fin ? *wk * std::tanh(*wk * h) : *wk;
      *w1 = std::sqrt(G * *v);
      if (fin) rc = hg_dispersion(*w1, h, nk, wvn);
      break;
  }
  return rc;
}

// Panel geometry, src/NormalProcess.f90 (CalPanelCentre :134-159,
// CalPanelArea :171-197 with CalDeltaArea_Improved :373-397,
// CalPanelChartLength :401-441, CalTransNormals :74-124, CalRotNormals
// :46-64).  Fortran (column-major) arrays: nodes(ntnd,3), ncon(n,4) 1-based,
// outputs xyz_p(n,3), ds(n), pnsz(n), dxyz_p(n,6); xr = rotation centre.
int hg_panel_geometry(int n, int ntnd, const double* nodes, const int* ncon, const int* ncn, const double* xr,
                      double* xyz_p, double* ds, double* pnsz, double* dxyz_p) {
  if (n <= 0) return -1;
  if (!nodes || !ncon || !ncn || !xr || !xyz_p || !ds || !pnsz || !dxyz_p) return -3;
  auto P = [&](int e, int c, int k) { return nodes[(ncon[e + (long)c * n] - 1) + (long)k * ntnd]; };
  auto darea = [](const double* p1, const double* p2, const double* p3) {
    double v21[3], v13[3], v23[3];
    for (int k = 0; k < 3; ++k) { v21[k] = p1[k] - p2[k]; v23[k] = p3[k] - p2[k]; v13[k] = p3[k] - p1[k]; }
    const double a = std::sqrt(v21[0] * v21[0] + v21[1] * v21[1] + v21[2] * v21[2]);
    const double b = std::sqrt(v13[0] * v13[0] + v13[1] * v13[1] + v13[2] * v13[2]);
    const double c = std::sqrt(v23[0] * v23[0] + v23[1] * v23[1] + v23[2] * v23[2]);
    return std::sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c))) / 4.0;
  };
  for (int e = 0; e < n; ++e) {
    const int nv = ncn[e];
    if (nv != 3 && nv != 4) return -5;
    for (int c = 0; c < nv; ++c) {
      const int id = ncon[e + (long)c * n];
      if (id < 1 || id > ntnd) return -4;
    }
    double v[4][3];
    for (int c = 0; c < nv; ++c)
      for (int k = 0; k < 3; ++k) v[c][k] = P(e, c, k);
    double cen[3] = {0, 0, 0};
    for (int c = 0; c < nv; ++c)
      for (int k = 0; k < 3; ++k) cen[k] = cen[k] + v[c][k];
    for (int k = 0; k < 3; ++k) { cen[k] = cen[k] / nv; xyz_p[e + (long)k * n] = cen[k]; }
    double a = darea(v[0], v[1], v[2]);
    if (nv == 4) a = a + darea(v[0], v[3], v[2]);
    ds[e] = a;
    double mx = 0.0;
    for (int c = 0; c < nv; ++c) {
      const double* p = v[c];
      const double* q = v[(c + 1) % nv];
      const double l = std::sqrt((q[0] - p[0]) * (q[0] - p[0]) + (q[1] - p[1]) * (q[1] - p[1]) + (q[2] - p[2]) * (q[2] - p[2]));
      mx = (c == 0 || l > mx) ? l : mx;
    }
    pnsz[e] = mx;
    double un[3];
    if (nv == 3) {
      double v21[3], v23[3];
      for (int k = 0; k < 3; ++k) { v21[k] = v[0][k] - v[1][k]; v23[k] = v[2][k] - v[1][k]; }
      un[0] = v21[1] * v23[2] - v21[2] * v23[1];
      un[1] = v21[2] * v23[0] - v21[0] * v23[2];
      un[2] = v21[0] * v23[1] - v21[1] * v23[0];
    } else {
      double v13[3], v24[3];
      for (int k = 0; k < 3; ++k) { v13[k] = v[2][k] - v[0][k]; v24[k] = v[3][k] - v[1][k]; }
      un[0] = v24[1] * v13[2] - v24[2] * v13[1];
      un[1] = v24[2] * v13[0] - v24[0] * v13[2];
      un[2] = v24[0] * v13[1] - v24[1] * v13[0];
    }
    const double aun = std::sqrt(un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
    double nn[3];
    for (int k = 0; k < 3; ++k) { nn[k] = un[k] / aun; dxyz_p[e + (long)k * n] = nn[k]; }
    dxyz_p[e + 3L * n] = (cen[1] - xr[1]) * nn[2] - (cen[2] - xr[2]) * nn[1];
    dxyz_p[e + 4L * n] = (cen[2] - xr[2]) * nn[0] - (cen[0] - xr[0]) * nn[2];
    dxyz_p[e + 5L * n] = (cen[0] - xr[0]) * nn[1] - (cen[1] - xr[1]) * nn[0];
  }
  return 0;
}

}  // extern "C"
