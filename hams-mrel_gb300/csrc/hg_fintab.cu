// Build of the finite-depth Green-function tables (hg_fintab.cuh): FP64
// evaluations of the reference's region methods (fin_regions, the method of
// the node's R segment) at the grid nodes, minus the propagating term that
// the pairs add back themselves.  Threads of a warp share a distance R_i (the
// fastest index runs along W or U), so they take the same method and series
// length.
#include "hg_fintab.cuh"
#include "hg_green.cuh"
#include "hg_kernels.cuh"

namespace hg {
namespace {

__device__ __forceinline__ void node_r(const FinTab& T, int i, double* r, int* g) {
  int s = 0;
  while (s + 1 < kFinSegs && i >= T.so[s + 1]) ++s;
  const double a = T.sa[s], b = T.sb[s], c = T.sc[s];
  const double u = (T.sn[s] > 1) ? (double)(i - T.so[s]) / (T.sn[s] - 1) : 0.0;
  *r = (c > 0.0) ? a + (b - a) * expm1(c * u) / expm1(c) : a + (b - a) * u;
  *g = s;
}

// F minus the propagating term at (R, W, U), by method g.
__device__ __forceinline__ void f_minus_prop(const FinState& fs, const FinTab& T, double r, double w, double u, int g,
                                             double out[6]) {
  const double zq = 0.5 * (u + w), zp = 0.5 * (u - w);
  double f[6], p[6];
  fin_regions(fs, r, zq, zp, f, g);
  fintab_prop<double>(fs.wk, T.pk_d, fs.h, r, zq, zp, p);
  for (int q = 0; q < 6; ++q) out[q] = f[q] - p[q];
}

// Nodes of the R segments from T.gmin on (the first i0 = T.so[T.gmin] R
// nodes are not built).
__global__ void k_fintab_build(FinState fs, FinTab T, float* __restrict__ tp, float* __restrict__ tq) {
  const int i0 = T.so[T.gmin];
  const long ntp = (long)(T.nr - i0) * T.nw, ntq = (long)(T.nr - i0) * T.nu;
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= ntp + ntq) return;
  const double h = fs.h;
  double f[6];
  float* out;
  if (e < ntp) {
    const int i = i0 + (int)(e / T.nw), j = (int)(e % T.nw);
    double r;
    int g;
    node_r(T, i, &r, &g);
    const double w = -h + (j + 0.5) * 2.0 * h / T.nw;
    f_minus_prop(fs, T, r, w, -h, g, f);
    out = tp + ((size_t)i * T.nw + j) * 8;
  } else {
    const long e2 = e - ntp;
    const int i = i0 + (int)(e2 / T.nu), k = (int)(e2 % T.nu);
    double r;
    int g;
    node_r(T, i, &r, &g);
    const double u = fmax(-(double)T.u0 * expm1((double)T.dt * (k + 0.5)), -1.98 * h);  // off the bottom image
    const double wr = 0.5 * fmin(fmin(-u, 2.0 * h + u), h);
    double f2[6];
    f_minus_prop(fs, T, r, wr, u, g, f);
    f_minus_prop(fs, T, r, wr, -h, g, f2);
    for (int q = 0; q < 6; ++q) f[q] -= f2[q];
    out = tq + ((size_t)i * T.nu + k) * 8;
  }
  for (int q = 0; q < 6; ++q) out[q] = (float)f[q];
  out[6] = 0.f;
  out[7] = 0.f;
}

}  // namespace

size_t fintab_floats() { return (size_t)8 * kFinTabR * (kFinTabW + kFinTabU); }

cudaError_t fintab_build(cudaStream_t st, const FinState& fs, double rmax, float* buf, FinTab* out, int gmin) {
  if (gmin < 0 || gmin >= kFinSegs) return cudaErrorInvalidValue;
  FinTab T = {};
  T.gmin = gmin;
  const double h = fs.h;
  T.nr = kFinTabR;
  T.nw = kFinTabW;
  T.nu = kFinTabU;
  T.h = (float)h;
  const double ends[kFinSegs + 1] = {0.0, 0.0005 * h, 0.05 * h, 0.5 * h, fmax(rmax, 0.5 * h + 1.0)};
  const double conc[kFinSegs] = {0.0, 3.0, 1.5, 1.0};
  int off = 0;
  for (int g = 0; g < kFinSegs; ++g) {
    T.sa[g] = (float)ends[g];
    T.sb[g] = (float)ends[g + 1];
    T.sc[g] = (float)conc[g];
    T.sx[g] = (float)expm1(conc[g]);
    T.so[g] = off;
    T.sn[g] = kFinSegN[g];
    off += kFinSegN[g];
  }
  T.u0 = 0.05f;
  T.dt = (float)(log1p(2.0 * h / T.u0) / (T.nu - 0.5));
  const double k0 = fs.wk;
  T.k0 = (float)k0;
  const double nm0e = 0.5 * h * exp(-2.0 * k0 * h) + (1.0 - exp(-4.0 * k0 * h)) / (8.0 * k0);  // N0 e^(-2 k0 h)
  T.pk_d = HG_PI / nm0e;
  T.pk = (float)T.pk_d;
  float* tp = buf;
  float* tq = tp + (size_t)8 * T.nr * T.nw;
  T.tp = tp;
  T.tq = tq;
  const long total = (long)(T.nr - T.so[gmin]) * (T.nw + T.nu);
  k_fintab_build<<<(unsigned)((total + 63) / 64), 64, 0, st>>>(fs, T, tp, tq);
  *out = T;
  return cudaGetLastError();
}

}  // namespace hg
