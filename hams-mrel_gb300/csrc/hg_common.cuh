// Shared device-side definitions of the GB300 per-frequency BEM library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define HG_PI 3.141592653589793

// Device status word bits (written by kernels, read by the host after each
// stage).  A kernel that hits an iteration cap or a bounded wait sets a bit
// and returns; it never traps.
enum {
  HG_DEV_OK = 0,
  HG_DEV_SERIES_CAP = 1,      // a convergence loop of the finite-depth Green function hit its cap
  HG_DEV_QUAD_STACK = 2,      // adaptive quadrature stack overflow
  HG_DEV_WAIT_TIMEOUT = 4,    // an mbarrier wait gave up
  HG_DEV_ZERO_PIVOT = 8,      // exact zero pivot in the LU
};

// Single-precision literal of the Fortran source promoted to double.
#define SPD(x) ((double)(float)(x))

struct zc {
  double re, im;
};

__host__ __device__ __forceinline__ double2 zmake(double r, double i) { return make_double2(r, i); }
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 zdiv(double2 a, double2 b) {
  // Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.y + b.x * r;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cdivf(float2 a, float2 b) {
  if (fabsf(b.x) >= fabsf(b.y)) {
    float r = b.y / b.x, d = b.x + b.y * r;
    return make_float2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    float r = b.x / b.y, d = b.y + b.x * r;
    return make_float2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}

// ---------------------------------------------------------------------------
// Source-panel record: everything the pair kernel needs about one hull
// panel, precomputed once per mesh (the Newman local frame of
// SingularIntgr.f90:150-179 for triangles and :372-427 for quadrilaterals).
// 36 doubles = 288 bytes, a multiple of 16 so a tile of records can be
// moved into shared memory by one bulk-async (TMA) copy.
// ---------------------------------------------------------------------------
enum {
  PR_XQ = 0,      // centroid x,y,z (XYZ_P)
  PR_N = 3,       // unit normal (DXYZ_P(:,1:3))
  PR_DS = 6,      // area DS
  PR_FLAGD = 7,   // 50 * PNSZ: pairs closer than this get the analytic Rankine integral
  PR_PO = 8,      // Newman origin
  PR_UI = 11,
  PR_UJ = 14,
  PR_UK = 17,
  PR_KSI = 20,    // local vertex coordinates (4)
  PR_ETA = 24,
  PR_L = 28,      // edge lengths (4)
  PR_NCN = 32,    // 3 or 4
  PR_SIZE = 36
};

struct HgStatus {
  int flags;
  int detail;
};

#ifdef __CUDACC__
__host__ __device__
#endif
inline void hg_set_status(int* status, int bit) {
#ifdef __CUDA_ARCH__
  if (status) atomicOr(status, bit);
#else
  if (status) *status |= bit;
#endif
}
