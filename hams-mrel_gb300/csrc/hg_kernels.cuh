// Host-callable launchers of the fill / right-hand-side / force kernels.
#pragma once
#include <cuda_runtime.h>
#include "hg_common.cuh"

namespace hg {

struct FinState;

__device__ __forceinline__ void store_c(double2* p, double re, double im) { *p = make_double2(re, im); }
__device__ __forceinline__ void store_c(float2* p, double re, double im) { *p = make_float2((float)re, (float)im); }

// Gauss points of the single-precision panel integrals (hg_green32.cuh,
// panel_gauss_f): kPanelGauss float4 per panel, relative to (ox, oy).
constexpr int kPanelGauss = 13;
cudaError_t launch_panel_gauss(cudaStream_t st, int n, const double* rec, double ox, double oy, float4* pg);

cudaError_t launch_prep_panels(cudaStream_t st, int n, int ntnd, const double* nodes, const int* ncon, const int* ncn,
                               const double* xyz_p, const double* ds, const double* pnsz, const double* dxyz_p,
                               double* rec, int* status);

template <typename OUT>
cudaError_t launch_green_fill(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                              const FinState& fs, bool deep, int grn_kind, OUT* A, OUT* S, long lda, int* status,
                              int* bins = nullptr, int ndiag = -1);  // ndiag: rows with the 2 pi free term (-1: all)

template <typename OUT>
cudaError_t launch_green_fill_fin(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                  const FinState& fs, int grn_kind, OUT* A, OUT* S, long lda, int* status,
                                  int* bins, int ndiag);
// Finite depth, complex64 output, compiled with FMA contraction (mixed form).
cudaError_t launch_green_fill_fin_fma(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                      const FinState& fs, int grn_kind, float2* A, float2* S, long lda, int* status,
                                      int* bins);
// Finite depth, complex64 output, only the pairs with R/h < 0.05 (LINTON and
// PIDCOCK), written over A and S with the reference's arithmetic (no FMA);
// bins: scratch of fin_bins_ints(n, tn) ints.
cudaError_t launch_fin_near(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                            const FinState& fs, int grn_kind, float2* A, float2* S, long lda, int* bins, int ndiag);
// The same pairs with their region-method values computed once per distinct
// (R, zq, zp), keyed exactly (hg_fill_fin.cu).  zsrc[n] / zfld[tn]: index of
// each source's / field point's depth in the mesh's distinct depths zlev (at
// most 2048).  near_count: number of near pairs into *counter (device).
// near_build: two hash tables of near_table_size(np) slots (cap) - R's bits,
// then the keys -, the pairs listed as (i + j tn, key slot), the distinct
// keys grouped by cost into ukeys (R's bits, depth indices) with
// slot2u[slot] = key index; counters[1 + 15] = number of keys afterwards.
// near_map: pair slots to key indices.  near_fill (per frequency): the
// region methods per key into F (6 doubles each), then A(i, j), S(i, j) of
// every near pair.
int near_count(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double h,
               const short* zsrc, const short* zfld, int* counter);
unsigned near_table_size(int npairs);
cudaError_t near_build(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double h,
                       const short* zsrc, const short* zfld, unsigned long long* tabr, unsigned long long* tabk,
                       unsigned cap, int* counters, int* slot2u, int2* pairs, longlong2* ukeys);
cudaError_t near_map(cudaStream_t st, int np, int2* pairs, const int* slot2u);
cudaError_t near_fill(cudaStream_t st, const double* rec, const double* fx, int ldf, int tn, int np, int nu,
                      const int2* pairs, const longlong2* ukeys, const double* zlev, double* F, const FinState& fs,
                      int grn_kind, float2* A, float2* S, long lda, int ndiag);
// Tabulated finite-depth Green function of the mixed form (hg_fintab.cu):
// fintab_floats() floats of device scratch; rmax = largest horizontal
// distance between a field point and a source; gmin = first R segment built
// and used (2: the pairs below R/h = 0.05 come from launch_fin_near).
struct FinTab;
size_t fintab_floats();
cudaError_t fintab_build(cudaStream_t st, const FinState& fs, double rmax, float* buf, FinTab* out, int gmin = 0);
// diag: device scratch of 6 n floats (the coincident pairs' FP64 values).
cudaError_t launch_green_fill_mixed_fin(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                        const FinState& fs, const FinTab& tab, double ox, double oy,
                                        const float4* pg, float* diag, float2* A, float2* S, long lda, int* status);
// Scratch ints of the cost-binned finite-depth fill: bin cursors + one pair index per pair.
inline size_t fin_bins_ints(int n, int tn) { return 16 + (size_t)n * tn; }
cudaError_t launch_green_points_fin(cudaStream_t st, int npts, const double* pts, const int* flags, const FinState& fs,
                                    double* out);

// ndiag: rows with the 2 pi free term (-1: all).  near_list (optional): the
// self and adjacent pairs (i + j tn, from mixed_near_build, near_np of them),
// evaluated by a kernel of their own after the FP32 tile kernel, which then
// skips them; without it the tile kernel evaluates every pair.
cudaError_t launch_green_fill_mixed(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn,
                                    double v, double ox, double oy, const float4* pg, float2* A, float2* S, long lda,
                                    int* status, int ndiag = -1, const int* near_list = nullptr, int near_np = 0);
// The deep-water mixed fill's self and adjacent pairs for the field points fx
// (tn rows): mixed_near_count into *counter (device), mixed_near_build lists
// them (list of *counter ints).
int mixed_near_count(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double ox,
                     double oy, int* counter);
cudaError_t mixed_near_build(cudaStream_t st, const double* rec, const double* fx, int ldf, int n, int tn, double ox,
                             double oy, int* counter, int* list);

cudaError_t launch_incident(cudaStream_t st, int n, const double* xyz_p, const double* dxyz_p, int nbeta,
                            const double* betas, double v, double wk, double w1, double h, double2* w);

size_t rhs_work_bytes(int n, int tn, int nbody, int nbeta);

template <typename IN>
cudaError_t launch_rhs(cudaStream_t st, int n, int tn, const IN* S, long lds, const double* dxyz_p, const int* body_of,
                       int nbody, int nbeta, const double2* w, double2* part, double2* B, long ldb);

// Source columns of the right-hand sides as one n x (6 nbody + nbeta) complex
// matrix: column 6b + k holds the k-th generalised normal on body b's panels
// (zero elsewhere), column 6 nbody + h the incident normal velocity w[:, h].
// B = S W then gives every right-hand side at once.
cudaError_t launch_rhs_cols(cudaStream_t st, int n, const double* dxyz_p, const int* body_of, int nbody, int nbeta,
                            const double2* w, double2* W, long ldw);

// Field points (hg_field.cu): onb[p] = 1 where point p (npts x 3 column-major,
// leading dimension ldp) lies on a panel; the finishing pass of the field
// potentials acc (npts x ncol, columns >= nrad are diffraction headings).
cudaError_t launch_field_on_body(cudaStream_t st, int npts, const double* px, int ldp, int n, int ntnd,
                                 const double* nodes, const int* ncon, const int* ncn, const double* dxyz,
                                 const double* pnsz, int* onb);
cudaError_t launch_field_finish(cudaStream_t st, int npts, int ncol, int nrad, double2* acc, long lda, const int* onb,
                                const double* px, int ldp, const double* betas, double v, double wk, double w1,
                                double h, double g, double rho, int isol, int kind);

cudaError_t launch_forces(cudaStream_t st, int n, const double2* X, long ldx, const double* xyz_p, const double* ds,
                          const double* dxyz_p, const int* body_start, const int* body_end, int nbody, int nbeta,
                          const double* betas, double v, double wk, double w1, double h, int isol, double rho,
                          double g, double* amas, double* bdmp, double2* exfc);

cudaError_t launch_green_points(cudaStream_t st, int npts, const double* pts, const int* flags, const FinState& fs,
                                bool deep, double* out);

}  // namespace hg
