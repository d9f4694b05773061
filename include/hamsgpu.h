/*
 * hamsgpu: GB300 (sm_103a) library for the HAMS-MREL per-frequency
 * boundary-integral path.  C ABI: plain pointers and sizes, no C++ or CUDA
 * types, callable from Fortran through ISO_C_BINDING.
 *
 * Array conventions follow the Fortran caller: every 2-D array is
 * column-major (Fortran order), node and panel indices inside NCON are
 * 1-based, complex numbers are interleaved (re, im) doubles, i.e.
 * COMPLEX*16.  The library owns every device buffer; host pointers passed
 * in are only read or written during the call.
 *
 * Status codes follow LAPACK: 0 success, < 0 the -k-th argument is invalid,
 * > 0 a zero pivot at that 1-based row of the LU.  CUDA failures and
 * device-side status bits return HG_ERR_CUDA / HG_ERR_DEVICE with a message
 * available from hg_last_error().  No call aborts the process.
 *
 * Threading: one context per host thread at a time; calls on a context are
 * serialised by the caller and run on the context's own CUDA stream.
 */
#ifndef HAMSGPU_H
#define HAMSGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_ERR_CUDA (-1000)
#define HG_ERR_DEVICE (-1001)
#define HG_ERR_STATE (-1002)
#define HG_ERR_ALLOC (-1003)

/* Precision of the solve. */
#define HG_PREC_FP64 0   /* plain form: complex128 throughout */
#define HG_PREC_MIXED 1  /* precision form: complex64 fill and LU, FP64 iterative refinement */

typedef struct hg_ctx hg_ctx;

typedef struct {
    int device;          /* CUDA device ordinal */
    int precision;       /* HG_PREC_FP64 or HG_PREC_MIXED */
    int grn_kind;        /* 8: Green values kept in double; 4: rounded to single precision
                            before assembly, as the reference's GRN_KIND=4 storage
                            (src/WavDynMods.f90:47) */
    int max_refine;      /* mixed form: maximum refinement sweeps (default 10) */
    double refine_tol;   /* mixed form: stop when max_k ||A x_k - b_k|| / ||b_k|| <= tol (default 1e-10) */
    double rho;          /* fluid density for the forces (reference Const_mod: 1000) */
    double g;            /* gravity for VINP (reference Const_mod: 9.80665) */
    int lu_tensor;       /* mixed form, order >= 1024: trailing updates of the complex64 LU on the
                            tensor cores, 2 = split BF16 (three products at the BF16 rate,
                            ~2^-16 product error, one refinement sweep at the benchmark
                            configurations; default), 3 = split TF32 (three products,
                            single-precision quality), 1 = TF32 (one product, more refinement
                            sweeps), 0 = FP32 SIMT kernels only.  Plain form, order >= 1024:
                            any value but 0 runs U12 and the trailing updates of the complex128
                            LU on the tensor cores as exact BF16 digit products (FP64
                            accuracy, Ozaki et al. 2012); 0 keeps them on the FP64 pipes */
    int refine_method;   /* mixed form: 0 = classical iterative refinement (x += LU^-1 r per
                            sweep; default), 1 = GMRES-based refinement (restarted GMRES of
                            src/IterativeSolvers.f90:324-488 on A d = r, right-preconditioned by
                            the complex64 LU); both stop on refine_tol / max_refine */
    int fin_table;       /* mixed form, finite depth: Green function from per-frequency tables of
                            FINGREEN3D's own values (exact split into functions of (R, zq-zp)
                            and (R, zq+zp), bicubic interpolation in FP32) for the pairs with
                            R/h >= 0.05; the pairs below (LINTON and PIDCOCK, whose values jump
                            with R) are evaluated per pair in FP64 after the tables; A, B, F
                            within 1e-4 of the FP64 oracle (measured 5e-6..4e-5):
                            1 on, 0 off (FP64 per pair), -1 automatic (on from 1e6 pairs; default) */
    int solver;          /* linear solver, the ControlFile's Solver_type (ISOLV, src/HAMS_Prog.f90:161):
                            1 = LU and triangular solves (default); 2 = restarted GMRES(25) of
                            src/IterativeSolvers.f90:324-488 on the dense matrix in device memory,
                            stopping at ||r||_2 < 1e-4 ||b||_2 per right-hand side or after 100
                            iterations, right-preconditioned by Jacobi (one body) or by the LU of
                            each body's diagonal block (several bodies), as the reference's
                            ZBLOCK_GMRES_SOLVE; hg_fill_factor then factors only those blocks */
    int hmatrix;         /* solver 2: 1 = the GMRES products through the reference's H-matrix
                            (src/HMatrix.f90: cluster tree of the panel centres, at most 32 per
                            leaf; admissible blocks, centres > 2 x the larger diameter apart,
                            compressed by ACA to 1e-4 with rank <= 50; dense near field), built
                            on the device from the assembled matrix after each fill, as the
                            reference's ISOLV = 2 does; 0 = the dense matrix (default: one
                            bandwidth-bound pass, no compression error) */
} hg_opts;

/* Fill opts with the defaults above (device 0, FP64, GRN_KIND 8, rho 1000, g 9.80665, lu_tensor 2,
 * solver 1, hmatrix 0). */
void hg_default_opts(hg_opts *opts);

/* Create / destroy a context.  opts may be NULL for the defaults. */
int hg_create(hg_ctx **ctx, const hg_opts *opts);
void hg_destroy(hg_ctx *ctx);
const char *hg_last_error(const hg_ctx *ctx);

/*
 * Mesh, once per run after CalNormals / BuildCombinedArrays
 * (src/ReadPanelMesh.f90:110-190, src/CalGreenFuncMulti.f90:53-106).
 * Replaces the module-global geometry that CALGREEN reads
 * (src/CalGreenFunc.f90:49-118): XYZ, NCON, NCN, XYZ_P, DS, PNSZ, DXYZ_P
 * and, for IRSP=1, iXYZ_P.
 *   n, ntnd          hull panels and nodes (global, body-major order)
 *   nodes[ntnd*3]    XYZ(NTND,3)
 *   ncon[n*4]        NCON(NELEM,4), 1-based node ids
 *   ncn[n]           NCN, 3 or 4
 *   xyz_p[n*3]       XYZ_P(NELEM,3) panel centroids
 *   ds[n], pnsz[n]   areas and longest edges
 *   dxyz_p[n*6]      DXYZ_P(NELEM,6) generalized normals
 *   nl, lid_xyz_p    lid (waterplane) panel count and centroids iXYZ_P(iNELEM,3); nl = 0 without lids
 *   nbody            number of bodies
 *   body_ranges[2*nbody]  1-based first,last hull panel of each body (NELEM_TOTAL_RAD)
 */
int hg_set_mesh(hg_ctx *ctx, int n, int ntnd, const double *nodes, const int *ncon, const int *ncn,
                const double *xyz_p, const double *ds, const double *pnsz, const double *dxyz_p,
                int nl, const double *lid_xyz_p, int nbody, const int *body_ranges);

/*
 * Wave state of one frequency, after CalWaveProperts (src/ImplementSubs.f90:40-151):
 * v = w^2/g (0 and -1 select the zero/infinite-frequency limits), wk = wave number,
 * w1 = circular frequency, h = depth (< 0 deep water), wvn[nk] = DISPERSION roots
 * (ignored in deep water; may be NULL then).
 */
int hg_set_frequency(hg_ctx *ctx, double v, double wk, double w1, double h, const double *wvn, int nk);

/*
 * CALGREEN / CALGREEN_IRR / CALGREEN_MULTI(_IRR) + ASSB_LEFT* including ZGETRF
 * (src/AssbMatx.f90:53-116, src/AssbMatx_irr.f90:53-180): Green fill, influence
 * matrix, for irsp = 1 the normal equations C = A^T A, and the LU.
 * Returns 0, or the 1-based row of a zero pivot, or an error code.
 */
int hg_fill_factor(hg_ctx *ctx, int irsp);

/*
 * ASSB_RBC* + RADIATION_SOLVER* (src/AssbMatx.f90:123-181, :257-312): radiation
 * potentials of all 6*nbody modes into mxpot (column-major, leading dimension
 * ldm >= n, 6*nbody columns, COMPLEX*16).
 */
int hg_solve_radiation(hg_ctx *ctx, double *mxpot, int ldm);

/*
 * ASSB_DBC* + DIFFRACTION_SOLVER* for nbeta headings at once (radians):
 * diffraction potentials into mxpot_dif (ldm >= n, nbeta columns).
 * hg_solve_diffraction is the one-heading form of the reference interface.
 */
int hg_solve_all_headings(hg_ctx *ctx, const double *betas, int nbeta, double *mxpot_dif, int ldm);
int hg_solve_diffraction(hg_ctx *ctx, double beta, double *mxpot_col);

/*
 * RFORCE_MULTI / EFORCE_MULTI (src/PotentWavForceMulti.f90:45-226) on the device
 * from the last radiation and diffraction solves:
 *   amas[6nb*6nb], bdmp[6nb*6nb]  column-major AMAS/BDMP (row = force DOF, column = mode)
 *   exfc[nbeta*6nb]               COMPLEX*16, column-major (heading, DOF)
 * isol = 1 adds the incident potential (ISOL of ControlFile.in).
 */
int hg_forces(hg_ctx *ctx, int isol, double *amas, double *bdmp, double *exfc);

/*
 * One frequency-solve in one call: set_frequency + fill_factor + radiation +
 * all headings + forces.  mxpot may be NULL (no potential read-back); else it
 * receives n x (6*nbody + nbeta) COMPLEX*16 with leading dimension ldm.
 */
int hg_solve_frequency(hg_ctx *ctx, double v, double wk, double w1, double h, const double *wvn, int nk,
                       int irsp, const double *betas, int nbeta, int isol, double *amas, double *bdmp,
                       double *exfc, double *mxpot, int ldm);

/*
 * Potential, pressure or free-surface elevation at field points from the last
 * solve of this context; replaces CalPotential / CalPressure / CalElevation
 * (src/PressureElevation.f90:53-336) and CalPotentialMulti / CalPressureMulti /
 * CalElevationMulti (src/PressureElevationMulti.f90:55-360), which the reference
 * calls once per point and mode from WritePressureElevation
 * (PressureElevation.f90:380-460): here every point and every solved column
 * in one call.
 *   xyz[npts*3]    field points XET(3, NPTS) (x, y, z of each point together)
 *   kind           0 potential, 1 pressure (i w rho pot), 2 elevation (i w/g pot)
 *   isol           1 adds the incident potential to the diffraction columns
 *   out            COMPLEX*16 (ldo, 6*nbody + nbeta): columns as in mxpot of
 *                  hg_solve_frequency (radiation mode 6b+m, then headings);
 *                  the heading columns only after a diffraction solve
 * SLD = 2 pi for points on a panel (the reference's on-surface test), 4 pi
 * elsewhere.  Needs a radiation solve first (HG_ERR_STATE otherwise).
 */
int hg_field_points(hg_ctx *ctx, int npts, const double *xyz, int kind, int isol, double *out, int ldo);

/*
 * A frequency sweep: the frequency loop of HAMS_Prog (src/HAMS_Prog.f90:255-304
 * single body, :613-704 multi-body) over nfreq frequencies of one mesh, depth,
 * heading set and irsp, each frequency the work of hg_solve_frequency.
 * Frequencies are independent, so nslots solve slots (child contexts holding
 * their own copy of the mesh, device buffers and CUDA stream, created on the
 * first call and kept) take them in turn from one queue and run concurrently
 * on the device: one slot's latency-bound LU panels share the GPU with
 * another's Green fill and tensor-core updates.  nslots = 1 runs them in order.
 *   v, wk, w1[nfreq]    wave state per frequency (as hg_set_frequency)
 *   wvn[nk * nfreq]     dispersion roots per frequency (finite depth only)
 *   amas, bdmp          (6nb x 6nb) x nfreq, column-major per frequency
 *   exfc                (nbeta x 6nb COMPLEX*16) x nfreq
 *   mxpot               optional (NULL: none): potentials, (ldm x (6nb + nbeta)
 *                       COMPLEX*16) x nfreq, radiation modes then headings
 *   latency_ms[nfreq]   optional: host wall time of each frequency-solve
 * Each slot holds about 5 n^2 x 8 bytes of device memory in the mixed form
 * (16 bytes per entry in the FP64 form).  On an error in any frequency the
 * other slots stop taking new frequencies and the call returns that error
 * (frequency and slot in hg_last_error).  The device work of the sweep is
 * ordered after earlier work on ctx's stream, and later work on ctx's stream
 * (e.g. hg_mark) after the sweep.
 */
int hg_solve_sweep(hg_ctx *ctx, int nfreq, const double *v, const double *wk, const double *w1, double h,
                   const double *wvn, int nk, int irsp, const double *betas, int nbeta, int isol, int nslots,
                   double *amas, double *bdmp, double *exfc, double *mxpot, int ldm, float *latency_ms);

/*
 * Device bytes one frequency-solve of this size holds in a context (matrices,
 * factor workspace, right-hand sides, refinement buffers, mesh) with the
 * default solver and classical refinement: what the serving loop below
 * reserves per solve in flight, plus, under opts.solver = 2 or
 * refine_method = 1, the GMRES bases (and solver 2's preconditioner blocks).
 * 0 for invalid sizes.
 */
size_t hg_solve_footprint(int precision, int n, int nl, int nbody, int nbeta, int irsp, int lu_tensor);

/*
 * Serving: continuous batching of frequency-solve requests (the serving form
 * of this path; the reference runs one request per process, HAMS_Prog).  A
 * request is a mesh (as hg_set_mesh), a depth, nfreq frequencies (wave state
 * per frequency as hg_set_frequency; wvn nk x nfreq for finite depth) and
 * nbeta headings.  hg_server_submit copies the request and returns at once;
 * nslots solve slots (contexts with their own stream and host thread) run
 * the frequencies of all admitted requests as slots free up, so requests
 * that arrive while others run join the mix and their solves overlap on the
 * device.  Admission: requests are admitted in arrival order while the
 * reserved device memory, min(nslots, nfreq) x hg_solve_footprint + mesh per
 * admitted request, stays within budget_bytes; a request larger than the
 * budget is rejected by hg_server_submit (-3).  Each result equals that of
 * hg_solve_frequency on a single context (same kernels, same order).
 *   hg_server_wait: blocks (timeout_s <= 0) or waits up to timeout_s seconds
 *     (returns 1 if the request is not finished); copies amas, bdmp
 *     ((6nb)^2 x nfreq), exfc (nbeta x 6nb COMPLEX*16 x nfreq) and
 *     latency_ms[2] = (submit to done, submit to admission); a ticket can be
 *     collected once.  A failed request returns its first error.
 *   hg_server_stats: stats[8] = requests done, frequency-solves done,
 *     reserved bytes, peak reserved bytes, most requests admitted at once,
 *     queued requests, admitted requests, budget.
 * hg_server_destroy stops the slots (unfinished requests are dropped).
 */
typedef struct hg_server hg_server;
typedef struct {
    int n, ntnd;
    const double *nodes;
    const int *ncon, *ncn;
    const double *xyz_p, *ds, *pnsz, *dxyz_p;
    int nl;
    const double *lid_xyz_p;
    int nbody;
    const int *body_ranges;
    double h;
    int nfreq;
    const double *v, *wk, *w1, *wvn;
    int nk, irsp, isol, nbeta;
    const double *betas;
} hg_request;

int hg_server_create(hg_server **srv, const hg_opts *opts, int nslots, double budget_bytes);
int hg_server_submit(hg_server *srv, const hg_request *req, long long *ticket);
int hg_server_wait(hg_server *srv, long long ticket, double timeout_s, double *amas, double *bdmp, double *exfc,
                   double *latency_ms);
int hg_server_stats(hg_server *srv, double *stats);
/* Device timeline of the finished frequency-solves (for showing that the
 * solves of different requests overlap on the GPU): out[4 k .. 4 k + 3] =
 * ticket, frequency index, start and end in milliseconds since the server
 * was created, from CUDA events recorded on the slot's stream around the
 * solve.  Copies min(max_entries, count) entries; returns count (all
 * entries so far), or < 0 on a bad argument. */
int hg_server_timeline(hg_server *srv, int max_entries, double *out);
const char *hg_server_last_error(const hg_server *srv);
void hg_server_destroy(hg_server *srv);

/* Diagnostics for tests: copy the tn x n influence matrix (which = 0, before
 * factorisation) or single-layer matrix (which = 1) of the last fill to host
 * memory (COMPLEX*16, leading dimension ld >= tn).  Requires hg_fill_factor
 * to have run with keep_matrices enabled by hg_keep_matrices(ctx, 1). */
int hg_keep_matrices(hg_ctx *ctx, int keep);
int hg_get_matrix(hg_ctx *ctx, int which, double *out, int ld);

/* Green function of the current frequency at npts arbitrary point pairs:
 * pts[6*k..] = (xq, yq, zq, xp, yp, zp) source and field, flags[k] in {0,1}
 * (FLAG of INFGREEN3D / FINGREEN3D), out[8*k..] = GRN(1..4) as (re, im). */
int hg_green_points(hg_ctx *ctx, int npts, const double *pts, const int *flags, double *out);

/* Host-side helpers (no device work).
 * hg_dispersion: DISPERSION (src/WavDynSubs.f90:40-126), nk roots for depth h > 0.
 * hg_wave_properties: CalWaveProperts (src/ImplementSubs.f90:40-151) for one
 *   frequency-list entry; inft as Input_frequency_type (1..5); h < 0 deep water.
 * hg_panel_geometry: CalPanelCentre / CalPanelArea / CalPanelChartLength /
 *   CalTransNormals / CalRotNormals (src/NormalProcess.f90) for n panels.
 * Each returns 0 or a negative argument index (> 0: a root failed to converge). */
int hg_dispersion(double w, double h, int nk, double *wvn);
int hg_wave_properties(int inft, double value, double h, int nk, double *v, double *wk, double *w1,
                       double *wvn);
int hg_panel_geometry(int n, int ntnd, const double *nodes, const int *ncon, const int *ncn, const double *xr,
                      double *xyz_p, double *ds, double *pnsz, double *dxyz_p);

/* hg_green_points without device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory once their run
 * is under way (a driver loop evaluating the wave field under a fixed memory
 * budget, a server that carves up device memory at start-up): the points,
 * flags and results are staged in one fixed array the library keeps in
 * device global memory (7.25 MiB on every GPU that loads the library, held
 * until exit), so the call makes no cudaMalloc / cudaFree.
 *   - npts may not exceed HG_NOALLOC_MAX_POINTS; larger calls return -2 with
 *     a message in hg_last_error (split them).
 *   - The first call on a device looks up the array's device address; make
 *     that first call before any stream capture.
 *   - All calls on a device share the array, and each call overwrites the
 *     part it uses: calls that overlap on the GPU (several host threads or
 *     contexts at once) race and must be serialised by the caller.
 *   - The looked-up address is kept for the life of the process.  A caller
 *     that resets a device (cudaDeviceReset) must not call this entry point
 *     on that device again in the same process: the kept address would no
 *     longer be valid.
 * Arguments, results and errors are those of hg_green_points. */
#define HG_NOALLOC_MAX_POINTS 65536
int hg_green_points_noalloc(hg_ctx *ctx, int npts, const double *pts, const int *flags, double *out);

/* Dense complex solve A X = B on the device, the ZGETRF + ZGETRS pair of
 * src/AssbMatx.f90:111,277 (and AssbMatx_irr.f90:175,491) for a matrix the
 * caller already holds.  a: n x n COMPLEX*16 (lda >= n), b: n x nrhs
 * (ldb >= n), ipiv: n 1-based pivot rows.
 *   precision 0 (ZGESV): a <- complex128 LU factors, b <- X, *iter = 0.
 *   precision 1 (ZCGESV-style): LU in complex64, X refined with residuals
 *     against the complex128 matrix until max|r|/max|b| <= refine_tol per
 *     column; a <- the complex64 factors widened to complex128, *iter = the
 *     sweeps taken.  If max_refine sweeps do not reach the tolerance the
 *     solve is redone in complex128 (a <- complex128 factors) and *iter = -31.
 * *info = 0, or i > 0 when U(i,i) is exactly zero (b is then left as it came).
 * Device buffers are allocated for the call and freed before it returns. */
int hg_gesv(hg_ctx *ctx, int precision, int n, int nrhs, double *a, int lda, int *ipiv, double *b, int ldb,
            int *iter, int *info);

/* Refinement sweeps taken and final relative residual of the last mixed-form solve. */
int hg_refine_info(const hg_ctx *ctx, int *sweeps, double *residual);
/* GMRES iterations (preconditioned operator applications) of the last mixed-form solve
 * with refine_method = 1 (0 otherwise). */
int hg_gmres_iterations(const hg_ctx *ctx, int *iterations);
/* Outcome of the last solve with opts.solver = 2: Arnoldi steps taken (the largest over the
 * right-hand sides, <= 100), restart cycles, right-hand sides left above the tolerance after
 * 100 steps (the reference prints "GMRES did not converge" for each; their solution is the
 * last iterate), and the largest final ||r||_2 / ||b||_2 estimate.  HG_ERR_STATE when
 * opts.solver is not 2. */
int hg_iter_info(const hg_ctx *ctx, int *iterations, int *restarts, int *unconverged, double *residual);

/* The H-matrix of the last fill (opts.solver 2 with opts.hmatrix 1): block count, dense and
 * low-rank blocks, mean rank of the low-rank blocks, and its storage against the dense matrix's
 * (n^2 complex128 entries over the blocks' entries).  HG_ERR_STATE without one. */
int hg_hmatrix_info(const hg_ctx *ctx, int *nblocks, int *ndense, int *nlowrank, double *mean_rank,
                    double *compression);

/* CUDA events on the context's stream, for callers that time a sequence of
 * calls on the device: hg_mark records event slot (0..15); hg_elapsed waits
 * for the later one and returns the milliseconds between two slots. */
int hg_mark(hg_ctx *ctx, int slot);
int hg_elapsed(hg_ctx *ctx, int slot0, int slot1, float *ms);

/* Average device time (ms) of the library's complex GEMM kernel
 * C = C - A B on an m x n x k problem, over iters launches on scratch
 * buffers; used to report the roofline of the LU trailing update.
 * precision (kernel variant): 0 complex128 SIMT, 1 complex64 SIMT,
 * 2 complex64 tensor cores split TF32 (3 products), 3 complex64 tensor
 * cores TF32 (1 product), 4 complex64 tensor cores split BF16 (3 products
 * at the BF16 rate), 5 complex128 tensor cores as exact BF16 digit products
 * (36 digit pairs, FP64 accuracy); 2-5 include their operand packing or
 * slicing. */
int hg_bench_gemm(hg_ctx *ctx, int precision, int m, int n, int k, int iters, float *ms_per_launch);

/* Average device time (ms, CUDA events around each launch) of the
 * complex64 32-column panel LU of the blocked factorisation (the 16-CTA
 * cluster kernel; the IZAMAX pivot search, interchange, scaling and rank-1
 * updates of ZGETF2 inside ZGETRF, src/AssbMatx.f90:111) on an m x 32 panel
 * of pseudo-random entries, restored before each of iters (<= 64) launches;
 * used to report the roofline of the panel. */
int hg_bench_panel(hg_ctx *ctx, int m, int iters, float *ms_per_launch);

/* C = C - A B through one of those kernel variants on host arrays (all
 * COMPLEX*16, column-major; variants 1-4 round A, B, C to complex64 on the
 * device and widen the result back, variants 0 and 5 stay in complex128).  A test hook for the LU update
 * kernels; the reference's counterpart is the ZGEMM step inside ZGETRF. */
int hg_gemm_check(hg_ctx *ctx, int variant, int m, int n, int k, const double *a, int lda, const double *b,
                  int ldb, double *c, int ldc);

/* out = b - A y (all COMPLEX*16, column-major; A rounded to complex64 on the
 * device, as the mixed form's matrix is) through the refinement residual's
 * kernels: variant 0 the double-float products on the FP32 pipes, 1 the
 * sliced products on the tensor cores (Ozaki et al. 2012: BF16 digits of the
 * row- and column-scaled operands, exact FP32 partial sums).  nc <= 40.  A
 * test hook for the residual of the refinement. */
/* y = H x for the H-matrix of the COMPLEX*16 n x n matrix a (lda) with panel centres xyz (n x 3,
 * column-major), for nc columns x (n x nc, leading dimension n; y the same), built on the device as
 * opts.hmatrix does (src/HMatrix.f90: HMATRIX_BUILD, HMATVEC).  stats (may be NULL) receives the
 * block count, dense blocks, low-rank blocks and the sum of their ranks.  A test hook for the
 * H-matrix. */
int hg_hmatrix_check(hg_ctx *ctx, int n, const double *a, int lda, const double *xyz, int nc, const double *x,
                     double *y, long long *stats);

/* The H-matrix's partition alone, on the host (no device needed): the cluster order perm (n
 * entries, 0-based original index at each cluster position, SPLIT_CLUSTER_ITERATIVE of
 * src/HMatrix.f90:236-381) and up to max_blocks blocks in build order (BUILD_BLOCK_TREE_ITERATIVE,
 * :390-497), five ints each: row start, rows, column start, columns (0-based cluster positions),
 * admissible (1) or a dense leaf pair (0).  Returns the block count, or a negative value on bad
 * arguments. */
int hg_hmatrix_partition(int n, const double *xyz, int *perm, int *blocks, int max_blocks);

int hg_resid_check(hg_ctx *ctx, int variant, int m, int nc, int k, const double *a, int lda, const double *y,
                   int ldy, const double *b, int ldb, double *out, int ldo);

/* Time (milliseconds, CUDA events on the context stream) of the stages of the
 * last hg_solve_frequency: [0] fill, [1] LU, [2] solves and refinement, [3] forces. */
int hg_stage_times(const hg_ctx *ctx, float *ms4);

/*
 * A whole HAMS run from its input deck (the HAMS_Prog executable's work for
 * NSYS = 1): ControlFile.in, HullMesh[_b].pnl, WaterPlaneMesh[_b].pnl (IRSP =
 * 1) and gen_mod_<b>_<dof>.txt in input_dir, read as ReadControlFile
 * (src/InputFiles.f90:46-224), ReadBodyMesh(Multi) / ReadWTPLMesh(Multi)
 * (src/ReadPanelMesh.f90, src/ReadPanelMeshMulti.f90) and CalNormals read
 * them; every frequency of the list solved on the device; results written as
 * the reference writes them:
 *   <out>/Hams_format/OAMASS1-6.txt, ODAMPING1-6.txt, OEXFOR1-6.txt
 *       (RFORCE / EFORCE, src/PotentWavForce.f90:100-218 and the Multi forms)
 *   <out>/Wamit_format/AmssDamp.1, ExcForce.3 (the same routines, in the
 *       order they write: per frequency and body pair)
 *   <out>/Wamit_format/PressureElevation.6p for field points
 *       (src/PressureElevation.f90:336-470, through hg_field_points); with
 *       several bodies also PressureElevationIncidence.6p, and with the
 *       control file's separate-files flag PressureElevationRadiation_<b>.6p
 *       per body plus PressureElevationDiffraction.6p instead
 *       (src/PressureElevationMulti.f90:407-587, src/InputFiles.f90:318-338)
 *   <out>/Wamit_format/Motion.4, Hydrostat.hst when Hydrostatic[_b].in are
 *       present (SolveMotion / SolveMotionMulti, src/SolveMotion*.f90;
 *       ReadHydroStatic, src/HydroStatic*.f90)
 *   <out>/Hydrostar_format/AddedMass_ij.rao, WaveDamping_ij.rao,
 *       Excitation_k.rao, Motion_k.rao for a single body (src/PrintOutput.f90)
 * hg_case_read parses and computes the panel geometry and wave properties
 * (host only); hg_case_info / hg_case_arrays expose what was read:
 *   info[12]  = n, nl, ntnd, nbody, nper, nbeta, irsp, isol, nfp, sybo, inft, ouft
 *   dinfo[2]  = h, refl
 *   freq[6*nper] = (V, WK, W1, TP, WL, OUFR) per entry
 * hg_case_run solves and writes (nslots frequencies in flight, as
 * hg_solve_sweep; one at a time when field points are written); the deck's
 * Solver_type (src/InputFiles.f90:177-191) sets opts->solver.
 * hg_case_write writes the result files from given A, B, F (per entry
 * blocks as hg_solve_sweep returns them); it also (re)creates the
 * pressure/elevation .6p files of the run empty, as the reference's
 * CreateWamitFiles does, so a driver writing its own field-point output to
 * output_dir must call it first.  Errors: non-zero return, message
 * in err[errlen].  Symmetry planes (ISX/ISY) are rejected. */
typedef struct hg_case hg_case;
int hg_case_read(const char *input_dir, hg_case **out, char *err, int errlen);
void hg_case_free(hg_case *c);
int hg_case_info(const hg_case *c, int *info, double *dinfo);
/* The deck's Solver_type (ISOLV, 1 or 2) and separate-files flag (0 or 1; always 0 for one body). */
int hg_case_options(const hg_case *c, int *isolv, int *separate);
int hg_case_arrays(const hg_case *c, double *nodes, int *ncon, int *ncn, double *xyz_p, double *ds, double *pnsz,
                   double *dxyz_p, double *lid_xyz_p, int *body_ranges, double *freq, double *headings);
int hg_case_run(hg_case *c, const char *output_dir, const hg_opts *opts, int nslots, char *err, int errlen);
int hg_case_write(const hg_case *c, const char *output_dir, const double *amas, const double *bdmp,
                  const double *exfc, double rho, double g, char *err, int errlen);

#ifdef __cplusplus
}
#endif
#endif
