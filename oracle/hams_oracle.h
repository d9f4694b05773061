/*
 * CPU oracle for the HAMS-MREL per-frequency boundary-integral path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * Fortran (HAMS-MREL v2.3, the src directory) used as the checker for the GPU
 * library.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product path never does.
 *
 * Numerical conventions follow the Fortran source literally:
 *   - every literal written without a D exponent in the Fortran is a
 *     single-precision constant promoted to double (SP() below);
 *   - integer powers x**k are repeated multiplication, real powers are pow();
 *   - loops accumulate in the reference's order (field row outer, source
 *     column inner) and the file is compiled with -ffp-contract=off so no
 *     fused multiply-add changes the rounding.
 * Parity is pinned against the reference's own golden outputs
 * (test/data/config1/expected_output, examples/example5_single_body/Output,
 * examples/example3_multi_bodies_gen_mod/Output).  The infinite-depth
 * Green function has no reference fixture (no shipped input uses H<0), so
 * that branch is pinned only through internal identities (reciprocity,
 * Haskind) in the tests.
 */
#ifndef HAMS_ORACLE_H
#define HAMS_ORACLE_H

#include <complex.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Fortran single-precision literal promoted to REAL*8. */
#define SP(x) ((double)(float)(x))

typedef double _Complex zdouble;

/* ---- special functions (FinGrnExtSubs.f90, InfGreen_Appr.f90) ---- */
void   or_error(double x, double *err);                       /* ERROR   FinGrnExtSubs.f90:62  */
void   or_e1xa(double x, double *e1);                         /* E1XA    FinGrnExtSubs.f90:119 */
void   or_enxa(int n, double x, double *en);                  /* ENXA    FinGrnExtSubs.f90:82  */
void   or_eix(double x, double *ei);                          /* EIX     FinGrnExtSubs.f90:146 */
void   or_limes(int n, double *s, double *rlimes);            /* Limes   FinGrnExtSubs.f90:370 */
void   or_ik01a(double x, double *bk0, double *bk1);          /* IK01A   FinGrnExtSubs.f90:538 */
void   or_jy01b(double x, double *j0, double *j1, double *y0, double *y1); /* JY01B :663 */
void   or_jy01bj(double x, double *j0, double *j1);           /* JY01BJ  :741 */
void   or_jy01by0(double x, double *y0);                      /* JY01BY0 :794 */
void   or_jy01by1(double x, double *y1);                      /* JY01BY1 :846 */

/* ---- Green functions ---- */
/* INFGREEN3D  InfGreen_Appr.f90:104-186.  grn[4] complex. */
void or_infgreen3d(double xf, double xp, double yf, double yp, double zf, double zp,
                   double v, zdouble grn[4], int flag);
/* FINGREEN3D  FinGreen3D.f90:81-155.  wvn[nk] from or_dispersion. */
void or_fingreen3d(double xf, double xp, double yf, double yp, double zf, double zp,
                   double v, const double *wvn, int nk, double h, zdouble grn[4], int flag);
/* Branch used by FINGREEN3D_R (FinGreen3D.f90:182-191): 0 LINTON, 1 PIDCOCK,
 * 2 EIGENE, 3 EIGEN.  Exposed so the tests can cover every region. */
int or_fingreen_region(double rr, double h);

/* ---- panel integrals and wave kinematics ---- */
/* SGLINTBD_TRI / SGLINTBD_QUAD  SingularIntgr.f90:44-244, 252-445.
 * xq = vertices [4][3], ncn = 3 or 4, xf = field point. */
void or_sglintbd(const double xq[4][3], int ncn, const double xf[3], double *sij, double dij[3]);
/* DISPERSION  WavDynSubs.f90:40-126 */
void or_dispersion(double *wvn, int nrt, double w, double h);
/* DINP / VINP  PatclVelct.f90:42-123 (XW = 0, AMP = 1 as set by Initialisation) */
void or_dinp(double x, double y, double z, double beta, double v, double wk, double w1,
             double h, zdouble *dpox, zdouble *dpoy, zdouble *dpoz);
zdouble or_vinp(double x, double y, double z, double beta, double v, double wk, double w1, double h);

/* ---- mesh geometry (NormalProcess.f90) ---- */
/* nodes[ntnd][3]; ncon[nelem][4] 1-based; outputs xyz_p[n][3], ds[n], pnsz[n], dxyz_p[n][6].
 * xr = rotation centre used by CalRotNormals. */
void or_geometry(int ntnd, const double *nodes, int nelem, const int *ncn, const int *ncon,
                 const double xr[3], double *xyz_p, double *ds, double *pnsz, double *dxyz_p);

/* ---- assembly (CalGreenFunc*.f90 + BodyIntgr*.f90 + AssbMatx*.f90) ----
 * Hull panels 0..n-1 are the sources for every row.  Rows 0..n-1 are the
 * hull field points; rows n..n+nl-1 the lid field points (IRSP=1).
 * Outputs, column-major with leading dimension tn = n + nl:
 *   amat[tn*n]  : double-layer matrix, 2*pi on the hull diagonal
 *   smat[tn*n]  : single-layer matrix (the DUM of RBC_RIGHT / DBC_RIGHT)
 * grn_kind = 8 keeps the Green values in double; 4 rounds RKBN/CGRN to
 * single precision before assembly as the as-shipped reference does.
 * h < 0 selects deep water.  nthreads <= 0 uses the OpenMP default. */
typedef struct {
    int n, nl, ntnd, ntnd_lid;
    const double *nodes;      /* [ntnd][3]        */
    const int    *ncn;        /* [n]              */
    const int    *ncon;       /* [n][4], 1-based  */
    const double *xyz_p;      /* [n][3]           */
    const double *ds;         /* [n]              */
    const double *pnsz;       /* [n]              */
    const double *dxyz_p;     /* [n][6]           */
    const double *lid_xyz_p;  /* [nl][3]          */
} or_mesh;

int or_assemble(const or_mesh *m, double v, const double *wvn, int nk, double h,
                int grn_kind, int nthreads, zdouble *amat, zdouble *smat);

/* Radiation RHS (ASSB_RBC / ASSB_RBC_MULTI): brmat[tn][6*nbody], with
 * body_start/body_end (0-based, inclusive/exclusive) giving each body's
 * hull panel range. */
void or_rhs_radiation(const or_mesh *m, const zdouble *smat, int nbody,
                      const int *body_start, const int *body_end, zdouble *brmat);
/* Diffraction RHS (ASSB_DBC): bdmat[tn] for heading beta (radians). */
void or_rhs_diffraction(const or_mesh *m, const zdouble *smat, double beta, double v,
                        double wk, double w1, double h, zdouble *bdmat);
/* IRR normal equations (ASSB_LEFT_IRR / ASSB_RBC_IRR): cmat = A^T A (no
 * conjugation), d = A^T b for nrhs columns. */
void or_normal_equations(int tn, int n, const zdouble *amat, zdouble *cmat);
void or_normal_rhs(int tn, int n, const zdouble *amat, int nrhs, const zdouble *b, zdouble *d);

/* RFORCE / RFORCE_MULTI: amas[6][6], bdmp[6][6] (row md1 = force direction)
 * for field panels [i0,i1) and potential columns phi[:, 0..5] (ld = ldphi). */
void or_rforce(int i0, int i1, const double *ds, const double *dxyz_p, double w1,
               const zdouble *phi, int ldphi, double *amas, double *bdmp);
/* EFORCE / EFORCE_MULTI (ISOL = 1 adds the incident potential). */
void or_eforce(int i0, int i1, const double *xyz_p, const double *ds, const double *dxyz_p,
               double w1, double beta, double v, double wk, double h, int isol,
               const zdouble *phi7, zdouble exfc[6]);

/* CalPotential / CalPotentialMulti (PressureElevation.f90:53-250,
 * PressureElevationMulti.f90:55-272), NSYS = 1: the potential at field points
 * xf[npts][3] of every solved column c of mxpot (n rows, leading dimension
 * ldm): c < 6 nbody radiation mode c % 6 of body c / 6 (source weight
 * DXYZ_P(j, mode) on that body's panels), c >= 6 nbody diffraction for
 * betas[c - 6 nbody] (weight -grad phi_I . n); pot = (sum_j DUM1 w - DUM2 phi)
 * / SLD, SLD = 2 pi for a point on a body panel and 4 pi elsewhere, plus VINP
 * for diffraction columns when isol = 1.  pot[p + c * npts]. */
void or_field_potential(const or_mesh *m, int npts, const double *xf, double v, double wk, double w1,
                        const double *wvn, int nk, double h, int nbody, const int *body_start, const int *body_end,
                        int nbeta, const double *betas, int isol, const zdouble *mxpot, int ldm, zdouble *pot);

#ifdef __cplusplus
}
#endif
#endif
