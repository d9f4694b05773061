/*
 * Oracle (test infrastructure only): the O(N^2) pair loop, influence
 * matrix and right-hand-side assembly, irregular-frequency normal
 * equations and force integration, restated from HAMS-MREL:
 *   src/CalGreenFunc.f90:49-252, src/CalGreenFuncMulti.f90:112-318,
 *   src/BodyIntgr.f90:48-173, src/BodyIntgr_irr.f90:49-234,
 *   src/AssbMatx.f90:53-251, src/AssbMatx_irr.f90:53-466,
 *   src/AssbMatxMulti.f90:124-251, src/PotentWavForce.f90:44-221,
 *   src/PotentWavForceMulti.f90:45-226.
 * NSYS = 1 (no geometric symmetry), as in every shipped fixture and
 * benchmark configuration; the symmetry factors are then all 1.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "hams_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI = 3.141592653589793;
static const double RHO = 1000.0;

static void panel_vertices(const or_mesh *m, int j, double xq[4][3])
{
    int k, c;
    for (c = 0; c < 4; ++c) {
        int id = (c < m->ncn[j]) ? m->ncon[4 * j + c] : m->ncon[4 * j + 0];
        for (k = 0; k < 3; ++k) xq[c][k] = m->nodes[3 * (id - 1) + k];
    }
}

/* Per pair: FLAG (CalGreenFunc.f90:72-77), Newman integral (used only when
 * FLAG=1, so skipped otherwise), Green function, GRN_KIND rounding. */
static void pair_terms(const or_mesh *m, const double *xf, int j, double v, const double *wvn,
                       int nk, double h, int grn_kind, int *flag, double rkn[4], zdouble grn[4])
{
    const double *xq = m->xyz_p + 3 * j;
    double dist = sqrt((xf[0] - xq[0]) * (xf[0] - xq[0]) + (xf[1] - xq[1]) * (xf[1] - xq[1])
                       + (xf[2] - xq[2]) * (xf[2] - xq[2]));
    int k;
    *flag = (dist <= 50.0 * m->pnsz[j]) ? 1 : 0;
    rkn[0] = rkn[1] = rkn[2] = rkn[3] = 0.0;
    if (*flag) {
        double verts[4][3];
        panel_vertices(m, j, verts);
        or_sglintbd(verts, m->ncn[j], xf, &rkn[0], &rkn[1]);
    }
    if (h < 0.0) or_infgreen3d(xq[0], xf[0], xq[1], xf[1], xq[2], xf[2], v, grn, *flag);
    else or_fingreen3d(xq[0], xf[0], xq[1], xf[1], xq[2], xf[2], v, wvn, nk, h, grn, *flag);
    if (grn_kind == 4) {
        for (k = 0; k < 4; ++k) {
            rkn[k] = (double)(float)rkn[k];
            grn[k] = (double)(float)creal(grn[k]) + I * (double)(float)cimag(grn[k]);
        }
    }
}

int or_assemble(const or_mesh *m, double v, const double *wvn, int nk, double h,
                int grn_kind, int nthreads, zdouble *amat, zdouble *smat)
{
    const int n = m->n, tn = m->n + m->nl;
    int i;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (i = 0; i < tn; ++i) {
        const double *xf = (i < n) ? m->xyz_p + 3 * i : m->lid_xyz_p + 3 * (i - n);
        int j;
        for (j = 0; j < n; ++j) {
            double rkn[4], ear = m->ds[j];
            const double *env = m->dxyz_p + 6 * j;
            zdouble grn[4], tindp, dum;
            int flag;
            pair_terms(m, xf, j, v, wvn, nk, h, grn_kind, &flag, rkn, grn);
            /* BODINT_LEFT  BodyIntgr.f90:64-74 */
            if (flag == 1)
                tindp = (rkn[1] + grn[1] * ear) * env[0] + (rkn[2] + grn[2] * ear) * env[1]
                      + (rkn[3] + grn[3] * ear) * env[2];
            else
                tindp = (grn[1] * env[0] + grn[2] * env[1] + grn[3] * env[2]) * ear;
            /* ASSB_LEFT  AssbMatx.f90:73-101: 2*pi on the hull diagonal */
            amat[(size_t)j * tn + i] = ((i == j) ? 2.0 * PI : 0.0) + tindp;
            /* DUM of RBC_RIGHT / DBC_RIGHT  BodyIntgr.f90:98-102 */
            dum = (flag == 1) ? rkn[0] + grn[0] * ear : grn[0] * ear;
            smat[(size_t)j * tn + i] = dum;
        }
    }
    return 0;
}

/* ASSB_RBC (AssbMatx.f90:123-181) and ASSB_RBC_MULTI (AssbMatxMulti.f90:124-181):
 * one 6-column block per body with the source loop restricted to that body. */
void or_rhs_radiation(const or_mesh *m, const zdouble *smat, int nbody,
                      const int *body_start, const int *body_end, zdouble *brmat)
{
    const int tn = m->n + m->nl;
    int b;
    for (b = 0; b < nbody; ++b) {
        int i;
#pragma omp parallel for schedule(dynamic, 16)
        for (i = 0; i < tn; ++i) {
            zdouble btmp[6] = {0, 0, 0, 0, 0, 0};
            int j, md;
            for (j = body_start[b]; j < body_end[b]; ++j) {
                zdouble dum = smat[(size_t)j * tn + i];
                for (md = 0; md < 6; ++md) btmp[md] = btmp[md] + dum * m->dxyz_p[6 * j + md];
            }
            for (md = 0; md < 6; ++md) brmat[(size_t)(6 * b + md) * tn + i] = btmp[md];
        }
    }
}

/* ASSB_DBC  AssbMatx.f90:187-251 with DBC_RIGHT BodyIntgr.f90:134-173 */
void or_rhs_diffraction(const or_mesh *m, const zdouble *smat, double beta, double v,
                        double wk, double w1, double h, zdouble *bdmat)
{
    const int n = m->n, tn = m->n + m->nl;
    zdouble *dum2 = (zdouble *)malloc(sizeof(zdouble) * (size_t)n);
    int i, j;
    for (j = 0; j < n; ++j) {
        const double *xq = m->xyz_p + 3 * j, *env = m->dxyz_p + 6 * j;
        zdouble dpox, dpoy, dpoz;
        or_dinp(xq[0], xq[1], xq[2], beta, v, wk, w1, h, &dpox, &dpoy, &dpoz);
        dum2[j] = dpox * env[0] + dpoy * env[1] + dpoz * env[2];
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (i = 0; i < tn; ++i) {
        zdouble btmp = 0.0;
        int jj;
        for (jj = 0; jj < n; ++jj) btmp = btmp + (0.0 - smat[(size_t)jj * tn + i] * dum2[jj]);
        bdmat[i] = btmp;
    }
    free(dum2);
}

/* CMAT = A^T A, AssbMatx_irr.f90:151-169 */
void or_normal_equations(int tn, int n, const zdouble *amat, zdouble *cmat)
{
    int i;
#pragma omp parallel for schedule(dynamic, 16)
    for (i = 0; i < n; ++i) {
        int j, k;
        for (j = 0; j < n; ++j) {
            zdouble s = 0.0;
            for (k = 0; k < tn; ++k) s = s + amat[(size_t)i * tn + k] * amat[(size_t)j * tn + k];
            cmat[(size_t)j * n + i] = s;
        }
    }
}

/* DRMAT / DDMAT = A^T b, AssbMatx_irr.f90:300-318, 447-463 */
void or_normal_rhs(int tn, int n, const zdouble *amat, int nrhs, const zdouble *b, zdouble *d)
{
    int i;
#pragma omp parallel for schedule(dynamic, 16)
    for (i = 0; i < n; ++i) {
        int c, k;
        for (c = 0; c < nrhs; ++c) {
            zdouble s = 0.0;
            for (k = 0; k < tn; ++k) s = s + b[(size_t)c * tn + k] * amat[(size_t)i * tn + k];
            d[(size_t)c * n + i] = s;
        }
    }
}

/* RFORCE  PotentWavForce.f90:136-221 (RFORCE_MULTI is the same over a
 * panel range and a column block). amas/bdmp are [6][6] row-major with
 * amas[k*6+md] = AMAS(k+1, md+1). */
void or_rforce(int i0, int i1, const double *ds, const double *dxyz_p, double w1,
               const zdouble *phi, int ldphi, double *amas, double *bdmp)
{
    int md, iel, k;
    for (k = 0; k < 36; ++k) { amas[k] = 0.0; bdmp[k] = 0.0; }
    for (md = 0; md < 6; ++md) {
        for (iel = i0; iel < i1; ++iel) {
            zdouble p = phi[(size_t)md * ldphi + iel];
            zdouble rphi = (I * RHO) * p * ds[iel];
            zdouble iphi = (I * RHO) * w1 * p * ds[iel];
            for (k = 0; k < 6; ++k) {
                amas[k * 6 + md] = amas[k * 6 + md] + cimag(rphi * dxyz_p[6 * iel + k]);
                bdmp[k * 6 + md] = bdmp[k * 6 + md] - creal(iphi * dxyz_p[6 * iel + k]);
            }
        }
    }
}

/* EFORCE  PotentWavForce.f90:44-131 */
void or_eforce(int i0, int i1, const double *xyz_p, const double *ds, const double *dxyz_p,
               double w1, double beta, double v, double wk, double h, int isol,
               const zdouble *phi7, zdouble exfc[6])
{
    zdouble force[6] = {0, 0, 0, 0, 0, 0};
    int iel, k;
    for (iel = i0; iel < i1; ++iel) {
        const double *xp = xyz_p + 3 * iel;
        zdouble p;
        if (isol == 1) p = (phi7[iel] + or_vinp(xp[0], xp[1], xp[2], beta, v, wk, w1, h)) * ds[iel];
        else p = phi7[iel] * ds[iel];
        for (k = 0; k < 6; ++k) force[k] = force[k] + p * dxyz_p[6 * iel + k];
    }
    for (k = 0; k < 6; ++k) exfc[k] = (I * w1) * RHO * force[k];
}

/* Single pair, for kernel-level parity tests: flag, rkn[4], grn[4]. */
void or_pair(const or_mesh *m, int row, int col, double v, const double *wvn, int nk, double h,
             int *flag, double rkn[4], zdouble grn[4])
{
    const double *xf = (row < m->n) ? m->xyz_p + 3 * row : m->lid_xyz_p + 3 * (row - m->n);
    pair_terms(m, xf, col, v, wvn, nk, h, 8, flag, rkn, grn);
}

/* Green function at arbitrary points, for kernel-level tests of every
 * finite-depth region. */
void or_green_point(double xq, double yq, double zq, double xp, double yp, double zp, double v,
                    const double *wvn, int nk, double h, int flag, double *out8)
{
    zdouble g[4];
    int k;
    if (h < 0.0) or_infgreen3d(xq, xp, yq, yp, zq, zp, v, g, flag);
    else or_fingreen3d(xq, xp, yq, yp, zq, zp, v, wvn, nk, h, g, flag);
    for (k = 0; k < 4; ++k) { out8[2 * k] = creal(g[k]); out8[2 * k + 1] = cimag(g[k]); }
}

/* CalPotential / CalPotentialMulti (src/PressureElevation.f90:53-250,
 * src/PressureElevationMulti.f90:55-272) for NSYS = 1, every solved column at
 * once; see hams_oracle.h. */
static int on_body(const or_mesh *m, const double *p)
{
    int j;
    for (j = 0; j < m->n; ++j) {
        const double *en = m->dxyz_p + 6 * j;
        const double tolp = fmax(1.0e-6, 1.0e-3 * m->pnsz[j]), tola = 1.0e-3 * m->pnsz[j] * m->pnsz[j];
        const int ncv = m->ncn[j];
        const double *va = m->nodes + 3 * (m->ncon[4 * j] - 1);
        double dpln = (p[0] - va[0]) * en[0] + (p[1] - va[1]) * en[1] + (p[2] - va[2]) * en[2];
        double smin = 1.0e30, smax = -1.0e30;
        int kk;
        if (fabs(dpln) > tolp) continue;
        for (kk = 0; kk < ncv; ++kk) {
            const double *a = m->nodes + 3 * (m->ncon[4 * j + kk] - 1);
            const double *b = m->nodes + 3 * (m->ncon[4 * j + (kk + 1 < ncv ? kk + 1 : 0)] - 1);
            const double ev[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
            const double wv[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
            const double cx = ev[1] * wv[2] - ev[2] * wv[1], cy = ev[2] * wv[0] - ev[0] * wv[2],
                         cz = ev[0] * wv[1] - ev[1] * wv[0];
            const double sv = cx * en[0] + cy * en[1] + cz * en[2];
            smin = fmin(smin, sv);
            smax = fmax(smax, sv);
        }
        if (smin >= -tola || smax <= tola) return 1;
    }
    return 0;
}

void or_field_potential(const or_mesh *m, int npts, const double *xf, double v, double wk, double w1,
                        const double *wvn, int nk, double h, int nbody, const int *body_start, const int *body_end,
                        int nbeta, const double *betas, int isol, const zdouble *mxpot, int ldm, zdouble *pot)
{
    const int n = m->n, ncol = 6 * nbody + nbeta;
    zdouble *dinc = (zdouble *)malloc(sizeof(zdouble) * (size_t)n * (nbeta > 0 ? nbeta : 1));
    int p, j, k;
    for (k = 0; k < nbeta; ++k)
        for (j = 0; j < n; ++j) {
            const double *xq = m->xyz_p + 3 * j, *env = m->dxyz_p + 6 * j;
            zdouble dx, dy, dz;
            or_dinp(xq[0], xq[1], xq[2], betas[k], v, wk, w1, h, &dx, &dy, &dz);
            dinc[(size_t)k * n + j] = dx * env[0] + dy * env[1] + dz * env[2];
        }
#pragma omp parallel for schedule(dynamic, 4)
    for (p = 0; p < npts; ++p) {
        const double *x = xf + 3 * p;
        zdouble *acc = (zdouble *)calloc((size_t)ncol, sizeof(zdouble));
        int jj, c, b;
        for (jj = 0; jj < n; ++jj) {
            double rkn[4], ear = m->ds[jj];
            const double *env = m->dxyz_p + 6 * jj;
            zdouble grn[4], dum1, dum2;
            int flag;
            pair_terms(m, x, jj, v, wvn, nk, h, 8, &flag, rkn, grn);
            if (flag == 1) {
                dum1 = rkn[0] + grn[0] * ear;
                dum2 = (rkn[1] + grn[1] * ear) * env[0] + (rkn[2] + grn[2] * ear) * env[1]
                     + (rkn[3] + grn[3] * ear) * env[2];
            } else {
                dum1 = grn[0] * ear;
                dum2 = (grn[1] * env[0] + grn[2] * env[1] + grn[3] * env[2]) * ear;
            }
            for (b = 0; b < nbody; ++b) {
                const int in = (jj >= body_start[b] && jj < body_end[b]);
                int md;
                for (md = 0; md < 6; ++md) {
                    c = 6 * b + md;
                    acc[c] += (in ? dum1 * env[md] : 0.0) - dum2 * mxpot[(size_t)c * ldm + jj];
                }
            }
            for (k = 0; k < nbeta; ++k) {
                c = 6 * nbody + k;
                acc[c] += -dum1 * dinc[(size_t)k * n + jj] - dum2 * mxpot[(size_t)c * ldm + jj];
            }
        }
        {
            const double sld = on_body(m, x) ? 2.0 * PI : 4.0 * PI;
            const int special = fabs(v) < (double)1.e-8f || fabs(v + 1.0) < (double)1.e-8f;
            for (c = 0; c < ncol; ++c) {
                zdouble r = acc[c] / sld;
                if (c >= 6 * nbody && isol == 1 && !special)
                    r += or_vinp(x[0], x[1], x[2], betas[c - 6 * nbody], v, wk, w1, h);
                pot[(size_t)c * npts + p] = r;
            }
        }
        free(acc);
    }
    free(dinc);
}

