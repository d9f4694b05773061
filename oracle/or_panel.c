/*
 * Oracle (test infrastructure only): panel geometry, Newman's closed-form
 * Rankine panel integrals, the dispersion relation and incident-wave
 * kinematics, restated from HAMS-MREL:
 *   src/NormalProcess.f90, src/SingularIntgr.f90, src/WavDynSubs.f90,
 *   src/PatclVelct.f90.
 */
#include <math.h>
#include "hams_oracle.h"

/* ---------------------------------------------------------------------
 * NormalProcess.f90: CalPanelCentre :134-159, CalPanelArea :171-197,
 * CalDeltaArea_Improved :373-397, CalPanelChartLength :401-441,
 * CalTransNormals :74-124, CalRotNormals :46-64.
 * ------------------------------------------------------------------- */
static void delta_area_improved(const double *p1, const double *p2, const double *p3, double *ds)
{
    double v21[3], v13[3], v23[3], a, b, c, l1, l2, l3, l4;
    int k;
    for (k = 0; k < 3; ++k) { v21[k] = p1[k] - p2[k]; v23[k] = p3[k] - p2[k]; v13[k] = p3[k] - p1[k]; }
    a = sqrt(v21[0] * v21[0] + v21[1] * v21[1] + v21[2] * v21[2]);
    b = sqrt(v13[0] * v13[0] + v13[1] * v13[1] + v13[2] * v13[2]);
    c = sqrt(v23[0] * v23[0] + v23[1] * v23[1] + v23[2] * v23[2]);
    l1 = a + (b + c);
    l2 = c - (a - b);
    l3 = c + (a - b);
    l4 = a + (b - c);
    *ds = sqrt(l1 * l2 * l3 * l4) / 4.0;
}

static double norm3(const double *v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

void or_geometry(int ntnd, const double *nodes, int nelem, const int *ncn, const int *ncon,
                 const double xr[3], double *xyz_p, double *ds, double *pnsz, double *dxyz_p)
{
    int e, j, k;
    (void)ntnd;
#define NODE(id) (nodes + 3 * ((id) - 1))
    for (e = 0; e < nelem; ++e) {
        const int *c = ncon + 4 * e;
        double *xp = xyz_p + 3 * e, *np = dxyz_p + 6 * e;
        /* centre */
        xp[0] = xp[1] = xp[2] = 0.0;
        for (j = 0; j < ncn[e]; ++j)
            for (k = 0; k < 3; ++k) xp[k] = xp[k] + NODE(c[j])[k];
        for (k = 0; k < 3; ++k) xp[k] = xp[k] / ncn[e];
        /* area */
        delta_area_improved(NODE(c[0]), NODE(c[1]), NODE(c[2]), &ds[e]);
        if (ncn[e] == 4) {
            double ads;
            delta_area_improved(NODE(c[0]), NODE(c[3]), NODE(c[2]), &ads);
            ds[e] = ds[e] + ads;
        }
        /* characteristic length */
        {
            double v[4][3], l[4] = {0.0, 0.0, 0.0, 0.0};
            int nv = ncn[e];
            for (j = 0; j < nv; ++j)
                for (k = 0; k < 3; ++k) v[j][k] = NODE(c[(j + 1) % nv])[k] - NODE(c[j])[k];
            for (j = 0; j < nv; ++j) l[j] = norm3(v[j]);
            pnsz[e] = l[0];
            for (j = 1; j < nv; ++j) if (l[j] > pnsz[e]) pnsz[e] = l[j];
        }
        /* unit normal */
        {
            double un[3], aun;
            if (ncn[e] == 3) {
                double v21[3], v23[3];
                for (k = 0; k < 3; ++k) { v21[k] = NODE(c[0])[k] - NODE(c[1])[k]; v23[k] = NODE(c[2])[k] - NODE(c[1])[k]; }
                un[0] = v21[1] * v23[2] - v21[2] * v23[1];
                un[1] = v21[2] * v23[0] - v21[0] * v23[2];
                un[2] = v21[0] * v23[1] - v21[1] * v23[0];
            } else {
                double v13[3], v24[3];
                for (k = 0; k < 3; ++k) { v13[k] = NODE(c[2])[k] - NODE(c[0])[k]; v24[k] = NODE(c[3])[k] - NODE(c[1])[k]; }
                un[0] = v24[1] * v13[2] - v24[2] * v13[1];
                un[1] = v24[2] * v13[0] - v24[0] * v13[2];
                un[2] = v24[0] * v13[1] - v24[1] * v13[0];
            }
            aun = norm3(un);
            np[0] = un[0] / aun; np[1] = un[1] / aun; np[2] = un[2] / aun;
        }
        /* rotational normals about xr */
        np[3] = (xp[1] - xr[1]) * np[2] - (xp[2] - xr[2]) * np[1];
        np[4] = (xp[2] - xr[2]) * np[0] - (xp[0] - xr[0]) * np[2];
        np[5] = (xp[0] - xr[0]) * np[1] - (xp[1] - xr[1]) * np[0];
    }
#undef NODE
}

/* ---------------------------------------------------------------------
 * SGLINTBD_TRI  SingularIntgr.f90:44-244.  Called for NCN=3 panels only
 * (CalGreenFunc.f90:90-96), so the second sub-triangle branch is not taken.
 * ------------------------------------------------------------------- */
static void sglint_tri(const double xq[4][3], const double xf[3], double *sij, double dij[3])
{
    double xv[3][3], p12[3], p13[3], po[3], po3[3], ui[3], uj[3], uk[3], pof[3], po1[3], po2[3];
    double alfa, x, y, z, ksi[4], eta[4], st = 0.0, sxt = 0.0, syt = 0.0, szt = 0.0, n12, n3;
    int i, k;
    *sij = 0.0; dij[0] = dij[1] = dij[2] = 0.0;
    for (k = 0; k < 3; ++k) { xv[0][k] = xq[0][k]; xv[1][k] = xq[1][k]; xv[2][k] = xq[2][k]; }
    for (k = 0; k < 3; ++k) { p12[k] = xv[1][k] - xv[0][k]; p13[k] = xv[2][k] - xv[0][k]; }
    alfa = (p12[0] * p13[0] + p12[1] * p13[1] + p12[2] * p13[2]) / (p12[0] * p12[0] + p12[1] * p12[1] + p12[2] * p12[2]);
    for (k = 0; k < 3; ++k) po[k] = xv[0][k] + alfa * p12[k];
    for (k = 0; k < 3; ++k) po3[k] = xv[2][k] - po[k];
    n12 = sqrt(p12[0] * p12[0] + p12[1] * p12[1] + p12[2] * p12[2]);
    n3 = sqrt(po3[0] * po3[0] + po3[1] * po3[1] + po3[2] * po3[2]);
    for (k = 0; k < 3; ++k) { ui[k] = p12[k] / n12; uj[k] = po3[k] / n3; }
    uk[0] = ui[1] * uj[2] - ui[2] * uj[1];
    uk[1] = ui[2] * uj[0] - ui[0] * uj[2];
    uk[2] = ui[0] * uj[1] - ui[1] * uj[0];
    for (k = 0; k < 3; ++k) pof[k] = xf[k] - po[k];
    x = ui[0] * pof[0] + ui[1] * pof[1] + ui[2] * pof[2];
    y = uj[0] * pof[0] + uj[1] * pof[1] + uj[2] * pof[2];
    z = uk[0] * pof[0] + uk[1] * pof[1] + uk[2] * pof[2];
    for (k = 0; k < 3; ++k) { po1[k] = xv[0][k] - po[k]; po2[k] = xv[1][k] - po[k]; }
    ksi[0] = -copysign(1.0, alfa) * sqrt(po1[0] * po1[0] + po1[1] * po1[1] + po1[2] * po1[2]);
    eta[0] = 0.0;
    ksi[1] = 0.0;
    eta[1] = sqrt(po3[0] * po3[0] + po3[1] * po3[1] + po3[2] * po3[2]);
    ksi[2] = sqrt(po2[0] * po2[0] + po2[1] * po2[1] + po2[2] * po2[2]);
    eta[2] = 0.0;
    ksi[3] = ksi[0];
    eta[3] = eta[0];
    for (i = 0; i < 3; ++i) {
        double dksi = ksi[i + 1] - ksi[i], deta = eta[i + 1] - eta[i];
        double r1 = sqrt((ksi[i] - x) * (ksi[i] - x) + (eta[i] - y) * (eta[i] - y) + z * z);
        double r2 = sqrt((ksi[i + 1] - x) * (ksi[i + 1] - x) + (eta[i + 1] - y) * (eta[i + 1] - y) + z * z);
        double l = sqrt((ksi[i + 1] - ksi[i]) * (ksi[i + 1] - ksi[i]) + (eta[i + 1] - eta[i]) * (eta[i + 1] - eta[i]));
        double b1 = deta * ((ksi[i] - x) * (ksi[i] - x) + z * z) - dksi * (ksi[i] - x) * (eta[i] - y);
        double a1 = r1 * z * dksi;
        double b2 = deta * ((ksi[i + 1] - x) * (ksi[i + 1] - x) + z * z) - dksi * (ksi[i + 1] - x) * (eta[i + 1] - y);
        double a2 = r2 * z * dksi;
        double lgrn;
        if (!(fabs(z) < 1.0e-6)) szt = szt + atan2((b1 * a2 - b2 * a1), (a1 * a2 + b1 * b2));
        if (fabs(r1 + r2 - l) < 1.0e-6) continue;
        lgrn = log((r1 + r2 + l) / (r1 + r2 - l));
        sxt = sxt - deta / l * lgrn;
        syt = syt + dksi / l * lgrn;
        st = st + (deta * (x - ksi[i]) - dksi * (y - eta[i])) / l * lgrn;
    }
    st = st - z * szt;
    *sij = *sij + st;
    for (k = 0; k < 3; ++k) dij[k] = dij[k] + ui[k] * sxt + uj[k] * syt + uk[k] * szt;
}

/* SGLINTBD_QUAD  SingularIntgr.f90:252-445 */
static void sglint_quad(const double xq[4][3], const double xf[3], double *sij, double dij[3])
{
    double xv[4][3], po[3], pov[4][3], pon[4][3], un[3], ui[3], uj[3], uk[3], pof[3];
    double x, y, z, ksi[5], eta[5], st = 0.0, sxt = 0.0, syt = 0.0, szt = 0.0, nn;
    int i, j, k;
    *sij = 0.0; dij[0] = dij[1] = dij[2] = 0.0;
    for (j = 0; j < 4; ++j) for (k = 0; k < 3; ++k) xv[j][k] = xq[j][k];
    for (k = 0; k < 3; ++k) po[k] = (xv[0][k] + xv[1][k] + xv[2][k] + xv[3][k]) / 4.0;
    for (k = 0; k < 3; ++k) { pov[0][k] = xv[0][k] - po[k]; pov[1][k] = xv[1][k] - po[k]; }
    un[0] = pov[0][1] * pov[1][2] - pov[0][2] * pov[1][1];
    un[1] = pov[0][2] * pov[1][0] - pov[0][0] * pov[1][2];
    un[2] = pov[0][0] * pov[1][1] - pov[0][1] * pov[1][0];
    nn = sqrt(pov[0][0] * pov[0][0] + pov[0][1] * pov[0][1] + pov[0][2] * pov[0][2]);
    for (k = 0; k < 3; ++k) ui[k] = pov[0][k] / nn;
    nn = sqrt(un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
    for (k = 0; k < 3; ++k) uk[k] = un[k] / nn;
    uj[0] = uk[1] * ui[2] - uk[2] * ui[1];
    uj[1] = uk[2] * ui[0] - uk[0] * ui[2];
    uj[2] = uk[0] * ui[1] - uk[1] * ui[0];
    for (k = 0; k < 3; ++k) pof[k] = xf[k] - po[k];
    x = ui[0] * pof[0] + ui[1] * pof[1] + ui[2] * pof[2];
    y = uj[0] * pof[0] + uj[1] * pof[1] + uj[2] * pof[2];
    z = uk[0] * pof[0] + uk[1] * pof[1] + uk[2] * pof[2];
    for (k = 0; k < 3; ++k) { pov[2][k] = xv[2][k] - po[k]; pov[3][k] = xv[3][k] - po[k]; }
    for (i = 0; i < 4; ++i) {
        double d = uk[0] * pov[i][0] + uk[1] * pov[i][1] + uk[2] * pov[i][2];
        for (j = 0; j < 3; ++j) pon[i][j] = pov[i][j] - d * uk[j];
    }
    for (i = 0; i < 4; ++i) {
        ksi[i] = ui[0] * pon[i][0] + ui[1] * pon[i][1] + ui[2] * pon[i][2];
        eta[i] = uj[0] * pon[i][0] + uj[1] * pon[i][1] + uj[2] * pon[i][2];
    }
    ksi[4] = ksi[0];
    eta[4] = eta[0];
    for (i = 0; i < 4; ++i) {
        double dksi = ksi[i + 1] - ksi[i], deta = eta[i + 1] - eta[i];
        double r1 = sqrt((ksi[i] - x) * (ksi[i] - x) + (eta[i] - y) * (eta[i] - y) + z * z);
        double r2 = sqrt((ksi[i + 1] - x) * (ksi[i + 1] - x) + (eta[i + 1] - y) * (eta[i + 1] - y) + z * z);
        double l = sqrt((ksi[i + 1] - ksi[i]) * (ksi[i + 1] - ksi[i]) + (eta[i + 1] - eta[i]) * (eta[i + 1] - eta[i]));
        double b1, a1, b2, a2, lgrn;
        if (fabs(l) < 1.0e-8) continue;
        b1 = deta * ((ksi[i] - x) * (ksi[i] - x) + z * z) - dksi * (ksi[i] - x) * (eta[i] - y);
        a1 = r1 * z * dksi;
        b2 = deta * ((ksi[i + 1] - x) * (ksi[i + 1] - x) + z * z) - dksi * (ksi[i + 1] - x) * (eta[i + 1] - y);
        a2 = r2 * z * dksi;
        if (!(fabs(z) < 1.0e-6)) szt = szt + atan2((b1 * a2 - b2 * a1), (a1 * a2 + b1 * b2));
        if (fabs(r1 + r2 - l) < 1.0e-6) continue;
        lgrn = log((r1 + r2 + l) / (r1 + r2 - l));
        sxt = sxt - deta / l * lgrn;
        syt = syt + dksi / l * lgrn;
        st = st - (deta * (x - ksi[i]) - dksi * (y - eta[i])) / l * lgrn;
    }
    st = st + z * szt;
    *sij = *sij + st;
    for (k = 0; k < 3; ++k) dij[k] = dij[k] + ui[k] * sxt + uj[k] * syt + uk[k] * szt;
    for (k = 0; k < 3; ++k) dij[k] = -dij[k];
}

void or_sglintbd(const double xq[4][3], int ncn, const double xf[3], double *sij, double dij[3])
{
    if (ncn == 3) sglint_tri(xq, xf, sij, dij);
    else sglint_quad(xq, xf, sij, dij);
}

/* ---------------------------------------------------------------------
 * DISPERSION  WavDynSubs.f90:40-126
 * ------------------------------------------------------------------- */
void or_dispersion(double *wvn, int nrt, double w, double h)
{
    const double g = 9.807, pi = 3.141592653589793;
    double x = w * w * h / g, y, t, u, trial, dnm, fun, dfun, d2fun, exx;
    int i;
    if (x > 0.0 && x <= 2.0) {
        y = sqrt(x) * (0.9994 + 0.1701 * x + SP(0.0305) * x * x);
    } else {
        t = x * exp(-2.0 * x);
        y = x + 2.0 * t - 6.0 * t * t;
    }
    if (fabs(y - x) < SP(1.e-10)) {
        wvn[0] = x / h;
    } else {
        exx = 1.0;
        while (exx > 1.0e-10) {
            trial = y;
            dnm = trial * trial - x * x;
            fun = log((trial + x) / (trial - x)) / 2.0 - trial;
            dfun = -x / dnm - 1.0;
            d2fun = 2.0 * x * trial / (dnm * dnm);
            y = trial - fun / dfun * (1.0 + (fun / dfun) * (d2fun / dfun) / 2.0);
            exx = fabs(y - trial);
        }
        wvn[0] = y / h;
    }
    u = 3.0 * x / (7.0 + 3.0 * x);
    t = 0.0159 + 0.1032 * u + 4.3152 * u * u - 2.8768 * u * u * u;
    for (i = 2; i <= nrt; ++i) {
        exx = 1.0;
        while (exx > 1.0e-10) {
            trial = t;
            y = (i - 1) * pi - trial;
            dnm = y * y + x * x;
            fun = atan2(x, y) - trial;
            dfun = x / dnm - 1.0;
            d2fun = 2.0 * x * trial / (dnm * dnm);
            t = trial - fun / dfun * (1.0 + (fun / dfun) * (d2fun / dfun) / 2.0);
            exx = fabs(t - trial);
        }
        y = (i - 1) * pi - t;
        wvn[i - 1] = y / h;
        t = t - pi * x / (x * x + pi * i * (pi * (i - 1) - t));
    }
}

/* ---------------------------------------------------------------------
 * VINP / DINP  PatclVelct.f90:42-123, with XW=(0,0) and AMP=1 (set once in
 * Initialisation, HydroStatic.f90:50-51).
 * ------------------------------------------------------------------- */
static void wave_scales(double v, double wk, double w1, double *w0, double *wk0)
{
    if (fabs(v) < SP(1.e-8)) { *w0 = SP(1.e-20); *wk0 = SP(1.e-20); }
    else if (fabs(v + 1.0) < SP(1.e-8)) { *w0 = SP(1.e+20); *wk0 = SP(1.e+20); }
    else { *w0 = w1; *wk0 = wk; }
}

zdouble or_vinp(double x, double y, double z, double beta, double v, double wk, double w1, double h)
{
    const double g = 9.80665, amp = 1.0;
    double w0, wk0, wkx, dum;
    zdouble r;
    wave_scales(v, wk, w1, &w0, &wk0);
    wkx = wk0 * ((x - 0.0) * cos(beta) + (y - 0.0) * sin(beta));
    if (h < 0.0 || h > 500.0) {
        r = -I * amp * g / w0 * exp(wk0 * z) * cexp(I * wkx);
    } else {
        dum = -amp * w0 / (wk0 * sinh(wk0 * h));
        r = I * dum * cosh(wk0 * (z + h)) * cexp(I * wkx);
    }
    return r / I;
}

void or_dinp(double x, double y, double z, double beta, double v, double wk, double w1,
             double h, zdouble *dpox, zdouble *dpoy, zdouble *dpoz)
{
    const double amp = 1.0;
    double w0, wk0, wkx;
    wave_scales(v, wk, w1, &w0, &wk0);
    wkx = wk0 * ((x - 0.0) * cos(beta) + (y - 0.0) * sin(beta));
    if (h < 0.0) {
        *dpox = w0 * amp * exp(wk0 * z) * cexp(I * wkx) * cos(beta);
        *dpoy = w0 * amp * exp(wk0 * z) * cexp(I * wkx) * sin(beta);
        *dpoz = -I * w0 * amp * exp(wk0 * z) * cexp(I * wkx);
    } else {
        double thkdh = cosh(wk0 * (z + h)) / sinh(wk0 * h);
        double thkdv = sinh(wk0 * (z + h)) / sinh(wk0 * h);
        *dpox = w0 * amp * thkdh * cexp(I * wkx) * cos(beta);
        *dpoy = w0 * amp * thkdh * cexp(I * wkx) * sin(beta);
        *dpoz = -I * w0 * amp * thkdv * cexp(I * wkx);
    }
    *dpox = *dpox / I;
    *dpoy = *dpoy / I;
    *dpoz = *dpoz / I;
}
