/*
 * Oracle (test infrastructure only): free-surface Green functions.
 *   - deep water: INFGREEN3D and the Wu-Noblesse global approximation,
 *     HAMS-MREL src/InfGreen_Appr.f90:104-872;
 *   - finite depth: FINGREEN3D and its four region methods,
 *     HAMS-MREL src/FinGreen3D.f90:81-2745.
 * Scratch values the Fortran keeps in module variables (GF_dd, GF_alpha...,
 * InfGreen_Appr.f90:89-96) are locals here, which gives the NTHREAD=1
 * semantics of the reference.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "hams_oracle.h"

static const double PI = 3.141592653589793;

/* ======================================================================
 * Deep water  (InfGreen_Appr.f90)
 * ==================================================================== */
typedef struct { double dd, alpha, beta, sigma, rho; } gf_par;

static double gf_func_a(double t)   /* GF_FuncA :298-326 */
{
    double g = (21859.0 + -4838.6 * t) * t;
    g = (-41592.9 + g) * t; g = (42002.57 + g) * t; g = (-24314.21 + g) * t;
    g = (8418.94 + g) * t;  g = (-1763.96 + g) * t; g = (215.896 + g) * t;
    g = (-13.328 + g) * t;  return 1.21 + g;
}
static double gf_func_b(double t)   /* GF_FuncB :329-357 */
{
    double g = (-29030.24 + 7671.22 * t) * t;
    g = (44894.06 + g) * t; g = (-36618.81 + g) * t; g = (17137.74 + g) * t;
    g = (-4780.77 + g) * t; g = (796.534 + g) * t;   g = (-67.92 + g) * t;
    g = (5.373 + g) * t;    return 0.938 + g;
}
static double gf_func_c(double t)   /* GF_FuncC :360-384 */
{
    double g = (9136.4 + -3272.62 * t) * t;
    g = (-9844.35 + g) * t; g = (5155.67 + g) * t; g = (-1397.89 + g) * t;
    g = (209.653 + g) * t;  g = (-9.747 + g) * t;  return 1.268 + g;
}
static double gf_func_d(double t)   /* GF_FuncD :387-416 */
{
    double g = (128170.2 + -33744.6 * t) * t;
    g = (-205690.43 + g) * t; g = (181856.75 + g) * t; g = (-96293.05 + g) * t;
    g = (31127.39 + g) * t;   g = (-6072.07 + g) * t;  g = (667.16 + g) * t;
    g = (-40.97 + g) * t;     return 0.632 + g;
}
static double gf_dfunc_a(double t)  /* GF_dFuncA :494-522 */
{
    double g = (-46688.0 + 12622.25 * t) * t;
    g = (68220.87 + g) * t; g = (-48811.41 + g) * t; g = (16370.75 + g) * t;
    g = (-1187.71 + g) * t; g = (-754.85 + g) * t;   g = (249.69 + g) * t;
    g = (-24.53 + g) * t;   return 2.948 + g;
}
static double gf_dfunc_b(double t)  /* GF_dFuncB :525-553 */
{
    double g = (-76209.82 + 19923.28 * t) * t;
    g = (118879.26 + g) * t; g = (-97014.11 + g) * t; g = (44270.15 + g) * t;
    g = (-11336.19 + g) * t; g = (1565.35 + g) * t;   g = (-76.765 + g) * t;
    g = (2.894 + g) * t;     return 1.11 + g;
}
static double gf_dfunc_c(double t)  /* GF_dFuncC :556-580 */
{
    double g = (3168.35 + -1590.27 * t) * t;
    g = (-2318.58 + g) * t; g = (847.8 + g) * t; g = (-148.24 + g) * t;
    return 14.19 + g;
}

static double bessel_j0(double xx)  /* BesselJ0 :583-624 */
{
    double yy, y2, f0, th;
    if (xx <= 3.0) {
        yy = (xx / 3.0) * (xx / 3.0);
        return 0.999999999 + (-2.249999879 + (1.265623060 + (-0.316394552 + (0.044460948
               + (-0.003954479 + 0.000212950 * yy) * yy) * yy) * yy) * yy) * yy;
    }
    yy = 3.0 / xx;
    y2 = yy * yy;
    f0 = 0.79788454 + (-0.00553897 + (0.00099336 + (-0.00044346 + (0.00020445 - 0.00004959 * y2)
         * y2) * y2) * y2) * y2;
    th = xx - 0.25 * PI + (-0.04166592 + (0.00239399 + (-0.00073984 + (0.00031099 - 0.00007605 * y2)
         * y2) * y2) * y2) * yy;
    return f0 * cos(th) / sqrt(xx);
}
static double bessel_j1(double xx)  /* BesselJ1 :627-671 */
{
    double yy, y2, f1, th, b;
    if (xx <= 3.0) {
        yy = xx / 3.0;
        y2 = yy * yy;
        b = 0.5 + (-0.562499992 + (0.210937377 + (-0.039550040 + (0.004447331 + (-0.000330547
            + 0.000015525 * y2) * y2) * y2) * y2) * y2) * y2;
        return b * xx;
    }
    yy = 3.0 / xx;
    y2 = yy * yy;
    f1 = 0.79788459 + (0.01662008 + (-0.00187002 + (0.00068519 + (-0.00029440 + 0.00006952 * y2)
         * y2) * y2) * y2) * y2;
    th = xx - 0.75 * PI + (0.12499895 + (-0.00605240 + (0.00135825 + (-0.00049616 + 0.00011531 * y2)
         * y2) * y2) * y2) * yy;
    return f1 * cos(th) / sqrt(xx);
}
/* BesselY0/Y1 :674-760, only reached for xx > 3 through StruveH0/H1. */
static double bessel_y0_large(double xx)
{
    double t = 3.0 / xx;
    double f0 = 0.79788454 - 0.00553897 * (t * t) + 0.00099336 * __builtin_powi(t, 4)
              - 0.00044346 * __builtin_powi(t, 6) + 0.00020445 * __builtin_powi(t, 8)
              - 0.00004959 * __builtin_powi(t, 10);
    double th = xx - 0.25 * PI - 0.04166592 * t + 0.00239399 * __builtin_powi(t, 3)
              - 0.00073984 * __builtin_powi(t, 5) + 0.00031099 * __builtin_powi(t, 7)
              - 0.00007605 * __builtin_powi(t, 9);
    return f0 * sin(th) / sqrt(xx);
}
static double bessel_y1_large(double xx)
{
    double t = 3.0 / xx;
    double f1 = 0.79788459 + 0.01662008 * (t * t) - 0.00187002 * __builtin_powi(t, 4)
              + 0.00068519 * __builtin_powi(t, 6) - 0.00029440 * __builtin_powi(t, 8)
              + 0.00006952 * __builtin_powi(t, 10);
    double th = xx - 3.0 * PI / 4.0 + 0.12499895 * t - 0.00605240 * __builtin_powi(t, 3)
              + 0.00135825 * __builtin_powi(t, 5) - 0.00049616 * __builtin_powi(t, 7)
              + 0.00011531 * __builtin_powi(t, 9);
    return f1 * sin(th) / sqrt(xx);
}
static double struve_h0(double xx)  /* StruveH0 :764-815 */
{
    double yy, c1, c2, h;
    if (xx <= 3.0) {
        yy = (xx / 3.0) * (xx / 3.0);
        h = 1.909859164 + (-1.909855001 + (0.687514637 + (-0.126164557 + (0.013828813
            - 0.000876918 * yy) * yy) * yy) * yy) * yy;
        return h * (xx / 3.0);
    }
    yy = (3.0 / xx) * (3.0 / xx);
    c1 = 2.0 * (0.99999906 + (4.77228920 + (3.85542044 + 0.32303607 * yy) * yy) * yy);
    c2 = PI * xx * (1.0 + (4.88331068 + (4.28957333 + 0.52120508 * yy) * yy) * yy);
    return c1 / c2 + bessel_y0_large(xx);
}
static double struve_h1(double xx)  /* StruveH1 :818-870 */
{
    double yy, c1, c2;
    if (xx <= 3.0) {
        yy = (xx / 3.0) * (xx / 3.0);
        return (1.909859286 + (-1.145914713 + (0.294656958 + (-0.042070508 + (0.003785727
               - 0.000207183 * yy) * yy) * yy) * yy) * yy) * yy;
    }
    yy = (3.0 / xx) * (3.0 / xx);
    c1 = 2.0 * (1.00000004 + (3.92205313 + (2.64893033 + 0.27450895 * yy) * yy) * yy);
    c2 = PI * (1.0 + (3.81095112 + (2.26216956 + 0.10885141 * yy) * yy) * yy);
    return c1 / c2 + bessel_y1_large(xx);
}

/* HavelockGF :189-205 with GF_DivParameters :209-224 and the L0/Lp/W and
 * Ls/Lsp/Wh pieces :227-491. */
static void havelock_gf(double hh, double vv, zdouble *gf, zdouble *gfh)
{
    const double gama = 0.5772156649;
    gf_par p;
    double pp, lp, rr, l0, ps, qs, lsp, ls, a, b, c, d;
    p.dd = sqrt(hh * hh + vv * vv);
    p.alpha = -vv / p.dd;
    p.beta = hh / p.dd;
    p.sigma = hh / (p.dd - vv);
    p.rho = p.dd / (1.0 + p.dd);

    /* GF_Func_L0 / GF_Func_Lp */
    pp = log(0.5 * (p.dd - vv)) + gama - 2.0 * p.dd * p.dd;
    pp = exp(vv) * pp;
    pp = pp + p.dd * p.dd - vv;
    a = gf_func_a(p.rho); b = gf_func_b(p.rho); c = gf_func_c(p.rho); d = gf_func_d(p.rho);
    rr = (1.0 - p.beta) * a;
    rr = rr - p.beta * b;
    rr = rr - p.alpha * c / (1.0 + 6.0 * p.alpha * p.rho * (1.0 - p.rho));
    rr = rr + p.beta * (1.0 - p.beta) * d;
    lp = p.rho * ((1.0 - p.rho) * (1.0 - p.rho) * (1.0 - p.rho)) * rr;
    l0 = 2.0 * pp / (1.0 + p.dd * p.dd * p.dd) + 2.0 * lp;
    /* GF_Func_W: 2*pi*(H0 - i J0)*exp(vv) */
    {
        double h0 = struve_h0(hh), j0 = bessel_j0(hh), e = exp(vv);
        *gf = l0 + (2.0 * PI * h0 * e) + I * (2.0 * PI * (-j0) * e);
    }
    /* GF_Func_Ls / GF_Func_Lsp */
    ps = (p.beta + hh) / (p.dd - vv);
    ps = ps - 2.0 * p.beta + 2.0 * exp(vv) * p.dd - hh;
    qs = exp(-p.dd) * (1.0 - p.beta);
    qs = qs * (1.0 + p.dd / (1.0 + p.dd * p.dd * p.dd));
    a = gf_dfunc_a(p.rho); b = gf_dfunc_b(p.rho); c = gf_dfunc_c(p.rho);
    rr = p.beta * a;
    rr = rr - (1.0 - p.alpha) * b;
    rr = rr + p.beta * (1.0 - p.beta) * p.rho * (1.0 - 2.0 * p.rho) * c;
    lsp = p.rho * ((1.0 - p.rho) * (1.0 - p.rho) * (1.0 - p.rho)) * rr;
    ls = 2.0 * ps / (1.0 + p.dd * p.dd * p.dd) - 4.0 * qs + 2.0 * lsp;
    /* GF_Func_Wh: 2*pi*(2/pi - H1 + i J1)*exp(vv) */
    {
        double h1 = struve_h1(hh), j1 = bessel_j1(hh), e = exp(vv);
        *gfh = ls + (2.0 * PI * (2.0 / PI - h1) * e) + I * (2.0 * PI * j1 * e);
    }
}

void or_infgreen3d(double xf, double xp, double yf, double yp, double zf, double zp,
                   double v, zdouble grn[4], int flag)
{
    double xpq = xf - xp, ypq = yf - yp, zpq = zp + zf;
    double rr = sqrt(xpq * xpq + ypq * ypq);
    double r = sqrt(rr * rr + (zp - zf) * (zp - zf));
    double r1 = sqrt(rr * rr + zpq * zpq);
    double r13 = r1 * r1 * r1, r3 = r * r * r;
    zdouble gf, gfh;
    grn[0] = grn[1] = grn[2] = grn[3] = 0.0;

    if (fabs(v) < SP(1.e-8)) {
        if (flag == 1) {
            grn[0] += 1.0 / r1; grn[1] -= xpq / r13; grn[2] -= ypq / r13; grn[3] -= zpq / r13;
        } else {
            grn[0] = grn[0] + 1.0 / r1 + 1.0 / r;
            grn[1] = grn[1] - xpq / r13 - xpq / r3;
            grn[2] = grn[2] - ypq / r13 - ypq / r3;
            grn[3] = grn[3] - zpq / r13 - (zf - zp) / r3;
        }
        return;
    }
    if (fabs(v + 1.0) < SP(1.e-8)) {
        if (flag == 1) {
            grn[0] -= 1.0 / r1; grn[1] += xpq / r13; grn[2] += ypq / r13; grn[3] += zpq / r13;
        } else {
            grn[0] = grn[0] - 1.0 / r1 + 1.0 / r;
            grn[1] = grn[1] + xpq / r13 - xpq / r3;
            grn[2] = grn[2] + ypq / r13 - ypq / r3;
            grn[3] = grn[3] + zpq / r13 - (zf - zp) / r3;
        }
        return;
    }
    havelock_gf(v * rr, v * zpq, &gf, &gfh);
    if (rr > SP(1.e-6)) {
        grn[1] = -(v * v) * gfh * xpq / rr;
        grn[2] = -(v * v) * gfh * ypq / rr;
    } else {
        grn[1] = 0.0;
        grn[2] = 0.0;
    }
    grn[0] = -v * gf;
    grn[3] = -(v * v) * gf + 2.0 * v / r1;
    if (flag == 1) {
        grn[0] = grn[0] + 1.0 / r1;
        grn[1] = grn[1] - xpq / r13;
        grn[2] = grn[2] - ypq / r13;
        grn[3] = grn[3] - zpq / r13;
    } else {
        grn[0] = grn[0] + 1.0 / r1 + 1.0 / r;
        grn[1] = grn[1] - xpq / r13 - xpq / r3;
        grn[2] = grn[2] - ypq / r13 - ypq / r3;
        grn[3] = grn[3] - zpq / r13 - (zf - zp) / r3;
    }
}

/* ======================================================================
 * Finite depth  (FinGreen3D.f90)
 * ==================================================================== */

/* Rankine image sums of Pidcock's method: IMGS / DGSR / DGSZ :908-1102.
 * AMN(M,N) is filled column-major by the DATA statement (M fastest). */
static const double AMN[5][5] = {  /* AMN[n][m] == AMN(M=m, N=n) */
    {0.0, -0.02525711, 0.00086546, -0.00004063, 0.00000193},
    {0.05051418, -0.00692380, 0.00073292, -0.00006636, 0.00000398},
    {0.00230838, -0.00097875, 0.00020597, -0.00003333, 0.00000524},
    {0.00012934, -0.00010879, 0.00003965, -0.00000891, 0.0},
    {0.00000913, -0.00001270, 0.00000466, 0.0, 0.0}};
#define AMN_MN(m, n) (AMN[(n)][(m)])

static double rs(double r, double z) { return sqrt(r * r + z * z); }

static double imgs(double r, double zf, double zp, double h)
{
    double t1 = r / h, t2 = (zf - zp) / h, t3 = (zf + zp + 2.0 * h) / h, s1 = 0.0, s2 = 0.0;
    int l, m, n;
    for (l = -1; l <= 1; ++l) s1 = s1 + 1.0 / rs(t1, t2 + 2.0 * l) + 1.0 / rs(t1, t3 + 2.0 * l);
    for (m = 0; m <= 4; ++m)
        for (n = 0; n <= 4; ++n)
            s2 = s2 + AMN_MN(m, n) * pow(t1, 2.0 * m) * (pow(t2, 2.0 * n) + pow(t3, 2.0 * n));
    return (s1 - 2.0 + s2) / h;
}
static double dgsr(double r, double zf, double zp, double h)
{
    double t1 = r / h, t2 = (zf - zp) / h, t3 = (zf + zp + 2.0 * h) / h, s1 = 0.0, s2 = 0.0, a, b;
    int l, m, n;
    for (l = -1; l <= 1; ++l) {
        a = rs(t1, t2 + 2.0 * l); b = rs(t1, t3 + 2.0 * l);
        s1 = s1 + t1 / (a * a * a) + t1 / (b * b * b);
    }
    for (m = 1; m <= 4; ++m)
        for (n = 0; n <= 4; ++n)
            s2 = s2 + 2.0 * m * AMN_MN(m, n) * pow(t1, 2.0 * m - 1.0) * (pow(t2, 2.0 * n) + pow(t3, 2.0 * n));
    return (-s1 + s2) / (h * h);
}
static double dgsz(double r, double zf, double zp, double h)
{
    double t1 = r / h, t2 = (zf - zp) / h, t3 = (zf + zp + 2.0 * h) / h, s1 = 0.0, s2 = 0.0, a, b;
    int l, m, n;
    for (l = -1; l <= 1; ++l) {
        a = rs(t1, t2 + 2.0 * l); b = rs(t1, t3 + 2.0 * l);
        s1 = s1 + (t2 + 2.0 * l) / (a * a * a) + (t3 + 2.0 * l) / (b * b * b);
    }
    for (m = 0; m <= 4; ++m)
        for (n = 1; n <= 4; ++n)
            s2 = s2 + 2.0 * n * AMN_MN(m, n) * pow(t1, 2.0 * m) * (pow(t2, 2.0 * n - 1.0) + pow(t3, 2.0 * n - 1.0));
    return (-s1 + s2) / (h * h);
}

/* Subtraction of the two Rankine terms shared by EIGEN/EIGENE/PIDCOCK. */
static void sub_rankine(double r, double zf, double zp, zdouble g[3])
{
    double sr = sqrt(r * r + (zf - zp) * (zf - zp));
    double sr1 = sqrt(r * r + (zf + zp) * (zf + zp));
    double dsrr = r / sr, dsrz = (zf - zp) / sr, dsr1r = r / sr1, dsr1z = (zf + zp) / sr1;
    g[0] = g[0] - (1.0 / sr + 1.0 / sr1);
    g[1] = g[1] + (dsrr / (sr * sr) + dsr1r / (sr1 * sr1));
    g[2] = g[2] + (dsrz / (sr * sr) + dsr1z / (sr1 * sr1));
}

/* EIGEN  :281-362 (R/h >= 0.5) */
static void eigen(double r, double zf, double zp, double wk, const double *wvn, double h, zdouble g[3])
{
    const int nt = 10;
    double zfh = zf + h, zph = zp + h, j0, j1, y0, y1, k0, k1;
    double nm0 = h / 2.0 * (1.0 + sinh(2.0 * wk * h) / (2.0 * wk * h));
    double p0 = PI / nm0 * cosh(wk * zfh) * cosh(wk * zph);
    double dp0 = PI / nm0 * sinh(wk * zfh) * cosh(wk * zph);
    int i;
    or_jy01b(wk * r, &j0, &j1, &y0, &y1);
    g[0] = p0 * (-y0) + I * (p0 * j0);
    g[1] = -(wk * p0) * (-y1) + I * (-(wk * p0) * j1);
    g[2] = (wk * dp0) * (-y0) + I * ((wk * dp0) * j0);
    for (i = 2; i <= nt; ++i) {
        double km = wvn[i - 1], twokmh = 2.0 * km * h;
        double pm = 4.0 / (1.0 + sin(twokmh) / twokmh) / h;
        double kzf, kzp, ckzf, ckzp, skzf, rm1, rm2, rm3;
        or_ik01a(km * r, &k0, &k1);
        kzf = km * zfh; kzp = km * zph;
        ckzf = cos(kzf); ckzp = cos(kzp); skzf = sin(kzf);
        rm1 = pm * k0 * ckzf * ckzp;
        rm2 = -(pm * km * k1 * ckzf * ckzp);
        rm3 = -(pm * km * k0 * skzf * ckzp);
        g[0] += rm1; g[1] += rm2; g[2] += rm3;
        if (fabs(rm1) < SP(1.e-6) && fabs(rm2) < SP(1.e-6) && fabs(rm3) < SP(1.e-6)) break;
    }
    sub_rankine(r, zf, zp, g);
}

/* EIGENE  :413-506 (0.05 <= R/h < 0.5), epsilon-algorithm acceleration */
static void eigene(double r, double zf, double zp, double wk, const double *wvn, int nk,
                   double h, zdouble g[3])
{
    double rhp = fabs(r / h);
    int nt = (int)(SP(-88.89) * rhp + SP(54.45));
    double zfh = zf + h, zph = zp + h, j0, j1, y0, y1, k0, k1, rl[3];
    double nm0 = h / 2.0 * (1.0 + sinh(2.0 * wk * h) / (2.0 * wk * h));
    double p0 = PI / nm0 * cosh(wk * zfh) * cosh(wk * zph);
    double dp0 = PI / nm0 * sinh(wk * zfh) * cosh(wk * zph);
    double *gs = (double *)calloc((size_t)3 * nk, sizeof(double));
    double *gr = gs + nk, *gz = gs + 2 * nk;
    int i;
    or_jy01b(wk * r, &j0, &j1, &y0, &y1);
    g[0] = p0 * (-y0) + I * (p0 * j0);
    g[1] = -(wk * p0) * (-y1) + I * (-(wk * p0) * j1);
    g[2] = (wk * dp0) * (-y0) + I * ((wk * dp0) * j0);
    for (i = 2; i <= nt; ++i) {
        double km = wvn[i - 1], twokmh = 2.0 * km * h;
        double pm = 4.0 / (1.0 + sin(twokmh) / twokmh) / h;
        double kzf, kzp, ckzf, ckzp, skzf;
        or_ik01a(km * r, &k0, &k1);
        kzf = km * zfh; kzp = km * zph;
        ckzf = cos(kzf); ckzp = cos(kzp); skzf = sin(kzf);
        gs[i - 1] = gs[i - 2] + pm * k0 * ckzf * ckzp;
        gr[i - 1] = gr[i - 2] + -(pm * km * k1 * ckzf * ckzp);
        gz[i - 1] = gz[i - 2] + -(pm * km * k0 * skzf * ckzp);
    }
    or_limes(nt - 1, gs, &rl[0]);
    or_limes(nt - 1, gr, &rl[1]);
    or_limes(nt - 1, gz, &rl[2]);
    free(gs);
    g[0] += rl[0]; g[1] += rl[1]; g[2] += rl[2];
    sub_rankine(r, zf, zp, g);
}

/* PIDCOCK  :558-660 (0.0005 <= R/h < 0.05) */
static void pidcock(double r, double zf, double zp, double v, double wk, const double *wvn, int nk,
                    double h, zdouble g[3])
{
    const double ga = 0.5772156649015328;
    double j0, j1, y0, y1, k0, k0t, k1, k1t, rl[3];
    double nm0 = h / 2.0 * (1.0 + sinh(2.0 * wk * h) / (2.0 * wk * h));
    double p0 = PI / nm0 * cosh(wk * (zf + h)) * cosh(wk * (zp + h));
    double dp0 = wk * PI / nm0 * sinh(wk * (zf + h)) * cosh(wk * (zp + h));
    double rhp = fabs(r / h);
    int nt = (int)(SP(-1010.10) * rhp + SP(100.50));
    double *gs = (double *)calloc((size_t)3 * nk, sizeof(double));
    double *gr = gs + nk, *gz = gs + 2 * nk;
    int i;
    or_jy01b(wk * r, &j0, &j1, &y0, &y1);
    g[0] = p0 * (-y0) + 2.0 / h * (ga + log(r / 4.0 / h)) + I * (p0 * j0);
    g[1] = -(wk * p0) * (-y1) + 2.0 / (r * h) + I * (-(wk * p0) * j1);
    g[2] = dp0 * (-y0) + I * (dp0 * j0);
    for (i = 2; i <= nt; ++i) {
        double mp = (i - 1) * PI, umt = mp / h, um = wvn[i - 1], x = um * r;
        double ac, am, amt, dam, damt;
        or_ik01a(x, &k0, &k1);
        or_ik01a(umt * r, &k0t, &k1t);
        ac = (um * um + v * v) / ((um * um + v * v) * h - v);
        am = ac * cos(um * (zf + h)) * cos(um * (zp + h));
        amt = cos(umt * (zf + h)) * cos(umt * (zp + h)) / h;
        dam = -(um * ac * sin(um * (zf + h)) * cos(um * (zp + h)));
        damt = -(umt * sin(umt * (zf + h)) * cos(umt * (zp + h)) / h);
        gs[i - 1] = gs[i - 2] + (am * k0 - amt * k0t);
        gr[i - 1] = gr[i - 2] + (-(um * am * k1) + umt * amt * k1t);
        gz[i - 1] = gz[i - 2] + (dam * k0 - damt * k0t);
    }
    or_limes(nt - 1, gs, &rl[0]);
    or_limes(nt - 1, gr, &rl[1]);
    or_limes(nt - 1, gz, &rl[2]);
    free(gs);
    g[0] = g[0] + 4.0 * rl[0] + imgs(r, zf, zp, h);
    g[1] = g[1] + 4.0 * rl[1] + dgsr(r, zf, zp, h);
    g[2] = g[2] + 4.0 * rl[2] + dgsz(r, zf, zp, h);
    sub_rankine(r, zf, zp, g);
}

/* ---- Linton's method helpers (:1168-2745) ---- */
static double erfcc(double x) { double e; or_error(x, &e); return 1.0 - e; }
static double derfcc(double x) { return -2.0 / sqrt(PI) * exp(-pow(x, 2.0)); }

static void chi(double zf, double zp, double h, double val[4])
{
    val[0] = -zp - zf;
    val[1] = 2.0 * h - zp + zf;
    val[2] = 2.0 * h + zp - zf;
    val[3] = 4.0 * h + zp + zf;
}
static const double DVAL[4] = {-1.0, 1.0, -1.0, 1.0};

static void rchi(double r, double zf, double zp, double h, double ro[4], double dror[4], double droz[4])
{
    double val[4];
    int i;
    chi(zf, zp, h, val);
    for (i = 0; i < 4; ++i) {
        ro[i] = sqrt(r * r + val[i] * val[i]);
        dror[i] = r / sqrt(r * r + val[i] * val[i]);
        droz[i] = val[i] * __builtin_powi(-1.0, i + 1) / sqrt(r * r + val[i] * val[i]);
    }
}

static zdouble nm_fn(double h, zdouble wvn)  /* NM :2262-2273 */
{
    return h / 2.0 * (1.0 + csin(2.0 * wvn * h) / (2.0 * wvn * h));
}

static double f1_fn(double r, double wvn, int no, double t)  /* F1 :1795 */
{
    if (fabs(t) < 1.0e-8) return 0.0;
    if (no == 1) return exp(-r * r / 4.0 / t + wvn * wvn * t) / 4.0 / PI / t;
    return exp(-r * r / 4.0 / t - wvn * wvn * t) / 4.0 / PI / t;
}
static double f2_fn(double r, double wvn, int no, double t)  /* F2 :1850 */
{
    if (fabs(t) < 1.0e-8) return 0.0;
    if (no == 1) return -r * exp(-r * r / 4.0 / t + wvn * wvn * t) / 8.0 / PI / (t * t);
    return -r * exp(-r * r / 4.0 / t - wvn * wvn * t) / 8.0 / PI / (t * t);
}
static double fun_fn(double r, double wvn, int no, double t, int tag)
{
    return tag == 1 ? f1_fn(r, wvn, no, t) : f2_fn(r, wvn, no, t);
}

typedef struct { double v, r, zf, zp, h; } gpar;
static double g_fn(const gpar *p, double t, int tag)  /* G1/G2/G3 :1904-2057 */
{
    double val[4], sum = 0.0;
    int i;
    if (fabs(t) < 1.0e-8) return 0.0;
    chi(p->zf, p->zp, p->h, val);
    if (tag == 1 || tag == 2) {
        for (i = 0; i < 4; ++i) sum = sum + exp(-p->v * val[i]) * erfcc(val[i] / 2.0 / t - p->v * t);
        if (tag == 1) return exp(p->v * p->v * (t * t) - p->r * p->r / 4.0 / (t * t)) * sum / t;
        return p->r / 2.0 / (t * t * t) * exp(p->v * p->v * (t * t) - p->r * p->r / 4.0 / (t * t)) * sum;
    }
    for (i = 0; i < 4; ++i)
        sum = sum - p->v * DVAL[i] * exp(-p->v * val[i]) * erfcc(val[i] / 2.0 / t - p->v * t)
                  + exp(-p->v * val[i]) * derfcc(val[i] / 2.0 / t - p->v * t) * DVAL[i] / 2.0 / t;
    return exp(p->v * p->v * (t * t) - p->r * p->r / 4.0 / (t * t)) * sum / t;
}

static const double XGQ[7] = {-0.949107912342759, -0.741531185599394, -0.405845151377397, 0.0,
                               0.405845151377397, 0.741531185599394, 0.949107912342759};
static const double WGQ[7] = {0.129484966168870, 0.279705391489277, 0.381830050505119,
                               0.417959183673469, 0.381830050505119, 0.279705391489277,
                               0.129484966168870};
static const double XKQ[15] = {-0.991455371120813, -0.949107912342759, -0.864864423359769,
    -0.741531185599394, -0.586087235467691, -0.405845151377397, -0.207784955007898, 0.0,
    0.207784955007898, 0.405845151377397, 0.586087235467691, 0.741531185599394,
    0.864864423359769, 0.949107912342759, 0.991455371120813};
static const double WKQ[15] = {0.022935322010529, 0.063092092629979, 0.104790010322250,
    0.140653259715525, 0.169004726639267, 0.190350578064785, 0.204432940075298,
    0.209482141084728, 0.204432940075298, 0.190350578064785, 0.169004726639267,
    0.140653259715525, 0.104790010322250, 0.063092092629979, 0.022935322010529};

/* GK_INTEGF + AQUADF :2387-2532 (recursive adaptive Gauss-Kronrod 7-15) */
static double aquadf(const gpar *p, double a, double b, double eps, int tag)
{
    double stf[7], gi = 0.0, gk = 0.0, err;
    int i;
    for (i = 0; i < 7; ++i) {
        stf[i] = g_fn(p, 0.5 * (b + a + (b - a) * XGQ[i]), tag);
        gi = gi + WGQ[i] * (b - a) / 2.0 * stf[i];
    }
    for (i = 1; i <= 15; ++i) {
        if (i % 2 == 0) gk = gk + WKQ[i - 1] * (b - a) / 2.0 * stf[i / 2 - 1];
        else gk = gk + WKQ[i - 1] * (b - a) / 2.0 * g_fn(p, 0.5 * (b + a + (b - a) * XKQ[i - 1]), tag);
    }
    err = pow(200.0 * fabs(gk - gi), 1.5);
    if (err > eps && fabs(a - b) > eps)
        return 0.0 + aquadf(p, a, (a + b) / 2.0, eps, tag) + aquadf(p, (a + b) / 2.0, b, eps, tag);
    return 0.0 + gk;
}

/* GK_INTEG + AQUAD :2599-2745 */
static double aquad(double r, double wvn, int no, double a, double b, double eps, int tag)
{
    double stf[7], gi = 0.0, gk = 0.0, err;
    int i;
    for (i = 0; i < 7; ++i) {
        stf[i] = fun_fn(r, wvn, no, 0.5 * (b + a + (b - a) * XGQ[i]), tag);
        gi = gi + WGQ[i] * (b - a) / 2.0 * stf[i];
    }
    for (i = 1; i <= 15; ++i) {
        if (i % 2 == 0) gk = gk + WKQ[i - 1] * (b - a) / 2.0 * stf[i / 2 - 1];
        else gk = gk + WKQ[i - 1] * (b - a) / 2.0 * fun_fn(r, wvn, no, 0.5 * (b + a + (b - a) * XKQ[i - 1]), tag);
    }
    err = pow(200.0 * fabs(gk - gi), 1.5);
    if (err > eps && fabs(a - b) > eps)
        return 0.0 + aquad(r, wvn, no, a, (a + b) / 2.0, eps, tag) + aquad(r, wvn, no, (a + b) / 2.0, b, eps, tag);
    return 0.0 + gk;
}

/* SA0 :1389-1430 */
static double sa0(double r, double pa, double wk)
{
    const double ga = 0.5772156649015328, eps = SP(1.e-6);
    int n = 1, p;
    double rm = 100.0, s = -ga - 2.0 * log(wk * pa / 2.0), sgn = -1.0, facn = 1.0, psi, en;
    while (fabs(rm) > eps) {
        or_enxa(n + 1, (r / pa) * (r / pa), &en);
        psi = 0.0;
        for (p = 1; p <= n; ++p) psi = psi + 1.0 / p;
        rm = sgn * pow(r / pa, 2.0 * n) / facn / n - pow(wk * pa / 2.0, 2.0 * n) / facn * en
           - 2.0 * sgn / (facn * facn) * pow(wk * r / 2.0, 2.0 * n) * (log(wk * r / 2.0) + ga - psi);
        s = s + rm;
        n = n + 1;
        sgn = -sgn;
        facn = facn * n;
    }
    return s / 4.0 / PI;
}
/* DSA0 :1483-1524 */
static double dsa0(double r, double pa, double wk)
{
    const double ga = 0.5772156649015328, eps = SP(1.e-6);
    int n = 1, p;
    double rm = 100.0, s = 0.0, sgn = -1.0, facn = 1.0, psi, en;
    while (fabs(rm) > eps) {
        or_enxa(n, (r / pa) * (r / pa), &en);
        psi = 0.0;
        for (p = 1; p <= n; ++p) psi = psi + 1.0 / p;
        rm = 2.0 * sgn * pow(r / pa, 2.0 * n - 1.0) / facn / pa
           + pow(wk * pa / 2.0, 2.0 * n) / facn * en * 2.0 * r / (pa * pa)
           - 2.0 * sgn * n * wk / (facn * facn) * pow(wk * r / 2.0, 2.0 * n - 1.0) * (log(wk * r / 2.0) + ga - psi)
           - 2.0 * sgn / (facn * facn) * pow(wk * r / 2.0, 2.0 * n) / r;
        s = s + rm;
        n = n + 1;
        sgn = -sgn;
        facn = facn * n;
    }
    return s / 4.0 / PI;
}
/* SAM :1575-1610 */
static double sam(double r, double pa, double wvn)
{
    const double eps = SP(1.e-6);
    int n = 0;
    double rm = 100.0, s = 0.0, sgn = 1.0, facn = 1.0, en;
    while (fabs(rm) > eps) {
        or_enxa(n + 1, (wvn * pa / 2.0) * (wvn * pa / 2.0), &en);
        rm = sgn * pow(r / pa, 2.0 * n) / facn * en;
        s = s + rm;
        n = n + 1;
        sgn = -sgn;
        facn = facn * n;
    }
    return s / 4.0 / PI;
}
/* DSAM :1659-1693 */
static double dsam(double r, double pa, double wvn)
{
    const double eps = SP(1.e-6);
    int n = 1;
    double rm = 100.0, s = 0.0, sgn = -1.0, facn = 1.0, en;
    while (fabs(rm) > eps) {
        or_enxa(n + 1, (wvn * pa / 2.0) * (wvn * pa / 2.0), &en);
        rm = 2.0 * n * sgn * pow(r / pa, 2.0 * n - 1.0) / facn / pa * en;
        s = s + rm;
        n = n + 1;
        sgn = -sgn;
        facn = facn * n;
    }
    return s / 4.0 / PI;
}

/* COEF :1170-1230 and DCOEF :1280-1340 */
static void coef(double r, double pa, double a, int m, const double *wvno, double wk, double *cof)
{
    const double eps = SP(1.e-6), step = 100.0;
    double dnt = pa * pa / 4.0, by0, ei, e1, p1;
    int i;
    if (fabs(r) < SP(1.e-6)) {
        or_eix(wk * wk * dnt, &ei);
        cof[0] = -ei / 4.0 / PI;
    } else if (r / a <= 0.5) {
        cof[0] = sa0(r, pa, wk);
    } else {
        or_jy01by0(wk * r, &by0);
        cof[0] = -by0 / 4.0 - aquad(r, wk, 1, 0.0, dnt, eps, 1);
    }
    for (i = 2; i <= m; ++i) {
        if (fabs(r) < SP(1.e-6)) {
            or_e1xa(wvno[i - 1] * wvno[i - 1] * dnt, &e1);
            cof[i - 1] = e1 / 4.0 / PI;
        } else if (r / a <= 1.0) {
            cof[i - 1] = sam(r, pa, wvno[i - 1]);
        } else {
            p1 = dnt + step;
            while (fabs(f1_fn(r, wvno[i - 1], i, p1)) > eps) p1 = p1 + step;
            cof[i - 1] = aquad(r, wvno[i - 1], i, dnt, p1, eps, 1);
        }
    }
}
static void dcoef(double r, double pa, double a, int m, const double *wvno, double wk, double *dcof)
{
    const double eps = SP(1.e-6), step = 100.0;
    double dnt = pa * pa / 4.0, by1, p1;
    int i;
    if (fabs(r) < SP(1.e-6)) {
        dcof[0] = 0.0;
    } else if (r / a <= 0.5) {
        dcof[0] = dsa0(r, pa, wk);
    } else {
        or_jy01by1(wk * r, &by1);
        dcof[0] = wk * by1 / 4.0 - aquad(r, wk, 1, 0.0, dnt, eps, 2);
    }
    for (i = 2; i <= m; ++i) {
        if (fabs(r) < SP(1.e-6)) {
            dcof[i - 1] = 0.0;
        } else if (r / a <= 1.0) {
            dcof[i - 1] = dsam(r, pa, wvno[i - 1]);
        } else {
            p1 = dnt + step;
            while (fabs(f2_fn(r, wvno[i - 1], i, p1)) > eps) p1 = p1 + step;
            dcof[i - 1] = aquad(r, wvno[i - 1], i, dnt, p1, eps, 2);
        }
    }
}

/* LINTON  :712-861 (R/h < 0.0005) */
static void linton(double r, double zf, double zp, double v, double wk, const double *wvno, int nk,
                   double h, zdouble grn[3])
{
    const double eps = SP(1.e-6);
    double a, pa, sr, sr1, sr2, ro[4], dror[4], droz[4], errsum[3], bj0, bj1;
    double dsrr, dsrz, dsr1r, dsr1z, dsr2r, dsr2z;
    double *cof = (double *)calloc((size_t)2 * nk, sizeof(double)), *dcof = cof + nk;
    gpar gp;
    zdouble km, rm[3];
    int i, nt;

    if (v < 0.02) a = 3324.2 * (v * v * v) - 258.89 * (v * v) + 8.3958 * v + 1.3208;
    else if (v < 0.1) a = -30.303 * (v * v * v) - 2.8138 * (v * v) + 2.7740 * v + 0.05052;
    else if (v < 1.0) a = 1.5699 * (v * v * v) - 2.5075 * (v * v) + 1.8316 * v + 0.1077;
    else a = -0.000069641 * (v * v * v) - 0.0017082 * (v * v) + 0.45566 * v + 0.80551;
    a = fabs(a) / (wk * h);

    pa = a * h;
    sr = sqrt(r * r + (zf - zp) * (zf - zp));
    sr1 = sqrt(r * r + (2.0 * h + zf + zp) * (2.0 * h + zf + zp));
    sr2 = sqrt(r * r + (zf + zp) * (zf + zp));
    rchi(r, zf, zp, h, ro, dror, droz);
    dsrr = r / sr; dsrz = (zf - zp) / sr;
    dsr1r = r / sr1; dsr1z = (2.0 * h + zf + zp) / sr1;
    dsr2r = r / sr2; dsr2z = (zf + zp) / sr2;

    grn[0] = grn[1] = grn[2] = 0.0;
    nt = 20;
    coef(r, pa, a, nt, wvno, wk, cof);
    dcoef(r, pa, a, nt, wvno, wk, dcof);
    for (i = 1; i <= nt; ++i) {
        zdouble nmv, c1, c2, s1;
        km = (i == 1) ? -I * wk : (zdouble)wvno[i - 1];
        nmv = nm_fn(h, km);
        c1 = ccos(km * (zf + h));
        c2 = ccos(km * (zp + h));
        s1 = csin(km * (zf + h));
        rm[0] = -(cof[i - 1] / nmv * c1 * c2);
        rm[1] = -(dcof[i - 1] / nmv * c1 * c2);
        rm[2] = cof[i - 1] * km / nmv * s1 * c2;
        grn[0] += rm[0]; grn[1] += rm[1]; grn[2] += rm[2];
        if (i > 2 && cabs(rm[0]) < eps && cabs(rm[1]) < eps && cabs(rm[2]) < eps) break;
    }

    errsum[0] = errsum[1] = errsum[2] = 0.0;
    for (i = 0; i < 4; ++i) {
        errsum[0] = errsum[0] + erfcc(ro[i] / pa) / (4.0 * PI * ro[i]);
        errsum[1] = errsum[1] + (derfcc(ro[i] / pa) / pa * dror[i] * ro[i] - dror[i] * erfcc(ro[i] / pa))
                                / (4.0 * PI * (ro[i] * ro[i]));
        errsum[2] = errsum[2] + (derfcc(ro[i] / pa) / pa * droz[i] * ro[i] - droz[i] * erfcc(ro[i] / pa))
                                / (4.0 * PI * (ro[i] * ro[i]));
    }
    if (fabs(sr) > SP(1.e-6)) {
        errsum[0] = errsum[0] + (erfcc(sr / pa) - 1.0) / (4.0 * PI * sr) + erfcc(sr1 / pa) / (4.0 * PI * sr1)
                  - 1.0 / (4.0 * PI * sr2);
        errsum[1] = errsum[1] - (erfcc(sr / pa) - 1.0) / (4.0 * PI * (sr * sr)) * dsrr
                  + derfcc(sr / pa) / (4.0 * PI * sr * pa) * dsrr
                  - erfcc(sr1 / pa) / (4.0 * PI * (sr1 * sr1)) * dsr1r
                  + derfcc(sr1 / pa) / (4.0 * PI * sr1 * pa) * dsr1r + dsr2r / (4.0 * PI * (sr2 * sr2));
        errsum[2] = errsum[2] - (erfcc(sr / pa) - 1.0) / (4.0 * PI * (sr * sr)) * dsrz
                  + derfcc(sr / pa) / (4.0 * PI * sr * pa) * dsrz
                  - erfcc(sr1 / pa) / (4.0 * PI * (sr1 * sr1)) * dsr1z
                  + derfcc(sr1 / pa) / (4.0 * PI * sr1 * pa) * dsr1z + dsr2z / (4.0 * PI * (sr2 * sr2));
    } else {
        errsum[0] = errsum[0] + erfcc(sr1 / pa) / (4.0 * PI * sr1) - 1.0 / (4.0 * PI * sr2);
        errsum[1] = errsum[1] - erfcc(sr1 / pa) / (4.0 * PI * (sr1 * sr1)) * dsr1r
                  + derfcc(sr1 / pa) / (4.0 * PI * sr1 * pa) * dsr1r + dsr2r / (4.0 * PI * (sr2 * sr2));
        errsum[2] = errsum[2] - erfcc(sr1 / pa) / (4.0 * PI * (sr1 * sr1)) * dsr1z
                  + derfcc(sr1 / pa) / (4.0 * PI * sr1 * pa) * dsr1z + dsr2z / (4.0 * PI * (sr2 * sr2));
    }

    gp.v = v; gp.r = r; gp.zf = zf; gp.zp = zp; gp.h = h;
    grn[0] = grn[0] - errsum[0] - v / 2.0 / PI * aquadf(&gp, 0.0, pa / 2.0, eps, 1);
    grn[1] = grn[1] - errsum[1] + v / 2.0 / PI * aquadf(&gp, 0.0, pa / 2.0, eps, 2);
    grn[2] = grn[2] - errsum[2] - v / 2.0 / PI * aquadf(&gp, 0.0, pa / 2.0, eps, 3);

    or_jy01bj(wk * r, &bj0, &bj1);
    km = -I * wk;
    {
        zdouble nmv = nm_fn(h, km);
        grn[0] = grn[0] - I / 4.0 / nmv * bj0 * cosh(wk * (zf + h)) * cosh(wk * (zp + h));
        grn[1] = grn[1] + I * wk / 4.0 / nmv * bj1 * cosh(wk * (zf + h)) * cosh(wk * (zp + h));
        grn[2] = grn[2] - I * wk / 4.0 / nmv * bj0 * sinh(wk * (zf + h)) * cosh(wk * (zp + h));
    }
    grn[0] = -4.0 * PI * grn[0];
    grn[1] = -4.0 * PI * grn[1];
    grn[2] = -4.0 * PI * grn[2];
    free(cof);
}

int or_fingreen_region(double rr, double h)
{
    double rhp = fabs(rr / h);
    if (rhp < 0.0005) return 0;
    if (rhp >= 0.0005 && rhp < 0.05) return 1;
    if (rhp >= 0.05 && rhp < 0.5) return 2;
    return 3;
}

/* FINGREEN3D_R :160-226 with TAG in {0,1}: no Rankine term is added. */
static void fingreen3d_r(double rr, double zf, double zp, double v, const double *wvn, int nk,
                         double h, zdouble out[3])
{
    zdouble fg[3];
    double wk = wvn[0];
    switch (or_fingreen_region(rr, h)) {
    case 0: linton(rr, zf, zp, v, wk, wvn, nk, h, fg); break;
    case 1: pidcock(rr, zf, zp, v, wk, wvn, nk, h, fg); break;
    case 2: eigene(rr, zf, zp, wk, wvn, nk, h, fg); break;
    default: eigen(rr, zf, zp, wk, wvn, h, fg); break;
    }
    out[1] = (rr != 0.0) ? fg[1] : 0.0;
    out[0] = fg[0];
    out[2] = fg[2];
}

void or_fingreen3d(double xf, double xp, double yf, double yp, double zf, double zp,
                   double v, const double *wvn, int nk, double h, zdouble grn[4], int flag)
{
    double xpq = xf - xp, ypq = yf - yp, zpq = zf + zp;
    double rr = sqrt(xpq * xpq + ypq * ypq);
    double r = sqrt(rr * rr + (zp - zf) * (zp - zf));
    double r1 = sqrt(rr * rr + zpq * zpq);
    double r13 = r1 * r1 * r1, r3 = r * r * r;
    zdouble fg[3];
    grn[0] = grn[1] = grn[2] = grn[3] = 0.0;
    if (fabs(v + 1.0) < SP(1.e-8) && !(fabs(v) < SP(1.e-8))) {
        /* label 200: infinite frequency */
        if (flag == 1) {
            grn[0] -= 1.0 / r1; grn[1] += xpq / r13; grn[2] += ypq / r13; grn[3] += zpq / r13;
        } else {
            grn[0] = grn[0] + (-1.0 / r1 + 1.0 / r);
            grn[1] = grn[1] + (xpq / r13 - xpq / r3);
            grn[2] = grn[2] + (ypq / r13 - ypq / r3);
            grn[3] = grn[3] + (zpq / r13 - (zf - zp) / r3);
        }
        return;
    }
    if (!(fabs(v) < SP(1.e-8))) {
        fingreen3d_r(rr, zf, zp, v, wvn, nk, h, fg);
        if (rr > SP(1.e-6)) {
            grn[1] = fg[1] * xpq / rr;
            grn[2] = fg[1] * ypq / rr;
        } else {
            grn[1] = 0.0;
            grn[2] = 0.0;
        }
        grn[0] = fg[0];
        grn[3] = fg[2];
    }
    /* label 100 */
    if (flag == 1) {
        grn[0] = grn[0] + 1.0 / r1;
        grn[1] = grn[1] - xpq / r13;
        grn[2] = grn[2] - ypq / r13;
        grn[3] = grn[3] - zpq / r13;
    } else {
        grn[0] = grn[0] + (1.0 / r1 + 1.0 / r);
        grn[1] = grn[1] - (xpq / r13 + xpq / r3);
        grn[2] = grn[2] - (ypq / r13 + ypq / r3);
        grn[3] = grn[3] - (zpq / r13 + (zf - zp) / r3);
    }
}
