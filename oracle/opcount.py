"""Operation count of one deep-water panel pair of the reference's influence
matrix fill (TEST AND MEASUREMENT INFRASTRUCTURE ONLY: nothing in the
library imports this module).

The fill's algorithmic work is N * (N + Nl) * F_pair.  F_pair is counted, not
estimated: the pair code below restates the oracle's C restatement of the
reference (``or_assemble.c`` ``pair_terms`` and the BODINT_LEFT / RBC_RIGHT
terms of ``or_assemble``, ``or_panel.c`` ``sglint_quad`` / ``sglint_tri``,
``or_green.c`` ``or_infgreen3d`` / ``havelock_gf``; reference lines cited at
each function) in a scalar type that counts what it executes:

  add / subtract = 1, multiply = 1 (a multiply-add counts 2);
  divide, sqrt, exp, log, sin, cos, atan2 = 1 each, also reported by name;
  negation, comparisons, fabs and copysign = 0.

Complex values are pairs of counted reals, so a complex-by-real product
counts two multiplies.  ``tests/test_oracle_opcount.py`` checks that this
restatement returns the C oracle's own A and S entries for the same pairs.

Usage: ``python oracle/opcount.py`` counts a seeded sample of the pairs of
the 6048-panel five-body array at several frequencies and prints the
per-pair averages.
"""
from __future__ import annotations

import math
from collections import Counter

import numpy as np

COUNTS: Counter = Counter()
PI = 3.141592653589793


def sp(x: float) -> float:
    """A single-precision Fortran literal as the reference's double sees it."""
    return float(np.float32(x))


class F:
    """A float that counts the arithmetic done on it."""
    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v.v if isinstance(v, F) else float(v)

    @staticmethod
    def _v(x):
        return x.v if isinstance(x, F) else float(x)

    def __add__(self, o):
        COUNTS["add"] += 1
        return F(self.v + F._v(o))

    __radd__ = __add__

    def __sub__(self, o):
        COUNTS["add"] += 1
        return F(self.v - F._v(o))

    def __rsub__(self, o):
        COUNTS["add"] += 1
        return F(F._v(o) - self.v)

    def __mul__(self, o):
        COUNTS["mul"] += 1
        return F(self.v * F._v(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        COUNTS["div"] += 1
        return F(self.v / F._v(o))

    def __rtruediv__(self, o):
        COUNTS["div"] += 1
        return F(F._v(o) / self.v)

    def __neg__(self):
        return F(-self.v)

    def __lt__(self, o):
        return self.v < F._v(o)

    def __le__(self, o):
        return self.v <= F._v(o)

    def __gt__(self, o):
        return self.v > F._v(o)

    def __ge__(self, o):
        return self.v >= F._v(o)

    def __float__(self):
        return self.v


def _fn(name, f):
    def g(*a):
        COUNTS[name] += 1
        return F(f(*[F._v(x) for x in a]))
    return g


sqrt = _fn("sqrt", math.sqrt)
exp = _fn("exp", math.exp)
log = _fn("log", math.log)
sin = _fn("sin", math.sin)
cos = _fn("cos", math.cos)
atan2 = _fn("atan2", math.atan2)


def fabs(x):
    return abs(F._v(x))


def powi(t, n):
    """Integer power by repeated squaring, as compilers expand T**n."""
    r, b = None, t
    while n:
        if n & 1:
            r = b if r is None else r * b
        n >>= 1
        if n:
            b = b * b
    return r


# --- deep-water Green function: InfGreen_Appr.f90 -------------------------
def _horner(t, c0, cs):
    """c0 + t*(c1 + t*(c2 + ...)), evaluated innermost first as the source does."""
    g = cs[-1] * t
    for c in reversed(cs[:-1]):
        g = (c + g) * t
    return c0 + g


def gf_func_a(t):   # GF_FuncA :298-326
    return _horner(t, 1.21, [-13.328, 215.896, -1763.96, 8418.94, -24314.21, 42002.57, -41592.9, 21859.0,
                             -4838.6])


def gf_func_b(t):   # GF_FuncB :329-357
    return _horner(t, 0.938, [5.373, -67.92, 796.534, -4780.77, 17137.74, -36618.81, 44894.06, -29030.24,
                              7671.22])


def gf_func_c(t):   # GF_FuncC :360-384
    return _horner(t, 1.268, [-9.747, 209.653, -1397.89, 5155.67, -9844.35, 9136.4, -3272.62])


def gf_func_d(t):   # GF_FuncD :387-416
    return _horner(t, 0.632, [-40.97, 667.16, -6072.07, 31127.39, -96293.05, 181856.75, -205690.43, 128170.2,
                              -33744.6])


def gf_dfunc_a(t):  # GF_dFuncA :494-522
    return _horner(t, 2.948, [-24.53, 249.69, -754.85, -1187.71, 16370.75, -48811.41, 68220.87, -46688.0,
                              12622.25])


def gf_dfunc_b(t):  # GF_dFuncB :525-553
    return _horner(t, 1.11, [2.894, -76.765, 1565.35, -11336.19, 44270.15, -97014.11, 118879.26, -76209.82,
                             19923.28])


def gf_dfunc_c(t):  # GF_dFuncC :556-580
    return _horner(t, 14.19, [-148.24, 847.8, -2318.58, 3168.35, -1590.27])


def _poly(y, cs):
    """cs[0] + (cs[1] + (cs[2] + ...) * y) * y, the nested form of the source."""
    g = cs[-1]
    for c in reversed(cs[:-1]):
        g = c + g * y
    return g


def bessel_j0(xx):  # BesselJ0 :583-624
    if xx <= 3.0:
        yy = (xx / 3.0) * (xx / 3.0)
        return _poly(yy, [0.999999999, -2.249999879, 1.265623060, -0.316394552, 0.044460948, -0.003954479,
                          0.000212950])
    yy = 3.0 / xx
    y2 = yy * yy
    f0 = _poly(y2, [0.79788454, -0.00553897, 0.00099336, -0.00044346, 0.00020445, -0.00004959])
    th = xx - 0.25 * PI + _poly(y2, [-0.04166592, 0.00239399, -0.00073984, 0.00031099, -0.00007605]) * yy
    return f0 * cos(th) / sqrt(xx)


def bessel_j1(xx):  # BesselJ1 :627-671
    if xx <= 3.0:
        yy = xx / 3.0
        y2 = yy * yy
        b = _poly(y2, [0.5, -0.562499992, 0.210937377, -0.039550040, 0.004447331, -0.000330547, 0.000015525])
        return b * xx
    yy = 3.0 / xx
    y2 = yy * yy
    f1 = _poly(y2, [0.79788459, 0.01662008, -0.00187002, 0.00068519, -0.00029440, 0.00006952])
    th = xx - 0.75 * PI + _poly(y2, [0.12499895, -0.00605240, 0.00135825, -0.00049616, 0.00011531]) * yy
    return f1 * cos(th) / sqrt(xx)


def bessel_y0_large(xx):  # BesselY0 :674-715, xx > 3
    t = 3.0 / xx
    f0 = (0.79788454 - 0.00553897 * (t * t) + 0.00099336 * powi(t, 4) - 0.00044346 * powi(t, 6)
          + 0.00020445 * powi(t, 8) - 0.00004959 * powi(t, 10))
    th = (xx - 0.25 * PI - 0.04166592 * t + 0.00239399 * powi(t, 3) - 0.00073984 * powi(t, 5)
          + 0.00031099 * powi(t, 7) - 0.00007605 * powi(t, 9))
    return f0 * sin(th) / sqrt(xx)


def bessel_y1_large(xx):  # BesselY1 :718-760, xx > 3
    t = 3.0 / xx
    f1 = (0.79788459 + 0.01662008 * (t * t) - 0.00187002 * powi(t, 4) + 0.00068519 * powi(t, 6)
          - 0.00029440 * powi(t, 8) + 0.00006952 * powi(t, 10))
    th = (xx - 3.0 * PI / 4.0 + 0.12499895 * t - 0.00605240 * powi(t, 3) + 0.00135825 * powi(t, 5)
          - 0.00049616 * powi(t, 7) + 0.00011531 * powi(t, 9))
    return f1 * sin(th) / sqrt(xx)


def struve_h0(xx):  # StruveH0 :764-815
    if xx <= 3.0:
        yy = (xx / 3.0) * (xx / 3.0)
        h = _poly(yy, [1.909859164, -1.909855001, 0.687514637, -0.126164557, 0.013828813, -0.000876918])
        return h * (xx / 3.0)
    yy = (3.0 / xx) * (3.0 / xx)
    c1 = 2.0 * _poly(yy, [0.99999906, 4.77228920, 3.85542044, 0.32303607])
    c2 = PI * xx * _poly(yy, [1.0, 4.88331068, 4.28957333, 0.52120508])
    return c1 / c2 + bessel_y0_large(xx)


def struve_h1(xx):  # StruveH1 :818-870
    if xx <= 3.0:
        yy = (xx / 3.0) * (xx / 3.0)
        return _poly(yy, [1.909859286, -1.145914713, 0.294656958, -0.042070508, 0.003785727, -0.000207183]) * yy
    yy = (3.0 / xx) * (3.0 / xx)
    c1 = 2.0 * _poly(yy, [1.00000004, 3.92205313, 2.64893033, 0.27450895])
    c2 = PI * _poly(yy, [1.0, 3.81095112, 2.26216956, 0.10885141])
    return c1 / c2 + bessel_y1_large(xx)


def havelock_gf(hh, vv):
    """HavelockGF :189-205 (GF_DivParameters :209-224, L0/Lp/W and Ls/Lsp/Wh
    :227-491).  Returns (gf, gfh) as (re, im) pairs."""
    gama = 0.5772156649
    dd = sqrt(hh * hh + vv * vv)
    alpha = -vv / dd
    beta = hh / dd
    rho = dd / (1.0 + dd)
    pp = log(0.5 * (dd - vv)) + gama - 2.0 * dd * dd
    pp = exp(vv) * pp
    pp = pp + dd * dd - vv
    a, b, c, d = gf_func_a(rho), gf_func_b(rho), gf_func_c(rho), gf_func_d(rho)
    rr = (1.0 - beta) * a
    rr = rr - beta * b
    rr = rr - alpha * c / (1.0 + 6.0 * alpha * rho * (1.0 - rho))
    rr = rr + beta * (1.0 - beta) * d
    lp = rho * ((1.0 - rho) * (1.0 - rho) * (1.0 - rho)) * rr
    l0 = 2.0 * pp / (1.0 + dd * dd * dd) + 2.0 * lp
    h0, j0, e = struve_h0(hh), bessel_j0(hh), exp(vv)
    gf = (l0 + (2.0 * PI * h0 * e), 2.0 * PI * (-j0) * e)
    ps = (beta + hh) / (dd - vv)
    ps = ps - 2.0 * beta + 2.0 * exp(vv) * dd - hh
    qs = exp(-dd) * (1.0 - beta)
    qs = qs * (1.0 + dd / (1.0 + dd * dd * dd))
    a, b, c = gf_dfunc_a(rho), gf_dfunc_b(rho), gf_dfunc_c(rho)
    rr = beta * a
    rr = rr - (1.0 - alpha) * b
    rr = rr + beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * c
    lsp = rho * ((1.0 - rho) * (1.0 - rho) * (1.0 - rho)) * rr
    ls = 2.0 * ps / (1.0 + dd * dd * dd) - 4.0 * qs + 2.0 * lsp
    h1, j1, e = struve_h1(hh), bessel_j1(hh), exp(vv)
    gfh = (ls + (2.0 * PI * (2.0 / PI - h1) * e), 2.0 * PI * j1 * e)
    return gf, gfh


def infgreen3d(xf, xp, yf, yp, zf, zp, v, flag):
    """INFGREEN3D :104-186 for a regular frequency (V neither 0 nor -1).
    Returns grn[4] as (re, im) pairs."""
    xpq, ypq, zpq = xf - xp, yf - yp, zp + zf
    rr = sqrt(xpq * xpq + ypq * ypq)
    r = sqrt(rr * rr + (zp - zf) * (zp - zf))
    r1 = sqrt(rr * rr + zpq * zpq)
    r13, r3 = r1 * r1 * r1, r * r * r
    gf, gfh = havelock_gf(v * rr, v * zpq)
    if rr > sp(1.e-6):
        vv = -(v * v)
        g1 = ((vv * gfh[0]) * xpq / rr, (vv * gfh[1]) * xpq / rr)
        g2 = ((vv * gfh[0]) * ypq / rr, (vv * gfh[1]) * ypq / rr)
    else:
        g1 = (F(0.0), F(0.0))
        g2 = (F(0.0), F(0.0))
    g0 = (-v * gf[0], -v * gf[1])
    vv = -(v * v)
    g3 = (vv * gf[0] + 2.0 * v / r1, vv * gf[1])
    if flag == 1:
        g0 = (g0[0] + 1.0 / r1, g0[1])
        g1 = (g1[0] - xpq / r13, g1[1])
        g2 = (g2[0] - ypq / r13, g2[1])
        g3 = (g3[0] - zpq / r13, g3[1])
    else:
        g0 = (g0[0] + 1.0 / r1 + 1.0 / r, g0[1])
        g1 = (g1[0] - xpq / r13 - xpq / r3, g1[1])
        g2 = (g2[0] - ypq / r13 - ypq / r3, g2[1])
        g3 = (g3[0] - zpq / r13 - (zf - zp) / r3, g3[1])
    return [g0, g1, g2, g3]


# --- Newman panel integrals: SingularIntgr.f90 ------------------------------
def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _edges(ksi, eta, x, y, z, nv, quad):
    st = sxt = syt = szt = F(0.0)
    for i in range(nv):
        dksi, deta = ksi[i + 1] - ksi[i], eta[i + 1] - eta[i]
        r1 = sqrt((ksi[i] - x) * (ksi[i] - x) + (eta[i] - y) * (eta[i] - y) + z * z)
        r2 = sqrt((ksi[i + 1] - x) * (ksi[i + 1] - x) + (eta[i + 1] - y) * (eta[i + 1] - y) + z * z)
        el = sqrt((ksi[i + 1] - ksi[i]) * (ksi[i + 1] - ksi[i]) + (eta[i + 1] - eta[i]) * (eta[i + 1] - eta[i]))
        if quad and fabs(el) < 1.0e-8:
            continue
        b1 = deta * ((ksi[i] - x) * (ksi[i] - x) + z * z) - dksi * (ksi[i] - x) * (eta[i] - y)
        a1 = r1 * z * dksi
        b2 = deta * ((ksi[i + 1] - x) * (ksi[i + 1] - x) + z * z) - dksi * (ksi[i + 1] - x) * (eta[i + 1] - y)
        a2 = r2 * z * dksi
        if not fabs(z) < 1.0e-6:
            szt = szt + atan2((b1 * a2 - b2 * a1), (a1 * a2 + b1 * b2))
        if fabs(r1 + r2 - el) < 1.0e-6:
            continue
        lgrn = log((r1 + r2 + el) / (r1 + r2 - el))
        sxt = sxt - deta / el * lgrn
        syt = syt + dksi / el * lgrn
        t = (deta * (x - ksi[i]) - dksi * (y - eta[i])) / el * lgrn
        st = st - t if quad else st + t
    return st, sxt, syt, szt


def sglint_quad(xv, xf):
    """SGLINTBD_QUAD :252-445: (SIJ, DIJ[3])."""
    po = [(xv[0][k] + xv[1][k] + xv[2][k] + xv[3][k]) / 4.0 for k in range(3)]
    pov = [[xv[j][k] - po[k] for k in range(3)] for j in range(2)]
    un = [pov[0][1] * pov[1][2] - pov[0][2] * pov[1][1], pov[0][2] * pov[1][0] - pov[0][0] * pov[1][2],
          pov[0][0] * pov[1][1] - pov[0][1] * pov[1][0]]
    nn = sqrt(_dot(pov[0], pov[0]))
    ui = [pov[0][k] / nn for k in range(3)]
    nn = sqrt(_dot(un, un))
    uk = [un[k] / nn for k in range(3)]
    uj = [uk[1] * ui[2] - uk[2] * ui[1], uk[2] * ui[0] - uk[0] * ui[2], uk[0] * ui[1] - uk[1] * ui[0]]
    pof = [xf[k] - po[k] for k in range(3)]
    x, y, z = _dot(ui, pof), _dot(uj, pof), _dot(uk, pof)
    pov += [[xv[j][k] - po[k] for k in range(3)] for j in (2, 3)]
    pon = []
    for i in range(4):
        d = _dot(uk, pov[i])
        pon.append([pov[i][j] - d * uk[j] for j in range(3)])
    ksi = [_dot(ui, pon[i]) for i in range(4)]
    eta = [_dot(uj, pon[i]) for i in range(4)]
    ksi.append(ksi[0])
    eta.append(eta[0])
    st, sxt, syt, szt = _edges(ksi, eta, x, y, z, 4, True)
    st = st + z * szt
    dij = [-(ui[k] * sxt + uj[k] * syt + uk[k] * szt) for k in range(3)]
    return st, dij


def sglint_tri(xv, xf):
    """SGLINTBD_TRI :44-244 (NCN = 3): (SIJ, DIJ[3])."""
    p12 = [xv[1][k] - xv[0][k] for k in range(3)]
    p13 = [xv[2][k] - xv[0][k] for k in range(3)]
    alfa = _dot(p12, p13) / _dot(p12, p12)
    po = [xv[0][k] + alfa * p12[k] for k in range(3)]
    po3 = [xv[2][k] - po[k] for k in range(3)]
    n12, n3 = sqrt(_dot(p12, p12)), sqrt(_dot(po3, po3))
    ui = [p12[k] / n12 for k in range(3)]
    uj = [po3[k] / n3 for k in range(3)]
    uk = [ui[1] * uj[2] - ui[2] * uj[1], ui[2] * uj[0] - ui[0] * uj[2], ui[0] * uj[1] - ui[1] * uj[0]]
    pof = [xf[k] - po[k] for k in range(3)]
    x, y, z = _dot(ui, pof), _dot(uj, pof), _dot(uk, pof)
    po1 = [xv[0][k] - po[k] for k in range(3)]
    po2 = [xv[1][k] - po[k] for k in range(3)]
    ksi = [F(-math.copysign(1.0, alfa.v)) * sqrt(_dot(po1, po1)), F(0.0), sqrt(_dot(po2, po2))]
    eta = [F(0.0), sqrt(_dot(po3, po3)), F(0.0)]
    ksi.append(ksi[0])
    eta.append(eta[0])
    st, sxt, syt, szt = _edges(ksi, eta, x, y, z, 3, False)
    st = st - z * szt
    dij = [ui[k] * sxt + uj[k] * syt + uk[k] * szt for k in range(3)]
    return st, dij


# --- one pair of the fill: CalGreenFunc.f90 + BodyIntgr.f90 -----------------
def pair_entries(xf, xq, pnsz, verts, ncn, ear, env, v):
    """A and S entries (without the 2 pi diagonal) of field point xf and
    source panel (centroid xq, size pnsz, vertices, area ear, normal env):
    the FLAG test and SGLINTBD of CALGREEN (CalGreenFunc.f90:49-118),
    INFGREEN3D, then BODINT_LEFT (BodyIntgr.f90:64-74) and the DUM of
    RBC_RIGHT (BodyIntgr.f90:98-102)."""
    xf = [F(t) for t in xf]
    xq = [F(t) for t in xq]
    dist = sqrt((xf[0] - xq[0]) * (xf[0] - xq[0]) + (xf[1] - xq[1]) * (xf[1] - xq[1])
                + (xf[2] - xq[2]) * (xf[2] - xq[2]))
    flag = 1 if dist <= F(pnsz) * 50.0 else 0
    rkn = [F(0.0)] * 4
    if flag:
        vv = [[F(t) for t in verts[k]] for k in range(ncn)]
        sij, dij = sglint_tri(vv, xf) if ncn == 3 else sglint_quad(vv, xf)
        rkn = [sij] + dij
    grn = infgreen3d(xq[0], xf[0], xq[1], xf[1], xq[2], xf[2], F(v), flag)
    ear, env = F(ear), [F(t) for t in env]
    if flag:
        a = [(rkn[k + 1] + grn[k + 1][0] * ear, grn[k + 1][1] * ear) for k in range(3)]
        tre = a[0][0] * env[0] + a[1][0] * env[1] + a[2][0] * env[2]
        tim = a[0][1] * env[0] + a[1][1] * env[1] + a[2][1] * env[2]
        dum = (rkn[0] + grn[0][0] * ear, grn[0][1] * ear)
    else:
        sre = grn[1][0] * env[0] + grn[2][0] * env[1] + grn[3][0] * env[2]
        sim = grn[1][1] * env[0] + grn[2][1] * env[1] + grn[3][1] * env[2]
        tre, tim = sre * ear, sim * ear
        dum = (grn[0][0] * ear, grn[0][1] * ear)
    return flag, complex(tre.v, tim.v), complex(dum[0].v, dum[1].v)


def count_sample(mesh, w, npairs=20000, seed=0, g=9.80665):
    """Average counted operations per pair over a seeded uniform sample of
    the mesh's (field, source) pairs at circular frequency w (deep water)."""
    v = w * w / g
    rng = np.random.default_rng(seed)
    n = mesh.n
    rows = rng.integers(0, n, npairs)
    cols = rng.integers(0, n, npairs)
    COUNTS.clear()
    near = 0
    for i, j in zip(rows, cols):
        verts = [mesh.nodes[mesh.ncon[j, k] - 1] for k in range(mesh.ncn[j])]
        f, _, _ = pair_entries(mesh.xyz_p[i], mesh.xyz_p[j], float(mesh.pnsz[j]), verts, int(mesh.ncn[j]),
                               float(mesh.ds[j]), mesh.dxyz_p[j, :3], v)
        near += f
    per = {k: c / npairs for k, c in COUNTS.items()}
    return per, near / npairs


def flops(per):
    """The convention's total: every counted operation weighs 1."""
    return sum(per.values())


def main():
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "hams-mrel_gb300"))
    import meshgen
    mesh = meshgen.five_body_array()
    freqs = np.linspace(0.1, 2.5, 60)
    tot, rows = [], []
    for w in freqs[::6]:
        per, near = count_sample(mesh, float(w), npairs=4000, seed=int(w * 1000))
        tot.append(flops(per))
        rows.append((w, near, per))
        print(f"w {w:5.3f}: near-field share {near:.3f}, F_pair {flops(per):7.1f}  "
              + ", ".join(f"{k} {per[k]:.2f}" for k in sorted(per)))
    print(f"mean F_pair over the sampled frequencies: {np.mean(tot):.1f}")


if __name__ == "__main__":
    main()
