"""Deep water pinned by physics the restatement cannot fake (CPU, oracle).

No input shipped with the reference uses infinite depth, so INFGREEN3D
(src/InfGreen_Appr.f90:104-205) and its consumers RFORCE / EFORCE
(src/PotentWavForce.f90:44-221) have no golden file.  These checks hold the
oracle's deep-water results to relations that any correct boundary-integral
solution satisfies, independently of how the Green function is coded:

* exact limits of a floating hemisphere (radius R, displaced mass
  M = rho 2/3 pi R^3).  At infinite frequency (V = -1: phi = 0 on the free
  surface) the heave potential of a sphere in unbounded fluid is odd in z,
  so the hemisphere's heave added mass is half the sphere's: A33 = M / 2.
  At zero frequency (V = 0: d phi / dz = 0 on the free surface) the sphere's
  sway potential is even in z, so A11 = M / 2.  Damping is zero at both
  limits, and the finite-frequency results approach the limits as w -> 0
  and w -> infinity;
* the Haskind relation between damping and excitation in deep water,
  B_ij = k w / (4 pi rho g^2) * integral over headings of Re(X_i conj(X_j)),
  which ties the radiation solution (wave part of the Green function, damping)
  to the diffraction solution plus the incident wave (excitation force);
* reciprocity: A and B symmetric, also between two different bodies.

Constant-panel collocation satisfies these only up to its discretisation
error, so each tolerance is set from the error measured on the test mesh
(about half the bound) and each check also asserts that the error shrinks
under mesh refinement: a wrong Green function leaves an O(1) residual that
refinement does not remove.  Measured with the oracle: hemisphere limits
A33/M = 0.4820 / 0.4956 / 0.4981 and A11/M = 0.4989 / 0.5001 / 0.5001 at
96 / 384 / 864 panels; Haskind residual (max-normalised) 6.1e-3 / 2.1e-3 /
1.1e-3 and asymmetry of A 3.4e-3 / 1.8e-3 / 1.1e-3 for a hemisphere and a
cylinder side by side at 156 / 624 / 1404 panels, w = 1.5 rad/s.
"""
import numpy as np
import pytest

from helpers import case_from_mesh

HEADINGS = 36


def hemisphere_mesh(pkg, scale):
    mg = pkg.meshgen
    return mg.combine([mg.hemisphere(1.0, 16 * scale, 6 * scale)])


def two_body_mesh(pkg, scale):
    mg = pkg.meshgen
    return mg.combine([mg.hemisphere(1.0, 16 * scale, 6 * scale),
                       mg.cylinder(0.8, 1.5, 12 * scale, 3 * scale, 2 * scale, cx=3.0, cy=1.0)])


def displaced_mass(rho=1000.0, radius=1.0):
    return rho * 2.0 / 3.0 * np.pi * radius ** 3


def oracle_limit(oracle, case, v):
    """Added mass and damping at V = 0 (zero frequency) or V = -1 (infinite)."""
    A, S = oracle.assemble(case, v, np.zeros(1))
    B = oracle.rhs(case, S, v, v, 1.0, [])
    X = oracle.lu_solve(np.asfortranarray(A), np.asfortranarray(B))
    amas, bdmp, _ = oracle.forces(case, X, v, v, 1.0, [])
    return amas, bdmp


def haskind_residual(amas, bdmp, exfc, w, rho=1000.0, g=9.80665):
    """max |B - B_Haskind| / max |B| and the asymmetry of A and B, for exfc
    over HEADINGS evenly spaced headings (rows)."""
    k = w * w / g
    H = (k * w / (4.0 * np.pi * rho * g * g)) * (2.0 * np.pi / exfc.shape[0]) * np.real(exfc.T @ exfc.conj())
    scale = np.abs(bdmp).max()
    return (float(np.abs(H - bdmp).max() / scale), float(np.abs(amas - amas.T).max() / np.abs(amas).max()),
            float(np.abs(bdmp - bdmp.T).max() / scale))


def headings_deg():
    return list(np.arange(HEADINGS) * 360.0 / HEADINGS)


def test_hemisphere_exact_limits(pkg, oracle):
    M = displaced_mass()
    errs = []
    for scale in (1, 2, 3):
        case = case_from_mesh(oracle, hemisphere_mesh(pkg, scale), h=-1.0)
        a_inf, b_inf = oracle_limit(oracle, case, -1.0)
        a_0, b_0 = oracle_limit(oracle, case, 0.0)
        assert np.all(b_inf == 0.0) and np.all(b_0 == 0.0)
        errs.append((abs(a_inf[2, 2] / M - 0.5), abs(a_0[0, 0] / M - 0.5)))
    assert errs[1][0] < 0.01 and errs[1][1] < 0.002, errs
    assert errs[2][0] < 0.5 * errs[0][0], errs  # heave converges to M / 2 (error ~ 1 / panels)


def test_hemisphere_frequency_limits(pkg, oracle):
    """w -> 0 approaches the V = 0 solution, w -> infinity the V = -1 one."""
    M = displaced_mass()
    case = case_from_mesh(oracle, hemisphere_mesh(pkg, 2), h=-1.0)
    a_0, _ = oracle_limit(oracle, case, 0.0)
    a_inf, _ = oracle_limit(oracle, case, -1.0)
    lo = oracle.solve_frequency(case, 0.01)
    assert np.abs(lo.amas - a_0).max() / M < 1e-3
    assert np.abs(lo.bdmp).max() / (M * 0.01) < 1e-4
    hi = oracle.solve_frequency(case, 20.0)  # kR = 41
    assert abs(hi.amas[2, 2] - a_inf[2, 2]) / M < 0.03
    assert hi.bdmp[2, 2] / (M * 20.0) < 1e-4


@pytest.mark.parametrize("w", [0.8, 1.5])
def test_haskind_and_reciprocity_converge(pkg, oracle, w):
    res = []
    for scale in (1, 2):
        case = case_from_mesh(oracle, two_body_mesh(pkg, scale), h=-1.0, headings_deg=headings_deg())
        r = oracle.solve_frequency(case, w)
        res.append(haskind_residual(r.amas, r.bdmp, r.exfc, w))
    hk, asa, asb = res[1]
    assert hk < 5e-3 and asa < 4e-3 and asb < 4e-3, res
    for q in range(3):
        assert res[1][q] < 0.7 * res[0][q], res  # 4x the panels: the residual shrinks
