"""The oracle's field-point potential (CalPotential, PressureElevation.f90:53-288)
checked on the CPU through an identity of the boundary-integral equation:
at a panel centroid the field point is on the body (SLD = 2 pi) and its panel
sums are exactly row i of the collocation system, so the field potential
reproduces the solved potential of that panel (scattered only with isol = 2,
plus the incident potential VINP with isol = 1)."""
import numpy as np
import pytest

from helpers import case_from_mesh, max_norm_err


@pytest.fixture(scope="module")
def cyl(pkg, oracle):
    case = case_from_mesh(oracle, pkg.meshgen.single_cylinder(), h=-1.0, headings_deg=(0.0, 60.0))
    res = oracle.solve_frequency(case, 1.0)
    return case, res


def test_centroids_reproduce_solved_potential(oracle, cyl):
    case, res = cyl
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, 1.0)
    betas = np.radians(case.ctl.headings)
    pot = oracle.field_potential(case, case.xyz_p, v, wk, w1, wvn, betas, res.mxpot, isol=2)
    assert pot.shape == res.mxpot.shape
    assert max_norm_err(pot, res.mxpot) < 1e-9


def test_isol1_adds_incident_potential(oracle, cyl):
    case, res = cyl
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, 1.0)
    betas = np.radians(case.ctl.headings)
    pts = np.array([[12.0, 3.0, -1.0], [-20.0, 0.0, 0.0]])
    p1 = oracle.field_potential(case, pts, v, wk, w1, wvn, betas, res.mxpot, isol=1)
    p2 = oracle.field_potential(case, pts, v, wk, w1, wvn, betas, res.mxpot, isol=2)
    nd = 6 * case.nbody
    assert np.array_equal(p1[:, :nd], p2[:, :nd])
    g = 9.80665
    for k, b in enumerate(betas):
        x, y, z = pts.T
        # deep-water VINP = -i g / w e^{k z} e^{i k (x cos b + y sin b)} / i
        vinp = -g / w1 * np.exp(wk * z) * np.exp(1j * wk * (x * np.cos(b) + y * np.sin(b)))
        assert np.allclose(p1[:, nd + k] - p2[:, nd + k], vinp, rtol=1e-12, atol=1e-12)
