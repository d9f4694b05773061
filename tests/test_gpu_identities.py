"""Deep water on the GPU held to the physical relations of
test_oracle_identities.py (exact hemisphere limits, Haskind, reciprocity),
in the plain and the mixed form, plus the plain form against the oracle at
the zero- and infinite-frequency limits (INFGREEN3D's V = 0 and V = -1
branches, src/InfGreen_Appr.f90:130-157)."""
import numpy as np
import pytest

from helpers import case_from_mesh, gpu_solver, max_norm_err
from test_oracle_identities import (displaced_mass, haskind_residual, headings_deg, hemisphere_mesh, oracle_limit,
                                    two_body_mesh)

pytestmark = pytest.mark.gpu

FORMS = [0, 1]  # HG_PREC_FP64, HG_PREC_MIXED


def gpu_limit(pkg, case, v, precision):
    s = gpu_solver(pkg, case, precision)
    amas, bdmp, _, _ = s.solve_frequency(v, v, 1.0, -1.0, None, np.zeros(0), want_potentials=False)
    s.close()
    return amas.copy(), bdmp.copy()


@pytest.mark.parametrize("precision", FORMS)
def test_hemisphere_exact_limits_gpu(pkg, oracle, precision):
    M = displaced_mass()
    case = case_from_mesh(oracle, hemisphere_mesh(pkg, 3), h=-1.0)
    a_inf, b_inf = gpu_limit(pkg, case, -1.0, precision)
    a_0, b_0 = gpu_limit(pkg, case, 0.0, precision)
    assert np.abs(b_inf).max() <= 1e-10 * np.abs(a_inf).max() and np.abs(b_0).max() <= 1e-10 * np.abs(a_0).max()
    assert abs(a_inf[2, 2] / M - 0.5) < 0.005
    assert abs(a_0[0, 0] / M - 0.5) < 0.002
    if precision == 0:
        for v, a in ((-1.0, a_inf), (0.0, a_0)):
            ref, _ = oracle_limit(oracle, case, v)
            assert max_norm_err(a, ref) < 1e-8


@pytest.mark.parametrize("precision", FORMS)
@pytest.mark.parametrize("w", [0.8, 1.5])
def test_haskind_and_reciprocity_gpu(pkg, oracle, precision, w):
    case = case_from_mesh(oracle, two_body_mesh(pkg, 2), h=-1.0, headings_deg=headings_deg())
    betas = np.array(headings_deg()) * np.pi / 180.0
    s = gpu_solver(pkg, case, precision)
    amas, bdmp, exfc, _ = s.solve_frequency(w * w / 9.80665, w * w / 9.80665, w, -1.0, None, betas,
                                            want_potentials=False)
    s.close()
    hk, asa, asb = haskind_residual(amas, bdmp, exfc, w)
    assert hk < 5e-3 and asa < 4e-3 and asb < 4e-3, (hk, asa, asb)
