"""Tabulated finite-depth Green function of the mixed form (fin_table).

The tables hold FINGREEN3D's own FP64 values on grids of (R, zq - zp) and
(R, zq + zp) (an exact split of the function); pairs interpolate them in
FP32.  Checked against the per-pair FP64 evaluation of the same mixed form
(fin_table = 0) through added mass, damping and excitation force, for two
depths, two frequencies and, with waterplane lids, the irregular-frequency
form (lid field points sit on the free surface).
"""
import numpy as np
import pytest

from helpers import max_norm_err

pytestmark = pytest.mark.gpu


def _run(pkg, mesh, h, w, table, irsp=0):
    hg = pkg.hamsgpu
    s = hg.Solver(precision=hg.HG_PREC_MIXED, fin_table=table)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges,
               mesh.lid_xyz_p if irsp == 1 else None)
    v, wk, w1, wvn = hg.wave_properties(3, w, h)
    a, b, f, _ = s.solve_frequency(v, wk, w1, h, wvn, np.array([0.0, 0.6]), irsp=irsp, want_potentials=False)
    rows = mesh.n + (len(mesh.lid_xyz_p) if irsp == 1 else 0)
    A = s.get_matrix(0, rows)
    S = s.get_matrix(1, rows)
    s.close()
    return a.copy(), b.copy(), f.copy(), A, S


# A, B, F of the table path against the per-pair FP64 evaluation of the same
# mixed form.  The reference's PIDCOCK values near the free surface carry
# rounding noise of O(1e-2) in single derivatives (its epsilon extrapolation
# of nearly converged sums); the tables interpolate noisy node values while
# the per-pair path reproduces the noise point by point, so the two differ by
# 1e-5 to 6e-4 (max-normalised) depending on depth and frequency, more than
# the 4e-5 by which two FP64 builds of the reference differ here.  The bound
# tested is that measured spread.
CASES = [(40.0, 0.8), (40.0, 2.0), (150.0, 0.8), (150.0, 2.0)]


@pytest.mark.parametrize("h,w", CASES)
def test_table_matches_per_pair_fp64(pkg, h, w):
    mesh = pkg.meshgen.three_cylinders(with_lid=False)
    ref = _run(pkg, mesh, h, w, 0)
    got = _run(pkg, mesh, h, w, 1)
    errs = [max_norm_err(got[k], ref[k]) for k in range(3)]
    assert max(errs) < 1e-3, errs


def test_table_with_lids(pkg):
    mesh = pkg.meshgen.three_cylinders(with_lid=True)
    ref = _run(pkg, mesh, 40.0, 1.3, 0, irsp=1)
    got = _run(pkg, mesh, 40.0, 1.3, 1, irsp=1)
    for k in range(3):
        assert max_norm_err(got[k], ref[k]) < 1e-3
