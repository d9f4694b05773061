"""GMRES-based refinement of the mixed form (refine_method = 1).

The reference's iterative solver (src/IterativeSolvers.f90:324-488,
ZGMRES_SOLVE: restarted GMRES with right preconditioning and Givens
rotations) is reused as the refinement engine: per outer step an FP64
residual, then GMRES on A d = r preconditioned by the complex64 LU.  Both
refinement methods must reach the same solution (they stop on the same 1e-10
residual), with the default split-BF16 factorisation, the split-TF32 one and
the weaker plain-TF32 one, where GMRES needs more than one Krylov step per
outer step.
"""
import numpy as np
import pytest

from helpers import max_norm_err

pytestmark = pytest.mark.gpu


def _solve(pkg, mesh, h, lu_tensor, refine_method, w=1.1):
    hg = pkg.hamsgpu
    s = hg.Solver(precision=hg.HG_PREC_MIXED, lu_tensor=lu_tensor, refine_method=refine_method)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    v, wk, w1, wvn = hg.wave_properties(3, w, h)
    a, b, f, x = s.solve_frequency(v, wk, w1, h, wvn, np.array([0.0, 0.9]))
    out = (a.copy(), b.copy(), f.copy(), x.copy(), s.refine_info(), s.gmres_iterations())
    s.close()
    return out


@pytest.mark.parametrize("lu_tensor", [2, 3, 1])
def test_gmres_refinement_matches_classical(pkg, lu_tensor):
    mesh = pkg.meshgen.three_cylinders(with_lid=False)
    assert mesh.n >= 1024  # the two-level LU with tensor-core updates
    ref = _solve(pkg, mesh, -1.0, 2, 0)
    got = _solve(pkg, mesh, -1.0, lu_tensor, 1)
    (sweeps, resid), its = got[4], got[5]
    assert resid <= 1e-10 and 1 <= sweeps <= 10 and its >= sweeps
    for k in range(4):
        assert max_norm_err(got[k], ref[k]) < 1e-8


def test_gmres_refinement_small_mesh(pkg):
    mesh = pkg.meshgen.single_cylinder()
    ref = _solve(pkg, mesh, -1.0, 3, 0)
    got = _solve(pkg, mesh, -1.0, 3, 1)
    assert got[4][1] <= 1e-10
    for k in range(4):
        assert max_norm_err(got[k], ref[k]) < 1e-8
