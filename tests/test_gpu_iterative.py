"""The iterative solver (opts.solver = 2; the reference's Solver_type /
ISOLV = 2: restarted GMRES(25), tolerance 1e-4, at most 100 iterations,
Jacobi or block-diagonal LU right preconditioner,
src/IterativeSolvers.f90:156-562).

1. On the GPU's own FP64 matrices the device GMRES takes the oracle's
   iteration count (restated ZGMRES_SOLVE with modified Gram-Schmidt; the
   device runs classical Gram-Schmidt twice) and reaches its iterate to
   1e-8: Jacobi for one body (also on the normal equations of
   irregular-frequency removal), per-body LU blocks for three.
2. The reference's own GMRES integration test
   (test/test_integration_gmres.f90:50-101): config1's deck with
   Solver_type 2 against the direct solve's expected outputs, relative
   Frobenius norm 1e-3 for added mass and 5e-2 for damping.
3. The mixed form with solver 2 (complex64 matrix, block LU preconditioner
   in complex64) against the direct solve, within the GMRES tolerance, with
   and without the normal equations of irregular-frequency removal.
"""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import case_from_mesh, gpu_frequency, gpu_solver, max_norm_err

pytestmark = pytest.mark.gpu

ITER_TOL = 1e-8        # device GMRES vs the oracle's, same matrices, same iteration count
SOLVE_TOL = 1e-3       # GMRES (1e-4 residual) vs the direct solve, max-norm relative in A, B, F


@pytest.fixture(scope="module")
def cyl_case(pkg, oracle):
    return case_from_mesh(oracle, pkg.meshgen.single_cylinder(), h=-1.0, headings_deg=(0.0, 45.0))


@pytest.fixture(scope="module")
def config1(oracle):
    return oracle.load_case(os.path.join(GOLDEN, "config1", "input"))


def _device_and_oracle(pkg, oracle, case, value):
    s = gpu_solver(pkg, case, 0, solver=2)
    s.keep_matrices(True)
    a, b, f, x = gpu_frequency(pkg, s, case, value)
    rows = case.n + case.nl
    A = s.get_matrix(0, rows)
    S = s.get_matrix(1, rows)
    its, restarts, unconv, resid = s.iter_info()
    s.close()
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, value)
    betas = [h * np.pi / 180.0 for h in case.ctl.headings]
    B = oracle.rhs(case, S, v, wk, w1, betas)
    if case.nl > 0:  # GMRES on the normal equations C = A^T A, D = A^T B
        A, B = oracle.normal_equations(case, A, B)
    xo, its_o, infos = oracle.gmres_columns(A, B, oracle.body_blocks(case))
    return x.copy(), xo, (its, restarts, unconv, resid), its_o, infos


@pytest.mark.parametrize("w", [0.5, 1.5])
def test_gmres_jacobi_matches_oracle(pkg, oracle, cyl_case, w):
    x, xo, (its, restarts, unconv, resid), its_o, infos = _device_and_oracle(pkg, oracle, cyl_case, w)
    assert unconv == 0 and all(i == 0 for i in infos)
    assert its == max(its_o) and restarts >= 1 and resid < 1e-4
    assert max_norm_err(x, xo) < ITER_TOL


def test_gmres_block_lu_matches_oracle(pkg, oracle, config1):
    x, xo, (its, restarts, unconv, resid), its_o, infos = _device_and_oracle(pkg, oracle, config1,
                                                                              config1.ctl.wvnb[1])
    assert unconv == 0 and all(i == 0 for i in infos)
    assert its == max(its_o)
    assert max_norm_err(x, xo) < ITER_TOL


def test_gmres_jacobi_normal_equations_matches_oracle(pkg, oracle):
    """example5: one body with lids, irregular-frequency removal (IRSP = 1):
    Jacobi on C = A^T A (AssbMatx_irr.f90:494-498), finite depth."""
    case = oracle.load_case(os.path.join(GOLDEN, "example5", "input"))
    x, xo, (its, restarts, unconv, resid), its_o, infos = _device_and_oracle(pkg, oracle, case, case.ctl.wvnb[2])
    assert unconv == 0 and all(i == 0 for i in infos)
    assert its == max(its_o)
    assert max_norm_err(x, xo) < ITER_TOL


def _frob_rows(path):
    with open(path) as f:
        return np.array([[float(t) for t in ln.split()] for ln in f if ln.strip()])


def test_config1_gmres_deck_against_lu_outputs(pkg, tmp_path):
    """test/data/config1_gmres: Solver_type 2 read from the deck."""
    deck = os.path.join(tmp_path, "input")
    shutil.copytree(os.path.join(GOLDEN, "config1", "input"), deck)
    shutil.copy(os.path.join(GOLDEN, "config1_gmres", "ControlFile.in"), os.path.join(deck, "ControlFile.in"))
    out_it = os.path.join(tmp_path, "gmres")
    out_lu = os.path.join(tmp_path, "lu")
    pkg.hamsgpu.Case(deck).run(out_it, precision=pkg.hamsgpu.HG_PREC_FP64, nslots=2)
    pkg.hamsgpu.Case(os.path.join(GOLDEN, "config1", "input")).run(out_lu, precision=pkg.hamsgpu.HG_PREC_FP64,
                                                                    nslots=2)
    differs = False
    for i in range(1, 7):
        for name, tol in (("OAMASS", 1e-3), ("ODAMPING", 5e-2)):
            exp = _frob_rows(os.path.join(GOLDEN, "config1", "expected", f"{name}{i}.txt"))
            got = _frob_rows(os.path.join(out_it, "Hams_format", f"{name}{i}.txt"))
            lu = _frob_rows(os.path.join(out_lu, "Hams_format", f"{name}{i}.txt"))
            assert got.shape == exp.shape
            err = np.linalg.norm(got - exp) / max(np.linalg.norm(exp), 1e-30)
            print(f"{name}{i}: GMRES vs shipped LU output {err:.2e} (limit {tol})")
            assert err < tol
            differs = differs or not np.array_equal(got, lu)
    assert differs  # the deck's Solver_type reached the solver


def _forces(pkg, mesh_or_case, h, precision, solver, w, betas=(0.0, 0.9), irsp=0):
    hg = pkg.hamsgpu
    s = hg.Solver(precision=precision, solver=solver)
    m = mesh_or_case
    s.set_mesh(m.nodes, m.ncon, m.ncn, m.xyz_p, m.ds, m.pnsz, m.dxyz_p, m.body_ranges,
               m.lid_xyz_p if irsp else None)
    v, wk, w1, wvn = hg.wave_properties(3, w, h)
    a, b, f, x = s.solve_frequency(v, wk, w1, h, wvn, np.array(betas), irsp=irsp)
    info = s.iter_info() if solver == 2 else None
    out = (a.copy(), b.copy(), f.copy(), info)
    s.close()
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_gmres_three_bodies_against_direct(pkg, precision):
    mesh = pkg.meshgen.three_cylinders(with_lid=False)
    assert mesh.n >= 1024
    ref = _forces(pkg, mesh, -1.0, precision, 1, 1.1)
    got = _forces(pkg, mesh, -1.0, precision, 2, 1.1)
    its, restarts, unconv, resid = got[3]
    assert unconv == 0 and resid < 1e-4 and 0 < its <= 100
    for k in range(3):
        err = max_norm_err(got[k], ref[k])
        print(f"three cylinders, precision {precision}: {'ABF'[k]} {err:.2e} in {its} iterations")
        assert err < SOLVE_TOL


def test_gmres_normal_equations_against_direct(pkg):
    mesh = pkg.meshgen.three_cylinders(with_lid=True)
    ref = _forces(pkg, mesh, -1.0, 1, 1, 1.1, irsp=1)
    got = _forces(pkg, mesh, -1.0, 1, 2, 1.1, irsp=1)
    its, restarts, unconv, resid = got[3]
    assert unconv == 0 and resid < 1e-4
    for k in range(3):
        err = max_norm_err(got[k], ref[k])
        print(f"three cylinders with lids (normal equations): {'ABF'[k]} {err:.2e} in {its} iterations")
        assert err < SOLVE_TOL
