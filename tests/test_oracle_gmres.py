"""The oracle's restatement of the reference's iterative solver (ISOLV = 2:
ZGMRES_SOLVE with the Jacobi or block-diagonal LU preconditioner,
src/IterativeSolvers.f90:156-562) on small dense systems: it stops at the
reference's tolerance, an exact preconditioner converges in one step, a zero
right-hand side takes none, and the iteration cap reports non-convergence."""
import numpy as np
import pytest


def _system(n, nrhs, seed, shift=3.0):
    rng = np.random.default_rng(seed)
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    a += shift * np.eye(n)
    b = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return a, b


def test_gmres_jacobi_reaches_tolerance(oracle):
    a, b = _system(120, 3, 1)
    x, its, infos = oracle.gmres_columns(a, b)
    assert infos == [0, 0, 0] and all(0 < it < 100 for it in its)
    for k in range(3):
        assert np.linalg.norm(b[:, k] - a @ x[:, k]) < 1e-4 * np.linalg.norm(b[:, k])
    # the stopping rule is what limits the error: a tighter tolerance takes more steps
    x2, its2, _ = oracle.gmres_columns(a, b, tol=1e-10)
    assert all(i2 > i1 for i1, i2 in zip(its, its2))
    assert np.abs(x2 - np.linalg.solve(a, b)).max() < 1e-8


def test_gmres_block_preconditioner_exact_block(oracle):
    a, b = _system(60, 2, 2)
    x, its, infos = oracle.gmres_columns(a, b, blocks=[(0, 60)])
    assert its == [1, 1] and infos == [0, 0]
    assert np.abs(x - np.linalg.solve(a, b)).max() < 1e-10


def test_gmres_two_blocks(oracle):
    a, b = _system(80, 2, 3)
    a[:40, 40:] *= 0.1
    a[40:, :40] *= 0.1
    xb, itb, _ = oracle.gmres_columns(a, b, blocks=[(0, 40), (40, 40)])
    xj, itj, _ = oracle.gmres_columns(a, b)
    assert max(itb) < max(itj)
    for x in (xb, xj):
        assert np.linalg.norm(b - a @ x, axis=0).max() < 1e-4 * np.linalg.norm(b, axis=0).max()


def test_gmres_zero_rhs_and_cap(oracle):
    a, b = _system(50, 1, 4)
    x, its, infos = oracle.gmres_columns(a, np.zeros((50, 1), complex))
    assert its == [0] and infos == [0] and not x.any()
    # a matrix with eigenvalues around the origin: GMRES(2) stalls, the cap ends it
    rng = np.random.default_rng(5)
    q = np.linalg.qr(rng.standard_normal((40, 40)))[0]
    hard = q @ np.diag(np.exp(2j * np.pi * np.arange(40) / 40)) @ q.T
    x, its, infos = oracle.gmres_columns(hard, b[:40], restart=2, maxit=10)
    assert its == [10] and infos == [1]


def test_oracle_gmres_on_config1_against_lu(oracle):
    """The restated ISOLV = 2 path on the reference's own GMRES test deck
    (test/data/config1_gmres = config1 with Solver_type 2): three bodies, so
    the block-diagonal LU preconditioner; added mass and damping against the
    direct solve within the reference's test tolerances
    (test/test_integration_gmres.f90:50-101: relative Frobenius norm 1e-3 and
    5e-2)."""
    import os
    from conftest import GOLDEN
    case = oracle.load_case(os.path.join(GOLDEN, "config1", "input"))
    assert oracle.body_blocks(case) == [(0, 234), (234, 234), (468, 234)]
    w = case.ctl.wvnb[1]
    lu = oracle.solve_frequency(case, w, solver=1)
    it = oracle.solve_frequency(case, w, solver=2)
    for got, exp, tol in ((it.amas, lu.amas, 1e-3), (it.bdmp, lu.bdmp, 5e-2)):
        assert np.linalg.norm(got - exp) / np.linalg.norm(exp) < tol
    assert np.abs(it.exfc - lu.exfc).max() < 1e-3 * np.abs(lu.exfc).max()
