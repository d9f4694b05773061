"""Dense complex LU and solves on the device (hg_gesv) against LAPACK.

The influence-matrix factorisation of the reference is ZGETRF followed by
ZGETRS (src/AssbMatx.f90:111,277); scipy's LAPACK wrappers of the same
routines are the checker here.  The shapes cover the library's code paths:
an odd leading dimension (8-byte operand staging), an even one (16-byte
staging), more than 64 right-hand sides (the wide GEMM with a 256-deep inner
dimension in the blocked solves) and a matrix small enough to skip the wide
GEMM altogether; orders >= 1024 take the complex64 two-level LU with
tensor-core updates and the block-inverse triangular solves (one and two
64-column chunks of right-hand sides).
"""
import numpy as np
import pytest
import scipy.linalg as sla

pytestmark = pytest.mark.gpu


def _system(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a += np.diag(np.full(n, 2.0 * np.sqrt(n)))  # keeps the condition number moderate
    b = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return np.asfortranarray(a), np.asfortranarray(b)


def _reconstruct(lu, ipiv):
    """P^T L U of LAPACK-style factors (rows interchanged in order)."""
    n = lu.shape[0]
    L = np.tril(lu, -1) + np.eye(n)
    U = np.triu(lu)
    m = L @ U
    for i in range(n - 1, -1, -1):
        p = ipiv[i] - 1
        if p != i:
            m[[i, p]] = m[[p, i]]
    return m


def _rel(x, y):
    return float(np.abs(x - y).max() / np.abs(y).max())


@pytest.fixture(scope="module")
def solver(pkg):
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_FP64)
    yield s
    s.close()


SHAPES = [(701, 3), (768, 70), (50, 4), (1030, 38), (1100, 70)]


@pytest.mark.parametrize("n,nrhs", SHAPES)
def test_gesv_fp64_matches_lapack(solver, n, nrhs):
    a, b = _system(n, nrhs, seed=n)
    lu, ipiv, x, it, info = solver.gesv(a, b, precision=0)
    assert info == 0 and it == 0
    lu_ref, piv_ref, info_ref = sla.lapack.zgetrf(a)
    assert info_ref == 0
    np.testing.assert_array_equal(ipiv, piv_ref + 1)
    assert _rel(lu, lu_ref) < 1e-12
    assert _rel(_reconstruct(lu, ipiv), a) < 1e-13
    x_ref, info_ref = sla.lapack.zgetrs(lu_ref, piv_ref, b)
    assert _rel(x, x_ref) < 1e-12


PIVOT_SHAPES = [(40, 3), (300, 5), (702, 48), (1030, 38)]


@pytest.mark.parametrize("n,nrhs", PIVOT_SHAPES)
def test_gesv_fp64_with_row_interchanges(solver, n, nrhs):
    """Plain Gaussian matrices: partial pivoting interchanges rows at almost
    every step (the diagonally weighted systems above need none), across
    panel and cluster-CTA boundaries; run three times (a race would show as
    run-to-run differences)."""
    rng = np.random.default_rng(1000 + n)
    a = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = np.asfortranarray(rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs)))
    lu_ref, piv_ref, info_ref = sla.lapack.zgetrf(a)
    x_ref, _ = sla.lapack.zgetrs(lu_ref, piv_ref, b)
    for _ in range(3):
        lu, ipiv, x, it, info = solver.gesv(a, b, precision=0)
        assert info == 0
        np.testing.assert_array_equal(ipiv, piv_ref + 1)
        assert _rel(lu, lu_ref) < 1e-12
        assert _rel(x, x_ref) < 1e-10


@pytest.mark.parametrize("n,nrhs", PIVOT_SHAPES + [(2100, 8), (8400, 4)])
def test_gesv_mixed_with_row_interchanges(solver, n, nrhs):
    """The complex64 LU (cluster panels, fused interchanges, tensor-core
    updates from order 1024) on Gaussian matrices, refined to the FP64
    solution.  Order 8400 takes both panel forms: the shared-memory panel
    while a panel has more than 16 x 512 rows, the register-resident one
    after."""
    rng = np.random.default_rng(2000 + n)
    a = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = np.asfortranarray(rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs)))
    x_ref = np.linalg.solve(a, b)
    for _ in range(2):
        lu, ipiv, x, it, info = solver.gesv(a, b, precision=1)
        assert info == 0 and it > 0
        assert _rel(x, x_ref) < 1e-9


@pytest.mark.parametrize("n,nrhs", SHAPES)
def test_gesv_mixed_refines_to_tolerance(solver, n, nrhs):
    a, b = _system(n, nrhs, seed=n + 1)
    lu, ipiv, x, it, info = solver.gesv(a, b, precision=1)
    assert info == 0
    assert 0 <= it <= 10
    # complex64 factors reproduce the matrix to single-precision accuracy
    assert _rel(_reconstruct(lu, ipiv), a) < 2e-6
    # refined solution: per-column residual within the default tolerance 1e-10
    r = b - a @ x
    worst = max(np.abs(r[:, k]).max() / np.abs(b[:, k]).max() for k in range(nrhs))
    assert worst < 1e-10
    x_ref = np.linalg.solve(a, b)
    assert _rel(x, x_ref) < 1e-9


def test_gesv_singular_reports_info(solver):
    n = 96
    a, b = _system(n, 2, seed=5)
    a[:, 40] = 0.0
    lu, ipiv, x, it, info = solver.gesv(a, b, precision=0)
    assert info == 41
    np.testing.assert_array_equal(x, b)  # left as it came
