"""The plain form's complex128 products on the tensor cores (hg_zgemm_tc.cu).

C -= A B with A, B, C in complex128, computed from eight balanced 7-bit BF16
digits of the row-scaled A and column-scaled B (Ozaki et al. 2012), the 36
digit pairs with s + t <= 9 summed exactly in FP32 per level, the levels
combined exactly in 64-bit integers and rounded once: FP64 accuracy, checked
per entry against numpy's complex128 result relative to |c| + sum_k |a_ik|
|b_kj| (the bound a double-precision c - a b is held to).  Shapes leave ragged tiles in both output dimensions,
inner dimensions below, at and above the 256 of one slicing pass, and rows
and columns whose entries span many orders of magnitude.  Then the two-level
complex128 LU built on it (hg_gesv, precision 0, order >= 1024) against the
FP64-pipe LU of the same matrix and LAPACK.
"""
import numpy as np
import pytest
import scipy.linalg as sla

pytestmark = pytest.mark.gpu


def _operands(m, n, k, seed, spread):
    rng = np.random.default_rng(seed)
    cx = lambda r, c: rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))  # noqa: E731
    a = cx(m, k) * np.exp(rng.uniform(-spread, 0, (m, 1))) * np.exp(rng.uniform(-spread, 0, (1, k)))
    b = cx(k, n) * np.exp(rng.uniform(-spread, 0, (1, n)))
    c = cx(m, n)
    return np.asfortranarray(a), np.asfortranarray(b), np.asfortranarray(c)


SHAPES = [(300, 520, 256), (65, 70, 32), (1000, 300, 256), (129, 257, 40), (257, 33, 600), (1, 1, 1)]


@pytest.fixture(scope="module")
def solver(pkg):
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_FP64)
    yield s
    s.close()


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("spread", [0.0, 12.0])
def test_sliced_zgemm_is_fp64_accurate(solver, m, n, k, spread):
    a, b, c = _operands(m, n, k, seed=m * 7 + n + k, spread=spread)
    ref = c - a @ b
    got = solver.gemm_check(5, a, b, c)
    # a double-precision c - a b is held to gamma_(k+1) (|c| + |a| |b|) per entry
    bound = np.abs(a) @ np.abs(b) + np.abs(c)
    err = float((np.abs(got - ref) / bound).max())
    # the digits' truncation (2^-57 of the row's and column's largest
    # entries) and two roundings, against numpy's own (k + 1) 2^-53 worst case
    assert err < 2e-15, f"{m}x{n}x{k} spread {spread}: {err:.3e}"


def test_sliced_zgemm_zero_operands(solver):
    """All-zero rows of A and columns of B (exponent 0) leave C unchanged."""
    a, b, c = _operands(200, 90, 70, seed=5, spread=0.0)
    a[17, :] = 0
    b[:, 3] = 0
    got = solver.gemm_check(5, a, b, c)
    np.testing.assert_array_equal(got[17, :], c[17, :])
    np.testing.assert_array_equal(got[:, 3], c[:, 3])


def _gesv(pkg, lu_tensor, a, b):
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_FP64, lu_tensor=lu_tensor)
    try:
        return s.gesv(a, b, precision=0)
    finally:
        s.close()


@pytest.mark.parametrize("n,nrhs", [(1100, 7), (2100, 8)])
def test_tensor_core_fp64_lu_matches_fp64_pipes_and_lapack(pkg, n, nrhs):
    """Gaussian matrices (a row interchange at almost every step): the same
    pivots as LAPACK and as the FP64-pipe LU (lu_tensor = 0); backward error
    max |P A - L U| / max |A| within 3x the FP64-pipe LU's (measured 1.5x:
    U12 from the inverse of L11 and one refinement step, against its
    triangular solve);
    factors within 1e-11 of both (forward differences of two correct
    factorisations grow with the order and the matrix's condition); solution
    within 1e-10 of LAPACK's."""
    rng = np.random.default_rng(4000 + n)
    a = np.asfortranarray(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = np.asfortranarray(rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs)))
    lu_ref, piv_ref, info_ref = sla.lapack.zgetrf(a)
    x_ref, _ = sla.lapack.zgetrs(lu_ref, piv_ref, b)
    lu_t, piv_t, x_t, _, info_t = _gesv(pkg, 2, a, b)
    lu_s, piv_s, x_s, _, info_s = _gesv(pkg, 0, a, b)
    assert info_t == 0 and info_s == 0 and info_ref == 0
    np.testing.assert_array_equal(piv_t, piv_ref + 1)
    np.testing.assert_array_equal(piv_t, piv_s)
    rel = lambda x, y: float(np.abs(x - y).max() / np.abs(y).max())  # noqa: E731

    def backward(lu, piv):
        m = (np.tril(lu, -1) + np.eye(n)) @ np.triu(lu)
        for i in range(n - 1, -1, -1):
            p = piv[i] - 1
            if p != i:
                m[[i, p]] = m[[p, i]]
        return float(np.abs(m - a).max() / np.abs(a).max())

    bt, bs = backward(lu_t, piv_t), backward(lu_s, piv_s)
    assert bt < 3 * bs and bt < 5e-13, (bt, bs)
    assert rel(lu_t, lu_ref) < 1e-11
    assert rel(lu_t, lu_s) < 1e-11
    assert rel(x_t, x_ref) < 1e-10
