"""The mixed form's FP64-accurate refinement residual r = b - A x (A the
complex64 matrix, exact in single precision; x, b complex128) through its two
kernels (hg_resid_check): the double-float products on the FP32 pipes
(hg_resid.cu) and the sliced products on the tensor cores (hg_resid_tc.cu:
Ozaki et al. 2012, BF16 digits of row- and column-scaled operands with exact
FP32 partial sums).  Both against numpy in complex128 on the complex64-rounded
A, relative to sum |a||x| per entry (numpy's own rounding reaches ~k 2^-53 of
that, 2e-13 at k = 2100): the double-float kernel to 1e-12, the
sliced one to 1e-11 (its digits keep 42 bits below each row's and each
column's largest entry, ~2e-13 of those maxima, which on rows whose entries
fall off over five orders of magnitude is a larger fraction of sum |a||x|),
at ragged shapes (rows and inner dimension not multiples of the kernels'
tiles) and with the near-cancelling b of a refinement step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(300, 38, 300), (1000, 38, 1000), (777, 17, 1301), (2100, 40, 2100)]


@pytest.fixture(scope="module")
def solver(pkg):
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_MIXED)
    yield s
    s.close()


def _case(m, nc, k, seed):
    rng = np.random.default_rng(seed)
    cx = lambda r, c: rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))  # noqa: E731
    # entries decaying away from the diagonal over ~5 orders of magnitude
    i = np.arange(m)[:, None]
    p = np.arange(k)[None, :]
    a = cx(m, k) * 10.0 ** (-5.0 * np.minimum(np.abs(i - p), 400) / 400.0)
    a = a.astype(np.complex64).astype(np.complex128)
    x = cx(k, nc) * 10.0 ** rng.uniform(-2, 2, (1, nc))
    b = a @ x + 1e-6 * cx(m, nc)  # a refinement step's near-cancelling right-hand side
    return a, x, b


@pytest.mark.parametrize("m,nc,k", SHAPES)
@pytest.mark.parametrize("variant,tol", [(0, 1e-12), (1, 5e-11)])
def test_residual_kernels_match_numpy(solver, m, nc, k, variant, tol):
    a, x, b = _case(m, nc, k, seed=m + 7 * nc + k)
    ref = b - a @ x
    scale = np.abs(a) @ np.abs(x)
    got = solver.resid_check(variant, a, x, b)
    err = float((np.abs(got - ref) / scale).max())
    assert err < tol, f"variant {variant} {m}x{nc}x{k}: {err:.3e}"
