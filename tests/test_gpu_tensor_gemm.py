"""The LU trailing-update GEMM on the tcgen05 tensor cores (hg_tc.cu).

C -= A B in complex64 is computed as one real product of twice the size
(each complex entry of A as its 2x2 real block), with operands split into
TF32 parts.  Checked against numpy in complex128 on the complex64-rounded
operands, at shapes that leave ragged tiles in both output dimensions and
inner dimensions that are and are not multiples of the 32-wide stage:
  - split TF32 (three products) to single-precision accuracy,
  - split BF16 (three products, 16 of the 24 bits) to ~2^-16,
  - plain TF32 (one product) to TF32 accuracy,
and through the LU of hg_gesv (order >= 1024 takes the two-level path whose
outer trailing updates run on these kernels), every variant refining to the
same 1e-10 residual.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _c64(x):
    return x.astype(np.complex64).astype(np.complex128)


def _operands(m, n, k, seed):
    rng = np.random.default_rng(seed)
    cx = lambda r, c: rng.standard_normal((r, c)) + 1j * rng.standard_normal((r, c))  # noqa: E731
    return (np.asfortranarray(_c64(cx(m, k))), np.asfortranarray(_c64(cx(k, n))),
            np.asfortranarray(_c64(cx(m, n))))


SHAPES = [(300, 520, 256), (65, 70, 32), (1000, 300, 256), (129, 257, 40)]


@pytest.fixture(scope="module")
def solver(pkg):
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_MIXED)
    yield s
    s.close()


@pytest.mark.parametrize("m,n,k", SHAPES)
@pytest.mark.parametrize("variant,tol", [(1, 3e-6), (2, 3e-6), (3, 3e-3), (4, 1e-4)])
def test_complex_gemm_variants(solver, m, n, k, variant, tol):
    a, b, c = _operands(m, n, k, seed=m * 7 + n + k)
    ref = c - a @ b
    got = solver.gemm_check(variant, a, b, c)
    # error relative to the size of the summed products, sqrt(k) * max|a| max|b|
    scale = np.sqrt(k) * np.abs(a).max() * np.abs(b).max()
    err = float(np.abs(got - ref).max() / scale)
    assert err < tol, f"variant {variant} {m}x{n}x{k}: {err:.3e}"


def test_split_tf32_beats_plain_tf32(solver):
    a, b, c = _operands(512, 512, 256, seed=11)
    ref = c - a @ b
    e3 = np.abs(solver.gemm_check(2, a, b, c) - ref).max()
    e1 = np.abs(solver.gemm_check(3, a, b, c) - ref).max()
    assert e3 * 20 < e1


@pytest.mark.parametrize("lu_tensor", [0, 1, 2, 3])
def test_lu_tensor_variants_refine(pkg, lu_tensor):
    n, nrhs = 1300, 5
    rng = np.random.default_rng(3)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a += np.diag(np.full(n, 2.0 * np.sqrt(n)))
    b = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    s = pkg.hamsgpu.Solver(precision=pkg.hamsgpu.HG_PREC_MIXED, lu_tensor=lu_tensor)
    try:
        lu, ipiv, x, it, info = s.gesv(a, b, precision=1)
    finally:
        s.close()
    assert info == 0 and 0 <= it <= 10
    r = b - a @ x
    assert max(np.abs(r[:, j]).max() / np.abs(b[:, j]).max() for j in range(nrhs)) < 1e-10
    # the factors reproduce the matrix to the accuracy of their update products
    n_ = lu.shape[0]
    L = np.tril(lu, -1) + np.eye(n_)
    U = np.triu(lu)
    m = L @ U
    for i in range(n_ - 1, -1, -1):
        p = ipiv[i] - 1
        if p != i:
            m[[i, p]] = m[[p, i]]
    rec = float(np.abs(m - a).max() / np.abs(a).max())
    assert rec < {1: 2e-3, 2: 2e-5}.get(lu_tensor, 2e-6)
