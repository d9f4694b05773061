"""GPU parity against the CPU oracle (restated reference Fortran).

Tolerances: the plain form is complex128 throughout and must match the
oracle to 1e-8 max-normalised relative error in added mass, damping and
excitation force (and the influence matrices element-wise to 1e-10); the
mixed form must stay within 1e-4.

Finite depth is the exception.  Its Pidcock-region series (0.0005 <= R/h <
0.05) are extrapolated with Wynn's epsilon algorithm, which turns last-bit
differences into much larger ones, so the reference's own results move when
only its rounding changes: the oracle compiled with fused multiply-adds
differs from the plain oracle by ~1e-7 in A and B (config1) and by up to
5e-4 in single influence-matrix entries.  One such rounding change is one
sample of the noise, and the GPU's math library is another (measured 1-4x
the FMA sample), so the GPU results are held to ten times that measured
spread, and never looser than the deep-water tolerances where the spread is
smaller.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import case_from_mesh, gpu_frequency, gpu_solver, max_norm_err

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-8
MATRIX_TOL = 1e-10
MIXED_TOL = 1e-4
SPREAD_FACTOR = 10.0


@pytest.fixture(scope="module")
def cyl_case(pkg, oracle):
    return case_from_mesh(oracle, pkg.meshgen.single_cylinder(), h=-1.0, headings_deg=(0.0, 45.0))


@pytest.fixture(scope="module")
def config1(oracle):
    return oracle.load_case(os.path.join(GOLDEN, "config1", "input"))


@pytest.fixture(scope="module")
def example5(oracle):
    return oracle.load_case(os.path.join(GOLDEN, "example5", "input"))


def _matrices_gpu(pkg, case, value, precision=0):
    s = gpu_solver(pkg, case, precision)
    s.keep_matrices(True)
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(case.ctl.inft, value, case.ctl.h)
    s.set_frequency(v, wk, w1, case.ctl.h, wvn)
    s.fill_factor(1 if case.nl > 0 else 0)
    rows = case.n + case.nl
    A = s.get_matrix(0, rows)
    S = s.get_matrix(1, rows)
    s.close()
    return A, S


@pytest.mark.parametrize("w", [0.3, 1.0, 2.0])
def test_fill_deep_matches_oracle(pkg, oracle, cyl_case, w):
    A, S = _matrices_gpu(pkg, cyl_case, w)
    v, wk, w1, wvn = oracle.wave_properties(cyl_case.ctl, w)
    Ao, So = oracle.assemble(cyl_case, v, wvn)
    assert max_norm_err(A, Ao) < MATRIX_TOL
    assert max_norm_err(S, So) < MATRIX_TOL


def _spread(oracle, fn):
    """(plain-oracle result, max-normalised spread to the FMA-built oracle)."""
    ref = fn()
    with oracle.use_library(oracle.build_fma_variant()):
        alt = fn()
    return ref, alt


def _check_within_spread(got, ref, alt, floor):
    spread = max_norm_err(alt, ref)
    err = max_norm_err(got, ref)
    assert err <= max(SPREAD_FACTOR * spread, floor), (err, spread)
    return err, spread


@pytest.mark.parametrize("case_name,freq_index", [("config1", 0), ("example5", 3)])
def test_fill_finite_depth_matches_oracle(pkg, oracle, config1, example5, case_name, freq_index):
    case = config1 if case_name == "config1" else example5
    w = case.ctl.wvnb[freq_index]
    A, S = _matrices_gpu(pkg, case, w)
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, w)
    (Ao, So), (Af, Sf) = _spread(oracle, lambda: oracle.assemble(case, v, wvn))
    assert A.shape == Ao.shape == (case.n + case.nl, case.n)
    _check_within_spread(A, Ao, Af, MATRIX_TOL)
    _check_within_spread(S, So, Sf, MATRIX_TOL)
    # entries outside the epsilon-algorithm region agree to the deep-water tolerance
    diff = np.abs(A - Ao) / np.abs(Ao).max()
    assert np.mean(diff > MATRIX_TOL) < 0.1


def _region_points(rng, h, count, lo, hi):
    """Source/field pairs with R/h in [lo, hi) below the free surface."""
    pts = []
    for _ in range(count):
        r = h * rng.uniform(lo, hi)
        th = rng.uniform(0, 2 * np.pi)
        zq = -rng.uniform(0.05, 0.9) * h
        zp = -rng.uniform(0.0, 0.9) * h
        pts.append([0.0, 0.0, zq, r * np.cos(th), r * np.sin(th), zp])
    return np.array(pts)


@pytest.mark.parametrize("region,lo,hi", [("linton", 0.0, 0.0005), ("pidcock", 0.0005, 0.05),
                                           ("eigene", 0.05, 0.5), ("eigen", 0.5, 6.0)])
def test_green_points_every_finite_depth_region(pkg, oracle, region, lo, hi):
    """Linton, eigenfunction and accelerated-eigenfunction regions to 1e-10;
    the Pidcock region to SPREAD_FACTOR times the oracle's own FMA spread at the same points."""
    rng = np.random.default_rng(11)
    h = 40.0
    for w in (0.4, 1.3):
        v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, w, h)
        pts = _region_points(rng, h, 24, lo, hi)
        if region == "linton":
            pts[:4, 3:5] = 0.0  # R = 0 exactly (vertically stacked panels)
        flags = np.array([k % 2 for k in range(len(pts))], dtype=np.int32)
        s = pkg.hamsgpu.Solver()
        s.set_frequency(v, wk, w1, h, wvn)
        got = s.green_points(pts, flags)
        s.close()
        import ctypes

        def evaluate():
            L = oracle.lib()
            wv = np.ascontiguousarray(wvn)
            out = np.zeros((len(pts), 4), dtype=np.complex128)
            for k, p in enumerate(pts):
                o8 = np.zeros(8)
                L.or_green_point(p[0], p[1], p[2], p[3], p[4], p[5], v,
                                 wv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(wv), h, int(flags[k]),
                                 o8.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
                out[k] = o8[0::2] + 1j * o8[1::2]
            return out

        exp, alt = _spread(oracle, evaluate)
        for q in range(4):
            scale = np.maximum(np.abs(exp[:, q]), 1e-12)
            err = (np.abs(got[:, q] - exp[:, q]) / scale).max()
            spread = (np.abs(alt[:, q] - exp[:, q]) / scale).max()
            tol = 1e-10 if region != "pidcock" else max(1e-10, SPREAD_FACTOR * spread)
            assert err < tol, (region, w, q, err, spread)


def test_green_points_deep_water(pkg, oracle):
    rng = np.random.default_rng(5)
    pts = np.column_stack([rng.uniform(-20, 20, 64), rng.uniform(-20, 20, 64), -rng.uniform(0.1, 10, 64),
                           rng.uniform(-20, 20, 64), rng.uniform(-20, 20, 64), -rng.uniform(0.0, 10, 64)])
    pts[:4, 3:5] = pts[:4, 0:2]  # vertically stacked
    flags = (np.arange(64) % 2).astype(np.int32)
    import ctypes
    L = oracle.lib()
    for w in (0.2, 1.0, 2.5):
        v = w * w / 9.80665
        s = pkg.hamsgpu.Solver()
        s.set_frequency(v, v, w, -1.0, None)
        got = s.green_points(pts, flags)
        s.close()
        for k, p in enumerate(pts):
            o8 = np.zeros(8)
            L.or_green_point(*[float(t) for t in p], v, None, 0, -1.0, int(flags[k]),
                             o8.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            exp = o8[0::2] + 1j * o8[1::2]
            assert np.abs(got[k] - exp).max() <= 1e-11 * max(1.0, np.abs(exp).max())


def _oracle_solve(oracle, case, value, betas=None):
    return oracle.solve_frequency(case, value, betas_deg=betas)


@pytest.mark.parametrize("w", [0.5, 1.2])
def test_plain_solve_deep_matches_oracle(pkg, oracle, cyl_case, w):
    s = gpu_solver(pkg, cyl_case)
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, w)
    s.close()
    ref = _oracle_solve(oracle, cyl_case, w)
    assert max_norm_err(amas, ref.amas) < PLAIN_TOL
    assert max_norm_err(bdmp, ref.bdmp) < PLAIN_TOL
    assert max_norm_err(exfc, ref.exfc) < PLAIN_TOL
    assert max_norm_err(mx, ref.mxpot) < PLAIN_TOL


def test_plain_solve_config1_matches_oracle_and_golden(pkg, oracle, config1):
    nb = config1.nbody
    E = [oracle.read_hams_rows(os.path.join(GOLDEN, "config1", "expected", f"OAMASS{k}.txt")) for k in range(1, 7)]
    s = gpu_solver(pkg, config1)
    for kk, w in enumerate(config1.ctl.wvnb):
        amas, bdmp, exfc, mx = gpu_frequency(pkg, s, config1, w)
        ref, alt = _spread(oracle, lambda: _oracle_solve(oracle, config1, w))
        _check_within_spread(amas, ref.amas, alt.amas, PLAIN_TOL)
        _check_within_spread(bdmp, ref.bdmp, alt.bdmp, PLAIN_TOL)
        _check_within_spread(exfc, ref.exfc, alt.exfc, PLAIN_TOL)
        for md1 in range(6):
            for bm in range(nb):
                for bn in range(nb):
                    row = E[md1][kk * nb * nb + bm * nb + bn][2:]
                    got = amas[6 * bm + md1, 6 * bn:6 * bn + 6]
                    # every printed 5-significant-digit value reproduced, entries far below the peak
                    # to the single-precision Green-value storage of the reference (5e-7 of the peak)
                    assert np.all(np.abs(got - row) <= 0.505e-4 * np.abs(row) + 5e-7 * np.abs(amas).max())
    s.close()


def test_plain_solve_irr_matches_oracle(pkg, oracle, example5):
    s = gpu_solver(pkg, example5)
    for w in example5.ctl.wvnb[:2]:
        amas, bdmp, exfc, mx = gpu_frequency(pkg, s, example5, w, betas_deg=example5.ctl.headings[:6])
        ref, alt = _spread(oracle, lambda: _oracle_solve(oracle, example5, w, betas=example5.ctl.headings[:6]))
        _check_within_spread(amas, ref.amas, alt.amas, PLAIN_TOL)
        _check_within_spread(bdmp, ref.bdmp, alt.bdmp, PLAIN_TOL)
        _check_within_spread(exfc, ref.exfc, alt.exfc, PLAIN_TOL)
    s.close()


def test_separate_calls_equal_one_call(pkg, cyl_case):
    """hg_fill_factor + hg_solve_radiation + hg_solve_all_headings + hg_forces
    (the Fortran subroutine sequence) equals hg_solve_frequency."""
    w = 0.8
    s = gpu_solver(pkg, cyl_case)
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, w)
    amas, bdmp, exfc = amas.copy(), bdmp.copy(), exfc.copy()
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, w, -1.0)
    s.set_frequency(v, wk, w1, -1.0, wvn)
    s.fill_factor(0)
    rad = s.solve_radiation()
    betas = np.array(cyl_case.ctl.headings) * np.pi / 180
    dif = s.solve_all_headings(betas)
    a2, b2, f2 = s.forces(len(betas))
    one = s.solve_diffraction(betas[1])
    s.close()
    assert np.allclose(rad, mx[:, :6], rtol=0, atol=1e-12 * np.abs(mx).max())
    assert np.allclose(dif, mx[:, 6:], rtol=0, atol=1e-12 * np.abs(mx).max())
    assert np.allclose(one, dif[:, 1], rtol=0, atol=1e-12 * np.abs(dif).max())
    assert max_norm_err(a2, amas) < 1e-13 and max_norm_err(b2, bdmp) < 1e-13 and max_norm_err(f2, exfc) < 1e-13


@pytest.mark.parametrize("w", [0.3, 1.0, 2.5])
def test_mixed_fill_deep_single_precision(pkg, oracle, cyl_case, w):
    """The single-precision fill of the mixed form (Chebyshev-basis local-flow
    polynomials, double-precision Newman integrals for near pairs) against
    the double-precision oracle."""
    A, S = _matrices_gpu(pkg, cyl_case, w, precision=1)
    v, wk, w1, wvn = oracle.wave_properties(cyl_case.ctl, w)
    Ao, So = oracle.assemble(cyl_case, v, wvn)
    assert max_norm_err(A, Ao) < 2e-6
    assert max_norm_err(S, So) < 2e-6


def test_mixed_solve_within_tolerance(pkg, oracle, cyl_case):
    s = gpu_solver(pkg, cyl_case, precision=1)
    for w in (0.5, 1.2):
        amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, w)
        ref = _oracle_solve(oracle, cyl_case, w)
        assert max_norm_err(amas, ref.amas) < MIXED_TOL
        assert max_norm_err(bdmp, ref.bdmp) < MIXED_TOL
        assert max_norm_err(exfc, ref.exfc) < MIXED_TOL
        sweeps, res = s.refine_info()
        assert res <= 1e-10
    s.close()


def test_mixed_solve_irr_within_tolerance(pkg, oracle, example5):
    s = gpu_solver(pkg, example5, precision=1)
    w = example5.ctl.wvnb[4]
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, example5, w, betas_deg=[0.0, 90.0])
    ref = _oracle_solve(oracle, example5, w, betas=[0.0, 90.0])
    s.close()
    assert max_norm_err(amas, ref.amas) < MIXED_TOL
    assert max_norm_err(bdmp, ref.bdmp) < MIXED_TOL
    assert max_norm_err(exfc, ref.exfc) < MIXED_TOL


def test_mixed_solve_finite_depth_within_tolerance(pkg, oracle, config1):
    """Finite depth in the mixed form (the FMA-contracted FP64 Green function, complex64 LU)."""
    s = gpu_solver(pkg, config1, precision=1)
    w = config1.ctl.wvnb[2]
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, config1, w)
    ref = _oracle_solve(oracle, config1, w)
    s.close()
    assert max_norm_err(amas, ref.amas) < MIXED_TOL
    assert max_norm_err(bdmp, ref.bdmp) < MIXED_TOL
    assert max_norm_err(exfc, ref.exfc) < MIXED_TOL

