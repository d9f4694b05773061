"""Field-point potential, pressure and elevation on the GPU (hg_field_points,
CalPotential / CalPressure / CalElevation of PressureElevation.f90:53-336 and
PressureElevationMulti.f90:55-360) against the oracle.

The oracle is given the GPU's own solved panel potentials, so the check
covers the field-point step alone (the solve has its own parity tests).
Deep water: the plain form's field-point Green function and panel sums are
FP64, held to 1e-10 max-normalised; the mixed form takes its single-precision
fill for the field rows and double-float products with the FP64 solution,
held to 1e-5 (inside the mixed form's 1e-4 contract).  Finite depth: the Pidcock-region
series noise of the Green function (see test_gpu_parity.py) bounds the
agreement; the GPU is held to ten times the measured spread between the
plain and the FMA-compiled oracle, never looser than 1e-10 where that spread
is smaller.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import case_from_mesh, gpu_frequency, gpu_solver, max_norm_err

pytestmark = pytest.mark.gpu

TOL = 1e-10
MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def cyl_case(pkg, oracle):
    return case_from_mesh(oracle, pkg.meshgen.single_cylinder(), h=-1.0, headings_deg=(0.0, 45.0))


@pytest.fixture(scope="module")
def config1(oracle):
    return oracle.load_case(os.path.join(GOLDEN, "config1", "input"))


def _points(case, rng, nfluid=24, nsurf=24, ncent=8):
    """Panel centroids (on the body), points in the fluid around the bodies and on the free surface."""
    lo = case.xyz_p.min(axis=0)
    hi = case.xyz_p.max(axis=0)
    span = hi - lo
    cen = case.xyz_p[rng.choice(case.n, ncent, replace=False)]
    fl = np.column_stack([rng.uniform(lo[0] - span[0], hi[0] + span[0], nfluid),
                          rng.uniform(lo[1] - span[1] - 5, hi[1] + span[1] + 5, nfluid),
                          rng.uniform(lo[2], -0.2, nfluid)])
    # keep the fluid points outside the hulls: shift those inside a cylinder's bounding box sideways
    fl[:, 1] += np.where(np.abs(fl[:, 1] - 0.5 * (lo[1] + hi[1])) < 0.6 * span[1] + 1, 1.2 * span[1] + 6, 0)
    fs = np.column_stack([rng.uniform(lo[0] - 3 * span[0], hi[0] + 3 * span[0], nsurf),
                          rng.uniform(hi[1] + 1.0, hi[1] + 4 * span[1] + 10, nsurf), np.zeros(nsurf)])
    return np.vstack([cen, fl, fs])


def _oracle_pot(oracle, case, pts, w, mx, isol=1):
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, w)
    betas = np.radians(case.ctl.headings)
    return oracle.field_potential(case, pts, v, wk, w1, wvn, betas, mx, isol=isol)


@pytest.mark.parametrize("precision", [0, 1])
def test_field_points_deep_match_oracle(pkg, oracle, cyl_case, precision):
    s = gpu_solver(pkg, cyl_case, precision)
    w = 0.9
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, w)
    pts = _points(cyl_case, np.random.default_rng(5))
    got = s.field_points(pts, kind=0, isol=1)
    ref = _oracle_pot(oracle, cyl_case, pts, w, mx)
    tol = TOL if precision == 0 else MIXED_TOL
    assert got.shape == ref.shape == (len(pts), 6 + 2)
    assert max_norm_err(got, ref) < tol
    for c in range(got.shape[1]):
        assert max_norm_err(got[:, c], ref[:, c]) < tol * 10
    # pressure = i w rho pot, elevation = i w / g pot
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, w, -1.0)
    prs = s.field_points(pts, kind=1, isol=1)
    elv = s.field_points(pts, kind=2, isol=1)
    assert np.allclose(prs, 1j * w1 * 1000.0 * got, rtol=1e-13, atol=0)
    assert np.allclose(elv, 1j * w1 / 9.80665 * got, rtol=1e-13, atol=0)
    # isol = 2 leaves out the incident potential
    g2 = s.field_points(pts, kind=0, isol=2)
    assert np.array_equal(g2[:, :6], got[:, :6])
    assert max_norm_err(g2, _oracle_pot(oracle, cyl_case, pts, w, mx, isol=2)) < tol
    s.close()


def test_centroids_reproduce_solved_potential(pkg, cyl_case):
    """At the collocation points the field potential is the solved potential."""
    s = gpu_solver(pkg, cyl_case, 0)
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, 1.3)
    got = s.field_points(cyl_case.xyz_p, kind=0, isol=2)
    assert max_norm_err(got, mx) < 1e-9
    s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_field_points_chunked(pkg, oracle, cyl_case, precision):
    """More points than one 2048-row chunk (the second chunk has an odd row count)."""
    s = gpu_solver(pkg, cyl_case, precision)
    w = 0.6
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, cyl_case, w)
    g = np.linspace(-60.0, 60.0, 47)
    X, Y = np.meshgrid(g, g, indexing="ij")
    pts = np.column_stack([X.ravel(), Y.ravel() + 0.37, np.zeros(X.size)])
    pts = pts[np.hypot(pts[:, 0], pts[:, 1]) > 6.0][:2191]
    assert len(pts) > 2048 and (len(pts) - 2048) % 2 == 1
    got = s.field_points(pts, kind=2, isol=1)
    ref = _oracle_pot(oracle, cyl_case, pts, w, mx)
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, w, -1.0)
    assert max_norm_err(got, 1j * w1 / 9.80665 * ref) < (TOL if precision == 0 else MIXED_TOL)
    s.close()


def test_field_points_finite_depth_multibody(pkg, oracle, config1):
    s = gpu_solver(pkg, config1, 0)
    w = config1.ctl.wvnb[1]
    amas, bdmp, exfc, mx = gpu_frequency(pkg, s, config1, w)
    pts = _points(config1, np.random.default_rng(11), nfluid=12, nsurf=12, ncent=6)
    got = s.field_points(pts, kind=0, isol=1)
    assert got.shape == (len(pts), 6 * config1.nbody + len(config1.ctl.headings))
    ref = _oracle_pot(oracle, config1, pts, w, mx)
    with oracle.use_library(oracle.build_fma_variant()):
        alt = _oracle_pot(oracle, config1, pts, w, mx)
    spread = max_norm_err(alt, ref)
    assert max_norm_err(got, ref) < max(10.0 * spread, TOL)
    s.close()


def test_field_points_need_a_solve(pkg, cyl_case):
    s = gpu_solver(pkg, cyl_case, 0)
    with pytest.raises(RuntimeError):
        s.field_points(np.zeros((1, 3)))
    s.close()


def test_field_points_plain_tensor_core_products_match_oracle(pkg, oracle):
    """Three cylinders (1536 panels, deep water): from order 1024 the plain
    form's products S W - A X run as exact digit products on the tensor
    cores (lu_tensor != 0), held to the same 1e-10 against the oracle and
    within rounding of the FP64-pipe products (lu_tensor 0)."""
    case = case_from_mesh(oracle, pkg.meshgen.three_cylinders(with_lid=False), h=-1.0, headings_deg=(0.0, 60.0))
    assert case.n >= 1024
    w = 1.1
    pts = _points(case, np.random.default_rng(9), nfluid=16, nsurf=16, ncent=8)
    got = {}
    for lu_tensor in (2, 0):
        s = gpu_solver(pkg, case, 0, lu_tensor=lu_tensor)
        amas, bdmp, exfc, mx = gpu_frequency(pkg, s, case, w)
        got[lu_tensor] = (s.field_points(pts, kind=0, isol=1), mx.copy())
        s.close()
    ref = _oracle_pot(oracle, case, pts, w, got[2][1])
    assert max_norm_err(got[2][0], ref) < TOL
    assert max_norm_err(got[2][0], got[0][0]) < TOL
