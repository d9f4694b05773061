"""Frequency sweeps on concurrent solve slots (hg_solve_sweep).

The reference loops over frequencies one at a time (src/HAMS_Prog.f90:255-304,
:613-704); every frequency is independent.  The sweep runs several
frequency-solves at once on separate slots (own buffers and stream) that
share the GPU.  Each result must be the same whether its frequency ran alone
on a single context or in the mix with others: the kernels are deterministic
(no floating-point atomics), so the comparison is exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(hg, freqs, h):
    vals = [hg.wave_properties(3, float(w), h) for w in freqs]
    v = np.array([x[0] for x in vals]); wk = np.array([x[1] for x in vals]); w1 = np.array([x[2] for x in vals])
    wvn = np.stack([x[3] for x in vals]) if h > 0 else None
    return v, wk, w1, wvn


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("h", [-1.0, 40.0])
def test_sweep_matches_one_by_one(pkg, precision, h):
    hg = pkg.hamsgpu
    mesh = pkg.meshgen.single_cylinder()
    freqs = np.linspace(0.3, 2.0, 7)
    betas = np.array([0.0, 0.7])
    v, wk, w1, wvn = _inputs(hg, freqs, h)
    alone = []
    s = hg.Solver(precision=precision)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    for i in range(len(freqs)):
        a, b, f, x = s.solve_frequency(v[i], wk[i], w1[i], h, None if wvn is None else wvn[i], betas)
        alone.append((a.copy(), b.copy(), f.copy(), x.copy()))
    for nslots in (1, 3):
        am, bm, fm, lat, xm = s.solve_sweep(v, wk, w1, h, wvn, betas, nslots=nslots, want_potentials=True)
        assert lat.shape == (len(freqs),) and np.all(lat > 0)
        for i, (a, b, f, x) in enumerate(alone):
            np.testing.assert_array_equal(am[i], a)
            np.testing.assert_array_equal(bm[i], b)
            np.testing.assert_array_equal(fm[i], f)
            np.testing.assert_array_equal(xm[i], x)
    s.close()


def test_sweep_reports_errors(pkg):
    hg = pkg.hamsgpu
    mesh = pkg.meshgen.single_cylinder()
    s = hg.Solver(precision=0)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    v, wk, w1, _ = _inputs(hg, [0.5, 1.0], -1.0)
    with pytest.raises(hg.HamsGpuError):
        s.solve_sweep(v, wk, w1, -1.0, None, [0.0], nslots=17)
    # finite depth without dispersion roots is rejected before any work
    with pytest.raises(hg.HamsGpuError):
        s.solve_sweep(v, wk, w1, 40.0, None, [0.0], nslots=2)
    s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_sweep_after_mesh_change_matches_fresh_context(pkg, precision):
    """Slots keep their buffers across sweeps and take a new mesh in their own
    worker thread: a sweep after set_mesh with another mesh (and with more
    slots than before, so old and new slots mix) gives exactly what a fresh
    context gives on that mesh."""
    hg = pkg.hamsgpu
    m1 = pkg.meshgen.single_cylinder()
    m2 = pkg.meshgen.combine([pkg.meshgen.hemisphere(5.0, 24, 8)])
    freqs = np.linspace(0.4, 1.6, 5)
    betas = np.array([0.0, 0.9])
    v, wk, w1, _ = _inputs(hg, freqs, -1.0)

    def mesh_args(m):
        return (m.nodes, m.ncon, m.ncn, m.xyz_p, m.ds, m.pnsz, m.dxyz_p, m.body_ranges)

    fresh = hg.Solver(precision=precision)
    fresh.set_mesh(*mesh_args(m2))
    ref = fresh.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=1, want_potentials=True)
    fresh.close()
    s = hg.Solver(precision=precision)
    s.set_mesh(*mesh_args(m1))
    s.solve_sweep(v[:2], wk[:2], w1[:2], -1.0, None, betas, nslots=2)
    s.set_mesh(*mesh_args(m2))
    got = s.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=3, want_potentials=True)
    # back to the first mesh with fewer slots, then the second again with all of them
    s.set_mesh(*mesh_args(m1))
    s.solve_sweep(v[:1], wk[:1], w1[:1], -1.0, None, betas, nslots=1)
    s.set_mesh(*mesh_args(m2))
    again = s.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=3, want_potentials=True)
    s.close()
    for k in (0, 1, 2, 4):
        np.testing.assert_array_equal(got[k], ref[k])
        np.testing.assert_array_equal(again[k], ref[k])
