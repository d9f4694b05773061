"""Serving: continuous batching of frequency-solve requests (hg_server_*).

Requests of different meshes, depths, frequency lists and headings are
submitted together; the server runs their frequencies on several solve slots
at once.  Every result must be identical to the same request solved alone on
a single context (the kernels are deterministic, so the comparison is
exact).  The admission test gives a budget that fits one request at a time
and checks that the reserved device memory never exceeded it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(pkg):
    hg = pkg.hamsgpu
    mg = pkg.meshgen
    specs = [
        (mg.single_cylinder(), -1.0, np.linspace(0.4, 1.8, 5), [0.0, 0.8], 0),
        (mg.three_cylinders(with_lid=False), 40.0, np.linspace(0.5, 1.5, 3), [0.0, 0.5, 1.2], 0),
        (mg.three_cylinders(with_lid=True), -1.0, np.array([0.7, 1.3]), [0.3], 1),
        (mg.single_cylinder(), 70.0, np.linspace(0.3, 2.2, 6), [0.0], 0),
    ]
    out = []
    for mesh, h, freqs, betas, irsp in specs:
        vals = [hg.wave_properties(3, float(w), h) for w in freqs]
        v = np.array([x[0] for x in vals]); wk = np.array([x[1] for x in vals]); w1 = np.array([x[2] for x in vals])
        wvn = np.stack([x[3] for x in vals]) if h > 0 else None
        out.append((mesh, h, v, wk, w1, wvn, np.array(betas), irsp))
    return out


def _alone(pkg, req):
    hg = pkg.hamsgpu
    mesh, h, v, wk, w1, wvn, betas, irsp = req
    s = hg.Solver(precision=hg.HG_PREC_MIXED)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges,
               mesh.lid_xyz_p if irsp == 1 else None)
    res = []
    for i in range(len(v)):
        a, b, f, _ = s.solve_frequency(v[i], wk[i], w1[i], h, None if wvn is None else wvn[i], betas, irsp=irsp,
                                       want_potentials=False)
        res.append((a.copy(), b.copy(), f.copy()))
    s.close()
    return res


@pytest.fixture(scope="module")
def requests_and_alone(pkg):
    reqs = _requests(pkg)
    return reqs, [_alone(pkg, r) for r in reqs]


def _check_same(got, ref):
    amas, bdmp, exfc = got[0], got[1], got[2]
    for i, (a, b, f) in enumerate(ref):
        np.testing.assert_array_equal(amas[i], a)
        np.testing.assert_array_equal(bdmp[i], b)
        np.testing.assert_array_equal(exfc[i], f)


def test_mix_equals_alone(pkg, requests_and_alone):
    reqs, ref = requests_and_alone
    srv = pkg.hamsgpu.Server(nslots=3, budget_bytes=100e9)
    tickets = [srv.submit(r[0], r[1], r[2], r[3], r[4], r[5], r[6], irsp=r[7]) for r in reqs]
    for t, rr in zip(tickets, ref):
        got = srv.wait(t)
        _check_same(got, rr)
        assert got[3] > 0
    st = srv.stats()
    assert st["requests_done"] == len(reqs)
    assert st["solves_done"] == sum(len(r[2]) for r in reqs)
    assert st["max_admitted"] >= 2  # the requests ran in the mix
    assert st["reserved_bytes"] == 0
    # their work overlapped on the device: the CUDA-event intervals of solves of
    # two different requests intersect
    tl = srv.timeline()
    assert len(tl) == st["solves_done"]
    assert np.all(tl[:, 3] > tl[:, 2])
    overlap = 0.0
    for a in range(len(tl)):
        for b in range(len(tl)):
            if tl[a, 0] != tl[b, 0]:
                overlap = max(overlap, min(tl[a, 3], tl[b, 3]) - max(tl[a, 2], tl[b, 2]))
    assert overlap > 0.0, tl
    srv.close()


def test_admission_budget(pkg, requests_and_alone):
    hg = pkg.hamsgpu
    reqs, ref = requests_and_alone
    same = [reqs[0], reqs[3]]  # two single-cylinder requests (384 panels)
    nslots = 2
    one = max(min(nslots, len(r[2])) * hg.solve_footprint(hg.HG_PREC_MIXED, r[0].n, 0, 1, len(r[6])) for r in same)
    budget = 1.5 * one + 1e6  # room for one request at a time
    srv = hg.Server(nslots=nslots, budget_bytes=budget)
    tickets = [srv.submit(r[0], r[1], r[2], r[3], r[4], r[5], r[6], irsp=r[7]) for r in same]
    for t, rr in zip(tickets, [ref[0], ref[3]]):
        _check_same(srv.wait(t), rr)
    st = srv.stats()
    assert st["max_admitted"] == 1
    assert st["peak_reserved_bytes"] <= budget
    # a request larger than the whole budget is refused at submission
    big = reqs[1]
    with pytest.raises(hg.HamsGpuError):
        srv.submit(big[0], big[1], big[2], big[3], big[4], big[5], big[6])
    srv.close()


def test_iterative_hmatrix_requests_equal_alone(pkg):
    """The iterative solver with the reference's H-matrix (solver 2,
    hmatrix 1) through the server: results equal to the same request on its
    own context, and the admission reserves the H-matrix's blocks on top of
    the dense GMRES's memory."""
    hg = pkg.hamsgpu
    mesh = pkg.meshgen.three_cylinders(with_lid=False)
    vals = [hg.wave_properties(3, w, -1.0) for w in (0.8, 1.3)]
    v = np.array([x[0] for x in vals]); wk = np.array([x[1] for x in vals]); w1 = np.array([x[2] for x in vals])
    betas = np.array([0.0, 0.6])
    s = hg.Solver(precision=hg.HG_PREC_MIXED, solver=2, hmatrix=1)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    ref = []
    for i in range(len(v)):
        a, b, f, _ = s.solve_frequency(v[i], wk[i], w1[i], -1.0, None, betas, want_potentials=False)
        ref.append((a.copy(), b.copy(), f.copy()))
    s.close()
    reserved = {}
    for hm in (1, 0):
        srv = hg.Server(nslots=2, budget_bytes=150e9, solver=2, hmatrix=hm)
        got = srv.wait(srv.submit(mesh, -1.0, v, wk, w1, None, betas))
        if hm:
            _check_same(got, ref)
        reserved[hm] = srv.stats()["peak_reserved_bytes"]
        srv.close()
    assert reserved[1] > reserved[0]
