"""The oracle against the reference's own golden outputs (CPU only).

config1  : the reference integration test (3 bodies, h = 70 m): every
           printed 5-significant-digit added mass, damping and excitation
           value is reproduced.
example5 : single body with waterplane lid (IRSP = 1): WAMIT-format
           AmssDamp.1 / ExcForce.3 (7 significant digits) reproduced to
           2e-6 of the largest entry.
example3 : two bodies with lids and a generalized mode: first frequency
           of AmssDamp.1 to 1e-5.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _close_to_print(got, printed, sig=5, floor=0.0):
    """|got - printed| within half a unit of the last printed digit (+1% slack),
    plus an absolute floor for entries far below the largest one (the
    reference stores Green values in single precision, GRN_KIND = 4, so
    couplings several orders below the peak carry that rounding)."""
    return np.abs(got - printed) <= 0.505 * 10.0 ** (-(sig - 1)) * np.abs(printed) + floor + 1e-30


@pytest.fixture(scope="module")
def config1_results(oracle):
    case = oracle.load_case(os.path.join(GOLDEN, "config1", "input"))
    return case, [oracle.solve_frequency(case, w) for w in case.ctl.wvnb]


def test_config1_added_mass_damping(oracle, config1_results):
    case, res = config1_results
    nb = case.nbody
    for name, attr in (("OAMASS", "amas"), ("ODAMPING", "bdmp")):
        for md1 in range(6):
            E = oracle.read_hams_rows(os.path.join(GOLDEN, "config1", "expected", f"{name}{md1 + 1}.txt"))
            assert E.shape == (len(res) * nb * nb, 8)
            for kk, r in enumerate(res):
                for bm in range(nb):
                    for bn in range(nb):
                        row = E[kk * nb * nb + bm * nb + bn]
                        assert abs(row[1] - r.w1) < 1e-3
                        full = getattr(r, attr)
                        got = full[6 * bm + md1, 6 * bn:6 * bn + 6]
                        floor = 5e-7 * np.abs(full).max()
                        assert np.all(_close_to_print(got, row[2:], 5, floor)), (name, md1, kk, bm, bn, got, row[2:])


def test_config1_excitation(oracle, config1_results):
    case, res = config1_results
    nb, nbeta = case.nbody, len(case.ctl.headings)
    for md in range(6):
        E = oracle.read_hams_rows(os.path.join(GOLDEN, "config1", "expected", f"OEXFOR{md + 1}.txt"))
        for kk, r in enumerate(res):
            for ii in range(nbeta):
                for bm in range(nb):
                    row = E[kk * nbeta * nb + ii * nb + bm]
                    got = r.exfc[ii, 6 * bm + md]
                    # E14.6 in EFORCE: 6 significant digits
                    floor = 5e-7 * np.abs(r.exfc).max()
                    assert _close_to_print(got.real, row[2], 6, floor) and _close_to_print(got.imag, row[3], 6, floor), \
                        (md, kk, ii, bm, got, row[2:4])


def _wamit(oracle, name, case, nfreq, tol_a, tol_f):
    am = oracle.read_hams_rows(os.path.join(GOLDEN, name, "expected", "AmssDamp.1"))
    ex = oracle.read_hams_rows(os.path.join(GOLDEN, name, "expected", "ExcForce.3"))
    nd = 6 * case.nbody
    heads = case.ctl.headings
    nfreq = min(nfreq, len(am) // (nd * nd))
    for kk in range(nfreq):
        r = oracle.solve_frequency(case, case.ctl.wvnb[kk])
        A = np.zeros((nd, nd)); B = np.zeros((nd, nd))
        for row in am[kk * nd * nd:(kk + 1) * nd * nd]:
            A[int(row[1]) - 1, int(row[2]) - 1] = row[3]
            B[int(row[1]) - 1, int(row[2]) - 1] = row[4]
        ga, gb = r.amas / oracle.RHO, r.bdmp / (oracle.RHO * r.w1)
        assert np.abs(ga - A).max() / np.abs(A).max() < tol_a
        assert np.abs(gb - B).max() / np.abs(B).max() < tol_a
        F = np.zeros((len(heads), nd), dtype=complex)
        for row in ex[kk * len(heads) * nd:(kk + 1) * len(heads) * nd]:
            ib = int(round((row[1] - heads[0]) / (heads[1] - heads[0])))
            F[ib, int(row[2]) - 1] = -row[6] - 1j * row[5]
        gf = r.exfc / (oracle.RHO * oracle.G)
        assert np.abs(gf - F).max() / np.abs(F).max() < tol_f


def test_example5_irr_wamit(oracle):
    case = oracle.load_case(os.path.join(GOLDEN, "example5", "input"))
    assert case.nl == 383 and case.ctl.irsp == 1
    _wamit(oracle, "example5", case, 3, 2e-6, 2e-6)


def test_example3_multibody_irr_genmode_wamit(oracle):
    case = oracle.load_case(os.path.join(GOLDEN, "example3", "input"))
    assert case.nbody == 2 and case.nl > 0
    _wamit(oracle, "example3", case, 1, 1e-5, 1e-5)


def test_oracle_edge_cases(oracle):
    """Zero- and infinite-frequency limits (V = 0, V = -1) give the Rankine-only
    Green function (InfGreen_Appr.f90:130-157, FinGreen3D.f90:100-148)."""
    import ctypes
    L = oracle.lib()
    o8 = np.zeros(8)
    dp = ctypes.POINTER(ctypes.c_double)
    for v in (0.0, -1.0):
        for h in (-1.0, 30.0):
            wvn = np.zeros(200)
            L.or_green_point(1.0, 2.0, -3.0, 4.0, 5.0, -1.0, v, wvn.ctypes.data_as(dp), 200, h, 0,
                             o8.ctypes.data_as(dp))
            r = np.sqrt(9 + 9 + 4.0)
            r1 = np.sqrt(9 + 9 + 16.0)
            assert abs(o8[0] - ((1 / r1 if v == 0 else -1 / r1) + 1 / r)) < 1e-14
            assert np.all(o8[1::2] == 0.0)
