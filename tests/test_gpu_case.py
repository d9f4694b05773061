"""A whole HAMS run on the GPU from the reference's own input decks
(hg_case_run): the result files against the files the reference ships
(pinned frequencies, rules of test_case_io.py) and, for every frequency,
against the same writer fed the oracle's results (ALL_FREQ_FLOOR of each
file's largest entry: the finite-depth Green function's extrapolated series
make both results rounding-dependent, and with irregular-frequency removal
the normal equations amplify that to 2e-5 at some frequencies of these decks,
measured between two equally valid FP64 evaluations).  Single-body
field points: PressureElevation.6p against the oracle's field potential put
through WamitNondimens (src/PressureElevation.f90:336-385), restated below."""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import compare_result_file
from test_case_io import FLOOR, NPER_EXPECTED, PINNED, SKIP, expected_files, scale_rule

pytestmark = pytest.mark.gpu

ALL_FREQ_FLOOR = {"config1": 1e-6, "example5": 1e-4, "example3": 1e-4}


@pytest.mark.parametrize("name", ["config1", "example5", "example3"])
def test_case_run_matches_shipped_and_oracle_files(pkg, oracle, name, tmp_path):
    d = os.path.join(GOLDEN, name, "input")
    c = pkg.hamsgpu.Case(d)
    gpu_dir = os.path.join(tmp_path, "gpu")
    c.run(gpu_dir, precision=pkg.hamsgpu.HG_PREC_FP64, nslots=2)
    # shipped files, pinned frequencies
    nf = PINNED[name]
    for exp_path, sub, fname in expected_files(name):
        with open(exp_path) as f:
            n_exp = len(f.read().splitlines())
        if fname == "Hydrostat.hst":
            nl = None
        elif fname.endswith(".rao"):
            nl = None if nf == NPER_EXPECTED[name] else nf
        else:
            nl = None if nf == c.info["nper"] == NPER_EXPECTED[name] else n_exp // NPER_EXPECTED[name] * nf
        if (name, fname) in SKIP:
            continue
        rule = scale_rule(os.path.dirname(exp_path), fname, nl)
        rule.setdefault("floor", FLOOR[name])
        compare_result_file(os.path.join(gpu_dir, sub, fname), exp_path, nlines=nl, **rule)
    # every frequency against the oracle's results through the same writer
    case = oracle.load_case(d)
    freqs = case.ctl.wvnb if name != "example5" else case.ctl.wvnb[:4]
    res = [oracle.solve_frequency(case, w) for w in freqs]
    ora_dir = os.path.join(tmp_path, "oracle")
    amas = np.array([r.amas for r in res])
    bdmp = np.array([r.bdmp for r in res])
    exfc = np.array([r.exfc for r in res])
    pad = c.info["nper"] - len(freqs)
    if pad:
        amas = np.concatenate([amas, np.repeat(amas[-1:], pad, axis=0)])
        bdmp = np.concatenate([bdmp, np.repeat(bdmp[-1:], pad, axis=0)])
        exfc = np.concatenate([exfc, np.repeat(exfc[-1:], pad, axis=0)])
    c.write(ora_dir, amas, bdmp, exfc)
    nper = c.info["nper"]
    for sub, fname in [("Hams_format", f"{s}{k}.txt") for s in ("OAMASS", "ODAMPING", "OEXFOR") for k in range(1, 7)] + \
                      [("Wamit_format", "AmssDamp.1"), ("Wamit_format", "ExcForce.3"), ("Wamit_format", "Motion.4"),
                       ("Wamit_format", "Hydrostat.hst")]:
        got, ref = os.path.join(gpu_dir, sub, fname), os.path.join(ora_dir, sub, fname)
        with open(ref) as f:
            n_ref = len(f.read().splitlines())
        nl = None if fname == "Hydrostat.hst" else n_ref // nper * len(freqs)
        rule = scale_rule(os.path.join(ora_dir, sub), fname, nl)
        rule["floor"] = max(rule.get("floor", 0.0), ALL_FREQ_FLOOR[name])
        compare_result_file(got, ref, nlines=nl, **rule)
    c.close()


def _nondim(vcp, pressure, diffraction, md, special, w1, refl, rho=1000.0, g=9.80665):
    """WamitNondimens (src/PressureElevation.f90:336-385), AMP = 1."""
    nfac = (rho if special else rho * g) if pressure else 1.0
    if diffraction:
        r = vcp / nfac
    else:
        mexp = 0 if md <= 3 else 1
        r = vcp / nfac / refl ** (mexp + 1) if special else vcp / nfac * (-1j * w1) / refl ** mexp
    r = np.where(np.abs(r) < 1e-15, 0.0, r)
    return (-r.imag - 1j * r.real) if diffraction else (r.real - 1j * r.imag)


def test_case_run_field_points_file(pkg, oracle, tmp_path):
    """example5 with two frequencies and four field points (two below the
    free surface: pressure; two on it: elevation)."""
    src = os.path.join(GOLDEN, "example5", "input")
    d = os.path.join(tmp_path, "deck")
    shutil.copytree(src, d)
    pts = np.array([[30.0, 5.0, -4.0], [-12.0, 25.0, -1.5], [40.0, -20.0, 0.0], [0.0, 60.0, 0.0]])
    with open(os.path.join(d, "ControlFile.in")) as f:
        lines = f.read().split("\n")
    out = []
    for ln in lines:
        if ln.startswith("    Number_of_frequencies"):
            ln = ln.replace("-10", " -2")
        if ln.startswith("    Number_of_headings"):
            ln = ln.replace("-36", " -3")
        if ln.startswith("    Number_of_field_points"):
            out.append(ln[:27] + "%16d" % len(pts))
            out += ["    %12.4f %12.4f %12.4f    Global_coords_point_%d" % (p[0], p[1], p[2], k + 1)
                    for k, p in enumerate(pts)]
            continue
        out.append(ln)
    with open(os.path.join(d, "ControlFile.in"), "w") as f:
        f.write("\n".join(out))
    c = pkg.hamsgpu.Case(d)
    assert c.info["nfp"] == 4 and c.info["nper"] == 2 and c.info["nbeta"] == 3
    c.run(os.path.join(tmp_path, "out"), precision=pkg.hamsgpu.HG_PREC_FP64, nslots=1)
    with open(os.path.join(tmp_path, "out", "Wamit_format", "PressureElevation.6p")) as f:
        rows = [ln.split() for ln in f.read().splitlines()]
    case = oracle.load_case(d)
    heads = case.ctl.headings
    betas = np.radians(heads)
    below = np.abs(pts[:, 2]) > 1e-6
    nrow = 0
    for w in case.ctl.wvnb:
        v, wk, w1, wvn = oracle.wave_properties(case.ctl, w)
        r = oracle.solve_frequency(case, w)
        pot = oracle.field_potential(case, pts, v, wk, w1, wvn, betas, r.mxpot, isol=case.ctl.isol)
        vcp = np.where(below[:, None], 1j * w1 * 1000.0 * pot, 1j * w1 / 9.80665 * pot)
        scale = np.abs(vcp).max()
        for p in np.flatnonzero(below):   # radiation lines: points below the free surface only
            row = rows[nrow]; nrow += 1
            assert int(row[1]) == p + 1 and abs(float(row[0]) - w1) < 1e-6
            for md in range(1, 7):
                z = _nondim(vcp[p, md - 1], True, False, md, False, w1, case.ctl.refl)
                got = float(row[2 * md]) + 1j * float(row[2 * md + 1])
                assert abs(got - z) <= 1e-6 * max(abs(z), 1e-12) + 1e-6 * scale * w1 / 9806.65
        zs = {(p, ib): _nondim(vcp[p, 6 + ib], bool(below[p]), True, 0, False, w1, case.ctl.refl)
              for ib in range(len(heads)) for p in range(len(pts))}
        zmax = max(abs(z) for z in zs.values())
        for ib, b in enumerate(heads):
            for p in range(len(pts)):
                row = rows[nrow]; nrow += 1
                z = zs[(p, ib)]
                tol = 2e-6 * abs(z) + 1e-6 * zmax
                assert int(row[2]) == p + 1 and abs(float(row[1]) - b) < 1e-9
                got = float(row[5]) + 1j * float(row[6])
                assert abs(got - z) <= tol, (p, b, got, z)
                assert abs(float(row[3]) - abs(z)) <= tol
    assert nrow == len(rows)
    c.close()


def test_case_run_zero_and_infinite_frequency_entries(pkg, tmp_path):
    """0_inf_frequency_limits = 1 adds the zero- and infinite-frequency limits
    as the first two entries (CalWaveProperts, src/ImplementSubs.f90:45-70):
    they write added mass only in AmssDamp.1 and no ExcForce.3 lines, and the
    regular entries are those of the same deck without them."""
    src = os.path.join(GOLDEN, "config1", "input")
    d = os.path.join(tmp_path, "deck")
    shutil.copytree(src, d)
    with open(os.path.join(d, "ControlFile.in")) as f:
        lines = f.read().split("\n")
    for i, ln in enumerate(lines):
        if "0_inf_frequency_limits" in ln:
            lines[i] = ln[:27] + "%16d" % 1
    with open(os.path.join(d, "ControlFile.in"), "w") as f:
        f.write("\n".join(lines))
    c = pkg.hamsgpu.Case(d)
    assert c.info["sybo"] == 1 and c.info["nper"] == 5
    freq = c.arrays()["freq"]
    assert list(freq[0, :4]) == [0.0, 0.0, 0.0, -1.0] and list(freq[1, :4]) == [-1.0, -1.0, -1.0, 0.0]
    c.run(os.path.join(tmp_path, "with"), precision=pkg.hamsgpu.HG_PREC_FP64, nslots=2)
    ref = pkg.hamsgpu.Case(src)
    ref.run(os.path.join(tmp_path, "without"), precision=pkg.hamsgpu.HG_PREC_FP64, nslots=2)
    nd = 18
    with open(os.path.join(tmp_path, "with", "Wamit_format", "AmssDamp.1")) as f:
        am = f.read().splitlines()
    with open(os.path.join(tmp_path, "without", "Wamit_format", "AmssDamp.1")) as f:
        am0 = f.read().splitlines()
    assert len(am) == 5 * nd * nd and len(am0) == 3 * nd * nd
    assert all(len(ln.split()) == 4 for ln in am[:2 * nd * nd])
    assert am[2 * nd * nd:] == am0
    with open(os.path.join(tmp_path, "with", "Wamit_format", "ExcForce.3")) as f:
        ex = f.read()
    with open(os.path.join(tmp_path, "without", "Wamit_format", "ExcForce.3")) as f:
        assert ex == f.read()
    with open(os.path.join(tmp_path, "with", "Hams_format", "OAMASS3.txt")) as f:
        oa = f.read().splitlines()
    assert len(oa) == 5 * 9 and oa[0].startswith("  0.000   0.000") and oa[9].startswith(" -1.000  -1.000")
    a = np.array([[float(t) for t in ln.split()] for ln in oa])
    assert np.all(np.isfinite(a))
    c.close()
    ref.close()


def _vinp(x, y, z, beta, wk, w1, h, g=9.80665):
    """VINP (src/PatclVelct.f90:42-76), AMP = 1, wave origin at 0."""
    e = np.exp(1j * wk * (x * np.cos(beta) + y * np.sin(beta)))
    if h < 0 or h > 500:
        return -g / w1 * np.exp(wk * z) * e
    return -w1 / (wk * np.sinh(wk * h)) * np.cosh(wk * (z + h)) * e


@pytest.mark.parametrize("separate", [False, True])
def test_case_run_field_points_multibody(pkg, oracle, tmp_path, separate):
    """config1 (three bodies, h = 70 m) with four field points: the WAMIT files
    of OutputPressureElevation_RadiationMulti / _DiffractionMulti /
    _IncidenceMulti (src/PressureElevationMulti.f90:407-587), combined or, with
    the control file's separate-files flag (src/InputFiles.f90:204-220), one
    radiation file per body and one diffraction file."""
    src = os.path.join(GOLDEN, "config1", "input")
    d = os.path.join(tmp_path, "deck")
    shutil.copytree(src, d)
    pts = np.array([[20.0, 30.0, -5.0], [-25.0, 60.0, -2.0], [15.0, -30.0, 0.0], [-40.0, 120.0, 0.0]])
    with open(os.path.join(d, "ControlFile.in")) as f:
        lines = f.read().split("\n")
    out, skip = [], False
    for ln in lines:
        if ln.startswith("    Number_of_field_points"):
            out.append(ln[:27] + "%16d" % len(pts))
            out += ["    %12.4f %12.4f %12.4f" % tuple(p) for p in pts]
            out.append("   #End Definition of Pressure and/or Elevation")
            out.append("   #Start Definition of WAMIT output")
            flag = "    Separate_wamit_diffraction_radiation_files"
            out.append(flag + " " * (50 - len(flag)) + "%16d" % (1 if separate else 0))
            skip = True
            continue
        if skip and ln.strip().startswith("#End Definition of Pressure"):
            skip = False
            continue
        out.append(ln)
    with open(os.path.join(d, "ControlFile.in"), "w") as f:
        f.write("\n".join(out))
    c = pkg.hamsgpu.Case(d)
    assert c.info["nfp"] == 4 and c.info["nbody"] == 3
    c.run(os.path.join(tmp_path, "out"), precision=pkg.hamsgpu.HG_PREC_FP64, nslots=1)
    wd = os.path.join(tmp_path, "out", "Wamit_format")

    def rows(name):
        with open(os.path.join(wd, name)) as f:
            return f.read().splitlines()

    comb = None if separate else rows("PressureElevation.6p")
    rad = [rows("PressureElevationRadiation_%d.6p" % (b + 1)) for b in range(3)] if separate else None
    dif = rows("PressureElevationDiffraction.6p") if separate else None
    inc = rows("PressureElevationIncidence.6p")
    assert os.path.exists(os.path.join(wd, "PressureElevation.6p")) == (not separate)
    case = oracle.load_case(d)
    heads = case.ctl.headings
    betas = np.radians(heads)
    below = np.abs(pts[:, 2]) > 1e-6
    ic = ir = idf = 0
    irb = [0, 0, 0]
    for w in case.ctl.wvnb:
        v, wk, w1, wvn = oracle.wave_properties(case.ctl, w)
        r = oracle.solve_frequency(case, w)
        pot = oracle.field_potential(case, pts, v, wk, w1, wvn, betas, r.mxpot, isol=case.ctl.isol)
        vcp = np.where(below[:, None], 1j * w1 * 1000.0 * pot, 1j * w1 / 9.80665 * pot)
        zr = np.array([[_nondim(vcp[p, q], bool(below[p]), False, q % 6 + 1, False, w1, case.ctl.refl)
                        for q in range(18)] for p in range(len(pts))])
        zmax = np.abs(zr).max()
        for p in range(len(pts)):
            for b in range(3):
                if separate:
                    t = rad[b][irb[b]].split(); irb[b] += 1
                    assert int(t[1]) == p + 1 and abs(float(t[0]) - w1) < 1e-6
                    vals = t[2:]
                else:
                    ln = comb[ic]; ic += 1
                    if b == 0:
                        t = ln.split()
                        assert int(t[1]) == p + 1 and abs(float(t[0]) - w1) < 1e-6
                        vals = t[2:]
                    else:
                        assert ln[:24] == " " * 24
                        vals = ln.split()
                assert len(vals) == 12
                for md in range(6):
                    z = zr[p, 6 * b + md]
                    got = float(vals[2 * md]) + 1j * float(vals[2 * md + 1])
                    assert abs(got - z) <= 1e-6 * abs(z) + 1e-6 * zmax, (p, b, md, got, z)
        zd = np.array([[_nondim(vcp[p, 18 + ib], bool(below[p]), True, 0, False, w1, case.ctl.refl)
                        for ib in range(len(heads))] for p in range(len(pts))])
        zdmax = np.abs(zd).max()
        for ib, b in enumerate(heads):
            for p in range(len(pts)):
                if separate:
                    t = dif[idf].split(); idf += 1
                else:
                    t = comb[ic].split(); ic += 1
                assert len(t) == 5 and int(t[2]) == p + 1 and abs(float(t[1]) - b) < 1e-9
                got = float(t[3]) + 1j * float(t[4])
                assert abs(got - zd[p, ib]) <= 2e-6 * abs(zd[p, ib]) + 1e-6 * zdmax
            for p in range(len(pts)):
                t = inc[ir].split(); ir += 1
                pi = _vinp(pts[p, 0], pts[p, 1], pts[p, 2], np.radians(b), wk, w1, case.ctl.h)
                vi = 1j * w1 * 1000.0 * pi if below[p] else 1j * w1 / 9.80665 * pi
                z = _nondim(vi, bool(below[p]), True, 0, False, w1, case.ctl.refl)
                assert len(t) == 7 and int(t[2]) == p + 1
                assert abs(float(t[5]) + 1j * float(t[6]) - z) <= 2e-6 * abs(z) + 1e-12
                assert abs(float(t[3]) - abs(z)) <= 2e-6 * abs(z) + 1e-12
    assert ir == len(inc)
    if separate:
        assert idf == len(dif) and all(irb[b] == len(rad[b]) for b in range(3))
    else:
        assert ic == len(comb)
    c.close()
