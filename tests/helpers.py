"""Test helpers bridging the oracle's case description and the GPU binding."""
import numpy as np


def max_norm_err(got, exp):
    """max |got - exp| / max |exp| (the max-normalised relative error)."""
    got = np.asarray(got)
    exp = np.asarray(exp)
    scale = np.abs(exp).max()
    return float(np.abs(got - exp).max() / (scale if scale > 0 else 1.0))


def case_from_mesh(oracle, mesh, h, headings_deg=(0.0,), isol=1, irsp=0, freqs=(1.0,)):
    starts = mesh.body_ranges[:, 0] - 1
    ends = mesh.body_ranges[:, 1]
    xr = [[0.0, 0.0, 0.0]] * len(starts)
    ctl = oracle.Control(h=h, sybo=0, inft=3, ouft=3, wvnb=list(freqs), nbody=len(starts), lcs=[],
                         headings=list(headings_deg), xr=xr, refl=1.0, isol=isol, irsp=irsp, nthread=0)
    lid = mesh.lid_xyz_p if irsp == 1 else np.zeros((0, 3))
    return oracle.Case(ctl, mesh.nodes, mesh.ncn.astype(np.int32), mesh.ncon.astype(np.int32), mesh.xyz_p, mesh.ds,
                       mesh.pnsz, mesh.dxyz_p, np.asarray(starts, dtype=np.int32), np.asarray(ends, dtype=np.int32),
                       lid)


def gpu_solver(pkg, case, precision=0, grn_kind=8, **kw):
    s = pkg.hamsgpu.Solver(precision=precision, grn_kind=grn_kind, **kw)
    ranges = np.stack([case.body_start + 1, case.body_end], axis=1)
    s.set_mesh(case.nodes, case.ncon, case.ncn, case.xyz_p, case.ds, case.pnsz, case.dxyz_p, ranges,
               case.lid_xyz_p if case.nl > 0 else None)
    return s


def gpu_frequency(pkg, solver, case, value, betas_deg=None):
    ctl = case.ctl
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(ctl.inft, value, ctl.h)
    if betas_deg is None:
        betas_deg = ctl.headings
    betas = np.array(betas_deg, dtype=np.float64) * np.pi / 180.0
    return solver.solve_frequency(v, wk, w1, ctl.h, wvn, betas, irsp=1 if case.nl > 0 else 0, isol=ctl.isol)


def _ulp(tok):
    """Unit in the last printed place of a Fortran-formatted number."""
    t = tok.upper()
    if "E" in t:
        mant, ex = t.split("E")
        dec = len(mant.split(".")[1]) if "." in mant else 0
        return 10.0 ** (int(ex) - dec)
    if "." in t:
        return 10.0 ** (-len(t.split(".")[1]))
    return 0.0


def file_values_max(path, first_value, nlines=None):
    """Largest magnitude among the fields from first_value on."""
    with open(path) as f:
        lines = f.read().splitlines()[:nlines]
    top = 0.0
    for ln in lines:
        for t in ln.split()[first_value:]:
            try:
                top = max(top, abs(float(t)))
            except ValueError:
                pass
    return top


def compare_result_file(got_path, exp_path, nlines=None, floor=1e-6, scale_by="column", first_value=0,
                        scale_value=None, phase=None, phase_unit=1.0, phase_pairs=None, phase_period=None,
                        skip_fields=()):
    """Compare two HAMS/WAMIT result files: the same number of lines (or the
    first nlines), every line of the same length (same edit descriptors), text
    tokens equal and numbers within one printed unit plus floor x the largest
    magnitude of their column (scale_by="column") or of all value columns of
    the file from field first_value on (scale_by="file"), or scale_value
    for those fields when given.  phase = (magnitude field, phase field):
    a phase is held to the angle that the floor of its magnitude's column
    subtends at that magnitude (times phase_unit per radian), since the
    phase of a near-zero complex number is rounding noise; phase_pairs does
    the same for several (magnitude, phase) field pairs, phase_period wraps
    phase differences (360 for [0, 360)); skip_fields are not compared
    (their width still is, through the line length).  Returns (worst excess,
    lines compared)."""
    with open(got_path) as f:
        got = f.read().splitlines()
    with open(exp_path) as f:
        exp = f.read().splitlines()
    if nlines is None:
        assert len(got) == len(exp), f"{got_path}: {len(got)} lines, expected {len(exp)}"
        nlines = len(exp)
    assert len(got) >= nlines and len(exp) >= nlines
    rows_g = [ln.split() for ln in got[:nlines]]
    rows_e = [ln.split() for ln in exp[:nlines]]
    ncol = max(len(r) for r in rows_e)
    scale = [0.0] * ncol
    for r in rows_e:
        for j, t in enumerate(r):
            try:
                scale[j] = max(scale[j], abs(float(t)))
            except ValueError:
                pass
    if scale_by == "file":
        top = max(scale[first_value:]) if ncol > first_value else 0.0
        if scale_value is not None:
            top = scale_value
        scale = [top if j >= first_value else scale[j] for j in range(ncol)]
    worst = 0.0
    for i, (lg, le, rg, re_) in enumerate(zip(got, exp, rows_g, rows_e)):
        assert len(lg) == len(le), f"{got_path}:{i + 1}: line length {len(lg)} != {len(le)}\n{lg}\n{le}"
        assert len(rg) == len(re_), f"{got_path}:{i + 1}: {len(rg)} fields != {len(re_)}"
        for j, (a, b) in enumerate(zip(rg, re_)):
            if j in skip_fields:
                continue
            try:
                x, y = float(a), float(b)
            except ValueError:
                assert a == b, f"{got_path}:{i + 1}: '{a}' != '{b}'"
                continue
            pairs = list(phase_pairs or []) + ([tuple(phase)] if phase is not None else [])
            magf = next((pm for pm, pp in pairs if pp == j), None)
            diff = abs(x - y)
            if magf is not None:
                mag = max(abs(float(re_[magf])), 1e-300)
                tol = 1.01 * max(_ulp(a), _ulp(b)) + 2.0 * phase_unit * floor * scale[magf] / mag
                if phase_period:
                    diff = min(diff, phase_period - diff)
            else:
                tol = 1.01 * max(_ulp(a), _ulp(b)) + floor * scale[j]
            excess = diff / tol if tol > 0 else (0.0 if x == y else float("inf"))
            assert excess <= 1.0, f"{got_path}:{i + 1} field {j + 1}: {a} vs {b} (tol {tol:.3g})\n{lg}\n{le}"
            worst = max(worst, excess)
    return worst, nlines


def rigid_body_matrices(mesh, rho=1000.0, g=9.80665):
    """Mass and hydrostatic restoring matrices (6 nbody square) of freely
    floating rigid bodies, from the hull panels alone (divergence theorem
    with the inward panel normals of the reference meshes): displaced
    volume V, centre of buoyancy, waterplane area and moments about each
    body's reference point (x, y of its panels' mean, z = 0).  The centre of
    gravity is put below the waterline at 1.5 z_b (so every body is stable)
    and the radii of gyration at 0.35 of the body's largest extent.  These
    stand in for the Hydrostatic.in decks of the reference (read by
    ReadHydroStatic, src/HydroStatic.f90) in the motion equations of
    SolveMotion (src/SolveMotion.f90:25-111)."""
    nb = len(mesh.body_ranges)
    M = np.zeros((6 * nb, 6 * nb))
    C = np.zeros((6 * nb, 6 * nb))
    for b, (f, l) in enumerate(mesh.body_ranges):
        sl = slice(f - 1, l)
        p = mesh.xyz_p[sl]
        nz = mesh.dxyz_p[sl, 2]
        ds = mesh.ds[sl]
        ref = np.array([p[:, 0].mean(), p[:, 1].mean(), 0.0])
        x, y, z = p[:, 0] - ref[0], p[:, 1] - ref[1], p[:, 2]
        vol = -np.sum(z * nz * ds)
        zb = -np.sum(0.5 * z * z * nz * ds) / vol
        awp = np.sum(nz * ds)
        sx, sy = np.sum(x * nz * ds), np.sum(y * nz * ds)
        ixx, iyy, ixy = np.sum(y * y * nz * ds), np.sum(x * x * nz * ds), np.sum(x * y * nz * ds)
        m = rho * vol
        zg = 1.5 * zb
        span = max(np.ptp(p[:, 0]), np.ptp(p[:, 1]), np.ptp(p[:, 2]))
        kg = 0.35 * span
        o = 6 * b
        Mb = np.diag([m, m, m, m * kg * kg, m * kg * kg, m * kg * kg])
        Mb[0, 4] = Mb[4, 0] = m * zg
        Mb[1, 3] = Mb[3, 1] = -m * zg
        Cb = np.zeros((6, 6))
        Cb[2, 2] = rho * g * awp
        Cb[2, 3] = Cb[3, 2] = rho * g * sy
        Cb[2, 4] = Cb[4, 2] = -rho * g * sx
        Cb[3, 3] = rho * g * (ixx + vol * zb) - m * g * zg
        Cb[4, 4] = rho * g * (iyy + vol * zb) - m * g * zg
        Cb[3, 4] = Cb[4, 3] = -rho * g * ixy
        M[o:o + 6, o:o + 6] = Mb
        C[o:o + 6, o:o + 6] = Cb
    return M, C


def motions(amas, bdmp, exfc, w, M, C):
    """Response amplitude operators of SolveMotion (src/SolveMotion.f90:45-50,
    linear damping only): [-w^2 (M + A) + i w B + C] x = -Im F - i Re F for
    every heading (rows of exfc); returns (nbeta, 6 nbody) complex."""
    left = -w * w * (M + amas) + 1j * w * bdmp + C
    right = -np.imag(exfc) - 1j * np.real(exfc)
    return np.linalg.solve(left, right.T).T
