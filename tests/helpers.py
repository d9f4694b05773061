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
