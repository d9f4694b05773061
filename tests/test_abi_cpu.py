"""The C-ABI library without a GPU: it builds, loads, exports every symbol of
include/hamsgpu.h, fails cleanly when no device is present, and its
host-side helpers (dispersion roots, wave properties, panel geometry) agree
with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def _header_symbols():
    with open(os.path.join(ROOT, "include", "hamsgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(hg_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.hamsgpu.load()
    declared = _header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(pkg.hamsgpu.EXPORTS) == declared


def test_create_without_gpu_fails_cleanly(pkg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pkg.hamsgpu.HamsGpuError):
        pkg.hamsgpu.Solver()


@pytest.mark.parametrize("w,h", [(0.05, 70.0), (0.5, 40.0), (1.3, 40.0), (3.0, 200.0), (0.2, 30.0)])
def test_dispersion_matches_oracle(pkg, oracle, w, h):
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, w, h)
    ref = oracle.dispersion(w, h)
    assert np.abs(wvn - ref).max() <= 1e-13 * np.abs(ref).max()
    assert wk == wvn[0]
    assert abs(v - w * w / 9.80665) < 1e-15


def test_wave_properties_deep_water(pkg):
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, 1.5, -1.0)
    assert wvn is None and wk == v and w1 == 1.5
    v2, wk2, w12, _ = pkg.hamsgpu.wave_properties(4, 2 * np.pi / 1.5, -1.0)
    assert abs(w12 - 1.5) < 1e-14


def test_panel_geometry_matches_oracle_and_meshgen(pkg, oracle):
    case = oracle.load_case(os.path.join(GOLDEN, "config1", "input"))
    s, e = int(case.body_start[1]), int(case.body_end[1])
    nodes = case.nodes
    xyz, ds, pn, dx = pkg.hamsgpu.panel_geometry(nodes, case.ncon[s:e], case.ncn[s:e], [0.0, 54.0, 0.0])
    assert np.abs(xyz - case.xyz_p[s:e]).max() < 1e-12
    assert np.abs(ds - case.ds[s:e]).max() < 1e-12
    assert np.abs(pn - case.pnsz[s:e]).max() < 1e-12
    assert np.abs(dx - case.dxyz_p[s:e]).max() < 1e-12
    m = pkg.meshgen.single_cylinder()
    xyz, ds, pn, dx = pkg.hamsgpu.panel_geometry(m.nodes, m.ncon, m.ncn, [0.0, 0.0, 0.0])
    assert np.abs(ds - m.ds).max() < 1e-12 and np.abs(dx - m.dxyz_p).max() < 1e-12


def test_benchmark_meshes(pkg):
    mg = pkg.meshgen
    assert mg.single_cylinder().n == 384
    m2 = mg.three_cylinders()
    assert m2.n == 1536 and len(m2.lid_xyz_p) == 384
    m3 = mg.five_body_array()
    assert m3.n == 6048 and len(m3.body_ranges) == 5
    assert np.all(np.abs(m2.lid_xyz_p[:, 2]) == 0.0)
