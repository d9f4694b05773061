"""The operation-counting restatement of one deep-water pair of the fill
(oracle/opcount.py) gives the C oracle's own influence and single-layer
entries, so the per-pair count it reports is the count of the pinned
algorithm (near pairs with the Newman integrals, far pairs without, both
branches of the Struve/Bessel approximations)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))

import opcount  # noqa: E402
from helpers import case_from_mesh  # noqa: E402


def test_counting_restatement_matches_oracle_entries(pkg, oracle):
    mesh = pkg.meshgen.three_cylinders(with_lid=False)
    case = case_from_mesh(oracle, mesh, h=-1.0)
    w = 1.1
    v, wk, w1, wvn = oracle.wave_properties(case.ctl, w)
    A, S = oracle.assemble(case, v, wvn)
    rng = np.random.default_rng(7)
    pairs = [(i, j) for i, j in zip(rng.integers(0, case.n, 60), rng.integers(0, case.n, 60))]
    pairs += [(5, 5), (5, 6), (400, 401), (900, 902)]   # self and adjacent pairs
    flags = set()
    worst = 0.0
    for i, j in pairs:
        verts = [case.nodes[case.ncon[j, k] - 1] for k in range(case.ncn[j])]
        f, a, s = opcount.pair_entries(case.xyz_p[i], case.xyz_p[j], float(case.pnsz[j]), verts,
                                       int(case.ncn[j]), float(case.ds[j]), case.dxyz_p[j, :3], v)
        flags.add(f)
        a_full = a + (2.0 * np.pi if i == j else 0.0)   # ASSB_LEFT's free term on the diagonal
        worst = max(worst, abs(a_full - A[i, j]) / abs(A[i, j]), abs(s - S[i, j]) / abs(S[i, j]))
    assert flags == {0, 1}
    assert worst < 1e-12


def test_count_is_stable_and_split_by_kind():
    """Counting the same pair twice gives the same tally, and a near pair
    (Newman integral) costs more than a far one."""
    opcount.COUNTS.clear()
    verts = [[0.0, 0.0, -1.0], [1.0, 0.0, -1.0], [1.0, 1.0, -1.2], [0.0, 1.0, -1.2]]
    args = ([0.5, 0.5, -1.1], 1.0, verts, 4, 1.0, [0.0, 0.0, 1.0], 0.3)
    opcount.pair_entries([0.3, 0.4, -2.0], [0.5, 0.5, -1.1], *args[1:])
    near = dict(opcount.COUNTS)
    opcount.COUNTS.clear()
    opcount.pair_entries([0.3, 0.4, -2.0], [0.5, 0.5, -1.1], *args[1:])
    assert dict(opcount.COUNTS) == near
    opcount.COUNTS.clear()
    opcount.pair_entries([300.0, 0.4, -2.0], [0.5, 0.5, -1.1], *args[1:])
    far = dict(opcount.COUNTS)
    assert near["log"] > far.get("log", 0) and opcount.flops(near) > opcount.flops(far)
