"""Small, self-contained GPU cases of the library's kernels, for profilers.

Each case runs one kernel family through the C ABI on synthetic data sized
to exceed the 129 MB L2 (so DRAM counters mean something) while holding at
most a few GB on the device, and prints one line of timing.  Run from the
repository root, e.g.

    python hams-mrel_gb300/profile_cases.py gemm 6016 6016 32
    python hams-mrel_gb300/profile_cases.py gesv 6048 38 1

  gemm M N K [ITERS] [PREC]  complex GEMM C -= A B (PREC: hg_bench_gemm's variant, 0 complex128
                             SIMT, 1 complex64 SIMT, 2-4 complex64 tensor cores, 5 complex128
                             digit-sliced tensor cores)
  gesv N NRHS PREC           dense solve (hg_gesv) of a random diagonally
                             dominated system: LU panels, trailing updates,
                             triangular solves, refinement residuals (PREC 0
                             plain, 1 mixed)
  step [PREC]                one frequency-solve of the 6048-panel 5-body
                             benchmark array (fill, LU, solves, forces)
  fill N H PREC              two Green fills + LUs of a cylinder array of about N
                             panels at depth H metres (H <= 0: deep water)
  panel M [ITERS]            the 32-column complex64 cluster panel LU of M rows
                             (hg_bench_panel), ITERS timed launches
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import hamsgpu  # noqa: E402


def case_gemm(m, n, k, iters=3, prec=1):
    s = hamsgpu.Solver(precision=hamsgpu.HG_PREC_FP64)
    ms = hamsgpu.ctypes.c_float()
    s._check(s.L.hg_bench_gemm(s.h, prec, m, n, k, iters, hamsgpu.ctypes.byref(ms)))
    flops = 8.0 * m * n * k
    print(f"gemm prec={prec} {m}x{n}x{k}: {ms.value:.4f} ms/launch, {flops / ms.value / 1e9:.2f} TFLOP/s")
    s.close()


def case_gesv(n, nrhs, prec):
    rng = np.random.default_rng(7)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a += np.diag(np.full(n, 2.0 * np.sqrt(n)))
    b = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    s = hamsgpu.Solver(precision=hamsgpu.HG_PREC_FP64)
    t0 = time.perf_counter()
    lu, ipiv, x, it, info = s.gesv(a, b, precision=prec)
    t1 = time.perf_counter()
    r = b - a @ x
    print(f"gesv n={n} nrhs={nrhs} prec={prec}: info={info} iter={it} host-timed {1e3 * (t1 - t0):.1f} ms, "
          f"max|r|/max|b| = {np.abs(r).max() / np.abs(b).max():.2e}")
    s.close()


def case_step(prec=1):
    import meshgen
    mesh = meshgen.five_body_array()
    s = hamsgpu.Solver(precision=prec)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    v, wk, w1, wvn = hamsgpu.wave_properties(3, 1.0, -1.0)
    betas = np.arange(8) * np.pi / 4
    s.solve_frequency(v, wk, w1, -1.0, wvn, betas, want_potentials=False)
    print(f"step prec={prec} n={len(mesh.ncn)}: stages (fill, lu, solve, forces) ms = "
          f"{', '.join(f'{t:.2f}' for t in s.stage_times())}")
    s.close()


def case_fill(n, h, prec):
    import meshgen
    mesh = meshgen.scaled_array(n)
    s = hamsgpu.Solver(precision=prec)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    hh = float(h) if h > 0 else -1.0
    v, wk, w1, wvn = hamsgpu.wave_properties(3, 1.0, hh)
    for rep in range(2):  # the second fill reuses what the first built once per mesh
        s.set_frequency(v, wk, w1, hh, wvn)
        s.fill_factor(0)
        t = s.stage_times()
        print(f"fill {rep + 1} n={len(mesh.ncn)} h={hh} prec={prec}: fill {t[0]:.2f} ms "
              f"({len(mesh.ncn) ** 2 / t[0] / 1e3:.3f} Mpairs/s), lu {t[1]:.2f} ms")
    s.close()


def case_panel(m, iters=4):
    s = hamsgpu.Solver(precision=hamsgpu.HG_PREC_MIXED)
    ms = s.bench_panel(m, iters)
    print(f"panel m={m}: {1e3 * ms:.1f} us/launch")
    s.close()


def main(argv):
    if not argv:
        print(__doc__)
        return 2
    cmd, args = argv[0], [int(x) for x in argv[1:]]
    if cmd == "gemm":
        case_gemm(*args)
    elif cmd == "gesv":
        case_gesv(*args)
    elif cmd == "step":
        case_step(*args)
    elif cmd == "fill":
        case_fill(*args)
    elif cmd == "panel":
        case_panel(*args)
    else:
        print(__doc__)
        return 2
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
