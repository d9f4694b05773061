"""Benchmark: frequency-solves per second of the per-frequency BEM path.

Workload (one "step" = one frequency-solve): the 5-body array of 6048
panels in deep water (3 cylinders R = 4 m, T = 8 m with 48 x 22 side and
48 x 8 bottom panels, 2 boxes 12 x 6 x 4 m with 0.5 m panels, on a 30 m grid
perturbed by U(-3, 3) m from seed 3), 60 frequencies uniform in 0.1-2.5
rad/s cycled step by step, 8 headings 0..315 deg, 30 rigid-body modes.  A
step is the Green-function fill + influence-matrix assembly + LU + solves
for all 30 modes and 8 headings + added mass, damping and excitation force.

Default arm (ours): the mixed-precision form (complex64 fill and LU, FP64
refinement) through the C ABI; the plain complex128 form is measured on a
few steps beside it, and the mixed results are checked against it (1e-4).
--impl reference: the CPU restatement of the reference (the oracle: C with
OpenMP over field rows, LAPACK zgetrf/zgetrs through scipy's OpenBLAS) on
all host cores; the reference itself is Fortran and no Fortran compiler
exists on either machine.

Multi-GPU (torchrun): frequencies are split round-robin over ranks, each
rank a full replica with its own context; the only collectives are the
barrier and the max over ranks of the timed region (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FREQ = 60
FREQS = np.linspace(0.1, 2.5, N_FREQ)
BETAS_DEG = np.arange(8) * 45.0
METRIC = "freq-solves/s at 6k panels (mixed vs FP64 GPU, <=1e-4 err); p50/p99 latency"
CONFIG = {"workload": "5-body array, 6048 panels, deep water, 60 freqs x 8 headings, 30 modes",
          "panels": 6048, "bodies": 5, "headings": 8, "modes": 30, "depth": "infinite",
          "l2": "inputs larger than L2 (A and S are 2 x 293 MB complex64 per step)"}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: wait (bounded) for its first sample so that the
            # samples after this point fall inside the timed region
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        self.start = len(self.lines)
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.start:] or self.lines
        for ln in lines:
            t = [x.strip() for x in ln.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx = float(t[2])
            except ValueError:
                continue
            for name, val in zip(names, t[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    """One process per GPU under torchrun (NCCL; gloo where no GPU is visible,
    as in the CPU tests of this host logic)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        rank = int(os.environ["RANK"])
        local = int(os.environ.get("LOCAL_RANK", rank))
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return dist, rank, ws, local
    return None, 0, 1, 0


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x, local):
    if dist is None:
        return x
    import torch
    dev = f"cuda:{local}" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_frequencies(rank, world, n):
    """Frequencies are independent: rank r takes entries r, r + world, ...
    (no data exchange; the ranks meet only at the timing barrier)."""
    return list(range(rank, n, world))


def _mesh():
    import __graft_entry__ as ge
    pkg = ge.load_package()
    return pkg, pkg.meshgen.five_body_array(seed=3)


def _frequency_inputs(pkg, w):
    v, wk, w1, wvn = pkg.hamsgpu.wave_properties(3, float(w), -1.0)
    return v, wk, w1


def cpu_reference(steps, warmup, rank, world):
    """The oracle (CPU restatement of the reference path), all host cores."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    pkg, mesh = _mesh()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import case_from_mesh
    case = case_from_mesh(oracle, mesh, h=-1.0, headings_deg=list(BETAS_DEG))
    cores = os.cpu_count()
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(cores))
    # one bounded step = one full frequency-solve (about 10-30 s of CPU work at 6048 panels)
    times = []
    for k in range(warmup + steps):
        w = FREQS[k % N_FREQ]
        t0 = time.perf_counter()
        oracle.solve_frequency(case, w, nthreads=cores)
        t1 = time.perf_counter()
        if k >= warmup:
            times.append(t1 - t0)
    total = sum(times)
    value = len(times) / total
    line = {"metric": METRIC, "value": value, "unit": "freq-solves/s", "n_gpus": world, "steps": steps,
            "warmup": warmup, "ms_per_step": 1e3 * total / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "complex128", "data": "synthetic",
            "config": CONFIG, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "freq-solves/s", "cores": cores, "kind": "port",
                             "sample": f"{len(times)} full frequency-solves of the 6048-panel workload"},
            "e2e": {"value": value, "unit": "freq-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _cpu_baseline_sample():
    """One full frequency-solve of the workload by the oracle on all host
    cores: (cpu_baseline entry, the oracle's result or None)."""
    try:
        return _cpu_baseline_sample_inner()
    except Exception as e:  # reported, never silently dropped
        return {"value": None, "unit": "freq-solves/s", "cores": os.cpu_count(), "kind": "port",
                "sample": f"failed: {e}"}, None


def _vs_oracle(pkg, mesh, s, ref, betas, local, prec):
    """Max-normalised error of the plain and the mixed form against the
    oracle's solve of the CPU sample's frequency: A, B, F and the motions
    (RAOs) of the freely floating bodies that these give."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import max_norm_err, motions, rigid_body_matrices
    hg = pkg.hamsgpu
    w = FREQS[17]
    fv, fwk, fw1 = _frequency_inputs(pkg, w)
    M, C = rigid_body_matrices(mesh)
    xr = motions(ref.amas, ref.bdmp, ref.exfc, w, M, C)

    def errs(res):
        a, b, f = res[0], res[1], res[2]
        return {"A": max_norm_err(a, ref.amas), "B": max_norm_err(b, ref.bdmp), "F": max_norm_err(f, ref.exfc),
                "RAO": max_norm_err(motions(a, b, f, w, M, C), xr)}

    out = {"w_rad_s": float(w)}
    sp = hg.Solver(precision=hg.HG_PREC_FP64, device=local)
    sp.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    out["plain"] = errs(sp.solve_frequency(fv, fwk, fw1, -1.0, None, betas, want_potentials=False))
    sp.close()
    if prec == hg.HG_PREC_MIXED:
        out["mixed"] = errs(s.solve_frequency(fv, fwk, fw1, -1.0, None, betas, want_potentials=False))
    return out


def _cpu_baseline_sample_inner():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    pkg, mesh = _mesh()
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import case_from_mesh
    case = case_from_mesh(oracle, mesh, h=-1.0, headings_deg=list(BETAS_DEG))
    cores = os.cpu_count()
    t0 = time.perf_counter()
    ref = oracle.solve_frequency(case, FREQS[17], nthreads=cores)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "freq-solves/s", "cores": cores, "kind": "port",
            "sample": "1 full frequency-solve (w = %.3f rad/s) of the 6048-panel workload: C oracle with OpenMP "
                      "over field rows + scipy/OpenBLAS zgetrf/zgetrs" % FREQS[17]}, ref


def ours(args, dist, rank, world, local):
    pkg, mesh = _mesh()
    hg = pkg.hamsgpu
    prec = hg.HG_PREC_MIXED if args.precision == "mixed" else hg.HG_PREC_FP64
    my_freqs = [FREQS[k] for k in shard_frequencies(rank, world, N_FREQ)]
    betas = BETAS_DEG * math.pi / 180.0
    nd = 30
    nslots = args.slots

    def inputs(count, offset):
        ws = [my_freqs[(offset + k) % len(my_freqs)] for k in range(count)]
        vals = [_frequency_inputs(pkg, w) for w in ws]
        return (np.array([x[0] for x in vals]), np.array([x[1] for x in vals]), np.array([x[2] for x in vals]))

    sopts = dict(lu_tensor=args.lu_tensor, refine_method=1 if args.refine == "gmres" else 0,
                 solver=2 if args.solver == "gmres" else 1, hmatrix=args.hmatrix)
    s = hg.Solver(precision=prec, device=local, **sopts)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    # set-up (not a step): one frequency per slot creates every slot and its device buffers
    v, wk, w1 = inputs(nslots, 0)
    s.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nslots)
    # warm-up: exactly the requested steps
    warm = args.warmup
    if warm > 0:
        v, wk, w1 = inputs(warm, nslots)
        s.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nslots)
    # ---- device-timed region: one sweep of `steps` frequencies, inputs resident ----
    v, wk, w1 = inputs(args.steps, nslots + warm)
    _barrier(dist)
    with ClockSampler(local) as clk:
        s.mark(0)
        _, _, _, lat, _ = s.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nslots)
        s.mark(1)
        ms = s.elapsed_ms(0, 1)
    lat = [float(x) for x in lat]
    sweeps, resid = s.refine_info()
    ms_max = _max_over_ranks(dist, ms, local)
    value = world * args.steps / (ms_max / 1e3)
    clocks = clk.summary()
    # stage breakdown of one frequency-solve running alone (outside the timed region)
    s.solve_frequency(v[0], wk[0], w1[0], -1.0, None, betas, want_potentials=False)
    stages = s.stage_times()
    iters = s.iter_info() if args.solver == "gmres" else None

    # ---- end to end through the C ABI with host buffers, as a user runs one request on a
    #      context that already exists: the mesh from host arrays (set_mesh, which every slot then
    #      takes too), the sweep from host frequency arrays, forces and all potentials read back
    #      to host memory.  Outside: the context's creation and its first sweep, which creates
    #      the slots and their device buffers once. ----
    s2 = hg.Solver(precision=prec, device=local, **sopts)
    s2.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    vs, wks, w1s = inputs(nslots, 0)
    s2.solve_sweep(vs, wks, w1s, -1.0, None, betas, nslots=nslots)
    _barrier(dist)
    t0 = time.perf_counter()
    s2.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    s2.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nslots, want_potentials=True)
    t_e2e = time.perf_counter() - t0
    t_e2e = _max_over_ranks(dist, t_e2e, local)
    s2.close()
    mesh_bytes = mesh.nodes.nbytes + mesh.ncon.nbytes + mesh.ncn.nbytes + mesh.xyz_p.nbytes + mesh.ds.nbytes + \
        mesh.pnsz.nbytes + mesh.dxyz_p.nbytes + mesh.body_ranges.nbytes
    h2d = mesh_bytes * (1 + nslots) / args.steps + betas.nbytes + 3 * 8
    d2h = 2 * nd * nd * 8 + 8 * nd * 16 + mesh.n * (nd + 8) * 16

    # ---- plain FP64 form on a few steps, and the accuracy of the mixed form against it ----
    fp64 = None
    if rank == 0 and prec == hg.HG_PREC_MIXED and args.fp64_steps > 0:
        sp = hg.Solver(precision=hg.HG_PREC_FP64, device=local)
        sp.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
        errs = []
        pms = []
        for k in range(args.fp64_steps):
            w = FREQS[(7 + 19 * k) % N_FREQ]
            fv, fwk, fw1 = _frequency_inputs(pkg, w)
            sp.mark(4)
            a64, b64, f64, _ = sp.solve_frequency(fv, fwk, fw1, -1.0, None, betas)
            sp.mark(5)
            pms.append(sp.elapsed_ms(4, 5))
            a64, b64, f64 = a64.copy(), b64.copy(), f64.copy()
            am, bm, fm, _ = s.solve_frequency(fv, fwk, fw1, -1.0, None, betas)
            e = lambda x, y: float(np.abs(x - y).max() / np.abs(y).max())  # noqa: E731
            errs.append({"A": e(am, a64), "B": e(bm, b64), "F": e(fm, f64)})
        # the plain form through the sweep's concurrent solve slots, as the mixed form runs
        nsl = 4
        v, wk, w1 = inputs(nsl, 0)
        sp.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nsl)  # set-up: creates the slots
        v, wk, w1 = inputs(2 * nsl, nsl)
        sp.mark(4)
        sp.solve_sweep(v, wk, w1, -1.0, None, betas, nslots=nsl)
        sp.mark(5)
        sweep_ms = sp.elapsed_ms(4, 5)
        zroof = _gemm_roofline(sp, mesh.n, hg.HG_PREC_FP64, hg, lu_tensor=2)
        sp.close()
        fp64 = {"freq_solves_per_s": 1e3 / statistics.mean(pms), "ms_per_step": statistics.mean(pms),
                "steps": args.fp64_steps, "slots": 1,
                "sweep": {"freq_solves_per_s": 2 * nsl / (sweep_ms / 1e3), "frequencies": 2 * nsl, "slots": nsl},
                "lu_trailing_update": zroof,
                "mixed_vs_fp64_max_norm_err": {k: max(d[k] for d in errs) for k in ("A", "B", "F")}}

    # ---- roofline of the dominant kernel (the LU trailing-update GEMM) ----
    roof = None
    if rank == 0 and args.solver == "lu":
        roof = _roofline(s, mesh.n, prec, hg, ms_max / args.steps, lu_tensor=args.lu_tensor)
    # ---- the CPU oracle on one frequency (the CPU baseline sample), and both GPU forms against it ----
    cpu, vs_oracle = None, None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, ref = _cpu_baseline_sample()
        if ref is not None:
            vs_oracle = _vs_oracle(pkg, mesh, s, ref, betas, local, prec)
    s.close()
    if rank != 0:
        return
    lat_sorted = sorted(lat)
    line = {"metric": METRIC, "value": value, "unit": "freq-solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "complex64+fp64-refine" if prec == hg.HG_PREC_MIXED else "complex128",
            "data": "synthetic",
            "config": dict(CONFIG, precision=args.precision, parallelism=f"replicas{world}", slots=nslots,
                           refine=args.refine, lu_tensor=args.lu_tensor, solver=args.solver,
                           **({"hmatrix": args.hmatrix} if args.solver == "gmres" else {})),
            "latency_ms": {"p50": lat_sorted[len(lat) // 2], "p99": lat_sorted[min(len(lat) - 1,
                                                                                  int(0.99 * len(lat)))],
                           "what": f"host wall time per frequency-solve with {nslots} solves in flight"},
            "stage_ms_alone": {"fill": stages[0], "lu": stages[1], "solve_refine": stages[2],
                               "forces_readback": stages[3]},
            "refine": {"sweeps": sweeps, "residual": resid},
            "e2e": {"value": world * args.steps / t_e2e, "unit": "freq-solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": _launch_count(mesh.n, prec, sweeps, lu_tensor=args.lu_tensor) * args.steps
            if iters is None else None,
            "clocks": clocks, "roofline": roof, "fp64_form": fp64}
    if iters is not None:
        line["iterative"] = {"what": "solver 2 (restarted GMRES(25), tolerance 1e-4), one frequency alone",
                             "iterations": iters[0], "restarts": iters[1], "unconverged": iters[2],
                             "residual": iters[3]}
        del line["refine"]
    if cpu is not None:
        line["cpu_baseline"] = cpu
        line["vs_oracle"] = vs_oracle
    print(json.dumps(line), flush=True)


def _request_inputs(hg, freqs, h):
    vals = [hg.wave_properties(3, float(w), h) for w in freqs]
    v = np.array([x[0] for x in vals]); wk = np.array([x[1] for x in vals]); w1 = np.array([x[2] for x in vals])
    wvn = np.stack([x[3] for x in vals]) if h > 0 else None
    return v, wk, w1, wvn


def served(args):
    """Batching and serving forms through the request server (hg_server_*).

    batch: `requests` independent single-frequency solves (1-4 cylinders,
      N log-uniform 300-4000, deep water with p = 0.5 else h ~ U(30, 200) m,
      1-4 headings), all submitted at once.
    serve: `requests` requests (1-6 bodies, N log-uniform 500-12000, 20-100
      frequencies, 1-8 headings) arriving as a Poisson stream whose rate is
      set from a calibration run of the same stream submitted at once (0.8 of
      the measured request throughput, i.e. about 80 % device utilisation).
    """
    import __graft_entry__ as ge
    pkg = ge.load_package()
    hg, mg = pkg.hamsgpu, pkg.meshgen
    rng = np.random.default_rng(4 if args.workload == "batch" else 5)
    reqs = []
    for _ in range(args.requests):
        if args.workload == "batch":
            mesh, h, w, heads = mg.batch_case(rng)
            freqs = np.array([w])
        else:
            mesh, h, freqs, heads = mg.serving_case(rng)
            if args.freq_cap:
                freqs = freqs[:: max(1, -(-len(freqs) // args.freq_cap))][: args.freq_cap]
        v, wk, w1, wvn = _request_inputs(hg, freqs, h)
        reqs.append((mesh, h, v, wk, w1, wvn, np.array(heads) * math.pi / 180.0))
    nsolves = sum(len(r[2]) for r in reqs)

    def run(arrivals):
        srv = hg.Server(nslots=args.slots, budget_bytes=150e9)
        t0 = time.perf_counter()
        tickets = []
        for r, ta in zip(reqs, arrivals):
            dt = ta - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            tickets.append(srv.submit(*r))
        lat = []
        for t in tickets:
            lat.append(srv.wait(t)[3])
        total = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return total, sorted(lat), st

    with ClockSampler(0) as clk:
        rate = None
        if args.workload == "serve":
            # calibration: the first (up to) 24 requests submitted at once give the capacity in requests/s
            full = reqs
            reqs = full[:24]
            t_cal, _, _ = run([0.0] * len(reqs))
            rate = 0.8 * len(reqs) / t_cal  # requests per second at ~80 % of the measured capacity
            reqs = full
            gaps = rng.exponential(1.0 / rate, size=len(reqs))
            total, lat, st = run(np.cumsum(gaps) - gaps[0])
        else:
            total, lat, st = run([0.0] * len(reqs))
    p = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))]  # noqa: E731
    line = {"metric": "freq-solves/s (%s form, mixed precision); p50/p99 request latency" % args.workload,
            "value": nsolves / total, "unit": "freq-solves/s", "n_gpus": 1, "steps": nsolves, "warmup": 0,
            "ms_per_step": 1e3 * total / nsolves, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "complex64+fp64-refine", "data": "synthetic",
            "config": {"workload": args.workload, "requests": len(reqs), "freq_solves": nsolves,
                       "freqs_per_request_cap": args.freq_cap,
                       "panels_min_max": [min(r[0].n for r in reqs), max(r[0].n for r in reqs)],
                       "slots": args.slots, "hbm_budget_bytes": 150e9,
                       "arrival_rate_per_s": rate, "timing": "host wall clock, submission to last result"},
            "latency_ms": {"p50": p(0.5), "p99": p(0.99)},
            "server": st, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def three_bodies(args):
    """The plain FP64 form on three cylinders in line (R 3 m, T 6 m, 15 m apart,
    32 x 12 + 32 x 4 panels each, 32 x 4 lid panels each: 1536 + 384), depth
    40 m, irregular-frequency removal (IRSP = 1), headings 0/45/90 deg, 18
    modes, frequencies from 0.2-3.0 rad/s; beside it the CPU oracle on one
    frequency and the difference between the two on that frequency."""
    import __graft_entry__ as ge
    pkg = ge.load_package()
    hg, mg = pkg.hamsgpu, pkg.meshgen
    mesh = mg.three_cylinders(with_lid=True)
    h = 40.0
    freqs = np.linspace(0.2, 3.0, 80)
    betas_deg = [0.0, 45.0, 90.0]
    betas = np.array(betas_deg) * math.pi / 180.0
    prec = hg.HG_PREC_FP64 if args.precision == "fp64" else hg.HG_PREC_MIXED
    sel = [freqs[(7 * k) % 80] for k in range(args.warmup + args.steps)]
    v, wk, w1, wvn = _request_inputs(hg, sel, h)
    s = hg.Solver(precision=prec)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges,
               mesh.lid_xyz_p)
    W = args.warmup
    s.solve_sweep(v[:W], wk[:W], w1[:W], h, wvn[:W], betas, irsp=1, nslots=args.slots)
    with ClockSampler(0) as clk:
        s.mark(0)
        am, bm, fm, lat, _ = s.solve_sweep(v[W:], wk[W:], w1[W:], h, wvn[W:], betas, irsp=1, nslots=args.slots)
        s.mark(1)
        ms = s.elapsed_ms(0, 1)
    s.close()
    # the CPU oracle on the first timed frequency, all host cores
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from helpers import case_from_mesh, max_norm_err
    case = case_from_mesh(oracle, mesh, h=h, headings_deg=betas_deg, irsp=1)
    t0 = time.perf_counter()
    ref = oracle.solve_frequency(case, sel[W], nthreads=os.cpu_count())
    tcpu = time.perf_counter() - t0
    lat = sorted(float(x) for x in lat)
    form = "plain FP64" if prec == hg.HG_PREC_FP64 else "mixed"
    line = {"metric": f"freq-solves/s ({form} form, 3 cylinders in line, finite depth, IRSP=1)",
            "value": args.steps / (ms / 1e3), "unit": "freq-solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": W, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "complex128" if prec == hg.HG_PREC_FP64 else "complex64+fp64-refine",
            "data": "synthetic",
            "config": {"workload": "3 cylinders R 3 m T 6 m, 1536 hull + 384 lid panels, h 40 m, 3 headings, 18 modes",
                       "slots": args.slots},
            "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[-1]},
            "vs_oracle_max_norm_err": {"A": max_norm_err(am[0], ref.amas), "B": max_norm_err(bm[0], ref.bdmp),
                                       "F": max_norm_err(fm[0], ref.exfc)},
            "cpu_baseline": {"value": 1.0 / tcpu, "unit": "freq-solves/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "1 frequency-solve of this workload (C oracle, OpenMP over field rows, "
                                       "OpenBLAS LU)"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def field_map(args):
    """A wave-field map of the 6048-panel array (deep water, one frequency,
    8 headings, 30 modes solved once, untimed): free-surface elevation at a
    64 x 64 grid of points around the bodies (those inside a body's waterline
    box left out) for all 38 columns, each step one hg_field_points call from
    host coordinates to host results.  Beside it the CPU oracle on 256 of the
    points, and the difference between the two there."""
    pkg, mesh = _mesh()
    hg = pkg.hamsgpu
    prec = hg.HG_PREC_MIXED if args.precision == "mixed" else hg.HG_PREC_FP64
    betas = BETAS_DEG * math.pi / 180.0
    w = 0.8
    v, wk, w1 = _frequency_inputs(pkg, w)
    s = hg.Solver(precision=prec)
    s.set_mesh(mesh.nodes, mesh.ncon, mesh.ncn, mesh.xyz_p, mesh.ds, mesh.pnsz, mesh.dxyz_p, mesh.body_ranges)
    _, _, _, mx = s.solve_frequency(v, wk, w1, -1.0, None, betas)
    lo, hi = mesh.xyz_p.min(axis=0), mesh.xyz_p.max(axis=0)
    gx = np.linspace(lo[0] - 40.0, hi[0] + 40.0, 64)
    gy = np.linspace(lo[1] - 40.0, hi[1] + 40.0, 64)
    X, Y = np.meshgrid(gx, gy, indexing="ij")
    pts = np.column_stack([X.ravel(), Y.ravel(), np.zeros(X.size)])
    inside = np.zeros(len(pts), dtype=bool)
    for b0, b1 in mesh.body_ranges:
        q = mesh.xyz_p[b0 - 1:b1]
        blo, bhi = q.min(axis=0) - 0.5, q.max(axis=0) + 0.5
        inside |= (pts[:, 0] > blo[0]) & (pts[:, 0] < bhi[0]) & (pts[:, 1] > blo[1]) & (pts[:, 1] < bhi[1])
    pts = pts[~inside]
    for _ in range(args.warmup):
        elv = s.field_points(pts, kind=2)
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            s.mark(0)
            elv = s.field_points(pts, kind=2)
            s.mark(1)
            times.append(s.elapsed_ms(0, 1))
    ncol = elv.shape[1]
    s.close()
    ms = float(np.mean(times))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from helpers import case_from_mesh, max_norm_err
    case = case_from_mesh(oracle, mesh, h=-1.0, headings_deg=list(BETAS_DEG))
    sample = pts[:: max(1, len(pts) // 256)][:256]
    idx = [int(np.flatnonzero((pts == p).all(axis=1))[0]) for p in sample]
    t0 = time.perf_counter()
    ref = oracle.field_potential(case, sample, v, wk, w1, None, betas, mx)
    tcpu = time.perf_counter() - t0
    ref = 1j * w1 / 9.80665 * ref
    line = {"metric": "field points/s (free-surface elevation, all 38 columns per point)",
            "value": len(pts) / (ms / 1e3), "unit": "points/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "complex64+fp64-refine" if prec == hg.HG_PREC_MIXED else "complex128", "data": "synthetic",
            "config": {"workload": "5-body array, 6048 panels, deep water, w 0.8 rad/s, 8 headings, 30 modes; "
                                   "%d free-surface points" % len(pts), "solve_form": args.precision,
                       "timing": "host coordinates in, host results out (hg_field_points), CUDA events"},
            "vs_oracle_max_norm_err": max_norm_err(elv[idx], ref),
            "cpu_baseline": {"value": len(sample) / tcpu, "unit": "points/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": "%d of the points, C oracle with OpenMP over points" % len(sample)},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def _launch_count(n, prec, sweeps=1, nd=30, nbeta=8, lu_tensor=2):
    """Kernels the library launches per frequency-solve, from its launch
    sequence (checked against the ncu launch list of one solve)."""
    nb, nbo = 32, 256
    if prec == 0 and n >= 1024 and lu_tensor != 0:
        # FP64 form on the tensor cores: each sliced product is 3 kernels (A's digits, B's digits,
        # the product).  Per outer panel of jbo columns: p = jbo / 16 panels, their interchanges
        # and L11 solves (when jbo > 16), p - 1 inner products, the other columns' interchanges; where
        # columns remain: I, L11^-1, the U12 operands, three U12 products and the trailing one.
        lu = 0
        for k in range(0, n, nbo):
            jbo = min(nbo, n - k)
            p = (jbo + 15) // 16
            lu += p + (p if jbo > 16 else 0) + 3 * (p - 1) + 1 + (15 if n - k - jbo > 0 else 0)
        blocks = (n + nbo - 1) // nbo
        getrs = 1 + 2 * blocks + 3 * 2 * (blocks - 1)
        return 1 + lu + 3 + getrs + 1  # fill, LU, incident / source columns / S W, solves, forces
    def inner(jb, split=False):  # 32-wide panels: panel + fused interchanges / L11 solve, then the update
        p = (jb + nb - 1) // nb   # while columns remain (the FP64 form splits it: next panel's columns, the rest)
        return 2 * p + ((2 * p - 3 if p >= 2 else 0) if split else p - 1)
    tc = prec == 1 and n >= 1024
    if tc:
        outer = (n + nbo - 1) // nbo
        # the permutation's start (1); per outer panel: pivots to the other columns, L_kk^-1; where columns
        # remain: I - L_kk^-1 and two tensor-core GEMMs (U12, trailing update) with their operand packing;
        # then one batched U_kk^-1
        lu = 1 + sum(inner(min(nbo, n - k)) for k in range(0, n, nbo)) + 2 * outer + 7 * (outer - 1) + 1
    else:
        lu = inner(n, split=prec == 0)
    blocks = (n + nbo - 1) // nbo
    # right-hand sides permuted (gather + copy with the block inverses, else one interchange kernel), then
    # (block-inverse product or trsm, gemm) down and up
    getrs = (2 if tc else 1) + 2 * (2 * blocks - 1)
    fill = 2 if prec == 1 else 1  # mixed deep water: the FP32 tile kernel and the self/adjacent-pair kernel
    forces = 1
    if prec == 0:
        return fill + lu + 3 + getrs + forces      # incident weights, source columns, S W product
    # mixed: RHS (incident, source columns, S W as a split product: 3 kernels);
    # 1 + sweeps solves, each followed by a residual check (product, split,
    # reduce) and bracketed by conversions; column norms of B and of each residual
    # (later sweeps update the residual with the correction: one more conversion each).
    # The first residual is the sliced tensor-core product (nd + nbeta <= 40): row maxima,
    # row exponents, A's digits, their K padding (when 2N is not a multiple of 128), y's
    # digits, the product, the sum: 4 or 3 kernels more than the split product.
    s1 = 1 + sweeps
    sliced = (4 if (2 * n) % 128 else 3) if nd + nbeta <= 40 else 0
    return fill + lu + 5 + s1 * getrs + 3 * s1 + sliced + (1 + s1) + 2 * s1 + sweeps + forces


# Counted per-pair work of the deep-water fill (oracle/opcount.py on the 6048-panel array): mean
# over the 0.1-2.5 rad/s sweep, in operations per pair.
F_PAIR_MEAN = 590.0


def _roofline(s, n, prec, hg, ms_per_step, nd=30, nbeta=8, lu_tensor=2):
    """Roofline of the dominant kernel, the 32-column complex64 LU panel
    (k_getf2_cluster_reg: 52 % of one solve's kernel time in the ncu launch
    list), timed with CUDA events on the library's stream at the height of the
    first panel (N rows): algorithmic bytes = the panel read once and written
    once, 2 x N x 32 x 8 B.  Beside it the LU trailing update (the tcgen05
    GEMM, timed at the first outer panel's shape m = n = N - 256, k = 256) and
    the whole step (the algorithmic flops of one frequency-solve over the
    measured time per step)."""
    peaks, kind = _peaks()
    out = None
    if prec == hg.HG_PREC_MIXED:
        try:
            pms = s.bench_panel(n, 16)
            pbytes = 2.0 * n * 32 * 8
            gbs = pbytes / (pms / 1e3) / 1e9
            out = {"kernel": "k_getf2_cluster_reg (32-column complex64 panel LU of the blocked factorisation, "
                             "cluster of ceil(rows / 512) CTAs, rows in registers)",
                   "bound": "hbm", "achieved": gbs, "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                   "frac": gbs / peaks.get("hbm_gbs", 6800.0), "peak_source": f"hbm_gbs of {kind} peaks",
                   "bytes_per_launch": pbytes, "ms_per_launch": pms,
                   # DRAM bytes of one panel launch from the committed ncu capture (a 5408-row panel,
                   # 1.63 MB read), scaled to N rows by the panel's size
                   "traffic": 1.625856e6 * n / 5408.0 if n == 6048 else None,
                   "note": "latency-bound: 32 dependent column steps, each a cluster-wide pivot search and one "
                           "DSMEM message round; bytes/time is far below the HBM peak by construction, and the "
                           "7 solves in flight hide it behind other solves' fills and tensor-core updates"}
        except Exception:
            out = None
    gemm = _gemm_roofline(s, n, prec, hg, lu_tensor)
    flops = 8.0 / 3.0 * n ** 3 + 8.0 * n * n * (nd + nbeta) + F_PAIR_MEAN * n * n
    tf = flops / (ms_per_step / 1e3) / 1e12
    whole = {"flops_per_step": flops, "achieved_tflops": tf, "peak_tflops": peaks.get("bf16_tflops", 1900.0),
             "frac": tf / peaks.get("bf16_tflops", 1900.0),
             "what": "LU (8/3) N^3 + solves 8 N^2 (30 modes + 8 headings) + fill N^2 x 590 counted operations per "
                     "pair, over ms_per_step, against the bf16 tensor peak"}
    if out is None:
        out = gemm
        if out is not None:
            out["whole_step"] = whole
        return out
    out["lu_trailing_update"] = gemm
    out["whole_step"] = whole
    return out


def _gemm_roofline(s, n, prec, hg, lu_tensor=2):
    """Roofline of the LU trailing update, the path's dense contraction: the
    library's tcgen05 GEMM (mixed form, the variant lu_tensor selects; FP64
    form: the exact digit-sliced complex128 product, or the SIMT GEMM with
    lu_tensor 0), timed with CUDA events on the library's stream at the shape
    of the first 256-wide outer panel (m = n = N - 256, k = 256)."""
    m, k = n - 256, 256
    # hg_bench_gemm variants: 2 split TF32, 3 TF32, 4 split BF16, 5 complex128 digit slices
    if prec == hg.HG_PREC_MIXED:
        variant = {3: 2, 1: 3, 2: 4}.get(lu_tensor, 1)
    else:
        variant = 5 if lu_tensor != 0 else 0
    try:
        ms = s.bench_gemm(variant, m, m, k, iters=10)
    except Exception:
        return None
    flops = 8.0 * m * m * k  # complex multiply-adds x 8 real flops
    achieved = flops / (ms / 1e3) / 1e12
    peaks, kind = _peaks()
    peak = peaks.get("bf16_tflops", 1900.0)
    names = {2: "k_cgemm_tc<3> (LU trailing update A22 -= L21 U12, complex64, tcgen05 split TF32)",
             3: "k_cgemm_tc<1> (LU trailing update A22 -= L21 U12, complex64, tcgen05 TF32)",
             4: "k_cgemm_tc<2> (LU trailing update A22 -= L21 U12, complex64, tcgen05 split BF16)",
             1: "k_cgemm_wide (LU trailing update, complex64 SIMT)",
             0: "k_gemm<double> (LU trailing update, complex128 SIMT)",
             5: "k_zoz_gemm (LU trailing update A22 -= L21 U12, complex128, tcgen05 exact BF16 digit products)"}
    out = {"kernel": names[variant],
           "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
           "peak_source": f"bf16_tflops of {kind} peaks", "flops_per_launch": flops, "ms_per_launch": ms,
           "traffic": None}
    if variant == 4:
        # DRAM bytes of one launch of this shape (5792 x 5792 x 256) from the committed ncu capture
        out["traffic"] = (313.024 + 217.851392) * 1e6 if n == 6048 else None
        out["note"] = ("algorithmic complex flops; the hardware does 3 BF16 products per real product at the bf16 "
                       "rate, so the tensor-pipe utilisation is about 3 x frac (ncu: 44.5 % tensor-pipe activity "
                       "at this shape)")
    if variant == 5:
        # DRAM bytes of the product kernel: C read and written once, each digit tile read once (eight
        # digits of A: m x 2k, of B: 2n x 2k, BF16); the 4096 x 4096 x 256 ncu capture measured 0.976 x
        # these, scaled here to this shape (the traffic grows with them)
        mp, np2, kp = -(-m // 128) * 128, -(-2 * m // 64) * 64, 2 * k
        algo = 2.0 * m * m * 16 + 8.0 * (mp + np2) * kp * 2
        out["traffic"] = 0.976 * algo
        out["note"] = ("algorithmic complex flops of an FP64-accurate product; the hardware does 36 BF16 digit "
                       "products (the digit pairs s + t <= 9 of eight 7-bit digits per operand) per real product "
                       "at the bf16 rate, so the tensor-pipe work is 36 x frac of the bf16 peak; includes the "
                       "two slicing kernels; traffic scaled from the 4096 x 4096 x 256 capture "
                       "(profiles/zgemm_sliced_4096x4096x256.md)")
        out["bf16_equivalent_frac"] = 36 * achieved / peak
    if variant == 2:
        # DRAM bytes of one launch of this shape (5792 x 5792 x 256) from the committed ncu capture
        out["traffic"] = (486.998528 + 235.5008) * 1e6 if n == 6048 else None
        out["note"] = ("algorithmic complex flops; the hardware does 3 TF32 products per real product and TF32 "
                       "runs at half the bf16 rate, so the tensor-pipe utilisation is about 6 x frac "
                       "(ncu: 72 % tensor-pipe activity at this shape)")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slots", type=int, default=0,
                    help="frequency-solves in flight (hg_solve_sweep slots); 0: at most 8, balanced over the steps")
    ap.add_argument("--refine", default="classical", choices=["classical", "gmres"],
                    help="mixed-form refinement: classical iterative refinement or GMRES-IR")
    ap.add_argument("--lu-tensor", type=int, default=2, choices=[0, 1, 2, 3],
                    help="LU trailing updates: 2 split-BF16 tensor cores, 3 split-TF32, 1 TF32, 0 FP32 SIMT")
    ap.add_argument("--hmatrix", type=int, default=0, choices=[0, 1],
                    help="with --solver gmres: the products through the reference's H-matrix (ACA)")
    ap.add_argument("--solver", default="lu", choices=["lu", "gmres"],
                    help="array workload: linear solver (gmres = the reference's Solver_type 2)")
    ap.add_argument("--workload", default="array", choices=["array", "batch", "serve", "three", "field"],
                    help="array: the 6048-panel frequency sweep (headline); batch / serve: the request server")
    ap.add_argument("--requests", type=int, default=None, help="batch / serve: number of requests")
    ap.add_argument("--freq-cap", type=int, default=0,
                    help="serve: at most this many of each request's frequencies (evenly spaced; 0: all)")
    args = ap.parse_args()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        cpu_reference(args.steps, args.warmup, rank, world)
        return
    auto_slots = args.slots <= 0
    if auto_slots:
        # at most 8 in flight (measured at 6048 panels: 4 -> 67.7, 6 -> 68.3, 8 -> 72.4 freq-solves/s),
        # spread evenly over the rounds the timed frequencies make
        rounds = -(-args.steps // 8)
        args.slots = max(1, -(-args.steps // rounds))
        if args.workload == "three":
            args.slots = min(args.slots, 4)
    if args.workload == "three":
        three_bodies(args)
        return
    if args.workload == "field":
        field_map(args)
        return
    if args.workload != "array":
        if args.requests is None:
            args.requests = 512 if args.workload == "batch" else 24
        if auto_slots:
            args.slots = 8
        served(args)
        return
    dist, rank, world, local = _dist()
    try:
        ours(args, dist, rank, world, local)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
