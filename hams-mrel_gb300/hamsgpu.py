"""ctypes binding of libhamsgpu.so (the C ABI declared in include/hamsgpu.h).

This is the binding a Python caller (tests, bench.py, a serving loop) uses;
the Fortran driver binds the same symbols through ISO_C_BINDING.  It loads
only the in-tree CUDA library and raises if that library or a GPU is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

HG_PREC_FP64 = 0
HG_PREC_MIXED = 1

# Every symbol include/hamsgpu.h declares (checked by the CPU test suite).
EXPORTS = [
    "hg_default_opts", "hg_create", "hg_destroy", "hg_last_error", "hg_set_mesh", "hg_set_frequency",
    "hg_fill_factor", "hg_solve_radiation", "hg_solve_all_headings", "hg_solve_diffraction", "hg_forces",
    "hg_solve_frequency", "hg_keep_matrices", "hg_get_matrix", "hg_green_points", "hg_refine_info",
    "hg_stage_times", "hg_dispersion", "hg_wave_properties", "hg_panel_geometry", "hg_mark", "hg_elapsed",
    "hg_bench_gemm", "hg_green_points_noalloc", "hg_gesv", "hg_gemm_check",
    "hg_solve_sweep", "hg_gmres_iterations", "hg_solve_footprint", "hg_server_create", "hg_server_submit",
    "hg_server_wait", "hg_server_stats", "hg_server_last_error", "hg_server_destroy", "hg_field_points",
    "hg_case_read", "hg_case_free", "hg_case_info", "hg_case_arrays", "hg_case_run", "hg_case_write",
    "hg_iter_info", "hg_case_options", "hg_server_timeline", "hg_bench_panel", "hg_resid_check",
    "hg_hmatrix_info", "hg_hmatrix_check", "hg_hmatrix_partition",
]


class HgOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("precision", ctypes.c_int), ("grn_kind", ctypes.c_int),
                ("max_refine", ctypes.c_int), ("refine_tol", ctypes.c_double), ("rho", ctypes.c_double),
                ("g", ctypes.c_double), ("lu_tensor", ctypes.c_int), ("refine_method", ctypes.c_int),
                ("fin_table", ctypes.c_int), ("solver", ctypes.c_int), ("hmatrix", ctypes.c_int)]


class HgRequest(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("ntnd", ctypes.c_int), ("nodes", ctypes.c_void_p), ("ncon", ctypes.c_void_p),
                ("ncn", ctypes.c_void_p), ("xyz_p", ctypes.c_void_p), ("ds", ctypes.c_void_p),
                ("pnsz", ctypes.c_void_p), ("dxyz_p", ctypes.c_void_p), ("nl", ctypes.c_int),
                ("lid_xyz_p", ctypes.c_void_p), ("nbody", ctypes.c_int), ("body_ranges", ctypes.c_void_p),
                ("h", ctypes.c_double), ("nfreq", ctypes.c_int), ("v", ctypes.c_void_p), ("wk", ctypes.c_void_p),
                ("w1", ctypes.c_void_p), ("wvn", ctypes.c_void_p), ("nk", ctypes.c_int), ("irsp", ctypes.c_int),
                ("isol", ctypes.c_int), ("nbeta", ctypes.c_int), ("betas", ctypes.c_void_p)]


_LIB = None


def library_path() -> str:
    return os.path.join(HERE, "_build", "libhamsgpu.so")


def load(build_if_missing: bool = True):
    """Load libhamsgpu.so (building it with nvcc first if needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build_if_missing:
        import importlib.util
        spec = importlib.util.spec_from_file_location("hams_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libhamsgpu.so is not built ({path}); run build() first")
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    L.hg_default_opts.argtypes = [P(HgOpts)]
    L.hg_default_opts.restype = None
    L.hg_create.argtypes = [P(c_void_p), P(HgOpts)]
    L.hg_destroy.argtypes = [c_void_p]
    L.hg_destroy.restype = None
    L.hg_last_error.argtypes = [c_void_p]
    L.hg_last_error.restype = ctypes.c_char_p
    L.hg_set_mesh.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              c_void_p, c_int, c_void_p, c_int, c_void_p]
    L.hg_set_frequency.argtypes = [c_void_p, c_double, c_double, c_double, c_double, c_void_p, c_int]
    L.hg_fill_factor.argtypes = [c_void_p, c_int]
    L.hg_solve_radiation.argtypes = [c_void_p, c_void_p, c_int]
    L.hg_solve_all_headings.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_int]
    L.hg_solve_diffraction.argtypes = [c_void_p, c_double, c_void_p]
    L.hg_forces.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    L.hg_solve_frequency.argtypes = [c_void_p, c_double, c_double, c_double, c_double, c_void_p, c_int, c_int,
                                     c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int]
    L.hg_field_points.argtypes = [c_void_p, c_int, c_void_p, c_int, c_int, c_void_p, c_int]
    L.hg_keep_matrices.argtypes = [c_void_p, c_int]
    L.hg_get_matrix.argtypes = [c_void_p, c_int, c_void_p, c_int]
    L.hg_green_points.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    L.hg_refine_info.argtypes = [c_void_p, P(c_int), P(c_double)]
    L.hg_gmres_iterations.argtypes = [c_void_p, P(c_int)]
    L.hg_iter_info.argtypes = [c_void_p, P(c_int), P(c_int), P(c_int), P(c_double)]
    L.hg_stage_times.argtypes = [c_void_p, P(ctypes.c_float)]
    L.hg_green_points_noalloc.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    L.hg_gesv.argtypes = [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p, c_int, P(c_int),
                          P(c_int)]
    L.hg_solve_sweep.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_int, c_int,
                                 c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                 c_void_p]
    L.hg_solve_footprint.argtypes = [c_int, c_int, c_int, c_int, c_int, c_int, c_int]
    L.hg_solve_footprint.restype = ctypes.c_size_t
    L.hg_server_create.argtypes = [P(c_void_p), P(HgOpts), c_int, c_double]
    L.hg_server_submit.argtypes = [c_void_p, P(HgRequest), P(ctypes.c_longlong)]
    L.hg_server_wait.argtypes = [c_void_p, ctypes.c_longlong, c_double, c_void_p, c_void_p, c_void_p, c_void_p]
    L.hg_server_stats.argtypes = [c_void_p, c_void_p]
    L.hg_server_timeline.argtypes = [c_void_p, c_int, c_void_p]
    L.hg_server_last_error.argtypes = [c_void_p]
    L.hg_server_last_error.restype = ctypes.c_char_p
    L.hg_server_destroy.argtypes = [c_void_p]
    L.hg_server_destroy.restype = None
    L.hg_bench_gemm.argtypes = [c_void_p, c_int, c_int, c_int, c_int, c_int, P(ctypes.c_float)]
    L.hg_bench_panel.argtypes = [c_void_p, c_int, c_int, P(ctypes.c_float)]
    L.hg_gemm_check.argtypes = [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                c_int]
    L.hg_resid_check.argtypes = [c_void_p, c_int, c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                 c_int, c_void_p, c_int]
    L.hg_hmatrix_info.argtypes = [c_void_p, P(c_int), P(c_int), P(c_int), P(c_double), P(c_double)]
    L.hg_hmatrix_check.argtypes = [c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    L.hg_hmatrix_partition.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_int]
    L.hg_mark.argtypes = [c_void_p, c_int]
    L.hg_elapsed.argtypes = [c_void_p, c_int, c_int, P(ctypes.c_float)]
    L.hg_dispersion.argtypes = [c_double, c_double, c_int, c_void_p]
    L.hg_wave_properties.argtypes = [c_int, c_double, c_double, c_int, P(c_double), P(c_double), P(c_double),
                                     c_void_p]
    L.hg_panel_geometry.argtypes = [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]
    L.hg_case_read.argtypes = [ctypes.c_char_p, P(c_void_p), ctypes.c_char_p, c_int]
    L.hg_case_free.argtypes = [c_void_p]
    L.hg_case_free.restype = None
    L.hg_case_info.argtypes = [c_void_p, c_void_p, c_void_p]
    L.hg_case_options.argtypes = [c_void_p, P(c_int), P(c_int)]
    L.hg_case_arrays.argtypes = [c_void_p] + [c_void_p] * 11
    L.hg_case_run.argtypes = [c_void_p, ctypes.c_char_p, P(HgOpts), c_int, ctypes.c_char_p, c_int]
    L.hg_case_write.argtypes = [c_void_p, ctypes.c_char_p, c_void_p, c_void_p, c_void_p, c_double, c_double,
                                ctypes.c_char_p, c_int]
    _LIB = L
    return L


NK = 200


def wave_properties(inft, value, h, nk=NK):
    """CalWaveProperts through the library: returns (v, wk, w1, wvn or None)."""
    L = load()
    v, wk, w1 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    wvn = np.zeros(nk) if h > 0 else None
    rc = L.hg_wave_properties(int(inft), float(value), float(h), nk, ctypes.byref(v), ctypes.byref(wk),
                              ctypes.byref(w1), _ptr(wvn))
    if rc != 0:
        raise HamsGpuError(rc, "hg_wave_properties failed")
    return v.value, wk.value, w1.value, wvn


def panel_geometry(nodes, ncon, ncn, xr):
    """CalNormals geometry through the library; ncon 1-based (n,4)."""
    L = load()
    nodes_f = np.asfortranarray(nodes, dtype=np.float64)
    ncon_f = np.asfortranarray(ncon, dtype=np.int32)
    ncn_c = np.ascontiguousarray(ncn, dtype=np.int32)
    n = len(ncn_c)
    xyz = np.zeros((n, 3), order="F"); ds = np.zeros(n); pn = np.zeros(n); dx = np.zeros((n, 6), order="F")
    xr_c = np.ascontiguousarray(xr, dtype=np.float64)
    rc = L.hg_panel_geometry(n, len(nodes_f), _ptr(nodes_f), _ptr(ncon_f), _ptr(ncn_c), _ptr(xr_c), _ptr(xyz),
                             _ptr(ds), _ptr(pn), _ptr(dx))
    if rc != 0:
        raise HamsGpuError(rc, "hg_panel_geometry failed")
    return xyz, ds, pn, dx


class HamsGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"hamsgpu error {code}: {msg}")
        self.code = code


def _ptr(a):
    return None if a is None else a.ctypes.data


def hmatrix_partition(xyz):
    """The H-matrix partition of panel centres xyz (n x 3) on the host
    (hg_hmatrix_partition): (perm, blocks), blocks an array of rows
    (row start, rows, column start, columns, admissible)."""
    L = load()
    xyz = np.asfortranarray(xyz, dtype=np.float64)
    n = xyz.shape[0]
    perm = np.zeros(n, dtype=np.int32)
    nb = L.hg_hmatrix_partition(n, _ptr(xyz), _ptr(perm), None, 0)
    if nb < 0:
        raise HamsGpuError(nb, "hg_hmatrix_partition failed")
    blocks = np.zeros((nb, 5), dtype=np.int32)
    L.hg_hmatrix_partition(n, _ptr(xyz), None, _ptr(blocks), nb)
    return perm, blocks


class Solver:
    """One library context (device buffers, stream, factorisation)."""

    def __init__(self, precision: int = HG_PREC_FP64, device: int = 0, grn_kind: int = 8,
                 max_refine: int = 10, refine_tol: float = 1e-10, rho: float = 1000.0, g: float = 9.80665,
                 lu_tensor: int = 2, refine_method: int = 0, fin_table: int = -1, solver: int = 1,
                 hmatrix: int = 0):
        self.L = load()
        opts = HgOpts()
        self.L.hg_default_opts(ctypes.byref(opts))
        opts.device, opts.precision, opts.grn_kind = device, precision, grn_kind
        opts.max_refine, opts.refine_tol, opts.rho, opts.g = max_refine, refine_tol, rho, g
        opts.lu_tensor = lu_tensor
        opts.refine_method = refine_method
        opts.fin_table = fin_table
        opts.solver = solver
        opts.hmatrix = hmatrix
        h = ctypes.c_void_p()
        rc = self.L.hg_create(ctypes.byref(h), ctypes.byref(opts))
        if rc != 0:
            raise HamsGpuError(rc, "hg_create failed (is a CUDA device present?)")
        self.h = h
        self.n = 0
        self.nbody = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.hg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise HamsGpuError(rc, self.L.hg_last_error(self.h).decode())
        return rc

    def set_mesh(self, nodes, ncon, ncn, xyz_p, ds, pnsz, dxyz_p, body_ranges, lid_xyz_p=None):
        """nodes (ntnd,3), ncon (n,4) 1-based, xyz_p (n,3), dxyz_p (n,6), body_ranges (nbody,2) 1-based."""
        f = lambda a, t=np.float64: np.asfortranarray(a, dtype=t)  # noqa: E731
        self._keep = [f(nodes), f(ncon, np.int32), np.ascontiguousarray(ncn, dtype=np.int32), f(xyz_p),
                      np.ascontiguousarray(ds, dtype=np.float64), np.ascontiguousarray(pnsz, dtype=np.float64),
                      f(dxyz_p)]
        lid = None if lid_xyz_p is None or len(lid_xyz_p) == 0 else f(lid_xyz_p)
        br = np.ascontiguousarray(np.asarray(body_ranges, dtype=np.int32).reshape(-1))
        n = len(self._keep[2])
        self._check(self.L.hg_set_mesh(self.h, n, len(self._keep[0]), *[_ptr(a) for a in self._keep],
                                       0 if lid is None else len(lid), _ptr(lid), len(br) // 2, _ptr(br)))
        self.n = n
        self.nbody = len(br) // 2
        self.nl = 0 if lid is None else len(lid)

    def set_frequency(self, v, wk, w1, h, wvn=None):
        w = None if wvn is None else np.ascontiguousarray(wvn, dtype=np.float64)
        self._check(self.L.hg_set_frequency(self.h, v, wk, w1, h, _ptr(w), 0 if w is None else len(w)))

    def fill_factor(self, irsp=0):
        return self._check(self.L.hg_fill_factor(self.h, irsp))

    def keep_matrices(self, keep=True):
        self._check(self.L.hg_keep_matrices(self.h, 1 if keep else 0))

    def get_matrix(self, which, rows):
        out = np.zeros((rows, self.n), dtype=np.complex128, order="F")
        self._check(self.L.hg_get_matrix(self.h, which, _ptr(out), rows))
        return out

    def solve_radiation(self):
        out = np.zeros((self.n, 6 * self.nbody), dtype=np.complex128, order="F")
        self._check(self.L.hg_solve_radiation(self.h, _ptr(out), self.n))
        self._ndif = 0
        return out

    def solve_all_headings(self, betas):
        b = np.ascontiguousarray(betas, dtype=np.float64)
        out = np.zeros((self.n, len(b)), dtype=np.complex128, order="F")
        self._check(self.L.hg_solve_all_headings(self.h, _ptr(b), len(b), _ptr(out), self.n))
        self._ndif = len(b)
        return out

    def solve_diffraction(self, beta):
        out = np.zeros(self.n, dtype=np.complex128)
        self._check(self.L.hg_solve_diffraction(self.h, float(beta), _ptr(out)))
        self._ndif = 1
        return out

    def forces(self, nbeta, isol=1):
        nd = 6 * self.nbody
        amas = np.zeros((nd, nd), order="F"); bdmp = np.zeros((nd, nd), order="F")
        exfc = np.zeros((max(nbeta, 1), nd), dtype=np.complex128, order="F")
        self._check(self.L.hg_forces(self.h, isol, _ptr(amas), _ptr(bdmp), _ptr(exfc)))
        return amas, bdmp, exfc[:nbeta]

    def solve_frequency(self, v, wk, w1, h, wvn, betas, irsp=0, isol=1, want_potentials=True, out=None):
        """One frequency-solve; returns (amas, bdmp, exfc, mxpot or None).

        ``out`` may hold preallocated (pinned) arrays to avoid allocations."""
        nd = 6 * self.nbody
        b = np.ascontiguousarray(betas, dtype=np.float64)
        nb = len(b)
        if out is None:
            out = {"amas": np.zeros((nd, nd), order="F"), "bdmp": np.zeros((nd, nd), order="F"),
                   "exfc": np.zeros((max(nb, 1), nd), dtype=np.complex128, order="F"),
                   "mxpot": np.zeros((self.n, nd + nb), dtype=np.complex128, order="F") if want_potentials else None}
        w = None if wvn is None or h <= 0 else np.ascontiguousarray(wvn, dtype=np.float64)
        mx = out.get("mxpot")
        self._check(self.L.hg_solve_frequency(self.h, v, wk, w1, h, _ptr(w), 0 if w is None else len(w), irsp,
                                              _ptr(b), nb, isol, _ptr(out["amas"]), _ptr(out["bdmp"]),
                                              _ptr(out["exfc"]), _ptr(mx), self.n))
        self._ndif = nb
        return out["amas"], out["bdmp"], out["exfc"][:nb], mx

    FIELD_POTENTIAL, FIELD_PRESSURE, FIELD_ELEVATION = 0, 1, 2

    def field_points(self, xyz, kind=0, isol=1):
        """Potential (kind 0), pressure (1) or elevation (2) at field points
        xyz (npts, 3) for every column of the last solve (hg_field_points):
        returns (npts, 6 nbody + nbeta) complex128."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(x), 6 * self.nbody + getattr(self, "_ndif", 0)), dtype=np.complex128, order="F")
        self._check(self.L.hg_field_points(self.h, len(x), _ptr(x), int(kind), int(isol), _ptr(out), max(len(x), 1)))
        return out

    def solve_sweep(self, v, wk, w1, h, wvn, betas, irsp=0, isol=1, nslots=1, out=None, want_potentials=False):
        """Frequency sweep over arrays v, wk, w1 (and wvn rows for finite depth)
        on nslots concurrent solve slots (hg_solve_sweep).

        Returns (amas[nfreq, nd, nd], bdmp, exfc[nfreq, nbeta, nd], latency_ms[nfreq],
        mxpot[nfreq, n, nd + nbeta] or None)."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        wk = np.ascontiguousarray(wk, dtype=np.float64)
        w1 = np.ascontiguousarray(w1, dtype=np.float64)
        nf = len(v)
        nd = 6 * self.nbody
        b = np.ascontiguousarray(betas, dtype=np.float64)
        nb = len(b)
        w = None
        nk = 0
        if h > 0 and wvn is not None:
            w = np.ascontiguousarray(wvn, dtype=np.float64).reshape(nf, -1)
            nk = w.shape[1]
        if out is None:
            out = {"amas": np.zeros((nf, nd, nd)), "bdmp": np.zeros((nf, nd, nd)),
                   "exfc": np.zeros((nf, nd, max(nb, 1)), dtype=np.complex128),
                   "lat": np.zeros(nf, dtype=np.float32),
                   "mxpot": np.zeros((nf, nd + nb, self.n), dtype=np.complex128) if want_potentials else None}
        mx = out.get("mxpot")
        self._check(self.L.hg_solve_sweep(self.h, nf, _ptr(v), _ptr(wk), _ptr(w1), float(h), _ptr(w), nk, irsp,
                                          _ptr(b), nb, isol, nslots, _ptr(out["amas"]), _ptr(out["bdmp"]),
                                          _ptr(out["exfc"]), _ptr(mx), self.n, _ptr(out["lat"])))
        # per frequency the arrays are column-major (Fortran): transpose the last two axes
        amas = out["amas"].transpose(0, 2, 1)
        bdmp = out["bdmp"].transpose(0, 2, 1)
        exfc = out["exfc"].transpose(0, 2, 1)[:, :nb, :]
        return amas, bdmp, exfc, out["lat"], None if mx is None else mx.transpose(0, 2, 1)

    def green_points(self, pts, flags):
        p = np.ascontiguousarray(pts, dtype=np.float64)
        fl = np.ascontiguousarray(flags, dtype=np.int32)
        out = np.zeros((len(fl), 8))
        self._check(self.L.hg_green_points(self.h, len(fl), _ptr(p), _ptr(fl), _ptr(out)))
        return out[:, 0::2] + 1j * out[:, 1::2]

    def green_points_noalloc(self, pts, flags):
        """hg_green_points through the entry point that allocates no device memory."""
        p = np.ascontiguousarray(pts, dtype=np.float64)
        fl = np.ascontiguousarray(flags, dtype=np.int32)
        out = np.zeros((len(fl), 8))
        self._check(self.L.hg_green_points_noalloc(self.h, len(fl), _ptr(p), _ptr(fl), _ptr(out)))
        return out[:, 0::2] + 1j * out[:, 1::2]

    def gesv(self, a, b, precision=HG_PREC_FP64):
        """Dense solve A X = B on the device (hg_gesv).

        Returns (lu, ipiv, x, iter, info): lu the n x n factors (unit-lower L
        below the diagonal, U on and above), ipiv 1-based LAPACK pivots."""
        lu = np.array(a, dtype=np.complex128, order="F", copy=True)
        n = lu.shape[0]
        bb = np.array(b, dtype=np.complex128, order="F", copy=True)
        if bb.ndim == 1:
            bb = bb.reshape(n, 1, order="F")
        ipiv = np.zeros(n, dtype=np.int32)
        it = ctypes.c_int(); info = ctypes.c_int()
        self._check(self.L.hg_gesv(self.h, precision, n, bb.shape[1], _ptr(lu), n, _ptr(ipiv), _ptr(bb), n,
                                   ctypes.byref(it), ctypes.byref(info)))
        return lu, ipiv, bb, it.value, info.value

    def gemm_check(self, variant, a, b, c):
        """C - A B through GEMM kernel `variant` (hg_gemm_check); complex128 in and out."""
        a = np.asfortranarray(a, dtype=np.complex128)
        b = np.asfortranarray(b, dtype=np.complex128)
        out = np.array(c, dtype=np.complex128, order="F", copy=True)
        m, k = a.shape
        n = b.shape[1]
        self._check(self.L.hg_gemm_check(self.h, variant, m, n, k, _ptr(a), m, _ptr(b), k, _ptr(out), m))
        return out

    def resid_check(self, variant, a, y, b):
        """b - A y through the refinement residual's kernel `variant` (hg_resid_check:
        0 double-float, 1 sliced on the tensor cores); A rounded to complex64 on the device."""
        a = np.asfortranarray(a, dtype=np.complex128)
        y = np.asfortranarray(y, dtype=np.complex128)
        b = np.asfortranarray(b, dtype=np.complex128)
        m, k = a.shape
        nc = y.shape[1]
        out = np.zeros((m, nc), dtype=np.complex128, order="F")
        self._check(self.L.hg_resid_check(self.h, variant, m, nc, k, _ptr(a), m, _ptr(y), k, _ptr(b), m, _ptr(out), m))
        return out

    def bench_gemm(self, variant, m, n, k, iters=3):
        ms = ctypes.c_float()
        self._check(self.L.hg_bench_gemm(self.h, variant, m, n, k, iters, ctypes.byref(ms)))
        return ms.value

    def bench_panel(self, m, iters=16):
        """Average ms of one complex64 32-column cluster panel LU of m rows."""
        ms = ctypes.c_float()
        self._check(self.L.hg_bench_panel(self.h, m, iters, ctypes.byref(ms)))
        return ms.value

    def gmres_iterations(self):
        it = ctypes.c_int()
        self.L.hg_gmres_iterations(self.h, ctypes.byref(it))
        return it.value

    def iter_info(self):
        """(iterations, restarts, unconverged columns, worst ||r||/||b||) of the last
        solve with solver = 2."""
        it, rs, un = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        r = ctypes.c_double()
        self._check(self.L.hg_iter_info(self.h, ctypes.byref(it), ctypes.byref(rs), ctypes.byref(un), ctypes.byref(r)))
        return it.value, rs.value, un.value, r.value

    def hmatrix_info(self):
        """(blocks, dense blocks, low-rank blocks, mean rank, compression) of the
        H-matrix of the last fill (solver = 2, hmatrix = 1)."""
        nb, nd, nl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        mr, cr = ctypes.c_double(), ctypes.c_double()
        self._check(self.L.hg_hmatrix_info(self.h, ctypes.byref(nb), ctypes.byref(nd), ctypes.byref(nl),
                                           ctypes.byref(mr), ctypes.byref(cr)))
        return nb.value, nd.value, nl.value, mr.value, cr.value

    def hmatrix_check(self, a, xyz, x):
        """H x through the device H-matrix of a (hg_hmatrix_check); xyz the n x 3
        panel centres.  Returns (y, (blocks, dense, low rank, sum of ranks))."""
        a = np.asfortranarray(a, dtype=np.complex128)
        n = a.shape[0]
        xyz = np.asfortranarray(xyz, dtype=np.float64)
        x = np.asfortranarray(x, dtype=np.complex128)
        if x.ndim == 1:
            x = x.reshape(n, 1, order="F")
        y = np.zeros(x.shape, dtype=np.complex128, order="F")
        st = np.zeros(4, dtype=np.int64)
        self._check(self.L.hg_hmatrix_check(self.h, n, _ptr(a), n, _ptr(xyz), x.shape[1], _ptr(x), _ptr(y), _ptr(st)))
        return y, tuple(int(v) for v in st)

    def refine_info(self):
        s = ctypes.c_int(); r = ctypes.c_double()
        self.L.hg_refine_info(self.h, ctypes.byref(s), ctypes.byref(r))
        return s.value, r.value

    def mark(self, slot):
        self._check(self.L.hg_mark(self.h, slot))

    def elapsed_ms(self, s0, s1):
        ms = ctypes.c_float()
        self._check(self.L.hg_elapsed(self.h, s0, s1, ctypes.byref(ms)))
        return ms.value

    def stage_times(self):
        a = (ctypes.c_float * 4)()
        self.L.hg_stage_times(self.h, a)
        return list(a)


def solve_footprint(precision, n, nl, nbody, nbeta, irsp=0, lu_tensor=2):
    """Device bytes one frequency-solve of this size holds (hg_solve_footprint)."""
    return int(load().hg_solve_footprint(precision, n, nl, nbody, nbeta, irsp, lu_tensor))


class Server:
    """Request server: continuous batching of frequency-solve requests (hg_server_*)."""

    def __init__(self, nslots=4, budget_bytes=150e9, precision=HG_PREC_MIXED, device=0, **opts_kw):
        self.L = load()
        opts = HgOpts()
        self.L.hg_default_opts(ctypes.byref(opts))
        opts.device, opts.precision = device, precision
        for k, v in opts_kw.items():
            setattr(opts, k, v)
        h = ctypes.c_void_p()
        rc = self.L.hg_server_create(ctypes.byref(h), ctypes.byref(opts), nslots, float(budget_bytes))
        if rc != 0:
            raise HamsGpuError(rc, "hg_server_create failed")
        self.h = h
        self._pending = {}

    def submit(self, mesh, h, v, wk, w1, wvn, betas, irsp=0, isol=1):
        """Queue one request (mesh as meshgen.Mesh; per-frequency wave state). Returns a ticket."""
        f = lambda a, t=np.float64: np.asfortranarray(a, dtype=t)  # noqa: E731
        keep = [f(mesh.nodes), f(mesh.ncon, np.int32), np.ascontiguousarray(mesh.ncn, dtype=np.int32), f(mesh.xyz_p),
                np.ascontiguousarray(mesh.ds, dtype=np.float64), np.ascontiguousarray(mesh.pnsz, dtype=np.float64),
                f(mesh.dxyz_p)]
        lid = mesh.lid_xyz_p if irsp == 1 else None
        lid = None if lid is None or len(lid) == 0 else f(lid)
        br = np.ascontiguousarray(np.asarray(mesh.body_ranges, dtype=np.int32).reshape(-1))
        vv = np.ascontiguousarray(v, dtype=np.float64)
        kk = np.ascontiguousarray(wk, dtype=np.float64)
        ww = np.ascontiguousarray(w1, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        wv = None
        nk = 0
        if h > 0 and wvn is not None:
            wv = np.ascontiguousarray(wvn, dtype=np.float64).reshape(len(vv), -1)
            nk = wv.shape[1]
        q = HgRequest(len(keep[2]), len(keep[0]), _ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]), _ptr(keep[3]),
                      _ptr(keep[4]), _ptr(keep[5]), _ptr(keep[6]), 0 if lid is None else len(lid), _ptr(lid),
                      len(br) // 2, _ptr(br), float(h), len(vv), _ptr(vv), _ptr(kk), _ptr(ww), _ptr(wv), nk, irsp,
                      isol, len(b), _ptr(b))
        t = ctypes.c_longlong()
        rc = self.L.hg_server_submit(self.h, ctypes.byref(q), ctypes.byref(t))
        if rc != 0:
            raise HamsGpuError(rc, self.L.hg_server_last_error(self.h).decode())
        self._pending[t.value] = (len(vv), len(br) // 2, len(b))
        return t.value

    def wait(self, ticket, timeout_s=0.0):
        """(amas[nfreq, nd, nd], bdmp, exfc[nfreq, nbeta, nd], latency_ms, admit_wait_ms), or None on timeout."""
        nf, nbody, nb = self._pending[ticket]
        nd = 6 * nbody
        amas = np.zeros((nf, nd, nd)); bdmp = np.zeros((nf, nd, nd))
        exfc = np.zeros((nf, nd, max(nb, 1)), dtype=np.complex128)
        lat = np.zeros(2)
        rc = self.L.hg_server_wait(self.h, ticket, float(timeout_s), _ptr(amas), _ptr(bdmp), _ptr(exfc), _ptr(lat))
        if rc == 1:
            return None
        del self._pending[ticket]
        if rc != 0:
            raise HamsGpuError(rc, self.L.hg_server_last_error(self.h).decode())
        return (amas.transpose(0, 2, 1), bdmp.transpose(0, 2, 1), exfc.transpose(0, 2, 1)[:, :nb, :], lat[0], lat[1])

    def stats(self):
        st = np.zeros(8)
        self.L.hg_server_stats(self.h, _ptr(st))
        keys = ["requests_done", "solves_done", "reserved_bytes", "peak_reserved_bytes", "max_admitted",
                "queued", "admitted", "budget_bytes"]
        return dict(zip(keys, st.tolist()))

    def timeline(self):
        """Device intervals of the finished frequency-solves: array of rows
        (ticket, frequency index, start ms, end ms), the times from CUDA
        events on each slot's stream, relative to the server's creation."""
        n = self.L.hg_server_timeline(self.h, 0, None)
        if n < 0:
            raise HamsGpuError(n, "hg_server_timeline failed")
        out = np.zeros((max(n, 1), 4))
        n = self.L.hg_server_timeline(self.h, n, _ptr(out))
        return out[:n]

    def close(self):
        if getattr(self, "h", None):
            self.L.hg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Case:
    """A HAMS input deck (ControlFile.in and meshes) read by the library
    (hg_case_*): inspect what was read, run every frequency on the GPU and
    write the HAMS- and WAMIT-format result files."""

    def __init__(self, input_dir):
        self.L = load()
        self.h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = self.L.hg_case_read(os.fsencode(input_dir), ctypes.byref(self.h), err, len(err))
        if rc != 0:
            self.h = None
            raise HamsGpuError(rc, err.value.decode())
        info = np.zeros(12, dtype=np.int32)
        dinfo = np.zeros(2)
        self.L.hg_case_info(self.h, _ptr(info), _ptr(dinfo))
        keys = ["n", "nl", "ntnd", "nbody", "nper", "nbeta", "irsp", "isol", "nfp", "sybo", "inft", "ouft"]
        self.info = {k: int(v) for k, v in zip(keys, info)}
        self.info["h"], self.info["refl"] = float(dinfo[0]), float(dinfo[1])
        isolv, sep = ctypes.c_int(), ctypes.c_int()
        self.L.hg_case_options(self.h, ctypes.byref(isolv), ctypes.byref(sep))
        self.info["isolv"], self.info["separate"] = isolv.value, sep.value

    def arrays(self):
        i = self.info
        n, nl, nt, nb, npr, nbeta = i["n"], i["nl"], i["ntnd"], i["nbody"], i["nper"], i["nbeta"]
        out = {"nodes": np.zeros((nt, 3), order="F"), "ncon": np.zeros((n, 4), dtype=np.int32, order="F"),
               "ncn": np.zeros(n, dtype=np.int32), "xyz_p": np.zeros((n, 3), order="F"), "ds": np.zeros(n),
               "pnsz": np.zeros(n), "dxyz_p": np.zeros((n, 6), order="F"), "lid_xyz_p": np.zeros((nl, 3), order="F"),
               "body_ranges": np.zeros((nb, 2), dtype=np.int32), "freq": np.zeros((npr, 6)),
               "headings": np.zeros(nbeta)}
        self.L.hg_case_arrays(self.h, *[_ptr(out[k]) for k in ("nodes", "ncon", "ncn", "xyz_p", "ds", "pnsz",
                                                                "dxyz_p", "lid_xyz_p", "body_ranges", "freq",
                                                                "headings")])
        return out

    def run(self, output_dir, precision=HG_PREC_FP64, nslots=2, device=0, **opts_kw):
        opts = HgOpts()
        self.L.hg_default_opts(ctypes.byref(opts))
        opts.device, opts.precision = device, precision
        for k, v in opts_kw.items():
            setattr(opts, k, v)
        err = ctypes.create_string_buffer(512)
        rc = self.L.hg_case_run(self.h, os.fsencode(output_dir), ctypes.byref(opts), int(nslots), err, len(err))
        if rc != 0:
            raise HamsGpuError(rc, err.value.decode())

    def write(self, output_dir, amas, bdmp, exfc, rho=1000.0, g=9.80665):
        """Result files from amas/bdmp (nper, nd, nd) and exfc (nper, nbeta, nd)."""
        a = np.ascontiguousarray(np.transpose(np.asarray(amas, dtype=np.float64), (0, 2, 1)))
        b = np.ascontiguousarray(np.transpose(np.asarray(bdmp, dtype=np.float64), (0, 2, 1)))
        f = np.ascontiguousarray(np.transpose(np.asarray(exfc, dtype=np.complex128), (0, 2, 1)))
        err = ctypes.create_string_buffer(512)
        rc = self.L.hg_case_write(self.h, os.fsencode(output_dir), _ptr(a), _ptr(b), _ptr(f), float(rho), float(g),
                                  err, len(err))
        if rc != 0:
            raise HamsGpuError(rc, err.value.decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.hg_case_free(self.h)
            self.h = None

    def __del__(self):
        self.close()
