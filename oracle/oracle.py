"""CPU oracle driver for the HAMS-MREL per-frequency path.

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use this module as the checker.  The product
library never imports it.

The pair loops (Green functions, Newman integrals, assembly, normal
equations, forces) run in ``liboracle.so`` (plain C restating the Fortran,
see ``hams_oracle.h``).  The dense solve is LAPACK ``zgetrf``/``zgetrs``
through scipy, the same routines the reference calls
(src/AssbMatx.f90:111, :277, :340).

Input parsing mirrors src/InputFiles.f90:46-224 (fixed-column
``ControlFile.in``), src/ReadPanelMesh*.f90 (``.pnl`` meshes, LCS
transform of src/ReadPanelMeshMulti.f90:48-52, generalized-mode normal
overrides :168-190) and src/CalGreenFuncMulti.f90:53-106 (body-major
global panel order).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = ["or_special.c", "or_green.c", "or_panel.c", "or_assemble.c"]

G = 9.80665
RHO = 1000.0
PI = 3.141592653589793
NK = 200


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (no fused multiply-add, OpenMP)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if not force and os.path.exists(LIB_PATH):
        newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "hams_oracle.h")])
        if os.path.getmtime(LIB_PATH) >= newest:
            return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_LIB = None
FMA_LIB_PATH = os.path.join(HERE, "_build", "liboracle_fma.so")


def build_fma_variant() -> str:
    """The same oracle compiled with fused multiply-add contraction.

    The finite-depth Green function of the reference extrapolates its series
    with Wynn's epsilon algorithm (src/FinGrnExtSubs.f90:370-503), which
    amplifies last-bit differences.  Comparing the oracle with this variant
    measures how far the reference's own results move under a different but
    equally valid rounding; the GPU parity tests of the finite-depth path are
    held to that spread."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if os.path.exists(FMA_LIB_PATH) and os.path.getmtime(FMA_LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
        return FMA_LIB_PATH
    os.makedirs(os.path.dirname(FMA_LIB_PATH), exist_ok=True)
    tmp = FMA_LIB_PATH + f".tmp{os.getpid()}"
    arch = ["-mfma"] if os.uname().machine == "x86_64" else []
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast"] + arch + ["-o", tmp] + srcs
                   + ["-lm"], check=True)
    os.replace(tmp, FMA_LIB_PATH)
    return FMA_LIB_PATH


class use_library:
    """Context manager: run the oracle functions with another build of liboracle."""

    def __init__(self, path):
        self.path = path

    def __enter__(self):
        global _LIB
        self.saved = _LIB
        _LIB = _configure(ctypes.CDLL(self.path))
        return self

    def __exit__(self, *exc):
        global _LIB
        _LIB = self.saved
        return False


def lib():
    global _LIB
    if _LIB is None:
        build()
        _LIB = _configure(ctypes.CDLL(LIB_PATH))
    return _LIB


def _configure(L):
    if True:
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.or_assemble.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.or_rhs_radiation.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ip, ip, ctypes.c_void_p]
        L.or_rhs_diffraction.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.or_normal_equations.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.or_normal_rhs.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]
        L.or_rforce.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double, ctypes.c_void_p,
                                ctypes.c_int, dp, dp]
        L.or_eforce.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                ctypes.c_void_p, ctypes.c_void_p]
        L.or_dispersion.argtypes = [dp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.or_geometry.argtypes = [ctypes.c_int, dp, ctypes.c_int, ip, ip, dp, dp, dp, dp, dp]
        L.or_pair.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int,
                              ctypes.c_double, ip, dp, ctypes.c_void_p]
        L.or_green_point.argtypes = [ctypes.c_double] * 7 + [dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp]
        L.or_sglintbd.argtypes = [dp, ctypes.c_int, dp, dp, dp]
        L.or_fingreen_region.argtypes = [ctypes.c_double, ctypes.c_double]
        L.or_fingreen_region.restype = ctypes.c_int
        L.or_vinp.argtypes = [ctypes.c_double] * 8
        L.or_vinp.restype = ctypes.c_double * 2
        L.or_field_potential.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ip, ip,
                                         ctypes.c_int, dp, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_void_p]
    return L


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# ---------------------------------------------------------------------------
# Input files
# ---------------------------------------------------------------------------
def _fortran_real(s: str, decimals: int = 15) -> float:
    """Fortran Fw.d input under the default BLANK='NULL' mode: blanks inside
    the field are ignored, an all-blank field reads as zero, a D exponent is
    accepted and a field without a point has ``decimals`` implied decimals."""
    t = s.replace(" ", "").replace("D", "E").replace("d", "e")
    if not t:
        return 0.0
    if "." in t or "E" in t or "e" in t:
        return float(t)
    return int(t) / (10 ** decimals)


def _fixed(line: str, skip: int, width: int) -> str:
    return line[skip:skip + width]


@dataclass
class Control:
    h: float
    sybo: int
    inft: int
    ouft: int
    wvnb: list
    nbody: int
    lcs: list
    headings: list
    xr: list
    refl: float
    isol: int
    irsp: int
    nthread: int
    isolv: int = 1


def read_control_file(path: str) -> Control:
    """Mirror of ReadControlFile, src/InputFiles.f90:46-224."""
    with open(path) as f:
        lines = f.read().split("\n")
    it = iter(lines)
    nxt = lambda: next(it)  # noqa: E731
    nxt(); nxt()
    h = _fortran_real(_fixed(nxt(), 14, 30))
    nxt(); nxt()
    sybo = int(_fixed(nxt(), 27, 16))
    inft = int(_fixed(nxt(), 25, 16))
    ouft = int(_fixed(nxt(), 25, 17))
    npet = int(_fixed(nxt(), 26, 16))
    ifs = 2 if sybo == 1 else 0
    wvnb = [0.0] * ifs
    if npet > 0:
        vals = []
        while len(vals) < npet:
            vals += [_fortran_real(t) for t in nxt().split()]
        wvnb += vals[:npet]
    elif npet < 0:
        npet = -npet
        wk1 = _fortran_real(_fixed(nxt(), 27, 30))
        dwk = _fortran_real(_fixed(nxt(), 19, 30))
        wvnb += [wk1 + (i - ifs - 1) * dwk for i in range(ifs + 1, ifs + npet + 1)]
    nxt(); nxt()
    body_check = nxt()
    nbody = int(_fixed(nxt(), 24, 16)) if "multi" in body_check else 1
    lcs = []
    if nbody > 1:
        for _ in range(nbody):
            ln = nxt()
            lcs.append([_fortran_real(_fixed(ln, 26 + 12 * k, 12), 3) for k in range(4)])
        nxt(); nxt(); nxt()
    nbeta = int(_fixed(nxt(), 23, 16))
    if nbeta > 0:
        vals = []
        while len(vals) < nbeta:
            vals += [_fortran_real(t) for t in nxt().split()]
        heads = vals[:nbeta]
    else:
        nbeta = -nbeta
        b1 = _fortran_real(_fixed(nxt(), 20, 30))
        db = _fortran_real(_fixed(nxt(), 17, 30))
        heads = [b1 + i * db for i in range(nbeta)]
    nxt(); nxt()
    xr = []
    for _ in range(nbody):
        ln = nxt()
        xr.append([_fortran_real(_fixed(ln, 28 + 12 * k, 12), 3) for k in range(3)])
    refl = _fortran_real(_fixed(nxt(), 26, 30))
    isol = int(_fixed(nxt(), 26, 16))
    irsp = int(_fixed(nxt(), 23, 16))
    nthread = int(_fixed(nxt(), 23, 16))
    isolv = 1
    ln = nxt()
    if "Solver_type" in ln:
        try:
            isolv = int(_fixed(ln, 26, 16))
        except ValueError:
            isolv = 1
    return Control(h, sybo, inft, ouft, wvnb, nbody, lcs, heads, xr, refl, isol, irsp, nthread, isolv)


@dataclass
class Pnl:
    nodes: np.ndarray    # (ntnd, 3)
    ncn: np.ndarray      # (nelem,)
    ncon: np.ndarray     # (nelem, 4), 1-based
    isx: int
    isy: int


def read_pnl(path: str, lcs=None, lid: bool = False) -> Pnl:
    """Mirror of ReadBodyMesh(Multi) / ReadWTPLMesh(Multi)."""
    with open(path) as f:
        lines = f.read().split("\n")
    nelem, ntnd, isx, isy = [int(t) for t in lines[3].split()[:4]]
    nodes = np.zeros((ntnd, 3))
    p = 6
    for i in range(ntnd):
        t = lines[p + i].split()
        x, y, z = float(t[1]), float(t[2]), float(t[3])
        if lid and abs(z) > 1.0e-10:
            raise ValueError(f"Z coordinate is not zero at node {i + 1}")
        if lcs is not None:
            c, s = math.cos(lcs[3]), math.sin(lcs[3])
            x, y = 0.0 + lcs[0] + c * x - s * y, 0.0 + lcs[1] + s * x + c * y
        nodes[i] = (x, y, z)
    p += ntnd + 3
    ncn = np.zeros(nelem, dtype=np.int32)
    ncon = np.zeros((nelem, 4), dtype=np.int32)
    for e in range(nelem):
        t = [int(v) for v in lines[p + e].split()]
        ncn[e] = t[1]
        ncon[e, :t[1]] = t[2:2 + t[1]]
        if t[1] == 3:
            ncon[e, 3] = ncon[e, 0]
    return Pnl(nodes, ncn, ncon, isx, isy)


def geometry(pnl: Pnl, xr):
    L = lib()
    n = len(pnl.ncn)
    nodes = np.ascontiguousarray(pnl.nodes, dtype=np.float64)
    ncn = np.ascontiguousarray(pnl.ncn, dtype=np.int32)
    ncon = np.ascontiguousarray(pnl.ncon, dtype=np.int32)
    xr = np.asarray(xr, dtype=np.float64)
    xyz_p = np.zeros((n, 3)); ds = np.zeros(n); pnsz = np.zeros(n); dxyz = np.zeros((n, 6))
    L.or_geometry(len(nodes), _dp(nodes), n, _ip(ncn), _ip(ncon), _dp(xr), _dp(xyz_p), _dp(ds),
                  _dp(pnsz), _dp(dxyz))
    return xyz_p, ds, pnsz, dxyz


@dataclass
class Case:
    ctl: Control
    nodes: np.ndarray
    ncn: np.ndarray
    ncon: np.ndarray
    xyz_p: np.ndarray
    ds: np.ndarray
    pnsz: np.ndarray
    dxyz_p: np.ndarray
    body_start: np.ndarray
    body_end: np.ndarray
    lid_xyz_p: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))

    @property
    def n(self):
        return len(self.ncn)

    @property
    def nl(self):
        return len(self.lid_xyz_p)

    @property
    def nbody(self):
        return len(self.body_start)


def load_case(inputdir: str) -> Case:
    """Read ControlFile.in and the meshes, compute the panel geometry and
    pack bodies in the global order of BuildCombinedArrays."""
    ctl = read_control_file(os.path.join(inputdir, "ControlFile.in"))
    nodes_all, ncn_all, ncon_all, xyz, ds, pnsz, dxyz, lids = [], [], [], [], [], [], [], []
    starts, ends = [], []
    node_base = 0
    elem_base = 0
    for b in range(ctl.nbody):
        if ctl.nbody == 1:
            hull = os.path.join(inputdir, "HullMesh.pnl")
            wpl = os.path.join(inputdir, "WaterPlaneMesh.pnl")
            lcs = None
        else:
            hull = os.path.join(inputdir, f"HullMesh_{b + 1}.pnl")
            wpl = os.path.join(inputdir, f"WaterPlaneMesh_{b + 1}.pnl")
            lcs = ctl.lcs[b]
        pnl = read_pnl(hull, lcs)
        xp, a, sz, nv = geometry(pnl, ctl.xr[b])
        # generalized modes (ReadPanelMesh.f90:135-160, ReadPanelMeshMulti.f90:168-190)
        for dof in range(1, 7):
            gname = os.path.join(inputdir, f"gen_mod_{b + 1}_{dof}.txt")
            if os.path.exists(gname):
                with open(gname) as f:
                    for k, ln in enumerate(f):
                        if k >= len(pnl.ncn):
                            break
                        t = ln.split()
                        if len(t) < 2:
                            break
                        nv[int(t[0]) - 1, dof - 1] = float(t[1].replace("D", "E"))
        nodes_all.append(pnl.nodes)
        ncn_all.append(pnl.ncn)
        ncon_all.append(pnl.ncon + node_base)
        xyz.append(xp); ds.append(a); pnsz.append(sz); dxyz.append(nv)
        starts.append(elem_base)
        elem_base += len(pnl.ncn)
        ends.append(elem_base)
        node_base += len(pnl.nodes)
        if ctl.irsp == 1 and os.path.exists(wpl):
            lp = read_pnl(wpl, lcs, lid=True)
            lxp, _, _, _ = geometry(lp, ctl.xr[b])
            lids.append(lxp)
    return Case(ctl, np.concatenate(nodes_all), np.concatenate(ncn_all).astype(np.int32),
                np.concatenate(ncon_all).astype(np.int32), np.concatenate(xyz), np.concatenate(ds),
                np.concatenate(pnsz), np.concatenate(dxyz), np.array(starts, dtype=np.int32),
                np.array(ends, dtype=np.int32),
                np.concatenate(lids) if lids else np.zeros((0, 3)))


class _Mesh(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("nl", ctypes.c_int), ("ntnd", ctypes.c_int), ("ntnd_lid", ctypes.c_int),
                ("nodes", ctypes.c_void_p), ("ncn", ctypes.c_void_p), ("ncon", ctypes.c_void_p),
                ("xyz_p", ctypes.c_void_p), ("ds", ctypes.c_void_p), ("pnsz", ctypes.c_void_p),
                ("dxyz_p", ctypes.c_void_p), ("lid_xyz_p", ctypes.c_void_p)]


def _mesh_struct(case: Case):
    keep = [np.ascontiguousarray(a) for a in (case.nodes, case.ncn, case.ncon, case.xyz_p, case.ds,
                                               case.pnsz, case.dxyz_p, case.lid_xyz_p)]
    m = _Mesh(case.n, case.nl, len(case.nodes), 0, *[k.ctypes.data for k in keep])
    return m, keep


# ---------------------------------------------------------------------------
# Wave properties (CalWaveProperts, src/ImplementSubs.f90:40-151)
# ---------------------------------------------------------------------------
def dispersion(w: float, h: float) -> np.ndarray:
    wvn = np.zeros(NK)
    lib().or_dispersion(_dp(wvn), NK, float(w), float(h))
    return wvn


def wave_properties(ctl: Control, value: float):
    """Return (v, wk, w1, wvn) for one entry of the frequency list."""
    h = ctl.h
    wvn = np.zeros(NK)
    if ctl.inft == 1:
        v = value
        w1 = math.sqrt(G * v)
        if h <= 0.0:
            wk = v
        else:
            wvn = dispersion(w1, h); wk = wvn[0]
    elif ctl.inft == 2:
        wk = value
        v = wk if h <= 0.0 else wk * math.tanh(wk * h)
        w1 = math.sqrt(G * v)
        if h > 0.0:
            wvn = dispersion(w1, h)
    elif ctl.inft == 3:
        w1 = value
        v = w1 * w1 / G
        if h <= 0.0:
            wk = v
        else:
            wvn = dispersion(w1, h); wk = wvn[0]
    elif ctl.inft == 4:
        w1 = 2.0 * PI / value
        v = w1 * w1 / G
        if h <= 0.0:
            wk = v
        else:
            wvn = dispersion(w1, h); wk = wvn[0]
    else:
        wk = 2.0 * PI / value
        v = wk if h <= 0.0 else wk * math.tanh(wk * h)
        w1 = math.sqrt(G * v)
        if h > 0.0:
            wvn = dispersion(w1, h)
    return v, wk, w1, wvn


# ---------------------------------------------------------------------------
# One frequency
# ---------------------------------------------------------------------------
@dataclass
class FreqResult:
    w1: float
    wk: float
    amas: np.ndarray     # (6NB, 6NB)
    bdmp: np.ndarray     # (6NB, 6NB)
    exfc: np.ndarray     # (nbeta, 6NB) complex
    mxpot: np.ndarray    # (N, 6NB + nbeta) complex


def assemble(case: Case, v: float, wvn: np.ndarray, grn_kind: int = 8, nthreads: int = 0):
    """Return (A, S) as Fortran-ordered (tn, n) complex arrays."""
    L = lib()
    tn, n = case.n + case.nl, case.n
    A = np.zeros((tn, n), dtype=np.complex128, order="F")
    S = np.zeros((tn, n), dtype=np.complex128, order="F")
    m, keep = _mesh_struct(case)
    wv = np.ascontiguousarray(wvn, dtype=np.float64)
    L.or_assemble(ctypes.byref(m), float(v), _dp(wv), len(wv), float(case.ctl.h), grn_kind, nthreads,
                  A.ctypes.data, S.ctypes.data)
    del keep
    return A, S


def rhs(case: Case, S: np.ndarray, v, wk, w1, betas_rad):
    L = lib()
    tn = case.n + case.nl
    m, keep = _mesh_struct(case)
    nb = case.nbody
    B = np.zeros((tn, 6 * nb + len(betas_rad)), dtype=np.complex128, order="F")
    st = np.ascontiguousarray(case.body_start); en = np.ascontiguousarray(case.body_end)
    L.or_rhs_radiation(ctypes.byref(m), S.ctypes.data, nb, _ip(st), _ip(en), B.ctypes.data)
    for k, b in enumerate(betas_rad):
        col = np.zeros(tn, dtype=np.complex128)
        L.or_rhs_diffraction(ctypes.byref(m), S.ctypes.data, float(b), float(v), float(wk), float(w1),
                             float(case.ctl.h), col.ctypes.data)
        B[:, 6 * nb + k] = col
    del keep
    return B


def lu_solve(M: np.ndarray, B: np.ndarray) -> np.ndarray:
    """ZGETRF + ZGETRS (LAPACK through scipy), as the reference does."""
    from scipy.linalg import lapack
    lu, piv, info = lapack.zgetrf(M)
    if info != 0:
        raise np.linalg.LinAlgError(f"zgetrf info={info}")
    x, info = lapack.zgetrs(lu, piv, B)
    if info != 0:
        raise np.linalg.LinAlgError(f"zgetrs info={info}")
    return x


def gmres_precond(M: np.ndarray, blocks=None):
    """The right preconditioner of the reference's GMRES, as a function
    r -> z.  blocks None: Jacobi, z = r / diag(M) with 1 where |M_ii| < 1e-30
    (SETUP_PRECONDITIONER, src/IterativeSolvers.f90:156-174, and
    APPLY_PRECONDITIONER :296-304).  blocks [(start, size), ...]: LU factors
    of each diagonal block (SETUP_BLOCK_PRECONDITIONER :190-262; APPLY
    :276-293)."""
    from scipy.linalg import lapack
    if blocks is None:
        d = np.diag(M).astype(np.complex128).copy()
        d[np.abs(d) < 1e-30] = 1.0
        return lambda r: r / d
    facs = []
    for s0, sz in blocks:
        lu, piv, _ = lapack.zgetrf(np.asfortranarray(M[s0:s0 + sz, s0:s0 + sz]))
        facs.append((s0, sz, lu, piv))

    def apply(r):
        z = np.array(r, dtype=np.complex128)
        for s0, sz, lu, piv in facs:
            z[s0:s0 + sz], _ = lapack.zgetrs(lu, piv, z[s0:s0 + sz])
        return z
    return apply


def _givens(a, b):
    """ZGIVENS_ROTATION (src/IterativeSolvers.f90:490-530)."""
    if abs(b) < 1e-300:
        return 1.0 + 0j, 0j
    if abs(a) < 1e-300:
        return 0j, 1.0 + 0j
    den = math.sqrt(abs(a) ** 2 + abs(b) ** 2)
    return abs(a) / den + 0j, (a / abs(a)) * np.conj(b) / den


def gmres_solve(M: np.ndarray, b: np.ndarray, precond, tol=1e-4, maxit=100, restart=25):
    """ZGMRES_SOLVE (src/IterativeSolvers.f90:324-488): restarted GMRES(m)
    with right preconditioning, modified Gram-Schmidt and Givens rotations,
    x0 = 0, stop when ||r||_2 / ||b||_2 < tol or after maxit Arnoldi steps.
    Returns (x, iterations, info) with info 0 converged, 1 not."""
    n = M.shape[0]
    x = np.zeros(n, dtype=np.complex128)
    bnorm = np.linalg.norm(b)
    if bnorm < 1e-30:
        return x, 0, 0
    it, info = 0, 1
    while it < maxit:
        r = b.copy() if it == 0 else b - M @ x
        beta = np.linalg.norm(r)
        if beta / bnorm < tol:
            info = 0
            break
        V = np.zeros((n, restart + 1), dtype=np.complex128)
        H = np.zeros((restart + 1, restart), dtype=np.complex128)
        cs = np.zeros(restart, dtype=np.complex128)
        sn = np.zeros(restart, dtype=np.complex128)
        g = np.zeros(restart + 1, dtype=np.complex128)
        V[:, 0] = r / beta
        g[0] = beta
        mact = 0
        for j in range(restart):
            it += 1
            if it > maxit:
                break
            w = M @ precond(V[:, j])
            for i in range(j + 1):
                H[i, j] = np.vdot(V[:, i], w)
                w = w - H[i, j] * V[:, i]
            H[j + 1, j] = np.linalg.norm(w)
            if abs(H[j + 1, j]) > 1e-30:
                V[:, j + 1] = w / H[j + 1, j]
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -np.conj(sn[i]) * H[i, j] + np.conj(cs[i]) * H[i + 1, j]
                H[i, j] = t
            cs[j], sn[j] = _givens(H[j, j], H[j + 1, j])
            H[j, j] = cs[j] * H[j, j] + sn[j] * H[j + 1, j]
            H[j + 1, j] = 0
            t = cs[j] * g[j] + sn[j] * g[j + 1]
            g[j + 1] = -np.conj(sn[j]) * g[j] + np.conj(cs[j]) * g[j + 1]
            g[j] = t
            mact = j + 1
            if abs(g[j + 1]) / bnorm < tol:
                info = 0
                break
        if mact > 0:
            y = g[:mact].copy()
            for i in range(mact - 1, -1, -1):
                y[i] = 0 if abs(H[i, i]) < 1e-30 else y[i] / H[i, i]
                y[:i] -= H[:i, i] * y[i]
            for j in range(mact):
                x += y[j] * precond(V[:, j])
        if info == 0:
            break
    return x, min(it, maxit), info


# ---------------------------------------------------------------------------
# H-matrix compression of the iterative solver (ISOLV = 2): src/HMatrix.f90
# ---------------------------------------------------------------------------
HM_NLEAF, HM_ETA, HM_ACA_TOL, HM_RANK_MAX = 32, 2.0, 1.0e-4, 50  # src/HMatrix.f90:58-61


@dataclass
class HMat:
    """The H-matrix of src/HMatrix.f90: cluster order ``perm`` (cluster
    position -> original index, 0-based) and blocks in build order, each
    ``(rs, nr, cs, nc, D)`` (dense) or ``(rs, nr, cs, nc, U, VH)`` (low rank)
    with rows/columns as 0-based positions in cluster order."""
    perm: np.ndarray
    blocks: list
    tree: list


def hmatrix_clusters(xyz: np.ndarray, nleaf: int = HM_NLEAF):
    """SPLIT_CLUSTER_ITERATIVE (src/HMatrix.f90:236-381): geometric bisection
    at the middle of the longest bounding-box side, explicit stack, left
    child first.  xyz is N x 3.  Returns (tree, perm): tree nodes as dicts
    (start, end inclusive, 0-based; left/right child node indices or -1;
    center; diameter)."""
    n = xyz.shape[0]
    w = np.array(xyz, dtype=np.float64, copy=True)
    perm = np.arange(n)
    tree = []
    stack = [(0, n - 1, -1, 0)]
    while stack:
        i0, i1, parent, side = stack.pop()
        size = i1 - i0 + 1
        if size <= 0:
            continue
        node = len(tree)
        tree.append({"start": i0, "end": i1, "left": -1, "right": -1})
        if parent >= 0:
            tree[parent]["left" if side == 1 else "right"] = node
        bmin = w[i0].copy()
        bmax = w[i0].copy()
        cx = cy = cz = 0.0
        for j in range(i0, i1 + 1):
            for d in range(3):
                if w[j, d] < bmin[d]:
                    bmin[d] = w[j, d]
                if w[j, d] > bmax[d]:
                    bmax[d] = w[j, d]
            cx += w[j, 0]
            cy += w[j, 1]
            cz += w[j, 2]
        tree[node]["center"] = (cx / size, cy / size, cz / size)
        blen = bmax - bmin
        tree[node]["diameter"] = math.sqrt(blen[0] ** 2 + blen[1] ** 2 + blen[2] ** 2)
        if size <= nleaf:
            continue
        dim = 0
        if blen[1] > blen[dim]:
            dim = 1
        if blen[2] > blen[dim]:
            dim = 2
        split = 0.5 * (bmin[dim] + bmax[dim])
        i, j = i0, i1
        while i <= j:
            if w[i, dim] <= split:
                i += 1
            else:
                w[[i, j]] = w[[j, i]]
                perm[[i, j]] = perm[[j, i]]
                j -= 1
        left_end = i - 1
        if left_end < i0:
            left_end = i0
        if left_end >= i1:
            left_end = i1 - 1
        stack.append((left_end + 1, i1, node, 2))
        stack.append((i0, left_end, node, 1))
    return tree, perm


def hmatrix_block_list(tree, eta: float = HM_ETA):
    """BUILD_BLOCK_TREE_ITERATIVE (src/HMatrix.f90:390-497): block pairs in
    the reference's traversal order, each (row node, col node, admissible)."""
    out = []
    stack = [(0, 0)]
    while stack:
        r, c = stack.pop()
        tr, tc = tree[r], tree[c]
        nr = tr["end"] - tr["start"] + 1
        nc = tc["end"] - tc["start"] + 1
        if nr <= 0 or nc <= 0:
            continue
        dist = math.sqrt((tr["center"][0] - tc["center"][0]) ** 2 + (tr["center"][1] - tc["center"][1]) ** 2 +
                         (tr["center"][2] - tc["center"][2]) ** 2)
        if dist > eta * max(tr["diameter"], tc["diameter"]) and nr > 1 and nc > 1:
            out.append((r, c, True))
            continue
        leaf_r, leaf_c = tr["left"] < 0, tc["left"] < 0
        if leaf_r and leaf_c:
            out.append((r, c, False))
            continue
        if leaf_r:
            stack += [(r, tc["right"]), (r, tc["left"])]
        elif leaf_c:
            stack += [(tr["right"], c), (tr["left"], c)]
        else:
            stack += [(tr["right"], tc["right"]), (tr["right"], tc["left"]), (tr["left"], tc["right"]),
                      (tr["left"], tc["left"])]
    return out


def hmatrix_aca(Ab: np.ndarray, tol: float = HM_ACA_TOL, rank_max: int = HM_RANK_MAX):
    """ADD_LOWRANK_BLOCK's partially pivoted ACA (src/HMatrix.f90:560-750) on
    the block Ab (NR x NC, cluster order).  Returns (U, VH) or None when the
    block is kept dense.  The stopping test uses the exact
    ||U V^H||_F^2 update, 2 Re sum_l (u_l^H u_k)(v_k^H v_l): the reference's
    cross term (:712-719) sums Re(conj(U(j,l)) U(j,k)) Re(conj(VH(k,j))
    VH(l,j)) over j = 1..NR for both factors, reading past VH's NC columns
    when NR > NC."""
    nr, nc = Ab.shape
    kmax = min(rank_max, nr, nc)
    if nr <= 4 or nc <= 4:
        return None
    U = np.zeros((nr, kmax), dtype=np.complex128)
    VH = np.zeros((kmax, nc), dtype=np.complex128)
    used = np.zeros(nr, dtype=bool)
    frob = 0.0
    rank = 0
    for k in range(kmax):
        if k == 0:
            pr = 0
        else:
            mags = np.abs(U[:, k - 1])
            mags[used] = -1.0
            pr = int(np.argmax(mags))
            if mags[pr] < 0.0:
                break
        used[pr] = True
        row = Ab[pr, :].astype(np.complex128)
        for l in range(k):
            row = row - U[pr, l] * VH[l, :]
        pc = int(np.argmax(np.abs(row)))
        pe = row[pc]
        if abs(pe) < 1.0e-30:
            break
        col = Ab[:, pc].astype(np.complex128)
        for l in range(k):
            col = col - U[:, l] * VH[l, pc]
        U[:, k] = col / pe
        VH[k, :] = row
        rank = k + 1
        uv = math.sqrt(float(np.sum(np.abs(U[:, k]) ** 2))) * math.sqrt(float(np.sum(np.abs(VH[k, :]) ** 2)))
        frob += uv * uv
        for l in range(k):
            frob += 2.0 * float(np.real(np.vdot(U[:, l], U[:, k]) * np.vdot(VH[l, :], VH[k, :])))
        if uv < tol * math.sqrt(max(frob, 1.0e-30)):
            break
    if rank == 0 or rank * (nr + nc) >= nr * nc:
        return None
    return U[:, :rank].copy(), VH[:rank, :].copy()


def hmatrix_build(M: np.ndarray, xyz: np.ndarray) -> HMat:
    """HMATRIX_BUILD (src/HMatrix.f90:135-196) of the assembled matrix M
    (N x N) with panel centres xyz (N x 3)."""
    tree, perm = hmatrix_clusters(xyz)
    blocks = []
    for r, c, adm in hmatrix_block_list(tree):
        rs, cs = tree[r]["start"], tree[c]["start"]
        nr, nc = tree[r]["end"] - rs + 1, tree[c]["end"] - cs + 1
        Ab = M[np.ix_(perm[rs:rs + nr], perm[cs:cs + nc])]
        lr = hmatrix_aca(Ab) if adm else None
        blocks.append((rs, nr, cs, nc, Ab.astype(np.complex128)) if lr is None else (rs, nr, cs, nc) + lr)
    return HMat(perm=perm, blocks=blocks, tree=tree)


def hmatvec(H: HMat, x: np.ndarray) -> np.ndarray:
    """HMATVEC (src/HMatrix.f90:760-820): y = H x for one or more columns."""
    xp = x[H.perm]
    yp = np.zeros(xp.shape, dtype=np.complex128)
    for b in H.blocks:
        rs, nr, cs, nc = b[:4]
        if len(b) == 5:
            yp[rs:rs + nr] += b[4] @ xp[cs:cs + nc]
        else:
            yp[rs:rs + nr] += b[4] @ (b[5] @ xp[cs:cs + nc])
    y = np.empty_like(yp)
    y[H.perm] = yp
    return y


def gmres_columns(M: np.ndarray, B: np.ndarray, blocks=None, **kw):
    """ZBLOCK_GMRES_SOLVE (src/IterativeSolvers.f90:535-562): every column
    separately with the same preconditioner.  Returns (X, iterations per
    column, info per column)."""
    P = gmres_precond(M, blocks)
    X = np.zeros(B.shape, dtype=np.complex128)
    its, infos = [], []
    for k in range(B.shape[1]):
        X[:, k], it, info = gmres_solve(M, B[:, k], P, **kw)
        its.append(it)
        infos.append(info)
    return X, its, infos


def normal_equations(case: Case, A: np.ndarray, B: np.ndarray):
    L = lib()
    tn, n = A.shape
    C = np.zeros((n, n), dtype=np.complex128, order="F")
    D = np.zeros((n, B.shape[1]), dtype=np.complex128, order="F")
    Af = np.asfortranarray(A); Bf = np.asfortranarray(B)
    L.or_normal_equations(tn, n, Af.ctypes.data, C.ctypes.data)
    L.or_normal_rhs(tn, n, Af.ctypes.data, B.shape[1], Bf.ctypes.data, D.ctypes.data)
    return C, D


def field_potential(case: Case, xf: np.ndarray, v, wk, w1, wvn, betas_rad, mxpot: np.ndarray, isol=None):
    """CalPotential(Multi) (src/PressureElevation.f90:53-250) at field points
    xf (npts, 3) for every column of mxpot (n x (6 nbody + nbeta)): returns
    pot (npts, 6 nbody + nbeta)."""
    L = lib()
    m, keep = _mesh_struct(case)
    npts = len(xf)
    x = np.ascontiguousarray(xf, dtype=np.float64)
    b = np.ascontiguousarray(betas_rad, dtype=np.float64)
    phi = np.asfortranarray(mxpot, dtype=np.complex128)
    ncol = phi.shape[1]
    out = np.zeros((npts, ncol), dtype=np.complex128, order="F")
    st = np.ascontiguousarray(case.body_start); en = np.ascontiguousarray(case.body_end)
    w = np.ascontiguousarray(wvn if wvn is not None else np.zeros(1), dtype=np.float64)
    L.or_field_potential(ctypes.byref(m), npts, _dp(x), float(v), float(wk), float(w1), _dp(w),
                         len(w) if wvn is not None else 0, float(case.ctl.h), case.nbody, _ip(st), _ip(en),
                         len(b), _dp(b), case.ctl.isol if isol is None else isol, phi.ctypes.data, phi.shape[0],
                         out.ctypes.data)
    del keep
    return out


def forces(case: Case, mxpot: np.ndarray, v, wk, w1, betas_rad):
    L = lib()
    nb = case.nbody
    amas = np.zeros((6 * nb, 6 * nb)); bdmp = np.zeros((6 * nb, 6 * nb))
    exfc = np.zeros((len(betas_rad), 6 * nb), dtype=np.complex128)
    ds = np.ascontiguousarray(case.ds); dx = np.ascontiguousarray(case.dxyz_p)
    xp = np.ascontiguousarray(case.xyz_p)
    phi = np.asfortranarray(mxpot)
    n = mxpot.shape[0]
    for bm in range(nb):
        i0, i1 = int(case.body_start[bm]), int(case.body_end[bm])
        for bn in range(nb):
            a = np.zeros(36); b = np.zeros(36)
            sub = np.asfortranarray(phi[:, 6 * bn:6 * bn + 6])
            L.or_rforce(i0, i1, _dp(ds), _dp(dx), float(w1), sub.ctypes.data, n, _dp(a), _dp(b))
            amas[6 * bm:6 * bm + 6, 6 * bn:6 * bn + 6] = a.reshape(6, 6)
            bdmp[6 * bm:6 * bm + 6, 6 * bn:6 * bn + 6] = b.reshape(6, 6)
        for k, beta in enumerate(betas_rad):
            e = np.zeros(6, dtype=np.complex128)
            col = np.ascontiguousarray(phi[:, 6 * nb + k])
            L.or_eforce(i0, i1, _dp(xp), _dp(ds), _dp(dx), float(w1), float(beta), float(v), float(wk),
                        float(case.ctl.h), int(case.ctl.isol), col.ctypes.data, e.ctypes.data)
            exfc[k, 6 * bm:6 * bm + 6] = e
    return amas, bdmp, exfc


def body_blocks(case: Case):
    """Diagonal blocks of the block preconditioner: one per body's hull
    panels (NELEM_MULTI), none for a single body (Jacobi)."""
    if case.nbody == 1:
        return None
    return [(int(case.body_start[b]), int(case.body_end[b] - case.body_start[b])) for b in range(case.nbody)]


def solve_frequency(case: Case, value: float, grn_kind: int = 8, nthreads: int = 0,
                    betas_deg=None, solver: int = 1) -> FreqResult:
    """One frequency; solver 1 = ZGETRF/ZGETRS, 2 = the GMRES of ISOLV = 2."""
    v, wk, w1, wvn = wave_properties(case.ctl, value)
    if betas_deg is None:
        betas_deg = case.ctl.headings
    betas = [b * PI / 180.0 for b in betas_deg]
    A, S = assemble(case, v, wvn, grn_kind, nthreads)
    B = rhs(case, S, v, wk, w1, betas)
    if case.nl > 0:
        M, R = normal_equations(case, A, B)
    else:
        M, R = np.asfortranarray(A), np.asfortranarray(B)
    if solver == 2:
        X = gmres_columns(M, R, body_blocks(case))[0]
    else:
        X = lu_solve(M, R)
    amas, bdmp, exfc = forces(case, X, v, wk, w1, betas)
    return FreqResult(w1, wk, amas, bdmp, exfc, X)


# ---------------------------------------------------------------------------
# HAMS text output (RFORCE_MULTI / EFORCE_MULTI line layout)
# ---------------------------------------------------------------------------
def read_hams_rows(path: str) -> np.ndarray:
    """Rows of an OAMASS/ODAMPING/OEXFOR file as floats (WK, W1, values...)."""
    rows = []
    with open(path) as f:
        for ln in f:
            t = ln.split()
            if t:
                rows.append([float(x.replace("D", "E")) for x in t])
    return np.array(rows)
