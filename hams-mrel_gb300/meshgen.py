"""Seeded synthetic hull meshes and panel geometry for the benchmark layouts.

The reference reads .pnl meshes and computes panel centroids, areas,
characteristic lengths and generalized normals once per run
(src/NormalProcess.f90:46-441, called from CalNormals*).  This module
builds the same quantities for generated cylinders and boxes so the
benchmark needs no input files:

  cylinder  vertical circular cylinder: n_az x n_vert side quads plus
            n_az x n_ring bottom panels in concentric rings (triangles in the
            innermost ring), normals pointing into the body as in the
            reference meshes;
  box       rectangular barge with square-ish quads of a given size;
  lid       waterplane (z = 0) panels of a cylinder for irregular-frequency
            removal.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Body:
    nodes: np.ndarray           # (ntnd, 3)
    panels: list                # lists of 3 or 4 0-based node ids
    center: tuple               # reference point (x, y, z) for rotational normals
    lid_nodes: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    lid_panels: list = field(default_factory=list)


def _ring_panels(nodes, n_az, r_out, r_in, z, cx, cy, inward_up=True):
    """Panels of one annulus between radii r_in < r_out at height z."""
    base = len(nodes)
    for k in range(n_az):
        t = 2.0 * math.pi * k / n_az
        nodes.append((cx + r_out * math.cos(t), cy + r_out * math.sin(t), z))
    panels = []
    if r_in <= 0.0:
        c = len(nodes)
        nodes.append((cx, cy, z))
        for k in range(n_az):
            panels.append([base + k, base + (k + 1) % n_az, c])
        return panels, base
    inner = len(nodes)
    for k in range(n_az):
        t = 2.0 * math.pi * k / n_az
        nodes.append((cx + r_in * math.cos(t), cy + r_in * math.sin(t), z))
    for k in range(n_az):
        k1 = (k + 1) % n_az
        panels.append([base + k, base + k1, inner + k1, inner + k])
    return panels, base


def cylinder(radius, draft, n_az, n_vert, n_ring, cx=0.0, cy=0.0, lid_rings=0) -> Body:
    nodes, panels = [], []
    zs = [-draft * i / n_vert for i in range(n_vert + 1)]
    for z in zs:
        for k in range(n_az):
            t = 2.0 * math.pi * k / n_az
            nodes.append((cx + radius * math.cos(t), cy + radius * math.sin(t), z))
    for i in range(n_vert):
        for k in range(n_az):
            k1 = (k + 1) % n_az
            a, b = i * n_az + k, i * n_az + k1
            panels.append([a, b, b + n_az, a + n_az])
    # bottom rings, the outermost sharing the lowest side nodes
    bottom_row = n_vert * n_az
    r_prev_ids = [bottom_row + k for k in range(n_az)]
    for ring in range(n_ring, 0, -1):
        r_in = radius * (ring - 1) / n_ring
        if r_in <= 0.0:
            c = len(nodes)
            nodes.append((cx, cy, -draft))
            for k in range(n_az):
                panels.append([r_prev_ids[k], r_prev_ids[(k + 1) % n_az], c])
        else:
            ids = []
            for k in range(n_az):
                t = 2.0 * math.pi * k / n_az
                ids.append(len(nodes))
                nodes.append((cx + r_in * math.cos(t), cy + r_in * math.sin(t), -draft))
            for k in range(n_az):
                k1 = (k + 1) % n_az
                panels.append([r_prev_ids[k], r_prev_ids[k1], ids[k1], ids[k]])
            r_prev_ids = ids
    body = Body(np.array(nodes, dtype=np.float64), panels, (cx, cy, 0.0))
    _orient_inward(body.nodes, body.panels, np.array([cx, cy, -draft / 2.0]))
    if lid_rings > 0:
        ln, lp = [], []
        ids = None
        for ring in range(lid_rings, 0, -1):
            r_out = radius * ring / lid_rings
            r_in = radius * (ring - 1) / lid_rings
            if ids is None:
                ids = []
                for k in range(n_az):
                    t = 2.0 * math.pi * k / n_az
                    ids.append(len(ln))
                    ln.append((cx + r_out * math.cos(t), cy + r_out * math.sin(t), 0.0))
            if r_in <= 0.0:
                c = len(ln)
                ln.append((cx, cy, 0.0))
                for k in range(n_az):
                    lp.append([ids[k], ids[(k + 1) % n_az], c])
            else:
                nid = []
                for k in range(n_az):
                    t = 2.0 * math.pi * k / n_az
                    nid.append(len(ln))
                    ln.append((cx + r_in * math.cos(t), cy + r_in * math.sin(t), 0.0))
                for k in range(n_az):
                    k1 = (k + 1) % n_az
                    lp.append([ids[k], ids[k1], nid[k1], nid[k]])
                ids = nid
        body.lid_nodes = np.array(ln, dtype=np.float64)
        body.lid_panels = lp
    return body


def hemisphere(radius, n_az, n_lat, cx=0.0, cy=0.0) -> Body:
    """Floating hemisphere (the submerged half of a sphere centred on the
    waterline): n_az x n_lat panels between latitude circles spaced evenly in
    polar angle, nodes on the sphere, triangles at the bottom pole."""
    nodes, panels = [], []
    for i in range(n_lat):
        th = 0.5 * math.pi * i / n_lat  # 0 at the waterline
        for k in range(n_az):
            t = 2.0 * math.pi * k / n_az
            nodes.append((cx + radius * math.cos(th) * math.cos(t), cy + radius * math.cos(th) * math.sin(t),
                          -radius * math.sin(th)))
    pole = len(nodes)
    nodes.append((cx, cy, -radius))
    for i in range(n_lat):
        for k in range(n_az):
            k1 = (k + 1) % n_az
            a, b = i * n_az + k, i * n_az + k1
            if i + 1 < n_lat:
                panels.append([a, b, b + n_az, a + n_az])
            else:
                panels.append([a, b, pole])
    body = Body(np.array(nodes, dtype=np.float64), panels, (cx, cy, 0.0))
    _orient_inward(body.nodes, body.panels, np.array([cx, cy, -radius / 2.0]))
    return body


def box(lx, ly, draft, dx, cx=0.0, cy=0.0) -> Body:
    """Rectangular barge centred at (cx, cy) with panels of side ~dx."""
    nx, ny, nz = max(1, round(lx / dx)), max(1, round(ly / dx)), max(1, round(draft / dx))
    nodes, index, panels = [], {}, []

    def node(p):
        key = (round(p[0], 9), round(p[1], 9), round(p[2], 9))
        if key not in index:
            index[key] = len(nodes)
            nodes.append(p)
        return index[key]

    xs = [cx - lx / 2 + lx * i / nx for i in range(nx + 1)]
    ys = [cy - ly / 2 + ly * j / ny for j in range(ny + 1)]
    zs = [-draft * k / nz for k in range(nz + 1)]
    for y in (ys[0], ys[-1]):           # faces y = const
        for i in range(nx):
            for k in range(nz):
                panels.append([node((xs[i], y, zs[k])), node((xs[i + 1], y, zs[k])),
                               node((xs[i + 1], y, zs[k + 1])), node((xs[i], y, zs[k + 1]))])
    for x in (xs[0], xs[-1]):           # faces x = const
        for j in range(ny):
            for k in range(nz):
                panels.append([node((x, ys[j], zs[k])), node((x, ys[j + 1], zs[k])),
                               node((x, ys[j + 1], zs[k + 1])), node((x, ys[j], zs[k + 1]))])
    for i in range(nx):                 # bottom
        for j in range(ny):
            panels.append([node((xs[i], ys[j], -draft)), node((xs[i + 1], ys[j], -draft)),
                           node((xs[i + 1], ys[j + 1], -draft)), node((xs[i], ys[j + 1], -draft))])
    body = Body(np.array(nodes, dtype=np.float64), panels, (cx, cy, 0.0))
    _orient_inward(body.nodes, body.panels, np.array([cx, cy, -draft / 2.0]))
    return body


def _normal(nodes, p):
    if len(p) == 3:
        v21 = nodes[p[0]] - nodes[p[1]]; v23 = nodes[p[2]] - nodes[p[1]]
        return np.cross(v21, v23)
    v13 = nodes[p[2]] - nodes[p[0]]; v24 = nodes[p[3]] - nodes[p[1]]
    return np.cross(v24, v13)


def _orient_inward(nodes, panels, inside):
    for k, p in enumerate(panels):
        c = nodes[p].mean(axis=0)
        if np.dot(_normal(nodes, p), c - inside) > 0:
            panels[k] = p[::-1]


# ---------------------------------------------------------------------------
# Panel geometry, following NormalProcess.f90 (centre, Heron-type area,
# longest edge, (P4-P2)x(P3-P1) or (P1-P2)x(P3-P2) unit normal, r x n).
# ---------------------------------------------------------------------------
def _area(p1, p2, p3):
    a = np.linalg.norm(p1 - p2, axis=-1); b = np.linalg.norm(p3 - p1, axis=-1); c = np.linalg.norm(p3 - p2, axis=-1)
    return np.sqrt((a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c))) / 4.0


def geometry(nodes, ncon, ncn, xr):
    """nodes (ntnd,3); ncon (n,4) 0-based with ncon[:,3] = ncon[:,0] for triangles."""
    P = nodes[ncon]                                  # (n, 4, 3)
    tri = ncn == 3
    xyz_p = np.where(tri[:, None], P[:, :3].sum(axis=1) / 3.0, P.sum(axis=1) / 4.0)
    ds = _area(P[:, 0], P[:, 1], P[:, 2]) + np.where(tri, 0.0, _area(P[:, 0], P[:, 3], P[:, 2]))
    e = np.stack([np.linalg.norm(P[:, (k + 1) % 4] - P[:, k], axis=-1) for k in range(4)], axis=1)
    e3 = np.stack([np.linalg.norm(P[:, (k + 1) % 3] - P[:, k], axis=-1) for k in range(3)], axis=1)
    pnsz = np.where(tri, e3.max(axis=1), e.max(axis=1))
    n_tri = np.cross(P[:, 0] - P[:, 1], P[:, 2] - P[:, 1])
    n_quad = np.cross(P[:, 3] - P[:, 1], P[:, 2] - P[:, 0])
    un = np.where(tri[:, None], n_tri, n_quad)
    un = un / np.linalg.norm(un, axis=1, keepdims=True)
    r = xyz_p - np.asarray(xr)
    rot = np.stack([r[:, 1] * un[:, 2] - r[:, 2] * un[:, 1],
                    r[:, 2] * un[:, 0] - r[:, 0] * un[:, 2],
                    r[:, 0] * un[:, 1] - r[:, 1] * un[:, 0]], axis=1)
    return xyz_p, ds, pnsz, np.concatenate([un, rot], axis=1)


@dataclass
class Mesh:
    """Global (body-major) arrays in the layout the C ABI takes."""
    nodes: np.ndarray
    ncon: np.ndarray        # (n,4) 1-based
    ncn: np.ndarray
    xyz_p: np.ndarray
    ds: np.ndarray
    pnsz: np.ndarray
    dxyz_p: np.ndarray
    body_ranges: np.ndarray  # (nbody, 2) 1-based first, last
    lid_xyz_p: np.ndarray

    @property
    def n(self):
        return len(self.ncn)


def combine(bodies) -> Mesh:
    nodes, ncon, ncn, xyz, ds, pn, dx, ranges, lids = [], [], [], [], [], [], [], [], []
    nbase = 0
    ebase = 0
    for b in bodies:
        m = len(b.panels)
        cn = np.zeros((m, 4), dtype=np.int64)
        nn = np.zeros(m, dtype=np.int32)
        for k, p in enumerate(b.panels):
            nn[k] = len(p)
            cn[k, :len(p)] = p
            if len(p) == 3:
                cn[k, 3] = p[0]
        gx, ga, gp, gn = geometry(b.nodes, cn, nn, b.center)
        nodes.append(b.nodes); ncon.append(cn + nbase + 1); ncn.append(nn)
        xyz.append(gx); ds.append(ga); pn.append(gp); dx.append(gn)
        ranges.append((ebase + 1, ebase + m))
        ebase += m
        nbase += len(b.nodes)
        if len(b.lid_panels):
            lc = np.zeros((len(b.lid_panels), 4), dtype=np.int64)
            ln = np.zeros(len(b.lid_panels), dtype=np.int32)
            for k, p in enumerate(b.lid_panels):
                ln[k] = len(p)
                lc[k, :len(p)] = p
                if len(p) == 3:
                    lc[k, 3] = p[0]
            lx, _, _, _ = geometry(b.lid_nodes, lc, ln, b.center)
            lids.append(lx)
    return Mesh(np.concatenate(nodes), np.concatenate(ncon).astype(np.int32), np.concatenate(ncn),
                np.concatenate(xyz), np.concatenate(ds), np.concatenate(pn), np.concatenate(dx),
                np.array(ranges, dtype=np.int32), np.concatenate(lids) if lids else np.zeros((0, 3)))


# ---------------------------------------------------------------------------
# Benchmark layouts
# ---------------------------------------------------------------------------
def single_cylinder(with_lid=False) -> Mesh:
    """R = 5 m, T = 5 m, 32 x 8 side + 32 x 4 bottom = 384 panels."""
    return combine([cylinder(5.0, 5.0, 32, 8, 4, lid_rings=4 if with_lid else 0)])


def three_cylinders(with_lid=True) -> Mesh:
    """R = 3 m, T = 6 m, centres x = 0, 15, 30; 32 x 12 + 32 x 4 = 512 panels each; 32 x 4 lids."""
    return combine([cylinder(3.0, 6.0, 32, 12, 4, cx=15.0 * k, lid_rings=4 if with_lid else 0) for k in range(3)])


def five_body_array(seed=3) -> Mesh:
    """3 cylinders (R = 4, T = 8, 48 x 22 + 48 x 8 = 1440 panels) and 2 boxes
    (12 x 6 x 4 m, 0.5 m quads, 864 panels) on a 30 m grid perturbed by
    U(-3, 3) m: 6048 panels."""
    rng = np.random.default_rng(seed)
    grid = [(0, 0), (1, 0), (2, 0), (0, 1), (1, 1)]
    jitter = rng.uniform(-3.0, 3.0, size=(5, 2))
    bodies = []
    for k, (i, j) in enumerate(grid):
        x, y = 30.0 * i + jitter[k, 0], 30.0 * j + jitter[k, 1]
        if k < 3:
            bodies.append(cylinder(4.0, 8.0, 48, 22, 8, cx=x, cy=y))
        else:
            bodies.append(box(12.0, 6.0, 4.0, 0.5, cx=x, cy=y))
    return combine(bodies)


def scaled_array(n_target, seed=0) -> Mesh:
    """Cylinder array whose panel count is close to n_target (for sweeps)."""
    rng = np.random.default_rng(seed)
    per = 1440
    nb = max(1, round(n_target / per))
    bodies = []
    for k in range(nb):
        x, y = 30.0 * (k % 4) + rng.uniform(-3, 3), 30.0 * (k // 4) + rng.uniform(-3, 3)
        bodies.append(cylinder(4.0, 8.0, 48, 22, 8, cx=x, cy=y))
    return combine(bodies)


def _cylinder_for(n_target, radius, draft, n_az, cx, cy):
    """Cylinder with about n_target panels at n_az azimuthal divisions."""
    rows = max(2, round(n_target / n_az))
    n_ring = max(1, round(rows * radius / (radius + draft)))
    n_vert = max(1, rows - n_ring)
    return cylinder(radius, draft, n_az, n_vert, n_ring, cx=cx, cy=cy)


def _box_for(n_target, lx, ly, draft, cx, cy):
    """Box with about n_target panels of equal size."""
    area = 2.0 * lx * draft + 2.0 * ly * draft + lx * ly
    return box(lx, ly, draft, math.sqrt(area / max(n_target, 6)), cx=cx, cy=cy)


def batch_case(rng) -> tuple:
    """One solve of the batching workload: 1-4 cylinders (R ~ U(2, 8) m,
    T ~ U(2, 10) m, azimuthal count ~ U{16..48}) sized so that the panel count
    is log-uniform on 300-4000; returns (mesh, depth, w, headings_deg)."""
    n_target = math.exp(rng.uniform(math.log(300.0), math.log(4000.0)))
    nb = int(rng.integers(1, 5))
    bodies = []
    for k in range(nb):
        r, t = rng.uniform(2.0, 8.0), rng.uniform(2.0, 10.0)
        n_az = int(rng.integers(16, 49))
        bodies.append(_cylinder_for(n_target / nb, r, t, n_az, 25.0 * k, 0.0))
    h = -1.0 if rng.uniform() < 0.5 else float(rng.uniform(30.0, 200.0))
    w = float(rng.uniform(0.1, 3.0))
    heads = list(np.linspace(0.0, 90.0, int(rng.integers(1, 5))))
    return combine(bodies), h, w, heads


def serving_case(rng) -> tuple:
    """One request of the serving workload: 1-6 bodies (cylinders and boxes) on
    a 30 m grid, panel count log-uniform on 500-12000, depth infinite or
    U(30, 200) m, 20-100 frequencies in 0.1-3.0 rad/s and 1-8 headings;
    returns (mesh, depth, frequencies, headings_deg)."""
    n_target = math.exp(rng.uniform(math.log(500.0), math.log(12000.0)))
    nb = int(rng.integers(1, 7))
    bodies = []
    for k in range(nb):
        x, y = 30.0 * (k % 3) + rng.uniform(-3, 3), 30.0 * (k // 3) + rng.uniform(-3, 3)
        if rng.uniform() < 0.6:
            bodies.append(_cylinder_for(n_target / nb, rng.uniform(2.0, 8.0), rng.uniform(2.0, 10.0),
                                        int(rng.integers(16, 49)), x, y))
        else:
            bodies.append(_box_for(n_target / nb, rng.uniform(6.0, 14.0), rng.uniform(4.0, 8.0),
                                   rng.uniform(2.0, 6.0), x, y))
    h = -1.0 if rng.uniform() < 0.5 else float(rng.uniform(30.0, 200.0))
    nf = int(rng.integers(20, 101))
    freqs = np.linspace(0.1, 3.0, nf)
    heads = list(np.linspace(0.0, 315.0, int(rng.integers(1, 9))))
    return combine(bodies), h, freqs, heads
