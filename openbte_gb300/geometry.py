"""Seeded periodic unit-cell meshes written as gmsh msh2 files.

The reference authors geometry with shapely polygons and meshes it with the
external gmsh binary (openbte/geometry.py:51-554, openbte/utils.py:35-40).
Neither is part of the transport hot path, so this module stands in for them:
it builds a seeded, jittered-point Delaunay triangulation of a periodic square
cell with one centred pore and writes it in the msh2 layout that the
reference's ``get_mesh`` parses (openbte/mesh.py:54-348):

* ``$PhysicalNames`` with ``Boundary`` (pore wall), ``Periodic_x_a/_b``,
  ``Periodic_y_a/_b`` and ``Bulk``; ``_a`` is the low-coordinate edge and
  ``_b`` the high one, as ``Geometry.set_periodicity`` orders them
  (openbte/geometry.py:120-158, 537-546);
* line elements listed before the triangles (``elem_physical_regions`` at
  openbte/mesh.py:132-134 assumes that order);
* a ``$Periodic`` block without ``Affine`` lines, slave = ``_a`` edge,
  master = ``_b`` edge (offsets at openbte/mesh.py:213-265).

Pore shapes follow the reference helpers: ``rectangle`` is an axis-aligned
square of the given area (openbte/geometry.py:22-30); ``circle`` is a regular
polygon of the given area (openbte/geometry.py:10-19) refined to the mesh step.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.spatial import Delaunay

__all__ = ["PeriodicCell2D", "porous_cell_2d", "write_msh2"]

# Physical region names, in the order their tags are written.
REGIONS = ["Boundary", "Periodic_x_a", "Periodic_x_b", "Periodic_y_a", "Periodic_y_b"]


@dataclass
class PeriodicCell2D:
    """A triangulated periodic cell before it is turned into a ``Mesh``.

    nodes      [n_nodes, 2] float64, nm, cell centred on the origin
    elems      [n_elems, 3] int64, node indices (0-based)
    segments   {region: [k, 2] int64} boundary line elements, node indices
    periodic   {'x'|'y': [k, 2] int64} (slave node, master node) pairs
    """

    nodes: np.ndarray
    elems: np.ndarray
    segments: dict
    periodic: dict
    size: float
    porosity: float
    pore: str
    seed: int
    meta: dict = field(default_factory=dict)

    @property
    def n_elems(self) -> int:
        return int(self.elems.shape[0])


def _edge_points(a, b, n):
    """n+1 evenly spaced points from a to b inclusive."""
    t = np.linspace(0.0, 1.0, n + 1)[:, None]
    return a[None, :] * (1.0 - t) + b[None, :] * t


def _dist_to_square(p, half):
    """Signed distance from points p to an axis-aligned square of half-side `half` (positive outside)."""
    q = np.abs(p) - half
    outside = np.linalg.norm(np.maximum(q, 0.0), axis=1)
    inside = np.minimum(np.max(q, axis=1), 0.0)
    return outside + inside


def porous_cell_2d(n_target: int = 2000, porosity: float = 0.25, pore: str = "square",
                   size: float = 100.0, seed: int = 0, jitter: float = 0.2) -> PeriodicCell2D:
    """Seeded periodic square cell of side `size` (nm) with one centred pore.

    ``n_target`` is the approximate triangle count. Interior points are a
    hexagonal lattice jittered by ``jitter``·h (seeded); boundary points are
    evenly spaced on the four cell edges (identical on opposite edges, so the
    periodic node pairs match exactly) and on the pore outline.
    """
    if pore not in ("square", "circle"):
        raise ValueError(f"unknown pore shape {pore!r}")
    if not (0.0 < porosity < 0.6):
        raise ValueError("porosity must be in (0, 0.6)")
    rng = np.random.default_rng(seed)
    half = size / 2.0
    area = size * size * (1.0 - porosity)
    # equilateral-triangle edge length giving about n_target triangles
    h = math.sqrt(4.0 * area / (math.sqrt(3.0) * n_target))

    # outer boundary: corners + evenly spaced edge points (same count on all edges)
    nb = max(4, int(round(size / h)))
    c00, c10 = np.array([-half, -half]), np.array([half, -half])
    c11, c01 = np.array([half, half]), np.array([-half, half])
    bottom = _edge_points(c00, c10, nb)          # includes both corners
    top = _edge_points(c01, c11, nb)
    left = _edge_points(c00, c01, nb)[1:-1]      # corners already present
    right = _edge_points(c10, c11, nb)[1:-1]
    outer = np.vstack([bottom, top, left, right])
    # exact edge coordinates, so opposite edges match bit for bit
    for ax in (0, 1):
        col = outer[:, ax]
        col[np.abs(col + half) < 1e-9 * size] = -half
        col[np.abs(col - half) < 1e-9 * size] = half

    # pore outline
    if pore == "square":
        a = size * math.sqrt(porosity)
        ha = a / 2.0
        npe = max(2, int(round(a / h)))
        q0, q1 = np.array([-ha, -ha]), np.array([ha, -ha])
        q2, q3 = np.array([ha, ha]), np.array([-ha, ha])
        ring = np.vstack([_edge_points(q0, q1, npe)[:-1], _edge_points(q1, q2, npe)[:-1],
                          _edge_points(q2, q3, npe)[:-1], _edge_points(q3, q0, npe)[:-1]])

        def pore_dist(p):
            return _dist_to_square(p, ha)
    else:
        r_area = size * math.sqrt(porosity / math.pi)
        npe = max(12, int(round(2.0 * math.pi * r_area / h)))
        # regular polygon with the pore's area (the circle() helper's radius rule)
        dphi = 2.0 * math.pi / npe
        r = math.sqrt(2.0 * porosity * size * size / npe / math.sin(dphi))
        phase = dphi / 2.0 + (np.arange(npe) - 1) * dphi
        ring = r * np.stack([np.cos(phase), np.sin(phase)], axis=1)
        ha = r

        def pore_dist(p):
            return np.linalg.norm(p, axis=1) - r

    # jittered hexagonal interior lattice
    dy = h * math.sqrt(3.0) / 2.0
    ny = int(math.ceil(size / dy)) + 2
    nx = int(math.ceil(size / h)) + 2
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    px = -half + (ii + 0.5 * (jj % 2)) * h
    py = -half + jj * dy
    lat = np.stack([px.ravel(), py.ravel()], axis=1)
    lat = lat + rng.uniform(-jitter * h, jitter * h, size=lat.shape)
    margin_outer = 0.45 * h
    margin_pore = 0.6 * h
    keep = (np.abs(lat[:, 0]) < half - margin_outer) & (np.abs(lat[:, 1]) < half - margin_outer)
    keep &= pore_dist(lat) > margin_pore
    interior = lat[keep]

    pts = np.vstack([outer, ring, interior])
    tri = Delaunay(pts)
    simp = tri.simplices.astype(np.int64)
    cen = pts[simp].mean(axis=1)
    inside_pore = pore_dist(cen) < 0.0
    simp = simp[~inside_pore]
    # drop degenerate (zero-area) triangles, if any
    p = pts[simp]
    ar = 0.5 * np.abs((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                      - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))
    simp = simp[ar > 1e-12 * h * h]

    # renumber used nodes
    used = np.unique(simp)
    remap = -np.ones(len(pts), dtype=np.int64)
    remap[used] = np.arange(len(used))
    nodes = pts[used]
    elems = remap[simp]

    n_outer = len(outer)
    n_ring = len(ring)

    # boundary segments: edges used by exactly one triangle
    e = np.concatenate([elems[:, [0, 1]], elems[:, [1, 2]], elems[:, [2, 0]]])
    e.sort(axis=1)
    ue, cnt = np.unique(e, axis=0, return_counts=True)
    bseg = ue[cnt == 1]
    tol = 1e-9 * size
    mid = nodes[bseg].mean(axis=1)
    segs = {k: [] for k in REGIONS}
    on_xa = np.abs(mid[:, 0] + half) < tol
    on_xb = np.abs(mid[:, 0] - half) < tol
    on_ya = np.abs(mid[:, 1] + half) < tol
    on_yb = np.abs(mid[:, 1] - half) < tol
    wall = ~(on_xa | on_xb | on_ya | on_yb)
    for name, mask in zip(REGIONS, [wall, on_xa, on_xb, on_ya, on_yb]):
        segs[name] = bseg[mask]

    # sanity: pore wall closed, outer edges complete
    if len(segs["Periodic_x_a"]) != nb or len(segs["Periodic_x_b"]) != nb \
            or len(segs["Periodic_y_a"]) != nb or len(segs["Periodic_y_b"]) != nb:
        raise RuntimeError("outer boundary is not conforming; change the seed")
    if len(segs["Boundary"]) != n_ring:
        raise RuntimeError("pore wall is not conforming; change the seed")

    # periodic node pairs (slave on the _a edge, master on the _b edge)
    def pairs(axis):
        other = 1 - axis
        lo = np.where(np.abs(nodes[:, axis] + half) < tol)[0]
        hi = np.where(np.abs(nodes[:, axis] - half) < tol)[0]
        lo = lo[np.argsort(nodes[lo, other])]
        hi = hi[np.argsort(nodes[hi, other])]
        if len(lo) != len(hi) or not np.allclose(nodes[lo, other], nodes[hi, other], atol=tol):
            raise RuntimeError("periodic boundary nodes do not match")
        return np.stack([lo, hi], axis=1)

    periodic = {"x": pairs(0), "y": pairs(1)}
    return PeriodicCell2D(nodes=nodes, elems=elems, segments=segs, periodic=periodic,
                          size=size, porosity=porosity, pore=pore, seed=seed,
                          meta={"h": h, "n_outer": n_outer, "n_ring": n_ring})


REGIONS_3D = ["Boundary", "Periodic_x_a", "Periodic_x_b", "Periodic_y_a", "Periodic_y_b",
              "Periodic_z_a", "Periodic_z_b"]


def porous_cube_3d(n_target: int = 100000, porosity: float = 0.10, size: float = 100.0, seed: int = 0,
                   jitter: float = 0.2) -> PeriodicCell2D:
    """Seeded periodic cube of side `size` (nm) with a centred spherical pore, tetrahedral Delaunay mesh.

    ``n_target`` is the approximate tetrahedron count. Opposite cube faces carry the same jittered 2D
    point set and cube edges a shared uniform grid, so the face triangulations are translates of each
    other (checked); the pore surface is a Fibonacci point set on the sphere. Tetrahedra inside the
    pore and flat (zero-volume) tetrahedra on the faces are removed. Returned in the same container as
    the 2D cells (``elems`` [n, 4], ``segments`` = boundary triangles per region, ``periodic`` =
    (slave, master) node pairs per axis).
    """
    rng = np.random.default_rng(seed)
    half = size / 2.0
    r = (3.0 * porosity * size ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)
    vol = size ** 3 * (1.0 - porosity)
    h = (vol * 6.3 / n_target) ** (1.0 / 3.0)          # about 6.3 tetrahedra per point
    nb = max(4, int(round(size / h)))
    g1 = np.linspace(-half, half, nb + 1)
    # cube edges: uniform grids shared by the faces that meet there
    pts = []
    for ax in range(3):
        for s1 in (-half, half):
            for s2 in (-half, half):
                e = np.zeros((nb + 1, 3))
                e[:, ax] = g1
                o = [a for a in range(3) if a != ax]
                e[:, o[0]] = s1
                e[:, o[1]] = s2
                pts.append(e)
    # face interiors: one jittered 2D set per axis, used on both faces of that axis
    for ax in range(3):
        o = [a for a in range(3) if a != ax]
        u, v = np.meshgrid(g1[1:-1], g1[1:-1], indexing="ij")
        uv = np.stack([u.ravel(), v.ravel()], axis=1)
        uv = uv + rng.uniform(-jitter * h, jitter * h, size=uv.shape)
        uv = np.clip(uv, -half + 0.3 * h, half - 0.3 * h)
        for s in (-half, half):
            f = np.zeros((len(uv), 3))
            f[:, ax] = s
            f[:, o[0]] = uv[:, 0]
            f[:, o[1]] = uv[:, 1]
            pts.append(f)
    # pore surface (Fibonacci sphere)
    ns = max(20, int(round(4.0 * math.pi * r * r / (0.8 * h * h))))
    k = np.arange(ns) + 0.5
    th = np.arccos(1.0 - 2.0 * k / ns)
    ph = math.pi * (1.0 + 5.0 ** 0.5) * k
    sph = r * np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], axis=1)
    pts.append(sph)
    # interior: jittered cubic lattice away from faces and pore
    gi = np.arange(-half + 0.5 * h, half, h)
    X, Y, Z = np.meshgrid(gi, gi, gi, indexing="ij")
    lat = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    lat = lat + rng.uniform(-jitter * h, jitter * h, size=lat.shape)
    keep = np.all(np.abs(lat) < half - 0.45 * h, axis=1) & (np.linalg.norm(lat, axis=1) > r + 0.6 * h)
    pts.append(lat[keep])
    P = np.vstack(pts)
    for ax in range(3):                                # exact face coordinates
        col = P[:, ax]
        col[np.abs(col + half) < 1e-9 * size] = -half
        col[np.abs(col - half) < 1e-9 * size] = half
    P, idx = np.unique(np.round(P, 12), axis=0, return_index=True)
    tri = Delaunay(P)
    T = tri.simplices.astype(np.int64)
    c = P[T].mean(axis=1)
    T = T[np.linalg.norm(c, axis=1) > r]
    a = P[T]
    v6 = np.abs(np.einsum("ij,ij->i", a[:, 1] - a[:, 0], np.cross(a[:, 2] - a[:, 0], a[:, 3] - a[:, 0])))
    T = T[v6 > 1e-9 * h ** 3]
    used = np.unique(T)
    remap = -np.ones(len(P), dtype=np.int64)
    remap[used] = np.arange(len(used))
    nodes = P[used]
    elems = remap[T]
    # boundary faces = faces of exactly one tetrahedron
    F = np.concatenate([elems[:, [1, 2, 3]], elems[:, [0, 2, 3]], elems[:, [0, 1, 3]], elems[:, [0, 1, 2]]])
    F.sort(axis=1)
    uf, cnt = np.unique(F, axis=0, return_counts=True)
    bf = uf[cnt == 1]
    tol = 1e-9 * size
    segs = {}
    on = {}
    for ax, name in enumerate("xyz"):
        on[(ax, 0)] = np.all(np.abs(nodes[bf][:, :, ax] + half) < tol, axis=1)
        on[(ax, 1)] = np.all(np.abs(nodes[bf][:, :, ax] - half) < tol, axis=1)
        segs[f"Periodic_{name}_a"] = bf[on[(ax, 0)]]
        segs[f"Periodic_{name}_b"] = bf[on[(ax, 1)]]
    outer = np.zeros(len(bf), dtype=bool)
    for v in on.values():
        outer |= v
    segs["Boundary"] = bf[~outer]
    # periodic node pairs, and a check that the face triangulations are translates
    periodic = {}
    for ax, name in enumerate("xyz"):
        lo = np.where(np.abs(nodes[:, ax] + half) < tol)[0]
        hi = np.where(np.abs(nodes[:, ax] - half) < tol)[0]
        o = [b for b in range(3) if b != ax]
        kl = {tuple(np.round(nodes[i, o], 9)): i for i in lo}
        kh = {tuple(np.round(nodes[i, o], 9)): i for i in hi}
        if set(kl) != set(kh):
            raise RuntimeError("periodic face nodes do not match; change the seed")
        pairs = np.array([[kl[key], kh[key]] for key in sorted(kl)], dtype=np.int64)
        periodic[name] = pairs
        m = dict(zip(pairs[:, 0], pairs[:, 1]))
        ta = {tuple(sorted(m[i] for i in t)) for t in segs[f"Periodic_{name}_a"]}
        tb = {tuple(sorted(t)) for t in segs[f"Periodic_{name}_b"]}
        if ta != tb:
            raise RuntimeError("periodic face triangulations differ; change the seed")
    return PeriodicCell2D(nodes=nodes, elems=elems, segments=segs, periodic=periodic, size=size,
                          porosity=porosity, pore="sphere", seed=seed, meta={"h": h, "r": r})


def write_msh2(cell: PeriodicCell2D, filename: str) -> str:
    """Write `cell` as gmsh msh2 text (``filename`` gets the ``.msh`` suffix if missing)."""
    if not filename.endswith(".msh"):
        filename = filename + ".msh"
    three = cell.elems.shape[1] == 4 and cell.nodes.shape[1] == 3
    regions = REGIONS_3D if three else REGIONS
    fdim, face_type, bulk_type = (2, 2, 4) if three else (1, 1, 2)
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$PhysicalNames", str(len(regions) + 1)]
    for t, name in enumerate(regions, start=1):
        out.append(f'{fdim} {t} "{name}"')
    bulk_tag = len(regions) + 1
    out.append(f'{fdim + 1} {bulk_tag} "Bulk"')
    out += ["$EndPhysicalNames", "$Nodes", str(len(cell.nodes))]
    for i, p in enumerate(cell.nodes, start=1):
        z = p[2] if three else 0
        out.append(f"{i} {p[0]:.17g} {p[1]:.17g} {z:.17g}" if three else f"{i} {p[0]:.17g} {p[1]:.17g} 0")
    out += ["$EndNodes", "$Elements"]
    lines = []
    eid = 1
    for t, name in enumerate(regions, start=1):
        for f in cell.segments[name]:
            lines.append(f"{eid} {face_type} 2 {t} {t} " + " ".join(str(int(x) + 1) for x in f))
            eid += 1
    for e in cell.elems:
        lines.append(f"{eid} {bulk_type} 2 {bulk_tag} 1 " + " ".join(str(int(x) + 1) for x in e))
        eid += 1
    out.append(str(len(lines)))
    out += lines
    axes = (("x", (2, 3)), ("y", (4, 5)), ("z", (6, 7))) if three else (("x", (2, 3)), ("y", (4, 5)))
    out += ["$EndElements", "$Periodic", str(len(axes))]
    # entity tags: 2 = x_a, 3 = x_b, 4 = y_a, 5 = y_b (, 6 = z_a, 7 = z_b); surfaces carry an Affine line
    for axis, (slave, master) in axes:
        pr = cell.periodic[axis]
        out.append(f"{fdim} {slave} {master}")
        if three:
            tr = [0.0, 0.0, 0.0]
            tr["xyz".index(axis)] = -cell.size
            out.append("Affine 1 0 0 {} 0 1 0 {} 0 0 1 {} 0 0 0 1".format(*tr))
        out.append(str(len(pr)))
        for s, m in pr:
            out.append(f"{s + 1} {m + 1}")
    out.append("$EndPeriodic")
    with open(filename, "w") as f:
        f.write("\n".join(out) + "\n")
    return filename
