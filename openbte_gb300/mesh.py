"""msh2 reader and vectorised ``Mesh`` builder.

Produces the same ``Mesh`` fields, side numbering and conventions as the
reference's ``get_mesh`` (openbte/mesh.py:54-348), with numpy array passes in
place of its per-side Python loops (6 s -> well under a second at 60k cells):

* sides are the lexicographically sorted unique node tuples; an element's
  side list follows its rotation order (openbte/mesh.py:98-112);
* ``side_elem_map`` lists the owning elements in increasing order, a boundary
  side repeats its single element (openbte/mesh.py:120-128);
* normals point out of ``side_elem_map[:, 0]`` (openbte/mesh.py:180-194);
* periodic pairing keeps the ``_b`` side and discards its ``_a`` image, then
  re-points the kept side across the wrap (openbte/mesh.py:205-280);
* ``internal`` = all sides minus boundary-region sides minus discarded
  periodic images (openbte/mesh.py:295-296);
* least-squares gradient weights are per-element pseudo-inverses of the
  centroid-difference matrix (openbte/mesh.py:304-320).
"""
from __future__ import annotations

import numpy as np

from .objects import Mesh

__all__ = ["get_mesh", "read_msh2", "build_mesh", "mesh_from_cell"]


def read_msh2(filename: str):
    """Parse the msh2 layout written by gmsh (and by ``geometry.write_msh2``).

    Returns (labels {tag: name}, nodes [n,3], elements [(type, phys_tag, [nodes])],
    periodic [(dim, slave, master, pairs[k,2])]) with 0-based node indices.
    """
    if not filename.endswith(".msh"):
        filename = filename + ".msh"
    with open(filename) as f:
        lines = [l.split() for l in f.read().splitlines()]
    i = 0
    labels = {}
    nodes = None
    elements = []
    periodic = []
    while i < len(lines):
        tok = lines[i][0] if lines[i] else ""
        if tok == "$PhysicalNames":
            nb = int(lines[i + 1][0])
            for k in range(nb):
                l = lines[i + 2 + k]
                labels[int(l[1])] = " ".join(l[2:]).replace('"', "")
            i += nb + 3
        elif tok == "$Nodes":
            n = int(lines[i + 1][0])
            nodes = np.array([l[1:4] for l in lines[i + 2:i + 2 + n]], dtype=np.float64)
            i += n + 3
        elif tok == "$Elements":
            n = int(lines[i + 1][0])
            for l in lines[i + 2:i + 2 + n]:
                ntag = int(l[2])
                elements.append((int(l[1]), int(l[3]), [int(x) - 1 for x in l[3 + ntag:]]))
            i += n + 3
        elif tok == "$Periodic":
            n = int(lines[i + 1][0])
            j = i + 2
            for _ in range(n):
                dim, slave, master = (int(x) for x in lines[j][:3])
                j += 1
                if lines[j][0].lower() == "affine":
                    j += 1
                npairs = int(lines[j][0])
                pairs = np.array([[int(x) - 1 for x in l[:2]] for l in lines[j + 1:j + 1 + npairs]],
                                 dtype=np.int64).reshape(-1, 2)
                periodic.append((dim, slave, master, pairs))
                j += 1 + npairs
            i = j + 1
        else:
            i += 1
    return labels, nodes, elements, periodic


def get_mesh(filename: str = "mesh") -> Mesh:
    """Build a ``Mesh`` from ``filename.msh`` (drop-in for openbte/mesh.py:54)."""
    labels, nodes, elements, periodic = read_msh2(filename)
    return build_mesh(labels, nodes, elements, periodic)


def mesh_from_cell(cell) -> Mesh:
    """Build a ``Mesh`` directly from a ``geometry`` cell, 2D or 3D (same result as write + read)."""
    from .geometry import REGIONS, REGIONS_3D
    three = cell.elems.shape[1] == 4 and cell.nodes.shape[1] == 3
    regions = REGIONS_3D if three else REGIONS
    face_type, bulk_type = (2, 4) if three else (1, 2)
    labels = {t: name for t, name in enumerate(regions, start=1)}
    labels[len(regions) + 1] = "Bulk"
    dimf = 3 if three else 2
    segs = [np.asarray(cell.segments[name], dtype=np.int64).reshape(-1, dimf) for name in regions]
    face_nodes = np.concatenate(segs) if segs else np.zeros((0, dimf), dtype=np.int64)
    face_tags = np.concatenate([np.full(len(f), t, dtype=np.int64) for t, f in enumerate(segs, start=1)])
    elems = np.asarray(cell.elems, dtype=np.int64)
    if three:
        nodes = np.asarray(cell.nodes, dtype=np.float64)
        periodic = [(2, 2, 3, cell.periodic["x"]), (2, 4, 5, cell.periodic["y"]), (2, 6, 7, cell.periodic["z"])]
    else:
        nodes = np.concatenate([cell.nodes, np.zeros((len(cell.nodes), 1))], axis=1)
        periodic = [(1, 2, 3, cell.periodic["x"]), (1, 4, 5, cell.periodic["y"])]
    return _build_mesh(labels, nodes, elems, np.full(len(elems), len(regions) + 1, dtype=np.int64), face_nodes,
                       face_tags, periodic)


def _row_keys(rows, n_nodes):
    """One int64 per row of sorted node indices, increasing in the rows' lexicographic order, or None when
    n_nodes ** width does not fit."""
    w = rows.shape[1]
    if n_nodes ** w >= 2 ** 62:
        return None
    key = rows[:, 0].astype(np.int64)
    for c in range(1, w):
        key = key * n_nodes + rows[:, c]
    return key


def _groups(tags, labels):
    """{label: [positions]} with labels in order of first appearance and positions in order (the grouping
    of a loop over the elements that appends each position to its label's list)."""
    out = {}
    if len(tags) == 0:
        return out
    u, first = np.unique(tags, return_index=True)
    for t in u[np.argsort(first)]:
        out.setdefault(labels[int(t)], []).append(np.nonzero(tags == t)[0])
    return {k: np.sort(np.concatenate(v)).tolist() for k, v in out.items()}


def build_mesh(labels, nodes3, elements, periodic) -> Mesh:
    """``Mesh`` from msh2 element records ``(type, tag, nodes)`` (openbte/mesh.py:54-348)."""
    nodes = np.asarray(nodes3, dtype=np.float64)
    dim = 2 if np.allclose(nodes[:, 2], np.zeros(nodes.shape[0])) else 3
    bulk_type = {2: (2, 3), 3: (4,)}[dim]
    face_type = {2: (1,), 3: (2,)}[dim]
    bulk = [e for e in elements if e[0] in bulk_type]
    faces = [e for e in elements if e[0] in face_type]
    nv = len(bulk[0][2])
    if any(len(e[2]) != nv for e in bulk):
        raise ValueError("mixed element types are not supported")
    elems = np.array([e[2] for e in bulk], dtype=np.int64)
    bulk_tags = np.array([e[1] for e in bulk], dtype=np.int64)
    face_nodes = np.array([e[2] for e in faces], dtype=np.int64).reshape(-1, dim)
    face_tags = np.array([e[1] for e in faces], dtype=np.int64)
    return _build_mesh(labels, nodes3, elems, bulk_tags, face_nodes, face_tags, periodic)


def _build_mesh(labels, nodes3, elems, bulk_tags, face_nodes, face_tags, periodic) -> Mesh:
    nodes = np.asarray(nodes3, dtype=np.float64)
    if np.allclose(nodes[:, 2], np.zeros(nodes.shape[0])):
        dim = 2
        nodes = nodes[:, :2]
    else:
        dim = 3
    n_nodes = len(nodes)
    size = np.zeros(3)
    for i in range(dim):
        size[i] = np.max(nodes[:, i]) - np.min(nodes[:, i])
    nv = elems.shape[1]
    n_elems = len(elems)

    # sides in rotation order: side r of an element = sorted(elem[(r+1+j) % nv], j < dim); the unique sides
    # in lexicographic order (np.unique over rows, through one integer key per row when it fits)
    rot = np.array([[(r + 1 + j) % nv for j in range(dim)] for r in range(nv)])
    all_sides = np.sort(elems[:, rot], axis=2).reshape(-1, dim)
    all_keys = _row_keys(all_sides, n_nodes)
    if all_keys is not None:
        side_keys, first, inverse = np.unique(all_keys, return_index=True, return_inverse=True)
        sides = all_sides[first]
    else:
        sides, inverse = np.unique(all_sides, axis=0, return_inverse=True)
    inverse = inverse.reshape(-1)
    n_sides = len(sides)
    esm = inverse.reshape(n_elems, nv).copy()          # elem -> sides (array form)

    owner = np.repeat(np.arange(n_elems), nv)
    order = np.lexsort((owner, inverse))
    s_sorted = inverse[order]
    o_sorted = owner[order]
    first = np.searchsorted(s_sorted, np.arange(n_sides), side="left")
    last = np.searchsorted(s_sorted, np.arange(n_sides), side="right") - 1
    side_elem_map = np.stack([o_sorted[first], o_sorted[last]], axis=1).astype(np.int64)

    elem_physical_regions = _groups(bulk_tags, labels)

    # side of each face element
    fs = np.sort(face_nodes, axis=1)
    if all_keys is not None and len(fs):
        fk = _row_keys(fs, n_nodes)
        face_side = np.searchsorted(side_keys, fk)
        if np.any(face_side >= n_sides) or np.any(side_keys[np.minimum(face_side, n_sides - 1)] != fk):
            raise KeyError("a face element is not a side of any bulk element")
    else:
        side_index = {tuple(s): k for k, s in enumerate(sides.tolist())}
        face_side = np.array([side_index[tuple(f)] for f in fs.tolist()], dtype=np.int64)
    side_physical_regions = {}
    for name, pos in _groups(face_tags, labels).items():
        side_physical_regions[name] = face_side[pos].tolist()

    if dim == 2:
        side_areas = np.linalg.norm(nodes[sides[:, 1]] - nodes[sides[:, 0]], axis=1)
    else:
        p = nodes[sides]
        side_areas = np.linalg.norm(np.cross(p[:, 0] - p[:, 1], p[:, 0] - p[:, 2]), axis=1) / 2

    if dim == 3:
        M = np.ones((n_elems, 4, 4))
        M[:, :, :3] = nodes[elems]
        elem_volumes = np.abs(np.linalg.det(M)) / 6.0
    else:
        if nv == 3:
            M = np.ones((n_elems, 3, 3))
            M[:, :, :2] = nodes[elems]
            elem_volumes = np.abs(0.5 * np.linalg.det(M))
        else:
            x = nodes[elems][:, :, 0]
            y = nodes[elems][:, :, 1]
            elem_volumes = 0.5 * np.abs(np.sum(x * np.roll(y, 1, axis=1), axis=1)
                                        - np.sum(y * np.roll(x, 1, axis=1), axis=1))

    side_centroids = nodes[sides].mean(axis=1)
    elem_centroids = nodes[elems].mean(axis=1)

    v1 = nodes[sides[:, 1]] - nodes[sides[:, 0]]
    if dim == 3:
        v2 = nodes[sides[:, 2]] - nodes[sides[:, 0]]
        v = np.cross(v1, v2)
    else:
        v = np.stack([v1[:, 1], -v1[:, 0]], axis=1)
    normal = v / np.linalg.norm(v, axis=1)[:, None]
    c = side_centroids - elem_centroids[side_elem_map[:, 0]]
    flip = np.einsum("ui,ui->u", normal, c) < 0
    normal[flip] = -normal[flip]
    normal_areas = normal * side_areas[:, None]

    e1, e2 = side_elem_map[:, 0], side_elem_map[:, 1]
    bnd = e1 == e2
    dists = elem_centroids[e2] - elem_centroids[e1]
    proj = np.einsum("si,si->s", normal, side_centroids - elem_centroids[e1])
    dists[bnd] = (normal * proj[:, None])[bnd]

    # periodic pairing (openbte/mesh.py:205-280)
    to_discard = []
    periodic_list = []
    periodic_sides_dict = {}
    if periodic:
        # node -> its sides in increasing side order
        flat = sides.reshape(-1)
        by_node = np.argsort(flat, kind="stable")
        nptr = np.searchsorted(flat[by_node], np.arange(n_nodes + 1))
        side_of = (by_node // dim).tolist()

        def sides_of(t):
            return side_of[nptr[t]:nptr[t + 1]]
        b_regions = [(k, set(v)) for k, v in side_physical_regions.items() if k[-2:] == "_b"]
        in_periodic = set()
        # candidate side pairs of every node pair (a, b): the sides of a x the sides of b, each visited in
        # Python-set order, as the reference does (openbte/mesh.py:236-244); in 3D one node pair matches
        # several sides.  The centroid test is the default np.allclose, |p - q| <= 1e-8 + 1e-5 |q| on every
        # component with q = centroid(s2) + (node a - node b), evaluated for all candidates at once.
        node_pairs = [(int(a), int(b)) for (_, _, _, pairs) in periodic for a, b in pairs.tolist()]
        c1, c2, cnt = [], [], []
        for a, b in node_pairs:
            S1 = np.fromiter(set(sides_of(a)), dtype=np.int64)
            S2 = np.fromiter(set(sides_of(b)), dtype=np.int64)
            c1.append(np.repeat(S1, len(S2)))
            c2.append(np.tile(S2, len(S1)))
            cnt.append(len(S1) * len(S2))
        offs = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
        if node_pairs:
            c1 = np.concatenate(c1)
            c2 = np.concatenate(c2)
            na_ = np.repeat(np.array([a for a, _ in node_pairs], dtype=np.int64), cnt)
            nb_ = np.repeat(np.array([b for _, b in node_pairs], dtype=np.int64), cnt)
            q = side_centroids[c2] + (nodes[na_] - nodes[nb_])
            match = np.all(np.abs(side_centroids[c1] - q) <= 1e-8 + 1e-5 * np.abs(q), axis=1)
            hits = np.nonzero(match)[0]
            hit_pair = np.searchsorted(offs, hits, side="right") - 1
            h1, h2 = c1[hits].tolist(), c2[hits].tolist()
            bounds = np.searchsorted(hit_pair, np.arange(len(node_pairs) + 1)).tolist()
        for k in range(len(node_pairs)):
            corr = list(zip(h1[bounds[k]:bounds[k + 1]], h2[bounds[k]:bounds[k + 1]]))
            for s1, s2 in corr:
                for key, value in b_regions:
                    if s1 in value and s1 not in in_periodic:
                        periodic_sides_dict.setdefault(key[:-2], []).append(s1)
                        periodic_list.append(s1)
                        in_periodic.add(s1)
                        to_discard.append(s2)
                    if s2 in value and s2 not in in_periodic:
                        periodic_sides_dict.setdefault(key[:-2], []).append(s2)
                        periodic_list.append(s2)
                        in_periodic.add(s2)
                        to_discard.append(s1)
        for key in periodic_sides_dict:
            side_physical_regions.pop(key + "_a", None)
            side_physical_regions.pop(key + "_b", None)
        # each kept side s2 couples to the element ea behind its discarded image s1, which takes s2 in
        # place of s1 in its side list (the pairs touch distinct s2 and distinct (ea, s1))
        if periodic_list:
            s1a = np.asarray(to_discard, dtype=np.int64)
            s2a = np.asarray(periodic_list, dtype=np.int64)
            ea = side_elem_map[s1a, 0]
            eb = side_elem_map[s2a, 0]
            side_elem_map[s2a, 1] = ea
            hit = esm[ea] == s1a[:, None]
            if not hit.any(axis=1).all() or len(np.unique(ea * n_sides + s1a)) != len(s1a):
                raise ValueError("periodic sides: a discarded image is not (or twice) a side of its element")
            esm[ea, np.argmax(hit, axis=1)] = s2a
            dists[s2a] = elem_centroids[ea] + side_centroids[s2a] - side_centroids[s1a] - elem_centroids[eb]

    boundary_sides = []
    for value in side_physical_regions.values():
        boundary_sides += list(value)

    second_order_correction = np.zeros((len(boundary_sides), dim))
    if boundary_sides:
        bs = np.array(boundary_sides)
        second_order_correction = dists[bs] - (side_centroids[bs] - elem_centroids[side_elem_map[bs, 0]])

    mask = np.ones(n_sides, dtype=bool)
    mask[np.array(boundary_sides + to_discard, dtype=np.int64)] = False
    internal = np.arange(n_sides)[mask]

    w = elem_centroids[side_elem_map[:, 0]] - nodes[sides[:, 0]]
    tmp2 = np.einsum("ui,ui->u", normal_areas, w)
    tmp = np.einsum("ui,ui->u", normal_areas, dists)
    interp_weights = 1 + tmp2 / tmp

    # least-squares gradient weights
    diff_dist = np.zeros((n_elems, nv, dim))
    keep = np.ones(n_sides, dtype=bool)
    keep[np.array(to_discard, dtype=np.int64)] = False
    # position of side s within its elements' side lists
    s_of = esm.reshape(-1)
    pos_e = np.repeat(np.arange(n_elems), nv)
    pos_r = np.tile(np.arange(nv), n_elems)
    # (elem, side) -> slot
    key = pos_e * (n_sides + 1) + s_of
    lookup_sorted = np.argsort(key)
    key_sorted = key[lookup_sorted]

    def slot(e, s):
        k = e * (n_sides + 1) + s
        idx = np.searchsorted(key_sorted, k)
        return pos_r[lookup_sorted[idx]]

    ks = np.where(keep)[0]
    ke1 = side_elem_map[ks, 0]
    ke2 = side_elem_map[ks, 1]
    inner = ke1 != ke2
    si = ks[inner]
    diff_dist[ke1[inner], slot(ke1[inner], si)] = dists[si]
    diff_dist[ke2[inner], slot(ke2[inner], si)] = -dists[si]
    sb = ks[~inner]
    eb = ke1[~inner]
    diff_dist[eb, slot(eb, sb)] = side_centroids[sb] - elem_centroids[eb]
    gradient_weights = np.linalg.pinv(diff_dist)

    elem_side_map = dict(enumerate(esm.tolist()))
    return Mesh(n_elems, n_nodes, dim, size, nodes, sides, elems, elem_side_map, side_elem_map,
                normal_areas, gradient_weights, interp_weights, elem_centroids, side_centroids,
                elem_volumes, side_areas, dists, second_order_correction, internal, boundary_sides,
                periodic_sides_dict, elem_physical_regions, side_physical_regions)
