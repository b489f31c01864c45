"""Host recomputation of the sweep schedule — TEST INFRASTRUCTURE ONLY.

An independent numpy implementation of the per-direction upwind ordering that
the library builds in C++: directed internal faces with coefficient
g = s_q·(±n A / V) (openbte/bte.py:48-60), inflow where g < 0, inflow across
kept periodic sides removed (those become interface unknowns), levels = longest
path from the sources computed by vectorised relaxation, order = (level, id).
Tests compare the library's schedule with this bit for bit.
"""
from __future__ import annotations

import numpy as np


def directed_faces(geo):
    sem = np.asarray(geo.side_elem_map)
    internal = np.asarray(geo.internal)
    i = sem[internal, 0]
    j = sem[internal, 1]
    k1 = geo.normal_areas[internal] / geo.elem_volumes[i][:, None]
    k2 = -geo.normal_areas[internal] / geo.elem_volumes[j][:, None]
    per = set()
    for sides in geo.periodic_sides.values():
        per.update(int(s) for s in sides)
    cut = np.array([int(s) in per for s in internal], dtype=bool)
    return (np.concatenate([i, j]), np.concatenate([j, i]), np.vstack([k1, k2]), np.concatenate([cut, cut]))


def levels(geo, direction, faces=None):
    """Longest-path level of every element for one direction (periodic inflow cut)."""
    row, nb, k, cut = faces if faces is not None else directed_faces(geo)
    d = np.asarray(direction, dtype=np.float64)[: geo.dim]
    g = k @ d
    e = (g < 0) & ~cut
    r, c = row[e], nb[e]
    lev = np.zeros(geo.n_elems, dtype=np.int64)
    for _ in range(geo.n_elems + 1):
        new = lev.copy()
        np.maximum.at(new, r, lev[c] + 1)
        if np.array_equal(new, lev):
            return lev
        lev = new
    raise RuntimeError("upwind graph has a cycle")


def schedule(geo, direction, faces=None):
    """(order, level_ptr) as the library reports them."""
    lev = levels(geo, direction, faces)
    order = np.lexsort((np.arange(geo.n_elems), lev))
    counts = np.bincount(lev, minlength=int(lev.max()) + 1)
    level_ptr = np.concatenate([[0], np.cumsum(counts)])
    return order, level_ptr
