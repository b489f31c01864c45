"""Result container and writers (openbte/objects.py:522-675, the mesh helpers 425-489).

``OpenBTEResults`` holds the material, the mesh and the solver results (``SolverResults`` of ``BTE_RTA`` and
``Fourier``, whose arrays are host numpy arrays) and offers the reference's outputs:

* ``get_variables``: every solver's ``variables`` merged into one dict;
* ``vtu``: a legacy-VTK ASCII file ``<filename>.vtk`` (unstructured grid, triangles / quads / tetrahedra,
  cell data, or node data averaged from the cells), optionally over ``repeat`` periodic copies of the cell;
* ``plot_over_line``: node-averaged values interpolated (linear, ``scipy.interpolate.griddata``) at the
  points ``x`` of a polyline, with the cumulative distance along it;
* ``save`` / ``load``: the same sqlite layout as the reference's ``utils.save`` (a table ``unnamed`` of
  pickled values keyed by field name), read and written with the standard library.

``repeat`` tiles the cell and its data like the reference (``duplicate_cells``: the data are tiled without
adding the periodic temperature jumps); copies along z are shifted by z x size[2] (the reference shifts them
by y x size[2]).
"""
from __future__ import annotations

import os
import pickle
import sqlite3
from typing import NamedTuple

import numpy as np

__all__ = ["OpenBTEResults", "duplicate_cells", "cell_to_node"]


def duplicate_cells(mesh, variables: dict, repeat=(1, 1, 1)):
    """(nodes, elems) of `repeat` copies of the cell; tiles the arrays of `variables` in place
    (openbte/objects.py:425-458)."""
    repeat = [int(r) for r in repeat]
    if repeat == [1, 1, 1]:
        return mesh.nodes, mesh.elems
    nodes = [np.asarray(mesh.nodes)]
    elems = [np.asarray(mesh.elems)]
    base_n = len(mesh.nodes)
    size = np.asarray(mesh.size, dtype=np.float64)
    k = 0
    for x in range(repeat[0]):
        for y in range(repeat[1]):
            for z in range(repeat[2]):
                if x == 0 and y == 0 and z == 0:
                    continue
                k += 1
                shift = np.zeros(mesh.dim)
                shift[0] = x * size[0]
                shift[1] = y * size[1]
                if mesh.dim == 3:
                    shift[2] = z * size[2]
                nodes.append(np.asarray(mesh.nodes) + shift[None, :])
                elems.append(np.asarray(mesh.elems) + k * base_n)
    copies = int(np.prod(repeat))
    for value in variables.values():
        d = np.asarray(value["data"])
        value["data"] = np.tile(d, copies) if d.ndim == 1 else np.tile(d, (copies,) + (1,) * (d.ndim - 1))
    return np.vstack(nodes), np.vstack(elems)


def cell_to_node(variables: dict, nodes, elems) -> dict:
    """Node values as the mean of the values of the cells sharing the node (openbte/objects.py:461-489)."""
    elems = np.asarray(elems)
    n_nodes = len(nodes)
    conn = np.bincount(elems.reshape(-1), minlength=n_nodes).astype(np.float64)
    out = {}
    for key, value in variables.items():
        d = np.asarray(value["data"], dtype=np.float64)
        acc = np.zeros((n_nodes,) + d.shape[1:])
        np.add.at(acc, elems.reshape(-1), np.repeat(d, elems.shape[1], axis=0))
        with np.errstate(invalid="ignore", divide="ignore"):
            acc = acc / (conn if d.ndim == 1 else conn[:, None])
        out[key] = {"data": acc, "units": value.get("units", "")}
    return out


class OpenBTEResults(NamedTuple):
    """Material, mesh and solver results (openbte/objects.py:522-551)."""

    material: object
    mesh: object
    solvers: dict = {}
    mat_mode: object = None

    @classmethod
    def load(cls, filename: str = "state"):
        con = sqlite3.connect(f"file:{filename}.db?mode=ro", uri=True)
        try:
            data = {k: pickle.loads(v) for k, v in con.execute("SELECT key, value FROM unnamed ORDER BY rowid")}
        finally:
            con.close()
        return cls(**{k: v for k, v in data.items() if k in cls._fields})

    def save(self, filename: str = "state"):
        fn = filename + ".db"
        con = sqlite3.connect(fn)
        try:
            con.execute("CREATE TABLE IF NOT EXISTS unnamed (key TEXT PRIMARY KEY, value BLOB)")
            for key, value in self._asdict().items():
                con.execute("REPLACE INTO unnamed (key, value) VALUES (?, ?)", (key, pickle.dumps(value)))
            con.commit()
        finally:
            con.close()

    def get_variables(self) -> dict:
        variables = {}
        for value in self.solvers.values():
            variables.update({k: dict(v) for k, v in value.variables.items()})
        return variables

    def plot_over_line(self, variables, x, direction="x", repeat=(1, 1, 1)):
        """(distance along the polyline x [N, dim], {variable: values at x})  (openbte/objects.py:555-582)."""
        from scipy.interpolate import griddata
        x = np.asarray(x, dtype=np.float64)
        cell_vars = self.get_variables()
        nodes, elems = duplicate_cells(self.mesh, cell_vars, repeat)
        node_vars = cell_to_node(cell_vars, nodes, elems)
        out = {v: griddata(np.asarray(nodes)[:, : self.mesh.dim], node_vars[v]["data"], x) for v in variables}
        dist = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(x, axis=0), axis=1))])
        return dist, out

    def vtu(self, filename: str = "output", dof: str = "cell", repeat=(1, 1, 1)):
        """Write `<filename>.vtk` (legacy VTK, ASCII unstructured grid) (openbte/objects.py:584-675)."""
        mesh = self.mesh
        variables = self.get_variables()
        nodes, elems = duplicate_cells(mesh, variables, repeat)
        nodes = np.asarray(nodes, dtype=np.float64)
        elems = np.asarray(elems)
        n_nodes, n_elems, nv = len(nodes), len(elems), elems.shape[1]
        if mesh.dim == 2:
            ctype = 5 if nv == 3 else 9
            pts = np.hstack([nodes[:, :2], np.zeros((n_nodes, 1))])
        else:
            ctype = 10
            pts = nodes[:, :3]
        if dof != "cell":
            variables = cell_to_node(variables, nodes, elems)
        lines = ["# vtk DataFile Version 2.0", "OpenBTE Data", "ASCII", "DATASET UNSTRUCTURED_GRID",
                 f"POINTS {n_nodes} double"]
        lines += [" ".join(repr(float(c)) for c in p) for p in pts]
        lines.append(f"CELLS {n_elems} {(nv + 1) * n_elems}")
        lines += [f"{nv} " + " ".join(str(int(i)) for i in e) for e in elems]
        lines.append(f"CELL_TYPES {n_elems}")
        lines.append(" ".join([str(ctype)] * n_elems))
        lines.append(f"{'CELL_DATA' if dof == 'cell' else 'POINT_DATA'} {n_elems if dof == 'cell' else n_nodes}")
        for key, value in variables.items():
            name = f"{key}[{value.get('units', '')}]"
            d = np.asarray(value["data"], dtype=np.float64)
            if d.ndim == 1:
                lines += [f"SCALARS {name} double", "LOOKUP_TABLE default", " ".join(repr(float(v)) for v in d)]
            elif d.ndim == 2:
                if d.shape[1] == 2:
                    d = np.hstack([d, np.zeros((len(d), 1))])
                lines.append(f"VECTORS {name} double")
                lines += [" ".join(repr(float(v)) for v in row) for row in d]
        with open(filename + ".vtk", "w") as f:
            f.write("\n".join(lines) + "\n")
        return os.path.abspath(filename + ".vtk")
