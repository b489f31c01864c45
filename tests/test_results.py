"""Result container and writers (vtk file, node averaging, line sampling, periodic copies, save/load)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _results():
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.results import OpenBTEResults
    geo = mesh_from_cell(porous_cell_2d(300, 0.2, "square", seed=2))
    T = np.asarray(geo.elem_centroids)[:, 0].copy()
    J = np.tile([1.0, 2.0], (geo.n_elems, 1))
    bte = O.SolverResults(kappa_eff=1.0, variables={"Temperature_BTE": {"data": T, "units": "K"},
                                                     "Flux_BTE": {"data": J, "units": "W/m/m"}})
    return geo, OpenBTEResults(material=None, mesh=geo, solvers={"bte": bte})


def test_vtk_file_layout(tmp_path):
    geo, res = _results()
    fn = res.vtu(str(tmp_path / "out"))
    lines = open(fn).read().split("\n")
    assert lines[:4] == ["# vtk DataFile Version 2.0", "OpenBTE Data", "ASCII", "DATASET UNSTRUCTURED_GRID"]
    assert lines[4] == f"POINTS {geo.n_nodes} double"
    i = lines.index(f"CELLS {geo.n_elems} {4 * geo.n_elems}")
    assert lines[i + 1].split()[0] == "3"
    j = lines.index(f"CELL_TYPES {geo.n_elems}")
    assert set(lines[j + 1].split()) == {"5"}
    assert lines[j + 2] == f"CELL_DATA {geo.n_elems}"
    k = lines.index("SCALARS Temperature_BTE[K] double")
    np.testing.assert_allclose(np.array(lines[k + 2].split(), dtype=float), res.get_variables()["Temperature_BTE"]["data"])
    v = lines.index("VECTORS Flux_BTE[W/m/m] double")
    assert lines[v + 1].split() == ["1.0", "2.0", "0.0"]
    fn = res.vtu(str(tmp_path / "pts"), dof="node")
    assert f"POINT_DATA {geo.n_nodes}" in open(fn).read()


def test_node_average_and_line_sampling():
    from openbte_gb300.results import cell_to_node
    geo, res = _results()
    nv = cell_to_node(res.get_variables(), geo.nodes, geo.elems)
    np.testing.assert_allclose(nv["Flux_BTE"]["data"], np.tile([1.0, 2.0], (geo.n_nodes, 1)))
    used = np.unique(np.asarray(geo.elems))
    err = np.abs(nv["Temperature_BTE"]["data"][used] - np.asarray(geo.nodes)[used, 0])
    h = np.sqrt(2 * np.sum(geo.elem_volumes) / geo.n_elems)       # typical element size
    assert err.max() < h                     # a centroid average sits within an element of the node
    # the cell spans [-50, 50]^2 with the pore at the centre: a line through the material
    x = np.stack([np.linspace(-45, 45, 19), np.full(19, -40.0)], axis=1)
    dist, out = res.plot_over_line(["Temperature_BTE"], x)
    np.testing.assert_allclose(dist[-1], 90.0)
    np.testing.assert_allclose(out["Temperature_BTE"], x[:, 0], atol=h)


def test_periodic_copies_and_save_load(tmp_path):
    from openbte_gb300.results import OpenBTEResults, duplicate_cells
    geo, res = _results()
    var = res.get_variables()
    nodes, elems = duplicate_cells(geo, var, [2, 3, 1])
    assert nodes.shape == (6 * geo.n_nodes, 2) and elems.shape == (6 * geo.n_elems, 3)
    assert len(var["Temperature_BTE"]["data"]) == 6 * geo.n_elems
    np.testing.assert_allclose(nodes[geo.n_nodes:2 * geo.n_nodes] - np.asarray(geo.nodes), [[0.0, geo.size[1]]] * geo.n_nodes)
    res.save(str(tmp_path / "state"))
    back = OpenBTEResults.load(str(tmp_path / "state"))
    np.testing.assert_array_equal(back.solvers["bte"].variables["Temperature_BTE"]["data"],
                                  res.solvers["bte"].variables["Temperature_BTE"]["data"])
    assert back.mesh.n_elems == geo.n_elems


def test_node_average_matches_reference():
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import ref_loader
    if not ref_loader.available():
        pytest.skip("reference checkout not present")
    from openbte_gb300.results import cell_to_node
    ref = ref_loader.load()
    geo, res = _results()
    var = res.get_variables()
    want = ref.objects.Mesh.cell_to_node(None, {k: dict(v) for k, v in var.items()}, geo.nodes, geo.elems)
    got = cell_to_node(var, geo.nodes, geo.elems)
    for k in var:
        np.testing.assert_allclose(got[k]["data"], want[k]["data"], rtol=1e-13, atol=1e-13)
