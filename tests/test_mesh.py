"""Mesh generation and the vectorised get_mesh against the reference's fields."""
import os

import numpy as np
import pytest

from openbte_gb300.geometry import porous_cell_2d, write_msh2
from openbte_gb300.mesh import get_mesh, mesh_from_cell


def test_mesh_matches_reference_fields(case):
    geo, _, _, _, d = case("a600")
    for fld in ["side_elem_map", "normal_areas", "elem_volumes", "side_areas", "internal", "interp_weights",
                "gradient_weights", "dists", "elem_centroids"]:
        a = np.asarray(getattr(geo, fld))
        b = d["mesh_" + fld]
        assert a.shape == b.shape, fld
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12, err_msg=fld)
    np.testing.assert_array_equal(geo.periodic_sides["Periodic_x"], d["mesh_periodic_x"])
    np.testing.assert_array_equal(geo.periodic_sides["Periodic_y"], d["mesh_periodic_y"])
    np.testing.assert_array_equal(geo.side_physical_regions["Boundary"], d["mesh_boundary"])


def test_msh2_roundtrip(tmp_path):
    cell = porous_cell_2d(400, 0.2, "circle", seed=3)
    path = write_msh2(cell, str(tmp_path / "m"))
    a = get_mesh(path[:-4])
    b = mesh_from_cell(cell)
    for fld in ["side_elem_map", "normal_areas", "elem_volumes", "internal", "gradient_weights"]:
        np.testing.assert_allclose(np.asarray(getattr(a, fld)), np.asarray(getattr(b, fld)), rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("pore", ["square", "circle"])
def test_generator_properties(pore):
    cell = porous_cell_2d(1500, 0.25, pore, seed=11)
    geo = mesh_from_cell(cell)
    area = geo.elem_volumes.sum()
    assert abs(area - 100.0 * 100.0 * 0.75) / area < 0.02
    assert 1200 < geo.n_elems < 1800
    # periodic pairs match exactly and every periodic side is an internal coupling
    assert len(geo.periodic_sides["Periodic_x"]) == len(cell.segments["Periodic_x_b"])
    internal = set(np.asarray(geo.internal).tolist())
    for s in geo.periodic_sides["Periodic_x"]:
        assert int(s) in internal
    # closed cells: sum of outward normal areas vanishes per element
    acc = np.zeros((geo.n_elems, 2))
    sem = geo.side_elem_map
    for s in list(internal) + list(geo.boundary_sides):
        i, j = sem[s]
        acc[i] += geo.normal_areas[s]
        if i != j:
            acc[j] -= geo.normal_areas[s]
    # periodic kept sides close the a-side element across the wrap; discarded images close nothing
    assert np.abs(acc).max() < 1e-9 * 100


def test_seeded_generator_is_deterministic():
    a = porous_cell_2d(800, 0.25, "square", seed=4)
    b = porous_cell_2d(800, 0.25, "square", seed=4)
    np.testing.assert_array_equal(a.nodes, b.nodes)
    np.testing.assert_array_equal(a.elems, b.elems)


@pytest.mark.parametrize("three", [False, True])
def test_row_key_and_fallback_paths_agree(monkeypatch, three):
    """Sides and face lookups through integer row keys give the mesh of the np.unique(axis=0) / dict path
    that very large meshes take (n_nodes ** dim beyond int64)."""
    from openbte_gb300 import mesh as M
    from openbte_gb300.geometry import porous_cube_3d
    cell = porous_cube_3d(800, 0.1, seed=2) if three else porous_cell_2d(600, 0.25, "circle", seed=9)
    a = mesh_from_cell(cell)
    monkeypatch.setattr(M, "_row_keys", lambda rows, n_nodes: None)
    b = mesh_from_cell(cell)
    for fld in a._fields:
        x, y = getattr(a, fld), getattr(b, fld)
        if isinstance(x, dict):
            assert list(x.keys()) == list(y.keys()), fld
            for k in x:
                np.testing.assert_array_equal(np.asarray(x[k]), np.asarray(y[k]), err_msg=f"{fld}[{k}]")
        else:
            np.testing.assert_array_equal(np.asarray(x), np.asarray(y), err_msg=fld)


def test_3d_mesh_matches_reference_fields(case):
    """The tetrahedral cell of cube1k5 against the reference get_mesh on the same cell
    (tests/golden/make_golden_mesh3d.py)."""
    geo, _, _, _, _ = case("cube1k5")
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "mesh3d_cube1k5.npz"))
    for fld in ["side_elem_map", "normal_areas", "elem_volumes", "side_areas", "internal", "interp_weights",
                "gradient_weights", "dists", "elem_centroids", "side_centroids", "second_order_correction"]:
        a, b = np.asarray(getattr(geo, fld)), d[fld]
        assert a.shape == b.shape, fld
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12, err_msg=fld)
    for k in ("Periodic_x", "Periodic_y", "Periodic_z"):
        np.testing.assert_array_equal(geo.periodic_sides[k], d["periodic_" + k])
    np.testing.assert_array_equal(geo.side_physical_regions["Boundary"], d["region_Boundary"])
