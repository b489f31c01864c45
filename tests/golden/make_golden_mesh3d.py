"""Golden 3D mesh fields: the unmodified reference ``get_mesh`` (openbte/mesh.py:54-348) on the tetrahedral
cell stored in ``cube1k5.npz`` (written as msh2 by this package's writer).

Run where the reference is available (see ``ref_loader``); writes ``tests/golden/mesh3d_cube1k5.npz``:

    python tests/golden/make_golden_mesh3d.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))   # ref_loader

import ref_loader  # noqa: E402
from openbte_gb300.geometry import write_msh2  # noqa: E402

FIELDS = ["side_elem_map", "normal_areas", "elem_volumes", "side_areas", "internal", "interp_weights",
          "gradient_weights", "dists", "elem_centroids", "side_centroids", "second_order_correction"]


def main():
    from conftest import load_case
    R = ref_loader.load()
    geo, _, _, _, d = load_case("cube1k5")
    from openbte_gb300.geometry import PeriodicCell2D
    segs = {k[4:]: d[k] for k in d if k.startswith("seg_")}
    cell = PeriodicCell2D(nodes=d["nodes"], elems=d["elems"], segments=segs,
                          periodic={"x": d["periodic_x"], "y": d["periodic_y"], "z": d["periodic_z"]},
                          size=float(d["size"]), porosity=float(d["porosity"]), pore=str(d["pore"]),
                          seed=int(d["seed"]))
    out = {}
    with tempfile.TemporaryDirectory(dir=HERE) as tmp:
        path = write_msh2(cell, os.path.join(tmp, "cube1k5"))
        ref = R.mesh.get_mesh(path[:-4])
    for f in FIELDS:
        out[f] = np.asarray(getattr(ref, f))
    for k, v in ref.periodic_sides.items():
        out["periodic_" + k] = np.asarray(v)
    for k, v in ref.side_physical_regions.items():
        out["region_" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "mesh3d_cube1k5.npz"), **out)
    print("mesh3d_cube1k5:", ref.n_elems, "tetrahedra,", {k: len(v) for k, v in ref.periodic_sides.items()})


if __name__ == "__main__":
    main()
