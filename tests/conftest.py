import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    # temporary files of tests (tmp_path) stay inside the checkout unless a base directory is given
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, ".pytest_tmp")
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


def load_case(name):
    """Golden fixture -> (geo, mat, bcs, ek, data) built with this package's own mesh builder."""
    from openbte_gb300.geometry import PeriodicCell2D
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300 import objects as O
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
    segs = {k[4:]: d[k] for k in d if k.startswith("seg_")}
    periodic = {"x": d["periodic_x"], "y": d["periodic_y"]}
    jumps = {"Periodic_x": 1, "Periodic_y": 0}
    if "periodic_z" in d:
        periodic["z"] = d["periodic_z"]
        jumps["Periodic_z"] = 0
    cell = PeriodicCell2D(nodes=d["nodes"], elems=d["elems"], segments=segs, periodic=periodic,
                          size=float(d["size"]), porosity=float(d["porosity"]), pore=str(d["pore"]),
                          seed=int(d["seed"]))
    geo = mesh_from_cell(cell)
    n_mfp, n_phi = d["t_coeff"].shape
    mat = O.Material(d["kappa_bulk"], d["sigma"], d["vmfp"], d["t_coeff"], d["mfps"], (n_mfp, n_phi), 0.0, 0.0)
    bcs = O.BoundaryConditions(periodic=jumps, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=float(d.get("normalization", -1.0)), contact="Periodic_x")
    return geo, mat, bcs, ek, d


@pytest.fixture
def case():
    return load_case


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
