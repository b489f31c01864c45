"""Generate golden fixtures by running the unmodified OpenBTE reference.

Run in a checkout where the reference is available (``OBTE_REFERENCE``, by
default the copy installed under baseline/_ref); the fixtures are committed so the
tests never need the reference at run time:

    python tests/golden/make_golden.py

Each case writes ``tests/golden/<name>.npz`` with the mesh as a seeded
``PeriodicCell2D`` (nodes, elements, boundary segments, periodic pairs), the
material, and the reference's outputs: ``Fourier`` (temperature, flux,
printed kappa) and ``BTE_RTA`` at bte_rtol=1e-12 (kappa, temperature, flux,
suppression). Case ``a600`` also stores the reference ``get_mesh`` fields.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))   # ref_loader

import ref_loader  # noqa: E402
from openbte_gb300.geometry import porous_cell_2d, porous_cube_3d, write_msh2  # noqa: E402
from openbte_gb300.material import synthetic_isotropic_2d, synthetic_isotropic_3d, Gray2D  # noqa: E402

CASES = [
    # name, n_tri, porosity, pore, seed, material kind, material args
    ("a600", 600, 0.25, "square", 5, "synthetic", dict(n_mfp=8, n_phi=16)),
    ("c0_2k", 2000, 0.25, "square", 1, "synthetic", dict(n_mfp=30, n_phi=48)),
    ("circ1k", 1000, 0.30, "circle", 2, "synthetic", dict(n_mfp=10, n_phi=24)),
    ("gray600", 600, 0.20, "square", 7, "gray", dict(MFP=100.0, n_phi=32, kappa=150.0)),
    ("cube1k5", 1500, 0.10, "sphere", 3, "synthetic3d", dict(n_mfp=6, n_theta=4, n_phi=8)),
]

MESH_FIELDS = ["side_elem_map", "normal_areas", "elem_volumes", "side_areas", "internal", "interp_weights",
               "gradient_weights", "dists", "elem_centroids"]


def run_case(R, name, n_tri, porosity, pore, seed, kind, margs, tmpdir):
    if pore == "sphere":
        cell = porous_cube_3d(n_tri, porosity, seed=seed)
        periodic = {"Periodic_x": 1, "Periodic_y": 0, "Periodic_z": 0}
    else:
        cell = porous_cell_2d(n_tri, porosity, pore, seed=seed)
        periodic = {"Periodic_x": 1, "Periodic_y": 0}
    path = write_msh2(cell, os.path.join(tmpdir, name))
    geo = R.mesh.get_mesh(path[:-4])
    if kind == "synthetic":
        mat = synthetic_isotropic_2d(**margs)
    elif kind == "synthetic3d":
        mat = synthetic_isotropic_3d(**margs)
    else:
        mat = Gray2D(**margs)
    rmat = R.objects.Material(*mat)
    bcs = R.objects.BoundaryConditions(periodic=periodic, diffuse="Boundary")
    # -L_x / (contact area per unit length in 2D, contact area in 3D) / DeltaT
    normalization = -1.0 if pore != "sphere" else -1.0 / cell.size
    ek = R.objects.EffectiveThermalConductivity(normalization=normalization, contact="Periodic_x")
    out = io.StringIO()
    t0 = time.time()
    with contextlib.redirect_stdout(out):
        f = R.fourier.Fourier(geo, rmat.thermal_conductivity, bcs, effective_thermal_conductivity=ek)
    printed = [l for l in out.getvalue().splitlines() if l.startswith("Kappa (Fourier)")]
    kappa_fourier = float(printed[-1].split(":")[1].split(",")[0])
    t1 = time.time()
    b = R.bte.BTE_RTA(geo, rmat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-12,
                      bte_max_iter=2000)
    t2 = time.time()
    b4 = R.bte.BTE_RTA(geo, rmat, bcs, fourier=f, effective_thermal_conductivity=ek)
    d = dict(
        nodes=cell.nodes, elems=cell.elems, size=cell.size, porosity=cell.porosity, pore=cell.pore, seed=cell.seed,
        periodic_x=cell.periodic["x"], periodic_y=cell.periodic["y"],
        **({"periodic_z": cell.periodic["z"]} if "z" in cell.periodic else {}),
        mat_kind=kind, mat_args=repr(margs), normalization=normalization, jumps=repr(periodic),
        mfps=mat.mfps, vmfp=mat.vmfp, sigma=mat.sigma, t_coeff=mat.t_coeff, kappa_bulk=mat.thermal_conductivity,
        fourier_T=f.variables["Temperature_Fourier"]["data"], fourier_J=f.variables["Flux_Fourier"]["data"],
        fourier_kappa_printed=kappa_fourier, fourier_kappa_returned=f.kappa_eff,
        bte_kappa=b.kappa_eff, bte_T=b.variables["Temperature_BTE"]["data"], bte_J=b.variables["Flux_BTE"]["data"],
        bte_S=b.aux["suppression"], bte_kappa_rtol1e4=b4.kappa_eff,
        t_fourier=t1 - t0, t_bte=t2 - t1,
    )
    for region, segs in cell.segments.items():
        d["seg_" + region] = segs
    if name == "a600":
        for fld in MESH_FIELDS:
            d["mesh_" + fld] = np.asarray(getattr(geo, fld))
        d["mesh_periodic_x"] = np.asarray(geo.periodic_sides["Periodic_x"])
        d["mesh_periodic_y"] = np.asarray(geo.periodic_sides["Periodic_y"])
        d["mesh_boundary"] = np.asarray(geo.side_physical_regions["Boundary"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: n={geo.n_elems} kappa_bte={b.kappa_eff:.12g} (rtol1e-4: {b4.kappa_eff:.8g}) "
          f"kappa_fourier={kappa_fourier:.8g} t_bte={t2 - t1:.1f}s")


def main():
    import tempfile
    R = ref_loader.load()
    only = sys.argv[1:]
    with tempfile.TemporaryDirectory(dir=HERE) as tmp:   # scratch msh files beside the fixtures
        for c in CASES:
            if only and c[0] not in only:
                continue
            run_case(R, *c, tmp)


if __name__ == "__main__":
    main()
