"""The oracle's Krylov solve of the source-iteration fixed point against its plain iteration (CPU)."""
import os

import numpy as np

import bte_oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_krylov_fixed_point_equals_source_iteration():
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cell_2d(300, 0.25, "square", seed=4))
    mat = synthetic_isotropic_2d(6, 12)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    k0, dT0, J0, *_ = bte_oracle.bte_rta(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-13,
                                         bte_max_iter=2000)
    k1, dT1, J1, *_, mv = bte_oracle.bte_rta_krylov(geo, mat, bcs, effective_thermal_conductivity=ek, rtol=1e-13)
    assert abs(k1 - k0) <= 1e-9 * abs(k0), (k0, k1)
    V = geo.elem_volumes
    c0 = dT0 - (V @ dT0) / V.sum()
    c1 = dT1 - (V @ dT1) / V.sum()
    assert np.abs(c1 - c0).max() <= 1e-9 * np.abs(c0).max()
    np.testing.assert_allclose(J1, J0, rtol=0, atol=1e-9 * np.abs(J0).max())
    assert mv < 200
