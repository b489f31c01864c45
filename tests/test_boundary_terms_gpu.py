"""Isothermal (mixed) walls and heat sources on the device path against the CPU oracle
(openbte/bte.py:90-96,127-130,211; openbte/fourier.py:70-86)."""
import numpy as np
import pytest

import bte_oracle
import fourier_oracle
from openbte_gb300 import objects as O

pytestmark = pytest.mark.gpu


def _cell():
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    return mesh_from_cell(porous_cell_2d(500, 0.2, "circle", seed=9)), synthetic_isotropic_2d(6, 12)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32_refine", 1e-6)])
def test_bte_isothermal_pore_matches_oracle(precision, tol):
    from openbte_gb300 import BTE_RTA
    geo, mat = _cell()
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0},
                               mixed={"Boundary": {"value": 0.3, "boundary_conductance": 1e3}})
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    k_ref, dT_ref, J_ref, *_ = bte_oracle.bte_rta(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-13,
                                                  bte_max_iter=3000)
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-11, precision=precision)
    assert abs(r.aux["kappa_eff"] - k_ref) <= tol * abs(k_ref), (r.aux["kappa_eff"], k_ref)
    # isothermal walls fix the temperature level: the fields compare directly
    dT = r.variables["Temperature_BTE"]["data"]
    assert np.abs(dT - dT_ref).max() <= 10 * tol * np.abs(dT_ref).max()
    J = r.variables["Flux_BTE"]["data"] / 1e9
    assert np.abs(J - J_ref).max() <= 10 * tol * np.abs(J_ref).max()


def test_bte_heat_source_matches_oracle():
    from openbte_gb300 import BTE_RTA
    geo, mat = _cell()
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 0, "Periodic_y": 0},
                               mixed={"Boundary": {"value": 0.0, "boundary_conductance": 1e3}})
    rng = np.random.default_rng(3)
    hs = O.SolverResults(variables={"Heat_Source": {"data": 1e-3 * (1 + rng.uniform(size=geo.n_elems))}})
    _, dT_ref, *_ = bte_oracle.bte_rta(geo, mat, bcs, heat_source=hs, bte_rtol=1e-13, bte_max_iter=3000)
    r = BTE_RTA(geo, mat, bcs, heat_source=hs, bte_rtol=1e-11, precision="fp64")
    dT = r.variables["Temperature_BTE"]["data"]
    assert np.abs(dT - dT_ref).max() <= 1e-8 * np.abs(dT_ref).max()


def test_fourier_isothermal_pore_matches_oracle():
    from openbte_gb300 import Fourier
    geo, mat = _cell()
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0},
                               mixed={"Boundary": {"value": 0.3, "boundary_conductance": 1e3}})
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    k_ref, T_ref, J_ref, _ = fourier_oracle.fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek)
    r = Fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek, verbose=False)
    assert abs(r.aux["kappa_eff"] - k_ref) <= 1e-9 * abs(k_ref), (r.aux["kappa_eff"], k_ref)
    T = r.variables["Temperature_Fourier"]["data"]
    assert np.abs(T - T_ref).max() <= 1e-9 * np.abs(T_ref).max()


def test_bte_kappa_on_isothermal_contact_matches_oracle():
    """kappa_eff from the heat flux into an isothermal region (contact kind Mixed, openbte/bte.py:144-148).

    With the periodic jump alone the net flux into the walls is zero (energy conservation); a heat source
    makes it the heat generated."""
    from openbte_gb300 import BTE_RTA
    geo, mat = _cell()
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0},
                               mixed={"Boundary": {"value": 0.3, "boundary_conductance": 1e3}})
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Boundary")
    hs = O.SolverResults(variables={"Heat_Source": {"data": np.full(geo.n_elems, 2e-3)}})
    k_ref, *_ = bte_oracle.bte_rta(geo, mat, bcs, effective_thermal_conductivity=ek, heat_source=hs, bte_rtol=1e-13,
                                   bte_max_iter=3000)
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, heat_source=hs, bte_rtol=1e-11, precision="fp64")
    assert abs(k_ref) > 1e-3
    assert abs(r.aux["kappa_eff"] - k_ref) <= 1e-9 * abs(k_ref), (r.aux["kappa_eff"], k_ref)


def test_bte_nanowire_matches_oracle():
    """The nanowire perturbation along z and its kappa over all elements (openbte/bte.py:113-119,135-140)."""
    from openbte_gb300 import BTE_RTA
    from openbte_gb300.geometry import porous_cube_3d
    from openbte_gb300.material import synthetic_isotropic_3d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cube_3d(700, 0.1, seed=2))
    mat = synthetic_isotropic_3d(4, 6, 8)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 0, "Periodic_y": 0, "Periodic_z": 0}, diffuse="Boundary",
                               is_nanowire=True)
    ek = O.EffectiveThermalConductivity(normalization=-1 / 1e6, contact="Periodic_z")
    k_ref, *_ = bte_oracle.bte_rta(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-13, bte_max_iter=3000)
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-11, precision="fp64")
    assert abs(r.aux["kappa_eff"] - k_ref) <= 1e-8 * abs(k_ref), (r.aux["kappa_eff"], k_ref)
