"""Data contract of the transport path, field-for-field with the reference.

The solver entry points accept either these types or the reference's own
instances (they only read attributes), so user scripts written against
OpenBTE keep working. Field names, order and defaults follow:

* ``Mesh``                         openbte/objects.py:244-268
* ``Material``                     openbte/objects.py:500-509
* ``BoundaryConditions``           openbte/objects.py:220-241
* ``EffectiveThermalConductivity`` openbte/objects.py:128-136
* ``SolverResults``                openbte/objects.py:493-497
"""
from __future__ import annotations

from typing import List, NamedTuple

import numpy as np

f64 = np.float64
i64 = np.int64


class BoundaryConditions(NamedTuple):
    """Boundary conditions (openbte/objects.py:220-241).

    diffuse      name of the side region with diffuse (thermalising) walls
    mixed        {region: {'value': T, 'boundary_conductance': h}}
    periodic     {region: temperature jump across the wrap}
    is_nanowire  nanowire perturbation along z (3D)
    """

    diffuse: str = ""
    mixed: dict = {}
    periodic: dict = {}
    is_nanowire: bool = False

    def get_bc_by_name(self, name: str):
        """'Mixed' or 'Periodic'; ValueError otherwise (openbte/objects.py:232-241).

        Like the reference, any name that is not a mixed region is reported as
        'Periodic' as soon as one periodic region exists.
        """
        if name in self.mixed.keys():
            return "Mixed"
        for _ in self.periodic.keys():
            return "Periodic"
        raise ValueError("{} failed (no region associated to side).".format(name))


class EffectiveThermalConductivity(NamedTuple):
    """Contact used for kappa_eff and its normalisation (openbte/objects.py:128-136)."""

    contact: str
    normalization: f64 = 0

    def get_diffusive(self, T, geometry, boundary_conditions, thermal_conductivity):
        """Diffusive flux through the contact (openbte/objects.py:139-172)."""
        bc = boundary_conditions.get_bc_by_name(self.contact)
        if bc == "Mixed":
            sides = np.asarray(geometry.side_physical_regions[self.contact])
        else:
            sides = np.asarray(geometry.periodic_sides[self.contact])
        k = np.asarray(thermal_conductivity)[: geometry.dim, : geometry.dim]
        na = geometry.normal_areas[sides]
        v_orth = np.einsum("ki,ij,kj->k", na, k, na) / np.einsum("ki,ki->k", na, geometry.dists[sides])
        e = geometry.side_elem_map[sides]
        T1 = T[e[:, 0]]
        if bc == "Mixed":
            T2 = boundary_conditions.mixed[self.contact]["value"]
            h = boundary_conditions.mixed[self.contact]["boundary_conductance"]
            tmp = v_orth * h / (h + v_orth / geometry.side_areas[sides])
        else:
            T2 = T[e[:, 1]] + boundary_conditions.periodic[self.contact]
            tmp = v_orth
        P = 0.0
        for d, t in zip(T1 - T2, tmp):
            P += d * t * self.normalization
        return P


class Mesh(NamedTuple):
    """Unstructured mesh (openbte/objects.py:244-268); built by ``get_mesh``."""

    n_elems: int
    n_nodes: int
    dim: int
    size: np.ndarray
    nodes: np.ndarray
    sides: np.ndarray
    elems: np.ndarray
    elem_side_map: dict
    side_elem_map: np.ndarray
    normal_areas: np.ndarray
    gradient_weights: np.ndarray
    interp_weights: np.ndarray
    elem_centroids: np.ndarray
    side_centroids: np.ndarray
    elem_volumes: np.ndarray
    side_areas: np.ndarray
    dists: np.ndarray
    second_order_correction: np.ndarray
    internal: np.ndarray
    boundary_sides: np.ndarray
    periodic_sides: dict = {}
    elem_physical_regions: dict = {}
    side_physical_regions: dict = {}

    def get_decomposed_directions(self, kappa):
        """Orthogonal / non-orthogonal split of kappa·n (openbte/objects.py:312-319)."""
        v_orth = np.einsum("ki,ij,kj->k", self.normal_areas, kappa, self.normal_areas) / \
            np.einsum("ki,ki->k", self.normal_areas, self.dists)
        v_non_orth = np.einsum("ij,kj->ki", kappa, self.normal_areas) - np.einsum("ki,k->ki", self.dists, v_orth)
        return v_orth, v_non_orth


class SolverResults(NamedTuple):
    """Solver output (openbte/objects.py:493-497)."""

    kappa_eff: float = 0
    aux: dict = {}
    variables: dict = {}


class MaterialRTA(NamedTuple):
    """Mode-resolved bulk data of a material in the relaxation-time approximation (openbte/objects.py:114-120).

    heat_capacity [n_modes] J/m^3/K, scattering_time [n_modes] s, group_velocity [n_modes, 3] m/s,
    frequency [n_modes], thermal_conductivity [3, 3] W/m/K (the last two are carried, not used by the
    binning).
    """

    heat_capacity: np.ndarray
    scattering_time: np.ndarray
    group_velocity: np.ndarray
    frequency: np.ndarray = np.zeros(0)
    thermal_conductivity: np.ndarray = np.zeros(0)


class Material(NamedTuple):
    """Ordinate data (openbte/objects.py:500-509).

    sigma  [n_mfp, n_dir, dim]   W/m/K/nm
    vmfp   [n_dir, dim]          unit directions
    t_coeff[n_mfp, n_dir]        lattice-temperature weights (sum 1)
    mfps   [n_mfp]               nm
    grid   (n_mfp, n_phi) or (n_mfp, n_theta, n_phi)
    """

    thermal_conductivity: np.ndarray
    sigma: np.ndarray
    vmfp: np.ndarray
    t_coeff: np.ndarray
    mfps: np.ndarray
    grid: List
    h: float
    heat_source_coeff: float
