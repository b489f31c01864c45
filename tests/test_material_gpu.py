"""BTE_RTA with a material binned from mode data (RTA2DSym) against the CPU oracle."""
import numpy as np
import pytest

import bte_oracle
from openbte_gb300 import objects as O

pytestmark = pytest.mark.gpu


def _node_modes(n_mfp, n_phi, mfp_min, mfp_max, seed):
    """Modes sitting on the (MFP, direction) nodes of RTA2DSym's grid, in +-v pairs.

    On the nodes the bilinear binning is exact, so sigma = W x MFP x direction per node and the diffuse walls
    conserve energy (for modes between nodes the binned sigma and W disagree at the 1e-5 level and the
    fixed point of the reference's iteration exists only up to that inconsistency).
    """
    rng = np.random.default_rng(seed)
    grid = np.logspace(np.log10(mfp_min) * 1.01, np.log10(mfp_max), n_mfp, endpoint=True)
    phi = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    cv_half = rng.uniform(0.2, 1.0, (n_mfp, n_phi // 2)) * 1e6
    cv = np.concatenate([cv_half, cv_half], axis=1)           # q and q + n_phi/2 are reversed directions
    tau = 1e-11
    r, p = np.meshgrid(grid, phi, indexing="ij")
    vg = np.stack([np.sin(p), np.cos(p), np.zeros_like(p)], axis=-1) * (r / tau)[..., None]
    return O.MaterialRTA(cv.reshape(-1), np.full(cv.size, tau), vg.reshape(-1, 3)), grid


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("fp32_refine", 1e-6)])
def test_rta2dsym_kappa_matches_oracle(precision, tol):
    from openbte_gb300 import BTE_RTA
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import RTA2DSym
    from openbte_gb300.mesh import mesh_from_cell
    n_mfp, n_phi = 8, 16
    data, grid = _node_modes(n_mfp, n_phi, 5e-9, 400e-9, 7)
    mat = RTA2DSym(data, n_phi=n_phi, n_mfp=n_mfp, mfp_min=5e-9, mfp_max=400e-9)
    np.testing.assert_allclose(mat.mfps, grid * 1e9, rtol=1e-12)
    geo = mesh_from_cell(porous_cell_2d(600, 0.2, "circle", seed=5))
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    k_ref, dT_ref, J_ref, *_ = bte_oracle.bte_rta_krylov(geo, mat, bcs, effective_thermal_conductivity=ek, rtol=1e-12)
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-10, precision=precision)
    k = r.aux["kappa_eff"]
    assert abs(k - k_ref) <= tol * abs(k_ref), (k, k_ref)
    V = geo.elem_volumes
    dT = r.variables["Temperature_BTE"]["data"]
    a, b = dT - (V @ dT) / V.sum(), dT_ref - (V @ dT_ref) / V.sum()
    assert np.abs(a - b).max() <= 100 * tol * np.abs(b).max()
