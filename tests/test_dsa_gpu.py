"""Diffusion-synthetic acceleration: the same fixed point in fewer sweeps.

On the transmission-interface pixel model (openbte/inverse/bte.py:145-163) the slow modes of the source
iteration are temperatures relaxing across the network of partially transmitting pixel sides; the
diffusion correction removes them.  kappa, the temperature field and the gradient are unchanged to the
solve tolerance; the sweep count drops."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density(n, seed):
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n)
    kk = k[:, None] ** 2 + k[None, :] ** 2
    z = np.real(np.fft.ifft2(np.fft.fft2(z) * np.exp(-kk * (n / 8.0) ** 2)))
    return ((z - z.min()) / (z.max() - z.min())).reshape(-1)


@pytest.mark.parametrize("precision,ktol,gtol", [("fp64", 1e-8, 1e-6), ("fp32_refine", 5e-8, 1e-5)])
def test_inverse_same_gradient_fewer_sweeps(precision, ktol, gtol):
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    n = 48
    mat = IsotropicMaterial.lognormal(12, 32)
    rho = _density(n, 3)
    out = {}
    for dsa in (-1, 1):
        solver = PixelSolver(n, mat, size=100.0, precision=precision, rtol=1e-10, dsa=dsa)
        k, g = solver.kappa_and_gradient(rho)
        out[dsa] = (k, g.cpu().numpy(), solver.last_info.n_sweeps)
    (k0, g0, s0), (k1, g1, s1) = out[-1], out[1]
    assert abs(k1 - k0) <= ktol * abs(k0), (k0, k1)
    # the field's minimum is a pixel of density 0, whose sides transmit 1e-12: its temperature is a mode
    # that I - K relaxes at a rate ~1e-12, which no iterative solve resolves (with or without the
    # acceleration), so its gradient is left out
    live = rho > 1e-6
    assert (~live).sum() <= 2
    assert np.max(np.abs(g1 - g0)[live]) <= gtol * np.max(np.abs(g0[live]))
    assert s1 < 0.7 * s0, (s0, s1)


def test_dsa_on_a_porous_cell_keeps_the_fixed_point():
    """Forced on where it is off by default (a porous 2D cell with diffuse walls and no interfaces): the
    same kappa and temperatures to the tolerance."""
    import torch
    from openbte_gb300 import objects as O
    from openbte_gb300.bte import solve_plan
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.runtime import HostProblem, Plan
    geo = mesh_from_cell(porous_cell_2d(1500, 0.25, "square", seed=7))
    mat = synthetic_isotropic_2d(16, 32)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device="cuda:0")
    res = {}
    for dsa in (-1, 1):
        plan = Plan(HostProblem(geo, mat, bcs, ek), 0)
        info, dT, J, K, _ = solve_plan(plan, dT0, precision="fp64", rtol=1e-10, max_sweeps=3000, restart=60,
                                       precond=-1, dsa=dsa)
        assert info.converged
        res[dsa] = (float(K.sum()), dT.cpu().numpy(), info.n_sweeps)
    (k0, t0, s0), (k1, t1, s1) = res[-1], res[1]
    assert abs(k1 - k0) <= 1e-8 * abs(k0), (k0, k1)
    assert np.max(np.abs(t1 - t0)) <= 1e-7 * np.max(np.abs(t0))


def test_dsa_with_isothermal_walls_matches_oracle():
    """Forced on with isothermal walls (the diffusion operator holds the correction at zero there and has no
    null vector, so no projection): kappa and the temperature field of the oracle to 1e-9."""
    import bte_oracle
    from openbte_gb300 import BTE_RTA, objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cell_2d(500, 0.2, "circle", seed=9))
    mat = synthetic_isotropic_2d(6, 12)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0},
                               mixed={"Boundary": {"value": 0.3, "boundary_conductance": 1e3}})
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    k_ref, dT_ref, *_ = bte_oracle.bte_rta(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-13,
                                           bte_max_iter=3000)
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-11, precision="fp64", dsa=1)
    assert abs(r.aux["kappa_eff"] - k_ref) <= 1e-9 * abs(k_ref), (r.aux["kappa_eff"], k_ref)
    dT = r.variables["Temperature_BTE"]["data"]
    assert np.abs(dT - dT_ref).max() <= 1e-8 * np.abs(dT_ref).max()


def test_dsa_on_the_3d_cube_keeps_the_fixed_point(case):
    """Forced on in 3D (tetrahedra, spherical pore): the reference's kappa (golden cube1k5) to 1e-6."""
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case("cube1k5")
    r = BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=1e-10, precision="fp64", dsa=1)
    assert abs(r.kappa_eff - d["bte_kappa"]) <= 1e-6 * abs(d["bte_kappa"]), (r.kappa_eff, d["bte_kappa"])
