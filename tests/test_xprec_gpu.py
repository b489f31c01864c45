"""Periodic-inflow preconditioner: same fixed point, fewer sweeps, and the build policy."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(n_tri=1500, n_mfp=16, n_dir=32, phi=0.25, pore="square", seed=7):
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cell_2d(n_tri, phi, pore, seed=seed))
    mat = synthetic_isotropic_2d(n_mfp, n_dir)          # MFPs 1 nm - 10 um: axis rays beside the pore circulate
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    return geo, mat, bcs, ek


def _plan(geo, mat, bcs, ek):
    from openbte_gb300.runtime import HostProblem, Plan
    return Plan(HostProblem(geo, mat, bcs, ek), 0)


def _info(plan):
    nb, ns, ms = C.c_int32(), C.c_int32(), C.c_double()
    assert plan.lib.obte_bte_precond_info(plan.handle, C.byref(nb), C.byref(ns), C.byref(ms)) == 0
    return nb.value, ns.value, ms.value


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_same_solution_fewer_sweeps(precision):
    import torch
    from openbte_gb300.bte import solve_plan
    geo, mat, bcs, ek = _problem()
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device="cuda:0")
    off = _plan(geo, mat, bcs, ek)
    i0, dT_off, J_off, K_off, _ = solve_plan(off, dT0, precision=precision, rtol=1e-10, max_sweeps=3000,
                                             restart=60, precond=-1)
    on = _plan(geo, mat, bcs, ek)
    i1, dT_on, J_on, K_on, _ = solve_plan(on, dT0, precision=precision, rtol=1e-10, max_sweeps=3000,
                                          restart=60, precond=1)
    assert i0.converged and i1.converged
    nblk, setup, _ = _info(on)
    assert nblk > 0 and setup > 0
    assert _info(off)[0] == 0
    # the same fixed point to the solve tolerance
    k0, k1 = float(K_off.sum()), float(K_on.sum())
    assert abs(k1 - k0) <= 1e-7 * abs(k0), (k0, k1)
    assert torch.allclose(dT_on, dT_off, rtol=0, atol=1e-7 * float(dT_off.abs().max()))
    assert i1.n_sweeps < i0.n_sweeps, (i0.n_sweeps, i1.n_sweeps)


def test_default_builds_on_second_solve():
    import torch
    from openbte_gb300.bte import solve_plan
    geo, mat, bcs, ek = _problem(n_tri=800, n_mfp=12, n_dir=24)
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device="cuda:0")
    plan = _plan(geo, mat, bcs, ek)
    a, *_ , Ka, _ = solve_plan(plan, dT0, precision="fp64", rtol=1e-10, max_sweeps=3000, restart=60)
    assert _info(plan)[0] == 0                          # one solve: no setup paid
    b, *_, Kb, _ = solve_plan(plan, dT0, precision="fp64", rtol=1e-10, max_sweeps=3000, restart=60)
    assert _info(plan)[0] > 0
    assert b.n_sweeps < a.n_sweeps
    assert abs(float(Kb.sum()) - float(Ka.sum())) <= 1e-7 * abs(float(Ka.sum()))
    # off on a plan that has one: the plain iteration again
    c, *_, Kc, _ = solve_plan(plan, dT0, precision="fp64", rtol=1e-10, max_sweeps=3000, restart=60, precond=-1)
    assert abs(c.n_sweeps - a.n_sweeps) <= 2
    assert abs(float(Kc.sum()) - float(Ka.sum())) <= 1e-9 * abs(float(Ka.sum()))


def test_blocks_are_the_slow_axis_ordinates():
    """The covered ordinates are long-MFP ones along the cell axes (rays beside the pore)."""
    import torch
    from openbte_gb300.bte import solve_plan
    geo, mat, bcs, ek = _problem()
    plan = _plan(geo, mat, bcs, ek)
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device="cuda:0")
    solve_plan(plan, dT0, precision="fp64", rtol=1e-8, max_sweeps=3000, restart=60, precond=1)
    nblk, _, _ = _info(plan)
    n_mfp, n_dir = np.asarray(mat.t_coeff).shape
    assert 0 < nblk < n_mfp * n_dir // 4


@pytest.mark.parametrize("precision,inner", [("fp32", 1e-5), ("fp32_refine", 1e-8)])
def test_fp32_stage_stops_at_its_floor(precision, inner):
    """A tolerance below the FP32 sweeps' rounding floor ends the FP32 stage instead of spinning."""
    import torch
    from openbte_gb300.bte import solve_plan
    geo, mat, bcs, ek = _problem()
    plan = _plan(geo, mat, bcs, ek)
    dT0 = torch.zeros(geo.n_elems, dtype=torch.float64, device="cuda:0")
    info, *_ = solve_plan(plan, dT0, precision=precision, rtol=1e-9, max_sweeps=3000, restart=40,
                          inner_rtol=inner, precond=1)
    assert info.n_sweeps < 400, info.n_sweeps
    if precision == "fp32_refine":
        assert info.converged and info.residual <= 1e-9
    else:
        assert info.residual < 1e-5
