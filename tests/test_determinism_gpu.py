"""Deterministic reductions (OBTE_DETERMINISTIC=1): bit-identical results run to run.

By default the sweep adds its partial sums into the lattice temperature, wall temperatures, flux and
per-ordinate kappa with FP64 atomics, whose order (which CTA finishes first) varies between runs, so results
agree only to rounding.  With OBTE_DETERMINISTIC=1 every (direction, MFP chunk) CTA stores its partials and
fixed-order reduction kernels add them: repeated sweeps and solves give the same bits, and they agree with
the atomic results to rounding.  The periodic-inflow preconditioner's set-up (probe sweeps on a subset of
the CTAs) still adds with atomics, so bit-identical solves need it off (precond=-1) or built once per plan.
"""
import ctypes as C

import numpy as np
import pytest

from openbte_gb300 import objects as O

pytestmark = pytest.mark.gpu


def _sweep(plan, prec, u, src=1):
    import torch
    from openbte_gb300 import _lib
    out = torch.zeros_like(u)
    _lib.check(plan.lib.obte_bte_sweep(plan.handle, _lib.PRECISION[prec], C.c_void_p(u.data_ptr()),
                                       C.c_void_p(out.data_ptr()), src), prec)
    return out.cpu().numpy()


@pytest.mark.parametrize("name", ["a600", "cube1k5", "gray600"])
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_deterministic_sweeps_repeat_bit_for_bit(case, monkeypatch, name, prec):
    import torch
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    u = torch.tensor(np.random.default_rng(3).standard_normal(plan.nu), dtype=torch.float64, device="cuda")
    monkeypatch.delenv("OBTE_DETERMINISTIC", raising=False)
    atomic = _sweep(plan, prec, u)
    monkeypatch.setenv("OBTE_DETERMINISTIC", "1")
    first = _sweep(plan, prec, u)
    for _ in range(3):
        np.testing.assert_array_equal(_sweep(plan, prec, u), first)
    np.testing.assert_allclose(first, atomic, rtol=0, atol=1e-12 * np.abs(atomic).max())


@pytest.mark.parametrize("prec,rtol", [("fp64", 1e-10), ("fp32_refine", 1e-8)])
def test_deterministic_solves_repeat_bit_for_bit(case, monkeypatch, prec, rtol):
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case("c0_2k")
    monkeypatch.setenv("OBTE_DETERMINISTIC", "1")
    # the periodic-inflow preconditioner stays off: the default policy builds it on the plan's second solve
    # (the two runs would then iterate differently), and its probe sweeps add with atomics
    runs = [BTE_RTA(geo, mat, bcs, effective_thermal_conductivity=ek, bte_rtol=rtol, precision=prec, precond=-1)
            for _ in range(2)]
    assert runs[0].kappa_eff == runs[1].kappa_eff
    for key in ("Temperature_BTE", "Flux_BTE"):
        np.testing.assert_array_equal(runs[0].variables[key]["data"], runs[1].variables[key]["data"])
    np.testing.assert_array_equal(runs[0].aux["suppression"], runs[1].aux["suppression"])
    assert abs(runs[0].kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"]) < 1e-6
