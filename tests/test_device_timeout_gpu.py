"""The sweep kernel's bounded waits give up with a status instead of hanging (failure detection).

Every wait of the sweep kernel for a level unit's bulk copy has a poll cap; on reaching it the CTA
raises the device error word, lets the copies it still has in flight land and leaves, and the call
returns OBTE_ERR_DEVICE_TIMEOUT.  The reference has no such detection: its workers meet at
multiprocessing barriers without a timeout (openbte/objects.py:88-101).

The test makes a wait run out safely: through obte_bte_plan_test_wait_timeout the plan's sweeps skip
issuing one unit's copy (a flag that nothing sets) and use a short poll cap.  Nothing faults or hangs;
the same plan then sweeps and solves normally.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["a600", "cube1k5"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_wait_that_runs_out_returns_timeout_and_plan_recovers(case, name, precision):
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.bte import solve_plan
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    lib = plan.lib
    code = _lib.PRECISION[precision]
    rng = np.random.default_rng(5)
    u = torch.tensor(0.3 * rng.standard_normal(plan.nu), dtype=torch.float64, device="cuda")

    def sweep():
        out = torch.zeros_like(u)
        rc = lib.obte_bte_sweep(plan.handle, code, C.c_void_p(u.data_ptr()), C.c_void_p(out.data_ptr()), 1)
        return rc, out.cpu().numpy()

    rc, ref = sweep()
    _lib.check(rc, "sweep")
    # unit 2 of every direction never arrives; each wait gives up after 4096 polls
    _lib.check(lib.obte_bte_plan_test_wait_timeout(plan.handle, 2, 4096), "test hook")
    rc, _ = sweep()
    assert rc == _lib.OBTE_ERR_DEVICE_TIMEOUT, (rc, lib.obte_last_error())
    assert "timed out" in lib.obte_last_error().decode()
    # the error word was cleared on read and the context is usable: a normal sweep and a solve follow
    _lib.check(lib.obte_bte_plan_test_wait_timeout(plan.handle, -1, 0), "test hook")
    rc, again = sweep()
    _lib.check(rc, "sweep after the timeout")
    np.testing.assert_allclose(again, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    dT0 = torch.zeros(plan.n, dtype=torch.float64, device="cuda")
    info, *_ = solve_plan(plan, dT0, precision="fp64" if precision == "fp64" else "fp32_refine", rtol=1e-8)
    assert info.converged


def test_wait_hook_rejects_bad_arguments(case):
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case("a600")
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    assert plan.lib.obte_bte_plan_test_wait_timeout(plan.handle, -2, 0) == _lib.OBTE_ERR_BAD_ARG
    assert plan.lib.obte_bte_plan_test_wait_timeout(plan.handle, 0, -1) == _lib.OBTE_ERR_BAD_ARG
