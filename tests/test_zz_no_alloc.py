"""The sweep on library-owned static scratch (obte_bte_sweep_static) against the allocating sweep.

Some callers cannot allocate device memory at the moment they sweep: a host framework that has
reserved nearly all of the GPU's memory for its own pool, or a latency-bound loop in which
cudaMalloc / cudaFree would synchronise the device.  obte_bte_sweep_static serves them: it runs the
same kernels as obte_bte_sweep with its scratch in an 8 MiB array held inside the library, and
allocates nothing.  These tests call both through the C ABI and compare them on two calls in a row,
at the tolerances of the other sweep tests (1e-11 in FP64, 2e-5 in FP32, relative to the largest
entry of the exact result).  The file name makes pytest collect it last, so it also runs after the
other tests have used the device; it passes on its own in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 2e-5}


def _call(fn, plan, precision, u, with_source):
    import torch
    from openbte_gb300 import _lib
    out = torch.full_like(u, float("nan"))
    rc = fn(plan.handle, _lib.PRECISION[precision], C.c_void_p(u.data_ptr()), C.c_void_p(out.data_ptr()),
            with_source)
    return rc, out.cpu().numpy()


def _state(plan, seed):
    import torch
    rng = np.random.default_rng(seed)
    return torch.tensor(0.3 * rng.standard_normal(plan.nu), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("name", ["a600", "cube1k5"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_scratch_sweep_matches_allocating_sweep(case, name, precision):
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    lib = plan.lib
    # two calls in a row with different states (and source flags): the second must not see the first's scratch
    for seed, with_source in ((1, 1), (2, 0)):
        u = _state(plan, seed)
        rc, ref = _call(lib.obte_bte_sweep, plan, precision, u, with_source)   # builds the tables on first use
        _lib.check(rc, "obte_bte_sweep")
        rc, got = _call(lib.obte_bte_sweep_static, plan, precision, u, with_source)
        _lib.check(rc, "obte_bte_sweep_static")
        assert np.isfinite(got).all()
        np.testing.assert_allclose(got, ref, rtol=0, atol=TOL[precision] * max(np.abs(ref).max(), 1.0))


def test_static_scratch_sweep_needs_tables_built_at_setup(case):
    """Before any allocating sweep in that precision the call is refused, not served by allocating."""
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case("a600")
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    rc, _ = _call(plan.lib.obte_bte_sweep_static, plan, "fp64", _state(plan, 3), 1)
    assert rc == 1
    assert b"set-up" in plan.lib.obte_last_error()


def test_static_scratch_sweep_rejects_problems_beyond_its_array():
    """96 directions x ~14k triangles x 8 bytes exceeds the 8 MiB array: rejected with a clear error."""
    from openbte_gb300 import _lib
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.runtime import HostProblem, Plan
    geo = mesh_from_cell(porous_cell_2d(14000, 0.25, "circle", seed=5))
    mat = synthetic_isotropic_2d(8, 96)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    assert geo.n_elems * 96 * 8 > 8 << 20
    for precision in ("fp32", "fp64"):
        rc, _ = _call(plan.lib.obte_bte_sweep_static, plan, precision, _state(plan, 4), 1)
        assert rc == 7
        msg = plan.lib.obte_last_error()
        assert b"bytes of static scratch" in msg and b"obte_bte_sweep" in msg
