"""Sweep orders and level sets built by the library (C++) vs an independent host recomputation, bit for bit."""
import numpy as np
import pytest

import sweep_order
from openbte_gb300.runtime import HostProblem, Plan


@pytest.mark.parametrize("name", ["a600", "c0_2k", "circ1k", "cube1k5"])
def test_schedule_bit_exact(case, name):
    geo, mat, bcs, ek, _ = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek), host_only=True)
    faces = sweep_order.directed_faces(geo)
    for q in range(mat.vmfp.shape[0]):
        order, lp, nslots = plan.schedule(q)
        o2, lp2 = sweep_order.schedule(geo, mat.vmfp[q], faces)
        np.testing.assert_array_equal(order, o2)
        np.testing.assert_array_equal(lp, lp2)
        assert nslots <= geo.n_elems


def test_front_fits_shared_memory(case):
    """The live front per direction stays far below the element count (2D: ~sqrt(n))."""
    geo, mat, bcs, ek, _ = case("c0_2k")
    plan = Plan(HostProblem(geo, mat, bcs, ek), host_only=True)
    slots = [plan.schedule(q)[2] for q in range(mat.vmfp.shape[0])]
    assert max(slots) < 0.2 * geo.n_elems
    assert max(slots) * 32 * 8 < 227 * 1024


def test_cycle_is_reported(case):
    """A mesh whose upwind graph has a cycle is rejected with OBTE_ERR_CYCLE (no hang, no wrong answer)."""
    from openbte_gb300 import _lib
    geo, mat, bcs, ek, _ = case("a600")
    # drop the periodic cut: treat periodic sides as ordinary couplings -> cycles through the wrap
    bcs2 = bcs._replace(periodic={})
    hp = HostProblem(geo, mat, bcs2, None)
    with pytest.raises(_lib.OBTEError) as ei:
        Plan(hp, host_only=True)
    assert ei.value.status == 6
