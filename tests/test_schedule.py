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


@pytest.mark.parametrize("name", ["a600", "c0_2k", "cube1k5"])
def test_operator_coefficients_match_oracle(case, name):
    """Per direction, in sweep order: the outflow diagonal D, the periodic jump source P and the row sums of
    the inflow coefficients (upwind faces, cut periodic faces and diffuse walls) equal the oracle's
    restatement of openbte/bte.py:47-110 (D, P, Gm, Gbm2) to rounding."""
    import ctypes as C
    import bte_oracle
    geo, mat, bcs, ek, _ = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek), host_only=True)
    ops = bte_oracle.setup_operators(geo, mat, bcs)
    n, nf = geo.n_elems, len(geo.elems[0])
    inflow = np.zeros((ops["n_angles"], n))
    np.add.at(inflow.T, ops["i_mat"], ops["Gm"].T)
    if ops["Gbm2"] is not None:
        np.add.at(inflow.T, ops["i_diffuse"], ops["Gbm2"].T)
    for q in range(ops["n_angles"]):
        order = plan.schedule(q)[0]
        cf, D, P = np.zeros(n * nf), np.zeros(n), np.zeros(n)
        _lib_check = plan.lib.obte_bte_schedule_coefficients(plan.handle, q, *[a.ctypes.data_as(C.c_void_p)
                                                                             for a in (cf, D, P)])
        assert _lib_check == 0
        scale = np.abs(ops["D"][q]).max()
        np.testing.assert_allclose(D, ops["D"][q][order], rtol=0, atol=1e-13 * scale)
        np.testing.assert_allclose(P, ops["perturbation"][q][order], rtol=0,
                                   atol=1e-13 * max(np.abs(ops["perturbation"]).max(), 1e-300))
        np.testing.assert_allclose(cf.reshape(n, nf).sum(axis=1), inflow[q][order], rtol=0, atol=1e-13 * scale)


@pytest.mark.parametrize("name", ["c0_2k", "cube1k5"])
def test_tables_do_not_depend_on_host_threads(case, name, monkeypatch):
    """The schedule and the packed sweep tables (FP32 and FP64) are the same for 1, 3 and 8 host threads."""
    import ctypes as C
    from openbte_gb300 import _lib
    geo, mat, bcs, ek, _ = case(name)
    digests = set()
    for threads in ("1", "3", "8"):
        monkeypatch.setenv("OBTE_HOST_THREADS", threads)
        plan = Plan(HostProblem(geo, mat, bcs, ek), host_only=True)
        d = []
        for prec in ("fp32", "fp64"):
            v = C.c_uint64()
            _lib.check(plan.lib.obte_bte_tables_digest(plan.handle, _lib.PRECISION[prec], C.byref(v)), "digest")
            d.append(v.value)
        d.append(tuple(int(x) for q in range(mat.vmfp.shape[0]) for x in plan.schedule(q)[0][:50]))
        digests.add(tuple(d))
    assert len(digests) == 1
