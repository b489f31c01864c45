"""Continuous batching on the GPU: every result is the same alone and in the mix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.serving import Request
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    specs = [(400, 0.10, "circle", 8, 16), (700, 0.25, "square", 10, 24), (900, 0.35, "circle", 12, 16),
             (500, 0.20, "square", 6, 32), (1200, 0.30, "square", 8, 24), (600, 0.15, "circle", 16, 16)]
    reqs = []
    for i, (n, phi, pore, nm, nq) in enumerate(specs):
        geo = mesh_from_cell(porous_cell_2d(n, phi, pore, seed=100 + i))
        reqs.append(Request(geo, synthetic_isotropic_2d(nm, nq), bcs, ek, precision="fp32_refine", rtol=1e-8,
                            rid=i))
    return reqs


def test_same_alone_and_in_the_mix():
    from openbte_gb300.serving import GPUBackend, Server, replay
    reqs = _requests()
    alone = {}
    srv = Server(backend=GPUBackend(), slots=1, builders=1)
    for r in reqs:
        res = replay(srv, [r])[0]
        assert res.status == "ok", res.error
        alone[r.rid] = res.kappa
    srv.close()
    srv = Server(backend=GPUBackend(), slots=4, builders=3)
    mixed = replay(srv, reqs)
    srv.close()
    assert srv.max_concurrent >= 2
    for res in mixed:
        assert res.status == "ok", res.error
        rel = abs(res.kappa - alone[res.rid]) / abs(alone[res.rid])
        assert rel < 1e-6, (res.rid, res.kappa, alone[res.rid])


def test_same_alone_and_in_the_mix_bit_for_bit(monkeypatch):
    """With deterministic reductions (OBTE_DETERMINISTIC=1) a served result does not depend on what else ran
    on the GPU at the same time: alone and in the mix give the same kappa, bit for bit."""
    from openbte_gb300.serving import GPUBackend, Server, replay
    monkeypatch.setenv("OBTE_DETERMINISTIC", "1")
    reqs = _requests()
    alone = {}
    srv = Server(backend=GPUBackend(), slots=1, builders=1)
    for r in reqs:
        res = replay(srv, [r])[0]
        assert res.status == "ok", res.error
        alone[r.rid] = res.kappa
    srv.close()
    srv = Server(backend=GPUBackend(), slots=4, builders=3)
    mixed = replay(srv, reqs)
    srv.close()
    assert srv.max_concurrent >= 2
    for res in mixed:
        assert res.status == "ok", res.error
        assert res.kappa == alone[res.rid], (res.rid, res.kappa, alone[res.rid])


def test_served_kappa_matches_oracle():
    import bte_oracle
    from openbte_gb300.serving import GPUBackend, Server, replay
    r = _requests()[1]
    k_ref = bte_oracle.bte_rta(r.geo, r.mat, r.bcs, effective_thermal_conductivity=r.ek, bte_rtol=1e-12,
                               bte_max_iter=3000)[0]
    srv = Server(backend=GPUBackend(), slots=2)
    res = replay(srv, [r])[0]
    srv.close()
    assert abs(res.kappa - k_ref) / abs(k_ref) < 1e-4       # the served form's stated tolerance


def test_repeated_geometry_stays_resident_and_warm_starts():
    from openbte_gb300.serving import GPUBackend, Server, replay
    r = _requests()[0]
    be = GPUBackend()
    srv = Server(backend=be, slots=1)
    first = replay(srv, [r])[0]
    r.warm_start = True
    again = replay(srv, [r])[0]
    srv.close()
    assert again.cached_plan and not first.cached_plan
    assert again.n_sweeps < first.n_sweeps
    assert abs(again.kappa - first.kappa) / abs(first.kappa) < 1e-6


def test_repeated_geometry_builds_the_preconditioner():
    """Three cold requests of one geometry, two slots: they solve one at a time on the shared plan; the
    second builds the periodic-inflow preconditioner inside its admission reservation, and the plan's
    resident bytes then include the preconditioner's blocks."""
    import ctypes as C
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    from openbte_gb300.serving import GPUBackend, Request, Server, replay
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    geo = mesh_from_cell(porous_cell_2d(1500, 0.25, "square", seed=7))
    mat = synthetic_isotropic_2d(16, 32)
    reqs = [Request(geo, mat, bcs, ek, precision="fp32_refine", rtol=1e-9, rid=i) for i in range(3)]
    be = GPUBackend()
    srv = Server(backend=be, slots=2)
    first = replay(srv, reqs[:1])[0]
    later = replay(srv, reqs[1:])
    srv.close()
    assert first.status == "ok" and all(r.status == "ok" for r in later), [r.error for r in later]
    assert all(r.cached_plan for r in later)
    (pl,) = list(be._cache.values())
    nb, ns, ms = C.c_int32(), C.c_int32(), C.c_double()
    assert pl.lib.obte_bte_precond_info(pl.handle, C.byref(nb), C.byref(ns), C.byref(ms)) == 0
    assert nb.value > 0
    resident, bound = pl.precond_bytes()
    assert resident > 0 and bound == 0 and pl.pending == 0
    a, b = pl.footprint("fp32_refine", be.restart)
    assert be.resident_bytes() == a + b >= resident
    for r in later:
        assert abs(r.kappa - first.kappa) <= 1e-7 * abs(first.kappa), (r.kappa, first.kappa)
    assert min(r.n_sweeps for r in later) < first.n_sweeps


def test_request_over_budget_is_rejected():
    from openbte_gb300.serving import GPUBackend, Server, replay
    r = _requests()[0]
    srv = Server(backend=GPUBackend(), slots=1, hbm_budget=1 << 20)
    res = replay(srv, [r])[0]
    srv.close()
    assert res.status == "rejected"


def test_concurrent_sweeps_with_different_footprints():
    """Two plans whose sweep kernels need different shared memory, swept from two threads on their own
    streams at the same time: every call succeeds and matches the same sweep run alone."""
    import ctypes as C
    import threading
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    from openbte_gb300 import objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    cases = [(400, 0.10, "circle", 8, 16), (3000, 0.30, "square", 24, 48)]
    plans, states, refs = [], [], []
    for i, (n, phi, pore, nm, nq) in enumerate(cases):
        stream = torch.cuda.Stream()
        geo = mesh_from_cell(porous_cell_2d(n, phi, pore, seed=200 + i))
        plan = Plan(HostProblem(geo, synthetic_isotropic_2d(nm, nq), bcs, ek), stream=stream.cuda_stream)
        u = torch.tensor(np.random.default_rng(i).standard_normal(plan.nu), dtype=torch.float64, device="cuda")
        out = torch.zeros_like(u)
        _lib.check(plan.lib.obte_bte_sweep(plan.handle, 2, C.c_void_p(u.data_ptr()), C.c_void_p(out.data_ptr()), 1))
        plans.append(plan); states.append(u); refs.append(out.cpu().numpy())
    errors = []

    def run(i):
        out = torch.zeros_like(states[i])
        for _ in range(40):
            st = plans[i].lib.obte_bte_sweep(plans[i].handle, 2, C.c_void_p(states[i].data_ptr()),
                                             C.c_void_p(out.data_ptr()), 1)
            if st != 0:
                errors.append(plans[i].lib.obte_last_error())
                return
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        if not np.allclose(got, refs[i], rtol=0, atol=1e-5 * np.abs(refs[i]).max()):
            errors.append(b"mismatch")

    threads = [threading.Thread(target=run, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors


def test_destroyed_plan_memory_is_recycled():
    """A destroyed plan's device buffers go to the library's cache (no cudaFree, which would synchronise
    the device under concurrent solves) and serve the next plan; trimming frees them."""
    import ctypes as C
    import gc
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.bte import solve_plan
    from openbte_gb300.runtime import HostProblem, Plan
    lib = _lib.load()
    reqs = _requests()
    cached = C.c_int64()
    plan = Plan(HostProblem(reqs[1].geo, reqs[1].mat, reqs[1].bcs, reqs[1].ek))
    dT0 = torch.zeros(plan.n, dtype=torch.float64, device="cuda")
    k0 = solve_plan(plan, dT0, precision="fp32_refine", rtol=1e-8)[0].kappa_eff
    del plan
    gc.collect()
    _lib.check(lib.obte_device_cache_bytes(C.byref(cached)), "cache bytes")
    assert cached.value > 0
    # the same problem again, on recycled memory: same kappa
    plan = Plan(HostProblem(reqs[1].geo, reqs[1].mat, reqs[1].bcs, reqs[1].ek))
    k1 = solve_plan(plan, dT0, precision="fp32_refine", rtol=1e-8)[0].kappa_eff
    assert abs(k1 - k0) <= 1e-9 * abs(k0)
    del plan
    gc.collect()
    freed = C.c_int64()
    _lib.check(lib.obte_device_cache_trim(C.byref(freed)), "trim")
    _lib.check(lib.obte_device_cache_bytes(C.byref(cached)), "cache bytes")
    assert freed.value > 0 and cached.value == 0
