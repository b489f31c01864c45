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


def test_request_over_budget_is_rejected():
    from openbte_gb300.serving import GPUBackend, Server, replay
    r = _requests()[0]
    srv = Server(backend=GPUBackend(), slots=1, hbm_budget=1 << 20)
    res = replay(srv, [r])[0]
    srv.close()
    assert res.status == "rejected"
