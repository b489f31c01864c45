"""GPU parity of the inverse-design path: kappa_eff(rho) and dkappa/drho on a periodic pixel grid.

Gray cases against the reference's own inverse model (golden vectors from openbte/inverse/bte.py);
MFP-resolved cases against the CPU oracle's explicit adjoint and against central finite differences
of the GPU solver itself.
"""
import os

import numpy as np
import pytest

import tim_oracle as T

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "inverse_gray.npz")


@pytest.mark.parametrize("name", ["g8_kn1", "g8_kn01", "g10_kn05"])
# kappa comes from FP64 reductions; the gradient from the final sweep's per-ordinate field stored in
# FP32, so its bar is 1e-6 (FP64 mode) / 1e-4 (FP32+refine) of the largest entry
@pytest.mark.parametrize("precision,ktol,gtol", [("fp64", 1e-8, 1e-6), ("fp32_refine", 1e-5, 1e-4)])
def test_gray_matches_reference(name, precision, ktol, gtol):
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    d = np.load(GOLD)
    n, kn, n_phi, _ = d[name + "_meta"]
    solver = PixelSolver(int(n), IsotropicMaterial.gray(kn, int(n_phi)), precision=precision,
                         rtol=1e-12 if precision == "fp64" else 1e-9)
    k, g = solver.kappa_and_gradient(d[name + "_rho"])
    kr, gr = d[name + "_kappa"][0], d[name + "_grad"]
    assert abs(k - kr) <= ktol * abs(kr), (k, kr)
    np.testing.assert_allclose(g.cpu().numpy(), gr, rtol=0, atol=gtol * np.abs(gr).max())


def test_mfp_resolved_matches_oracle_adjoint():
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    mfps, kappas = [0.05, 0.4, 2.0], [0.5, 0.3, 0.2]
    rng = np.random.default_rng(7)
    rho = rng.uniform(0.05, 1.0, 64)
    grid = T.pixel_grid(8)
    mat = T.material(mfps, kappas, 16)
    k_ref, g_ref, _ = T.kappa_and_gradient(rho, grid, mat, method="adjoint")
    solver = PixelSolver(8, IsotropicMaterial(mfps, kappas, 16), precision="fp64", rtol=1e-12)
    k, g = solver.kappa_and_gradient(rho)
    assert abs(k - k_ref) <= 1e-8 * abs(k_ref)
    np.testing.assert_allclose(g.cpu().numpy(), g_ref, rtol=0, atol=1e-6 * np.abs(g_ref).max())


def test_gradient_against_central_differences():
    """Adjoint dkappa/drho within 1e-4 of central differences of the GPU solver (lognormal 12 x 16, 24^2)."""
    import torch
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    n = 24
    rng = np.random.default_rng(11)
    rho = rng.uniform(0.1, 1.0, n * n)
    mat = IsotropicMaterial.lognormal(12, 16)
    solver = PixelSolver(n, mat, size=100.0, precision="fp64", rtol=1e-12)
    k, g = solver.kappa_and_gradient(rho)
    g = g.cpu().numpy()
    h = 1e-3
    for p in rng.choice(n * n, 6, replace=False):
        r1, r2 = rho.copy(), rho.copy()
        r1[p] += h
        r2[p] -= h
        fd = (solver.kappa_and_gradient(r1)[0] - solver.kappa_and_gradient(r2)[0]) / (2 * h)
        assert abs(g[p] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(g).max()), (p, g[p], fd)


def test_autograd_function_and_reference_factory():
    import torch
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver, get_solver, kappa_eff
    d = np.load(GOLD)
    name = "g8_kn1"
    n, kn, n_phi, _ = d[name + "_meta"]
    rho = torch.tensor(d[name + "_rho"], dtype=torch.float64, device="cuda", requires_grad=True)
    solver = PixelSolver(int(n), IsotropicMaterial.gray(kn, int(n_phi)), precision="fp64", rtol=1e-12)
    k = kappa_eff(rho, solver)
    (2.0 * k).backward()
    np.testing.assert_allclose(rho.grad.cpu().numpy(), 2.0 * d[name + "_grad"], rtol=0,
                               atol=2e-6 * np.abs(d[name + "_grad"]).max())
    func = get_solver(grid=int(n), Kn=kn, n_phi=int(n_phi), directions=[[1, 0]], precision="fp64", rtol=1e-12)
    (kap, _), jac = func(d[name + "_rho"])
    assert abs(kap[0] - d[name + "_kappa"][0]) <= 1e-8 * abs(kap[0])
    np.testing.assert_allclose(jac[0], d[name + "_grad"], rtol=0, atol=1e-6 * np.abs(d[name + "_grad"]).max())


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_updated_plan_matches_new_plan(precision):
    """A plan whose transmissions were replaced (obte_bte_plan_set_transmission) sweeps exactly like a plan
    built for the new density field (same coefficients in the FP32 and FP64 tables), and gives its kappa and
    gradient."""
    import ctypes as C
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    lib = _lib.load()
    n = 16
    rng = np.random.default_rng(5)
    mat = IsotropicMaterial.lognormal(8, 16)
    rtol = 1e-11 if precision == "fp64" else 1e-8
    # FP64 solves repeat to rounding; FP32+refine solves differ run to run up to the solve tolerance (the
    # order of the FP32 sweep's atomic accumulations moves where GMRES stops)
    ktol, gtol = (1e-12, 1e-12) if precision == "fp64" else (2e-8, 1e-5)
    reused = PixelSolver(n, mat, size=50.0, precision=precision, rtol=rtol)
    for step in range(3):
        rho = rng.uniform(0.05, 1.0, n * n)
        fresh = PixelSolver(n, mat, size=50.0, precision=precision, rtol=rtol)
        k1, g1 = reused.kappa_and_gradient(rho)
        k2, g2 = fresh.kappa_and_gradient(rho)
        if step:
            assert reused.last_upload_bytes > 0      # the coefficients of the tables it holds
        # one sweep of each table precision through both plans, on the same state
        ne, nd, nx = C.c_int64(), C.c_int64(), C.c_int64()
        _lib.check(lib.obte_bte_state_layout(fresh._h, C.byref(ne), C.byref(nd), C.byref(nx)), "layout")
        nu = ne.value + nd.value + nx.value
        u = torch.as_tensor(rng.standard_normal(nu), device="cuda")
        torch.cuda.synchronize()
        for prec in ("fp64", "fp32"):
            outs = []
            for h in (reused._h, fresh._h):
                o = torch.empty_like(u)
                _lib.check(lib.obte_bte_sweep(h, _lib.PRECISION[prec], C.c_void_p(u.data_ptr()),
                                              C.c_void_p(o.data_ptr()), 1), "sweep")
                outs.append(o.cpu().numpy())
            tol = 1e-13 if prec == "fp64" else 1e-6
            np.testing.assert_allclose(outs[0], outs[1], rtol=0, atol=tol * np.abs(outs[1]).max())
        fresh.close()
        assert abs(k1 - k2) <= ktol * abs(k2), (step, k1, k2)
        g1, g2 = g1.cpu().numpy(), g2.cpu().numpy()
        np.testing.assert_allclose(g1, g2, rtol=0, atol=gtol * np.abs(g2).max())
    reused.close()


def test_direction_set_not_closed_under_reversal_matches_oracle_adjoint():
    """An odd number of directions (phi_q = 2 pi q / 15: no -s_q in the set): the adjoint comes from a second
    plan with the reversed directions, whose forward solve is the transposed, reverse-order sweep of every
    ordinate.  kappa and dkappa/drho against the oracle's explicit adjoint (A^T lam = dkappa/dX)."""
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    mfps, kappas = [0.05, 0.4, 2.0], [0.5, 0.3, 0.2]
    rng = np.random.default_rng(11)
    rho = rng.uniform(0.05, 1.0, 64)
    grid = T.pixel_grid(8)
    mat = T.material(mfps, kappas, 15)
    k_ref, g_ref, _ = T.kappa_and_gradient(rho, grid, mat, method="adjoint")
    solver = PixelSolver(8, IsotropicMaterial(mfps, kappas, 15), precision="fp64", rtol=1e-12)
    assert solver.paired
    k, g = solver.kappa_and_gradient(rho)
    assert solver.last_adjoint_info is not None and solver.last_adjoint_info.converged
    assert abs(k - k_ref) <= 1e-8 * abs(k_ref), (k, k_ref)
    np.testing.assert_allclose(g.cpu().numpy(), g_ref, rtol=0, atol=1e-6 * np.abs(g_ref).max())
    # a second density field on the same pair of plans (both get the new transmissions)
    rho2 = np.clip(rho + 0.1 * rng.standard_normal(64), 0.05, 1.0)
    k2_ref, g2_ref, _ = T.kappa_and_gradient(rho2, grid, mat, method="adjoint")
    k2, g2 = solver.kappa_and_gradient(rho2)
    assert abs(k2 - k2_ref) <= 1e-8 * abs(k2_ref)
    np.testing.assert_allclose(g2.cpu().numpy(), g2_ref, rtol=0, atol=1e-6 * np.abs(g2_ref).max())


def test_unpaired_gradient_of_an_open_direction_set_is_refused():
    """Without the reversed plan the single-solve identity does not apply: OBTE_ERR_UNSUPPORTED."""
    from openbte_gb300 import _lib
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    solver = PixelSolver(8, IsotropicMaterial([0.4], [1.0], 15), precision="fp64", rtol=1e-10)
    solver.paired = False
    with pytest.raises(_lib.OBTEError, match="closed under reversal"):
        solver.kappa_and_gradient(np.full(64, 0.7))


def test_gradient_fields_through_the_correction_pass():
    """FP32+refine gradient solves update the stored per-ordinate temperatures through the FP32 pass at the
    refinement's correction d (X(u + d) = X(u) + X_0(d)) instead of a second FP64 pass: one FP64 sweep, and
    the same gradient as the FP64 solve."""
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.3, 1.0, 16 * 16)
    mat = IsotropicMaterial([0.3, 2.0], [0.6, 0.4], 16)
    s64 = PixelSolver(16, mat, precision="fp64", rtol=1e-12)
    k64, g64 = s64.kappa_and_gradient(rho)
    s32 = PixelSolver(16, mat, precision="fp32_refine", rtol=1e-10)
    k32, g32 = s32.kappa_and_gradient(rho)
    assert s32.last_info.n_sweeps_fp64 == 1, (s32.last_info.n_sweeps_fp64, s32.last_info.n_sweeps)
    assert s32.last_info.residual <= 1e-10
    assert abs(k32 - k64) <= 1e-9 * abs(k64), (k32, k64)
    g32, g64 = g32.cpu().numpy(), g64.cpu().numpy()
    np.testing.assert_allclose(g32, g64, rtol=0, atol=2e-6 * np.abs(g64).max())
