"""GPU parity: the CUDA sweep and solver against the CPU oracle and the reference's golden vectors."""
import numpy as np
import pytest

import bte_oracle
import sweep_order
from openbte_gb300 import objects as O

pytestmark = pytest.mark.gpu


def _state_from_exact(geo, mat, bcs, dT, TB):
    """Per-ordinate exact solves (the reference's splu) and the interface values they imply."""
    ops = bte_oracle.setup_operators(geo, mat, bcs)
    solver = bte_oracle.OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)
    row, nb, k, cut = sweep_order.directed_faces(geo)
    n = geo.n_elems
    idf = ops["i_diffuse"]
    out_T = np.zeros(n)
    out_B = np.zeros(len(idf))
    xs = []
    for q in range(ops["n_angles"]):
        g = k @ np.asarray(mat.vmfp[q])[: geo.dim]
        src = np.unique(nb[(g < 0) & cut])
        Tq = []
        for m, mfp in enumerate(mat.mfps):
            B = dT + mfp * ops["perturbation"][q]
            np.add.at(B, idf, mfp * (-TB * ops["Gbm2"][q]))
            T = solver.solve(q, m, B)
            out_T += mat.t_coeff[m, q] * T
            out_B -= T[idf] * ops["GG"][m, q]
            Tq.append(T[src])
        xs.append(np.array(Tq).T.reshape(-1))       # [src, m] -> (k * n_mfp + m)
    return out_T, out_B, np.concatenate(xs)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("df", 1e-11), ("fp32", 2e-5)])
def test_sweep_equals_exact_ordinate_solves(case, precision, tol):
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, get_plan
    import ctypes as C
    geo, mat, bcs, ek, d = case("a600")
    rng = np.random.default_rng(0)
    n = geo.n_elems
    dT = 0.3 * rng.standard_normal(n)
    TB = 0.3 * rng.standard_normal(len(geo.side_physical_regions["Boundary"]))
    refT, refB, x = _state_from_exact(geo, mat, bcs, dT, TB)
    plan = get_plan(HostProblem(geo, mat, bcs, ek))
    assert plan.nx == len(x)
    u = torch.tensor(np.concatenate([dT, TB, x]), dtype=torch.float64, device="cuda")
    out = torch.zeros_like(u)
    _lib.check(plan.lib.obte_bte_sweep(plan.handle, _lib.PRECISION[precision], C.c_void_p(u.data_ptr()),
                                       C.c_void_p(out.data_ptr()), 1), "sweep")
    o = out.cpu().numpy()
    scale = max(np.abs(refT).max(), 1.0)
    np.testing.assert_allclose(o[:n], refT, rtol=0, atol=tol * scale)
    np.testing.assert_allclose(o[n:n + len(TB)], refB, rtol=0, atol=tol * scale)
    np.testing.assert_allclose(o[n + len(TB):], x, rtol=0, atol=tol * scale)


@pytest.mark.parametrize("name", ["a600", "gray600", "circ1k", "c0_2k", "cube1k5"])
def test_bte_fp64_matches_reference(case, name):
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case(name)
    f = O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    r = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-11, precision="fp64")
    # FP64 mode: 1e-6 relative on kappa and the temperature field
    assert abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"]) < 1e-6, (r.kappa_eff, d["bte_kappa"])
    T = r.variables["Temperature_BTE"]["data"]
    np.testing.assert_allclose(T, d["bte_T"], rtol=0, atol=1e-6 * np.abs(d["bte_T"]).max())
    J = r.variables["Flux_BTE"]["data"]
    np.testing.assert_allclose(J, d["bte_J"], rtol=0, atol=1e-6 * np.abs(d["bte_J"]).max())
    np.testing.assert_allclose(r.aux["suppression"], d["bte_S"], rtol=0, atol=1e-6 * np.abs(d["bte_S"]).max())


@pytest.mark.parametrize("precision,tol", [("fp32_refine", 1e-6), ("fp32", 1e-4)])
def test_bte_reduced_precision(case, precision, tol):
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case("c0_2k")
    f = O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    r = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-9 if precision != "fp32" else 1e-6,
                precision=precision)
    err = abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"])
    assert err < tol, (precision, err, r.aux)
    T = r.variables["Temperature_BTE"]["data"]
    np.testing.assert_allclose(T, d["bte_T"], rtol=0, atol=10 * tol * np.abs(d["bte_T"]).max())


@pytest.mark.parametrize("name", ["a600", "cube1k5", "gray600"])
def test_double_float_sweep_equals_fp64_sweep(case, name):
    """The double-float output pass (pairs of FP32 on the FP32 pipe) against the FP64 sweep on the same state:
    every output within 1e-12 of the largest, on random states with and without the source."""
    import ctypes as C
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, d = case(name)
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    rng = np.random.default_rng(4)
    for src in (1, 0):
        u = torch.tensor(rng.standard_normal(plan.nu), dtype=torch.float64, device="cuda")
        outs = {}
        for prec in ("fp64", "df"):
            out = torch.zeros_like(u)
            _lib.check(plan.lib.obte_bte_sweep(plan.handle, _lib.PRECISION[prec], C.c_void_p(u.data_ptr()),
                                               C.c_void_p(out.data_ptr()), src), prec)
            outs[prec] = out.cpu().numpy()
        scale = np.abs(outs["fp64"]).max()
        np.testing.assert_allclose(outs["df"], outs["fp64"], rtol=0, atol=1e-12 * scale)


@pytest.mark.parametrize("double_float", [False, True])
def test_fp32_refine_output_pass(case, monkeypatch, double_float):
    """FP32+refine solves run their output pass in FP64, or with OBTE_REFINE_DF=1 in double-float arithmetic on
    the FP32 pipe; either keeps the reference's kappa (golden c0_2k at bte_rtol 1e-12) to 1e-8."""
    from openbte_gb300 import BTE_RTA
    if double_float:
        monkeypatch.setenv("OBTE_REFINE_DF", "1")
    else:
        monkeypatch.delenv("OBTE_REFINE_DF", raising=False)
    geo, mat, bcs, ek, d = case("c0_2k")
    f = O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    r = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-10, precision="fp32_refine")
    if double_float:
        assert r.aux["n_sweeps_df"] >= 1 and r.aux["n_sweeps_fp64"] == 0, r.aux
    else:
        assert r.aux["n_sweeps_fp64"] >= 1 and r.aux["n_sweeps_df"] == 0, r.aux
    assert abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"]) < 1e-8


def test_fp32_refine_loose_tolerance_runs_no_fp64_sweep(case, monkeypatch):
    """At a tolerance of 5e-6 or looser the output pass is FP32 (its rounding is under a tenth of the
    tolerance): no FP64 sweep, kappa within the tolerance of the reference's (golden c0_2k), and the same
    solve with the FP64 pass forced agrees to the tolerance."""
    from openbte_gb300 import BTE_RTA
    monkeypatch.delenv("OBTE_REFINE_DF", raising=False)
    geo, mat, bcs, ek, d = case("c0_2k")
    f = O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    r = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-5, precision="fp32_refine")
    assert r.aux["n_sweeps_fp64"] == 0 and r.aux["residual"] <= 1e-5, r.aux
    assert abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"]) < 1e-4
    monkeypatch.setenv("OBTE_REFINE_FP64_PASS", "1")
    r64 = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-5, precision="fp32_refine")
    assert r64.aux["n_sweeps_fp64"] >= 1
    assert abs(r.kappa_eff - r64.kappa_eff) / abs(r64.kappa_eff) < 1e-5


@pytest.mark.parametrize("name", ["c0_2k", "cube1k5"])
def test_fp64_sweep_with_and_without_the_reciprocal_table(case, monkeypatch, name):
    """FP64 sweeps multiply by the plan's table of 1 / (1 + mfp D); with the table off (OBTE_SWEEP64_RINV=0)
    they divide (an FP32 seed with one quotient correction, relative error <= 2^-42).  Both give the same sweep
    to 1e-12 of the largest output, with and without the source."""
    import ctypes as C
    import torch
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, d = case(name)
    rng = np.random.default_rng(6)
    outs = {}
    for rinv in ("1", "0"):
        monkeypatch.setenv("OBTE_SWEEP64_RINV", rinv)
        plan = Plan(HostProblem(geo, mat, bcs, ek))
        u = torch.tensor(rng.standard_normal(plan.nu) if rinv == "1" else outs["u"], dtype=torch.float64,
                         device="cuda")
        outs["u"] = u.cpu().numpy()
        for src in (1, 0):
            out = torch.zeros_like(u)
            _lib.check(plan.lib.obte_bte_sweep(plan.handle, _lib.PRECISION["fp64"], C.c_void_p(u.data_ptr()),
                                               C.c_void_p(out.data_ptr()), src), "fp64")
            outs[(rinv, src)] = out.cpu().numpy()
    for src in (1, 0):
        a, b = outs[("1", src)], outs[("0", src)]
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * np.abs(b).max())
