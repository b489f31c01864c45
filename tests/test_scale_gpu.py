"""GPU parity at the benchmark sizes.

* One sweep of the full 2D benchmark plan (60k triangles, 100 MFPs x 96 directions) against the
  reference's exact per-ordinate solves (SuperLU of the periodic operator, openbte/bte.py:181-185,
  217-218) on 20 sampled ordinates: the four axis-aligned directions at the three longest MFPs (rays in
  the free channels beside the pore, which wrap the cell ~100 times) and eight seeded others.
* One sweep of the full 3D benchmark plan (110k tetrahedra, 30 MFPs x 16 x 32 directions) against the
  oracle's cut-periodic solve (the same operator with the inflow across the periodic boundary given;
  SuperLU of the periodic operator takes ~290 s per ordinate there) on 16 sampled ordinates, including
  the directions 5.6 degrees off the z axis at the longest MFPs.
* Full solves against the unmodified reference run with reduced ordinate sets (fixtures from
  tests/golden/make_golden_scale.py) on the 2D benchmark mesh and on the 3D benchmark cube at ~45k tetrahedra
  (the reference's SuperLU on the 110k-tetrahedron mesh takes hours): kappa within 1e-6, fields within 1e-6
  of their maxima in FP64; kappa within 1e-4 in FP32+refine.

Per-ordinate temperatures come from obte_bte_sweep_fields.  Tolerances: 1e-11 (FP64, and the double-float
output pass of FP32+refine) and 2e-5 (FP32) of the largest sampled temperature, as in the small-mesh sweep tests.
"""
import ctypes as C

import numpy as np
import pytest

import bte_oracle
import sweep_order
from openbte_gb300 import objects as O

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "df": 1e-11, "fp32": 2e-5}


def _benchmark_2d():
    """The 2D benchmark workload: porous_cell_2d(60000, 0.25, 'square', seed=1), 100 MFPs x 96 directions."""
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cell_2d(60000, 0.25, "square", seed=1))
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    return geo, synthetic_isotropic_2d(100, 96), bcs, ek


def _benchmark_3d():
    """The 3D benchmark workload: porous_cube_3d(100000, 0.10, seed=1), 30 MFPs x 16 x 32 directions."""
    from openbte_gb300.geometry import porous_cube_3d
    from openbte_gb300.material import synthetic_isotropic_3d
    from openbte_gb300.mesh import mesh_from_cell
    cell = porous_cube_3d(100000, 0.10, seed=1)
    geo = mesh_from_cell(cell)
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0, "Periodic_z": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1.0 / cell.size, contact="Periodic_x")
    return geo, synthetic_isotropic_3d(30, 16, 32), bcs, ek


class _Setup:
    """Oracle operators, a random state (DeltaT, T_B) and the per-direction periodic source elements."""

    def __init__(self, geo, mat, bcs, seed):
        self.geo, self.mat = geo, mat
        self.ops = bte_oracle.setup_operators(geo, mat, bcs)
        self.mfps = np.asarray(mat.mfps, dtype=np.float64)
        self.solver = bte_oracle.OrdinateSolver(geo, self.mfps, self.ops)
        self.faces = sweep_order.directed_faces(geo)
        row, nb, k, cut = self.faces
        self.n_mfp, self.n_dir = np.asarray(mat.t_coeff).shape
        self.srcs = [np.unique(nb[((k @ np.asarray(mat.vmfp[q])[: geo.dim]) < 0) & cut]) for q in range(self.n_dir)]
        self.x_base = np.concatenate([[0], np.cumsum([len(s) for s in self.srcs])])
        rng = np.random.default_rng(seed)
        self.dT = 0.3 * rng.standard_normal(geo.n_elems)
        self.TB = 0.3 * rng.standard_normal(len(self.ops["i_diffuse"]))

    def rhs(self, q, m):
        """B of openbte/bte.py:199-214 at the state, with the periodic-jump source."""
        ops = self.ops
        B = self.dT + self.mfps[m] * ops["perturbation"][q]
        if len(self.TB):
            np.add.at(B, ops["i_diffuse"], self.mfps[m] * (-self.TB * ops["Gbm2"][q]))
        return B

    def x_index(self, q, m):
        return (self.x_base[q] + np.arange(len(self.srcs[q]))) * self.n_mfp + m


def _sweep_fields(plan, precision, u):
    import torch
    from openbte_gb300 import _lib
    n_dir, n, n_mfp = plan.hp.n_dir, plan.n, plan.hp.n_mfp
    T = torch.empty((n_dir, n, n_mfp), dtype=torch.float32 if precision == "fp32" else torch.float64, device="cuda")
    out = torch.zeros_like(u)
    _lib.check(plan.lib.obte_bte_sweep_fields(plan.handle, _lib.PRECISION[precision], C.c_void_p(u.data_ptr()),
                                              C.c_void_p(out.data_ptr()), 1, C.c_void_p(T.data_ptr())),
               "obte_bte_sweep_fields")
    return T


@pytest.fixture(scope="module")
def exact_2d():
    """Exact periodic solves of the sampled ordinates of the 2D benchmark (SuperLU, as the reference)."""
    geo, mat, bcs, ek = _benchmark_2d()
    st = _Setup(geo, mat, bcs, seed=11)
    n_mfp, n_dir = st.n_mfp, st.n_dir
    rng = np.random.default_rng(12)
    axis = [0, n_dir // 4, n_dir // 2, 3 * n_dir // 4]          # phi = 0, 90, 180, 270 degrees
    sample = [(q, m) for q in axis for m in range(n_mfp - 3, n_mfp)]
    while len(sample) < 20:
        qm = (int(rng.integers(n_dir)), int(rng.integers(n_mfp)))
        if qm not in sample:
            sample.append(qm)
    x = np.zeros(int(st.x_base[-1]) * n_mfp)
    exact = {}
    for q, m in sample:
        T = st.solver.solve(q, m, st.rhs(q, m))
        st.solver.cache.clear()
        exact[(q, m)] = T
        x[st.x_index(q, m)] = T[st.srcs[q]]
    return geo, mat, bcs, ek, st, x, exact


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
def test_benchmark_2d_sweep_equals_exact_ordinate_solves(exact_2d, precision):
    import torch
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, st, x, exact = exact_2d
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    assert plan.nx == len(x)
    u = torch.tensor(np.concatenate([st.dT, st.TB, x]), dtype=torch.float64, device="cuda")
    T = _sweep_fields(plan, precision, u)
    scale = max(np.abs(t).max() for t in exact.values())
    for (q, m), ref in exact.items():
        got = T[q, :, m].double().cpu().numpy()
        err = np.abs(got - ref).max() / scale
        assert err <= TOL[precision], (precision, q, m, err)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_benchmark_3d_sweep_equals_cut_operator_solves(precision):
    import torch
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek = _benchmark_3d()
    st = _Setup(geo, mat, bcs, seed=21)
    n_mfp, n_dir = st.n_mfp, st.n_dir
    plan = Plan(HostProblem(geo, mat, bcs, ek))
    assert plan.nx == int(st.x_base[-1]) * n_mfp
    rng = np.random.default_rng(22)
    # arbitrary periodic inflow for every ordinate: the cut solve takes it as given
    x = 0.3 * rng.standard_normal(plan.nx)
    # directions 5.6 degrees off +z / -z (the slowest inflow modes of the cube) at the two longest MFPs,
    # and seeded others
    sample = [(q, m) for q in (0, 8, 16, 24, n_dir - 32, n_dir - 16) for m in (n_mfp - 1, n_mfp - 2)]
    while len(sample) < 16:
        qm = (int(rng.integers(n_dir)), int(rng.integers(n_mfp)))
        if qm not in sample:
            sample.append(qm)
    exact = {}
    for q, m in sample:
        order, _, _ = plan.schedule(q)
        exact[(q, m)] = bte_oracle.cut_ordinate_solve(st.solver, st.faces, q, m, st.rhs(q, m), x[st.x_index(q, m)],
                                                      st.srcs[q], order)
    u = torch.tensor(np.concatenate([st.dT, st.TB, x]), dtype=torch.float64, device="cuda")
    T = _sweep_fields(plan, precision, u)
    scale = max(np.abs(t).max() for t in exact.values())
    for (q, m), ref in exact.items():
        got = T[q, :, m].double().cpu().numpy()
        err = np.abs(got - ref).max() / scale
        assert err <= TOL[precision], (precision, q, m, err)


def _guess(d):
    if bool(d["fourier_guess"]):
        return O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    return None


@pytest.mark.parametrize("name", ["c1scale", "c2mid"])
def test_benchmark_mesh_fp64_matches_reference(case, name):
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case(name)
    r = BTE_RTA(geo, mat, bcs, fourier=_guess(d), effective_thermal_conductivity=ek, bte_rtol=1e-11,
                precision="fp64", max_sweeps=3000)
    err = abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"])
    assert err < 1e-6, (name, r.kappa_eff, float(d["bte_kappa"]), err)
    for key, ref in (("Temperature_BTE", d["bte_T"]), ("Flux_BTE", d["bte_J"])):
        got = r.variables[key]["data"]
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-6 * np.abs(ref).max(), err_msg=f"{name} {key}")
    np.testing.assert_allclose(r.aux["suppression"], d["bte_S"], rtol=0, atol=1e-6 * np.abs(d["bte_S"]).max())


@pytest.mark.parametrize("name", ["c1scale", "c2mid"])
def test_benchmark_mesh_fp32_refine_matches_reference(case, name):
    from openbte_gb300 import BTE_RTA
    geo, mat, bcs, ek, d = case(name)
    r = BTE_RTA(geo, mat, bcs, fourier=_guess(d), effective_thermal_conductivity=ek, bte_rtol=1e-7,
                precision="fp32_refine", max_sweeps=3000)
    err = abs(r.kappa_eff - d["bte_kappa"]) / abs(d["bte_kappa"])
    assert err < 1e-4, (name, r.kappa_eff, float(d["bte_kappa"]), err)
    T = r.variables["Temperature_BTE"]["data"]
    np.testing.assert_allclose(T, d["bte_T"], rtol=0, atol=1e-4 * np.abs(d["bte_T"]).max())


def test_benchmark_mesh_fourier_matches_reference(case):
    """The device Fourier first guess on the 60k-triangle mesh against the reference's SuperLU Fourier."""
    from openbte_gb300 import Fourier
    geo, mat, bcs, ek, d = case("c1scale")
    f = Fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek, verbose=False)
    T = f.variables["Temperature_Fourier"]["data"]
    np.testing.assert_allclose(T, d["fourier_T"], rtol=0, atol=1e-8 * np.abs(d["fourier_T"]).max())
    J = f.variables["Flux_Fourier"]["data"]
    np.testing.assert_allclose(J, d["fourier_J"], rtol=0, atol=1e-7 * np.abs(d["fourier_J"]).max())
    assert abs(f.aux["kappa_eff"] - float(d["fourier_kappa_printed"])) <= 1e-6 * abs(float(d["fourier_kappa_printed"]))
