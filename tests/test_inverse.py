"""Host side of the inverse-design solver (no GPU)."""
import numpy as np
import pytest


def test_reversed_material_and_closure():
    from openbte_gb300.inverse import IsotropicMaterial
    even = IsotropicMaterial([0.1, 1.0], [0.4, 0.6], 16)
    odd = IsotropicMaterial([0.1, 1.0], [0.4, 0.6], 15)
    assert even.closed_under_reversal() and not odd.closed_under_reversal()
    r = odd.reversed()
    np.testing.assert_array_equal(r.vmfp, -odd.vmfp)
    np.testing.assert_array_equal(r.sigma, -odd.sigma)
    np.testing.assert_array_equal(r.t_coeff, odd.t_coeff)
    np.testing.assert_array_equal(r.mfps, odd.mfps)
    # equally spaced directions: sum sigma = 0, as the reversed problem's re-emitting sides require
    assert np.abs(odd.sigma.sum(axis=(0, 1))).max() < 1e-12 * np.abs(odd.sigma).sum()


def _dsa_expected(grid, mat, t, floor_frac=0.05, reg_frac=1e-6):
    """The acceleration's diffusion operator restated in numpy (dense): per side A sum_m 1 / (d / D_m +
    (1 - t) / (G_m t)) (A D / d for t = 1), diagonal floored at 5 % of the upper median per volume, plus 1e-6 of
    the largest diagonal."""
    sem = grid["side_elem_map"]
    V = grid["elem_volumes"]
    A = np.linalg.norm(grid["normal_areas"], axis=1)
    d = 2 * V[sem[:, 0]] / (4 * A) + 2 * V[sem[:, 1]] / (4 * A)    # dim V / (sides x area), both halves
    tau, L, v = mat.t_coeff, mat.mfps, mat.vmfp
    v2 = (v ** 2).sum(axis=1)
    Dm = (tau * L[:, None] ** 2 * v2[None, :]).sum(axis=1) / 2
    Gm = (tau * L[:, None] * np.sqrt(v2)[None, :]).sum(axis=1) / np.pi
    coef = np.empty(len(t))
    for k in range(len(t)):
        if t[k] >= 1:
            coef[k] = A[k] * Dm.sum() / d[k]
        else:
            coef[k] = A[k] * np.sum(1.0 / (d[k] / Dm + (1 - t[k]) / (Gm * t[k])))
    n = len(V)
    M = np.zeros((n, n))
    diag = np.zeros(n)
    for k, (i, j) in enumerate(sem):
        diag[i] += coef[k]
        diag[j] += coef[k]
        M[i, j] -= coef[k]
        M[j, i] -= coef[k]
    reg = reg_frac * diag.max()
    med = np.sort(diag / V)[n // 2]                      # the upper median (element n / 2 of the sorted values)
    diag = np.maximum(diag, floor_frac * med * V)
    M[np.arange(n), np.arange(n)] += diag + reg
    return M


def test_dsa_operator_matches_its_restatement():
    """The acceleration's cell diffusion operator of a transmission-interface plan (host-only plan, no GPU)
    equals the numpy restatement of its conductances, floor and shift, and is symmetric."""
    import ctypes as C
    from openbte_gb300 import _lib
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    rng = np.random.default_rng(3)
    n = 8
    mat = IsotropicMaterial.lognormal(4, 8)
    solver = PixelSolver(n, mat, size=100.0)
    rho = rng.uniform(0.0, 1.0, n * n)
    rho[5] = 0.0                                         # one pore pixel: its sides transmit ~1e-12
    sem = solver.grid["side_elem_map"]
    r = 1e-12 + rho * (1.0 - 1e-12)
    t = np.ascontiguousarray(2 * r[sem[:, 0]] * r[sem[:, 1]] / (r[sem[:, 0]] + r[sem[:, 1]]))
    lib = solver.lib
    prob, cm = solver._problem(t), mat.c_struct()
    h = C.c_void_p()
    _lib.check(lib.obte_bte_plan_create(None, C.byref(prob), C.byref(cm), C.byref(h)), "plan_create")
    try:
        nnz, proj = C.c_int64(0), C.c_int32()
        _lib.check(lib.obte_bte_dsa_operator(h, C.byref(nnz), None, None, None, C.byref(proj)), "dsa size")
        rp = np.zeros(n * n + 1, np.int32)
        ci = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        _lib.check(lib.obte_bte_dsa_operator(h, C.byref(nnz), rp.ctypes.data_as(C.c_void_p),
                                             ci.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p),
                                             C.byref(proj)), "dsa operator")
    finally:
        lib.obte_bte_plan_destroy(h)
    assert proj.value == 1
    Mgot = np.zeros((n * n, n * n))
    for i in range(n * n):
        cols = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(cols) > 0)
        Mgot[i, cols] = val[rp[i]:rp[i + 1]]
    np.testing.assert_allclose(Mgot, Mgot.T, rtol=1e-14, atol=0)
    Mexp = _dsa_expected(solver.grid, mat, t)
    np.testing.assert_allclose(Mgot, Mexp, rtol=1e-12, atol=1e-12 * np.abs(Mexp).max())
    # the pore pixel's row is the floor (its sides' conductances are ~1e-12)
    assert Mgot[5, 5] > 1e6 * np.abs(np.delete(Mgot[5], 5)).max()


@pytest.mark.parametrize("name", ["a600", "cube1k5"])
def test_dsa_operator_on_unstructured_meshes(case, name):
    """The acceleration's operator on triangles and tetrahedra (host-only plan): per internal side
    A sum_m D_m / d with d = sum over the side's two elements of dim V / (sides x A) (exact for simplices),
    the floor and the shift, against a numpy restatement; symmetric, with the source projected (no
    isothermal walls)."""
    import ctypes as C
    from openbte_gb300 import _lib
    from openbte_gb300.runtime import HostProblem, Plan
    geo, mat, bcs, ek, _ = case(name)
    hp = HostProblem(geo, mat, bcs, ek)
    plan = Plan(hp, host_only=True)
    n = hp.n_elems
    nnz, proj = C.c_int64(0), C.c_int32()
    _lib.check(plan.lib.obte_bte_dsa_operator(plan.handle, C.byref(nnz), None, None, None, C.byref(proj)), "size")
    rp, ci, val = np.zeros(n + 1, np.int32), np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    _lib.check(plan.lib.obte_bte_dsa_operator(plan.handle, C.byref(nnz), rp.ctypes.data_as(C.c_void_p),
                                              ci.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p),
                                              C.byref(proj)), "operator")
    assert proj.value == 1
    M = np.zeros((n, n))
    for i in range(n):
        M[i, ci[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    np.testing.assert_allclose(M, M.T, rtol=1e-14, atol=0)
    # restatement
    dim, nf = hp.dim, hp.elem_nv
    V = hp.vol
    tc, L = np.asarray(mat.t_coeff, dtype=np.float64), np.asarray(mat.mfps, dtype=np.float64)
    v = np.asarray(mat.vmfp, dtype=np.float64)[:, :dim]
    Dsum = (tc * L[:, None] ** 2 * (v ** 2).sum(axis=1)[None, :]).sum() / dim
    E = np.zeros((n, n))
    diag = np.zeros(n)
    for sd in hp.internal:
        i, j = hp.sem[sd]
        A = np.linalg.norm(hp.na[sd])
        d = dim * V[i] / (nf * A) + dim * V[j] / (nf * A)
        c = A * Dsum / d
        diag[i] += c
        diag[j] += c
        E[i, j] -= c
        E[j, i] -= c
    reg = 1e-6 * diag.max()
    diag = np.maximum(diag, 0.05 * np.sort(diag / V)[n // 2] * V)
    E[np.arange(n), np.arange(n)] += diag + reg
    np.testing.assert_allclose(M, E, rtol=1e-11, atol=1e-11 * np.abs(E).max())
