"""The oracle's cut-periodic ordinate solve against the reference's full per-ordinate LU (CPU).

``bte_oracle.cut_ordinate_solve`` is the exact check of the GPU sweep on meshes where the reference's
SuperLU factorisation of the periodic operator is too slow (about 290 s per ordinate on the
110k-tetrahedron benchmark cube).  Given the exact periodic values at the source elements it must
reproduce the full LU solve of openbte/bte.py:181-185, 217-218.
"""
import numpy as np
import pytest

import bte_oracle
import sweep_order


@pytest.mark.parametrize("name,ordinates", [("a600", [(0, 7), (4, 7), (9, 3), (13, 0)]),
                                            ("cube1k5", [(0, 5), (17, 5), (31, 2)])])
def test_cut_solve_with_exact_inflow_equals_full_lu(case, name, ordinates):
    geo, mat, bcs, ek, _ = case(name)
    ops = bte_oracle.setup_operators(geo, mat, bcs)
    solver = bte_oracle.OrdinateSolver(geo, np.asarray(mat.mfps, dtype=np.float64), ops)
    faces = sweep_order.directed_faces(geo)
    row, nb, k, cut = faces
    rng = np.random.default_rng(3)
    for q, m in ordinates:
        B = rng.standard_normal(geo.n_elems)
        T = solver.solve(q, m, B)
        g = k @ np.asarray(mat.vmfp[q])[: geo.dim]
        src = np.unique(nb[(g < 0) & cut])
        order, _ = sweep_order.schedule(geo, mat.vmfp[q], faces)
        Tc = bte_oracle.cut_ordinate_solve(solver, faces, q, m, B, T[src], src, order)
        np.testing.assert_allclose(Tc, T, rtol=0, atol=1e-12 * np.abs(T).max())
        # an order that is not topological is refused instead of giving a wrong solution
        with pytest.raises(ValueError):
            bte_oracle.cut_ordinate_solve(solver, faces, q, m, B, T[src], src, order[::-1])
