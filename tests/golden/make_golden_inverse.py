"""Golden vectors of the reference's gray inverse-design model (openbte/inverse/bte.py).

Test infrastructure only.  Runs the reference's own ``get_common``, ``get_rho_dependent``,
``operator`` and ``compute_kappa_and_gradient`` (openbte/inverse/bte.py:27-168) on the numpy
stand-in for jax from ``ref_loader.load_inverse`` and freezes kappa_eff and dkappa/drho for a few
seeded density grids into ``inverse_gray.npz``.

The reference drives its operator through ``utils.solver`` (openbte/utils.py:86-145), a
``scipy.sparse.linalg.lgmres`` wrapper that passes ``tol=`` (removed from scipy in 1.14; the call
raises, the wrapper swallows the error and returns the callback at a zero state) and stops early
once kappa and the gradient change by less than 1e-4.  Here the same operator is solved to 1e-13
with lgmres (from a zero start; the system is singular with a constant null vector and
consistent), and the reference's gradient function is evaluated at that state.

Run: python tests/golden/make_golden_inverse.py   (needs the reference checkout)
"""
import os
import sys
from functools import partial

import numpy as np
from scipy.sparse.linalg import LinearOperator, lgmres

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))   # ref_loader
import ref_loader  # noqa: E402

CASES = [
    # name, grid N, Kn (MFP / cell side), n_phi, density seed
    ("g8_kn1", 8, 1.0, 16, 0),
    ("g8_kn01", 8, 0.1, 16, 1),
    ("g10_kn05", 10, 0.5, 24, 2),
]


def seeded_density(n, seed):
    """Smoothed Gaussian random field in [0, 1] on an n x n periodic grid (pixel order i*n + j)."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((n, n))
    k = np.fft.fftfreq(n)
    kk = k[:, None] ** 2 + k[None, :] ** 2
    z = np.real(np.fft.ifft2(np.fft.fft2(z) * np.exp(-kk * (n / 3.0) ** 2)))
    z = (z - z.min()) / (z.max() - z.min())
    return 0.05 + 0.9 * z.reshape(-1)


def reference_gray(n, kn, n_phi, rho):
    ns = ref_loader.load_inverse()
    ib = ns.bte
    common = ib.get_common(grid=n, Kn=kn, n_phi=n_phi, directions=[[1, 0]])
    aux = ib.get_rho_dependent(ns.asarray(rho), common)
    (gm_direct, gp_direct, t_flat, P_vec, dt_sparse, dt_sparseT, i_mat, j_mat, gm, gp, D, GG, ind_extremes,
     reflection, f, gm_reflected) = aux
    L = partial(ib.operator, aux3=(D, i_mat, j_mat, gm_direct, GG, gm_reflected))
    P = np.einsum("i,iuc->cu", np.array([1.0, 0.0]), np.asarray(P_vec))
    kj, ki = ind_extremes[0, 0], ind_extremes[0, 1]
    size = P.size
    op = LinearOperator((size, size), matvec=lambda x: np.asarray(L(ns.asarray(x))), dtype=np.float64)
    x, info = lgmres(op, P.reshape(-1), rtol=1e-13, atol=0.0, maxiter=5000)
    assert info == 0, info
    res = np.linalg.norm(np.asarray(L(ns.asarray(x))) - P.reshape(-1)) / np.linalg.norm(P)
    assert res < 1e-11, res
    kappa, grad = ib.compute_kappa_and_gradient(ns.asarray(x), aux, (ki, kj, ns.asarray(P)))
    return float(kappa), np.asarray(grad, dtype=np.float64), np.asarray(x), np.asarray(t_flat)


def main():
    out = {}
    for name, n, kn, n_phi, seed in CASES:
        rho = seeded_density(n, seed)
        kappa, grad, x, t = reference_gray(n, kn, n_phi, rho)
        out[f"{name}_meta"] = np.array([n, kn, n_phi, seed], dtype=np.float64)
        out[f"{name}_rho"] = rho
        out[f"{name}_kappa"] = np.array([kappa])
        out[f"{name}_grad"] = grad
        out[f"{name}_T"] = x
        out[f"{name}_t"] = t
        print(name, "kappa", kappa, "|grad|", np.abs(grad).max())
    np.savez_compressed(os.path.join(HERE, "inverse_gray.npz"), **out)


if __name__ == "__main__":
    main()
