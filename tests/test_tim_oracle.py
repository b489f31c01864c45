"""The transmission-interface (TIM) oracle against the reference's gray inverse-design model.

Golden vectors come from the reference's own openbte/inverse/bte.py (run by
tests/golden/make_golden_inverse.py); the MFP-resolved generalisation is pinned by its explicit
adjoint and by central finite differences.
"""
import os

import numpy as np
import pytest

import tim_oracle as T

GOLD = os.path.join(os.path.dirname(__file__), "golden", "inverse_gray.npz")


@pytest.mark.parametrize("name", ["g8_kn1", "g8_kn01", "g10_kn05"])
def test_gray_kappa_and_gradient_match_reference(name):
    d = np.load(GOLD)
    n, kn, n_phi, _ = d[name + "_meta"]
    grid = T.pixel_grid(int(n))
    mat = T.gray_material(kn, int(n_phi))
    rho = d[name + "_rho"]
    k, g, X = T.kappa_and_gradient(rho, grid, mat)
    assert abs(k - d[name + "_kappa"][0]) <= 1e-10 * abs(k)
    np.testing.assert_allclose(g, d[name + "_grad"], rtol=0, atol=1e-10 * np.abs(g).max())
    # the reference's state is X for one MFP, [q][pixel]; equal up to the constant null mode
    dX = X[0] - d[name + "_T"].reshape(X.shape[1:])
    assert np.ptp(dX) <= 1e-8 * np.abs(X).max()


def test_multi_mfp_adjoint_identity_and_finite_differences():
    grid = T.pixel_grid(6)
    mat = T.material([0.05, 0.4, 2.0], [0.5, 0.3, 0.2], 8)
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.1, 1.0, 36)
    k, g_refl, _ = T.kappa_and_gradient(rho, grid, mat)
    _, g_adj, _ = T.kappa_and_gradient(rho, grid, mat, method="adjoint")
    np.testing.assert_allclose(g_refl, g_adj, rtol=0, atol=1e-11 * np.abs(g_adj).max())
    pix = rng.choice(36, 5, replace=False)
    fd = T.kappa_fd(rho, grid, mat, pix, h=1e-6)
    np.testing.assert_allclose(g_refl[pix], fd, rtol=1e-6, atol=1e-8 * np.abs(g_refl).max())


def test_reference_inverse_golden_regenerates():
    """When the reference checkout is present, its inverse model still produces the committed vectors."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import ref_loader
    if not ref_loader.available_inverse():
        pytest.skip("reference inverse-design modules absent (a source checkout is needed: OBTE_REFERENCE)")
    import make_golden_inverse as M
    d = np.load(GOLD)
    name, n, kn, n_phi, seed = M.CASES[0]
    rho = M.seeded_density(n, seed)
    np.testing.assert_array_equal(rho, d[name + "_rho"])
    kappa, grad, _, _ = M.reference_gray(n, kn, n_phi, rho)
    assert abs(kappa - d[name + "_kappa"][0]) <= 1e-12 * abs(kappa)
    np.testing.assert_allclose(grad, d[name + "_grad"], rtol=0, atol=1e-12 * np.abs(grad).max())
