"""Host side of the inverse-design solver (no GPU)."""
import numpy as np


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
