"""The CPU oracle against golden vectors frozen from the unmodified reference."""
import numpy as np
import pytest

import bte_oracle
import fourier_oracle
from openbte_gb300 import objects as O


@pytest.mark.parametrize("name", ["a600", "circ1k", "gray600", "cube1k5"])
def test_fourier_oracle_matches_reference(case, name):
    geo, mat, bcs, ek, d = case(name)
    k, T, J, it = fourier_oracle.fourier(geo, mat.thermal_conductivity, bcs, ek)
    assert abs(k - d["fourier_kappa_printed"]) / abs(k) < 1e-6       # printed with 7 digits
    np.testing.assert_allclose(T, d["fourier_T"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(J * 1e9, d["fourier_J"], rtol=1e-10, atol=1e-10 * np.abs(d["fourier_J"]).max())
    assert d["fourier_kappa_returned"] == 0                           # the reference's while/else


@pytest.mark.parametrize("name", ["a600", "gray600", "cube1k5"])
def test_bte_oracle_matches_reference(case, name):
    geo, mat, bcs, ek, d = case(name)
    f = O.SolverResults(variables={"Temperature_Fourier": {"data": d["fourier_T"]}})
    k, dT, J, K, S, it = bte_oracle.bte_rta(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek,
                                            bte_rtol=1e-12, bte_max_iter=2000)
    assert abs(k - d["bte_kappa"]) / abs(d["bte_kappa"]) < 1e-12
    np.testing.assert_allclose(dT, d["bte_T"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(J * 1e9, d["bte_J"], rtol=0, atol=1e-9 * np.abs(d["bte_J"]).max())
    np.testing.assert_allclose(S, d["bte_S"], rtol=0, atol=1e-10 * np.abs(d["bte_S"]).max())


def test_reference_default_tolerance_is_loose(case):
    """At its default bte_rtol=1e-4 the reference stops ~1e-3 away from its converged kappa."""
    _, _, _, _, d = case("c0_2k")
    rel = abs(d["bte_kappa_rtol1e4"] - d["bte_kappa"]) / d["bte_kappa"]
    assert 1e-5 < rel < 1e-2
