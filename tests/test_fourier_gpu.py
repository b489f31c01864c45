"""GPU parity of the device Fourier solver against the reference's golden Fourier outputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["a600", "circ1k", "gray600", "c0_2k", "cube1k5"])
def test_fourier_matches_reference(case, name):
    from openbte_gb300 import Fourier
    geo, mat, bcs, ek, d = case(name)
    f = Fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek, verbose=False)
    assert f.kappa_eff == 0                                     # the reference's returned value
    k = f.aux["kappa_eff"]
    assert abs(k - d["fourier_kappa_printed"]) / abs(k) < 1e-6   # printed with 7 significant digits
    T = f.variables["Temperature_Fourier"]["data"]
    np.testing.assert_allclose(T, d["fourier_T"], rtol=0, atol=1e-9 * max(1.0, np.abs(d["fourier_T"]).max()))
    J = f.variables["Flux_Fourier"]["data"]
    np.testing.assert_allclose(J, d["fourier_J"], rtol=0, atol=1e-8 * np.abs(d["fourier_J"]).max())


def test_fourier_first_guess_feeds_bte(case):
    """Device Fourier -> device BTE matches the reference pipeline (Fourier guess then BTE_RTA)."""
    from openbte_gb300 import BTE_RTA, Fourier
    geo, mat, bcs, ek, d = case("a600")
    f = Fourier(geo, mat.thermal_conductivity, bcs, effective_thermal_conductivity=ek, verbose=False)
    r = BTE_RTA(geo, mat, bcs, fourier=f, effective_thermal_conductivity=ek, bte_rtol=1e-11)
    assert abs(r.kappa_eff - d["bte_kappa"]) / d["bte_kappa"] < 1e-6
    np.testing.assert_allclose(r.variables["Temperature_BTE"]["data"], d["bte_T"], rtol=0,
                               atol=1e-6 * np.abs(d["bte_T"]).max())
