"""The product path has no CPU fallback: without a usable GPU every solve fails loudly.

Runs only where no CUDA device is visible (this is the build host's situation; on a GPU machine it is
skipped)."""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="a GPU is visible")


def test_bte_rta_raises_without_a_gpu():
    from openbte_gb300 import BTE_RTA, objects as O
    from openbte_gb300.geometry import porous_cell_2d
    from openbte_gb300.material import synthetic_isotropic_2d
    from openbte_gb300.mesh import mesh_from_cell
    geo = mesh_from_cell(porous_cell_2d(200, 0.25, "square", seed=2))
    bcs = O.BoundaryConditions(periodic={"Periodic_x": 1, "Periodic_y": 0}, diffuse="Boundary")
    ek = O.EffectiveThermalConductivity(normalization=-1, contact="Periodic_x")
    with pytest.raises(Exception) as ei:
        BTE_RTA(geo, synthetic_isotropic_2d(4, 8), bcs, effective_thermal_conductivity=ek)
    assert "cuda" in str(ei.value).lower() or "device" in str(ei.value).lower() or "gpu" in str(ei.value).lower(), \
        ei.value


def test_context_create_reports_the_missing_device():
    import ctypes as C
    from openbte_gb300 import _lib
    lib = _lib.load()
    ctx = C.c_void_p()
    st = lib.obte_context_create(0, None, C.byref(ctx))
    assert st != _lib.OBTE_OK
    assert lib.obte_last_error()
