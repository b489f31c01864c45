"""GB300-native (sm_103a) phonon BTE transport: a drop-in for OpenBTE's BTE_RTA / Fourier path.

Public names follow the reference's exports (openbte/__init__.py:7-16) for the
transport path: ``BTE_RTA``, ``Fourier``, ``get_mesh`` and the data types.
"""
from .objects import (BoundaryConditions, EffectiveThermalConductivity, Material, Mesh,  # noqa: F401
                      SolverResults)
from .mesh import get_mesh  # noqa: F401
from .material import Gray2D, RTA2DSym, RTA3D, load_rta, synthetic_isotropic_2d, synthetic_isotropic_3d  # noqa: F401
from .objects import MaterialRTA  # noqa: F401
from .results import OpenBTEResults  # noqa: F401


def __getattr__(name):
    # the solvers load the CUDA library on first use
    if name == "BTE_RTA":
        from .bte import BTE_RTA
        return BTE_RTA
    if name == "Fourier":
        from .fourier import Fourier
        return Fourier
    raise AttributeError(name)
