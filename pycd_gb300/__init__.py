"""GB300-native (sm_103a) lattice-KMC hot path of PyCD.

Drop-in ``Material`` / ``Neighbors`` / ``System`` / ``Run`` / ``Analysis``
whose Ewald array build, KMC loop and MSD analysis run as hand-written CUDA
kernels behind the C ABI declared in include/pycd_gb300.h
(``libpycd_gb300.so``).
"""
from .core import Material, Neighbors, ReturnValues, Run, System  # noqa: F401
from .analysis import Analysis  # noqa: F401
from . import constants  # noqa: F401

__all__ = ["Material", "Neighbors", "System", "Run", "Analysis", "ReturnValues",
           "constants"]
