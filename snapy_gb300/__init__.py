"""snapy_gb300: the snapy MeshBlock hydro stage on GB300 (sm_103a).

Drop-in surface of the reference's ``snapy`` module for the hydro-stage path:
``MeshBlockOptions.from_yaml`` and ``MeshBlock`` with the same deck keys.  The
compute runs in the in-tree CUDA library ``libsnapy_gb300.so`` (C ABI:
include/snapy_gb300.h); there is no CPU path.
"""
from .options import (CoordinateOptions, DeckError, EquationOfStateOptions,
                      HydroOptions, IntegratorOptions, MeshBlockOptions,
                      ReconstructOptions, RiemannSolverOptions)
from .meshblock import MeshBlock, kICY, kIDN, kIPR, kIV1, kIVX, kIVY, kIVZ

__all__ = [
    "MeshBlockOptions", "MeshBlock", "CoordinateOptions", "HydroOptions",
    "IntegratorOptions", "EquationOfStateOptions", "ReconstructOptions",
    "RiemannSolverOptions", "DeckError", "kIDN", "kIVX", "kIVY", "kIVZ",
    "kIPR", "kICY", "kIV1",
]
__version__ = "0.1.0"
