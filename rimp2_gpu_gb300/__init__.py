"""rimp2_gpu_gb300 -- GB300-native (sm_103a) RI-MP2 amplitude and energy path.

Drop-in for the subroutines of januseriksen/rimp2_gpu's RIMP2.F90 through a
C-ABI library (``include/rimp2_gpu.h``); this package is its Python host
side.  See ``api`` for the reference-shaped entry points.
"""
from ._lib import LIB_PATH, Rimp2Error, lib  # noqa: F401
from . import api  # noqa: F401

__all__ = ["api", "lib", "Rimp2Error", "LIB_PATH"]
