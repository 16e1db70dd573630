"""gbem: GB300-native BEM matrix assembly and dense complex LU for SCUFF-EM's hot path.

The compute path is libgbem.so (hand-written sm_103a CUDA behind the C ABI in
include/gbem.h); this package is a thin Python mirror of the reference's
RWGGeometry / HMatrix interface on top of it.
"""
from . import mesh  # noqa: F401
from ._lib import C128, C64, F64, GbemError, lib  # noqa: F401
from .api import HMatrix, Material, RWGGeometry, ZVAC, solve_mixed_batch  # noqa: F401
from . import casimir  # noqa: F401

__all__ = ["RWGGeometry", "HMatrix", "Material", "GbemError", "C128", "C64", "ZVAC", "mesh", "lib"]
