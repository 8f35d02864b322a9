"""richmol_gb300: GB300-native Krylov time propagation for rotational dynamics.

Drop-in for the propagation path of CFEL-CMI/richmol: ``TDSE.update`` applied
to ``CarTens`` operators, computed by hand-written sm_103a CUDA kernels behind
a C ABI (include/richmol_gb300.h).
"""
from .field import CarTens, clear_plan_cache, filter  # noqa: F401
from .tdse import TDSE, ExpokitError  # noqa: F401
from .trove import CarTensTrove  # noqa: F401
from . import convert_units  # noqa: F401

__all__ = ["CarTens", "CarTensTrove", "TDSE", "ExpokitError", "convert_units", "clear_plan_cache", "filter"]
