"""mps_gb300: GB300-native (sm_103a) block-sparse U(1) tensor contractions for the 2-site DMRG
hot path of amiragha/mps.

The compute lives in ``libmpsgb300.so`` (hand-written CUDA + a C++ sector planner, C ABI in
``include/mpsgb300.h``).  This package is the host-side mirror of the reference's SymTensors /
TensorNetAlgs API on top of that library.
"""
from . import _lib
from .symtensors import *  # noqa: F401,F403
from .symtensors import __all__ as _st_all

LIB_PATH = _lib.LIB_PATH

__all__ = list(_st_all) + ["LIB_PATH"]
