"""GB300-native fluidLB D2Q9 step for PyLaBolt case dictionaries.

The compute path is ``liblbm_gb300.so`` (hand-written sm_103a CUDA, C-ABI in
include/lbm_gb300.h); :class:`FluidLBM` is the Python host object over it and
:class:`Case` the validated case.
"""
from .config import Case
from .lbm import FluidLBM

__version__ = "0.1.0+gb300"

__all__ = ["Case", "FluidLBM"]
