"""GB300-native GFM combustion-space SIMPLER solver.

Public pieces: ``configs`` (synthetic furnace cases), ``Case`` (host start-up
in the reference layout), ``GpuSolver`` (the CUDA path behind the C ABI of
include/gfm_gb300.h).  There is no CPU execution path: every solver call runs
on the GPU and fails loudly when the native library or the device is absent.
"""
from . import abi, configs
from .solver import Case, Fields, GfmError, GpuSolver

__all__ = ["abi", "configs", "Case", "Fields", "GfmError", "GpuSolver"]
