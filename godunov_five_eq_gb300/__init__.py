"""GB300-native (sm_103a) block timestep of the two-material five-equation
Godunov solver, a drop-in for kalypsso-dev/godunov_five_eq's
GodunovImplemBase (per-block ConvertToPrimitives -> limited slopes ->
MUSCL-Hancock / THINC -> HLLC -> conservative update -> volume-fraction
renormalisation -> CFL reduction, fused in one CUDA kernel).

The C ABI is include/g5gpu.h (libg5gpu.so); `GodunovImplemGB300` is the
Python host mirror of the reference interface.
"""
from .implem import G5_MODE_FP64, G5_MODE_MIXED, G5Error, GodunovImplemGB300, gpu_flag_fn, load_library  # noqa: F401

__all__ = ["GodunovImplemGB300", "G5Error", "G5_MODE_FP64", "G5_MODE_MIXED", "gpu_flag_fn", "load_library"]
