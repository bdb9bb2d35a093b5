"""sucrose_gb300: the SUCROSE molecular-dynamics hot path on one GB300 (sm_103a).

Pair forces (LJ, WCA, Gay-Berne, ECP), the Verlet list and the VV / quaternion /
Langevin / Nose-Hoover updates run as hand-written CUDA kernels behind the C ABI
in include/sucrose_gpu.h; this package is the Python host mirror of it.
"""
from . import capi
from .capi import SgError
from .system import GpuSystem

__all__ = ["capi", "SgError", "GpuSystem"]
