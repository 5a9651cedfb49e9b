"""minimmerflow_gb300: GB300-native (sm_103a) finite-volume compressible-Euler step.

Hot path of optimad/minimmerflow (reconstruction, LLF interface flux and
residual, SSP-RK3 stage update, CFL time step) as hand-written CUDA behind a
C ABI (include/mmf_gb300.h).  Python modules here are the host-side mirror of
the reference's entry points; the arithmetic runs only on the GPU.
"""
from . import capi, problem, settings
from ._build import build as build_library
from .solver import CartesianEuler

__all__ = ["capi", "problem", "build_library", "CartesianEuler"]
