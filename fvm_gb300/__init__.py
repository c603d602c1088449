"""GB300 (sm_103a) time step of the fractional 4-step incompressible Navier-Stokes
finite-volume solver on a cylinder O-grid.

The compute path is the CUDA library behind include/fvm.h; fvm_gb300.capi is its
ctypes binding and fvm_gb300.grid generates the O-grid cases.
"""
from . import grid  # noqa: F401

__all__ = ["grid", "capi", "build"]
