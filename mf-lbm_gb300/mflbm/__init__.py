"""mflbm -- host-side interface of the GB300 MF-LBM step library (libmflbm.so).

Submodules:
  _capi     ctypes binding of include/mflbm.h
  solver    Solver: one device context, methods mirroring the C ABI
  geometry  wall arrays, boundary-node lists, inlet profile, synthetic media, file formats
  deck      simulation_control.txt parsing into run parameters
"""
from ._capi import (MFLBM_FP16, MFLBM_FP32, MFLBM_FP64, MFLBM_FP64FF, MFLBM_FF, MFLBM_FAILED, MFLBM_RUNNING, MflbmError, Params, load)
from .solver import Solver, make_params

__all__ = ["Solver", "make_params", "Params", "MflbmError", "load", "MFLBM_FP64", "MFLBM_FP32", "MFLBM_FP16", "MFLBM_FP64FF", "MFLBM_FF",
           "MFLBM_FAILED", "MFLBM_RUNNING"]
