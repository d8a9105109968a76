"""finchgb -- GB300 (sm_103a) execution backend for Finch.jl's sparse loop nests.

Layers:
  _lib       ctypes binding of libfinchgb.so (the C ABI of include/finchgb.h)
  device     device-resident level buffers + the kernel calls
  workloads  seeded synthetic inputs in Finch's level layout
"""
from . import _lib
from ._lib import FinchGBError
from .device import DeviceSparse, context, ewise, ewise_reduce, sddmm, spmm, spmv

__all__ = ["FinchGBError", "DeviceSparse", "context", "spmv", "spmm", "sddmm", "ewise",
           "ewise_reduce", "_lib"]
