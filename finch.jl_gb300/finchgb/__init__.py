"""finchgb -- GB300 (sm_103a) execution backend for Finch.jl's sparse loop nests.

Finch-facing API (mirrors Finch.jl names):
  levels     Dense, SparseList, SparseCOO, Element, Pattern
  tensors    Tensor, swizzle, csr, fsparse, fsprand, transfer, gpu
  fileio     fread, fwrite (.bspnpy, .mtx/.ttx, .tns)
  front ends einsum (@einsum), lazy/compute, finch (@finch programs),
             tensordot, reduce, permutedims, broadcast, minimum, maximum
  scheduler  GB300Scheduler, set_scheduler, with_scheduler, Scalar
Lower layers:
  _lib       ctypes binding of libfinchgb.so (the C ABI of include/finchgb.h)
  device     device-resident level buffers + the kernel calls
  workloads  seeded synthetic inputs in Finch's level layout
"""
from . import _lib
from ._lib import FinchGBError
from .algebra import AbstractAlgebra, DefaultAlgebra
from .fileio import FinchExtensionError, fread, fwrite
from .device import DeviceSparse, context, ewise, ewise_reduce, sddmm, spmm, spmv
from .logic import LazyTensor, broadcast, lazy, maximum, minimum, permutedims, reduce, tensordot
from .scheduler import (FinchGBUnsupported, GB300Scheduler, Scalar, compute, default_scheduler,
                        einsum, finch, get_scheduler, set_scheduler, with_scheduler)
from .tensors import (GPU, Dense, Element, Pattern, SparseByteMap, SparseCOO, SparseList, SwizzleArray,
                      Tensor, csr, fsparse, fsprand, gpu, isequal, pattern, set_fill_value, sparse, swizzle,
                      transfer)
from .galley import GalleyScheduler, galley_scheduler

__all__ = [
    "SparseByteMap", "pattern", "set_fill_value", "AbstractAlgebra", "DefaultAlgebra",
    "FinchGBError", "FinchGBUnsupported", "DeviceSparse", "context", "spmv", "spmm", "sddmm",
    "ewise", "ewise_reduce", "LazyTensor", "lazy", "compute", "einsum", "finch", "tensordot",
    "reduce", "permutedims", "broadcast", "minimum", "maximum", "GB300Scheduler", "Scalar",
    "default_scheduler", "get_scheduler", "set_scheduler", "with_scheduler", "GPU", "Dense",
    "Element", "Pattern", "SparseCOO", "SparseList", "SwizzleArray", "Tensor", "csr", "fsparse", "fsprand", "fread", "fwrite", "FinchExtensionError",
    "gpu", "isequal", "sparse", "swizzle", "transfer", "_lib", "GalleyScheduler", "galley_scheduler",
]
