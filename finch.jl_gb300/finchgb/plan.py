"""Autotuned, graph-captured plans (fgb_plan_*).

    p = Plan.spmm(A, B, C, tune_reps=3)   # search the schedule space, capture
    p.execute()                           # replay the graph (same buffers)

The plan binds the operand buffers given at creation; refresh their
contents in place and execute again.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L
from . import device as dev


class Plan:
    def __init__(self, desc: L.FgbPlanDesc, A: dev.DeviceSparse, keep: tuple, tune_reps: int):
        self._A_desc = A.desc()
        desc.A = ctypes.addressof(self._A_desc)
        self._keep = keep  # the bound buffers stay alive with the plan
        h = ctypes.c_void_p()
        L.call("fgb_plan_create", dev.context(), ctypes.byref(desc), tune_reps, ctypes.byref(h))
        self.h = h

    @classmethod
    def spmv(cls, A, x, y, semiring=L.PLUS_TIMES, flags=0, tune_reps=5):
        d = L.FgbPlanDesc(0, semiring, dev.dtype_code(x), flags, None, x.data_ptr(), None,
                          y.data_ptr(), 0, 0, 0, 0)
        return cls(d, A, (A, x, y), tune_reps)

    @classmethod
    def spmm(cls, A, B, C, flags=0, tune_reps=3):
        d = L.FgbPlanDesc(1, 0, dev.dtype_code(B), flags, None, B.data_ptr(), None, C.data_ptr(),
                          B.stride(0), 0, C.stride(0), B.shape[1])
        return cls(d, A, (A, B, C), tune_reps)

    @classmethod
    def sddmm(cls, A, X, Y, out, flags=0, tune_reps=3):
        d = L.FgbPlanDesc(2, 0, dev.dtype_code(X), flags, None, X.data_ptr(), Y.data_ptr(),
                          out.data_ptr(), X.stride(0), Y.stride(0), 0, X.shape[1])
        return cls(d, A, (A, X, Y, out), tune_reps)

    def execute(self):
        L.call("fgb_plan_execute", self.h, dev.stream_ptr())

    def info(self) -> dict:
        i = L.FgbPlanInfo()
        L.call("fgb_plan_info_get", self.h, ctypes.byref(i))
        return {f: getattr(i, f) for f, _ in L.FgbPlanInfo._fields_ if f != "reserved"}

    def close(self):
        if getattr(self, "h", None):
            L.call("fgb_plan_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
