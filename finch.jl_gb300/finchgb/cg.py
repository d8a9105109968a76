"""Conjugate gradients, two ways.

`cg_solve` runs the native mixed-precision solver (fgb_cg_solve): the
iteration SpMV reads FP32 or BF16 values and sums them in FP32, in FP64, or
-- with the whole iteration -- in pairs of FP32 numbers (about 48 bits, no
FP64 arithmetic per row: the fast mode on GB300, whose FP64 rate is a small
fraction of its FP32 rate); FP64 reliable updates of the residual bring the
true residual to rtol, and chunks of iterations replay as CUDA graphs.

`cg_finch` is the same algorithm written as Finch programs -- every step is an
`@einsum` matched onto a kernel by the GB300 scheduler -- for readability and
as a cross-check; it launches one kernel per step from the host.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from . import device as dev

PRECISIONS = {"f64": L.F64, "f32": L.F32, "bf16": L.BF16}
ACCUMULATE = {"f32": 0, "f64": 1, "pair": 2, "spmv_pair": 3}  # FGB_CG_SUM_F32, _F64, _PAIR, _SPMV_PAIR


@dataclass
class CGResult:
    iterations: int
    replacements: int
    true_rel_residual: float
    seconds: float
    converged: bool
    compact_index: bool = False


def low_precision_copy(A: dev.DeviceSparse, precision: str) -> dev.DeviceSparse:
    """Same pattern as A with values stored as FP32 or BF16."""
    t = {"f32": torch.float32, "bf16": torch.bfloat16}[precision]
    return dev.DeviceSparse(A.nrows, A.ncols, A.ptr, A.idx, A.val.to(t), A.orient, A.base)


def cg_solve(A64: dev.DeviceSparse, b: torch.Tensor, x: torch.Tensor | None = None,
             precision: str = "f32", rtol: float = 1e-10, max_iter: int = 100_000,
             chunk: int = 64, replace_every: int = 512, Alow: dev.DeviceSparse | None = None,
             accumulate: str = "f32") -> tuple[torch.Tensor, CGResult]:
    """Solves A x = b (A SPD, CSR, FP64 values); returns (x, result).
    precision: the stored values of the iteration SpMV (f64, f32, bf16);
    accumulate: the arithmetic for f32/bf16 values: "f32" (FP32 SpMV sums),
    "f64" (values widened, FP64 sums), "spmv_pair" (SpMV sums as pairs of FP32
    numbers, vectors, dots and updates FP64) or "pair" (pairs of FP32 numbers
    for the SpMV sums, vectors, dots and updates)."""
    if A64.orient != "csr":
        raise ValueError("cg_solve needs a CSR matrix")
    if x is None:
        x = torch.zeros_like(b)
    prec = PRECISIONS[precision]
    if prec != L.F64 and Alow is None:
        Alow = low_precision_copy(A64, precision)
    opts = L.FgbCgOptions(rtol, max_iter, chunk, prec, replace_every, ACCUMULATE[accumulate], 0)
    res = L.FgbCgResult()
    da = A64.desc()
    dl = None if prec == L.F64 else ctypes.byref(Alow.desc())
    L.call("fgb_cg_solve", dev.context(b.device.index), ctypes.byref(da), dl, b.data_ptr(),
           x.data_ptr(), ctypes.byref(opts), ctypes.byref(res), dev.stream_ptr())
    return x, CGResult(res.iterations, res.replacements, res.true_rel_residual, res.seconds,
                       bool(res.converged), bool(res.compact_index))


def cg_finch(A, b, rtol: float = 1e-10, max_iter: int = 10_000):
    """CG written as Finch programs (each line one matched @einsum).

    A: a Finch Tensor (Dense(SparseList(Element))); b: a Dense vector
    Tensor.  Returns (x, iterations)."""
    from .scheduler import einsum
    from .tensors import Dense, Element, Tensor

    n = b.shape[0]
    x = Tensor(Dense(Element(0.0)), np.zeros(n))
    r = einsum("r[i] = b[i] - q[i]", b=b, q=einsum("q[i] += A[i,j] * x[j]", A=A, x=x))
    p = einsum("p[i] = r[i] + z[i]", r=r, z=Tensor(Dense(Element(0.0)), np.zeros(n)))
    rr = einsum("s[] += r[i] * r[i]", r=r)
    bb = einsum("s[] += b[i] * b[i]", b=b).value
    it = 0
    while it < max_iter and rr.value > (rtol ** 2) * bb:
        q = einsum("q[i] += A[i,j] * p[j]", A=A, p=p)
        pq = einsum("s[] += p[i] * q[i]", p=p, q=q)
        alpha = einsum("a[] = rr[] / pq[]", rr=rr, pq=pq)
        x = einsum("x[i] = x[i] + alpha[] * p[i]", x=x, alpha=alpha, p=p)
        r = einsum("r[i] = r[i] - alpha[] * q[i]", r=r, alpha=alpha, q=q)
        rr_new = einsum("s[] += r[i] * r[i]", r=r)
        beta = einsum("b[] = n[] / o[]", n=rr_new, o=rr)
        p = einsum("p[i] = r[i] + beta[] * p[i]", r=r, beta=beta, p=p)
        rr = rr_new
        it += 1
    return x, it
