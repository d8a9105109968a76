"""Shared helpers for the GPU parity tests: upload host level buffers,
compute oracle results, and compare with a stated tolerance."""
from __future__ import annotations

import numpy as np
import torch

import oracle
from finchgb import device as dev
from finchgb.workloads import SparseBuffers

# Float tolerances: |gpu - oracle| <= RTOL * sum_j |A[i,j] * x[j]| (+ tiny atol).
# Summation order differs (lane-parallel reductions, atomics), so the bound
# scales with the magnitude of the summed terms, not the result.
RTOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 2e-5}


def upload(b: SparseBuffers, val_dtype=None, as_bf16=False) -> dev.DeviceSparse:
    vd = torch.bfloat16 if as_bf16 else val_dtype
    return dev.DeviceSparse.from_host(b.nrows, b.ncols, b.ptr, b.idx, b.val, orient=b.orient,
                                      base=1, val_dtype=vd)


def to_dev(a: np.ndarray) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype == torch.bool:
        t = t.to(torch.uint8)
    return t.cuda()


def to_host(t: torch.Tensor) -> np.ndarray:
    torch.cuda.synchronize()
    return t.cpu().numpy()


def oracle_spmv(sr, b: SparseBuffers, x, fma=True, bf16=False):
    """Finch's nest for b's orientation (CSC serial, or CSR row pull)."""
    val = b.val
    if bf16:
        val = bf16_bits(val)
    if b.orient == "csc":
        return oracle.spmv_csc(sr, b.nrows, b.ncols, b.ptr, b.idx, val, x, fma=fma, bf16=bf16)
    return oracle.spmv_csr(sr, b.nrows, b.ncols, b.ptr, b.idx, val, x, fma=fma, bf16=bf16)


def abs_terms(b: SparseBuffers, x):
    """sum_j |A[i,j] x[j]| per output, for the float tolerance bound."""
    bb = SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, np.abs(b.val).astype(np.float64), b.orient)
    return oracle_spmv(0, bb, np.abs(np.asarray(x, dtype=np.float64)))


def bf16_bits(v: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even bf16 bit patterns of float values (via torch)."""
    t = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float32)).to(torch.bfloat16)
    return t.view(torch.int16).numpy().view(np.uint16)


def assert_close(got, want, scale, dtype):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    tol = RTOL[np.dtype(dtype)] * np.asarray(scale, dtype=np.float64) + 1e-30
    bad = np.abs(got - want) > tol
    assert not bad.any(), (f"{int(bad.sum())} of {bad.size} outside tolerance; first at "
                           f"{np.flatnonzero(bad)[:5]}: got {got[bad][:5]} want {want[bad][:5]}")
