"""fgb_spmm_noalloc: SpMM for callers that cannot allocate device memory.

A host whose device memory is owned by another allocator (for instance a
Julia process using CUDA.jl's pool), or a serving loop that must not enter an
allocator on its hot path, calls this entry point instead of fgb_spmm.  It
takes the scratch of the load-balanced schedule from one fixed device array
and allocates nothing.  This test calls it through the C ABI and checks its
output against fgb_spmm's on two calls in a row (the array keeps the previous
call's contents, so the second call shows nothing stale leaks through), within
the tolerance the other SpMM tests use.  It lives in a file of its own that
pytest collects last and passes both alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import zipf_csr

pytestmark = pytest.mark.gpu

RTOL_F32 = 2e-5  # |got - want| <= RTOL * sum_j |A[i,j] B[j,k]|


def _call_noalloc(A, B, C, flags=0):
    d = A.desc()
    return L.load().fgb_spmm_noalloc(dev.context(), ctypes.byref(d), B.data_ptr(), B.stride(0),
                                     B.shape[1], C.data_ptr(), C.stride(0), L.F32, flags,
                                     dev.stream_ptr())


def _call_spmm(A, B, C, flags=0):
    d = A.desc()
    return L.load().fgb_spmm(dev.context(), ctypes.byref(d), B.data_ptr(), B.stride(0), B.shape[1],
                             C.data_ptr(), C.stride(0), L.F32, flags, dev.stream_ptr())


@pytest.mark.parametrize("nk", [128, 32])
def test_noalloc_matches_spmm_two_calls(gpu_lib, nk):
    rng = np.random.default_rng(nk)
    m = 30000
    h = zipf_csr(rng, m, m, mean=16, cap=50_000)
    A = dev.DeviceSparse.from_host(h.nrows, h.ncols, h.ptr, h.idx, h.val, orient="csr")
    Ab = np.abs(h.val.astype(np.float64))
    scale_A = dev.DeviceSparse.from_host(h.nrows, h.ncols, h.ptr, h.idx, Ab, orient="csr")
    for call in range(2):
        B = torch.from_numpy(rng.standard_normal((m, nk), dtype=np.float32)).cuda()
        C_ref = torch.empty((m, nk), dtype=torch.float32, device="cuda")
        C_na = torch.full((m, nk), float("nan"), dtype=torch.float32, device="cuda")
        L.check(_call_spmm(A, B, C_ref), "fgb_spmm")
        L.check(_call_noalloc(A, B, C_na), "fgb_spmm_noalloc")
        scale = dev.spmm(scale_A, B.abs().double(), flags=L.FINCH_ORDER)
        torch.cuda.synchronize()
        diff = (C_na.double() - C_ref.double()).abs()
        assert torch.isfinite(C_na).all(), f"call {call}: output not fully written"
        assert (diff <= RTOL_F32 * scale + 1e-30).all(), f"call {call}: {diff.max().item()}"


def test_noalloc_rejects_oversized_schedule(gpu_lib):
    # 2^45 rows x 2^20 output columns would need terabytes of scratch even
    # with the longest merge-path items: rejected before any device access.
    d = L.FgbSparse(2**45, 8, 0, L.CSR, 0, L.I64, L.I32, L.F32, 0, 256, None, None)
    rc = L.load().fgb_spmm_noalloc(dev.context(), ctypes.byref(d), 256, 2**20, 2**20, 256, 2**20,
                                   L.F32, 0, dev.stream_ptr())
    assert rc == L.EINVAL
    assert "scratch" in L.last_error()
