"""The int64 ptr layout, which a SparseList level with 2^31 or more stored
entries needs, gives the same bits as the int32 layout of the same matrix in
every kernel. Covered: SpMV in both orientations, SpMM's merge-path and
virtual-row schedules, SDDMM, SpGEMM, elementwise merges, elementwise+reduce
and the transpose."""
import numpy as np
import pytest
import torch

from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import zipf_csr
from helpers import upload

pytestmark = pytest.mark.gpu


def ptr64(A: dev.DeviceSparse) -> dev.DeviceSparse:
    return dev.DeviceSparse(A.nrows, A.ncols, A.ptr.to(torch.int64), A.idx, A.val, A.orient, A.base)


@pytest.fixture(scope="module")
def mats():
    rng = np.random.default_rng(64)
    a = zipf_csr(rng, 6000, 5000, mean=12.0, a=1.5, cap=3000, dtype=np.float32)
    b = zipf_csr(rng, 6000, 5000, mean=12.0, a=1.5, cap=3000, dtype=np.float32)
    A, Bm = upload(a), upload(b)
    assert A.ptr.dtype == torch.int32
    return A, Bm


def same(x, y):
    torch.cuda.synchronize()
    return torch.equal(x, y)


def test_spmv_both_orientations(gpu_lib, mats):
    A, _ = mats
    x = torch.randn(A.ncols, device="cuda")
    assert same(dev.spmv(A, x), dev.spmv(ptr64(A), x))
    # CSC: the push kernel adds into y with atomics, so float sums land in any
    # order; small integer values make every order exact
    At = A.transposed_storage()
    Atq = dev.DeviceSparse(At.nrows, At.ncols, At.ptr, At.idx, torch.round(At.val * 4), At.orient, At.base)
    xt = torch.randint(-8, 9, (At.ncols,), device="cuda").to(torch.float32)
    assert same(dev.spmv(Atq, xt), dev.spmv(ptr64(Atq), xt))
    xi = torch.randint(0, 100, (A.ncols,), dtype=torch.int32, device="cuda")
    Ai = dev.DeviceSparse(A.nrows, A.ncols, A.ptr, A.idx, (A.val * 10).to(torch.int32), A.orient, A.base)
    assert same(dev.spmv(Ai, xi, semiring=L.MIN_PLUS), dev.spmv(ptr64(Ai), xi, semiring=L.MIN_PLUS))


@pytest.mark.parametrize("kw", [{}, {"lanes": 8, "path": 128, "variant": 2},
                                {"lanes": 8, "path": 128, "variant": 3}, {"lanes": 4, "path": 256}])
def test_spmm_schedules(gpu_lib, mats, kw):
    A, _ = mats
    B = torch.randn((A.ncols, 64), device="cuda")
    assert same(dev.spmm(A, B, **kw), dev.spmm(ptr64(A), B, **kw))


@pytest.mark.parametrize("kw", [{}, {"variant": 2, "chunk": 64}, {"lanes": 8, "chunk": 128}])
def test_sddmm(gpu_lib, mats, kw):
    A, _ = mats
    X = torch.randn((A.nrows, 32), device="cuda")
    Y = torch.randn((A.ncols, 32), device="cuda")
    assert same(dev.sddmm(A, X, Y, **kw), dev.sddmm(ptr64(A), X, Y, **kw))


def test_spgemm_merges_reduce_transpose(gpu_lib, mats):
    A, Bm = mats
    A64 = dev.DeviceSparse(A.nrows, A.ncols, A.ptr, A.idx, A.val.double(), A.orient, A.base)
    At64 = A64.transposed_storage()
    AtT = dev.DeviceSparse(At64.ncols, At64.nrows, At64.ptr, At64.idx, At64.val, "csr", At64.base)
    C32 = dev.spgemm(A64, AtT)
    C64 = dev.spgemm(ptr64(A64), ptr64(AtT))
    torch.cuda.synchronize()
    assert torch.equal(C32.ptr.to(torch.int64), C64.ptr.to(torch.int64))
    assert torch.equal(C32.idx, C64.idx) and torch.equal(C32.val, C64.val)
    for op in (L.EW_MUL, L.EW_ADD):
        E32, E64 = dev.ewise(op, A, Bm), dev.ewise(op, ptr64(A), ptr64(Bm))
        torch.cuda.synchronize()
        assert torch.equal(E32.ptr, E64.ptr) and torch.equal(E32.idx, E64.idx)
        assert torch.equal(E32.val, E64.val)
    for dims in (0, 1, 2):
        assert same(dev.ewise_reduce(dims, A, Bm), dev.ewise_reduce(dims, ptr64(A), ptr64(Bm)))
    T32, T64 = A.transposed_storage(), ptr64(A).transposed_storage()
    torch.cuda.synchronize()
    assert torch.equal(T32.ptr.to(torch.int64), T64.ptr.to(torch.int64))
    assert torch.equal(T32.idx, T64.idx) and torch.equal(T32.val, T64.val)
