"""Empty and ragged inputs across the kernels: matrices without stored
entries, with empty rows and columns, with zero rows, single entries, and
dense widths that leave lanes of a slab unused -- against the oracle (exact
for integer and Bool semirings and for sums in a fixed order)."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.plan import Plan
from finchgb.workloads import SparseBuffers, csc_from_dense, csr_from_dense
from helpers import RTOL, oracle_spmv, to_dev, to_host, upload

pytestmark = pytest.mark.gpu


def csr(D, dtype=np.float64):
    b = csr_from_dense(np.asarray(D, dtype=np.float64))
    b.val = b.val.astype(dtype)
    return b


def empty_csr(m, n, dtype=np.float64):
    return SparseBuffers(m, n, np.ones(m + 1, np.int64), np.zeros(0, np.int64), np.zeros(0, dtype), "csr")


def ragged(m, n, seed, dtype=np.float64):
    """Rows of very different lengths, some empty, one dense, empty columns."""
    rng = np.random.default_rng(seed)
    D = np.zeros((m, n))
    for i in range(m):
        k = [0, 0, 1, 3, n // 2][i % 5]
        cols = rng.choice(n - 2, size=min(k, n - 2), replace=False)  # the last 2 columns stay empty
        D[i, cols] = rng.integers(1, 9, size=cols.size)
    D[m // 2, : n - 2] = rng.integers(1, 9, size=n - 2)
    return D.astype(dtype)


@pytest.mark.parametrize("shape", [(0, 5), (6, 0), (7, 4)])
def test_spgemm_with_empty_operands(gpu_lib, shape):
    m, k = shape
    A = upload(empty_csr(m, k)) if k == 0 or m == 0 else upload(csr(ragged(m, k, 1)))
    B = upload(empty_csr(k, 9))
    C = dev.spgemm(A, B)
    ptr, idx, val = C.to_host()
    assert C.nnz == 0 and ptr.size == m + 1 and (ptr == 1).all()


def test_spgemm_ragged_exact(gpu_lib):
    Da, Db = ragged(40, 30, 2), ragged(30, 25, 3)
    a, b = csr(Da), csr(Db)
    C = dev.spgemm(upload(a), upload(b))
    want = oracle.spgemm_csr(a.nrows, b.ncols, a.ptr, a.idx, a.val, b.ptr, b.idx, b.val)
    ptr, idx, val = C.to_host()
    assert np.array_equal(ptr, want[0]) and np.array_equal(idx, want[1]) and np.array_equal(val, want[2])
    assert np.array_equal(C.to_host()[0][-1] - 1, (Da @ Db != 0).sum())


@pytest.mark.parametrize("orient", ["csr", "csc"])
def test_semirings_over_empty_rows_and_columns(gpu_lib, orient):
    D = ragged(33, 20, 4)
    b = csr_from_dense(D) if orient == "csr" else csc_from_dense(D)
    bi = SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, b.val.astype(np.int32), b.orient)
    x = np.arange(20, dtype=np.int32) * 3 - 7
    A = upload(bi)
    for sr, srp in ((L.MIN_PLUS, oracle.SR_MINP), (L.MAX_PLUS, oracle.SR_MAXP), (L.PLUS_TIMES, 0)):
        y = to_host(dev.spmv(A, to_dev(x), semiring=sr))
        assert np.array_equal(y, oracle_spmv(srp, bi, x)), sr
    bp = SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, None, b.orient)
    xb = (np.arange(20) % 3 == 0).astype(np.uint8)
    yb = to_host(dev.spmv(upload(bp), to_dev(xb), semiring=L.OR_AND))
    assert np.array_equal(yb, oracle_spmv(oracle.SR_OA, bp, xb))


def test_sddmm_without_entries_every_variant(gpu_lib):
    A = upload(empty_csr(50, 40, np.float32))
    X = torch.randn((50, 16), device="cuda")
    Y = torch.randn((40, 16), device="cuda")
    for kw in ({}, {"variant": 1, "chunk": 64}, {"variant": 2, "chunk": 64}, {"lanes": 8, "chunk": 128}):
        out = dev.sddmm(A, X, Y, **kw)
        assert out.numel() == 0


@pytest.mark.parametrize("nk", [4, 8, 12, 40])
@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_slab_spmm_narrow_widths(gpu_lib, nk, lanes):
    """k below or not a multiple of the slab: masked lanes, a partial last slab."""
    D = ragged(90, 70, 5, np.float32)
    b = csr(D, np.float32)
    B = np.random.default_rng(6).standard_normal((70, nk)).astype(np.float32)
    want = D.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(D).astype(np.float64) @ np.abs(B).astype(np.float64)
    A = upload(b)
    for variant in (2, 3):
        C = to_host(dev.spmm(A, to_dev(B), lanes=lanes, path=8, variant=variant))
        assert (np.abs(C - want) <= RTOL[np.dtype(np.float32)] * scale + 1e-30).all()


def test_plans_on_a_single_entry(gpu_lib):
    b = csr([[2.5]])
    A = upload(b)
    x = to_dev(np.array([4.0]))
    y = torch.empty(1, dtype=torch.float64, device="cuda")
    p = Plan.spmv(A, x, y, tune_reps=1)
    p.execute()
    assert to_host(y)[0] == 10.0
    bf = csr([[2.5]], np.float32)
    Af = upload(bf)
    B = to_dev(np.full((1, 8), 2.0, np.float32))
    C = torch.empty((1, 8), dtype=torch.float32, device="cuda")
    Plan.spmm(Af, B, C, tune_reps=1).execute()
    assert (to_host(C) == 5.0).all()


def test_spmv_zero_by_zero(gpu_lib):
    A = upload(empty_csr(0, 0))
    y = dev.spmv(A, torch.empty(0, dtype=torch.float64, device="cuda"))
    assert y.numel() == 0
