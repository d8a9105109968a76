"""fgb_random_csr: fsprand's distribution generated on the device
(src/interface/fsparse.jl:173-290).  Each (i, j) is stored independently with
probability p, so nnz is Binomial(m n, p).  Columns within a row are ascending
and distinct, and the values are N(0,1) for F32 and U[0,1) for F64.  The
output depends only on (seed, m, n, p).  The distribution checks use 6-sigma
bounds."""
import ctypes

import numpy as np
import pytest
import torch

from finchgb import _lib as L
from finchgb import device as dev
from finchgb.server import random_csr

pytestmark = pytest.mark.gpu


def host(A):
    torch.cuda.synchronize()
    return A.ptr.cpu().numpy().astype(np.int64), A.idx.cpu().numpy(), A.val.cpu().numpy()


def test_same_seed_same_matrix_other_seed_other_matrix(gpu_lib):
    a, b, c = (host(random_csr(s, 700, 900, 0.01)) for s in (5, 5, 6))
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not (np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1]))


@pytest.mark.parametrize("m,n,p", [(2000, 3000, 0.004), (50, 100_000, 0.001), (1, 1, 0.5), (300, 200, 0.0)])
def test_structure_and_count(gpu_lib, m, n, p):
    ptr, idx, val = host(random_csr(11, m, n, p))
    assert ptr[0] == 0 and (np.diff(ptr) >= 0).all() and ptr[-1] == idx.size == val.size
    assert idx.size == 0 or (idx.min() >= 0 and idx.max() < n)
    rows = np.repeat(np.arange(m), np.diff(ptr))
    keys = rows * n + idx
    assert (np.diff(keys) > 0).all()  # ascending and distinct within every row
    mean, sd = m * n * p, np.sqrt(m * n * p * (1 - p))
    assert abs(idx.size - mean) <= 6 * sd + 1


def test_positions_and_values_follow_the_distribution(gpu_lib):
    m, n, p = 4000, 4000, 0.005
    ptr, idx, val = host(random_csr(21, m, n, p))
    k = idx.size
    # every quarter of the columns and of the rows gets its share of the entries
    for counts in (np.bincount(idx * 4 // n, minlength=4),
                   np.bincount(np.repeat(np.arange(m), np.diff(ptr)) * 4 // m, minlength=4)):
        assert (np.abs(counts - k / 4) <= 6 * np.sqrt(k * 0.25 * 0.75)).all()
    assert abs(val.mean()) <= 6 / np.sqrt(k) and abs(val.var() - 1) <= 6 * np.sqrt(2 / k)
    # F64: U[0,1)
    ctx = dev.context()
    ptr64 = torch.empty(m + 1, dtype=torch.int32, device="cuda")
    nnz = ctypes.c_int64()
    L.call("fgb_random_csr", ctx, 21, m, n, p, L.F64, ptr64.data_ptr(), None, None, ctypes.byref(nnz),
           dev.stream_ptr())
    i64 = torch.empty(nnz.value, dtype=torch.int32, device="cuda")
    v64 = torch.empty(nnz.value, dtype=torch.float64, device="cuda")
    L.call("fgb_random_csr", ctx, 21, m, n, p, L.F64, ptr64.data_ptr(), i64.data_ptr(), v64.data_ptr(),
           ctypes.byref(nnz), dev.stream_ptr())
    torch.cuda.synchronize()
    u = v64.cpu().numpy()
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) <= 6 * np.sqrt(1 / 12 / u.size)
    # the positions do not depend on the value type
    assert np.array_equal(ptr64.cpu().numpy(), ptr) and np.array_equal(i64.cpu().numpy(), idx)
