"""reduce(max | min, A; dims) -- maximum(A; dims), minimum(A; dims),
`y[j] <<max>>= A[i,j]` -- on the GPU against the oracle, which folds every
(i, j) in Finch's order with @fastmath's first-operand max/min: bit for
bit (NaN and signed zeros compared by their bits) for every fill, value
type, storage and dims."""
import numpy as np
import pytest
import torch

import finchgb as F
import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import fsprand

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def matrix(rng, m, n, p, dt, special=False):
    g = fsprand(rng, m, n, p)
    if np.dtype(dt).kind == "i":
        g.val = rng.integers(-50, 50, g.nnz).astype(dt)
    else:
        v = rng.standard_normal(g.nnz)
        if special:  # NaN and both zeros among the stored values
            k = rng.choice(g.nnz, min(g.nnz, 12), replace=False)
            v[k[:4]] = np.nan
            v[k[4:8]] = 0.0
            v[k[8:]] = -0.0
        g.val = v.astype(dt)
    return g


@pytest.mark.parametrize("dt", [np.float64, np.float32, np.int64, np.int32])
@pytest.mark.parametrize("op", ["max", "min"])
def test_reduce_minmax_all_fills_dims_storages(gpu_lib, dt, op):
    rng = np.random.default_rng(5)
    m, n = 150, 120
    fills = [0, 7] if np.dtype(dt).kind == "i" else [0.0, -np.inf, np.inf, 1.5, -0.0]
    for fill in fills:
        for p in (0.05, 0.6):
            g = matrix(rng, m, n, p, dt, special=np.dtype(dt).kind == "f")
            fmt = F.Dense(F.SparseList(F.Element(np.asarray(fill, dt)[()])))
            t = F.Tensor.from_buffers(fmt, g)
            for dims in (1, 2, None):
                got = (t.maximum(dims=dims) if op == "max" else t.minimum(dims=dims))
                got = np.atleast_1d(got.todense() if hasattr(got, "todense") else got.value)
                want = oracle.reduce_minmax(op == "max", {1: 1, 2: 2, None: 0}[dims], m, n, g.ptr, g.idx,
                                            g.val.astype(np.float64), float(fill))
                if np.dtype(dt).kind == "i":
                    assert np.array_equal(got.astype(np.int64), want.astype(np.int64)), (fill, p, dims)
                else:
                    assert bits_equal(got.astype(np.float64), want), (fill, p, dims)


def test_reduce_minmax_through_einsum_and_csr(gpu_lib):
    rng = np.random.default_rng(6)
    g = matrix(rng, 90, 70, 0.1, np.float64)
    t = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))), g)
    y = F.einsum("y[j] <<max>>= A[i,j]", A=t).todense()
    assert bits_equal(y, oracle.reduce_minmax(True, 1, 90, 70, g.ptr, g.idx, g.val, 0.0))
    y = F.einsum("y[i] <<min>>= A[i,j]", A=t).todense()
    assert bits_equal(y, oracle.reduce_minmax(False, 2, 90, 70, g.ptr, g.idx, g.val, 0.0))
    # the same matrix handed over as CSR: maximum over rows needs the transposed storage
    D = t.todense()
    r = F.csr(D)
    assert bits_equal(r.maximum(dims=1).todense(), oracle.reduce_minmax(True, 1, 90, 70, g.ptr, g.idx, g.val, 0.0))
    assert bits_equal(r.minimum(dims=2).todense(), oracle.reduce_minmax(False, 2, 90, 70, g.ptr, g.idx, g.val, 0.0))


def test_reduce_minmax_edges(gpu_lib):
    # a matrix that stores nothing: every output is the fill
    e = F.Tensor(F.Dense(F.SparseList(F.Element(2.5))), shape=(4, 3))
    assert e.maximum(dims=1).todense().tolist() == [2.5] * 3 and e.minimum().value == 2.5
    # a full column: the fill does not take part
    D = np.array([[1.0, 0.0], [3.0, 0.0], [2.0, -1.0]])
    t = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), D)
    assert t.maximum(dims=1).todense().tolist() == [3.0, 0.0]
    assert t.minimum(dims=1).todense().tolist() == [1.0, -1.0]
    assert t.maximum().value == 3.0 and t.minimum().value == -1.0
    # the library refuses the reduction against the storage's orientation
    b = t.host_buffers()
    A = dev.DeviceSparse.from_host(3, 2, b.ptr, b.idx, b.val, orient="csc", base=b.base)
    with pytest.raises(L.FinchGBError):
        dev.reduce_minmax(L.MAP_MAX, 2, A, 0.0)
    y = dev.reduce_minmax(L.MAP_MAX, 1, A, 0.0, init=10.0)
    assert y.cpu().tolist() == [10.0, 10.0]  # the fold starts from init
