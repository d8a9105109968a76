"""scipy.sparse matrices on the GPU path: Tensor(A) keeps scipy's 0-based
int32 (or int64) buffers, which reach the kernels as index base 0, so a
scipy CSC or CSR (through swizzle(Tensor(A.T), 2, 1)) runs the same kernels
as Finch's own 1-based Int64 buffers.  Results are checked against the
oracle and, on the headline matrix, against the Finch-buffer route bit for
bit (same kernels, same schedule, same order)."""
import numpy as np
import pytest

import finchgb as F
import oracle
from finchgb.workloads import SparseBuffers, zipf_csr
from helpers import assert_close

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")


def finch_buffers(A):
    """1-based Int64 ptr/idx of a canonical CSC or CSR (for the oracle)."""
    return A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1


def dense2(B):
    return F.Tensor(F.Dense(F.Dense(F.Element(np.zeros((), B.dtype)[()]))), B)


def vec(x):
    return F.Tensor(F.Dense(F.Element(np.zeros((), x.dtype)[()])), x)


@pytest.mark.parametrize("index_dtype", [np.int32, np.int64])
def test_spmv_on_scipy_csc(gpu_lib, index_dtype):
    rng = np.random.default_rng(7)
    A = sp.random(3000, 2000, density=0.004, format="csc", random_state=8)
    A.indices, A.indptr = A.indices.astype(index_dtype), A.indptr.astype(index_dtype)
    x = rng.standard_normal(2000)
    t = F.Tensor(A)
    assert t.buf.base == 0 and t.buf.idx.dtype == index_dtype
    y = F.einsum("y[i] += A[i,j] * x[j]", A=t, x=vec(x))
    assert t.dsparse.base == 0
    ptr, idx = finch_buffers(A)
    want = oracle.spmv_csc(oracle.SR_PT, 3000, 2000, ptr, idx, A.data, x)
    scale = oracle.spmv_csc(oracle.SR_PT, 3000, 2000, ptr, idx, np.abs(A.data), np.abs(x))
    assert_close(y.todense(), want, scale, np.float64)


def test_spmm_on_scipy_csr_and_csc(gpu_lib):
    rng = np.random.default_rng(9)
    R = sp.random(4000, 3000, density=0.003, format="csr", random_state=10, dtype=np.float32)
    B = rng.standard_normal((3000, 40)).astype(np.float32)
    ptr, idx = finch_buffers(R)
    want = oracle.spmm_csr(4000, 3000, ptr, idx, R.data, B)
    scale = oracle.spmm_csr(4000, 3000, ptr, idx, np.abs(R.data).astype(np.float64),
                            np.abs(B).astype(np.float64))
    # CSR without copies: swizzle(Tensor(R^T), 2, 1) over R's own buffers
    A = F.swizzle(F.Tensor(R.T), 2, 1)
    C = F.compute(F.lazy(A) @ F.lazy(dense2(B))).todense()
    assert_close(C, want, scale, np.float32)
    # the same through Finch's 1-based buffers: the same kernels, bit for bit
    At = SparseBuffers(3000, 4000, ptr, idx, R.data, "csc")
    fmt = F.Dense(F.SparseList(F.Element(np.float32(0))))
    C1 = F.compute(F.lazy(F.swizzle(F.Tensor.from_buffers(fmt, At), 2, 1)) @ F.lazy(dense2(B))).todense()
    assert np.array_equal(C, C1)
    # a CSC operand is transposed on the device from its 0-based buffers
    Cc = F.compute(F.lazy(F.Tensor(R.tocsc())) @ F.lazy(dense2(B))).todense()
    assert_close(Cc, want, scale, np.float32)


def test_sddmm_and_reduce_on_scipy(gpu_lib):
    rng = np.random.default_rng(11)
    R = sp.random(500, 400, density=0.02, format="csr", random_state=12)
    D = R.toarray()
    A = F.swizzle(F.Tensor(R.T), 2, 1)
    X = rng.standard_normal((500, 16))
    Y = rng.standard_normal((400, 16))
    S = F.compute(F.lazy(A) * (F.lazy(dense2(X)) @ F.lazy(dense2(Y)).T))
    np.testing.assert_allclose(S.todense(), D * (X @ Y.T), rtol=1e-12, atol=1e-12)
    rs = F.compute(F.lazy(A).sum(dims=2))
    np.testing.assert_allclose(rs.todense(), D.sum(axis=1), rtol=1e-12, atol=1e-12)
    # and back to scipy from the device-resident result
    Sp = F.sparse(S)
    np.testing.assert_allclose(Sp.toarray(), D * (X @ Y.T), rtol=1e-12, atol=1e-12)


def test_headline_matrix_as_scipy_csr(gpu_lib):
    """The 1M x 1M Zipf CSR with 16M entries handed over as a scipy
    csr_matrix: no dense intermediate, and C equals the Finch-buffer
    route's bit for bit."""
    rng = np.random.default_rng(20261203)
    r = zipf_csr(rng, 1_000_000, 1_000_000, mean=16, a=1.5, cap=50_000, dtype=np.float32)
    B = rng.standard_normal((1_000_000, 128), dtype=np.float32)
    R = sp.csr_matrix((r.val, r.idx - 1, r.ptr - 1), shape=(r.nrows, r.ncols))
    assert R.has_canonical_format and R.nnz == 16_000_000
    Bt = dense2(B)
    C = F.compute(F.lazy(F.swizzle(F.Tensor(R.T), 2, 1)) @ F.lazy(Bt)).todense()
    At = SparseBuffers(r.ncols, r.nrows, r.ptr, r.idx, r.val, "csc")
    fmt = F.Dense(F.SparseList(F.Element(np.float32(0))))
    C1 = F.compute(F.lazy(F.swizzle(F.Tensor.from_buffers(fmt, At), 2, 1)) @ F.lazy(Bt)).todense()
    assert C.shape == (1_000_000, 128) and np.array_equal(C, C1)
    rows = np.r_[np.argsort(np.diff(r.ptr))[-8:], rng.integers(0, r.nrows, 500)]
    for i in rows:  # sampled rows against FP64 (the whole product is checked in the full-size tests)
        a, b = r.ptr[i] - 1, r.ptr[i + 1] - 1
        want = r.val[a:b].astype(np.float64) @ B[r.idx[a:b] - 1].astype(np.float64)
        scale = np.abs(r.val[a:b]).astype(np.float64) @ np.abs(B[r.idx[a:b] - 1]).astype(np.float64)
        assert_close(C[i], want, scale, np.float32)
