"""The oracle's Gustavson SpGEMM pinned to the reference's own check:
test/suites/kernel_tests.jl:89-129 computes B = A * A with Finch's
Gustavson nest (column form, SparseByteMap workspace) on the square
MatrixMarket fixtures and asserts B == SparseArrays' A * A."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from finchgb.workloads import coo_to_csr

GOLDEN = Path(__file__).parent / "golden"


def fixture_csc(name):
    z = np.load(GOLDEN / f"mtx_{name}.npz")
    m, n = (int(v) for v in z["shape"])
    # CSR of A^T == CSC of A
    b = coo_to_csr(n, m, z["j"], z["i"], z["v"])
    return m, n, b.ptr, b.idx, b.val, z


@pytest.mark.parametrize("name", ["west0132"])  # the square fixture
def test_gustavson_equals_sparse_matmul(name):
    sp = pytest.importorskip("scipy.sparse")
    m, n, ptr, idx, val, z = fixture_csc(name)
    assert m == n
    # Finch's column form on CSC operands = the row form on the transposed problem
    cp, ci, cv = oracle.spgemm_csr(n, m, ptr, idx, val, ptr, idx, val, fma=False)
    D = np.zeros((m, n))
    for j in range(n):
        D[ci[cp[j] - 1:cp[j + 1] - 1] - 1, j] = cv[cp[j] - 1:cp[j + 1] - 1]
    A = sp.csc_matrix((z["v"], (z["i"] - 1, z["j"] - 1)), shape=(m, n))
    assert np.array_equal(D, (A @ A).toarray())
    for j in range(n):  # coordinates ascending in every fiber
        assert np.all(np.diff(ci[cp[j] - 1:cp[j + 1] - 1]) > 0)
