"""COO assembly (Finch's fsparse + copy into Dense(SparseList)): the oracle
against SparseArrays-style assembly and the reference's own case, and the
host-side fsparse tensor.  The GPU path's parity is in test_gpu_coo.py."""
import numpy as np
import pytest

import oracle
from finchgb import Dense, Element, SparseCOO, SparseList, Tensor, fsparse


def scipy_like(m, n, I, J, V, csc=True):
    """Reference assembly: sort by (fiber, coordinate), sum duplicates."""
    sp = pytest.importorskip("scipy.sparse")
    A = (sp.csc_matrix if csc else sp.csr_matrix)((V, (I - 1, J - 1)), shape=(m, n))
    A.sum_duplicates()
    A.sort_indices()
    return A.indptr + 1, A.indices + 1, A.data


def test_reference_issue_case():
    # test/suites/issue_tests.jl:1019-1024 compares fsparse(I, J, V) with sparse(I, J, V)
    I, J, V = np.array([6, 6, 6, 9]), np.array([1, 3, 10, 5]), np.ones(4, dtype=np.int64)
    ptr, idx, val = oracle.coo_assemble(9, 10, I, J, V)
    assert ptr.tolist() == [1, 2, 2, 3, 3, 4, 4, 4, 4, 4, 5]
    assert idx.tolist() == [6, 6, 9, 6] and val.tolist() == [1, 1, 1, 1]


@pytest.mark.parametrize("csc", [True, False])
def test_oracle_matches_sparse_assembly(csc):
    rng = np.random.default_rng(5)
    I, J = rng.integers(1, 60, 3000), rng.integers(1, 45, 3000)
    V = rng.integers(-50, 50, 3000).astype(np.int64)  # integers: any order sums exactly
    ptr, idx, val = oracle.coo_assemble(59, 44, I, J, V, csc=csc)
    p2, i2, v2 = scipy_like(59, 44, I, J, V, csc)
    assert np.array_equal(ptr, p2) and np.array_equal(idx, i2) and np.array_equal(val, v2)


def test_oracle_folds_in_input_order():
    # float + is not associative: the fold is foldl over the duplicates in input order
    I, J = np.array([2, 1, 2, 2]), np.array([1, 1, 1, 1])
    V = np.array([1e16, 5.0, 1.0, -1e16])
    ptr, idx, val = oracle.coo_assemble(2, 1, I, J, V)
    assert idx.tolist() == [1, 2]
    assert val[1] == (1e16 + 1.0) + -1e16  # = 0.0, not 1.0
    _, _, vmin = oracle.coo_assemble(2, 1, I, J, np.array([0.0, 1.0, -0.0, 3.0]), combine=2)
    assert np.signbit(vmin[1])  # min(0.0, -0.0) == -0.0
    _, _, vlast = oracle.coo_assemble(2, 1, I, J, V, combine=4)
    assert vlast[1] == -1e16
    with pytest.raises(ValueError):
        oracle.coo_assemble(2, 1, np.array([3]), np.array([1]), np.array([1.0]))


def test_host_fsparse_tensor():
    I, J = np.array([3, 1, 3, 2]), np.array([2, 1, 2, 2])
    t = fsparse(I, J, np.array([1.0, 2.0, 4.0, 8.0]), (3, 2))
    D = t.todense()
    assert D.tolist() == [[2.0, 0.0], [0.0, 8.0], [0.0, 5.0]]
    tb = fsparse(I, J, np.array([True, False, False, True]), (3, 2))
    assert tb.todense().tolist() == [[False, False], [False, True], [False, True]]
    tm = fsparse(I, J, np.array([1, 2, 4, 8]), (3, 2), combine="max")
    assert tm.todense()[2, 1] == 4
    with pytest.raises(ValueError):
        fsparse(np.array([4]), np.array([1]), np.array([1.0]), (3, 2))
    # a COO tensor from a dense array holds every non-fill entry
    A = np.array([[0.0, 1.5], [2.0, 0.0]])
    assert np.array_equal(Tensor(SparseCOO(2, Element(0.0)), A).todense(), A)
