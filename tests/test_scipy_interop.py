"""scipy.sparse interop on the host, the Python counterpart of Finch's
SparseArrays extension (ext/SparseArraysExt.jl): Tensor(A) maps a canonical
CSC matrix's own 0-based buffers (stored zeros kept, fill zero(T));
Tensor(fmt, A) copies through Finch's dropfills! semantics without a dense
intermediate; sparse(t) gives a scipy.sparse matrix back, reusing 0-based
buffers and refusing a non-zero fill.  No GPU."""
import numpy as np
import pytest

import finchgb as F
from finchgb.workloads import csr_from_dense

sp = pytest.importorskip("scipy.sparse")

CSC_F64 = F.Dense(F.SparseList(F.Element(0.0)))


def rand_csc(m, n, density, seed, dtype=np.float64):
    return sp.random(m, n, density=density, format="csc", random_state=seed, dtype=dtype)


def test_tensor_maps_a_csc_matrix_without_copies():
    A = rand_csc(50, 40, 0.1, 2)
    A.data[3] = 0.0  # a stored zero stays stored, as in Tensor(::SparseMatrixCSC)
    t = F.Tensor(A)
    b = t.buf
    assert b.base == 0 and b.orient == "csc"
    assert np.shares_memory(b.ptr, A.indptr) and np.shares_memory(b.idx, A.indices)
    assert np.shares_memory(b.val, A.data)
    assert t.countstored() == A.nnz and t.fill_value == 0.0 and t.dtype == np.float64
    assert t.fmt.lvl.index_type == A.indices.dtype.type
    assert np.array_equal(t.todense(), A.toarray())


@pytest.mark.parametrize("dtype", [np.float32, np.int32, np.bool_])
def test_tensor_keeps_the_value_type(dtype):
    A = rand_csc(30, 30, 0.2, 5, dtype=np.float64)
    A.data = (A.data * 10 + 1).astype(dtype)
    t = F.Tensor(A)
    assert t.dtype == np.dtype(dtype) and t.fill_value == dtype(0)
    assert np.array_equal(t.todense(), A.toarray())


def test_other_formats_and_duplicates_are_converted():
    D = np.zeros((6, 5))
    D[0, 1], D[3, 4], D[5, 0] = 1.5, -2.0, 3.0
    R = sp.csr_matrix(D)
    t = F.Tensor(R)
    assert not np.shares_memory(t.buf.idx, R.indices)
    assert np.array_equal(t.todense(), D)
    # duplicates are summed and coordinates sorted (SparseMatrixCSC's invariant)
    C = sp.coo_matrix((np.array([1.0, 2.0, 4.0]), (np.array([2, 0, 0]), np.array([1, 1, 1]))), shape=(3, 3))
    t = F.Tensor(C)
    assert np.array_equal(t.buf.idx, [0, 2]) and np.array_equal(t.buf.val, [6.0, 1.0])


def test_one_dimensional_scipy_arrays_are_refused():
    try:
        v = sp.coo_array((np.ones(2), (np.array([1, 3]),)), shape=(5,))
    except (TypeError, ValueError):
        pytest.skip("this scipy has no 1-d sparse arrays")
    with pytest.raises(ValueError, match="2-D"):
        F.Tensor(v)
    with pytest.raises(ValueError, match="2-D"):
        F.Tensor(CSC_F64, v)


def test_tensor_with_a_format_drops_stored_fills():
    A = rand_csc(40, 30, 0.15, 7)
    A.data[::5] = 0.0
    want = A.toarray()
    t = F.Tensor(CSC_F64, A)
    assert t.buf.base == 0 and t.countstored() == int(np.count_nonzero(A.data))
    assert np.array_equal(t.todense(), want)
    assert not np.shares_memory(t.buf.val, A.data)  # the stored zeros were dropped: a copy
    # canonical, no stored zeros, same value type: the arrays are A's own
    B = rand_csc(40, 30, 0.15, 8)
    t = F.Tensor(CSC_F64, B)
    assert np.shares_memory(t.buf.idx, B.indices) and np.shares_memory(t.buf.val, B.data)
    # another value type: values converted, coordinates shared
    t32 = F.Tensor(F.Dense(F.SparseList(F.Element(np.float32(0)))), B)
    assert t32.buf.val.dtype == np.float32 and np.shares_memory(t32.buf.idx, B.indices)
    assert np.array_equal(t32.todense(), B.toarray().astype(np.float32))
    # a pattern stores the true entries
    tp = F.Tensor(F.Dense(F.SparseList(F.Pattern())), A)
    assert tp.buf.val is None and np.array_equal(tp.todense(), want != 0)
    # COO: column-major, 1-based coordinates
    tc = F.Tensor(F.SparseCOO(2, F.Element(0.0)), A)
    I, J, V = tc.coo
    assert np.all(np.diff(J) >= 0) and I.min() >= 1 and np.array_equal(tc.todense(), want)


def test_a_nonzero_fill_stores_the_implicit_zeros():
    A = rand_csc(10, 8, 0.2, 9)
    t = F.Tensor(F.Dense(F.SparseList(F.Element(1.0))), A)
    assert t.countstored() == int(np.count_nonzero(A.toarray() != 1.0))
    assert np.array_equal(t.todense(), A.toarray())


def test_sparse_gives_scipy_back():
    A = rand_csc(50, 40, 0.1, 2)
    S = F.sparse(F.Tensor(A))
    assert isinstance(S, sp.csc_matrix) and (S != A).nnz == 0
    assert np.shares_memory(S.indices, A.indices) and np.shares_memory(S.data, A.data)
    # Finch's own 1-based buffers
    D = np.where(np.random.default_rng(3).random((20, 15)) < 0.3, 2.5, 0.0)
    S = F.sparse(F.Tensor(CSC_F64, D))
    assert np.array_equal(S.toarray(), D)
    # CSR: swizzle(Tensor(A^T), 2, 1) maps a csr_matrix's buffers, and comes back as CSR
    R = sp.random(30, 20, density=0.2, format="csr", random_state=3)
    sw = F.swizzle(F.Tensor(R.T), 2, 1)
    assert np.shares_memory(sw.body.buf.idx, R.indices)
    S = F.sparse(sw)
    assert isinstance(S, sp.csr_matrix) and abs(S - R).max() == 0
    # pattern: true entries
    P = F.sparse(F.Tensor(F.Dense(F.SparseList(F.Pattern())), D))
    assert P.dtype == np.bool_ and np.array_equal(P.toarray(), D != 0)
    # dense tensors convert
    assert np.array_equal(F.sparse(F.Tensor(F.Dense(F.Dense(F.Element(0.0))), D)).toarray(), D)


def test_sparse_refuses_what_scipy_cannot_hold():
    with pytest.raises(ValueError, match="zero fill"):
        F.sparse(F.Tensor(F.Dense(F.SparseList(F.Element(1.0))), np.eye(3)))
    with pytest.raises(ValueError, match="matrices"):
        F.sparse(F.Tensor(F.Dense(F.Element(0.0)), np.ones(3)))


def test_zero_based_buffers_through_file_io(tmp_path):
    A = rand_csc(25, 18, 0.2, 11)
    t = F.Tensor(A)
    for name in ("a.bspnpy", "a.mtx", "a.tns"):
        F.fwrite(str(tmp_path / name), t)
        back = F.fread(str(tmp_path / name))
        got = back.todense() if hasattr(back, "todense") else back
        assert np.array_equal(np.asarray(got, dtype=np.float64), A.toarray()), name


def test_galley_degrees_read_zero_based_buffers():
    from finchgb.galley import _body_degrees

    D = np.zeros((7, 6))
    D[2, :] = 1.0
    D[:, 4] = 2.0
    a = _body_degrees(F.Tensor(sp.csc_matrix(D)))
    b = _body_degrees(F.Tensor(CSC_F64, D))
    assert a == b == (6.0, 7.0)


def test_finch_buffers_keep_base_one():
    r = csr_from_dense(np.eye(4))
    assert r.base == 1 and r.ptr[0] == 1


def huge_csc(fill=0.0):
    """A 1M x 1M CSC with five stored entries: any dense intermediate (8 TB)
    would fail, so these conversions must work on the stored entries."""
    n = 1_000_000
    cols = np.array([3, 3, 70_000, 999_999, 999_999])
    rows = np.array([10, 500_000, 2, 0, 999_999])
    vals = np.array([1.5, -2.0, 3.25, 4.0, 0.5])
    ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(cols, minlength=n), out=ptr[1:])
    from finchgb.workloads import SparseBuffers

    b = SparseBuffers(n, n, ptr + 1, rows.astype(np.int64) + 1, vals, "csc")
    return F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(fill))), b), rows, cols, vals


def test_sparse_to_sparse_conversions_skip_the_dense_form():
    t, rows, cols, vals = huge_csc()
    t32 = F.Tensor(F.Dense(F.SparseList(F.Element(np.float32(0)))), t)  # another value type
    assert t32.dtype == np.float32 and t32.countstored() == 5
    S = F.sparse(t32)
    assert S.dtype == np.float32 and np.array_equal(S[rows, cols].A1, vals.astype(np.float32))
    tp = F.Tensor(F.Dense(F.SparseList(F.Pattern())), t)  # pattern
    assert tp.buf.val is None and tp.countstored() == 5
    tc = F.Tensor(F.SparseCOO(2, F.Element(0.0)), t)  # COO, column-major
    I, J, V = tc.coo
    assert np.array_equal(J - 1, cols) and np.array_equal(I - 1, rows) and np.array_equal(V, vals)
    tt = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), F.swizzle(t, 2, 1))  # CSC of the transpose
    St = F.sparse(tt)
    assert tt.countstored() == 5 and np.array_equal(St[cols, rows].A1, vals)
    # csr() of a scipy matrix stays sparse too
    R = sp.csr_matrix((vals, (rows, cols)), shape=(1_000_000, 1_000_000))
    A = F.csr(R)
    assert A.shape == (1_000_000, 1_000_000) and A.body.countstored() == 5


def test_conversions_drop_stored_fills_of_any_value():
    D = np.array([[np.inf, 2.0, np.inf], [1.0, np.inf, 5.0]])
    src = F.Tensor(F.Dense(F.SparseList(F.Element(np.inf))), D)
    assert src.countstored() == 3
    # the same fill in another value type: stored entries only
    t = F.Tensor(F.Dense(F.SparseList(F.Element(np.float32(np.inf)))), src)
    assert t.countstored() == 3 and np.array_equal(t.todense(), D.astype(np.float32))
    # a stored entry equal to the fill is dropped (dropfills!)
    b = src.host_buffers()
    b.val[0] = np.inf
    t = F.Tensor(F.Dense(F.SparseList(F.Element(np.inf))), src)
    assert t.countstored() == 2 and np.array_equal(t.todense(), src.todense())
    # NaN fills compare equal, as isequal does
    N = np.array([[np.nan, 1.0], [2.0, np.nan]])
    tn = F.Tensor(F.Dense(F.SparseList(F.Element(np.nan))), N)
    t = F.Tensor(F.Dense(F.SparseList(F.Element(np.float32(np.nan)))), tn)
    assert t.countstored() == 2
    # different fills: the implicit entries become stored
    t = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), src)
    assert t.countstored() == 6 and np.array_equal(t.todense(), src.todense())


def test_equality_walks_stored_entries_only():
    """== and isequal as src/interface/compare.jl: every coordinate compared,
    two sparse matrices over the union of their stored entries and their
    fills, which holds for 1M x 1M operands."""
    t, rows, cols, vals = huge_csc()
    same = F.Tensor(sp.csc_matrix((vals, (rows, cols)), shape=t.shape))  # 0-based buffers
    assert t == same and F.isequal(t, same)
    other = sp.csc_matrix((vals * 2, (rows, cols)), shape=t.shape)
    assert not (t == F.Tensor(other))
    # an explicitly stored fill equals an implicit one
    extra = sp.csc_matrix((np.r_[vals, 0.0], (np.r_[rows, 7], np.r_[cols, 8])), shape=t.shape)
    assert t == F.Tensor(extra)
    # fills differ where neither stores an entry
    t1, *_ = huge_csc(fill=1.0)
    assert not (t == t1)
    # the CSR view of the transpose
    tt = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), F.swizzle(t, 2, 1))
    assert F.swizzle(tt, 2, 1) == t
    # NaN: == is false, isequal true
    N = np.array([[np.nan, 1.0], [0.0, 2.0]])
    a, b = F.Tensor(CSC_F64, N), F.Tensor(sp.csc_matrix(N))
    assert not (a == b) and F.isequal(a, b)
    # against a dense array
    assert a.__eq__(np.array([[1.0, 1.0], [0.0, 2.0]])) is False
    assert F.isequal(a, N) and not F.isequal(a, N[:1])
