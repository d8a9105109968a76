"""The oracle against independent evaluations on small seeded inputs: dense
numpy products and scipy.sparse assembly, merges and products.  Every
semiring of SpMV in both orientations, SpMM, SDDMM, the two-finger merges,
elementwise+reduce, COO assembly with each combine and SpGEMM -- exact for
integers and Bool, within a stated bound for floats -- and the threaded
row-parallel nests equal the serial ones bit for bit (each row is summed by
one thread in storage order, as Finch's static split does)."""
import numpy as np
import pytest

import oracle
from finchgb.workloads import SparseBuffers, csc_from_dense, csr_from_dense

I32_MAX, I32_MIN = np.iinfo(np.int32).max, np.iinfo(np.int32).min
F64_BOUND = 64 * np.finfo(np.float64).eps  # per unit of sum |terms|, for sums of <= 60 terms


def sparse_dense(m, n, density, seed, lo=1, hi=10, dtype=np.int64):
    """A dense matrix with about density * m * n nonzeros in [lo, hi), and a
    few empty rows and columns."""
    rng = np.random.default_rng(seed)
    D = np.where(rng.random((m, n)) < density, rng.integers(lo, hi, (m, n)), 0).astype(dtype)
    D[m // 3, :] = 0
    D[:, n // 2] = 0
    return D


def buffers(D, orient, dtype=None):
    b = csr_from_dense(D) if orient == "csr" else csc_from_dense(D)
    if dtype is not None:
        b.val = b.val.astype(dtype)
    return b


def run_spmv(sr, b, x, **kw):
    f = oracle.spmv_csc if b.orient == "csc" else oracle.spmv_csr
    return f(sr, b.nrows, b.ncols, b.ptr, b.idx, b.val, x, **kw)


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("fma", [True, False])
def test_plus_times_float_matches_dense(orient, fma):
    rng = np.random.default_rng(1)
    D = sparse_dense(47, 39, 0.2, 2).astype(np.float64) * rng.standard_normal((47, 39))
    x = rng.standard_normal(39)
    y = run_spmv(oracle.SR_PT, buffers(D, orient), x, fma=fma)
    bound = F64_BOUND * (np.abs(D) @ np.abs(x)) + 1e-300
    assert (np.abs(y - D @ x) <= bound).all()


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_plus_times_integers_exact(orient, dtype):
    D = sparse_dense(50, 41, 0.25, 3, lo=-9, hi=10)
    x = np.random.default_rng(4).integers(-20, 20, 41)
    y = run_spmv(oracle.SR_PT, buffers(D, orient, dtype), x.astype(dtype))
    assert y.dtype == dtype and np.array_equal(y.astype(np.int64), D @ x)


@pytest.mark.parametrize("orient", ["csc", "csr"])
def test_min_and_max_plus_exact(orient):
    D = sparse_dense(44, 36, 0.2, 5, lo=1, hi=1000)
    x = np.random.default_rng(6).integers(0, 5000, 36)
    b = buffers(D, orient, np.int32)
    stored = D != 0
    terms = np.where(stored, D + x[None, :], 0)
    want_min = np.where(stored.any(1), np.where(stored, terms, I32_MAX).min(1), I32_MAX)
    want_max = np.where(stored.any(1), np.where(stored, terms, I32_MIN).max(1), I32_MIN)
    assert np.array_equal(run_spmv(oracle.SR_MINP, b, x.astype(np.int32)), want_min)
    assert np.array_equal(run_spmv(oracle.SR_MAXP, b, x.astype(np.int32)), want_max)


@pytest.mark.parametrize("orient", ["csc", "csr"])
def test_or_and_pattern_exact(orient):
    D = sparse_dense(61, 53, 0.05, 7)
    b = buffers(D, orient)
    pat = SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, None, b.orient)
    for seed in range(3):
        x = (np.random.default_rng(seed).random(53) < 0.2).astype(np.uint8)
        y = run_spmv(oracle.SR_OA, pat, x)
        assert np.array_equal(y.astype(bool), ((D != 0) & (x[None, :] != 0)).any(1))


def test_init_false_accumulates_into_y():
    D = sparse_dense(20, 15, 0.3, 8)
    x = np.arange(15, dtype=np.int64)
    y0 = np.arange(20, dtype=np.int64) * 100
    b = buffers(D, "csc")
    y = oracle.spmv_csc(oracle.SR_PT, 20, 15, b.ptr, b.idx, b.val, x, y=y0.copy(), init=False)
    assert np.array_equal(y, y0 + D @ x)


@pytest.mark.parametrize("nthreads", [2, 3, 7])
def test_threaded_row_nests_equal_serial(nthreads):
    rng = np.random.default_rng(9)
    D = sparse_dense(83, 70, 0.15, 10).astype(np.float64) * rng.standard_normal((83, 70))
    b = buffers(D, "csr")
    x = rng.standard_normal(70)
    B = rng.standard_normal((70, 12))
    X, Y = rng.standard_normal((83, 9)), rng.standard_normal((70, 9))
    one = dict(nthreads=1)
    many = dict(nthreads=nthreads)
    assert np.array_equal(oracle.spmv_csr(0, 83, 70, b.ptr, b.idx, b.val, x, **one),
                          oracle.spmv_csr(0, 83, 70, b.ptr, b.idx, b.val, x, **many))
    assert np.array_equal(oracle.spmm_csr(83, 70, b.ptr, b.idx, b.val, B, **one),
                          oracle.spmm_csr(83, 70, b.ptr, b.idx, b.val, B, **many))
    assert np.array_equal(oracle.sddmm_csr(83, b.ptr, b.idx, b.val, X, Y, **one),
                          oracle.sddmm_csr(83, b.ptr, b.idx, b.val, X, Y, **many))


def test_spmm_and_sddmm_match_dense():
    rng = np.random.default_rng(11)
    D = sparse_dense(64, 48, 0.2, 12).astype(np.float64) * rng.standard_normal((64, 48))
    b = buffers(D, "csr")
    B = rng.standard_normal((48, 16))
    C = oracle.spmm_csr(64, 48, b.ptr, b.idx, b.val, B)
    assert (np.abs(C - D @ B) <= F64_BOUND * (np.abs(D) @ np.abs(B)) + 1e-300).all()
    X, Y = rng.standard_normal((64, 8)), rng.standard_normal((48, 8))
    out = oracle.sddmm_csr(64, b.ptr, b.idx, b.val, X, Y)
    rows = np.repeat(np.arange(64), np.diff(b.ptr))
    cols = b.idx - 1
    want = b.val * np.einsum("qk,qk->q", X[rows], Y[cols])
    scale = np.abs(b.val) * np.einsum("qk,qk->q", np.abs(X[rows]), np.abs(Y[cols]))
    assert (np.abs(out - want) <= F64_BOUND * scale + 1e-300).all()


def scipy_csr(D):
    sp = pytest.importorskip("scipy.sparse")
    A = sp.csr_matrix(D)
    A.sort_indices()
    return A


@pytest.mark.parametrize("op", [0, 1])
def test_two_finger_merges_match_scipy(op):
    Da, Db = sparse_dense(37, 29, 0.3, 13), sparse_dense(37, 29, 0.3, 14)
    a, b = buffers(Da, "csr"), buffers(Db, "csr")
    ptr, idx, val = oracle.ewise(op, 37, a.ptr, a.idx, a.val, b.ptr, b.idx, b.val)
    # positive values: the product's pattern is the intersection, the sum's the union
    want = scipy_csr(Da * Db if op == 0 else Da + Db)
    assert np.array_equal(ptr, want.indptr + 1) and np.array_equal(idx, want.indices + 1)
    assert np.array_equal(val, want.data)


@pytest.mark.parametrize("dims", [0, 1, 2])
def test_elementwise_reduce_matches_dense(dims):
    Da, Db = sparse_dense(31, 26, 0.35, 15, lo=-5, hi=6), sparse_dense(31, 26, 0.35, 16, lo=-5, hi=6)
    a, b = buffers(Da, "csr", np.float64), buffers(Db, "csr", np.float64)
    P = (Da * Db).astype(np.float64)
    want = P.sum() if dims == 0 else P.sum(axis=0 if dims == 1 else 1)
    y = oracle.ewise_reduce(dims, 31, 26, a.ptr, a.idx, a.val, b.ptr, b.idx, b.val)
    assert np.array_equal(y, np.atleast_1d(want))  # small integers: every order is exact
    yd = oracle.ewise_reduce(dims, 31, 26, a.ptr, a.idx, a.val, Bd=Db.astype(np.float64))
    assert np.array_equal(yd, np.atleast_1d(want))


@pytest.mark.parametrize("combine", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("csc", [True, False])
def test_coo_assembly_folds_every_combine(combine, csc):
    rng = np.random.default_rng(17 + combine)
    I, J = rng.integers(1, 12, 400), rng.integers(1, 9, 400)
    V = rng.integers(-100, 100, 400).astype(np.int64)
    if combine == 1:  # | folds Bool values (the library accepts it for Bool only)
        V = (V > 0).astype(np.uint8)
    fold = {0: lambda a, v: a + v, 1: lambda a, v: a | v, 2: min, 3: max, 4: lambda a, v: v}[combine]
    acc = {}
    for i, j, v in zip(I.tolist(), J.tolist(), V.tolist()):  # input order
        acc[(i, j)] = fold(acc[(i, j)], v) if (i, j) in acc else v
    fib = (lambda ij: (ij[1], ij[0])) if csc else (lambda ij: ij)
    keys = sorted(acc, key=fib)
    ptr, idx, val = oracle.coo_assemble(11, 8, I, J, V, csc=csc, combine=combine)
    nfib = 8 if csc else 11
    counts = np.bincount([fib(k)[0] - 1 for k in keys], minlength=nfib)
    assert np.array_equal(ptr, np.concatenate([[1], 1 + np.cumsum(counts)]))
    assert idx.tolist() == [fib(k)[1] for k in keys]
    assert val.tolist() == [acc[k] for k in keys]


def test_coo_assembly_rejects_out_of_range():
    with pytest.raises(ValueError):
        oracle.coo_assemble(4, 4, np.array([1, 5]), np.array([1, 1]), np.ones(2))


def test_spgemm_matches_scipy():
    Da, Db = sparse_dense(45, 38, 0.12, 18), sparse_dense(38, 41, 0.12, 19)
    a, b = buffers(Da, "csr", np.float64), buffers(Db, "csr", np.float64)
    want = scipy_csr(Da @ Db)  # positive values: touched coordinates are the nonzeros
    for fma in (True, False):  # small integers: exact either way
        ptr, idx, val = oracle.spgemm_csr(45, 41, a.ptr, a.idx, a.val, b.ptr, b.idx, b.val, fma=fma)
        assert np.array_equal(ptr, want.indptr + 1) and np.array_equal(idx, want.indices + 1)
        assert np.array_equal(val, want.data)
    with pytest.raises(TypeError):
        oracle.spgemm_csr(45, 41, a.ptr, a.idx, a.val.astype(np.int64), b.ptr, b.idx, b.val)


def test_coo_or_on_integers_is_bitwise():
    # Julia's | on integers (the oracle's contract; the library folds | over Bool only)
    ptr, idx, val = oracle.coo_assemble(2, 2, np.array([1, 1, 2]), np.array([1, 1, 2]),
                                        np.array([5, 2, 8], dtype=np.int64), combine=1)
    assert ptr.tolist() == [1, 2, 3] and idx.tolist() == [1, 2] and val.tolist() == [7, 8]
