"""GPU parity of semiring SpMV (fgb_spmv through the C ABI) against the
oracle: bit-exact for integer, Bool and min/max semirings and for float sums
in Finch's serial order; within RTOL * sum|terms| otherwise."""
import json
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import SparseBuffers, csc_from_dense, fsprand, random_graph
from helpers import abs_terms, assert_close, oracle_spmv, to_dev, to_host, upload

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "finch_kats.json").read_text())["kats"]


def csr_of(b: SparseBuffers) -> SparseBuffers:
    """The same logical matrix stored by rows (host-side, for oracle inputs)."""
    from finchgb.workloads import csr_from_dense

    if b.val is None:
        D = b.todense() != 0
        r = csr_from_dense(D.astype(np.float64))
        return SparseBuffers(r.nrows, r.ncols, r.ptr, r.idx, None, "csr")
    D = b.todense()
    r = csr_from_dense(D)
    r.val = r.val.astype(b.val.dtype)
    return r


def test_kat_spmv_csc(gpu_lib):
    k = KATS["spmv_csc"]
    b = csc_from_dense(np.array(k["A"]))
    A = upload(b)
    x = to_dev(np.array(k["x"]))
    # CSC push (atomics)
    y = to_host(dev.spmv(A, x))
    np.testing.assert_allclose(y, k["y"], rtol=1e-15)
    # Finch order: transpose once on the device, then one running sum per row
    At = A.transposed_storage()
    for flags in (L.FINCH_ORDER, L.FINCH_ORDER | L.NO_FMA):
        y = to_host(dev.spmv(At, x, flags=flags))
        assert y.tolist() == k["y"]


def test_kat_transposed_int(gpu_lib):
    k = KATS["spmv_transposed_int"]
    b = csc_from_dense(np.array(k["A"], dtype=np.int64))
    A = upload(b)
    x = to_dev(np.array(k["x"], dtype=np.int64))
    y = to_host(dev.spmv(A.T(), x))  # A^T x: CSC buffers read as CSR of A^T
    assert y.tolist() == [int(v) for v in k["y"]]


FLOAT_CASES = [(np.float64, False), (np.float32, False), (np.float32, True)]


@pytest.mark.parametrize("dtype,bf16", FLOAT_CASES)
@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("shape,p", [((300, 200), 0.05), ((64, 1000), 0.3), ((1000, 1000), 0.001)])
def test_plus_times_float(gpu_lib, dtype, bf16, orient, shape, p):
    rng = np.random.default_rng([shape[0], shape[1], int(p * 1e6), orient == "csr"])
    b = fsprand(rng, shape[0], shape[1], p, dtype=np.float64)
    b.val = (b.val * 2 - 1).astype(dtype)
    if orient == "csr":
        b = csr_of(b)
    x = (rng.random(shape[1]) * 2 - 1).astype(dtype)
    A = upload(b, as_bf16=bf16)
    y = to_host(dev.spmv(A, to_dev(x)))
    want = oracle_spmv(0, b, x, bf16=bf16)
    assert_close(y, want, abs_terms(b, x), dtype)
    if orient == "csr":
        # Finch order is bit-exact with the oracle's fused / unfused nests
        for flags, fma in ((L.FINCH_ORDER, True), (L.FINCH_ORDER | L.NO_FMA, False)):
            y = to_host(dev.spmv(A, to_dev(x), flags=flags))
            assert np.array_equal(y, oracle_spmv(0, b, x, fma=fma, bf16=bf16))


# float plus-times sums are covered by the tolerance tests
EXACT_CASES = [(sr, dt) for sr in (L.PLUS_TIMES, L.MIN_PLUS, L.MAX_PLUS)
               for dt in (np.int32, np.int64, np.float64, np.float32)
               if not (sr == L.PLUS_TIMES and np.dtype(dt).kind == "f")]


@pytest.mark.parametrize("sr,dtype", EXACT_CASES)
@pytest.mark.parametrize("orient", ["csc", "csr"])
def test_exact_semirings(gpu_lib, sr, dtype, orient):
    rng = np.random.default_rng(7 + sr)
    b = fsprand(rng, 500, 400, 0.02, dtype=np.float64)
    if np.dtype(dtype).kind == "i":
        info = np.iinfo(dtype)
        # full-range values so that + and * wrap
        b.val = rng.integers(info.min // 2, info.max // 2, size=b.nnz, dtype=dtype)
        x = rng.integers(info.min // 2, info.max // 2, size=400, dtype=dtype)
    else:
        b.val = rng.integers(-1000, 1000, size=b.nnz).astype(dtype)
        x = rng.integers(-1000, 1000, size=400).astype(dtype)
    if orient == "csr":
        b = csr_of(b)
    A = upload(b)
    y = to_host(dev.spmv(A, to_dev(x), semiring=sr))
    want = oracle_spmv(sr, b, x)
    assert np.array_equal(y, want)


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("pattern", [True, False])
def test_or_and(gpu_lib, orient, pattern):
    rng = np.random.default_rng(11)
    b = random_graph(rng, 3000, 6.0, pattern=True)
    if not pattern:
        b.val = rng.random(b.nnz) < 0.7
    if orient == "csr":
        b = csr_of(b)
    x = rng.random(3000) < 0.1
    A = upload(b)
    y = to_host(dev.spmv(A, to_dev(x.astype(np.uint8)), semiring=L.OR_AND))
    want = oracle_spmv(oracle.SR_OA, b, x.astype(np.uint8))
    assert np.array_equal(y, want)


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("frontier", ["none", "one", "sparse", "half", "all"])
@pytest.mark.parametrize("pattern", [True, False])
def test_or_and_short_circuits(gpu_lib, orient, frontier, pattern):
    """The push skips false columns and the pull stops at a row's first true
    product: the result is still the full nest's for every frontier density,
    lane count (heuristic, Finch's serial order, every plan candidate),
    accumulation into a preset y, and Bool values holding explicit falses."""
    from finchgb.plan import Plan

    rng = np.random.default_rng(29)
    n = 5000
    b = random_graph(rng, n, 9.0, pattern=True)
    if not pattern:
        b.val = rng.random(b.nnz) < 0.8
    if orient == "csr":
        b = csr_of(b)
    x = {"none": np.zeros(n, bool), "one": np.arange(n) == 17, "sparse": rng.random(n) < 0.01,
         "half": rng.random(n) < 0.5, "all": np.ones(n, bool)}[frontier].astype(np.uint8)
    want = oracle_spmv(oracle.SR_OA, b, x)
    A, xd = upload(b), to_dev(x)
    assert np.array_equal(to_host(dev.spmv(A, xd, semiring=L.OR_AND)), want)
    y0 = (rng.random(n) < 0.3).astype(np.uint8)
    y = to_dev(y0)
    dev.spmv(A, xd, y, semiring=L.OR_AND, flags=L.ACCUMULATE)
    assert np.array_equal(to_host(y), want | y0)
    if orient == "csr":
        y1 = torch.empty(n, dtype=torch.uint8, device="cuda")
        dev.spmv(A, xd, y1, semiring=L.OR_AND, flags=L.FINCH_ORDER)
        assert np.array_equal(to_host(y1), want)
        y2 = to_dev(y0)
        dev.spmv(A, xd, y2, semiring=L.OR_AND, flags=L.FINCH_ORDER | L.ACCUMULATE)
        assert np.array_equal(to_host(y2), want | y0)
    yp = torch.empty(n, dtype=torch.uint8, device="cuda")
    plan = Plan.spmv(A, xd, yp, semiring=L.OR_AND, tune_reps=1)
    plan.execute()
    assert np.array_equal(to_host(yp), want)


def test_minplus_bellman_ford_rounds(gpu_lib):
    """20 relaxation rounds y .= inf; y[i] <<min>>= A[i,j] + x[j]; x = min(x, y)."""
    rng = np.random.default_rng(3)
    n = 20000
    b = random_graph(rng, n, 8.0)
    sentinel = np.int32(2**30)
    x = np.full(n, sentinel, dtype=np.int32)
    x[0] = 0
    A = upload(b)
    xd = to_dev(x)
    xh = x.copy()
    for _ in range(20):
        yd = dev.spmv(A, xd, semiring=L.MIN_PLUS)
        xd = torch.minimum(xd, yd)
        yh = oracle.spmv_csc(oracle.SR_MINP, n, n, b.ptr, b.idx, b.val, xh)
        xh = np.minimum(xh, yh)
    assert np.array_equal(to_host(xd), xh)
    assert (xh < sentinel).sum() > n // 2  # the search actually reached most nodes


@pytest.mark.parametrize("sr,dtype", [(L.MIN_PLUS, np.int32), (L.PLUS_TIMES, np.int64),
                                      (L.MAX_PLUS, np.int64), (L.PLUS_TIMES, np.float32)])
def test_short_row_blocks(gpu_lib, sr, dtype):
    """CSR pull on short rows with irregular ones among them: empty rows, one
    row of 2000 entries, a row count that is not a multiple of 32, and
    accumulation.  Exact for integer semirings."""
    rng = np.random.default_rng(41 + sr)
    m, n = 3007, 2500
    D = np.where(rng.random((m, n)) < 0.002, 1.0, 0.0)
    D[40, :2000] = 1.0   # 2000 entries in the second block of rows
    D[64:96] = 0.0       # a whole block of empty rows
    D[3006, ::3] = 1.0   # the last (partial) block
    from finchgb.workloads import csr_from_dense

    b = csr_from_dense(D)
    if np.dtype(dtype).kind == "i":
        info = np.iinfo(dtype)
        b.val = rng.integers(info.min // 2, info.max // 2, size=b.nnz, dtype=dtype)
        x = rng.integers(info.min // 2, info.max // 2, size=n, dtype=dtype)
    else:
        b.val = rng.standard_normal(b.nnz).astype(dtype)
        x = rng.standard_normal(n).astype(dtype)
    assert b.nnz / m <= 16  # the short-row kernel's range
    A = upload(b)
    y = to_host(dev.spmv(A, to_dev(x), semiring=sr))
    want = oracle_spmv(sr, b, x)
    if np.dtype(dtype).kind == "i":
        assert np.array_equal(y, want)
        y0 = rng.integers(-1000, 1000, size=m).astype(dtype)
        yd = to_dev(y0)
        dev.spmv(A, to_dev(x), yd, semiring=sr, flags=L.ACCUMULATE)
        add = {L.MIN_PLUS: np.minimum, L.MAX_PLUS: np.maximum}.get(sr)
        if add is None:
            exp = (y0.astype(np.int64) + want.astype(np.int64)).astype(dtype)  # wraps like Julia
        else:
            exp = add(y0, want)
        assert np.array_equal(to_host(yd), exp)
    else:
        assert_close(y, want, abs_terms(b, x), np.float32)


@pytest.mark.parametrize("sr,dtype", [(L.PLUS_TIMES, np.float64), (L.PLUS_TIMES, np.float32),
                                      (L.MIN_PLUS, np.int32), (L.MAX_PLUS, np.int64),
                                      (L.PLUS_TIMES, np.int64)])
def test_adaptive_pull_on_many_rows(gpu_lib, sr, dtype):
    """A CSR with more rows than 2048 per SM takes the adaptive pull without a
    plan: short rows one lane each, rows over 32 entries a warp each.  Rows of
    0 to ~15 entries, 64 rows of 33 to 3000 entries, a partial last warp;
    exact semirings bit for bit (accumulating too), float sums within the
    bound.  A plan over the same matrix picks one of its candidates, the
    adaptive pull among them, and gives the same result."""
    from finchgb.plan import Plan
    from finchgb.workloads import _fibers_from_lengths, _ptr

    rng = np.random.default_rng(90 + sr)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    m, n = sms * 2048 + 1013, 60_000
    lengths = rng.poisson(4.0, m).astype(np.int64)
    lengths[rng.choice(m, 64, replace=False)] = rng.integers(33, 3001, 64)
    lengths[5 * 32:6 * 32] = 0  # a warp of empty rows
    cols = _fibers_from_lengths(rng, lengths, n)
    b = SparseBuffers(m, n, _ptr(lengths), cols + 1, None, "csr")
    if np.dtype(dtype).kind == "i":
        info = np.iinfo(dtype)
        b.val = rng.integers(info.min // 2, info.max // 2, size=b.nnz, dtype=dtype)
        x = rng.integers(info.min // 2, info.max // 2, size=n, dtype=dtype)
    else:
        b.val = rng.standard_normal(b.nnz).astype(dtype)
        x = rng.standard_normal(n).astype(dtype)
    A = upload(b)
    y = to_host(dev.spmv(A, to_dev(x), semiring=sr))
    want = oracle_spmv(sr, b, x)
    if np.dtype(dtype).kind == "i":
        assert np.array_equal(y, want)
        y0 = rng.integers(-1000, 1000, size=m).astype(dtype)
        yd = to_dev(y0)
        dev.spmv(A, to_dev(x), yd, semiring=sr, flags=L.ACCUMULATE)
        add = {L.MIN_PLUS: np.minimum, L.MAX_PLUS: np.maximum}.get(sr)
        exp = (y0.astype(np.int64) + want.astype(np.int64)).astype(dtype) if add is None else add(y0, want)
        assert np.array_equal(to_host(yd), exp)
    else:
        assert_close(y, want, abs_terms(b, x), dtype)
    xd, yp = to_dev(x), torch.empty(m, dtype=to_dev(x).dtype, device="cuda")
    plan = Plan.spmv(A, xd, yp, semiring=sr, tune_reps=2)
    assert plan.info()["lanes"] in (1, 2, 4, 8, 32)
    plan.execute()
    if np.dtype(dtype).kind == "i":
        assert np.array_equal(to_host(yp), want)
    else:
        assert_close(to_host(yp), want, abs_terms(b, x), dtype)


@pytest.mark.parametrize("ptr_i64", [False, True])
def test_edge_cases(gpu_lib, ptr_i64):
    # empty matrix, empty fibers, a long fiber, 1x1
    cases = []
    cases.append(SparseBuffers(5, 4, np.ones(5, np.int64), np.zeros(0, np.int64),
                               np.zeros(0), "csc"))
    D = np.zeros((50, 3000))
    D[7, :] = np.arange(3000) % 7 - 3.0  # one row with 2571 stored entries
    D[9, 5] = 2.0
    cases.append(csc_from_dense(D))
    cases.append(csr_of(csc_from_dense(D)))
    cases.append(csc_from_dense(np.array([[2.5]])))
    for b in cases:
        x = np.linspace(-1, 1, b.ncols)
        A = upload(b)
        if ptr_i64:
            A.ptr = A.ptr.to(torch.int64)
            A._desc = None
        y = to_host(dev.spmv(A, to_dev(x)))
        want = oracle_spmv(0, b, x)
        assert_close(y, want, abs_terms(b, x), np.float64)


@pytest.mark.parametrize("name", ["west0132", "lpi_itest6", "lp_blend", "Trec4"])
def test_matrixmarket_fixtures(gpu_lib, name):
    z = np.load(Path(__file__).parent / "golden" / f"mtx_{name}.npz")
    m, n = (int(v) for v in z["shape"])
    from finchgb.workloads import coo_to_csr

    r = coo_to_csr(m, n, z["i"], z["j"], z["v"])
    x = np.cos(np.arange(n))
    A = upload(r)
    y = to_host(dev.spmv(A, to_dev(x), flags=L.FINCH_ORDER))
    assert np.array_equal(y, oracle_spmv(0, r, x))
    At = A.transposed_storage()  # CSC of the same matrix
    y2 = to_host(dev.spmv(At, to_dev(x)))
    assert_close(y2, oracle_spmv(0, r, x), abs_terms(r, x), np.float64)


def test_transpose_roundtrip(gpu_lib):
    rng = np.random.default_rng(5)
    b = fsprand(rng, 700, 300, 0.03)
    A = upload(b)
    At = A.transposed_storage()
    ptr, idx, val = At.to_host()
    r = csr_of(b)
    assert np.array_equal(ptr, r.ptr) and np.array_equal(idx, r.idx)
    assert np.array_equal(val, r.val)
    back = At.transposed_storage()
    p2, i2, v2 = back.to_host()
    assert np.array_equal(p2, b.ptr) and np.array_equal(i2, b.idx) and np.array_equal(v2, b.val)


def test_errors_are_status_codes(gpu_lib):
    b = csc_from_dense(np.eye(3))
    A = upload(b)
    x = to_dev(np.ones(3, dtype=np.float32))  # dtype mismatch with f64 values
    with pytest.raises(L.FinchGBError) as e:
        dev.spmv(A, x)
    assert e.value.status == L.EUNSUPPORTED
    with pytest.raises(L.FinchGBError) as e:
        dev.spmv(A, to_dev(np.ones(3)), flags=L.FINCH_ORDER)  # CSC + Finch order
    assert e.value.status == L.EUNSUPPORTED
