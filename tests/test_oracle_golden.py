"""Pins the oracle (the C restatement of Finch's loop nests) against the
numeric results printed in Finch.jl's own test fixtures
(tests/golden/finch_kats.json, extracted by tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from finchgb.workloads import csc_from_dense, csr_from_dense

KATS = json.loads((Path(__file__).parent / "golden" / "finch_kats.json").read_text())["kats"]


@pytest.mark.parametrize("fma", [0, 1])
def test_spmv_csc_kat(fma):
    k = KATS["spmv_csc"]
    A = np.array(k["A"])
    b = csc_from_dense(A)
    x = np.array(k["x"], dtype=np.float64)  # Finch's Int x promotes to Float64
    y = oracle.spmv_csc(oracle.SR_PT, 4, 3, b.ptr, b.idx, b.val, x, fma=fma)
    assert y.tolist() == k["y"]  # bit-exact
    # the fixture's y had stale contents; `y .= 0` re-initialises it
    y0 = np.array([1.0, 2.0, 3.0, 4.0])
    oracle.spmv_csc(oracle.SR_PT, 4, 3, b.ptr, b.idx, b.val, x, y=y0, init=True, fma=fma)
    assert y0.tolist() == k["y"]


def test_spmv_sparsematrixcsc_kat():
    k = KATS["spmv_sparsematrixcsc"]
    b = csc_from_dense(np.array(k["A"]))
    y = oracle.spmv_csc(oracle.SR_PT, 4, 3, b.ptr, b.idx, b.val, np.array([1.0, 2.0, 3.0]))
    assert y.tolist() == k["y"]


def test_spmv_csr_row_pull_equals_csc_serial_kat():
    k = KATS["spmv_csc"]
    A = np.array(k["A"])
    r = csr_from_dense(A)
    for nthreads in (1, 2, 3):
        y = oracle.spmv_csr(oracle.SR_PT, 4, 3, r.ptr, r.idx, r.val, np.array(k["x"]),
                            nthreads=nthreads)
        assert y.tolist() == k["y"]


def test_transposed_int_spmv_kat():
    k = KATS["spmv_transposed_int"]
    A = np.array(k["A"], dtype=np.int64)
    b = csc_from_dense(A)  # Finch's CSC of A; its fibers are the rows of A^T
    x = np.array(k["x"], dtype=np.int64)
    y = oracle.spmv_csr(oracle.SR_PT, 2, 2, b.ptr, b.idx, b.val, x)
    assert y.tolist() == [int(v) for v in k["y"]]


def test_merge_twofinger_add_kat():
    k = KATS["merge_twofinger_add"]
    x, y, z = k["x"], k["y"], k["z"]
    ptr, idx, val = oracle.ewise(1, 1, np.array(x["ptr"]), np.array(x["idx"]),
                                 np.array(x["val"]), np.array(y["ptr"]), np.array(y["idx"]),
                                 np.array(y["val"]))
    assert ptr.tolist() == z["ptr"]
    assert idx.tolist() == z["idx"]
    assert val.tolist() == z["val"]


def test_merge_twofinger_mul_intersection():
    k = KATS["merge_twofinger_add"]
    x, y = k["x"], k["y"]
    ptr, idx, val = oracle.ewise(0, 1, np.array(x["ptr"]), np.array(x["idx"]),
                                 np.array(x["val"]), np.array(y["ptr"]), np.array(y["idx"]),
                                 np.array(y["val"]))
    assert idx.tolist() == [5]  # the only shared coordinate
    assert val.tolist() == [4.0 * 1.0]


def test_einsum_matmul_kat():
    k = KATS["einsum_matmul"]
    A = np.array(k["A"], dtype=np.float64)
    B = np.array(k["B"], dtype=np.float64)
    r = csr_from_dense(A)
    C = oracle.spmm_csr(2, 2, r.ptr, r.idx, r.val, B)
    assert C.tolist() == k["C"]
    assert int(np.abs(C).sum()) == k["s_abs"]


@pytest.mark.parametrize("dims,key", [(1, "dims1"), (2, "dims2"), (0, "all")])
def test_reduce_kat(dims, key):
    k = KATS["reduce"]
    A = np.array(k["A"])
    r = csr_from_dense(A)
    ones = np.ones_like(A)
    y = oracle.ewise_reduce(dims, 4, 3, r.ptr, r.idx, r.val, Bd=ones)
    want = k[key] if isinstance(k[key], list) else [k[key]]
    np.testing.assert_allclose(y, want, rtol=0, atol=1e-12)


def test_semiring_identities_and_wrap():
    # min-plus with Int32 wraps like Julia's Int32 `+`
    A = np.array([[2**31 - 1, 0], [5, 7]], dtype=np.int32)
    b = csc_from_dense(A)
    b.val = A.T[A.T != 0].astype(np.int32)  # values in CSC order
    x = np.array([1, 1], dtype=np.int32)
    y = oracle.spmv_csc(oracle.SR_MINP, 2, 2, b.ptr, b.idx, b.val, x)
    assert y.tolist() == [-(2**31), 6]
    # or-and on a Pattern level
    P = csc_from_dense(np.array([[0, 1], [1, 0]], dtype=np.float64))
    xb = np.array([1, 0], dtype=np.uint8)
    yb = oracle.spmv_csc(oracle.SR_OA, 2, 2, P.ptr, P.idx, None, xb)
    assert yb.tolist() == [0, 1]


def test_scansearch_seek_path():
    # A fiber whose first stored coordinate is 0 (below the extent's start)
    # exercises the scansearch seek of the CSC nest.
    ptr = np.array([1, 4], dtype=np.int64)
    idx = np.array([0, 2, 3], dtype=np.int64)  # coordinate 0 lies outside 1:m
    val = np.array([100.0, 2.0, 3.0])
    y = oracle.spmv_csc(oracle.SR_PT, 3, 1, ptr, idx, val, np.array([1.0]))
    assert y.tolist() == [0.0, 2.0, 3.0]
