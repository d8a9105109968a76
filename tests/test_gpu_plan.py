"""Autotuned, graph-captured plans give the same results as the direct calls
(bit-exact where the schedule cannot change the summation, within tolerance
otherwise) and replay correctly after the bound inputs change in place."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.plan import Plan
from finchgb.workloads import fsprand, random_graph, zipf_csr
from helpers import assert_close, to_dev, to_host, upload

pytestmark = pytest.mark.gpu


def test_spmm_plan_matches_and_replays(gpu_lib):
    rng = np.random.default_rng(0)
    r = zipf_csr(rng, 20000, 20000, mean=16)
    A = upload(r)
    B = to_dev(rng.standard_normal((20000, 64)).astype(np.float32))
    C = torch.empty((20000, 64), dtype=torch.float32, device="cuda")
    p = Plan.spmm(A, B, C, tune_reps=2)
    info = p.info()
    assert info["candidates"] > 1 and info["lanes"] in (8, 16, 32)
    for trial in range(2):
        B.copy_(to_dev(rng.standard_normal((20000, 64)).astype(np.float32)))
        C.fill_(float("nan"))
        p.execute()
        want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, to_host(B))
        scale = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, np.abs(r.val), np.abs(to_host(B)))
        assert_close(to_host(C), want, scale, np.float32)
    p2 = Plan.spmm(A, B, C, tune_reps=2)  # same shape class: cached choice
    assert p2.info()["from_cache"] == 1


def test_spmv_plan_exact_semiring_and_finch_order(gpu_lib):
    rng = np.random.default_rng(1)
    g = random_graph(rng, 5000, 8.0)
    A = upload(g)
    x = to_dev(rng.integers(0, 100, 5000).astype(np.int32))
    y = torch.empty(5000, dtype=torch.int32, device="cuda")
    p = Plan.spmv(A, x, y, semiring=L.MIN_PLUS)
    p.execute()
    want = oracle.spmv_csc(oracle.SR_MINP, 5000, 5000, g.ptr, g.idx, g.val, to_host(x))
    assert np.array_equal(to_host(y), want)
    b = fsprand(rng, 800, 700, 0.02)
    Ad = upload(b).transposed_storage()  # CSR
    xf = to_dev(rng.random(700))
    yf = torch.empty(800, dtype=torch.float64, device="cuda")
    pf = Plan.spmv(Ad, xf, yf, flags=L.FINCH_ORDER)
    pf.execute()
    assert np.array_equal(to_host(yf), oracle.spmv_csc(0, 800, 700, b.ptr, b.idx, b.val, to_host(xf)))


def test_sddmm_plan(gpu_lib):
    rng = np.random.default_rng(2)
    r = zipf_csr(rng, 3000, 3000, mean=12, cap=2000)
    A = upload(r)
    X = to_dev(rng.standard_normal((3000, 64)).astype(np.float32))
    Y = to_dev(rng.standard_normal((3000, 64)).astype(np.float32))
    out = torch.empty(r.nnz, dtype=torch.float32, device="cuda")
    p = Plan.sddmm(A, X, Y, out, tune_reps=2)
    p.execute()
    want = oracle.sddmm_csr(r.nrows, r.ptr, r.idx, r.val, to_host(X), to_host(Y), acc64=True)
    scale = np.abs(r.val.astype(np.float64)) * oracle.sddmm_csr(
        r.nrows, r.ptr, r.idx, np.ones(r.nnz), np.abs(to_host(X)).astype(np.float64),
        np.abs(to_host(Y)).astype(np.float64))
    assert_close(to_host(out), want, scale, np.float32)
