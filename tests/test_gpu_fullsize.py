"""Parity at the benchmark's full sizes, through properties that do not
depend on size: schedules that must agree bit for bit, rows sampled from the
full result against the oracle on those rows, integer semirings exact, and
for SpGEMM the whole product against the oracle (it finishes in seconds).

Inputs are the benchmark's own seeded workloads: the 1M x 1M Zipf(1.5)
matrix with 16M entries (SpMM k = 128, SDDMM k = 64), the 4M-node
Poisson(8) graph (min-plus and or-and), the 2048^2 Poisson matrix (SpGEMM,
CG) and 16M random COO triplets."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import SparseBuffers, poisson2d, random_graph, zipf_csr
from helpers import RTOL, to_host, upload

pytestmark = pytest.mark.gpu
SEED = 20261203  # the benchmark's seed


def rows_of(b: SparseBuffers, rows: np.ndarray) -> SparseBuffers:
    """The CSR sub-matrix of the given rows (host)."""
    lens = (b.ptr[rows + 1] - b.ptr[rows]).astype(np.int64)
    ptr = np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int64)
    sel = np.concatenate([np.arange(b.ptr[r] - 1, b.ptr[r + 1] - 1) for r in rows]) if len(rows) else \
        np.zeros(0, np.int64)
    return SparseBuffers(len(rows), b.ncols, ptr, b.idx[sel], None if b.val is None else b.val[sel], "csr")


def sample_rows(b: SparseBuffers, rng, n=1500, longest=20):
    lens = np.diff(b.ptr)
    pick = np.unique(np.concatenate([rng.choice(b.nrows, n, replace=False), np.argsort(lens)[-longest:]]))
    return pick


@pytest.fixture(scope="module")
def zipf():
    rng = np.random.default_rng(SEED)
    A = zipf_csr(rng, 1_000_000, 1_000_000, mean=16.0, a=1.5, cap=50_000, dtype=np.float32)
    B = rng.standard_normal((1_000_000, 128), dtype=np.float32)
    return A, B


def test_spmm_headline_full_size(gpu_lib, zipf):
    """The headline SpMM, all 1M x 128 outputs, against the oracle's row nest
    run in FP64 (only the GPU's FP32 rounding is tolerated), for the plan's
    banded schedule, the unbanded slab schedule and the merge path."""
    A_h, B_h = zipf
    A, B = upload(A_h), torch.from_numpy(B_h).cuda()
    Cb = to_host(dev.spmm(A, B, lanes=8, path=128, variant=3, bands=4))  # column bands
    assert np.array_equal(Cb, to_host(dev.spmm(A, B, lanes=8, path=128, variant=3, bands=4)))  # deterministic
    assert np.array_equal(Cb, to_host(dev.spmm(A, B, lanes=8, path=128, variant=2, bands=4)))  # register gathers
    C3 = to_host(dev.spmm(A, B, lanes=8, path=128, variant=3))  # unbanded slabs
    assert np.array_equal(C3, to_host(dev.spmm(A, B, lanes=8, path=128, variant=2)))
    Cm = to_host(dev.spmm(A, B))  # the per-call default schedule
    B64 = B_h.astype(np.float64)
    nt = oracle.max_threads()
    want = oracle.spmm_csr(A_h.nrows, A_h.ncols, A_h.ptr, A_h.idx, A_h.val.astype(np.float64), B64, nthreads=nt)
    np.abs(B64, out=B64)
    scale = oracle.spmm_csr(A_h.nrows, A_h.ncols, A_h.ptr, A_h.idx, np.abs(A_h.val).astype(np.float64), B64,
                            nthreads=nt)
    del B64
    tol = RTOL[np.dtype(np.float32)] * scale + 1e-30
    for name, got in (("banded", Cb), ("slabs", C3), ("default", Cm)):
        err = np.abs(got.astype(np.float64) - want)
        assert (err <= tol).all(), f"{name}: {int((err > tol).sum())} of {err.size} outside tolerance"


def test_sddmm_full_size(gpu_lib, zipf):
    """All 16M SDDMM outputs against an FP64 evaluation of A .* (X Y^T)."""
    A_h, _ = zipf
    rng = np.random.default_rng(SEED + 1)
    X = rng.standard_normal((1_000_000, 64), dtype=np.float32)
    Y = rng.standard_normal((1_000_000, 64), dtype=np.float32)
    A, Xd, Yd = upload(A_h), torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    o2 = to_host(dev.sddmm(A, Xd, Yd, chunk=256, variant=2, slab=32))
    assert np.array_equal(o2, to_host(dev.sddmm(A, Xd, Yd, chunk=256, variant=1, slab=32)))
    assert np.array_equal(o2, to_host(dev.sddmm(A, Xd, Yd, chunk=256, variant=2, slab=32, bands=4)))
    nt = oracle.max_threads()
    want = oracle.sddmm_csr(A_h.nrows, A_h.ptr, A_h.idx, A_h.val, X, Y, acc64=True, nthreads=nt)
    scale = oracle.sddmm_csr(A_h.nrows, A_h.ptr, A_h.idx, np.abs(A_h.val), np.abs(X), np.abs(Y), acc64=True,
                             nthreads=nt)
    err = np.abs(o2.astype(np.float64) - want)
    assert (err <= RTOL[np.dtype(np.float32)] * scale + 1e-30).all()


def test_spmv_config1_full_size(gpu_lib):
    """SpMV y[i] += A[i,j]*x[j] at its full size: A 10,000 x 10,000 CSC from
    fsprand(0.001), FP64, seeded as the benchmark seeds it.  The push over
    columns (atomics) lies within the FP64 tolerance of Finch's serial CSC
    nest; the pull in Finch's order equals that nest bit for bit, fused and
    unfused."""
    from finchgb.workloads import fsprand

    rng = np.random.default_rng(SEED + 1)
    n = 10_000
    b = fsprand(rng, n, n, 0.001)
    x = rng.random(n)
    Ad = upload(b)
    Ar = Ad.transposed_storage()
    xd = torch.from_numpy(x).cuda()
    want_f = oracle.spmv_csc(oracle.SR_PT, n, n, b.ptr, b.idx, b.val, x, fma=True)
    want_u = oracle.spmv_csc(oracle.SR_PT, n, n, b.ptr, b.idx, b.val, x, fma=False)
    scale = oracle.spmv_csc(oracle.SR_PT, n, n, b.ptr, b.idx, np.abs(b.val), np.abs(x))
    push = to_host(dev.spmv(Ad, xd))
    assert (np.abs(push - want_f) <= RTOL[np.dtype(np.float64)] * scale + 1e-300).all()
    pull = to_host(dev.spmv(Ar, xd))
    assert (np.abs(pull - want_f) <= RTOL[np.dtype(np.float64)] * scale + 1e-300).all()
    assert to_host(dev.spmv(Ar, xd, flags=L.FINCH_ORDER | L.FMA)).tobytes() == want_f.tobytes()
    assert to_host(dev.spmv(Ar, xd, flags=L.FINCH_ORDER | L.NO_FMA)).tobytes() == want_u.tobytes()


@pytest.fixture(scope="module")
def graph():
    rng = np.random.default_rng(SEED + 3)
    return random_graph(rng, 4_000_000, 8.0)


def test_minplus_and_or_and_full_size(gpu_lib, graph):
    g = graph
    n = g.nrows
    Ad = upload(g)  # CSC: columns are sources
    Ar = Ad.transposed_storage()
    x = torch.full((n,), 2**30, dtype=torch.int32, device="cuda")
    x[0] = 0
    xp = x.clone()
    for _ in range(20):  # Bellman-Ford rounds, push and pull: bit-identical
        y = dev.spmv(Ad, x, semiring=L.MIN_PLUS)
        dev.dense_map(L.MAP_MIN, x, y, x)
        yp = dev.spmv(Ar, xp, semiring=L.MIN_PLUS)
        dev.dense_map(L.MAP_MIN, xp, yp, xp)
    assert torch.equal(x, xp)
    # one round checked against the oracle's pull nest on sampled rows
    xh = to_host(x)
    y1 = to_host(dev.spmv(Ar, x, semiring=L.MIN_PLUS))
    ptr, idx, val = Ar.to_host()
    csr = SparseBuffers(n, n, ptr, idx, val, "csr")
    rows = sample_rows(csr, np.random.default_rng(3), n=3000)
    sub = rows_of(csr, rows)
    want = oracle.spmv_csr(oracle.SR_MINP, sub.nrows, n, sub.ptr, sub.idx, sub.val, xh)
    assert np.array_equal(y1[rows], want)
    # or-and at a quarter frontier: push over the true columns == pull with early exit == oracle rows
    f = torch.from_numpy((np.random.default_rng(4).random(n) < 0.25).astype(np.uint8)).cuda()
    Ap = dev.DeviceSparse(n, n, Ad.ptr, Ad.idx, None, "csc", Ad.base)
    Arp = dev.DeviceSparse(n, n, Ar.ptr, Ar.idx, None, "csr", Ar.base)
    yo = to_host(dev.spmv(Ap, f, semiring=L.OR_AND))
    assert np.array_equal(yo, to_host(dev.spmv(Arp, f, semiring=L.OR_AND)))
    subp = SparseBuffers(sub.nrows, n, sub.ptr, sub.idx, None, "csr")
    assert np.array_equal(yo[rows], oracle.spmv_csr(oracle.SR_OA, sub.nrows, n, subp.ptr, subp.idx, None,
                                                    to_host(f)))


def test_spgemm_poisson_square_full_size(gpu_lib):
    b = poisson2d(2048)
    A = upload(b)
    C = dev.spgemm(A, A)
    want = oracle.spgemm_csr(b.nrows, b.ncols, b.ptr, b.idx, b.val, b.ptr, b.idx, b.val, fma=True)
    assert np.array_equal(to_host(C.ptr).astype(np.int64), want[0])
    assert np.array_equal(to_host(C.idx).astype(np.int64), want[1])
    assert to_host(C.val).tobytes() == want[2].tobytes()


def test_coo_assembly_full_size(gpu_lib):
    rng = np.random.default_rng(SEED + 7)
    m = n = 1_000_000
    k = 16_000_000
    I = rng.integers(1, m + 1, k)
    J = rng.integers(1, n + 1, k)
    V = rng.standard_normal(k, dtype=np.float32)
    A = dev.coo_assemble(m, n, torch.from_numpy(I).cuda(), torch.from_numpy(J).cuda(),
                         torch.from_numpy(V).cuda(), orient="csc")
    ptr, idx, val = A.to_host()
    assert ptr[0] == 1 and (np.diff(ptr) >= 0).all() and ptr[-1] - 1 == A.nnz
    assert A.nnz == np.unique((J - 1) * m + (I - 1)).size
    # sampled columns: the oracle on exactly the triplets of those columns
    cols = np.random.default_rng(5).choice(n, 2000, replace=False) + 1
    sel = np.isin(J, cols)
    order = np.argsort(cols)
    remap = np.zeros(n + 1, np.int64)
    remap[cols[order]] = np.arange(1, cols.size + 1)
    wp, wi, wv = oracle.coo_assemble(m, cols.size, I[sel], remap[J[sel]], V[sel], csc=True, combine=0)
    for c_new, c in enumerate(cols[order]):
        got_i = idx[ptr[c - 1] - 1: ptr[c] - 1]
        got_v = val[ptr[c - 1] - 1: ptr[c] - 1]
        assert np.array_equal(got_i, wi[wp[c_new] - 1: wp[c_new + 1] - 1])
        assert got_v.tobytes() == wv[wp[c_new] - 1: wp[c_new + 1] - 1].tobytes()


def test_cg_full_size_reaches_tolerance(gpu_lib):
    from finchgb import cg

    b = poisson2d(2048)
    rhs = np.random.default_rng(SEED + 4).uniform(-1, 1, b.nrows)
    A = dev.DeviceSparse.from_host(b.nrows, b.ncols, b.ptr, b.idx, b.val, orient="csr")
    x, res = cg.cg_solve(A, torch.from_numpy(rhs).cuda(), precision="f64", rtol=1e-10)
    assert res.converged
    # the true residual, recomputed on the host in FP64
    xh = to_host(x)
    r = rhs - oracle.spmv_csr(0, b.nrows, b.ncols, b.ptr, b.idx, b.val, xh)
    assert np.linalg.norm(r) <= 1.01e-10 * np.linalg.norm(rhs)
