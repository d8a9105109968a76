"""PageRank (docs/examples/pagerank.jl) on the GPU: the example's @finch
programs run through the matchers onto fgb_ewise_reduce (out-degree
counts), fgb_sparse_scale (the masked transition matrix), fgb_dense_affine
and the Finch-order SpMV, and the result equals the oracle's restatement
bit for bit (its fused variant: the library fuses a*b+c in Finch programs,
one of the two roundings Finch's @fastmath code can give).  The new kernels are also checked on their own: value types,
both orientations, both axes, counts of Pattern and Bool matrices."""
import numpy as np
import pytest
import torch

import finchgb as F
import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb import examples
from finchgb.workloads import fsprand

pytestmark = pytest.mark.gpu


def graph(n, p, seed):
    """fsprand CSC adjacency with an entry in every column (no vertex
    without out-edges)."""
    rng = np.random.default_rng(seed)
    g = fsprand(rng, n, n, p)
    D = g.todense() != 0
    empty = ~D.any(axis=0)
    D[rng.integers(0, n, int(empty.sum())), np.flatnonzero(empty)] = True
    return F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), D.astype(np.float64)), D


def csc_of(D):
    t = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), np.asarray(D, dtype=np.float64))
    b = t.host_buffers()
    return b.ptr, b.idx, b.val


@pytest.mark.parametrize("n,p,seed", [(30, 0.5, 1), (700, 0.01, 2), (2000, 0.002, 3)])
def test_pagerank_example_equals_the_oracle(gpu_lib, n, p, seed):
    t, D = graph(n, p, seed)
    edges = F.pattern(t)  # the reference test's pattern!(Tensor(input))
    r = examples.pagerank(edges, nsteps=20, damp=0.85).todense()
    ptr, idx, _ = csc_of(D)
    want = oracle.pagerank(n, ptr, idx, None, 20, 0.85, fma=True)
    assert np.array_equal(r, want)
    assert abs(r.sum() - 1.0) < 1e-12


def test_pagerank_on_weighted_and_swizzled_edges(gpu_lib):
    rng = np.random.default_rng(5)
    _, D = graph(400, 0.02, 6)
    W = np.where(D, rng.random(D.shape) + 0.5, 0.0)
    ptr, idx, val = csc_of(W)
    want = oracle.pagerank(400, ptr, idx, val, 20, 0.85, fma=True)
    r = examples.pagerank(F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), W), nsteps=20).todense()
    np.testing.assert_allclose(r, want, rtol=1e-12, atol=0)  # out-degree sums may associate differently
    # the same graph handed over as a CSR (swizzle of the transpose's CSC)
    sw = F.swizzle(F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), W.T), 2, 1)
    np.testing.assert_allclose(examples.pagerank(sw, nsteps=20).todense(), want, rtol=1e-12, atol=0)


def test_pagerank_refuses_a_vertex_without_out_edges(gpu_lib):
    g = fsprand(np.random.default_rng(4), 50, 50, 0.02)
    assert (np.diff(g.ptr) == 0).any()
    edges = F.pattern(F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))), g))
    with pytest.raises(F.FinchGBUnsupported, match="0/0"):
        examples.pagerank(edges)
    assert np.isnan(oracle.pagerank(50, g.ptr, g.idx)).any()  # what Finch's nest would give


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("vt", [np.float64, np.float32, np.int32, np.int64, np.bool_, None])
def test_sparse_scale_types_axes_orientations(gpu_lib, orient, vt):
    rng = np.random.default_rng(7)
    m, n = 120, 90
    M = np.where(rng.random((m, n)) < 0.1, rng.integers(1, 9, (m, n)), 0)
    vals = None if vt is None else M.astype(vt)
    b = csc_of(M) if orient == "csc" else csc_of(M.T)
    ptr, idx, _ = b
    nz = np.nonzero(M.T)[::-1] if orient == "csc" else np.nonzero(M)
    ent = None if vt is None else (vals[nz] if orient == "csr" else vals[nz])
    A = dev.DeviceSparse.from_host(m, n, ptr, idx, ent, orient=orient, base=1)
    rows_by = torch.tensor(rng.integers(1, 5, m), device="cuda")  # int64
    cols_by = torch.tensor(rng.random(n) + 0.5, dtype=torch.float32, device="cuda")
    keep = torch.tensor(rng.random(n) < 0.7, dtype=torch.uint8, device="cuda")
    Mv = (M != 0).astype(np.float64) if vt in (None, np.bool_) else M.astype(np.float64)
    # A[i, j] / cols_by[j] where keep[j] (F32 with F32 stays F32 unless A is F64)
    res, changed = dev.sparse_scale(A, cols_by, L.AXIS_COL, keep, L.AXIS_COL, L.MAP_DIV, torch.float64)
    assert changed == 0 and res.orient == orient
    got = F.sparse(F.tensors.sparse_from_device(res)).toarray()
    f32 = vt in (np.float32, np.int32, np.int64, np.bool_, None)
    cb = cols_by.cpu().numpy()
    if f32:
        want = (Mv.astype(np.float32) / cb[None, :]).astype(np.float64)
    else:
        want = Mv / cb.astype(np.float64)[None, :]
    want = np.where((M != 0) & (keep.cpu().numpy()[None, :] != 0), want, 0.0)
    assert np.array_equal(got, want)
    assert res.nnz == int(((M != 0) & (keep.cpu().numpy()[None, :] != 0)).sum())
    # A[i, j] * rows_by[i], every entry kept: F64 (an integer vector promotes in F64)
    res, changed = dev.sparse_scale(A, rows_by, L.AXIS_ROW, None, L.AXIS_ROW, L.MAP_MUL, torch.float32)
    assert changed == 0 and res.nnz == int((M != 0).sum())
    got = F.sparse(F.tensors.sparse_from_device(res)).toarray()
    mul = Mv.astype(np.float32) * rows_by.cpu().numpy().astype(np.float32)[:, None] if vt == np.float32 else \
        (Mv * rows_by.cpu().numpy()[:, None]).astype(np.float32)
    assert np.array_equal(got, np.where(M != 0, mul, 0.0).astype(np.float32))


def test_sparse_scale_counts_fill_changes_and_edges(gpu_lib):
    A = dev.DeviceSparse.from_host(4, 3, *csc_of(np.array([[1.0, 0, 2], [0, 0, 3], [4, 0, 0], [0, 0, 5]]))[:2],
                                   np.array([1.0, 4.0, 2.0, 3.0, 5.0]), orient="csc", base=1)
    by = torch.tensor([2.0, 0.0, float("nan")], dtype=torch.float64, device="cuda")
    res, changed = dev.sparse_scale(A, by, L.AXIS_COL)
    assert changed == 2  # 0/0 and 0/NaN
    got = F.sparse(F.tensors.sparse_from_device(res)).toarray()
    assert np.array_equal(got[:, 0], [0.5, 0, 2.0, 0]) and np.isnan(got[[0, 1, 3], 2]).all()
    res, changed = dev.sparse_scale(A, torch.tensor([1.0, float("inf"), 2.0], device="cuda", dtype=torch.float64),
                                    L.AXIS_COL, op=L.MAP_MUL)
    assert changed == 1  # 0 * Inf
    empty = dev.DeviceSparse.from_host(5, 4, np.ones(5, np.int64), np.zeros(0, np.int64), np.zeros(0), "csc", 1)
    res, changed = dev.sparse_scale(empty, torch.ones(4, dtype=torch.float64, device="cuda"), L.AXIS_COL)
    assert res.nnz == 0 and res.ptr.cpu().tolist() == [0] * 5
    with pytest.raises(L.FinchGBError):
        dev.sparse_scale(A, by, 7)


@pytest.mark.parametrize("orient", ["csc", "csr"])
def test_pattern_and_bool_reduce_counts(gpu_lib, orient):
    rng = np.random.default_rng(8)
    M = rng.random((60, 45)) < 0.2
    ptr, idx, _ = csc_of(M) if orient == "csc" else csc_of(M.T)
    nz = np.nonzero(M.T)[::-1] if orient == "csc" else np.nonzero(M)
    vals = rng.random(len(nz[0])) < 0.5  # Bool values, some stored false
    Mb = np.zeros_like(M)
    Mb[nz] = vals
    P = dev.DeviceSparse.from_host(60, 45, ptr, idx, None, orient=orient, base=1)
    Bt = dev.DeviceSparse.from_host(60, 45, ptr, idx, vals, orient=orient, base=1)
    for dims, axis in ((1, 0), (2, 1)):
        y = dev.ewise_reduce(dims, P)
        assert y.dtype == torch.int64 and np.array_equal(y.cpu().numpy(), M.sum(axis=axis))
        assert np.array_equal(dev.ewise_reduce(dims, Bt).cpu().numpy(), Mb.sum(axis=axis))
    assert int(dev.ewise_reduce(0, P).item()) == int(M.sum())
    assert int(dev.ewise_reduce(0, Bt).item()) == int(Mb.sum())


def _round_once(q, dt):
    """The value of dt nearest to the rational q, ties to even: one
    rounding, what a fused a*x+b gives."""
    from fractions import Fraction

    f = dt(float(q))
    cands = [f, np.nextafter(f, dt(np.inf)), np.nextafter(f, dt(-np.inf))]
    best = min(cands, key=lambda c: (abs(Fraction(float(c)) - q),
                                     int(np.frombuffer(np.asarray(c, dt).tobytes(), np.uint8)[0]) & 1))
    return best


def test_dense_affine_is_fused(gpu_lib):
    from fractions import Fraction

    rng = np.random.default_rng(9)
    x = rng.standard_normal(2001)
    for dt, npt in ((torch.float64, np.float64), (torch.float32, np.float32)):
        xs, an, bn = x.astype(npt), npt(0.85), npt(0.15 / 7)
        out = dev.dense_affine(torch.tensor(an, device="cuda"), torch.tensor(xs, device="cuda"),
                               torch.tensor(bn, device="cuda"), torch.empty(len(x), dtype=dt, device="cuda"))
        got = out.cpu().numpy()
        want = [_round_once(Fraction(float(an)) * Fraction(float(v)) + Fraction(float(bn)), npt) for v in xs]
        assert np.array_equal(got, np.array(want, dtype=npt))
        fill = dev.dense_affine(None, None, torch.tensor(bn, device="cuda"), torch.empty_like(out)).cpu().numpy()
        assert (fill == bn).all()
