"""The choose/minby graph programs on the GPU, bit-exact against the oracle's
restatement of Finch's loops: single rounds of fgb_bfs_pull, fgb_or_count,
fgb_minby_map and fgb_minby_relax through the C ABI, and the reference's
whole BFS and Bellman-Ford examples (docs/examples/bfs.jl,
shortest_paths.jl) running through finch(...) onto those kernels.  Like
test/suites/examples_tests.jl:33-86, the results are also checked against an
independent BFS and shortest-path computation."""
import heapq

import numpy as np
import pytest
import torch

import finchgb as F
import oracle
from finchgb import device as dev
from finchgb import examples
from finchgb.workloads import fsprand, random_graph
from helpers import to_host, upload

pytestmark = pytest.mark.gpu


def _bfs_oracle(g, source):
    n = g.nrows
    Fr = np.zeros(n, np.uint8)
    Fr[source - 1] = 1
    V, P = Fr.copy(), np.zeros(n, np.int64)
    P[source - 1] = source
    while Fr.any():
        Fr, _ = oracle.bfs_round(n, g.ptr, g.idx, Fr, V, P)
    return P


def _bf_oracle(g, w, source):
    n = g.nrows
    dprev, pprev = np.full(n, np.inf), np.zeros(n, np.int64)
    dprev[source - 1] = 0.0
    dist, par = np.full(n, np.inf), np.zeros(n, np.int64)
    aprev = np.zeros(n, np.uint8)
    aprev[source - 1] = 1
    for _ in range(n):
        act = oracle.minby_round(n, g.ptr, g.idx, w, dprev, pprev, aprev, dist, par)
        if not act.any():
            return dist, par
        dprev, dist = dist, dprev
        pprev, par = par, pprev
        aprev = act
    return dprev, pprev


@pytest.mark.parametrize("n,p", [(300, 0.02), (20000, 0.0004)])
def test_bfs_rounds_bit_exact(gpu_lib, n, p):
    rng = np.random.default_rng(n)
    g = fsprand(rng, n, n, p)  # CSC: column j lists the k with edges[k, j]
    A = upload(g).transposed_storage()  # CSR: row k lists its j
    Fr = np.zeros(n, np.uint8)
    Fr[:3] = 1
    V = Fr.copy()
    P = np.zeros(n, np.int64)
    P[:3] = [1, 2, 3]
    Fd, Vd, Pd = (torch.from_numpy(a.copy()).cuda() for a in (Fr, V, P))
    P32 = torch.from_numpy(P.astype(np.int32)).cuda()
    for _ in range(12):
        nd = dev.bfs_pull(A, Fd, Vd, Pd)
        dev.bfs_pull(A, Fd, Vd, P32)  # the Int32 parent layout: the same numbers
        cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
        dev.or_count(Vd, nd, cnt)
        Fr, c = oracle.bfs_round(n, g.ptr, g.idx, Fr, V, P)
        assert np.array_equal(to_host(nd), Fr) and int(cnt.item()) == c
        assert np.array_equal(to_host(Vd), V) and np.array_equal(to_host(Pd), P)
        assert np.array_equal(to_host(P32), P.astype(np.int32))
        Fd = nd


@pytest.mark.parametrize("wtype", [np.float64, np.float32, np.int32])
def test_minby_rounds_bit_exact(gpu_lib, wtype):
    rng = np.random.default_rng(7)
    n = 5000
    g = random_graph(rng, n, 6.0)
    w = (rng.random(g.nnz) if np.dtype(wtype).kind == "f" else rng.integers(1, 1000, g.nnz)).astype(wtype)
    g.val = w
    A = upload(g).transposed_storage()  # row i lists the j with edges[i, j]
    inf = np.inf if np.dtype(wtype).kind == "f" else 2**30  # an integer sentinel below overflow
    dprev = np.full(n, inf, dtype=wtype)
    dprev[0] = 0
    pprev = np.zeros(n, np.int64)
    aprev = np.zeros(n, np.uint8)
    aprev[0] = 1
    dist, par = np.full(n, inf, dtype=wtype), np.zeros(n, np.int64)
    d_dev = [torch.from_numpy(x.copy()).cuda() for x in (dprev, pprev, dist, par)]
    a_dev = torch.from_numpy(aprev.copy()).cuda()
    for _ in range(10):
        dpd, ppd, dd, pd = d_dev
        dev.minby_map(a_dev, (dpd, ppd), (dd, pd))
        act_d = dev.minby_relax(A, dpd, a_dev, (dd, pd))
        if wtype == np.float32:  # FP32 sums: the same loops read in float32 arithmetic
            d64 = dist.copy()
            act = _relax_f32(n, g, w, dprev, pprev, aprev, d64, par)
        else:  # the oracle's nest (FP64; Int32 sums below 2^31 are exact in it)
            d64 = dist.astype(np.float64)
            act = oracle.minby_round(n, g.ptr, g.idx, w.astype(np.float64), dprev.astype(np.float64), pprev,
                                     aprev, d64, par)
        assert np.array_equal(to_host(act_d), act)
        assert np.array_equal(to_host(dd).astype(np.float64), d64.astype(np.float64))
        assert np.array_equal(to_host(pd), par)
        dist = d64.astype(wtype)
        dprev, dist = dist, dprev
        pprev, par = par, pprev
        aprev = act
        d_dev = [dd, pd, dpd, ppd]
        a_dev = act_d


def _relax_f32(n, g, w, dprev, pprev, aprev, dist, par):
    """shortest_paths.jl:22-40 over float32 values, as written (j outer)."""
    for j in range(n):
        if aprev[j] and dist[j] > dprev[j]:
            dist[j], par[j] = dprev[j], pprev[j]
    act = np.zeros(n, np.uint8)
    for j in np.flatnonzero(aprev):
        for q in range(g.ptr[j] - 1, g.ptr[j + 1] - 1):
            i = g.idx[q] - 1
            d = np.float32(dprev[j]) + np.float32(w[q])
            if dist[i] > d:
                dist[i], par[i] = d, j + 1
            act[i] |= np.uint8(d < dprev[i])
    return act


def test_minby_relax_rejects(gpu_lib):
    g = random_graph(np.random.default_rng(1), 100, 3.0)
    g.val = np.random.default_rng(2).random(g.nnz)
    A = upload(g).transposed_storage()
    d = torch.zeros(100, dtype=torch.float64, device="cuda")
    p = torch.zeros(100, dtype=torch.int64, device="cuda")
    a = torch.zeros(100, dtype=torch.uint8, device="cuda")
    with pytest.raises(F.FinchGBError):
        dev.minby_relax(A, d, a, (d, p))  # dist_prev and dist alias
    with pytest.raises(F.FinchGBError):
        dev.minby_relax(upload(g), torch.zeros_like(d), a, (d, p))  # CSC: needs the rows


def _level_bfs_parents(g, source):
    """An independent BFS: vertices by level, each parent the smallest
    previous-level vertex with an edge to it."""
    n = g.nrows
    nbrs = [g.idx[g.ptr[j] - 1: g.ptr[j + 1] - 1] - 1 for j in range(n)]  # column j -> its k
    P = np.zeros(n, np.int64)
    P[source - 1] = source
    frontier = [source - 1]
    while frontier:
        nxt = {}
        for j in sorted(frontier):
            for k in nbrs[j]:
                if P[k] == 0 and k not in nxt:
                    nxt[k] = j + 1
        for k, j in nxt.items():
            P[k] = j
        frontier = list(nxt)
    return P


@pytest.mark.parametrize("n,p,seed", [(50, 0.5, 3), (400, 0.01, 4), (3000, 0.002, 5)])
def test_bfs_example_through_finch(gpu_lib, n, p, seed):
    rng = np.random.default_rng(seed)
    g = fsprand(rng, n, n, p)
    source = int(rng.integers(1, n + 1))
    edges = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))), g)
    P = examples.bfs(edges, source)
    got = P.todense()
    assert np.array_equal(got, _bfs_oracle(g, source))
    assert np.array_equal(got, _level_bfs_parents(g, source))


def _dijkstra(g, w, source):
    n = g.nrows
    dist = np.full(n, np.inf)
    dist[source - 1] = 0.0
    h = [(0.0, source - 1)]
    while h:
        d, j = heapq.heappop(h)
        if d > dist[j]:
            continue
        for q in range(g.ptr[j] - 1, g.ptr[j + 1] - 1):
            i = g.idx[q] - 1
            nd = d + w[q]
            if nd < dist[i]:
                dist[i] = nd
                heapq.heappush(h, (nd, i))
    return dist


@pytest.mark.parametrize("n,p,seed", [(50, 0.5, 6), (800, 0.006, 8)])
def test_bellmanford_example_through_finch(gpu_lib, n, p, seed):
    rng = np.random.default_rng(seed)
    g = fsprand(rng, n, n, p)
    source = int(rng.integers(1, n + 1))
    edges = F.set_fill_value(F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))), g), np.inf)
    out = examples.bellmanford(edges, source).todense()
    d_or, p_or = _bf_oracle(g, g.val, source)
    assert np.array_equal(out["f0"], d_or) and np.array_equal(out["f1"], p_or)
    assert np.allclose(out["f0"], _dijkstra(g, g.val, source), rtol=1e-12, atol=0)
