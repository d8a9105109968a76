"""The choose/minby graph programs on the host: the @finch parser reads the
reference's BFS and Bellman-Ford programs (docs/examples/bfs.jl,
shortest_paths.jl), the matchers bind them and refuse altered ones, and the
oracle's restatement of each round equals a direct Python reading of the
same loops on small random graphs."""
import numpy as np
import pytest

import oracle
from finchgb import examples, notation, programs
from finchgb.workloads import fsprand


def test_parser_reads_the_reference_programs():
    for src in (examples.BFS_ROUND, examples.BFS_COUNT, examples.RELAX_KEEP, examples.RELAX):
        assert notation.stmts(notation.parse(src))
    tree = notation.parse("y .= 0; for j=_, i=_; y[i] += A[i,j]*x[j] end")
    init, loop = notation.stmts(tree)
    assert isinstance(init, notation.Init) and init.name == "y"
    assert isinstance(loop, notation.Loop) and loop.idx == "j" and loop.body.idx == "i"
    with pytest.raises(SyntaxError):
        notation.parse("for j = 1:10; y[j] = 1 end")


def test_matchers_bind_names():
    m = programs.match_bfs_round(notation.parse(examples.BFS_ROUND))
    assert m == {"next": "_F", "frontier": "F", "edges": "edges", "visited": "V", "parent": "P", "fill": 0}
    assert programs.match_or_count(notation.parse(examples.BFS_COUNT)) == {"next": "_F", "visited": "V",
                                                                            "count": "c"}
    assert programs.match_minby_map(notation.parse(examples.RELAX_KEEP)) == {
        "mask": "active_prev", "dst": "dists", "src": "dists_prev"}
    assert programs.match_minby_relax(notation.parse(examples.RELAX)) == {
        "active": "active", "active_prev": "active_prev", "dist_prev": "dists_prev", "edges": "edges",
        "dist": "dists"}
    # renamed tensors and indices still match
    renamed = examples.BFS_ROUND.replace("edges", "G").replace("P[", "parent[").replace("j", "u")
    assert programs.match_bfs_round(notation.parse(renamed))["parent"] == "parent"


@pytest.mark.parametrize("src", [
    examples.BFS_ROUND.replace("!(V[k])", "V[k]"),           # not the visited test
    examples.BFS_ROUND.replace("choose(0)", "min"),         # another reduction
    examples.BFS_ROUND.replace("edges[k, j]", "edges[j, k]"),  # transposed access
    examples.RELAX.replace("(d, j)", "(d, i)"),             # the wrong parent
    examples.RELAX.replace("d < first(dists_prev[i])", "d < first(dists_prev[j])"),
])
def test_matchers_refuse_other_programs(src):
    t = notation.parse(src)
    assert all(f(t) is None for f in (programs.match_bfs_round, programs.match_or_count,
                                     programs.match_minby_map, programs.match_minby_relax))


def _py_bfs_round(n, ptr, idx, F, V, P):
    """bfs.jl:25-42 read directly: j outer, k over column j."""
    nF = [0] * n
    for j in range(n):
        for q in range(ptr[j] - 1, ptr[j + 1] - 1):
            k = idx[q] - 1
            if F[j] and not V[k]:
                nF[k] = 1
                P[k] = j + 1 if P[k] == 0 else P[k]  # choose(0)
    c = 0
    for k in range(n):
        V[k] |= nF[k]
        c += nF[k]
    return nF, c


def _py_relax(n, ptr, idx, w, dprev, pprev, aprev, dist, par):
    """shortest_paths.jl:22-40 read directly, minby(a, b) = a[1] > b[1] ? b : a."""
    for j in range(n):
        if aprev[j] and dist[j] > dprev[j]:
            dist[j], par[j] = dprev[j], pprev[j]
    act = [0] * n
    for j in range(n):
        if not aprev[j]:
            continue
        for q in range(ptr[j] - 1, ptr[j + 1] - 1):
            i = idx[q] - 1
            d = dprev[j] + w[q]
            if dist[i] > d:
                dist[i], par[i] = d, j + 1
            act[i] |= int(d < dprev[i])
    return act


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_rounds_equal_direct_reading(seed):
    rng = np.random.default_rng(seed)
    n = 60
    g = fsprand(rng, n, n, 0.08)
    src = int(rng.integers(n))
    F = np.zeros(n, np.uint8)
    F[src] = 1
    V, P = F.copy(), np.zeros(n, np.int64)
    P[src] = src + 1
    Fp, Vp, Pp = F.tolist(), V.tolist(), P.tolist()
    for _ in range(8):
        F, c = oracle.bfs_round(n, g.ptr, g.idx, F, V, P)
        Fp, cp = _py_bfs_round(n, g.ptr.tolist(), g.idx.tolist(), Fp, Vp, Pp)
        assert F.tolist() == Fp and c == cp and V.tolist() == Vp and P.tolist() == Pp
    w = rng.random(g.nnz)
    dprev = np.full(n, np.inf)
    dprev[src] = 0.0
    pprev = np.zeros(n, np.int64)
    aprev = np.zeros(n, np.uint8)
    aprev[src] = 1
    dist, par = np.full(n, np.inf), np.zeros(n, np.int64)
    for _ in range(6):
        d_py, p_py = dist.tolist(), par.tolist()
        act_py = _py_relax(n, g.ptr.tolist(), g.idx.tolist(), w.tolist(), dprev.tolist(), pprev.tolist(),
                           aprev.tolist(), d_py, p_py)
        act = oracle.minby_round(n, g.ptr, g.idx, w, dprev, pprev, aprev, dist, par)
        assert act.tolist() == act_py and dist.tolist() == d_py and par.tolist() == p_py
        dprev, dist = dist, dprev
        pprev, par = par, pprev
        aprev = act
