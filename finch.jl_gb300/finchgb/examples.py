"""Finch's graph examples written against this package's Finch API, so that
their @finch programs run through the matcher onto the GPU kernels:

  bfs(edges, source)          docs/examples/bfs.jl
  bellmanford(edges, source)  docs/examples/shortest_paths.jl
  pagerank(edges, nsteps, damp)  docs/examples/pagerank.jl

The programs are the reference's, statement for statement; vertex numbers
are 1-based as in Finch.  Each round's tensors stay in HBM between the
@finch calls.
"""
from __future__ import annotations

import numpy as np

from .scheduler import Scalar, finch
from .tensors import Dense, Element, Pattern, SparseByteMap, Tensor, pattern

BFS_ROUND = """
    _F .= false
    for j=_, k=_
        if F[j] && edges[k, j] && !(V[k])
            _F[k] |= true
            P[k] << choose(0) >>= j #Only set the parent for this vertex
        end
    end
"""

BFS_COUNT = """
    for k=_
        let _f = _F[k]
            V[k] |= _f
            c[] += _f
        end
    end
"""

RELAX_KEEP = """
    for j=_
        if active_prev[j]
            dists[j] << minby >>= dists_prev[j]
        end
    end
"""

RELAX = """
    active .= false
    for j=_
        if active_prev[j]
            for i=_
                let d = first(dists_prev[j]) + edges[i, j]
                    dists[i] << minby >>= (d, j)
                    active[i] |= d < first(dists_prev[i])
                end
            end
        end
    end
"""


OUT_DEGREE = """
    out_degree .= 0
    for j=_, i=_
        out_degree[j] += edges[i, j]
    end
"""

SCALE_EDGES = """
    scaled_edges .= 0
    for j=_, i=_
        if out_degree[i] != 0
            scaled_edges[i, j] = edges[i, j] / out_degree[j]
        end
    end
"""

RANK_INIT = """
    r .= 0.0
    for j=_
        r[j] = 1.0 / n
    end
"""

RANK_STEP = """
    rank .= 0
    for j=_, i=_
        rank[i] += scaled_edges[i, j] * r[j]
    end
"""

RANK_DAMP = """
    r .= 0.0
    for i=_
        r[i] = beta_score + damp * rank[i]
    end
"""


def pagerank(edges, nsteps: int = 20, damp: float = 0.85) -> Tensor:
    """`nsteps` steps of PageRank on the adjacency matrix `edges` (edges[i, j]
    an edge j -> i), as pagerank.jl computes it: out-degrees, the masked
    transition matrix, then rank = scaled_edges * r and r = beta + damp * rank
    per step.  The rank sums run in Finch's serial order.  A vertex without
    out-edges makes pagerank.jl divide 0 by 0 where `edges` stores nothing;
    that program is refused (FinchGBUnsupported)."""
    n, m = edges.shape
    assert n == m
    out_degree = finch(OUT_DEGREE, edges=edges)["out_degree"]
    scaled_edges = finch(SCALE_EDGES, edges=edges, out_degree=out_degree)["scaled_edges"]
    r = finch(RANK_INIT, r=Tensor(Dense(Element(0.0)), shape=(n,)), n=n)["r"]
    rank = Tensor(Dense(Element(0.0)), shape=(n,))
    beta_score = (1 - damp) / n
    for _ in range(nsteps):
        rank = finch(RANK_STEP, rank=rank, scaled_edges=scaled_edges, r=r)["rank"]
        r = finch(RANK_DAMP, r=r, beta_score=beta_score, damp=damp, rank=rank)["r"]
    return r


def bfs(edges, source: int = 5) -> Tensor:
    """Breadth-first search from `source`: the parent of every vertex (0
    where unreached), as bfs.jl numbers them."""
    n, m = edges.shape
    assert n == m
    edges = pattern(edges)
    F = Tensor(SparseByteMap(Pattern()), shape=(n,))
    _F = Tensor(SparseByteMap(Pattern()), shape=(n,))
    F[source] = True
    F_nnz = 1
    V = Tensor(Dense(Element(False)), shape=(n,))
    V[source] = True
    P = Tensor(Dense(Element(0)), shape=(n,))
    P[source] = source
    while F_nnz > 0:
        _F = finch(BFS_ROUND, F=F, _F=_F, edges=edges, V=V, P=P)["_F"]
        c = Scalar(0, dtype=np.int64)
        finch(BFS_COUNT, _F=_F, V=V, c=c)
        F, _F = _F, F
        F_nnz = int(c.value)
    return P


def bellmanford(edges, source: int = 1) -> Tensor:
    """Shortest paths from `source` over the weights `edges` (fill Inf =
    unconnected): a vector of (distance, parent) pairs."""
    n, m = edges.shape
    assert n == m
    dt = np.dtype(edges.body.dtype if hasattr(edges, "body") else edges.dtype)
    inf = np.array(np.inf, dtype=dt)[()]
    dists_prev = Tensor(Dense(Element((inf, 0))), shape=(n,))
    dists_prev[source] = (0.0, 0)
    dists = Tensor(Dense(Element((inf, 0))), shape=(n,))
    active_prev = Tensor(SparseByteMap(Pattern()), shape=(n,))
    active_prev[source] = True
    active = Tensor(SparseByteMap(Pattern()), shape=(n,))
    for _ in range(n):
        finch(RELAX_KEEP, active_prev=active_prev, dists=dists, dists_prev=dists_prev)
        active = finch(RELAX, active=active, active_prev=active_prev, dists_prev=dists_prev, edges=edges,
                       dists=dists)["active"]
        if not bool(active.ddata.any()):
            return dists
        dists_prev, dists = dists, dists_prev
        active_prev, active = active, active_prev
    return dists_prev
