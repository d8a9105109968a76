"""Finch's graph examples written against this package's Finch API, so that
their @finch programs run through the matcher onto the GPU kernels:

  bfs(edges, source)          docs/examples/bfs.jl
  bellmanford(edges, source)  docs/examples/shortest_paths.jl

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
