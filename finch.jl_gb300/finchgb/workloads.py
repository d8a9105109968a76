"""Seeded synthetic inputs with the shapes and distributions of the
benchmark configurations (numpy PCG64; no datasets are downloaded).

All generators return Finch level buffers: 1-based Int64 `ptr`/`idx` of a
SparseList level plus the Element values, fibers sorted ascending and free
of duplicate coordinates (SparseList's invariant,
src/tensors/levels/sparse_list_levels.jl:37-53).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SparseBuffers:
    """Host level buffers of a 2-D SparseList matrix (Finch layout).

    Finch's own buffers are 1-based Int64 (`base` 1).  Buffers mapped from
    scipy.sparse keep its 0-based int32/int64 arrays (`base` 0), as Finch
    reads 0-based buffers through PlusOneVector (src/util/vectors.jl:3-37)."""

    nrows: int
    ncols: int
    ptr: np.ndarray  # nfibers + 1 offsets, ptr[0] == base
    idx: np.ndarray  # coordinates counted from base
    val: np.ndarray | None
    orient: str  # "csc" (fibers = columns) or "csr" (fibers = rows)
    base: int = 1

    @property
    def nnz(self) -> int:
        return int(self.idx.size)

    @property
    def nfibers(self) -> int:
        return self.ncols if self.orient == "csc" else self.nrows

    def todense(self) -> np.ndarray:
        dt = np.float64 if self.val is None else self.val.dtype
        out = np.zeros((self.nrows, self.ncols), dtype=dt)
        f = np.repeat(np.arange(self.nfibers), np.diff(self.ptr))
        c = np.asarray(self.idx, dtype=np.int64) - self.base
        v = 1 if self.val is None else self.val
        if self.orient == "csc":
            out[c, f] = v
        else:
            out[f, c] = v
        return out


def _fibers_from_lengths(rng, lengths: np.ndarray, extent: int) -> np.ndarray:
    """Sorted, duplicate-free coordinates (0-based) for fibers of the given
    lengths, uniform without replacement inside each fiber."""
    nf = lengths.size
    nnz = int(lengths.sum())
    fib = np.repeat(np.arange(nf, dtype=np.int64), lengths)
    coord = rng.integers(0, extent, size=nnz, dtype=np.int64)
    while True:
        key = fib * extent + coord
        order = np.argsort(key, kind="stable")
        key = key[order]
        coord = coord[order]
        dup = np.zeros(nnz, dtype=bool)
        dup[1:] = key[1:] == key[:-1]
        nd = int(dup.sum())
        if nd == 0:
            return coord
        coord[dup] = rng.integers(0, extent, size=nd, dtype=np.int64)


def _ptr(lengths: np.ndarray) -> np.ndarray:
    p = np.empty(lengths.size + 1, dtype=np.int64)
    p[0] = 1
    np.cumsum(lengths, out=p[1:])
    p[1:] += 1
    return p


def fsprand(rng: np.random.Generator, m: int, n: int, p: float, dtype=np.float64,
            nnz: int | None = None) -> SparseBuffers:
    """Finch's fsprand (src/interface/fsparse.jl:173-290) as a CSC matrix:
    nnz ~ Binomial(m*n, p), positions uniform without replacement, values
    U[0,1).  Same distribution as Finch's sampler, not the same stream."""
    if nnz is None:
        nnz = int(rng.binomial(m * n, p))
    lin = np.unique(rng.integers(0, m * n, size=nnz, dtype=np.int64))
    while lin.size < nnz:
        extra = rng.integers(0, m * n, size=nnz - lin.size, dtype=np.int64)
        lin = np.unique(np.concatenate([lin, extra]))
    # column-major order: j = lin // m, i = lin % m (sorted by (j, i))
    j = lin // m
    i = lin % m
    lengths = np.bincount(j, minlength=n).astype(np.int64)
    if np.dtype(dtype).kind == "f":
        val = rng.random(nnz).astype(dtype)
    elif np.dtype(dtype) == np.bool_:
        val = np.ones(nnz, dtype=np.bool_)
    else:
        val = rng.integers(1, 10, size=nnz).astype(dtype)
    return SparseBuffers(m, n, _ptr(lengths), i + 1, val, "csc")


def zipf_csr(rng: np.random.Generator, m: int, n: int, mean: float = 16.0, a: float = 1.5,
             cap: int = 50_000, dtype=np.float32) -> SparseBuffers:
    """CSR with power-law row lengths: Zipf(a) draws capped at `cap`, then
    rescaled by stochastic rounding so the total is exactly m*mean; columns
    uniform without replacement per row; values N(0,1)."""
    raw = np.minimum(rng.zipf(a, size=m), cap).astype(np.float64)
    target = int(round(m * mean))
    scaled = raw * (target / raw.sum())
    lengths = np.floor(scaled).astype(np.int64)
    lengths += (rng.random(m) < (scaled - lengths)).astype(np.int64)
    diff = target - int(lengths.sum())
    if diff > 0:
        lengths[rng.choice(m, size=diff, replace=False)] += 1
    elif diff < 0:
        nz = np.flatnonzero(lengths)
        lengths[rng.choice(nz, size=-diff, replace=False)] -= 1
    lengths = np.minimum(lengths, n)
    coord = _fibers_from_lengths(rng, lengths, n)
    val = rng.standard_normal(int(lengths.sum()), dtype=np.float64).astype(dtype)
    return SparseBuffers(m, n, _ptr(lengths), coord + 1, val, "csr")


def random_graph(rng: np.random.Generator, n: int, mean_degree: float = 8.0,
                 wmax: int = 1000, pattern: bool = False) -> SparseBuffers:
    """Directed graph as Finch's adjacency Dense(SparseList(Element)):
    column j holds node j's out-edges (rows = targets).  Out-degree
    ~ Poisson(mean_degree), targets uniform (no duplicate edges), Int32
    weights U{1..wmax} (or no values for a Pattern level)."""
    lengths = np.minimum(rng.poisson(mean_degree, size=n), n).astype(np.int64)
    coord = _fibers_from_lengths(rng, lengths, n)
    val = None if pattern else rng.integers(1, wmax + 1, size=coord.size, dtype=np.int32)
    return SparseBuffers(n, n, _ptr(lengths), coord + 1, val, "csc")


def poisson2d(N: int, dtype=np.float64) -> SparseBuffers:
    """2-D 5-point Poisson matrix on an N x N grid (n = N^2), CSR, values 4
    on the diagonal and -1 off it, columns ascending in every row."""
    n = N * N
    r = np.arange(n, dtype=np.int64)
    gi, gj = r // N, r % N
    cols, rows, vals = [], [], []
    for di, dj, v in ((-1, 0, -1.0), (0, -1, -1.0), (0, 0, 4.0), (0, 1, -1.0), (1, 0, -1.0)):
        ok = (gi + di >= 0) & (gi + di < N) & (gj + dj >= 0) & (gj + dj < N)
        rows.append(r[ok])
        cols.append(r[ok] + di * N + dj)
        vals.append(np.full(int(ok.sum()), v))
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    vals = np.concatenate(vals)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    lengths = np.bincount(rows, minlength=n).astype(np.int64)
    return SparseBuffers(n, n, _ptr(lengths), cols + 1, vals.astype(dtype), "csr")


def csr_from_dense(D: np.ndarray) -> SparseBuffers:
    """CSR buffers of the nonzeros of a dense matrix."""
    rows, cols = np.nonzero(D)
    lengths = np.bincount(rows, minlength=D.shape[0]).astype(np.int64)
    return SparseBuffers(D.shape[0], D.shape[1], _ptr(lengths), cols.astype(np.int64) + 1,
                         D[rows, cols], "csr")


def csc_from_dense(D: np.ndarray) -> SparseBuffers:
    """CSC buffers (Finch's Dense(SparseList(Element))) of a dense matrix."""
    cols, rows = np.nonzero(D.T)
    lengths = np.bincount(cols, minlength=D.shape[1]).astype(np.int64)
    return SparseBuffers(D.shape[0], D.shape[1], _ptr(lengths), rows.astype(np.int64) + 1,
                         D[rows, cols], "csc")


def coo_to_csr(m: int, n: int, I: np.ndarray, J: np.ndarray, V: np.ndarray) -> SparseBuffers:
    """CSR buffers from 1-based COO triplets (duplicates summed)."""
    key = (np.asarray(I, np.int64) - 1) * n + (np.asarray(J, np.int64) - 1)
    uk, inv = np.unique(key, return_inverse=True)
    v = np.zeros(uk.size, dtype=np.asarray(V).dtype)
    np.add.at(v, inv, V)
    rows, cols = uk // n, uk % n
    lengths = np.bincount(rows, minlength=m).astype(np.int64)
    return SparseBuffers(m, n, _ptr(lengths), cols + 1, v, "csr")
