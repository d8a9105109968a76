"""Finch's tensor construction API over level formats, host and device.

Mirrors the constructors of Finch.jl's levels and Tensor wrapper:

    Tensor(Dense(SparseList(Element(0.0))), A)      # CSC (Finch's CSCFormat)
    Tensor(Dense(SparseList(Pattern())), A)         # Boolean pattern
    Tensor(Dense(Element(0.0)), x)                  # dense vector
    Tensor(Dense(Dense(Element(0.0))), B)           # dense matrix
    Tensor(SparseCOO(2, Element(0.0)), A)           # COO
    swizzle(Tensor(Dense(SparseList(Element(0.0))), A.T), 2, 1)  # CSR of A

(src/tensors/levels/{dense,sparse_list,sparse_coo,element,pattern}_levels.jl,
src/tensors/tensors.jl:10-69, src/tensors/combinators/swizzle.jl:1-58,
src/Finch.jl:188-258).  Host buffers use Finch's layout (1-based Int64
ptr/idx).  `Tensor(A)` of a scipy.sparse matrix keeps A's own 0-based
buffers, as Finch's Tensor(::SparseMatrixCSC) does, and `sparse(t)` gives
a scipy.sparse matrix back (ext/SparseArraysExt.jl).  `transfer(gpu(), t)`
moves the level buffers into HBM once (narrowing Int64 idx to int32);
tensors then stay resident across calls.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .workloads import SparseBuffers, csc_from_dense


# ---------------------------------------------------------------- levels


def pair_dtype(fill) -> np.dtype:
    """The element type of a 2-tuple fill value such as (Inf, 0): a record of
    the two components' types (Finch's Tuple{Float64, Int64} elements)."""
    a, b = fill
    return np.dtype([("f0", np.asarray(a).dtype), ("f1", np.asarray(b).dtype)])


@dataclass(frozen=True)
class Element:
    """Leaf level holding values; `fill_value` is the implicit value (a
    2-tuple fill gives tuple elements, e.g. the (distance, parent) pairs of
    docs/examples/shortest_paths.jl)."""

    fill_value: object = 0.0
    dtype: object = None

    def eltype(self):
        if self.dtype is not None:
            return np.dtype(self.dtype)
        if isinstance(self.fill_value, tuple):
            return pair_dtype(self.fill_value)
        return np.asarray(self.fill_value).dtype


@dataclass(frozen=True)
class Pattern:
    """Leaf level of a Boolean structure: stored entries are true, fill false."""

    fill_value: bool = False

    def eltype(self):
        return np.dtype(np.bool_)


@dataclass(frozen=True)
class SparseList:
    """Compressed fiber level (ptr/idx)."""

    lvl: object
    index_type: object = np.int64

    def eltype(self):
        return self.lvl.eltype()

    @property
    def fill_value(self):
        return self.lvl.fill_value


@dataclass(frozen=True)
class Dense:
    """Dense fiber level."""

    lvl: object

    def eltype(self):
        return self.lvl.eltype()

    @property
    def fill_value(self):
        return self.lvl.fill_value


@dataclass(frozen=True)
class SparseCOO:
    """N-d coordinate list level."""

    ndim: int
    lvl: object

    def eltype(self):
        return self.lvl.eltype()

    @property
    def fill_value(self):
        return self.lvl.fill_value


@dataclass(frozen=True)
class SparseByteMap:
    """Finch's SparseByteMap level over a Pattern (a Boolean vector with a
    byte per coordinate, src/tensors/levels/sparse_bytemap_levels.jl): in
    HBM it is the dense byte table itself, which is what the graph kernels
    read; the list of set coordinates is not kept."""

    lvl: object

    def eltype(self):
        return np.dtype(np.bool_)

    @property
    def fill_value(self):
        return False


def _kind(fmt) -> str:
    if isinstance(fmt, Dense) and isinstance(fmt.lvl, (Element, Pattern)):
        return "dense1"
    if isinstance(fmt, SparseByteMap) and isinstance(fmt.lvl, Pattern):
        return "dense1"
    if isinstance(fmt, Dense) and isinstance(fmt.lvl, Dense):
        return "dense2"
    if isinstance(fmt, Dense) and isinstance(fmt.lvl, SparseList):
        return "csc"
    if isinstance(fmt, SparseList) and isinstance(fmt.lvl, (Element, Pattern)):
        return "sparse1"
    if isinstance(fmt, SparseCOO) and fmt.ndim == 2:
        return "coo"
    raise NotImplementedError(f"level format {fmt} is outside the GB300 backend's formats")


# ---------------------------------------------------------------- tensors


def _eager(op: str, a, b):
    """compute() of a lazy `a op b` (src/interface/eager.jl:82-143): numbers
    stay scalars, arrays and scipy.sparse matrices become tensors."""
    from .logic import LazyTensor, lazy
    from .scheduler import compute

    def lz(x):
        if isinstance(x, (int, float, np.integer, np.floating)) and not isinstance(x, (bool, np.bool_)):
            return x
        if not isinstance(x, (Tensor, SwizzleArray)):
            sp_x = _scipy_sparse(x)
            if sp_x is not None:
                x = Tensor(sp_x)
            else:
                x = np.asarray(x)
                el = Element(x.dtype.type(0))
                x = Tensor(Dense(el) if x.ndim == 1 else Dense(Dense(el)), x)
        return lazy(x)

    la, lb = lz(a), lz(b)
    if op == "@":
        return compute(la @ lb)
    if not isinstance(la, LazyTensor):  # a number on the left: put the tensor first
        if op == "-":
            return compute(lb * -1 + la)  # c - x = c + (-1) * x, exactly
        la, lb = lb, la
    elif op == "-" and not isinstance(lb, LazyTensor):
        return compute(la + (-lb))  # x - c = x + (-c), exactly
    if op == "+":
        return compute(la + lb)
    if op == "-":
        return compute(la - lb)
    return compute(la * lb)


class _EagerOps:
    """Finch's eager operations on tensors (src/interface/eager.jl:82-143),
    each the compute() of its lazy form.  `a @ b` is Julia's `a * b` between
    tensors, tensordot over a's last and b's first index (SpMV, SpMM or
    SpGEMM); `a * b` is Julia's `a .* b` (with a number, a scale); `+` and
    `-` are elementwise."""

    def __matmul__(self, other):
        return _eager("@", self, other)

    def __rmatmul__(self, other):
        return _eager("@", other, self)

    def __add__(self, other):
        return _eager("+", self, other)

    def __radd__(self, other):
        return _eager("+", other, self)

    def __sub__(self, other):
        return _eager("-", self, other)

    def __rsub__(self, other):
        return _eager("-", other, self)

    def __mul__(self, other):
        return _eager("*", self, other)

    def __rmul__(self, other):
        return _eager("*", other, self)

    def sum(self, dims=None):
        """sum(A; dims) (src/interface/eager.jl:149): dims 1 sums over rows,
        2 over columns, None everything (a Scalar)."""
        from .logic import lazy
        from .scheduler import compute

        return compute(lazy(self).sum(dims=dims))

    def maximum(self, dims=None):
        """maximum(A; dims) (src/interface/eager.jl:156-158): reduce(max, A; dims),
        the fill counted where nothing is stored."""
        from .logic import lazy, reduce
        from .scheduler import compute

        return compute(reduce("max", lazy(self), dims))

    def minimum(self, dims=None):
        """minimum(A; dims) (src/interface/eager.jl:153-155): reduce(min, A; dims)."""
        from .logic import lazy, reduce
        from .scheduler import compute

        return compute(reduce("min", lazy(self), dims))


class Tensor(_EagerOps):
    """A Finch tensor: a level format plus its buffers (host or device).

    Storage by kind:
      dense1/dense2   `data` (numpy, logical shape) / `ddata` (torch, row-major)
      csc             `buf` (SparseBuffers, orient csc) / `dsparse` (DeviceSparse)
      sparse1         a 1 x n CSR in `buf` / `dsparse`
      coo             COO triplets (converted to CSC on transfer)
    """

    def __init__(self, fmt, arr=None, shape=None, _buf=None):
        sp_in = _scipy_sparse(fmt) if arr is None and _buf is None else None
        if sp_in is not None:  # Tensor(A): the scipy.sparse matrix's own buffers
            fmt, _buf = _map_scipy(sp_in)
        self.fmt = fmt
        self.kind = _kind(fmt)
        self.fill_value = fmt.fill_value
        self.dtype = fmt.eltype()
        self.data = None
        self.buf: SparseBuffers | None = _buf
        self.ddata = None
        self.dsparse = None
        self.coo = None
        self.combine = "+"
        if _buf is not None:
            self.shape = (_buf.nrows, _buf.ncols) if self.kind != "sparse1" else (_buf.ncols,)
            return
        if arr is None:
            if shape is None:
                raise ValueError("Tensor needs an array or a shape")
            if self.kind in ("csc", "coo") and len(shape) == 2:  # an empty sparse matrix, no dense form
                self.shape = tuple(map(int, shape))
                m, n = self.shape
                if self.kind == "coo":
                    e = np.zeros(0, np.int64)
                    self.coo = (e, e, np.zeros(0, self.dtype))
                else:
                    val = None if isinstance(self.fmt.lvl.lvl, Pattern) else np.zeros(0, self.dtype)
                    self.buf = SparseBuffers(m, n, np.ones(n + 1, np.int64), np.zeros(0, np.int64), val, "csc")
                return
            if self.dtype.names:
                arr = np.empty(shape, dtype=self.dtype)
                arr[...] = tuple(self.fill_value)
            else:
                arr = np.full(shape, self.fill_value, dtype=self.dtype)
        if isinstance(arr, (Tensor, SwizzleArray)):
            # a sparse source with the same fill: its stored entries only
            # (dropfills!, src/interface/copy.jl:77-113), no dense intermediate
            if (self.kind in ("csc", "coo") and arr.kind == "csc" and not self.dtype.names
                    and _same_fill(arr.fill_value, self.fill_value)):
                M = _stored_scipy(arr)
                if M is not None:
                    self._from_scipy(M)
                    return
            arr = arr.todense()
        if self.dtype.names:  # tuple elements: a record array
            arr = np.asarray(arr, dtype=self.dtype)
            assert arr.ndim == 1 and self.kind == "dense1", "tuple elements: Dense(Element((a, b))) vectors"
            self.shape = tuple(arr.shape)
            self.data = np.ascontiguousarray(arr)
            return
        sp_in = _scipy_sparse(arr)
        if sp_in is not None and self.kind in ("csc", "coo") and not np.any(np.asarray(self.fill_value)):
            self._from_scipy(sp_in)
            return
        arr = _as_array(arr, self.dtype)
        self.shape = tuple(arr.shape)
        fill = np.asarray(self.fill_value, dtype=self.dtype)
        if self.kind == "dense1":
            assert arr.ndim == 1, "Dense(Element) holds a vector"
            self.data = np.ascontiguousarray(arr)
        elif self.kind == "dense2":
            assert arr.ndim == 2
            self.data = np.ascontiguousarray(arr)
        elif self.kind == "csc":
            assert arr.ndim == 2
            # stored: every entry that differs from the fill (a 0 is stored when the fill is not 0)
            mask = arr != fill
            cols, rows = np.nonzero(mask.T)
            lengths = np.bincount(cols, minlength=arr.shape[1]).astype(np.int64)
            ptr = np.empty(arr.shape[1] + 1, dtype=np.int64)
            ptr[0] = 1
            np.cumsum(lengths, out=ptr[1:])
            ptr[1:] += 1
            val = None if isinstance(fmt.lvl.lvl, Pattern) else arr[rows, cols].astype(self.dtype)
            self.buf = SparseBuffers(arr.shape[0], arr.shape[1], ptr, rows.astype(np.int64) + 1, val, "csc")
        elif self.kind == "sparse1":
            assert arr.ndim == 1
            nz = np.flatnonzero(arr != fill)
            self.buf = SparseBuffers(1, arr.size, np.array([1, nz.size + 1], np.int64),
                                     nz.astype(np.int64) + 1,
                                     None if isinstance(fmt.lvl, Pattern) else arr[nz].astype(self.dtype),
                                     "csr")
        elif self.kind == "coo":
            I, J = np.nonzero(arr != fill)
            order = np.lexsort((I, J))  # Finch sorts by reverse coordinates (column-major)
            self.coo = (I[order] + 1, J[order] + 1, arr[I[order], J[order]])

    def _from_scipy(self, A):
        """Tensor(fmt, A) for a scipy.sparse A whose implicit entries equal
        the format's fill: Finch's dropfills! copy (src/interface/copy.jl:
        77-113) without a dense intermediate.  Stored entries equal to the
        fill are dropped, duplicates summed and coordinates sorted; a
        canonical CSC A in the format's value type keeps its own arrays
        (0-based, `base` 0)."""
        if A.ndim != 2:
            raise ValueError("Tensor from scipy.sparse: 2-D matrices only")
        self.shape = tuple(map(int, A.shape))
        if self.kind == "coo":
            C = A.tocoo(copy=True)
            C.sum_duplicates()
            keep = ~_isfill(C.data, self.fill_value)
            I, J, V = C.row[keep].astype(np.int64), C.col[keep].astype(np.int64), C.data[keep]
            order = np.lexsort((I, J))  # Finch sorts by reverse coordinates (column-major)
            self.coo = (I[order] + 1, J[order] + 1, V[order].astype(self.dtype))
            return
        C = _canonical_csc(A)
        ptr, idx, data = C.indptr, C.indices, C.data
        drop = _isfill(data, self.fill_value)
        if drop.any():
            keep = ~drop
            fib = np.repeat(np.arange(self.shape[1]), np.diff(ptr))
            ptr = np.zeros(self.shape[1] + 1, dtype=ptr.dtype)
            np.cumsum(np.bincount(fib[keep], minlength=self.shape[1]), out=ptr[1:])
            idx, data = idx[keep], data[keep]
        val = None if isinstance(self.fmt.lvl.lvl, Pattern) else data.astype(self.dtype, copy=False)
        self.buf = SparseBuffers(self.shape[0], self.shape[1], ptr, idx, val, "csc", base=0)

    # -- constructors from level buffers (zero-copy on the host)
    @classmethod
    def from_buffers(cls, fmt, buf: SparseBuffers) -> "Tensor":
        return cls(fmt, _buf=buf)

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def on_device(self) -> bool:
        return self.ddata is not None or self.dsparse is not None

    def is_sparse(self) -> bool:
        return self.kind in ("csc", "sparse1", "coo")

    def todense(self) -> np.ndarray:
        if self.kind in ("dense1", "dense2"):
            if isinstance(self.ddata, tuple):  # tuple elements: two device arrays
                out = np.empty(self.shape, dtype=self.dtype)
                out["f0"] = self.ddata[0].cpu().numpy()
                out["f1"] = self.ddata[1].cpu().numpy()
                return out
            if self.data is not None:
                return self.data
            return read_back(self.ddata)  # read back each time: kernels may have updated it
        if self.kind == "coo":
            out = np.full(self.shape, self.fill_value, dtype=self.dtype)
            I, J, V = self.coo
            if len(I):
                # fsparse folds duplicates with `combine`, in input order
                key = (np.asarray(J, np.int64) - 1) * self.shape[0] + (np.asarray(I, np.int64) - 1)
                order = np.argsort(key, kind="stable")
                k, v = key[order], np.asarray(V)[order]
                heads = np.flatnonzero(np.r_[True, k[1:] != k[:-1]])
                ends = np.r_[heads[1:], k.size]
                folded = [_fold(self.combine, v[a:b]) for a, b in zip(heads, ends)]
                uk = k[heads]
                out[uk % self.shape[0], uk // self.shape[0]] = folded
            return out
        buf = self.host_buffers()  # stored entries over the fill, one dense array
        out = np.full((buf.nrows, buf.ncols), self.fill_value, dtype=self.dtype)
        f = np.repeat(np.arange(buf.nfibers), np.diff(buf.ptr))
        c = np.asarray(buf.idx, dtype=np.int64) - buf.base
        v = True if buf.val is None else buf.val
        if buf.orient == "csc":
            out[c, f] = v
        else:
            out[f, c] = v
        return out.reshape(self.shape)

    def pair_device(self):
        """The two component arrays in HBM of a vector of tuple elements."""
        if not (self.kind == "dense1" and self.dtype.names):
            raise TypeError("pair_device: not a vector of tuple elements")
        if not isinstance(self.ddata, tuple):
            transfer(GPU(0 if not hasattr(self, "_gb_device") else self._gb_device), self)
        return self.ddata

    def __setitem__(self, key, value):
        """Host-side element write, as Finch's `t[i] = v` (1-based i)."""
        if self.kind != "dense1":
            raise NotImplementedError("element writes into Dense(Element) vectors")
        i = int(key) - 1
        if isinstance(self.ddata, tuple):
            for comp, v in zip(self.ddata, value):
                comp[i] = v
        elif self.ddata is not None:
            self.ddata[i] = value
            self.data = None
        else:
            self.data[i] = value

    def host_buffers(self) -> SparseBuffers:
        if self.buf is None and self.dsparse is not None:
            ptr, idx, val = self.dsparse.to_host()
            d = self.dsparse
            self.buf = SparseBuffers(d.nrows, d.ncols, ptr, idx, val, d.orient)
        return self.buf

    def countstored(self) -> int:
        if self.kind in ("dense1", "dense2"):
            return int(np.prod(self.shape))
        if self.kind == "coo":
            return len(self.coo[0])
        return self.dsparse.nnz if self.dsparse is not None else self.buf.nnz

    def __repr__(self):
        where = "HBM" if self.on_device else "host"
        return f"Tensor({self.fmt}, shape={self.shape}, {where})"

    def __eq__(self, other):  # value-wise, like src/interface/compare.jl
        return _equal(self, other, nan_equal=False)

    __hash__ = None


def _scipy_sparse(x):
    """x when it is a scipy.sparse matrix or array, else None (scipy is
    imported only for objects of its own)."""
    if not type(x).__module__.startswith("scipy.sparse"):
        return None
    import scipy.sparse as sp

    return x if sp.issparse(x) else None


def _isfill(data: np.ndarray, fill) -> np.ndarray:
    """Entries equal to the fill value (NaN equals NaN, as in isequal)."""
    f = np.asarray(fill)
    if f.dtype.kind in "fc" and np.isnan(f):
        return np.isnan(data)
    return data == f


def _same_fill(a, b) -> bool:
    if isinstance(a, tuple) or isinstance(b, tuple):
        return False
    a, b = np.asarray(a), np.asarray(b)
    return bool(a == b) or bool(a.dtype.kind in "fc" and b.dtype.kind in "fc" and np.isnan(a) and np.isnan(b))


def _stored_scipy(t):
    """The stored entries of a Dense(SparseList) tensor or swizzle as a
    scipy.sparse matrix of its logical shape (a pattern's entries true);
    the host buffers are shared where they are 0-based.  None without
    scipy."""
    try:
        import scipy.sparse as sp
    except ImportError:
        return None
    body = t.body if isinstance(t, SwizzleArray) else t
    if isinstance(t, SwizzleArray) and t.dims != (2, 1):
        raise ValueError(f"swizzle {t.dims}")
    b = body.host_buffers()
    ptr, idx = b.ptr, b.idx
    if b.base:
        ptr, idx = np.asarray(ptr) - b.base, np.asarray(idx) - b.base
    val = np.ones(b.nnz, dtype=np.bool_) if b.val is None else b.val
    make = sp.csc_matrix if b.orient == "csc" else sp.csr_matrix
    M = make((val, idx, ptr), shape=(b.nrows, b.ncols))
    return M.T if isinstance(t, SwizzleArray) else M


def _coord_values(t):
    """Sorted linear coordinates (column-major) of a sparse matrix's stored
    entries and their values; None when t is not a Dense(SparseList)."""
    if not isinstance(t, (Tensor, SwizzleArray)) or t.kind != "csc" or t.ndim != 2:
        return None
    M = _stored_scipy(t)
    if M is None:
        return None
    C = _canonical_csc(M)
    cols = np.repeat(np.arange(C.shape[1], dtype=np.int64), np.diff(C.indptr))
    return cols * C.shape[0] + C.indices.astype(np.int64), C.data


def _equal(a, b, nan_equal: bool) -> bool:
    """A == B (or isequal) over every coordinate, Finch's helper_equal
    (src/interface/compare.jl:1-61).  Two sparse matrices are compared on the
    union of their stored coordinates, and their fills once where neither
    stores an entry, so no dense form is built."""
    def eq(x, y):
        r = np.asarray(x == y)
        if nan_equal:
            xn = np.isnan(x) if np.asarray(x).dtype.kind in "fc" else False
            yn = np.isnan(y) if np.asarray(y).dtype.kind in "fc" else False
            r = r | (np.asarray(xn) & np.asarray(yn))
        return r

    if tuple(getattr(a, "shape", np.shape(a))) != tuple(getattr(b, "shape", np.shape(b))):
        return False
    ca, cb = _coord_values(a), _coord_values(b)
    if ca is None or cb is None:
        x = a.todense() if hasattr(a, "todense") else np.asarray(a)
        y = b.todense() if hasattr(b, "todense") else np.asarray(b)
        return bool(np.all(eq(x, y)))
    (ka, va), (kb, vb) = ca, cb
    keys = np.union1d(ka, kb)
    fa, fb = np.asarray(a.fill_value), np.asarray(b.fill_value)

    def at(k, v, fill):
        out = np.full(keys.size, fill, dtype=np.result_type(v.dtype, fill.dtype))
        pos = np.searchsorted(keys, k)
        out[pos] = v
        return out

    if not np.all(eq(at(ka, va, fa), at(kb, vb, fb))):
        return False
    total = int(np.prod(a.shape))
    return keys.size == total or bool(eq(fa, fb))


def isequal(a, b) -> bool:
    """Finch's isequal on tensors: == with NaN equal to NaN
    (src/interface/compare.jl:29-61)."""
    return _equal(a, b, nan_equal=True)


def _canonical_csc(A):
    """A in CSC with sorted, distinct coordinates in every column (Julia's
    SparseMatrixCSC invariant); a canonical CSC A is returned as it is."""
    C = A.tocsc()
    if not C.has_canonical_format:
        C = C.copy()
        C.sum_duplicates()
    return C


def _map_scipy(A):
    """Finch's Tensor(::SparseMatrixCSC) (ext/SparseArraysExt.jl:17-22) for
    scipy.sparse: Dense(SparseList(Element(zero(T)))) over A's own indptr,
    indices and data (0-based, `base` 0), stored zeros kept.  A matrix that
    is not canonical CSC is converted first."""
    if A.ndim != 2:
        raise ValueError("Tensor from scipy.sparse: 2-D matrices only")
    C = _canonical_csc(A)
    fmt = Dense(SparseList(Element(C.data.dtype.type(0)), index_type=C.indices.dtype.type))
    return fmt, SparseBuffers(int(C.shape[0]), int(C.shape[1]), C.indptr, C.indices, C.data, "csc", base=0)


def sparse(t):
    """The scipy.sparse matrix of a 2-D tensor or swizzle, Finch's
    sparse(::Tensor) (ext/SparseArraysExt.jl:61-76).  Only a zero fill value
    can be represented.  A Dense(SparseList) tensor's host buffers are
    reused where their layout allows (0-based ones are); a swizzled CSC comes
    back as the CSR view of its transpose."""
    import scipy.sparse as sp

    if t.ndim != 2:
        raise ValueError(f"sparse: scipy.sparse holds matrices, got a {t.ndim}-d tensor")
    if np.any(np.asarray(t.fill_value)):
        raise ValueError(f"sparse: scipy.sparse only supports zero fill values, was given {t.fill_value!r}")
    if t.kind == "csc":
        return _stored_scipy(t)
    return sp.csc_matrix(t.todense())


def _as_array(arr, dtype) -> np.ndarray:
    try:
        import scipy.sparse as sp

        if sp.issparse(arr):
            arr = arr.toarray()
    except ImportError:
        pass
    return np.asarray(arr).astype(dtype, copy=False)


class SwizzleArray(_EagerOps):
    """A permuted view of a tensor (src/tensors/combinators/swizzle.jl).

    swizzle(Tensor(Dense(SparseList(...)), A^T), 2, 1) is Finch's CSR of A."""

    def __init__(self, body: Tensor, dims: tuple[int, ...]):
        self.body = body
        self.dims = tuple(dims)
        self.shape = tuple(body.shape[d - 1] for d in self.dims)
        self.dtype = body.dtype
        self.fill_value = body.fill_value

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def kind(self):
        return self.body.kind

    def is_sparse(self):
        return self.body.is_sparse()

    def todense(self):
        return np.transpose(self.body.todense(), [d - 1 for d in self.dims])

    def __eq__(self, other):
        return _equal(self, other, nan_equal=False)

    __hash__ = None

    def __repr__(self):
        return f"swizzle({self.body!r}, {', '.join(map(str, self.dims))})"


def swizzle(t, *dims) -> SwizzleArray:
    if isinstance(t, SwizzleArray):
        return SwizzleArray(t.body, tuple(t.dims[d - 1] for d in dims))
    return SwizzleArray(t, dims)


def csr(A, fill_value=0.0, dtype=None) -> SwizzleArray:
    """Finch's CSR of a matrix: swizzle(Tensor(Dense(SparseList(Element)), A^T), 2, 1)."""
    if _scipy_sparse(A) is None:
        A = np.asarray(A)
    el = Element(fill_value, dtype or A.dtype)
    return swizzle(Tensor(Dense(SparseList(el)), A.T), 2, 1)


_COMBINE = {"+": 0, "|": 1, "min": 2, "max": 3, "last": 4}


def _fold(combine: str, v: np.ndarray):
    acc = v[0]
    for t in v[1:]:
        if combine == "+":
            acc = acc + t if v.dtype != np.bool_ else (acc | t)
        elif combine == "|":
            acc = acc | t
        elif combine == "min":
            acc = t if t < acc else acc
        elif combine == "max":
            acc = t if t > acc else acc
        else:
            acc = t
    return acc


def fsparse(I, J, V, shape=None, combine: str = "+", fill_value=None) -> Tensor:
    """Finch's fsparse(I, J, V, (m, n), combine) (src/interface/fsparse.jl):
    a COO tensor whose duplicate coordinates are folded with `combine` (+, |,
    min, max or last; + means | for Bool).  Coordinates are 1-based.  The
    triplets stay as given until the tensor is moved to the GPU, where they
    are sorted and folded in HBM (fgb_coo_assemble)."""
    I = np.asarray(I, dtype=np.int64)
    J = np.asarray(J, dtype=np.int64)
    V = np.asarray(V)
    if combine not in _COMBINE:
        raise ValueError(f"combine must be one of {sorted(_COMBINE)}")
    if shape is None:
        shape = (int(I.max()) if I.size else 0, int(J.max()) if J.size else 0)
    if I.size and (I.min() < 1 or J.min() < 1 or I.max() > shape[0] or J.max() > shape[1]):
        raise ValueError("fsparse: a coordinate lies outside the shape")  # Finch: 1 <= I <= M
    fill = np.zeros((), V.dtype)[()] if fill_value is None else fill_value
    t = Tensor.__new__(Tensor)
    t.fmt = SparseCOO(2, Element(fill, V.dtype))
    t.kind, t.fill_value, t.dtype = "coo", fill, V.dtype
    t.data, t.buf, t.ddata, t.dsparse = None, None, None, None
    t.coo, t.combine, t.shape = (I, J, V), combine, (int(shape[0]), int(shape[1]))
    return t


def fsprand(rng, m: int, n: int, p: float, dtype=np.float64) -> Tensor:
    """Finch's fsprand + Tensor(Dense(SparseList(Element(0))), ...)."""
    from .workloads import fsprand as _fsprand

    b = _fsprand(rng, m, n, p, dtype=dtype)
    return Tensor.from_buffers(Dense(SparseList(Element(np.zeros((), dtype)[()], dtype))), b)


# ---------------------------------------------------------------- devices


@dataclass(frozen=True)
class GPU:
    """The CUDA device target (Finch's AbstractDevice, src/architecture.jl)."""

    index: int = 0


def gpu(index: int = 0) -> GPU:
    return GPU(index)


# Read-backs of at least this many bytes go through page-locked memory.
_PINNED_READBACK = 1 << 20


def read_back(d):
    """A device array as a numpy array.  A large one is copied into
    page-locked memory from torch's caching host allocator (the copy engine
    writes it at link speed; a fresh pageable array is filled several times
    slower) and returned as a view of it, so later read-backs of the same
    size reuse the pinned block."""
    import torch

    if d.numel() * d.element_size() < _PINNED_READBACK:
        return d.cpu().numpy()
    h = torch.empty(d.shape, dtype=d.dtype, pin_memory=True)
    h.copy_(d, non_blocking=True)
    torch.cuda.current_stream(d.device).synchronize()
    return h.numpy()


def transfer(device, t):
    """Moves a tensor's level buffers into HBM (Finch's transfer(device, tns)).

    Sparse levels are narrowed to int32 idx once; dense levels are copied
    row-major.  Returns the same tensor object, now resident."""
    import torch

    from . import device as dev

    if isinstance(t, SwizzleArray):
        transfer(device, t.body)
        return t
    if t.on_device:
        return t
    idx = device.index if isinstance(device, GPU) else int(device)
    if t.kind == "dense1" and t.dtype.names:  # tuple elements: one device array per component
        d = torch.device("cuda", idx)
        t.ddata = tuple(torch.from_numpy(np.ascontiguousarray(t.data[f])).to(d) for f in t.dtype.names)
        t.data = None
        return t
    if t.kind in ("dense1", "dense2"):
        src = np.ascontiguousarray(t.data)
        tt = torch.from_numpy(src if src.dtype != np.bool_ else src.astype(np.uint8))
        t.ddata = tt.to(torch.device("cuda", idx))
        t.data = None  # the HBM copy is the tensor now (kernels may update it in place)
        return t
    if t.kind == "coo":  # assembled in HBM: sort, fold duplicates, build ptr
        I, J, V = t.coo
        d = torch.device("cuda", idx)
        Id = torch.from_numpy(np.ascontiguousarray(I, dtype=np.int64)).to(d)
        Jd = torch.from_numpy(np.ascontiguousarray(J, dtype=np.int64)).to(d)
        Vh = np.ascontiguousarray(V)
        Vd = torch.from_numpy(Vh if Vh.dtype != np.bool_ else Vh.astype(np.uint8)).to(d)
        t.dsparse = dev.coo_assemble(t.shape[0], t.shape[1], Id, Jd, Vd, orient="csc",
                                     combine=_COMBINE[t.combine])
        t.kind, t.coo, t.buf = "csc", None, None
        return t
    b = t.buf
    val = b.val
    t.dsparse = dev.DeviceSparse.from_host(b.nrows, b.ncols, b.ptr, b.idx, val, orient=b.orient,
                                           base=b.base, device=idx)
    return t


def pattern(t):
    """Finch's pattern!(t): the same structure with a Pattern level (every
    stored entry true), sharing the coordinate buffers."""
    if isinstance(t, SwizzleArray):
        return SwizzleArray(pattern(t.body), t.dims)
    if t.kind != "csc":
        raise NotImplementedError("pattern! of a Dense(SparseList) matrix")
    out = Tensor.__new__(Tensor)
    out.__dict__.update(t.__dict__)
    out.fmt = Dense(SparseList(Pattern()))
    out.fill_value, out.dtype = False, np.dtype(np.bool_)
    if t.buf is not None:
        b = t.buf
        out.buf = SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, None, b.orient, b.base)
    if t.dsparse is not None:
        d = t.dsparse
        out.dsparse = type(d)(d.nrows, d.ncols, d.ptr, d.idx, None, d.orient, d.base)
    for k in ("_gb_transposed", "_gb_uses"):
        out.__dict__.pop(k, None)
    return out


def set_fill_value(t, fill):
    """Finch's set_fill_value!(t, fill): the same stored entries, another
    implicit value (e.g. Inf for unconnected edges)."""
    body = t.body if isinstance(t, SwizzleArray) else t
    out = Tensor.__new__(Tensor)
    out.__dict__.update(body.__dict__)
    lvl = body.fmt
    chain = []
    while not isinstance(lvl, (Element, Pattern)):
        chain.append(type(lvl))
        lvl = lvl.lvl
    new = Element(np.asarray(fill, dtype=body.dtype)[()], body.dtype)
    for c in reversed(chain):
        new = c(new)
    out.fmt, out.fill_value = new, np.asarray(fill, dtype=body.dtype)[()]
    return SwizzleArray(out, t.dims) if isinstance(t, SwizzleArray) else out


def dense_from_device(x, fill_value=0.0) -> Tensor:
    """Wraps a device array (torch) as a Dense tensor resident in HBM."""
    dt = np.dtype(str(x.dtype).replace("torch.", "").replace("uint8", "bool"))
    fmt = Dense(Element(fill_value, dt)) if x.dim() == 1 else Dense(Dense(Element(fill_value, dt)))
    t = Tensor.__new__(Tensor)
    t.fmt, t.kind = fmt, ("dense1" if x.dim() == 1 else "dense2")
    t.fill_value, t.dtype = fill_value, dt
    t.data, t.buf, t.ddata, t.dsparse, t.coo = None, None, x, None, None
    t.shape = tuple(x.shape)
    return t


def sparse_from_device(d, fill_value=0.0) -> Tensor:
    """Wraps a DeviceSparse as a resident tensor (CSC kind, or swizzled CSR)."""
    import torch

    dt = np.float64 if d.val is None else np.dtype(str(d.val.dtype).replace("torch.", "").replace("bfloat16", "float32"))
    lvl = Pattern() if d.val is None else Element(fill_value, dt)
    fmt = Dense(SparseList(lvl))
    t = Tensor.__new__(Tensor)
    t.fmt, t.kind, t.fill_value, t.dtype = fmt, "csc", fill_value, np.dtype(dt)
    t.data, t.buf, t.ddata, t.coo = None, None, None, None
    if d.orient == "csc":
        t.dsparse, t.shape = d, (d.nrows, d.ncols)
        return t
    t.dsparse, t.shape = d.T(), (d.ncols, d.nrows)  # CSR of A == CSC of A^T
    return swizzle(t, 2, 1)
