"""Device-resident level buffers and the kernel calls behind the matcher.

`DeviceSparse` is a SparseList matrix whose ptr/idx/val live in HBM -- what
Finch's `transfer(device, lvl)` recursion (src/tensors/levels/
sparse_list_levels.jl:64-69, element_levels.jl:46-48) produces for a GPU
device.  Finch's 1-based Int64 idx are narrowed to int32 once, at upload,
and keep their base; ptr stays Int64 only when nnz needs it.

PyTorch supplies device memory and the current stream; every computation is
a libfinchgb call.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib as L

_TORCH_CODE = {torch.float64: L.F64, torch.float32: L.F32, torch.bfloat16: L.BF16,
               torch.int32: L.I32, torch.int64: L.I64, torch.uint8: L.BOOL, torch.bool: L.BOOL}
_NP_TO_TORCH = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
                np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
                np.dtype(np.bool_): torch.uint8, np.dtype(np.uint8): torch.uint8}

_ctxs: dict[int, ctypes.c_void_p] = {}


def require_gpu() -> None:
    if not torch.cuda.is_available():
        raise L.FinchGBError(L.ECUDA, "no CUDA device: the GB300 backend has no CPU fallback")


def context(device: int | None = None) -> ctypes.c_void_p:
    """The libfinchgb context of `device` (created on first use)."""
    require_gpu()
    dev = torch.cuda.current_device() if device is None else int(device)
    if dev not in _ctxs:
        h = ctypes.c_void_p()
        L.call("fgb_ctx_create", dev, ctypes.byref(h))
        _ctxs[dev] = h
    return _ctxs[dev]


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def dtype_code(t: torch.Tensor | None) -> int:
    return L.NONE if t is None else _TORCH_CODE[t.dtype]


def _dptr(t: torch.Tensor | None) -> int | None:
    return None if t is None or t.numel() == 0 else t.data_ptr()


def gather_ceiling(working_set_bytes: int, gather_bytes: int, gathers: int = 1 << 24) -> float:
    """GB/s at which random gathers of `gather_bytes` contiguous bytes are served
    from a device working set of `working_set_bytes` (fgb_gather_ceiling): the
    limit that binds the kernels gathering dense rows."""
    out = ctypes.c_double()
    L.call("fgb_gather_ceiling", context(), int(working_set_bytes), int(gather_bytes), int(gathers),
           ctypes.byref(out), stream_ptr())
    return out.value


@dataclass
class DeviceSparse:
    """A 2-D SparseList matrix in HBM.

    orient 'csr': ptr over rows, idx = columns; 'csc': ptr over columns,
    idx = rows (Finch's Dense(SparseList(Element)))."""

    nrows: int
    ncols: int
    ptr: torch.Tensor
    idx: torch.Tensor
    val: torch.Tensor | None
    orient: str = "csr"
    base: int = 0
    _desc: L.FgbSparse | None = field(default=None, repr=False)

    @property
    def nnz(self) -> int:
        return int(self.idx.numel())

    @property
    def shape(self) -> tuple[int, int]:
        return (self.nrows, self.ncols)

    @property
    def dtype(self):
        return None if self.val is None else self.val.dtype

    def desc(self) -> L.FgbSparse:
        if self._desc is None:
            self._desc = L.FgbSparse(
                self.nrows, self.ncols, self.nnz, L.CSR if self.orient == "csr" else L.CSC,
                self.base, dtype_code(self.ptr), dtype_code(self.idx), dtype_code(self.val),
                0, _dptr(self.ptr), _dptr(self.idx), _dptr(self.val))
        return self._desc

    def nbytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in (self.ptr, self.idx, self.val)
                   if t is not None)

    @classmethod
    def from_host(cls, nrows: int, ncols: int, ptr, idx, val, orient: str = "csc", base: int = 1,
                  device: int | None = None, val_dtype: torch.dtype | None = None,
                  pinned: bool = False) -> "DeviceSparse":
        """Uploads level buffers (ptr/idx counted from `base`) to HBM: Finch's
        Int64 buffers are narrowed to int32 on the device; int32 buffers
        (scipy.sparse's usual width) are uploaded as they are."""
        ctx = context(device)
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        ptr, idx = np.asarray(ptr), np.asarray(idx)
        nnz = idx.size
        s = stream_ptr()
        if idx.dtype == np.int32:
            d_idx = torch.from_numpy(np.ascontiguousarray(idx)).to(dev)
        else:
            idx = np.ascontiguousarray(idx, dtype=np.int64)
            d_idx = torch.empty(nnz, dtype=torch.int32, device=dev)
            if nnz:
                tmp = torch.from_numpy(idx).to(dev, non_blocking=pinned)
                L.call("fgb_narrow_index", ctx, tmp.data_ptr(), d_idx.data_ptr(), nnz, 0, s)
        if ptr.dtype == np.int32:
            d_ptr = torch.from_numpy(np.ascontiguousarray(ptr)).to(dev)
        elif nnz + base < 2**31 - 1:
            ptr = np.ascontiguousarray(ptr, dtype=np.int64)
            d_ptr = torch.empty(ptr.size, dtype=torch.int32, device=dev)
            tmp = torch.from_numpy(ptr).to(dev)
            L.call("fgb_narrow_index", ctx, tmp.data_ptr(), d_ptr.data_ptr(), ptr.size, 0, s)
        else:
            d_ptr = torch.from_numpy(np.ascontiguousarray(ptr, dtype=np.int64)).to(dev)
        d_val = None
        if val is not None:
            v = torch.as_tensor(np.ascontiguousarray(val))
            if v.dtype == torch.bool:
                v = v.to(torch.uint8)
            if val_dtype is not None:
                v = v.to(val_dtype)
            d_val = v.to(dev)
        return cls(nrows, ncols, d_ptr, d_idx, d_val, orient, base)

    def transposed_storage(self) -> "DeviceSparse":
        """Same logical matrix, the other orientation (stable device transpose)."""
        ctx = context(self.ptr.device.index)
        nout = self.nrows if self.orient == "csc" else self.ncols
        dev = self.ptr.device
        out_ptr = torch.empty(nout + 1, dtype=torch.int64, device=dev)
        out_idx = torch.empty(self.nnz, dtype=torch.int32, device=dev)
        out_val = None if self.val is None else torch.empty_like(self.val)
        d = self.desc()
        L.call("fgb_transpose", ctx, ctypes.byref(d), out_ptr.data_ptr(), _dptr(out_idx),
               _dptr(out_val), stream_ptr())
        if self.nnz < 2**31 - 1:
            p32 = torch.empty(nout + 1, dtype=torch.int32, device=dev)
            L.call("fgb_narrow_index", ctx, out_ptr.data_ptr(), p32.data_ptr(), nout + 1, 0,
                   stream_ptr())
            out_ptr = p32
        return DeviceSparse(self.nrows, self.ncols, out_ptr, out_idx, out_val,
                            "csr" if self.orient == "csc" else "csc", 0)

    def T(self) -> "DeviceSparse":
        """The transpose A^T as a view: same buffers, other orientation."""
        return DeviceSparse(self.ncols, self.nrows, self.ptr, self.idx, self.val,
                            "csr" if self.orient == "csc" else "csc", self.base)

    def to_host(self):
        """(ptr, idx, val) as numpy in Finch's 1-based Int64 layout."""
        torch.cuda.current_stream().synchronize()
        ptr = self.ptr.cpu().numpy().astype(np.int64) - self.base + 1
        idx = self.idx.cpu().numpy().astype(np.int64) - self.base + 1
        val = None if self.val is None else self.val.cpu()
        if val is not None and val.dtype == torch.bfloat16:
            val = val.float()
        return ptr, idx, (None if val is None else val.numpy())


# ---------------------------------------------------------------- kernel calls

def _ctx_for(t: torch.Tensor):
    return context(t.device.index)


def coo_assemble(nrows: int, ncols: int, I: torch.Tensor, J: torch.Tensor,
                 V: torch.Tensor | None, orient: str = "csc", combine: int = L.COMBINE_ADD,
                 in_base: int = 1, out_base: int = 1) -> DeviceSparse:
    """fsparse(I, J, V, (nrows, ncols), combine) assembled in HBM as CSC
    (Finch's Dense(SparseList)) or CSR; I/J are device int32/int64
    coordinates with base `in_base`, V device values (None: Pattern)."""
    ctx = context(I.device.index)
    dev = I.device
    n_in = int(I.numel())
    nfib = ncols if orient == "csc" else nrows
    ptr_t = torch.int32 if n_in + out_base < 2**31 - 1 else torch.int64
    ptr = torch.empty(nfib + 1, dtype=ptr_t, device=dev)
    idx = torch.empty(max(n_in, 1), dtype=torch.int32, device=dev)
    val = None if V is None else torch.empty(max(n_in, 1), dtype=V.dtype, device=dev)
    out = L.FgbSparse(nrows, ncols, 0, L.CSC if orient == "csc" else L.CSR, out_base,
                      dtype_code(ptr), L.I32, dtype_code(val), 0, _dptr(ptr), _dptr(idx), _dptr(val))
    nnz = ctypes.c_int64()
    L.call("fgb_coo_assemble", ctx, nrows, ncols, n_in, dtype_code(I), _dptr(I), _dptr(J), in_base,
           dtype_code(V), _dptr(V), combine, ctypes.byref(out), ctypes.byref(nnz), stream_ptr())
    k = nnz.value
    return DeviceSparse(nrows, ncols, ptr, idx[:k], None if val is None else val[:k], orient, out_base)


def spmv(A: DeviceSparse, x: torch.Tensor, y: torch.Tensor | None = None,
         semiring: int = L.PLUS_TIMES, flags: int = 0) -> torch.Tensor:
    """y <<add>>= A (*) x over `semiring` (y is created and initialised if None)."""
    if y is None:
        y = torch.empty(A.nrows, dtype=x.dtype, device=x.device)
        flags &= ~L.ACCUMULATE
    d = A.desc()
    L.call("fgb_spmv", _ctx_for(x), semiring, ctypes.byref(d), _dptr(x), dtype_code(x), _dptr(y),
           dtype_code(y), flags, stream_ptr())
    return y


def spmm(A: DeviceSparse, B: torch.Tensor, C: torch.Tensor | None = None, flags: int = 0,
         lanes: int = 0, path: int = 0, variant: int = 0, bands: int = 0) -> torch.Tensor:
    """C (+)= A @ B for row-major B (n x nk); lanes/path/variant/bands override
    the schedule (bands: column bands of the virtual-row variants 2 and 3)."""
    nk = B.shape[1]
    if C is None:
        C = torch.empty((A.nrows, nk), dtype=B.dtype, device=B.device)
        flags &= ~L.ACCUMULATE
    d = A.desc()
    tune = L.FgbSpmmTuning(lanes, variant, path, bands)
    L.call("fgb_spmm_ex", _ctx_for(B), ctypes.byref(d), _dptr(B), B.stride(0), nk, _dptr(C),
           C.stride(0), dtype_code(B), flags, ctypes.byref(tune), stream_ptr())
    return C


def sparse_to_dense(A: DeviceSparse, fill) -> torch.Tensor:
    """Row-major dense copy of A with `fill` where nothing is stored
    (fgb_sparse_to_dense); a Pattern becomes a uint8 0/1 matrix."""
    dt = torch.uint8 if A.val is None else A.val.dtype
    out = torch.empty((A.nrows, A.ncols), dtype=dt, device=A.idx.device)
    npdt = {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32, torch.int64: np.int64,
            torch.uint8: np.uint8}[dt]
    f = np.array([fill], dtype=npdt)
    d = A.desc()
    L.call("fgb_sparse_to_dense", _ctx_for(A.idx), ctypes.byref(d), f.ctypes.data, _dptr(out), A.ncols,
           stream_ptr())
    return out


def spmm_semiring(A: DeviceSparse, B: torch.Tensor, C: torch.Tensor | None = None, semiring: int = L.MAX_PLUS,
                  flags: int = 0) -> torch.Tensor:
    """C <<add>>= A (*) B over an exact semiring (fgb_spmm_semiring), row-major B."""
    nk = B.shape[1]
    if C is None:
        C = torch.empty((A.nrows, nk), dtype=B.dtype, device=B.device)
        flags &= ~L.ACCUMULATE
    d = A.desc()
    L.call("fgb_spmm_semiring", _ctx_for(B), semiring, ctypes.byref(d), _dptr(B), B.stride(0), nk, _dptr(C),
           C.stride(0), dtype_code(B), flags, stream_ptr())
    return C


class Panels:
    """Column-panel layout of a CSR matrix (fgb_panels_*) for SpMM with an
    L2-resident slice of B per panel."""

    def __init__(self, A: DeviceSparse, npanels: int):
        self.A = A
        self.npanels = npanels
        h = ctypes.c_void_p()
        d = A.desc()
        L.call("fgb_panels_create", context(A.idx.device.index), ctypes.byref(d), npanels,
               ctypes.byref(h))
        self.h = h

    def spmm(self, B: torch.Tensor, C: torch.Tensor | None = None, flags: int = 0,
             lanes: int = 0, path: int = 0, variant: int = 0) -> torch.Tensor:
        nk = B.shape[1]
        if C is None:
            C = torch.empty((self.A.nrows, nk), dtype=B.dtype, device=B.device)
            flags &= ~L.ACCUMULATE
        tune = L.FgbSpmmTuning(lanes, variant, path)
        L.call("fgb_panels_spmm", _ctx_for(B), self.h, _dptr(B), B.stride(0), nk, _dptr(C),
               C.stride(0), dtype_code(B), flags, ctypes.byref(tune), stream_ptr())
        return C

    def close(self):
        if getattr(self, "h", None):
            L.call("fgb_panels_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sddmm(A: DeviceSparse, X: torch.Tensor, Y: torch.Tensor, out: torch.Tensor | None = None,
          flags: int = 0, lanes: int = 0, chunk: int = 0, slab: int = -1,
          variant: int = 0, bands: int = 0) -> torch.Tensor:
    """out[e] = A.val[e] * <X[i,:], Y[j,:]> over A's stored entries
    (lanes/chunk/slab/variant override the schedule; slab 0 = all of k per
    launch; variant 1 = virtual rows of at most `chunk` entries; bands:
    column bands of the virtual-row variants)."""
    if out is None:
        out = torch.empty(A.nnz, dtype=X.dtype, device=X.device)
    d = A.desc()
    tune = L.FgbSddmmTuning(lanes, variant, chunk, slab, bands)
    L.call("fgb_sddmm_ex", _ctx_for(X), ctypes.byref(d), _dptr(X), X.stride(0), _dptr(Y),
           Y.stride(0), X.shape[1], _dptr(out), dtype_code(X), flags, ctypes.byref(tune),
           stream_ptr())
    return out


def spgemm(A: DeviceSparse, B: DeviceSparse, flags: int = 0) -> DeviceSparse:
    """C = A * B (Gustavson, plus-times), same orientation and base as A."""
    ctx = _ctx_for(A.idx)
    d = A.idx.device
    nf = A.nrows if A.orient == "csr" else B.ncols
    c_ptr = torch.empty(nf + 1, dtype=torch.int64, device=d)
    nnz = ctypes.c_int64()
    da, db = A.desc(), B.desc()
    L.call("fgb_spgemm_symbolic", ctx, ctypes.byref(da), ctypes.byref(db), c_ptr.data_ptr(),
           ctypes.byref(nnz), stream_ptr())
    k = nnz.value
    c_idx = torch.empty(max(k, 1), dtype=torch.int32, device=d)
    c_val = torch.empty(max(k, 1), dtype=A.val.dtype, device=d)
    dc = L.FgbSparse(A.nrows, B.ncols, k, L.CSR if A.orient == "csr" else L.CSC, A.base, L.I64,
                     L.I32, dtype_code(c_val), 0, c_ptr.data_ptr(), c_idx.data_ptr(), c_val.data_ptr())
    L.call("fgb_spgemm_numeric", ctx, ctypes.byref(da), ctypes.byref(db), dtype_code(A.val), flags,
           ctypes.byref(dc), stream_ptr())
    if k < 2**31 - 1:  # the upload layout: 32-bit ptr below 2^31 entries
        p32 = torch.empty(nf + 1, dtype=torch.int32, device=d)
        L.call("fgb_narrow_index", ctx, c_ptr.data_ptr(), p32.data_ptr(), nf + 1, 0, stream_ptr())
        c_ptr = p32
    return DeviceSparse(A.nrows, B.ncols, c_ptr, c_idx[:k], c_val[:k], A.orient, A.base)


def spgemm_dense(A: DeviceSparse, B: DeviceSparse, flags: int = 0) -> torch.Tensor:
    """C = A * B into a dense row-major array (fgb_spgemm_dense)."""
    C = torch.empty((A.nrows, B.ncols), dtype=A.val.dtype, device=A.idx.device)
    da, db = A.desc(), B.desc()
    L.call("fgb_spgemm_dense", _ctx_for(A.idx), ctypes.byref(da), ctypes.byref(db), dtype_code(A.val), flags,
           _dptr(C), B.ncols, stream_ptr())
    return C


def ewise(op: int, A: DeviceSparse, B: DeviceSparse) -> DeviceSparse:
    """C = A .* B (op EW_MUL) or A .+ B (EW_ADD) of two same-shape matrices."""
    ctx = _ctx_for(A.idx)
    nf = A.nrows if A.orient == "csr" else A.ncols
    out_ptr = torch.empty(nf + 1, dtype=torch.int64, device=A.idx.device)
    nnz = ctypes.c_int64()
    da, db = A.desc(), B.desc()
    L.call("fgb_ewise_count", ctx, op, ctypes.byref(da), ctypes.byref(db), out_ptr.data_ptr(),
           ctypes.byref(nnz), stream_ptr())
    out_idx = torch.empty(nnz.value, dtype=torch.int32, device=A.idx.device)
    out_val = torch.empty(nnz.value, dtype=A.val.dtype, device=A.idx.device)
    L.call("fgb_ewise_fill", ctx, op, ctypes.byref(da), ctypes.byref(db), out_ptr.data_ptr(),
           _dptr(out_idx), _dptr(out_val), stream_ptr())
    return DeviceSparse(A.nrows, A.ncols, out_ptr, out_idx, out_val, A.orient, 0)


def dot(x: torch.Tensor, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """0-d device scalar sum_i x[i] y[i] (deterministic)."""
    if out is None:
        out = torch.empty((), dtype=x.dtype, device=x.device)
    L.call("fgb_dense_dot", _ctx_for(x), dtype_code(x), x.numel(), _dptr(x), _dptr(y),
           out.data_ptr(), stream_ptr())
    return out


def axpby(alpha: torch.Tensor | None, x: torch.Tensor, beta: torch.Tensor | None,
          y: torch.Tensor | None, out: torch.Tensor | None = None, signs: int = 0) -> torch.Tensor:
    """out = (+/-)alpha*x + (+/-)beta*y with device-scalar alpha/beta (None = 1)."""
    if out is None:
        out = torch.empty_like(x)
    L.call("fgb_dense_axpby", _ctx_for(x), dtype_code(x), x.numel(),
           None if alpha is None else alpha.data_ptr(), _dptr(x),
           None if beta is None else beta.data_ptr(), _dptr(y), _dptr(out), signs, stream_ptr())
    return out


def dense_affine(alpha: torch.Tensor | None, x: torch.Tensor | None, beta: torch.Tensor | None,
                 out: torch.Tensor) -> torch.Tensor:
    """out = alpha*x + beta (fused), or out = beta with x None
    (fgb_dense_affine): device-scalar alpha/beta (None: 1 and 0)."""
    L.call("fgb_dense_affine", _ctx_for(out), dtype_code(out), out.numel(),
           None if alpha is None else alpha.data_ptr(), _dptr(x),
           None if beta is None else beta.data_ptr(), _dptr(out), stream_ptr())
    return out


_NP_OF = {torch.float64: np.float64, torch.float32: np.float32, torch.int64: np.int64, torch.int32: np.int32}


def reduce_minmax(op: int, dims: int, A: DeviceSparse, fill, init=None) -> torch.Tensor:
    """reduce(max | min, A; dims) with A's fill folded where it stores
    nothing (fgb_reduce_minmax); dims 1 needs A stored CSC, 2 CSR, 0 either.
    init None: Finch's initial value (-Inf / typemin for max)."""
    length = 1 if dims == 0 else (A.ncols if dims == 1 else A.nrows)
    y = torch.empty(length, dtype=A.val.dtype, device=A.idx.device)
    npt = _NP_OF[A.val.dtype]
    f = np.array([fill], dtype=npt)
    i0 = None if init is None else np.array([init], dtype=npt)
    desc = A.desc()
    L.call("fgb_reduce_minmax", _ctx_for(A.idx), op, dims, ctypes.byref(desc), f.ctypes.data,
           None if i0 is None else i0.ctypes.data, _dptr(y), stream_ptr())
    return y


def sparse_scale(A: DeviceSparse, by: torch.Tensor, by_axis: int, keep: torch.Tensor | None = None,
                 keep_axis: int = L.AXIS_ROW, op: int = L.MAP_DIV,
                 out_dtype: torch.dtype = torch.float64) -> tuple[DeviceSparse, int]:
    """The stored entries of A combined with `by` over one index and kept
    where `keep` over an index is non-zero (fgb_sparse_scale).  Returns the
    0-based result in A's orientation and how many elements of `by` turn
    the fill 0 into something else (0 means skipping unstored entries was
    exact)."""
    nf = A.ncols if A.orient == "csc" else A.nrows
    d = A.idx.device
    out_ptr = torch.empty(nf + 1, dtype=torch.int64, device=d)
    out_idx = torch.empty(A.nnz, dtype=torch.int32, device=d)
    out_val = torch.empty(A.nnz, dtype=out_dtype, device=d)
    kept, changed = ctypes.c_int64(), ctypes.c_int64()
    desc = A.desc()
    L.call("fgb_sparse_scale", _ctx_for(A.idx), ctypes.byref(desc), op, by_axis, dtype_code(by), _dptr(by),
           keep_axis, 0 if keep is None else dtype_code(keep), _dptr(keep), dtype_code(out_val),
           out_ptr.data_ptr(), _dptr(out_idx), _dptr(out_val), ctypes.byref(kept), ctypes.byref(changed),
           stream_ptr())
    n = kept.value
    return DeviceSparse(A.nrows, A.ncols, out_ptr, out_idx[:n], out_val[:n], A.orient, 0), changed.value


def dense_map(op: int, x: torch.Tensor, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """out = op.(x, y) for op in MAP_ADD/SUB/MUL/MIN/MAX."""
    if out is None:
        out = torch.empty_like(x)
    L.call("fgb_dense_map", _ctx_for(x), op, dtype_code(x), x.numel(), _dptr(x), _dptr(y),
           _dptr(out), stream_ptr())
    return out


def scalar_op(op: int, a: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """0-d device scalar op(a, b)."""
    if out is None:
        out = torch.empty((), dtype=a.dtype, device=a.device)
    L.call("fgb_scalar_op", _ctx_for(a), op, dtype_code(a), a.data_ptr(), b.data_ptr(),
           out.data_ptr(), stream_ptr())
    return out


def ewise_reduce(dims: int, A: DeviceSparse, B: DeviceSparse | None = None,
                 B_dense: torch.Tensor | None = None, y: torch.Tensor | None = None) -> torch.Tensor:
    """sum(A .* B; dims) (dims 0 = all, 1 = over rows, 2 = over columns)."""
    length = 1 if dims == 0 else (A.nrows if dims == 2 else A.ncols)
    counts = B is None and B_dense is None and (A.val is None or A.val.dtype == torch.uint8)
    if y is None:  # a Pattern or Bool matrix sums into Int64 counts, as Julia sums Bools
        y = torch.empty(length, dtype=torch.int64 if counts else A.val.dtype, device=A.idx.device)
    da = A.desc()
    db = None if B is None else ctypes.byref(B.desc())
    L.call("fgb_ewise_reduce", _ctx_for(A.idx), dims, ctypes.byref(da), db, _dptr(B_dense),
           0 if B_dense is None else B_dense.stride(0), _dptr(y), L.I64 if counts else dtype_code(A.val), 0,
           stream_ptr())
    return y


# ---------------------------------------------------------------- graph programs (choose / minby)

def bfs_pull(A: DeviceSparse, frontier: torch.Tensor, visited: torch.Tensor, parent: torch.Tensor,
             next_frontier: torch.Tensor | None = None, choose_fill: int = 0, index_offset: int = 1) -> torch.Tensor:
    """One BFS round (fgb_bfs_pull): A is the CSR of the adjacency (row k
    lists the j with edges[k, j]); frontier/visited uint8; parent int32/int64
    updated by choose(choose_fill); returns the next frontier (uint8)."""
    if next_frontier is None:
        next_frontier = torch.empty(A.nrows, dtype=torch.uint8, device=visited.device)
    d = A.desc()
    L.call("fgb_bfs_pull", _ctx_for(visited), ctypes.byref(d), _dptr(frontier), _dptr(visited), _dptr(parent),
           dtype_code(parent), choose_fill, index_offset, _dptr(next_frontier), stream_ptr())
    return next_frontier


def or_count(visited: torch.Tensor, next_frontier: torch.Tensor, count: torch.Tensor) -> torch.Tensor:
    """visited |= next; count (device int64, 1 element) += number of true in next."""
    L.call("fgb_or_count", _ctx_for(visited), visited.numel(), _dptr(visited), _dptr(next_frontier),
           _dptr(count), stream_ptr())
    return count


def minby_map(mask: torch.Tensor | None, src: tuple, dst: tuple) -> tuple:
    """dst <<minby>>= src where mask (pairs as (first, second) device arrays)."""
    sd, sp = src
    dd, dp = dst
    L.call("fgb_minby_map", _ctx_for(dd), dtype_code(dd), dd.numel(), _dptr(mask), _dptr(sd), _dptr(sp),
           _dptr(dd), _dptr(dp), stream_ptr())
    return dst


def minby_relax(A: DeviceSparse, dist_prev: torch.Tensor, active_prev: torch.Tensor, dst: tuple,
                active: torch.Tensor | None = None, index_offset: int = 1) -> torch.Tensor:
    """One relaxation (fgb_minby_relax): A is the CSR of the weights (row i
    lists the j with edges[i, j]); dst = (dist, parent) updated in place;
    returns the new active flags (uint8)."""
    dd, dp = dst
    if active is None:
        active = torch.empty(A.nrows, dtype=torch.uint8, device=dd.device)
    d = A.desc()
    L.call("fgb_minby_relax", _ctx_for(dd), ctypes.byref(d), _dptr(dist_prev), _dptr(active_prev), _dptr(dd),
           _dptr(dp), _dptr(active), index_offset, stream_ptr())
    return active
