"""TEST INFRASTRUCTURE ONLY -- the oracle.

ctypes wrapper around finch_oracle.c, a CPU restatement of the loop nests
Finch.jl v1.2.12 generates for SpMV (CSC serial and CSR row-parallel), SpMM,
SDDMM, two-finger elementwise merges and elementwise+reduce.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it, and only
to check or time against.  The GPU library never calls it.

Sparse operands are passed in Finch's own layout: 1-based Int64 ptr/idx of a
SparseList level and the Element values (numpy arrays).  bf16 values are
passed as their uint16 bit patterns with ``vt=T_BF16``.

Parity of this restatement is pinned by tests/test_oracle_golden.py against
the numeric results printed in Finch's test fixtures.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "finch_oracle.c"
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"
# The same source built as Finch's CPU code runs (@fastmath: contraction and
# reassociation allowed, loops unrolled), timed as the CPU baseline only; the
# parity checks use LIB_PATH, whose float results are fixed by its explicit
# fma()/no-contraction choices on every host.
FAST_LIB_PATH = BUILD_DIR / "liboracle_fastmath.so"

SR_PT, SR_MINP, SR_MAXP, SR_OA = 0, 1, 2, 3
T_NONE, T_F64, T_F32, T_BF16, T_I32, T_I64, T_BOOL = -1, 0, 1, 2, 3, 4, 5

_lock = threading.Lock()
_lib = None
_fast_lib = None


def _compile(out: Path, flags: list[str], force: bool) -> None:
    if force or not out.exists() or out.stat().st_mtime < SRC.stat().st_mtime:
        tmp = out.with_suffix(".so.tmp")
        cmd = [os.environ.get("CC", "gcc"), *flags, "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC),
               "-o", str(tmp), "-lm"]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        os.replace(tmp, out)


def build(force: bool = False) -> Path:
    """Compiles finch_oracle.c with gcc: the parity build (OpenMP, no FP
    contraction) and the CPU-baseline build (-O3 -ffast-math -funroll-loops,
    the freedom Finch's @fastmath kernels give LLVM).  No -march=native: both
    builds must be portable between the build host and the GPU host, and on
    the GPU host's aarch64 the base ISA already has the 128-bit FMA vectors
    its SVE2 units would offer."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    _compile(LIB_PATH, ["-O3", "-ffp-contract=off"], force)
    _compile(FAST_LIB_PATH, ["-O3", "-ffast-math", "-funroll-loops"], force)
    return LIB_PATH


def lib(fast: bool = False) -> ctypes.CDLL:
    """The parity build, or with fast=True the CPU-baseline build."""
    global _lib, _fast_lib
    with _lock:
        if (_fast_lib if fast else _lib) is None:
            build()
            L = ctypes.CDLL(str(FAST_LIB_PATH if fast else LIB_PATH))
            i64, i32, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
            L.orc_spmv_csc.argtypes = [i32, i32, i32, i64, i64, vp, vp, vp, vp, vp, i32, i32]
            L.orc_spmv_csr.argtypes = [i32, i32, i32, i64, i64, vp, vp, vp, vp, vp, i32, i32, i32]
            L.orc_spmm_csr.argtypes = [i32, i32, i64, i64, i64, vp, vp, vp, vp, i64, vp, i64, i32,
                                       i32, i32]
            L.orc_sddmm_csr.argtypes = [i32, i64, i64, vp, vp, vp, vp, i64, vp, i64, vp, i32, i32,
                                        i32]
            L.orc_ewise.argtypes = [i32, i32, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
            L.orc_ewise_reduce.argtypes = [i32, i32, i64, i64, vp, vp, vp, vp, vp, vp, vp, i64, vp]
            L.orc_max_threads.argtypes = []
            L.orc_coo_assemble.argtypes = [i32, i32, i32, i64, i64, i64, vp, vp, vp, vp, vp, vp]
            L.orc_coo_assemble.restype = i64
            L.orc_spgemm_csr.argtypes = [i32, i32, i64, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
            L.orc_spgemm_csr.restype = i64
            L.orc_bfs_round.argtypes = [i64, vp, vp, vp, vp, vp, i64, vp]
            L.orc_bfs_round.restype = i64
            L.orc_minby_round.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
            L.orc_minby_round.restype = None
            L.orc_pagerank.argtypes = [i64, vp, vp, vp, i64, ctypes.c_double, i32, vp]
            L.orc_pagerank.restype = i32
            L.orc_reduce_minmax.argtypes = [i32, i32, i64, i64, vp, vp, vp, ctypes.c_double, ctypes.c_double, vp]
            L.orc_reduce_minmax.restype = None
            if fast:
                _fast_lib = L
            else:
                _lib = L
    return _fast_lib if fast else _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def dtype_code(a: np.ndarray | None, bf16: bool = False) -> int:
    if a is None:
        return T_NONE
    if bf16:
        return T_BF16
    return {np.dtype(np.float64): T_F64, np.dtype(np.float32): T_F32, np.dtype(np.int32): T_I32,
            np.dtype(np.int64): T_I64, np.dtype(np.bool_): T_BOOL,
            np.dtype(np.uint8): T_BOOL}[a.dtype]


def _i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def max_threads() -> int:
    return int(lib().orc_max_threads())


def spmv_csc(sr, m, n, ptr, idx, val, x, y=None, init=True, fma=True, bf16=False):
    """Finch's serial CSC nest y[i] <<(+)>>= A[i,j] (*) x[j] (1-based buffers)."""
    x = np.ascontiguousarray(x)
    at = dtype_code(x)
    if y is None:
        y = np.zeros(m, dtype=x.dtype)
    val = None if val is None else np.ascontiguousarray(val)
    lib().orc_spmv_csc(sr, dtype_code(val, bf16), at, m, n, _p(_i64(ptr)), _p(_i64(idx)), _p(val),
                       _p(x), _p(y), int(init), int(fma))
    return y


def spmv_csr(sr, m, n, ptr, idx, val, x, y=None, init=True, fma=True, bf16=False, nthreads=1):
    """Finch's row-pull nest (static thread split) over a CSR matrix."""
    x = np.ascontiguousarray(x)
    at = dtype_code(x)
    if y is None:
        y = np.zeros(m, dtype=x.dtype)
    val = None if val is None else np.ascontiguousarray(val)
    lib().orc_spmv_csr(sr, dtype_code(val, bf16), at, m, n, _p(_i64(ptr)), _p(_i64(idx)), _p(val),
                       _p(x), _p(y), int(init), int(fma), int(nthreads))
    return y


def spmm_csr(m, n, ptr, idx, val, B, C=None, init=True, fma=True, bf16=False, nthreads=1, fast=False):
    """C[i,k] += A[i,j] * B[j,k] for CSR A and row-major B (fast: the
    CPU-baseline build, for timing only)."""
    B = np.ascontiguousarray(B)
    nk = B.shape[1]
    if C is None:
        C = np.zeros((m, nk), dtype=B.dtype)
    at = dtype_code(B)
    val = np.ascontiguousarray(val)
    lib(fast).orc_spmm_csr(dtype_code(val, bf16), at, m, n, nk, _p(_i64(ptr)), _p(_i64(idx)), _p(val),
                       _p(B), B.shape[1], _p(C), C.shape[1], int(init), int(fma), int(nthreads))
    return C


def sddmm_csr(m, ptr, idx, val, X, Y, fma=True, acc64=False, nthreads=1):
    """out[q] = A(q) * sum_k X[i,k] Y[j,k] over the stored entries of CSR A."""
    X = np.ascontiguousarray(X)
    Y = np.ascontiguousarray(Y)
    val = np.ascontiguousarray(val)
    at = dtype_code(X)
    out = np.zeros(len(val), dtype=np.float64 if (acc64 or at == T_F64) else X.dtype)
    lib().orc_sddmm_csr(at, m, X.shape[1], _p(_i64(ptr)), _p(_i64(idx)), _p(val), _p(X),
                        X.shape[1], _p(Y), Y.shape[1], _p(out), int(fma), int(acc64),
                        int(nthreads))
    return out


def ewise(op, nf, pa, ia, va, pb, ib, vb):
    """Two-finger merge of two same-shape SparseList matrices (op 0 = *, 1 = +).

    Returns (ptr, idx, val) in Finch's 1-based layout."""
    va = np.ascontiguousarray(va)
    vb = np.ascontiguousarray(vb)
    pa, ia, pb, ib = _i64(pa), _i64(ia), _i64(pb), _i64(ib)
    out_ptr = np.zeros(nf + 1, dtype=np.int64)
    L = lib()
    L.orc_ewise(op, dtype_code(va), nf, _p(pa), _p(ia), _p(va), _p(pb), _p(ib), _p(vb),
                _p(out_ptr), None, None)
    nnz = int(out_ptr[-1] - 1)
    out_idx = np.zeros(nnz, dtype=np.int64)
    out_val = np.zeros(nnz, dtype=va.dtype)
    L.orc_ewise(op, dtype_code(va), nf, _p(pa), _p(ia), _p(va), _p(pb), _p(ib), _p(vb),
                _p(out_ptr), _p(out_idx), _p(out_val))
    return out_ptr, out_idx, out_val


def ewise_reduce(dims, m, n, pa, ia, va, pb=None, ib=None, vb=None, Bd=None):
    """sum(A .* B; dims) in double (B sparse CSR or dense row-major Bd)."""
    va = np.ascontiguousarray(va)
    length = 1 if dims == 0 else (m if dims == 2 else n)
    y = np.zeros(length, dtype=np.float64)
    if Bd is not None:
        Bd = np.ascontiguousarray(Bd, dtype=va.dtype)
    lib().orc_ewise_reduce(dims, dtype_code(va), m, n, _p(_i64(pa)), _p(_i64(ia)), _p(va),
                           None if pb is None else _p(_i64(pb)),
                           None if ib is None else _p(_i64(ib)),
                           None if vb is None else _p(np.ascontiguousarray(vb)),
                           _p(Bd), 0 if Bd is None else Bd.shape[1], _p(y))
    return y


def coo_assemble(m, n, I, J, V, csc=True, combine=0):
    """fsparse(I, J, V, (m, n), combine) copied into Dense(SparseList) (csc) or
    its row-major swizzle: returns 1-based (ptr, idx, val); val is None for a
    Pattern (V None).  Raises ValueError for out-of-range coordinates."""
    I, J = _i64(I), _i64(J)
    nin = I.size
    nfib = n if csc else m
    ptr = np.zeros(nfib + 1, dtype=np.int64)
    idx = np.zeros(max(nin, 1), dtype=np.int64)
    V = None if V is None else np.ascontiguousarray(V)
    val = None if V is None else np.zeros(max(nin, 1), dtype=V.dtype)
    q = lib().orc_coo_assemble(int(csc), dtype_code(V), combine, m, n, nin, _p(I), _p(J), _p(V),
                               _p(ptr), _p(idx), _p(val))
    if q < 0:
        raise ValueError("coordinate out of range")
    return ptr, idx[:q], (None if val is None else val[:q])


def spgemm_csr(m, n, lp, li, lv, rp, ri, rv, fma=True):
    """Gustavson's row-form SpGEMM of CSR buffers (1-based): (ptr, idx, val)
    of C = L * R with m rows and n columns, sums in the order of k."""
    lp, li, rp, ri = _i64(lp), _i64(li), _i64(rp), _i64(ri)
    lv, rv = np.ascontiguousarray(lv), np.ascontiguousarray(rv)
    if lv.dtype not in (np.float64, np.float32) or rv.dtype != lv.dtype:
        raise TypeError("spgemm_csr: F64 or F32 values of one type")
    ptr = np.zeros(m + 1, dtype=np.int64)
    nnz = lib().orc_spgemm_csr(dtype_code(lv), int(fma), m, n, _p(lp), _p(li), _p(lv), _p(rp),
                               _p(ri), _p(rv), _p(ptr), None, None)
    idx = np.zeros(max(nnz, 1), dtype=np.int64)
    val = np.zeros(max(nnz, 1), dtype=lv.dtype)
    lib().orc_spgemm_csr(dtype_code(lv), int(fma), m, n, _p(lp), _p(li), _p(lv), _p(rp), _p(ri),
                         _p(rv), _p(ptr), _p(idx), _p(val))
    return ptr, idx[:nnz], val[:nnz]


def bfs_round(n, ptr, idx, F, V, P, fill=0):
    """One round of Finch's BFS program (docs/examples/bfs.jl:25-42) over
    the CSC adjacency (column j lists the k with edges[k, j]): returns the
    next frontier and the count; V (uint8) and P (int64) update in place."""
    nF = np.zeros(n, dtype=np.uint8)
    c = lib().orc_bfs_round(n, _p(_i64(ptr)), _p(_i64(idx)), _p(np.ascontiguousarray(F, dtype=np.uint8)),
                            _p(V), _p(P), int(fill), _p(nF))
    return nF, int(c)


def pagerank(n, ptr, idx, w=None, nsteps=20, damp=0.85, fma=False):
    """Finch's PageRank example (docs/examples/pagerank.jl:7-51) over the
    CSC adjacency (column j lists the i with edges[i, j]); w None for a
    Pattern.  Returns r (float64).  The transition matrix is built over
    every (i, j) as Finch's nest builds it, so this needs n * n doubles."""
    r = np.zeros(n, dtype=np.float64)
    wp = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    rc = lib().orc_pagerank(n, _p(_i64(ptr)), _p(_i64(idx)), None if wp is None else _p(wp), int(nsteps),
                            float(damp), int(bool(fma)), _p(r))
    if rc != 0:
        raise MemoryError(f"oracle pagerank: {n} x {n} scratch")
    return r


def reduce_minmax(is_max, dims, m, n, ptr, idx, val, fill, init=None):
    """reduce(max | min, A; dims) of the CSC (ptr, idx, val) with fill `fill`,
    every coordinate folded in Finch's order (orc_reduce_minmax); float64."""
    if init is None:
        init = -np.inf if is_max else np.inf
    y = np.zeros(n if dims == 1 else (m if dims == 2 else 1), dtype=np.float64)
    lib().orc_reduce_minmax(int(bool(is_max)), int(dims), m, n, _p(_i64(ptr)), _p(_i64(idx)),
                            _p(np.ascontiguousarray(val, dtype=np.float64)), float(fill), float(init), _p(y))
    return y


def minby_round(n, ptr, idx, w, dprev, pprev, aprev, dist, par):
    """One relaxation round of Finch's Bellman-Ford program
    (docs/examples/shortest_paths.jl:22-42) over the CSC weights: (dist,
    par) update in place; returns the new active flags."""
    active = np.zeros(n, dtype=np.uint8)
    lib().orc_minby_round(n, _p(_i64(ptr)), _p(_i64(idx)), _p(np.ascontiguousarray(w, dtype=np.float64)),
                          _p(np.ascontiguousarray(dprev, dtype=np.float64)),
                          _p(np.ascontiguousarray(pprev, dtype=np.int64)),
                          _p(np.ascontiguousarray(aprev, dtype=np.uint8)), _p(dist), _p(par), _p(active))
    return active
