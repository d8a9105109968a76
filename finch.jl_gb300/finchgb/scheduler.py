"""The GB300 scheduler: matches Finch logic plans onto libfinchgb kernels.

This is the matcher that sits where Finch's LogicExecutor hands a plan to
its compiler (src/scheduler/LogicExecutor.jl:71-96): it inspects the plan's
structure -- output indices, reduction operator, the pointwise body and the
level formats of the operands -- and calls the kernel that computes it.
A plan with no kernel raises FinchGBUnsupported: there is no CPU fallback.

Matched plans (A sparse, x/B/X/Y dense, s a 0-d Scalar):
  y[i]   (+)= A[i,j] (*) x[j]             semiring SpMV (+,*) (min,+) (max,+) (|,&)
  C[i,k]  += A[i,j] * B[j,k]              SpMM
  C[i,j]  += A[i,j] * X[i,k] * Y[j,k]     SDDMM (also A .* (X * Y^T))
  C[i,j]   = A[i,j] (*|+) B[i,j]          sparse elementwise (two-finger merge)
  y[..]   += A[i,j] (* B[i,j])            fused elementwise + reduce, reduce(+, A)
  s[]     += x[i] * y[i]                  dense dot
  z[i]     = x[i] (+|-|*|min|max) y[i], x[i] +/- s[] * y[i], ...   dense maps
  s[]      = a[] (op) b[]                 scalar arithmetic
"""
from __future__ import annotations

import contextlib
import functools
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib as L
from . import device as dev
from .algebra import AbstractAlgebra, DefaultAlgebra
from .logic import (Access, Aggregate, EinsumPlan, LazyTensor, Literal, MapJoin, Node, Reorder,
                    flatten, indices_of, parse_einsum, parse_finch)
from .tensors import (GPU, SwizzleArray, Tensor, dense_from_device, sparse_from_device, transfer)


class FinchGBUnsupported(NotImplementedError):
    """The plan has no GB300 kernel (and there is no CPU fallback)."""


class Scalar:
    """Finch's 0-d Scalar (src/tensors/scalars.jl:22-93), held in HBM."""

    def __init__(self, value, dtype=np.float64):
        if isinstance(value, torch.Tensor):
            self.t = value.reshape(())
        else:
            self.t = torch.tensor(value, dtype=_torch_dtype(np.dtype(dtype)), device="cuda")
        self.shape = ()

    def __getitem__(self, key):
        assert key == () or key is Ellipsis
        return self.t.item()

    @property
    def value(self):
        return self.t.item()

    def device_value(self, dtype) -> torch.Tensor:
        """The 0-d device value, which kernels update in place (of `dtype`)."""
        if self.t.dtype != dtype:
            raise FinchGBUnsupported(f"Scalar of {self.t.dtype}, expected {dtype}")
        return self.t

    def __float__(self):
        return float(self.t.item())

    def __repr__(self):
        return f"Scalar({self.value})"


def _torch_dtype(dt: np.dtype):
    return {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
            np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
            np.dtype(np.bool_): torch.uint8}[np.dtype(dt)]


# ---------------------------------------------------------------- operands


def _is_sparse(t) -> bool:
    return isinstance(t, (Tensor, SwizzleArray)) and t.is_sparse()


def _is_dense(t) -> bool:
    return isinstance(t, (Tensor, SwizzleArray)) and not t.is_sparse()


def _device_index():
    return torch.cuda.current_device()


def sparse_operand(t, idxs: tuple, want: tuple) -> dev.DeviceSparse:
    """DeviceSparse of the logical matrix M with M[want] = t[idxs]."""
    body = t.body if isinstance(t, SwizzleArray) else t
    transfer(GPU(_device_index()), body)
    d = body.dsparse
    if body.kind == "sparse1":
        raise FinchGBUnsupported("sparse vectors as matrix operands")
    if isinstance(t, SwizzleArray):
        if t.dims != (2, 1):
            raise FinchGBUnsupported(f"swizzle {t.dims}")
        d = d.T()
    if tuple(idxs) == tuple(want):
        return d
    if tuple(idxs) == tuple(reversed(want)):
        return d.T()
    raise FinchGBUnsupported(f"access {idxs} vs {want}")


def dense_operand(t, idxs: tuple, want: tuple) -> torch.Tensor:
    """Row-major device array D with D[want] = t[idxs]."""
    body = t.body if isinstance(t, SwizzleArray) else t
    transfer(GPU(_device_index()), body)
    d = body.ddata
    order = list(idxs)
    if isinstance(t, SwizzleArray):
        order = [None] * len(idxs)
        for pos, dim in enumerate(t.dims):
            order[dim - 1] = idxs[pos]
    if order == list(want):
        return d
    if sorted(order) == sorted(want) and len(want) == 2:
        return d.t().contiguous()
    raise FinchGBUnsupported(f"dense access {idxs} vs {want}")


_CONST_OPS = {"+": lambda a, b: a + b, "-": lambda a, b: a - b, "*": lambda a, b: a * b,
              "/": lambda a, b: a / b}


def _constant(n):
    """The value of an expression of literals (Julia's arithmetic on Float64
    and Int values, evaluated on the host), else None."""
    if isinstance(n, Literal):
        v = n.value
        return v if isinstance(v, (int, float, np.integer, np.floating)) and not isinstance(v, bool) else None
    if isinstance(n, MapJoin) and n.op in _CONST_OPS and len(n.args) == 2:
        a, b = _constant(n.args[0]), _constant(n.args[1])
        if a is None or b is None:
            return None
        if n.op == "/":  # Julia's / always gives a float
            return float(a) / float(b) if b != 0 else (float("nan") if a == 0 else float(np.sign(a)) * float("inf"))
        return _CONST_OPS[n.op](a, b)
    return None


_LITERALS: dict = {}


def _scalar_tensor(x, like_dtype) -> torch.Tensor:
    """The device scalar of a Scalar, or of a literal.  A literal's device
    copy is made once per (value, type, device) and reused: kernels only
    read these, and a fresh copy costs a synchronous host-to-device
    transfer per call."""
    if isinstance(x, Scalar):
        return x.t
    key = (type(x), x, like_dtype, torch.cuda.current_device())
    t = _LITERALS.get(key)
    if t is None:
        t = torch.tensor(x, dtype=like_dtype, device="cuda")
        if len(_LITERALS) < 1024:  # entries are never dropped: a kernel on any stream may still read one
            _LITERALS[key] = t
    return t


# ---------------------------------------------------------------- matching


@dataclass
class Match:
    outs: tuple
    agg: str | None
    init: object
    red: tuple
    core: Node


def _decompose(root: Node) -> Match:
    root = flatten(root)
    if not isinstance(root, Reorder):
        root = Reorder(root, indices_of(root))
    body = root.arg
    if isinstance(body, Aggregate):
        return Match(root.idxs, body.op, body.init, body.idxs, body.arg)
    return Match(root.idxs, None, None, (), body)


_SEMIRINGS = {("+", "*"): L.PLUS_TIMES, ("min", "+"): L.MIN_PLUS, ("max", "+"): L.MAX_PLUS,
              ("|", "&"): L.OR_AND}


def _args(core: Node, op: str):
    if isinstance(core, MapJoin) and core.op == op:
        return list(core.args)
    return None


class GB300Scheduler:
    """Callable scheduler object: scheduler(plan) -> result.

    `finch_order=True` evaluates float sums in Finch's serial order (one
    running value per output, j ascending), bit-identical to Finch's CPU
    nest; otherwise lane-parallel reductions are used.  `algebra` decides,
    as Finch's algebra does, whether a sparse operand's fill may be skipped:
    every kernel visits stored entries only, so a plan matches one only when
    the fill annihilates the product (or, for sums of one operand, is the
    identity of the sum)."""

    # the options that make two schedulers equal (src/scheduler/
    # LogicExecutor.jl:77-78 compares and hashes the options, not the state)
    OPTIONS = ("finch_order", "verbose", "algebra")

    def __init__(self, finch_order: bool = False, verbose: bool = False,
                 algebra: AbstractAlgebra | None = None):
        self.finch_order = finch_order
        self.verbose = verbose
        self.algebra = algebra if algebra is not None else DefaultAlgebra()
        self.last_kernel = None

    def options(self) -> dict:
        return {k: getattr(self, k) for k in self.OPTIONS}

    def set_options(self, **kw):
        """A new scheduler with the given options changed, the others kept
        (src/scheduler/LogicExecutor.jl:81-82); an unknown option raises."""
        unknown = sorted(set(kw) - set(self.OPTIONS))
        if unknown:
            raise TypeError(f"unknown scheduler option(s) {unknown}; known: {list(self.OPTIONS)}")
        return type(self)(**{**self.options(), **kw})

    def __eq__(self, other):
        return type(self) is type(other) and self.options() == other.options()

    def __hash__(self):
        return hash((type(self).__name__, tuple(sorted(self.options().items()))))

    def _skippable(self, t, op: str, kind: str = "annihilator") -> None:
        """Refuses a sparse operand whose fill the algebra does not let the
        kernel skip: op's annihilator (a product) or identity (a sum)."""
        fill = (t.body if isinstance(t, SwizzleArray) else t).fill_value
        test = self.algebra.isannihilator if kind == "annihilator" else self.algebra.isidentity
        if not test(op, fill):
            raise FinchGBUnsupported(
                f"the fill {fill!r} of {t!r} is not the {kind} of {op!r} in {self.algebra!r}: the kernels "
                f"skip unstored entries (declare it in an algebra of your own)")

    def __call__(self, plan: Node, out=None, accumulate=False):
        m = _decompose(plan)
        for rule in (self._spmv, self._spmm, self._spmm_semiring, self._spgemm, self._sddmm, self._ewise,
                     self._ewise_reduce, self._reduce_minmax, self._dot, self._dense_map, self._dense_fill,
                     self._scalar):
            r = rule(m, out, accumulate)
            if r is not None:
                if self.verbose:
                    print(f"[finchgb] {plan!r} -> {self.last_kernel}")
                return r
        raise FinchGBUnsupported(f"no GB300 kernel matches {plan!r}")

    # -- y[i] (+)= A[i,j] (*) x[j]
    def _spmv(self, m: Match, out, accumulate):
        if m.agg not in ("+", "min", "max", "|") or len(m.outs) != 1 or len(m.red) != 1:
            return None
        (i,), (j,) = m.outs, m.red
        for mul in ("*", "+", "&"):
            args = _args(m.core, mul)
            if args is None or len(args) != 2 or (m.agg, mul) not in _SEMIRINGS:
                continue
            for a, x in (args, args[::-1]):
                if (isinstance(a, Access) and _is_sparse(a.tns) and len(a.idxs) == 2
                        and set(a.idxs) == {i, j} and isinstance(x, Access) and _is_dense(x.tns)
                        and x.idxs == (j,)):
                    sr = _SEMIRINGS[(m.agg, mul)]
                    self._skippable(a.tns, mul)
                    A = sparse_operand(a.tns, a.idxs, (i, j))
                    xv = dense_operand(x.tns, x.idxs, (j,))
                    flags = 0
                    if self.finch_order and sr == L.PLUS_TIMES and xv.is_floating_point():
                        flags |= L.FINCH_ORDER
                        if A.orient == "csc":
                            A = _csr_copy(a.tns, A)
                    elif A.orient == "csc" and _reused(a.tns):
                        # a CSC operand used again (an iterative program): pull over
                        # a CSR copy built once -- no atomics, deterministic sums
                        A = _csr_copy(a.tns, A)
                    y = None
                    if out is not None:
                        y = dense_operand(out, (i,), (i,))
                        if accumulate:
                            flags |= L.ACCUMULATE
                    self.last_kernel = f"fgb_spmv[{sr},{A.orient}]"
                    y = dev.spmv(A, xv, y, semiring=sr, flags=flags)
                    return dense_from_device(y, m.init if m.init is not None else 0)
        return None

    # -- C[i,k] += A[i,j] * B[j,k]
    def _spmm(self, m: Match, out, accumulate):
        if m.agg != "+" or len(m.outs) != 2 or len(m.red) != 1:
            return None
        args = _args(m.core, "*")
        if not args or len(args) != 2:
            return None
        (i, k), (j,) = m.outs, m.red
        for a, b in (args, args[::-1]):
            if (isinstance(a, Access) and _is_sparse(a.tns) and set(a.idxs) == {i, j}
                    and isinstance(b, Access) and _is_dense(b.tns) and set(b.idxs) == {j, k}):
                self._skippable(a.tns, "*")
                A = sparse_operand(a.tns, a.idxs, (i, j))
                if A.orient == "csc":
                    A = _csr_copy(a.tns, A)
                B = dense_operand(b.tns, b.idxs, (j, k))
                flags = L.ACCUMULATE if (out is not None and accumulate) else 0
                C = None if out is None else dense_operand(out, (i, k), (i, k))
                self.last_kernel = "fgb_spmm"
                C = dev.spmm(A, B, C, flags=flags)
                return dense_from_device(C)
        return None

    # -- C[i,k] <<min|max>>= A[i,j] + B[j,k], C[i,k] |= A[i,j] & B[j,k]: exact semiring products
    def _spmm_semiring(self, m: Match, out, accumulate):
        if m.agg not in ("min", "max", "|") or len(m.outs) != 2 or len(m.red) != 1:
            return None
        (i, k), (j,) = m.outs, m.red
        for mul in ("+", "&"):
            args = _args(m.core, mul)
            if args is None or len(args) != 2 or (m.agg, mul) not in _SEMIRINGS:
                continue
            for a, b in (args, args[::-1]):
                if not (isinstance(a, Access) and _is_sparse(a.tns) and set(a.idxs) == {i, j}
                        and isinstance(b, Access) and set(b.idxs) == {j, k}):
                    continue
                sr = _SEMIRINGS[(m.agg, mul)]
                # only A's stored entries are visited, which is exact when A's
                # fill annihilates the product: +-Inf for (+), false for (&)
                # (src/symbolic/symbolic.jl:89-166)
                self._skippable(a.tns, mul)
                want = {L.MAX_PLUS: -np.inf, L.MIN_PLUS: np.inf, L.OR_AND: False}[sr]
                A = sparse_operand(a.tns, a.idxs, (i, j))
                if A.orient == "csc":
                    A = _csr_copy(a.tns, A)
                if _is_dense(b.tns):
                    B = dense_operand(b.tns, b.idxs, (j, k))
                else:  # a sparse right operand: its dense copy in HBM, fill included
                    bs = sparse_operand(b.tns, b.idxs, (j, k))
                    bfill = (b.tns.body if isinstance(b.tns, SwizzleArray) else b.tns).fill_value
                    B = dev.sparse_to_dense(bs, bfill)
                if A.val is not None and A.val.dtype != B.dtype:
                    raise FinchGBUnsupported(f"semiring product of {A.val.dtype} and {B.dtype}")
                flags = L.ACCUMULATE if (out is not None and accumulate) else 0
                C = None if out is None else dense_operand(out, (i, k), (i, k))
                self.last_kernel = f"fgb_spmm_semiring[{sr}]"
                C = dev.spmm_semiring(A, B, C, semiring=sr, flags=flags)
                return dense_from_device(C, m.init if m.init is not None else want)
        return None

    # -- C[i,k] += A[i,j] * B[j,k] with both sparse: a sparse result (Gustavson)
    def _spgemm(self, m: Match, out, accumulate):
        if m.agg != "+" or len(m.outs) != 2 or len(m.red) != 1 or out is not None:
            return None
        args = _args(m.core, "*")
        if not args or len(args) != 2:
            return None
        (i, k), (j,) = m.outs, m.red
        a, b = args
        if not all(isinstance(t, Access) and _is_sparse(t.tns) for t in (a, b)):
            return None
        if set(a.idxs) != {i, j}:
            a, b = b, a
        if set(a.idxs) != {i, j} or set(b.idxs) != {j, k}:
            return None
        self._skippable(a.tns, "*")
        self._skippable(b.tns, "*")
        A = sparse_operand(a.tns, a.idxs, (i, j))
        B = sparse_operand(b.tns, b.idxs, (j, k))
        if A.val is None or B.val is None:
            return None
        if B.orient != A.orient:
            B = _other_orientation(b.tns, B)
        self.last_kernel = "fgb_spgemm"
        return sparse_from_device(dev.spgemm(A, B))

    # -- C[i,j] = A[i,j] * sum_k X[i,k] * Y[j,k]
    def _sddmm(self, m: Match, out, accumulate):
        if len(m.outs) != 2:
            return None
        i, j = m.outs
        A = X = Y = None
        if m.agg == "+" and len(m.red) == 1:
            k = m.red[0]
            args = _args(m.core, "*")
            if not args or len(args) != 3:
                return None
        elif m.agg is None:
            args = _args(m.core, "*")
            if not args or len(args) != 2:
                return None
            inner = [a for a in args if isinstance(a, Aggregate)]
            if len(inner) != 1 or inner[0].op != "+" or len(inner[0].idxs) != 1:
                return None
            k = inner[0].idxs[0]
            ia = _args(flatten(inner[0].arg), "*")
            if not ia or len(ia) != 2:
                return None
            args = [a for a in args if not isinstance(a, Aggregate)] + ia
        else:
            return None
        for a in args:
            if not isinstance(a, Access):
                return None
            if _is_sparse(a.tns) and set(a.idxs) == {i, j}:
                A = a
            elif _is_dense(a.tns) and set(a.idxs) == {i, k}:
                X = a
            elif _is_dense(a.tns) and set(a.idxs) == {j, k}:
                Y = a
        if A is None or X is None or Y is None:
            return None
        self._skippable(A.tns, "*")
        Ad = sparse_operand(A.tns, A.idxs, (i, j))
        Xd = dense_operand(X.tns, X.idxs, (i, k))
        Yd = dense_operand(Y.tns, Y.idxs, (j, k))
        flags = L.FINCH_ORDER if self.finch_order else 0
        self.last_kernel = "fgb_sddmm"
        vals = dev.sddmm(Ad, Xd, Yd, flags=flags)
        res = dev.DeviceSparse(Ad.nrows, Ad.ncols, Ad.ptr, Ad.idx, vals, Ad.orient, Ad.base)
        return sparse_from_device(res)

    # -- C[i,j] = A[i,j] (*|+) B[i,j]
    def _ewise(self, m: Match, out, accumulate):
        if m.agg is not None or len(m.outs) != 2 or not isinstance(m.core, MapJoin):
            return None
        if m.core.op not in ("*", "+") or len(m.core.args) != 2:
            return None
        a, b = m.core.args
        if not (isinstance(a, Access) and isinstance(b, Access) and _is_sparse(a.tns)
                and _is_sparse(b.tns)):
            return None
        i, j = m.outs
        # a product is stored where both are (each fill annihilates it); a
        # sum where either is (each fill the identity of the sum)
        kind = "annihilator" if m.core.op == "*" else "identity"
        self._skippable(a.tns, m.core.op, kind)
        self._skippable(b.tns, m.core.op, kind)
        Ad = sparse_operand(a.tns, a.idxs, (i, j))
        Bd = sparse_operand(b.tns, b.idxs, (i, j))
        if Ad.orient != Bd.orient:
            Bd = _other_orientation(b.tns, Bd)
        self.last_kernel = "fgb_ewise"
        C = dev.ewise(L.EW_MUL if m.core.op == "*" else L.EW_ADD, Ad, Bd)
        return sparse_from_device(C)

    # -- y[..] += A[i,j] (* B[i,j])
    def _ewise_reduce(self, m: Match, out, accumulate):
        if m.agg != "+":
            return None
        terms = _args(m.core, "*") or [m.core]
        sp = [t for t in terms if isinstance(t, Access) and _is_sparse(t.tns)]
        if not sp or len(terms) > 2 or not all(isinstance(t, Access) for t in terms):
            return None
        a = sp[0]
        if len(a.idxs) != 2:
            return None
        i, j = a.idxs
        if set(m.outs) | set(m.red) != {i, j}:
            return None
        others = [t for t in terms if t is not a]
        if others and set(others[0].idxs) != {i, j}:
            return None
        if others:
            self._skippable(a.tns, "*")
        else:
            self._skippable(a.tns, "+", "identity")
        Ad = sparse_operand(a.tns, a.idxs, (i, j))
        Bs = Bdn = None
        if others:
            o = others[0]
            if _is_sparse(o.tns):
                Bs = sparse_operand(o.tns, o.idxs, (i, j))
                if Bs.orient != Ad.orient:
                    Bs = _other_orientation(o.tns, Bs)
            else:
                Bdn = dense_operand(o.tns, o.idxs, (i, j))
        dims = 0 if not m.outs else (2 if m.outs == (i,) else 1)
        self.last_kernel = "fgb_ewise_reduce"
        y = dev.ewise_reduce(dims, Ad, B=Bs, B_dense=Bdn)
        if dims == 0:
            return Scalar(y.reshape(()))
        return dense_from_device(y)

    # -- y[j] <<max|min>>= A[i,j] (or over both indices): reduce(max|min, A; dims),
    #    the fill folded where A stores nothing, so any fill is exact
    def _reduce_minmax(self, m: Match, out, accumulate):
        if m.agg not in ("max", "min") or (out is not None and accumulate):
            return None
        a = m.core
        if not (isinstance(a, Access) and _is_sparse(a.tns) and len(a.idxs) == 2) or len(m.outs) > 1:
            return None
        i, j = a.idxs
        if set(m.outs) | set(m.red) != {i, j}:
            return None
        Ad = sparse_operand(a.tns, a.idxs, (i, j))
        if Ad.val is None or Ad.val.dtype not in (torch.float64, torch.float32, torch.int64, torch.int32):
            return None
        dims = 0 if not m.outs else (1 if m.outs == (j,) else 2)
        want = {1: "csc", 2: "csr"}.get(dims, Ad.orient)
        if Ad.orient != want:
            Ad = _other_orientation(a.tns, Ad)
        fill = (a.tns.body if isinstance(a.tns, SwizzleArray) else a.tns).fill_value
        init = m.init
        if init is not None and not Ad.val.dtype.is_floating_point and isinstance(init, float) and np.isinf(init):
            init = None  # -Inf / +Inf: typemin / typemax for integers
        self.last_kernel = "fgb_reduce_minmax"
        y = dev.reduce_minmax(L.MAP_MAX if m.agg == "max" else L.MAP_MIN, dims, Ad, fill, init)
        if dims == 0:
            return Scalar(y.reshape(()))
        return dense_from_device(y)

    # -- s[] += x[i] * y[i]
    def _dot(self, m: Match, out, accumulate):
        if m.agg != "+" or m.outs or len(m.red) != 1:
            return None
        args = _args(m.core, "*")
        if not args or len(args) != 2 or not all(isinstance(a, Access) and _is_dense(a.tns)
                                                 for a in args):
            return None
        x = dense_operand(args[0].tns, args[0].idxs, m.red)
        y = dense_operand(args[1].tns, args[1].idxs, m.red)
        o = None if out is None else out.t
        self.last_kernel = "fgb_dense_dot"
        return Scalar(dev.dot(x, y, o))

    # -- z[i] = pointwise over dense vectors and scalars
    def _dense_map(self, m: Match, out, accumulate):
        if m.agg is not None or len(m.outs) != 1 or not isinstance(m.core, MapJoin):
            return None
        (i,) = m.outs
        core = m.core

        def vec(n):
            if isinstance(n, Access) and _is_dense(n.tns) and n.idxs == (i,):
                return dense_operand(n.tns, n.idxs, (i,))
            return None

        def scaled(n):  # s[] * v[i] or v[i] * s[]
            if isinstance(n, MapJoin) and n.op == "*" and len(n.args) == 2:
                for s, v in (n.args, n.args[::-1]):
                    vv = vec(v)
                    if vv is not None and (isinstance(s, Literal) or (
                            isinstance(s, Access) and isinstance(s.tns, Scalar))):
                        sv = s.value if isinstance(s, Literal) else s.tns
                        return _scalar_tensor(sv, vv.dtype), vv
            vv = vec(n)
            return (None, vv) if vv is not None else None

        o = None if out is None else dense_operand(out, (i,), (i,))
        if core.op in ("+", "-") and len(core.args) == 2:
            p, q = scaled(core.args[0]), scaled(core.args[1])
            if p is not None and q is not None:
                self.last_kernel = "fgb_dense_axpby"
                signs = 2 if core.op == "-" else 0
                r = dev.axpby(p[0], p[1], q[0], q[1], o, signs=signs)
                return dense_from_device(r)
        ops = {"+": L.MAP_ADD, "-": L.MAP_SUB, "*": L.MAP_MUL, "min": L.MAP_MIN, "max": L.MAP_MAX}
        if core.op in ops and len(core.args) == 2:
            x, y = vec(core.args[0]), vec(core.args[1])
            if x is not None and y is not None:
                self.last_kernel = "fgb_dense_map"
                return dense_from_device(dev.dense_map(ops[core.op], x, y, o))
        if core.op == "*" and len(core.args) == 2:
            s = scaled(core)
            if s is not None:
                self.last_kernel = "fgb_dense_axpby"
                return dense_from_device(dev.axpby(s[0], s[1], None, None, o))
        if core.op == "+" and len(core.args) == 2:  # c + s*x or s*x + c, c a constant
            for c, t in (core.args, core.args[::-1]):
                cv = _constant(c)
                sx = scaled(t)
                if cv is not None and sx is not None:
                    x = sx[1]
                    self.last_kernel = "fgb_dense_affine"
                    r = dev.dense_affine(sx[0], x, _scalar_tensor(cv, x.dtype),
                                         torch.empty_like(x) if o is None else o)
                    return dense_from_device(r)
        return None

    # -- z[i] = c: an assignment of a constant, the extent taken from the output
    def _dense_fill(self, m: Match, out, accumulate):
        if m.agg is not None or len(m.outs) != 1 or out is None:
            return None
        cv = _constant(m.core)
        if cv is None:
            return None
        (i,) = m.outs
        o = dense_operand(out, (i,), (i,))
        self.last_kernel = "fgb_dense_affine"
        return dense_from_device(dev.dense_affine(None, None, _scalar_tensor(cv, o.dtype), o))

    # -- s[] = a[] op b[]
    def _scalar(self, m: Match, out, accumulate):
        if m.agg is not None or m.outs or not isinstance(m.core, MapJoin) or len(m.core.args) != 2:
            return None
        ops = {"+": L.MAP_ADD, "-": L.MAP_SUB, "*": L.MAP_MUL, "/": L.MAP_DIV, "min": L.MAP_MIN,
               "max": L.MAP_MAX}
        if m.core.op not in ops:
            return None
        vals = []
        for n in m.core.args:
            if isinstance(n, Access) and isinstance(n.tns, Scalar):
                vals.append(n.tns.t)
            elif isinstance(n, Literal):
                vals.append(None)
            else:
                return None
        like = next((v for v in vals if v is not None), None)
        if like is None:
            return None
        a = vals[0] if vals[0] is not None else _scalar_tensor(m.core.args[0].value, like.dtype)
        b = vals[1] if vals[1] is not None else _scalar_tensor(m.core.args[1].value, like.dtype)
        self.last_kernel = "fgb_scalar_op"
        return Scalar(dev.scalar_op(ops[m.core.op], a, b, None if out is None else out.t))


def _reused(t) -> bool:
    """Counts SpMV uses of a tensor; true from its second use on."""
    body = t.body if isinstance(t, SwizzleArray) else t
    n = getattr(body, "_gb_uses", 0) + 1
    body._gb_uses = n
    return n >= 2


def _csr_copy(t, A: dev.DeviceSparse) -> dev.DeviceSparse:
    """A CSR copy of a CSC operand, built once on the device and cached."""
    return _other_orientation(t, A)


def _other_orientation(t, A: dev.DeviceSparse) -> dev.DeviceSparse:
    body = t.body if isinstance(t, SwizzleArray) else t
    cache = getattr(body, "_gb_transposed", None)
    if cache is None:
        cache = {}
        body._gb_transposed = cache
    key = (A.orient, A.nrows, A.ncols, A.ptr.data_ptr())
    if key not in cache:
        cache[key] = A.transposed_storage()
    return cache[key]


# ---------------------------------------------------------------- scheduler selection

_scheduler = GB300Scheduler()


def get_scheduler() -> GB300Scheduler:
    return _scheduler


def set_scheduler(s: GB300Scheduler) -> None:
    """set_scheduler! (src/interface/lazy.jl:666-712)."""
    global _scheduler
    _scheduler = s


@contextlib.contextmanager
def with_scheduler(s: GB300Scheduler):
    global _scheduler
    prev, _scheduler = _scheduler, s
    try:
        yield s
    finally:
        _scheduler = prev


def default_scheduler(**kw) -> GB300Scheduler:
    return GB300Scheduler(**kw)


# ---------------------------------------------------------------- front ends


def compute(x, ctx: GB300Scheduler | None = None, verbose: bool = False):
    """compute(lazy_expr; ctx) (src/interface/lazy.jl:709-730)."""
    if not isinstance(x, LazyTensor):
        return x
    sched = ctx or _scheduler
    if verbose:
        sched.verbose = True
    return sched(Reorder(x.node, x.idxs))


def _with_algebra(sched: GB300Scheduler, algebra: AbstractAlgebra | None) -> GB300Scheduler:
    return sched if algebra is None or sched.algebra == algebra else sched.set_options(algebra=algebra)


def einsum(stmt: str, init=None, ctx: GB300Scheduler | None = None, algebra: AbstractAlgebra | None = None,
           **tensors):
    """@einsum (src/interface/einsum.jl:190-201):

        y = einsum("y[i] += A[i,j] * x[j]", A=A, x=x)
        y = einsum("y[i] <<min>>= A[i,j] + x[j]", A=A, x=x)
        s = einsum("s[] += r[i] * r[i]", r=r)

    algebra: as Finch's `@finch algebra ...`, the properties that decide
    whether unstored entries may be skipped (default: DefaultAlgebra)."""
    plan: EinsumPlan = parse_einsum(stmt, tensors, init)
    return _with_algebra(ctx or _scheduler, algebra)(plan.logic())


def _device_vector(t, dtype) -> torch.Tensor:
    """The HBM array of a Dense(Element) vector (moved there once); Bool
    vectors are one byte per entry.  dtype None: any element type."""
    body = t.body if isinstance(t, SwizzleArray) else t
    if not isinstance(body, Tensor) or body.kind != "dense1":
        raise FinchGBUnsupported("expected a Dense(Element) vector")
    transfer(GPU(_device_index()), body)
    d = body.ddata
    if dtype is not None and d.dtype != dtype:
        raise FinchGBUnsupported(f"vector of {d.dtype}, expected {dtype}")
    return d


def _rows_of(t) -> dev.DeviceSparse:
    """The CSR of matrix t (row i lists the j with t[i, j] stored), built
    once on the device from Finch's Dense(SparseList) and cached."""
    A = sparse_operand(t, ("i", "j"), ("i", "j"))
    return A if A.orient == "csr" else _csr_copy(t, A)


@functools.lru_cache(maxsize=256)
def _program_tree(program: str):
    """The FinchNotation tree of a program's text, parsed once per text (as
    Finch compiles a program once per type signature, src/util/staging.jl:
    22-79); None when it does not parse."""
    from . import notation

    try:
        return notation.parse(program)
    except SyntaxError:
        return None


@functools.lru_cache(maxsize=256)
def _program_match(program: str):
    """The whole-program match of a program's text (programs.match), found
    once per text."""
    from . import programs

    tree = _program_tree(program)
    return None if tree is None else programs.match(tree)


@functools.lru_cache(maxsize=256)
def _finch_program(program: str):
    return parse_finch(program)


def finch(program: str, ctx: GB300Scheduler | None = None, algebra: AbstractAlgebra | None = None,
          **tensors) -> dict:
    """@finch over a loop program; returns {output name: tensor}.

    A program that initialises its output (`y .= 0`) gets a fresh result;
    without it the output tensor passed in is accumulated into.  Float sums
    use Finch's serial order, so results equal Finch's CPU nest.  Graph
    programs with several statements (the choose/minby rounds of Finch's BFS
    and Bellman-Ford examples) are matched as whole programs and update
    their tensors in place."""
    from . import programs

    found = _program_match(program)
    if found is not None:
        return programs.run_matched(found[0], found[1], tensors, _rows_of)
    prog = _finch_program(program)
    plan = parse_einsum(prog.stmt, tensors)
    name = plan.out_name
    sched = _with_algebra(ctx or GB300Scheduler(finch_order=True), algebra)
    if name in prog.init:
        init = prog.init[name]
        if plan.op is not None and init != _identity_value(plan.op, init):
            raise FinchGBUnsupported(f"@finch: {name} .= {init} is not the identity of {plan.op}")
        if name in tensors and set(plan.out_idxs) - set(indices_of(flatten(plan.rhs))):
            # `r[j] = c`: no operand gives j its extent, the output does (and is overwritten)
            res = sched(plan.logic(), out=tensors[name], accumulate=False)
        else:
            res = sched(plan.logic())
    else:
        if name not in tensors:
            raise KeyError(f"@finch: output {name} must be passed when it is not initialised")
        res = sched(plan.logic(), out=tensors[name], accumulate=True)
    return {name: res}


def _identity_value(op, init):
    from .logic import IDENTITY

    ident = IDENTITY[op]
    if isinstance(init, (int, float)) and isinstance(ident, float) and np.isinf(ident):
        return init if np.isinf(init) or abs(init) >= 2**31 - 1 else ident
    return ident
