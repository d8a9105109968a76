"""Cost-based planning of sum-product expressions onto the GB300 kernels.

Finch's Galley optimizer (`galley_scheduler`, src/Galley/FinchCompat/
executor.jl:173-181) plans a sum-product query by eliminating its reduced
indices one at a time.  Each elimination is a smaller query, and its cost is
estimated from sparsity statistics of its inputs: uniform `NaiveStats` or
degree-constraint `DCStats` (src/Galley/TensorStats/tensor-stats.jl:181-305).
The greedy order is src/Galley/LogicalOptimizer/greedy-optimizer.jl:1-40.
Each intermediate's level format then follows from its estimated density
(src/Galley/PhysicalOptimizer/format-selector.jl:27-65).

`GalleyScheduler` does the same onto this library's kernels, each a binary
contraction with its output kept in HBM:

  S[i,v] * x[v]    -> dense y[i]      fgb_spmv
  S[i,v] * D[v,k]  -> dense C[i,k]    fgb_spmm
  S[i,v] * T[v,k]  -> sparse C[i,k]   fgb_spgemm (a SparseList intermediate)
  S[i,v] * X[i,v]  -> dense y[i]      fgb_ewise_reduce (X sparse or dense)
  S[i,v]           -> dense y[i]      fgb_ewise_reduce
  x[v] * y[v]      -> scalar          fgb_dense_dot
  S[i,k] .* T[i,k] -> sparse C[i,k]   fgb_ewise (pointwise, after every reduction)

It searches every elimination order (greedy beyond 5 reduced indices).  Each
step is costed with this device's measured rates: HBM streaming, random
gathers from an L2-resident or HBM-sized working set, and SpGEMM products
per second.  The plan with the least estimated time runs.  A query that no
order maps onto these kernels (a reduced index shared by three factors, a
dense-by-dense contraction) raises FinchGBUnsupported; there is no CPU
fallback.

Unlike Galley, which also chooses among dense, bytemap, hash and sparse-list
intermediates, this module's intermediate formats follow from the kernel:
sparse-by-sparse gives a sparse list, anything with a dense operand a dense
array.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .logic import Access, Aggregate, MapJoin, Node, Reorder, flatten, indices_of
from .scheduler import (FinchGBUnsupported, GB300Scheduler, Scalar, _csr_copy, _is_dense, _is_sparse,
                        _other_orientation)
from .tensors import SwizzleArray, swizzle

# Rates of this library's kernels on a GB300, measured by its benchmark.
HBM_BPS = 6.7e12         # streaming copy bandwidth
GATHER_L2_BPS = 9.5e12   # random 128-byte gathers from a working set that fits L2 (<= 64 MB)
GATHER_HBM_BPS = 5.6e12  # the same from a working set far larger than L2 (>= 512 MB)
SECTOR_GATHERS = 2.2e11  # random 4- or 8-byte gathers per second from an L2-resident vector
SPGEMM_PRODUCTS = 1.66e10  # products per second of the row-wise SpGEMM
LAUNCH_S = 4e-6          # one kernel launch
L2_BYTES = 126e6


def gather_bps(working_set: float) -> float:
    """Random-gather rate for a working set, interpolated in log space between
    the L2-resident and the HBM-sized measurements."""
    if working_set <= 64e6:
        return GATHER_L2_BPS
    if working_set >= 512e6:
        return GATHER_HBM_BPS
    f = math.log(working_set / 64e6) / math.log(8.0)
    return GATHER_L2_BPS * (1 - f) + GATHER_HBM_BPS * f


# ---------------------------------------------------------------- statistics


@dataclass
class Stats:
    """Sparsity statistics of one factor.

    dims: extent per index.  nnz: stored entries (estimated for
    intermediates).  deg: per index, the most stored entries that share one
    value of that index (a degree constraint; DCStats keeps such bounds).
    esz: bytes per value."""

    dims: dict
    nnz: float
    dense: bool
    deg: dict = field(default_factory=dict)
    esz: int = 8

    @property
    def size(self) -> float:
        return float(np.prod([self.dims[i] for i in self.dims])) if self.dims else 1.0

    @property
    def density(self) -> float:
        return self.nnz / self.size if self.size else 0.0


def _esz(t) -> int:
    return int(np.dtype(t.dtype).itemsize) if t.dtype != np.bool_ else 1


def stats_of(t, idxs: tuple) -> Stats:
    """Statistics of an input tensor accessed as t[idxs]."""
    dims = dict(zip(idxs, t.shape))
    esz = _esz(t)
    if not t.is_sparse():
        n = float(np.prod(t.shape))
        return Stats(dims, n, True, {i: n / dims[i] for i in idxs}, esz)
    body = t.body if isinstance(t, SwizzleArray) else t
    if body.kind != "csc" or len(idxs) != 2:
        raise FinchGBUnsupported("galley: sparse operands must be matrices")
    per_dim = _body_degrees(body)  # (max stored per row, max stored per column) of the body
    if isinstance(t, SwizzleArray):
        per_dim = per_dim[::-1]
    nnz = float(body.countstored())
    return Stats(dims, nnz, False, {idxs[0]: per_dim[0], idxs[1]: per_dim[1]}, esz)


def _body_degrees(body) -> tuple:
    """(most entries in one row, most entries in one column) of a CSC body."""
    if body.buf is not None:
        b = body.buf
        col = float(np.diff(b.ptr).max(initial=0))
        row = (float(np.bincount(np.asarray(b.idx, dtype=np.int64) - b.base, minlength=b.nrows).max(initial=0))
               if b.nnz else 0.0)
        return (row, col) if b.orient == "csc" else (col, row)
    d = body.dsparse  # resident only: the fiber lengths are exact, the other side uniform
    ptr = d.ptr.cpu().numpy()
    fib = float(np.diff(ptr).max(initial=0))
    other = math.ceil(d.nnz / max(d.nrows if d.orient == "csc" else d.ncols, 1)) * 4.0
    return (other, fib) if d.orient == "csc" else (fib, other)


# ---------------------------------------------------------------- queries


@dataclass
class Factor:
    name: str
    idxs: tuple
    stats: Stats


@dataclass
class Query:
    """sum over `red` of the product of `factors`, indexed by `out`."""

    factors: list
    out: tuple
    red: tuple
    tensors: dict  # factor name -> (tensor, idxs) of the inputs


def query_of(plan: Node) -> Query | None:
    """The sum-product query of a logic plan, or None if it is not one.

    Nested sums of products (chained tensordots) are pulled into one query:
    lazy's tensordot names its reduced indices freshly, so pulling an inner
    sum out of a product captures no index."""
    root = flatten(plan)
    out = root.idxs if isinstance(root, Reorder) else indices_of(root)
    body = root.arg if isinstance(root, Reorder) else root
    red: list = []
    accesses: list = []

    def walk(n) -> bool:
        if isinstance(n, Access):
            accesses.append(n)
            return True
        if isinstance(n, Aggregate):
            if n.op != "+":
                return False
            red.extend(n.idxs)
            return walk(n.arg)
        if isinstance(n, MapJoin):
            return n.op == "*" and all(walk(a) for a in n.args)
        return False

    if not walk(body) or len(accesses) < 1:
        return None
    if len(set(red)) != len(red) or any(i in out for i in red):
        return None
    tensors, factors = {}, []
    for k, a in enumerate(accesses):
        if len(set(a.idxs)) != len(a.idxs):
            return None
        name = f"t{k}"
        tensors[name] = (a.tns, a.idxs)
        factors.append(Factor(name, tuple(a.idxs), stats_of(a.tns, a.idxs)))
    present = {i for f in factors for i in f.idxs}
    if not set(out) <= present:
        return None
    return Query(factors, tuple(out), tuple(red), tensors)


# ---------------------------------------------------------------- steps and costs


@dataclass
class Step:
    kind: str
    eliminated: tuple
    inputs: tuple  # factor names
    out: str
    out_idxs: tuple
    cost: float
    fmt: str  # "sparse", "dense" or "scalar"


@dataclass
class GalleyPlan:
    steps: list
    cost: float
    result: str
    result_idxs: tuple


# Output formats by estimated density (src/Galley/PhysicalOptimizer/
# format-selector.jl:27-65): dense past one half while the dense copy stays
# under 3e10 elements, a sparse list below.  Galley's middle choice between
# 5% and 50% (a bytemap) has no GPU kernel here; such outputs stay sparse lists.
DENSE_FRACTION = 0.5
DENSE_LIMIT = 3e10


def select_output_format(nnz: float, rows: float, cols: float, esz: int) -> str:
    """'dense' or 'sparse' for a rows x cols output of about nnz entries."""
    cells = rows * cols
    if cells > 0 and nnz / cells > DENSE_FRACTION and cells < DENSE_LIMIT:
        return "dense"
    return "sparse"


def _uniform_products(a: Stats, b: Stats, v: str) -> float:
    return a.nnz * b.nnz / max(a.dims[v], 1)


def spgemm_estimate(a: Stats, ai: tuple, b: Stats, bi: tuple, v: str, estimator: str):
    """(products, output entries, output degrees) of C[i,k] = sum_v A[i,v] B[v,k]."""
    i = ai[0] if ai[1] == v else ai[1]
    k = bi[1] if bi[0] == v else bi[0]
    prods = _uniform_products(a, b, v)
    if estimator == "dc":  # degree-constraint bound on the join size
        prods = min(a.nnz * b.deg.get(v, b.nnz), b.nnz * a.deg.get(v, a.nnz))
    cells = float(a.dims[i]) * float(b.dims[k])
    nnz = cells * -math.expm1(-prods / cells) if cells else 0.0
    deg = {i: min(float(b.dims[k]), a.deg.get(i, a.nnz) * b.deg.get(v, b.nnz)),
           k: min(float(a.dims[i]), b.deg.get(k, b.nnz) * a.deg.get(v, a.nnz))}
    return prods, nnz, deg


def _step_options(fs: list, v: str, red_left: set, out: tuple, estimator: str):
    """The ways to eliminate `v` given the factors that hold it: a list of
    (kind, eliminated indices, result idxs, result Stats, cost seconds)."""
    opts = []
    if len(fs) == 1:
        (f,) = fs
        s = f.stats
        if not s.dense and len(f.idxs) == 2:
            other = f.idxs[0] if f.idxs[1] == v else f.idxs[1]
            elim = (v, other) if other in red_left else (v,)
            res = () if len(elim) == 2 else (other,)
            cost = ((4 + s.esz) * s.nnz) / HBM_BPS + LAUNCH_S
            rs = Stats({other: s.dims[other]} if res else {}, float(s.dims[other]) if res else 1.0, True,
                       {other: 1.0} if res else {}, s.esz)
            opts.append(("reduce", elim, res, rs, cost))
        return opts
    if len(fs) != 2:
        return opts
    a, b = fs
    for x, y in ((a, b), (b, a)):
        sx, sy = x.stats, y.stats
        if sx.dense or len(x.idxs) != 2:
            continue
        i = x.idxs[0] if x.idxs[1] == v else x.idxs[1]
        m, n = float(sx.dims[i]), float(sx.dims[v])
        # S[i,v] * x[v] -> y[i]
        if sy.dense and y.idxs == (v,):
            stream = 4 * (m + 1) + (4 + sx.esz) * sx.nnz + sy.esz * m
            g = sx.nnz / SECTOR_GATHERS if n * sy.esz <= L2_BYTES else sx.nnz * 32 / GATHER_HBM_BPS
            cost = max(stream / HBM_BPS, g) + LAUNCH_S
            rs = Stats({i: int(m)}, m, True, {i: 1.0}, sy.esz)
            opts.append(("spmv", (v,), (i,), rs, cost))
        # S[i,v] * D[v,k] -> C[i,k]
        if sy.dense and len(y.idxs) == 2 and v in y.idxs:
            k = y.idxs[0] if y.idxs[1] == v else y.idxs[1]
            if k != i:
                nk = float(sy.dims[k])
                slabs = max(1.0, math.ceil(nk * sy.esz / 128))
                gathered = sx.nnz * nk * sy.esz
                g = gathered / (0.75 * gather_bps(n * min(nk * sy.esz, 128)))
                stream = slabs * (4 + sx.esz) * sx.nnz + sy.esz * m * nk
                cost = g + stream / HBM_BPS + LAUNCH_S * (slabs + 1)
                rs = Stats({i: int(m), k: int(nk)}, m * nk, True, {i: nk, k: m}, sy.esz)
                opts.append(("spmm", (v,), (i, k), rs, cost))
        # S[i,v] * T[v,k] -> C[i,k], sparse or dense by its estimated density
        if not sy.dense and len(y.idxs) == 2 and v in y.idxs:
            k = y.idxs[0] if y.idxs[1] == v else y.idxs[1]
            if k != i:
                prods, nnz, deg = spgemm_estimate(sx, x.idxs, sy, y.idxs, v, estimator)
                esz = max(sx.esz, sy.esz)
                fmt = select_output_format(nnz, m, float(sy.dims[k]), esz)
                if fmt == "dense":
                    cells = m * float(sy.dims[k])
                    cost = prods / SPGEMM_PRODUCTS + esz * cells / HBM_BPS + LAUNCH_S
                    rs = Stats({i: int(m), k: sy.dims[k]}, cells, True,
                               {i: float(sy.dims[k]), k: m}, esz)
                    opts.append(("spgemm_dense", (v,), (i, k), rs, cost))
                else:
                    cost = prods / SPGEMM_PRODUCTS + (12 * nnz + 8 * m) / HBM_BPS + 6 * LAUNCH_S
                    rs = Stats({i: int(m), k: sy.dims[k]}, nnz, False, deg, esz)
                    opts.append(("spgemm", (v,), (i, k), rs, cost))
        # S[i,v] * X[i,v] -> y[i] (or a scalar when i is reduced too)
        if set(y.idxs) == set(x.idxs):
            elim = (v, i) if i in red_left else (v,)
            res = () if len(elim) == 2 else (i,)
            # a dense X is read at S's positions: one 32-byte sector per entry
            other_bytes = 32 * sx.nnz if sy.dense else (4 + sy.esz) * sy.nnz
            cost = ((4 + sx.esz) * sx.nnz + other_bytes) / HBM_BPS + LAUNCH_S
            rs = Stats({i: int(m)} if res else {}, m if res else 1.0, True, {i: 1.0} if res else {}, sx.esz)
            opts.append(("ewise_reduce", elim, res, rs, cost))
    if a.stats.dense and b.stats.dense and a.idxs == (v,) and b.idxs == (v,):
        n = float(a.stats.dims[v])
        opts.append(("dot", (v,), (), Stats({}, 1.0, True, {}, a.stats.esz),
                     2 * a.stats.esz * n / HBM_BPS + LAUNCH_S))
    return opts


def _finish(factors: list, out: tuple):
    """Pointwise products of what is left after every reduction: a list of
    (kind, inputs, result idxs, Stats, cost) steps, or None if unsupported."""
    steps = []
    fs = list(factors)
    while len(fs) > 1:
        a, b = fs[0], fs[1]
        if a.stats.dense or b.stats.dense or set(a.idxs) != set(b.idxs) or len(a.idxs) != 2:
            return None
        p = min(a.stats.nnz, b.stats.nnz) * max(a.stats.density, b.stats.density)
        s = Stats(dict(a.stats.dims), p, False,
                  {i: min(a.stats.deg.get(i, a.stats.nnz), b.stats.deg.get(i, b.stats.nnz)) for i in a.idxs},
                  max(a.stats.esz, b.stats.esz))
        cost = 2 * 12 * (a.stats.nnz + b.stats.nnz) / HBM_BPS + 2 * LAUNCH_S
        steps.append(("ewise", (a.name, b.name), a.idxs, s, cost))
        fs = [Factor(f"p{len(steps)}", a.idxs, s)] + fs[2:]
    if fs and set(fs[0].idxs) != set(out):
        return None
    return steps


def optimize(q: Query, estimator: str = "dc", exhaustive_limit: int = 5) -> GalleyPlan:
    """The cheapest elimination order (exhaustive for up to
    `exhaustive_limit` reduced indices, greedy beyond) and its steps."""
    best: list = [math.inf, None]

    def search(factors: list, red: set, steps: list, cost: float, counter: list, greedy: bool):
        if cost >= best[0]:
            return
        if not red:
            fin = _finish(factors, q.out)
            if fin is None:
                return
            all_steps = list(steps)
            cur = list(factors)
            total = cost
            for kind, names, idxs, s, c in fin:
                name = f"w{counter[0]}"
                counter[0] += 1
                all_steps.append(Step(kind, (), names, name, idxs, c, "sparse"))
                cur = [Factor(name, idxs, s)] + [f for f in cur if f.name not in names]
                total += c
            if total < best[0]:
                result = cur[0] if cur else None
                best[0], best[1] = total, (all_steps, result)
            return
        choices = []
        for v in sorted(red):
            fs = [f for f in factors if v in f.idxs]
            for kind, elim, res, s, c in _step_options(fs, v, red, q.out, estimator):
                choices.append((c, v, fs, kind, elim, res, s))
        if not choices:
            return
        choices.sort(key=lambda t: t[0])
        if greedy:
            choices = choices[:1]
        for c, v, fs, kind, elim, res, s in choices:
            name = f"w{counter[0]}"
            counter[0] += 1
            fmt = "scalar" if not res else ("dense" if s.dense else "sparse")
            st = Step(kind, elim, tuple(f.name for f in fs), name, res, c, fmt)
            rest = [f for f in factors if f not in fs]
            search(rest + [Factor(name, res, s)], red - set(elim), steps + [st], cost + c, counter, greedy)

    search(list(q.factors), set(q.red), [], 0.0, [0], len(q.red) > exhaustive_limit)
    if best[1] is None:
        raise FinchGBUnsupported("galley: no order of this query maps onto the GB300 kernels")
    steps, result = best[1]
    name = result.name if result is not None else q.factors[0].name
    idxs = result.idxs if result is not None else q.factors[0].idxs
    return GalleyPlan(steps, best[0], name, idxs)


# ---------------------------------------------------------------- execution


def _run_step(st: Step, env: dict):
    from . import device as dev
    from .scheduler import dense_operand, sparse_operand
    from .tensors import dense_from_device, sparse_from_device

    ins = [env[n] for n in st.inputs]
    if st.kind == "reduce":
        (t, idxs), = ins
        v = st.eliminated[0]
        other = idxs[0] if idxs[1] == v else idxs[1]
        A = sparse_operand(t, idxs, (other, v))
        y = dev.ewise_reduce(0 if len(st.eliminated) == 2 else 2, A)
        return (Scalar(y.reshape(())), ()) if len(st.eliminated) == 2 else (dense_from_device(y), (other,))
    if st.kind == "dot":
        (x, xi), (y, yi) = ins
        return Scalar(dev.dot(dense_operand(x, xi, xi), dense_operand(y, yi, yi))), ()
    # binary kinds: put the sparse operand first
    (a, ai), (b, bi) = ins
    if _is_dense(a) and not isinstance(a, Scalar):
        (a, ai), (b, bi) = (b, bi), (a, ai)
    v = st.eliminated[0] if st.eliminated else None
    if st.kind == "spmv":
        i = ai[0] if ai[1] == v else ai[1]
        A = sparse_operand(a, ai, (i, v))
        y = dev.spmv(A, dense_operand(b, bi, (v,)))
        return dense_from_device(y), (i,)
    if st.kind == "spmm":
        i = ai[0] if ai[1] == v else ai[1]
        k = bi[0] if bi[1] == v else bi[1]
        A = sparse_operand(a, ai, (i, v))
        if A.orient == "csc":
            A = _csr_copy(a, A)
        C = dev.spmm(A, dense_operand(b, bi, (v, k)))
        return dense_from_device(C), (i, k)
    if st.kind == "spgemm":
        i = ai[0] if ai[1] == v else ai[1]
        k = bi[0] if bi[1] == v else bi[1]
        A = sparse_operand(a, ai, (i, v))
        B = sparse_operand(b, bi, (v, k))
        if B.orient != A.orient:
            B = _other_orientation(b, B)
        return sparse_from_device(dev.spgemm(A, B)), (i, k)
    if st.kind == "spgemm_dense":
        i = ai[0] if ai[1] == v else ai[1]
        k = bi[0] if bi[1] == v else bi[1]
        A = sparse_operand(a, ai, (i, v))
        B = sparse_operand(b, bi, (v, k))
        if A.orient != "csr":
            A = _other_orientation(a, A)
        if B.orient != "csr":
            B = _other_orientation(b, B)
        return dense_from_device(dev.spgemm_dense(A, B)), (i, k)
    if st.kind == "ewise_reduce":
        i = ai[0] if ai[1] == v else ai[1]
        A = sparse_operand(a, ai, (i, v))
        Bs = Bd = None
        if _is_sparse(b):
            Bs = sparse_operand(b, bi, (i, v))
            if Bs.orient != A.orient:
                Bs = _other_orientation(b, Bs)
        else:
            Bd = dense_operand(b, bi, (i, v))
        scalar = len(st.eliminated) == 2
        y = dev.ewise_reduce(0 if scalar else 2, A, B=Bs, B_dense=Bd)
        return (Scalar(y.reshape(())), ()) if scalar else (dense_from_device(y), (i,))
    if st.kind == "ewise":
        A = sparse_operand(a, ai, ai)
        B = sparse_operand(b, bi, ai)
        if B.orient != A.orient:
            B = _other_orientation(b, B)
        return sparse_from_device(dev.ewise(L.EW_MUL, A, B)), ai
    raise FinchGBUnsupported(f"galley: step {st.kind}")


def execute(p: GalleyPlan, q: Query):
    env = dict(q.tensors)
    for st in p.steps:
        env[st.out] = _run_step(st, env)
    t, idxs = env[p.result]
    if isinstance(t, Scalar) or tuple(idxs) == tuple(q.out):
        return t
    if len(idxs) == 2 and tuple(idxs) == tuple(reversed(q.out)):
        return swizzle(t, 2, 1)
    raise FinchGBUnsupported(f"galley: result order {idxs} vs {q.out}")


class GalleyScheduler(GB300Scheduler):
    """Callable scheduler: plans sum-product queries by estimated cost, and
    hands every other plan to the single-kernel matcher.  `last_plan` holds
    the chosen steps and their estimated seconds."""

    OPTIONS = ("finch_order", "verbose", "estimator", "algebra")

    def __init__(self, estimator: str = "dc", verbose: bool = False, **kw):
        super().__init__(verbose=verbose, **kw)
        if estimator not in ("dc", "uniform"):
            raise ValueError("estimator must be 'dc' or 'uniform'")
        self.estimator = estimator
        self.last_plan: GalleyPlan | None = None

    def __call__(self, plan: Node, out=None, accumulate=False):
        q = query_of(plan) if out is None else None
        if q is None or (len(q.factors) == 1 and not q.red):
            return super().__call__(plan, out, accumulate)
        p = optimize(q, self.estimator)
        self.last_plan = p
        self.last_kernel = "galley:" + ",".join(s.kind for s in p.steps)
        if self.verbose:
            for s in p.steps:
                print(f"[galley] {s.out}{list(s.out_idxs)} = {s.kind}{s.inputs} over {s.eliminated} "
                      f"({s.fmt}, {s.cost * 1e6:.1f} us)")
        if not p.steps:
            return super().__call__(plan, out, accumulate)
        return execute(p, q)


def galley_scheduler(verbose: bool = False, estimator: str = "dc") -> GalleyScheduler:
    """galley_scheduler() (src/Galley/FinchCompat/executor.jl:173-181)."""
    return GalleyScheduler(estimator=estimator, verbose=verbose)
