"""Finch's front ends -- @einsum, lazy/compute and @finch programs -- as a
small logic IR that the GB300 scheduler matches onto kernels.

The node kinds follow FinchLogic (src/FinchLogic/nodes.jl:5-19):
  Access    relabel(table(tns), idxs...)   a tensor read with index names
  Literal   immediate(val)
  MapJoin   mapjoin(op, args...)           pointwise op over the union of
                                           the args' indices
  Aggregate aggregate(op, init, arg, idxs) reduction over idxs
  Reorder   reorder(arg, idxs...)          the output's index order

`einsum` builds reorder(aggregate(op, init, mapjoin(...), reduced), outs)
the way src/interface/einsum.jl:58-78 does; `lazy`/`compute` build the same
nodes from broadcast, tensordot and sum (src/interface/lazy.jl:207-404);
`finch` parses the loop programs of `@finch` (src/execute.jl:178-218).
"""
from __future__ import annotations

import ast
import functools
import itertools
import re
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------- IR


class Node:
    pass


@dataclass(eq=False)
class Access(Node):
    tns: object
    idxs: tuple

    def __repr__(self):
        return f"{getattr(self.tns, 'name', 'T')}[{','.join(self.idxs)}]"


@dataclass(eq=False)
class Literal(Node):
    value: object

    def __repr__(self):
        return repr(self.value)


@dataclass(eq=False)
class MapJoin(Node):
    op: str
    args: list

    def __repr__(self):
        return f"mapjoin({self.op}, {', '.join(map(repr, self.args))})"


@dataclass(eq=False)
class Aggregate(Node):
    op: str
    init: object
    arg: Node
    idxs: tuple

    def __repr__(self):
        return f"aggregate({self.op}, {self.init}, {self.arg!r}, {self.idxs})"


@dataclass(eq=False)
class Reorder(Node):
    arg: Node
    idxs: tuple

    def __repr__(self):
        return f"reorder({self.arg!r}, {self.idxs})"


ASSOCIATIVE = {"+", "*", "min", "max", "|", "&"}
# identities of the reduction operators (src/symbolic/symbolic.jl:95-104)
IDENTITY = {"+": 0, "*": 1, "min": float("inf"), "max": float("-inf"), "|": False, "&": True}


def indices_of(n: Node) -> tuple:
    """Free indices of a node, in first-appearance order."""
    if isinstance(n, Access):
        return n.idxs
    if isinstance(n, Literal):
        return ()
    if isinstance(n, MapJoin):
        out = []
        for a in n.args:
            for i in indices_of(a):
                if i not in out:
                    out.append(i)
        return tuple(out)
    if isinstance(n, Aggregate):
        return tuple(i for i in indices_of(n.arg) if i not in n.idxs)
    if isinstance(n, Reorder):
        return n.idxs
    raise TypeError(n)


def flatten(n: Node) -> Node:
    """Flattens nested MapJoins of the same associative operator."""
    if isinstance(n, MapJoin):
        args = []
        for a in map(flatten, n.args):
            if isinstance(a, MapJoin) and a.op == n.op and n.op in ASSOCIATIVE:
                args.extend(a.args)
            else:
                args.append(a)
        return MapJoin(n.op, args)
    if isinstance(n, Aggregate):
        return Aggregate(n.op, n.init, flatten(n.arg), n.idxs)
    if isinstance(n, Reorder):
        return Reorder(flatten(n.arg), n.idxs)
    return n


# ---------------------------------------------------------------- einsum

_OPS = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.BitOr: "|", ast.BitAnd: "&",
        ast.Div: "/"}
_LHS = re.compile(r"^\s*(\w+)\s*\[([\w\s,]*)\]\s*(<<\s*([\w+*|&]+(?:\([^)]*\))?)\s*>>=|\+=|\*=|\|=|&=|=)"
                  r"\s*(.+)$", re.S)
_REDUCERS = {"+": "+", "*": "*", "|": "|", "&": "&", "min": "min", "max": "max", "or": "|",
             "and": "&"}


@functools.lru_cache(maxsize=512)
def _rhs_tree(src: str):
    """The Python syntax tree of a right-hand side, parsed once per text (the
    names are bound to tensors per call)."""
    src = re.sub(r"(\w+)\[\s*\]", r"\1[()]", src)  # s[] -> s[()]
    return ast.parse(src.strip(), mode="eval").body


def _parse_rhs(src: str, tensors: dict) -> Node:
    tree = _rhs_tree(src)

    def conv(e):
        if isinstance(e, ast.BinOp) and type(e.op) in _OPS:
            return MapJoin(_OPS[type(e.op)], [conv(e.left), conv(e.right)])
        if isinstance(e, ast.UnaryOp) and isinstance(e.op, ast.USub):
            return MapJoin("neg", [conv(e.operand)])
        if isinstance(e, ast.Call) and isinstance(e.func, ast.Name):
            return MapJoin(e.func.id, [conv(a) for a in e.args])
        if isinstance(e, ast.Subscript):
            name = e.value.id
            sl = e.slice
            if isinstance(sl, ast.Tuple):
                idxs = tuple(x.id for x in sl.elts)
            elif isinstance(sl, ast.Name):
                idxs = (sl.id,)
            else:
                idxs = ()
            if name not in tensors:
                raise KeyError(f"einsum: tensor {name!r} not given")
            t = tensors[name]
            return Access(t, idxs)
        if isinstance(e, ast.Constant):
            return Literal(e.value)
        if isinstance(e, ast.Name) and e.id in tensors:
            return Literal(tensors[e.id])
        raise SyntaxError(f"einsum: unsupported expression {ast.dump(e)}")

    return conv(tree)


@dataclass
class EinsumPlan:
    """A parsed `@einsum` statement."""

    out_name: str
    out_idxs: tuple
    op: str | None  # reduction operator, None for plain `=`
    init: object
    rhs: Node

    def logic(self) -> Node:
        rhs = flatten(self.rhs)
        red = tuple(i for i in indices_of(rhs) if i not in self.out_idxs)
        body = rhs
        if self.op is not None:
            body = Aggregate(self.op, self.init, rhs, red)
        elif red:
            raise ValueError("einsum: `=` with indices that are not on the left-hand side")
        return Reorder(body, self.out_idxs)


def parse_einsum(stmt: str, tensors: dict, init=None) -> EinsumPlan:
    """Parses `out[i,...] <op>= expr` (src/interface/einsum.jl:136-201)."""
    m = _LHS.match(stmt)
    if not m:
        raise SyntaxError(f"einsum: cannot parse {stmt!r}")
    name, idxs, assign, custom, rhs = m.groups()
    out_idxs = tuple(s.strip() for s in idxs.split(",") if s.strip())
    if custom and (custom == "overwrite" or custom.startswith("initwrite(")):
        # overwrite(a, b) = b and initwrite(z)(a, b) = b (src/util/special_
        # functions.jl): assignments, not reductions -- the `=` form, with
        # initwrite's z as the output's initial value
        op = None
        if custom.startswith("initwrite(") and init is None:
            init = ast.literal_eval(custom[len("initwrite("):-1].strip() or "0")
    elif custom:
        op = _REDUCERS[custom]
    elif assign == "=":
        op = None
    else:
        op = _REDUCERS[assign[0]]
    if op is not None and init is None:
        init = IDENTITY[op]
    return EinsumPlan(name, out_idxs, op, init, _parse_rhs(rhs, tensors))


# ---------------------------------------------------------------- lazy

_counter = itertools.count()


def _fresh(n: int) -> tuple:
    k = next(_counter)
    return tuple(f"_i{k}_{d}" for d in range(n))


class LazyTensor:
    """A deferred tensor expression (src/interface/lazy.jl)."""

    def __init__(self, node: Node, idxs: tuple, shape: tuple):
        self.node, self.idxs, self.shape = node, tuple(idxs), tuple(shape)

    @property
    def ndim(self):
        return len(self.shape)

    def _rename(self, new: tuple) -> Node:
        mapping = dict(zip(self.idxs, new))
        return _rename(self.node, mapping)

    def _bin(self, other, op):
        if not isinstance(other, LazyTensor):
            return LazyTensor(MapJoin(op, [self.node, Literal(other)]), self.idxs, self.shape)
        if other.shape != self.shape:
            raise ValueError(f"broadcast of shapes {self.shape} and {other.shape}")
        return LazyTensor(MapJoin(op, [self.node, other._rename(self.idxs)]), self.idxs,
                          self.shape)

    def __mul__(self, o):  # Julia's `.*`
        return self._bin(o, "*")

    __rmul__ = __mul__

    def __add__(self, o):
        return self._bin(o, "+")

    __radd__ = __add__

    def __sub__(self, o):
        return self._bin(o, "-")

    def __and__(self, o):
        return self._bin(o, "&")

    def __or__(self, o):
        return self._bin(o, "|")

    def __matmul__(self, o):  # Julia's `*` on matrices: tensordot(a, b, (2, 1))
        return tensordot(self, o, ((self.ndim,), (1,)))

    @property
    def T(self):
        return permutedims(self, (2, 1))

    def sum(self, dims=None):
        return reduce("+", self, dims)

    def __repr__(self):
        return f"LazyTensor({self.node!r}, shape={self.shape})"


def _rename(n: Node, m: dict) -> Node:
    if isinstance(n, Access):
        return Access(n.tns, tuple(m.get(i, i) for i in n.idxs))
    if isinstance(n, MapJoin):
        return MapJoin(n.op, [_rename(a, m) for a in n.args])
    if isinstance(n, Aggregate):
        return Aggregate(n.op, n.init, _rename(n.arg, m), tuple(m.get(i, i) for i in n.idxs))
    if isinstance(n, Reorder):
        return Reorder(_rename(n.arg, m), tuple(m.get(i, i) for i in n.idxs))
    return n


def lazy(t) -> LazyTensor:
    """lazy(tns) (src/interface/lazy.jl:640)."""
    if isinstance(t, LazyTensor):
        return t
    idxs = _fresh(len(t.shape))
    return LazyTensor(Access(t, idxs), idxs, t.shape)


def tensordot(a: LazyTensor, b: LazyTensor, axes) -> LazyTensor:
    """tensordot(a, b, (ia, ib)) with 1-based axes (src/interface/lazy.jl:215-257)."""
    ia, ib = axes
    ia = (ia,) if isinstance(ia, int) else tuple(ia)
    ib = (ib,) if isinstance(ib, int) else tuple(ib)
    shared = _fresh(len(ia))
    ai = list(_fresh(a.ndim))
    bi = list(_fresh(b.ndim))
    for s, x, y in zip(shared, ia, ib):
        if a.shape[x - 1] != b.shape[y - 1]:
            raise ValueError("tensordot: contracted dimensions differ")
        ai[x - 1] = s
        bi[y - 1] = s
    body = MapJoin("*", [a._rename(tuple(ai)), b._rename(tuple(bi))])
    out = [i for i in ai if i not in shared] + [i for i in bi if i not in shared]
    shape = [a.shape[d] for d in range(a.ndim) if d + 1 not in ia] + \
            [b.shape[d] for d in range(b.ndim) if d + 1 not in ib]
    return LazyTensor(Aggregate("+", 0, body, shared), tuple(out), tuple(shape))


def reduce(op: str, a: LazyTensor, dims=None) -> LazyTensor:
    """reduce(op, a; dims) / sum(a; dims) with 1-based dims."""
    if dims is None:
        dims = tuple(range(1, a.ndim + 1))
    dims = (dims,) if isinstance(dims, int) else tuple(dims)
    red = tuple(a.idxs[d - 1] for d in dims)
    keep = tuple(i for i in a.idxs if i not in red)
    shape = tuple(s for d, s in enumerate(a.shape) if d + 1 not in dims)
    return LazyTensor(Aggregate(op, IDENTITY[op], a.node, red), keep, shape)


def permutedims(a: LazyTensor, perm) -> LazyTensor:
    return LazyTensor(a.node, tuple(a.idxs[p - 1] for p in perm),
                      tuple(a.shape[p - 1] for p in perm))


def broadcast(op: str, *args) -> LazyTensor:
    """broadcast(op, args...) over same-shape lazy tensors."""
    first = next(a for a in args if isinstance(a, LazyTensor))
    nodes = [a._rename(first.idxs) if isinstance(a, LazyTensor) else Literal(a) for a in args]
    return LazyTensor(MapJoin(op, nodes), first.idxs, first.shape)


def minimum(a, b):
    return broadcast("min", a, b)


def maximum(a, b):
    return broadcast("max", a, b)


# ---------------------------------------------------------------- @finch programs

_LOOP = re.compile(r"for\s+(\w+)\s*=\s*_\s*")


@dataclass
class FinchProgram:
    """A parsed `@finch` loop program: initialisation, loop order, body."""

    init: dict = field(default_factory=dict)  # tensor name -> init value
    loops: tuple = ()
    stmt: str = ""


def parse_finch(src: str) -> FinchProgram:
    """Parses programs of the form

        y .= 0
        for j = _, i = _          (or nested `for j=_; for i=_ ... end end`)
            y[i] += A[i, j] * x[j]
        end

    -- the shape of the nests Finch lowers for this backend
    (test/reference64/typical/typical_spmv_csc.txt:18-25)."""
    prog = FinchProgram()
    text = re.sub(r"\b(end|begin)\b", "\n", src.replace(";", "\n"))
    loops = []
    body = []
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line == "end" or line in ("begin",):
            continue
        if line.startswith("for "):
            for part in line[4:].split(","):
                m = re.match(r"\s*(\w+)\s*=\s*_\s*$", part)
                if not m:
                    raise SyntaxError(f"@finch: loop {line!r} must range over `_`")
                loops.append(m.group(1))
            continue
        m = re.match(r"^(\w+)\s*\.=\s*(.+)$", line)
        if m:
            prog.init[m.group(1)] = ast.literal_eval(m.group(2).replace("Inf", "1e999").replace("true", "True").replace("false", "False"))
            continue
        body.append(line)
    if len(body) != 1:
        raise SyntaxError("@finch: the GB300 backend matches single-assignment loop bodies")
    prog.loops = tuple(loops)
    prog.stmt = body[0]
    return prog
