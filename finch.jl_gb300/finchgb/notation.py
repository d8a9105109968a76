"""A subset of FinchNotation: the loop programs `@finch` takes, parsed into a
small statement tree the scheduler matches onto kernels.

The statement kinds follow FinchNotation's (src/FinchNotation/nodes.jl):
  Loop(idx, body)          for idx = _ ... end      (loop over an index)
  Sieve(cond, body)        if cond ... end          (sieve)
  Define(name, val, body)  let name = val ... end   (define)
  Assign(lhs, op, rhs)     lhs[..] <<op>>= rhs, +=, |=, &=, *=, = (assign;
                           `op` is the reduction, None for plain `=`)
  Init(name, value)        name .= value            (declare + initialise)
  Block(stmts)             a sequence
and expressions Index(tensor name, index expressions), Var(name),
Lit(value), Call(function, args) -- operators included -- and Tup(items)
for tuple literals such as `(d, j)`.  `for j=_, k=_` is two nested loops,
outer first (src/FinchNotation/syntax.jl).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field


# ---------------------------------------------------------------- tree


@dataclass
class Var:
    name: str


@dataclass
class Lit:
    value: object


@dataclass
class Index:
    tns: str
    idxs: tuple


@dataclass
class Call:
    fn: str
    args: tuple


@dataclass
class Tup:
    items: tuple


@dataclass
class Block:
    stmts: list = field(default_factory=list)


@dataclass
class Loop:
    idx: str
    body: object


@dataclass
class Sieve:
    cond: object
    body: object


@dataclass
class Define:
    name: str
    value: object
    body: object


@dataclass
class Assign:
    lhs: Index
    op: object  # None (plain `=`), an operator name, or a Call such as choose(0)
    rhs: object


@dataclass
class Init:
    name: str
    value: object


# ---------------------------------------------------------------- lexer

_TOKEN = re.compile(r"""
    (?P<ws>[ \t\r]+|\#[^\n]*) |
    (?P<nl>[\n;]) |
    (?P<num>\d+\.\d*(?:e[-+]?\d+)?|\d+(?:e[-+]?\d+)?|\.\d+) |
    (?P<op><<|>>=|\.=|\+=|-=|\*=|\|=|&=|==|!=|<=|>=|&&|\|\||[=+\-*/<>!(),\[\]]) |
    (?P<name>[A-Za-z_][A-Za-z_0-9]*)
""", re.VERBOSE)

KEYWORDS = {"for", "in", "end", "if", "let", "begin"}


def _lex(src: str) -> list[tuple[str, str]]:
    out = []
    pos = 0
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise SyntaxError(f"@finch: unexpected {src[pos:pos + 10]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group()))
    out.append(("eof", ""))
    return out


# ---------------------------------------------------------------- parser


class _Parser:
    def __init__(self, src: str):
        self.toks = _lex(src)
        self.i = 0

    def peek(self, k=0):
        return self.toks[self.i + k]

    def take(self, value=None):
        kind, v = self.toks[self.i]
        if value is not None and v != value:
            raise SyntaxError(f"@finch: expected {value!r}, got {v!r}")
        self.i += 1
        return v

    def skip_nl(self):
        while self.peek()[0] == "nl":
            self.i += 1

    # -- statements
    def block(self, stop=("end", "")) -> Block:
        stmts = []
        while True:
            self.skip_nl()
            kind, v = self.peek()
            if kind == "eof" or (kind == "name" and v in stop):
                return Block(stmts)
            stmts.append(self.stmt())

    def stmt(self):
        kind, v = self.peek()
        if kind == "name" and v == "for":
            self.take()
            idxs = [self.loopvar()]
            while self.peek()[1] == ",":
                self.take(",")
                idxs.append(self.loopvar())
            body = self.block()
            self.take("end")
            for idx in reversed(idxs):
                body = Loop(idx, body)
            return body
        if kind == "name" and v == "if":
            self.take()
            cond = self.expr()
            body = self.block()
            self.take("end")
            return Sieve(cond, body)
        if kind == "name" and v == "let":
            self.take()
            name = self.take()
            self.take("=")
            val = self.expr()
            body = self.block()
            self.take("end")
            return Define(name, val, body)
        if kind == "name" and v == "begin":
            self.take()
            body = self.block()
            self.take("end")
            return body
        # name .= value, or an assignment to an access
        if kind == "name" and self.peek(1)[1] == ".=":
            name = self.take()
            self.take(".=")
            return Init(name, self.expr())
        lhs = self.postfix()
        if isinstance(lhs, Var):
            lhs = Index(lhs.name, ())
        if not isinstance(lhs, Index):
            raise SyntaxError("@finch: assignment target must be an access")
        op_tok = self.take()
        if op_tok == "<<":
            op = self.postfix()
            self.take(">>=")
            op = op.name if isinstance(op, Var) else op
        elif op_tok in ("+=", "-=", "*=", "|=", "&="):
            op = op_tok[0]
        elif op_tok == "=":
            op = None
        else:
            raise SyntaxError(f"@finch: unexpected {op_tok!r} after {lhs}")
        return Assign(lhs, op, self.expr())

    def loopvar(self) -> str:
        name = self.take()
        sep = self.take()
        if sep not in ("=", "in"):
            raise SyntaxError(f"@finch: loop over {name} needs `= _`")
        if self.take() != "_":
            raise SyntaxError(f"@finch: loop {name} must range over `_`")
        return name

    # -- expressions, loosest first
    def expr(self):
        return self.binary(0)

    _LEVELS = [("||",), ("&&",), ("<", ">", "<=", ">=", "==", "!="), ("+", "-"), ("*", "/")]

    def binary(self, level):
        if level == len(self._LEVELS):
            return self.unary()
        left = self.binary(level + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self._LEVELS[level]:
            op = self.take()
            right = self.binary(level + 1)
            left = Call(op, (left, right))
        return left

    def unary(self):
        if self.peek()[1] == "!":
            self.take()
            return Call("!", (self.unary(),))
        if self.peek()[1] == "-":
            self.take()
            return Call("-", (self.unary(),))
        return self.postfix()

    def postfix(self):
        node = self.atom()
        while True:
            v = self.peek()[1]
            if v == "(" and isinstance(node, Var):
                node = Call(node.name, self.args("(", ")"))
            elif v == "[" and isinstance(node, Var):
                node = Index(node.name, self.args("[", "]"))
            else:
                return node

    def args(self, open_, close):
        self.take(open_)
        out = []
        if self.peek()[1] != close:
            out.append(self.expr())
            while self.peek()[1] == ",":
                self.take(",")
                out.append(self.expr())
        self.take(close)
        return tuple(out)

    def atom(self):
        kind, v = self.peek()
        if kind == "num":
            self.take()
            return Lit(float(v) if any(c in v for c in ".e") else int(v))
        if kind == "name":
            self.take()
            if v == "true":
                return Lit(True)
            if v == "false":
                return Lit(False)
            if v == "Inf":
                return Lit(float("inf"))
            return Var(v)
        if v == "(":
            items = self.args("(", ")")
            return items[0] if len(items) == 1 else Tup(items)
        raise SyntaxError(f"@finch: unexpected {v!r}")


def parse(src: str) -> Block:
    """Parses an @finch program into a Block of statements."""
    p = _Parser(src)
    b = p.block(stop=("",))
    if p.peek()[0] != "eof":
        raise SyntaxError(f"@finch: unexpected {p.peek()[1]!r}")
    return b


def stmts(node) -> list:
    """The statements of a node as a flat list (a Block's, else [node])."""
    if isinstance(node, Block):
        out = []
        for s in node.stmts:
            out.extend(stmts(s))
        return out
    return [node]


def single(node):
    """The one statement of a body, or None."""
    s = stmts(node)
    return s[0] if len(s) == 1 else None
