"""Algebras: the properties of operators the GB300 matcher relies on.

Finch decides which regions of a sparse tensor a loop may skip by asking its
algebra whether the fill value annihilates the operator applied to it
(src/symbolic/symbolic.jl:89-166).  Every kernel here visits stored entries
only, so a program maps onto one only when that skip is exact: the fill of
the sparse operand must annihilate the product operator (0 for `*`, +-Inf
for `+`, false for `&`).  `DefaultAlgebra` restates the reference's
definitions; a program whose fill the default algebra does not cover (an
Int32 min-plus graph with `typemax(Int32)` for "no edge", say) declares it in
an algebra of its own, as Finch programs do
(docs/src/docs/user-defined_functions.md, "Separate Algebras"):

    class GraphAlgebra(DefaultAlgebra):
        def isannihilator(self, op, x):
            if op == "+" and x == np.iinfo(np.int32).max:
                return True
            return super().isannihilator(op, x)

    y = einsum("y[i] <<min>>= A[i,j] + x[j]", A=A, x=x, algebra=GraphAlgebra())

Operators are named by their Finch spelling: "+", "*", "min", "max", "|",
"&".  Algebras compare equal by type, as Julia's singleton algebra values do.
"""
from __future__ import annotations

import numpy as np


def _is_missing(x) -> bool:
    return x is None


def _isinf(x) -> bool:
    try:
        return bool(np.isinf(x))
    except TypeError:
        return False


def _iszero(x) -> bool:
    return bool(x == 0)


def _all_ones(x) -> bool:
    """x == ~zero(x): true, or an integer with every bit set."""
    if isinstance(x, (bool, np.bool_)):
        return bool(x)
    if isinstance(x, (int, np.integer)):
        return int(x) == -1
    return False


class AbstractAlgebra:
    """The algebra protocol: override the properties to declare them."""

    def isannihilator(self, op: str, x) -> bool:
        """True when op(a..., x, b...) == x."""
        return False

    def isidentity(self, op: str, x) -> bool:
        """True when op(a..., x, b...) == op(a..., b...)."""
        return False

    def isassociative(self, op: str) -> bool:
        return False

    def iscommutative(self, op: str) -> bool:
        return False

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self).__qualname__)

    def __repr__(self):
        return f"{type(self).__name__}()"


class DefaultAlgebra(AbstractAlgebra):
    """src/symbolic/symbolic.jl's definitions for the built-in operators."""

    def isannihilator(self, op, x):
        if op == "+":
            return _is_missing(x) or _isinf(x)
        if op == "*":
            return _is_missing(x) or _iszero(x)
        if op == "min":
            return _is_missing(x) or (_isinf(x) and x < 0)
        if op == "max":
            return _is_missing(x) or (_isinf(x) and x > 0)
        if op == "|":
            return not _is_missing(x) and _all_ones(x)
        if op == "&":
            return not _is_missing(x) and _iszero(x)
        return False

    def isidentity(self, op, x):
        if _is_missing(x):
            return False
        if op == "+":
            return _iszero(x)
        if op == "*":
            return bool(x == 1)
        if op == "min":
            return _isinf(x) and x > 0
        if op == "max":
            return _isinf(x) and x < 0
        if op == "|":
            return _iszero(x)
        if op == "&":
            return _all_ones(x)
        return False

    def isassociative(self, op):
        return op in ("+", "*", "min", "max", "|", "&")

    def iscommutative(self, op):
        return op in ("+", "*", "min", "max", "|", "&")
