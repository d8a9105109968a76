"""Algebras on the host: DefaultAlgebra restates the reference's annihilator
and identity table (src/symbolic/symbolic.jl:89-166); the matcher refuses a
sparse operand whose fill its algebra does not let a kernel skip, before any
device work; a user's algebra declares more (an Int32 "no edge" value for
min-plus), and schedulers compare and hash by their algebra like their other
options."""
import numpy as np
import pytest

import finchgb as F
from finchgb.scheduler import GB300Scheduler

D = F.DefaultAlgebra()


@pytest.mark.parametrize("op,x,want", [
    ("+", np.inf, True), ("+", -np.inf, True), ("+", 0.0, False), ("+", np.int32(2**31 - 1), False),
    ("*", 0.0, True), ("*", 0, True), ("*", 1.0, False),
    ("min", -np.inf, True), ("min", np.inf, False), ("max", np.inf, True), ("max", -np.inf, False),
    ("&", False, True), ("&", 0, True), ("&", True, False),
    ("|", True, True), ("|", -1, True), ("|", False, False),
    ("gcd", 1, False),
])
def test_default_annihilators(op, x, want):
    assert D.isannihilator(op, x) is want


@pytest.mark.parametrize("op,x,want", [
    ("+", 0.0, True), ("+", 1.0, False), ("*", 1.0, True), ("*", 0.0, False),
    ("min", np.inf, True), ("min", -np.inf, False), ("max", -np.inf, True),
    ("|", False, True), ("&", True, True), ("&", False, False), ("&", -1, True),
])
def test_default_identities(op, x, want):
    assert D.isidentity(op, x) is want


class GraphAlgebra(F.DefaultAlgebra):
    def isannihilator(self, op, x):
        if op == "+" and x == np.iinfo(np.int32).max:
            return True
        return super().isannihilator(op, x)


def _int_graph():
    A = np.full((6, 6), np.iinfo(np.int32).max, dtype=np.int32)
    A[0, 1], A[1, 2], A[2, 0], A[4, 5] = 3, 4, 1, 7
    fill = np.int32(np.iinfo(np.int32).max)
    return F.Tensor(F.Dense(F.SparseList(F.Element(fill, np.int32))), A)


def test_matcher_refuses_a_fill_the_algebra_cannot_skip():
    A = _int_graph()
    x = F.Tensor(F.Dense(F.Element(np.int32(0), np.int32)), np.zeros(6, np.int32))
    with pytest.raises(F.FinchGBUnsupported, match="annihilator"):
        F.einsum("y[i] <<min>>= A[i,j] + x[j]", A=A, x=x)
    B = F.Tensor(F.Dense(F.SparseList(F.Element(1.0))), np.eye(4) + 1.0)  # fill 1: not skippable for *
    v = F.Tensor(F.Dense(F.Element(0.0)), np.ones(4))
    with pytest.raises(F.FinchGBUnsupported):
        F.einsum("y[i] += B[i,j] * v[j]", B=B, v=v)
    with pytest.raises(F.FinchGBUnsupported):  # reduce(+, B): the fill must be the identity of +
        F.compute(F.lazy(B).sum(dims=1))


def test_declared_annihilator_passes_the_check():
    A = _int_graph()
    GraphAlgebra_ = GraphAlgebra()
    GB300Scheduler(algebra=GraphAlgebra_)._skippable(A, "+")  # no error
    with pytest.raises(F.FinchGBUnsupported):
        GB300Scheduler()._skippable(A, "+")


def test_schedulers_compare_by_algebra():
    a, b = GB300Scheduler(), GB300Scheduler(algebra=F.DefaultAlgebra())
    assert a == b and hash(a) == hash(b)
    c = a.set_options(algebra=GraphAlgebra())
    assert c != a and c.algebra == GraphAlgebra() and c.finch_order == a.finch_order
    assert GraphAlgebra() != F.DefaultAlgebra() and hash(GraphAlgebra()) == hash(GraphAlgebra())


def test_overwrite_and_initwrite_parse_as_assignments():
    """overwrite(a, b) = b and initwrite(z)(a, b) = b (src/util/special_functions.jl)
    are assignments: the `=` form, initwrite's z the initial value; a write
    that would keep the last of a reduced index's values is refused."""
    from finchgb.logic import parse_einsum

    H = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), np.eye(3))
    p = parse_einsum("J[i,j] <<overwrite>>= H[i,j] * H[i,j]", {"H": H})
    assert p.op is None and p.init is None
    p = parse_einsum("J[i,j] <<initwrite(0.0)>>= H[i,j]", {"H": H})
    assert p.op is None and p.init == 0.0
    with pytest.raises(ValueError):
        parse_einsum("y[i] <<overwrite>>= H[i,j]", {"H": H}).logic()
