"""PageRank (docs/examples/pagerank.jl) on the host: the example's five
@finch programs parse into the plans the matchers expect, the masked scale
matcher binds the transition-matrix program and refuses altered ones, and
the oracle's restatement equals an independent power iteration -- and,
where a vertex has no out-edges, gives the NaN that Finch's nest writes
(0 / 0 in the fill region of `/`, which has no annihilator)."""
import numpy as np
import pytest

import oracle
from finchgb import examples, notation, programs
from finchgb.logic import flatten, indices_of, parse_einsum, parse_finch
from finchgb.scheduler import _constant
from finchgb.workloads import fsprand


def test_example_programs_parse_into_plans():
    import finchgb as F

    A = F.Tensor(F.Dense(F.SparseList(F.Pattern())), np.eye(3) > 0)
    x = F.Tensor(F.Dense(F.Element(0.0)), np.ones(3))
    tens = {"edges": A, "scaled_edges": A, "r": x, "rank": x, "out_degree": x, "n": 3, "beta_score": 0.05,
            "damp": 0.85}
    want = {"OUT_DEGREE": ("out_degree", "+", ("j",)), "RANK_INIT": ("r", None, ("j",)),
            "RANK_STEP": ("rank", "+", ("i",)), "RANK_DAMP": ("r", None, ("i",))}
    for name, (out, op, idxs) in want.items():
        prog = parse_finch(getattr(examples, name))
        plan = parse_einsum(prog.stmt, tens)
        assert (plan.out_name, plan.op, plan.out_idxs) == (out, op, idxs) and out in prog.init
    # r[j] = 1.0 / n binds no index on its right: the output gives the extent
    plan = parse_einsum(parse_finch(examples.RANK_INIT).stmt, tens)
    assert set(plan.out_idxs) - set(indices_of(flatten(plan.rhs))) == {"j"}
    assert _constant(plan.logic().arg) == 1.0 / 3
    # the transition matrix is a whole-program match, not a plan
    assert programs.match_masked_scale(notation.parse(examples.SCALE_EDGES)) == {
        "out": "scaled_edges", "init": 0, "edges": "edges", "by": "out_degree", "by_axis": "col", "op": "/",
        "keep": "out_degree", "keep_axis": "row"}


def test_constant_folding_follows_julia_division():
    from finchgb.logic import Literal, MapJoin

    assert _constant(MapJoin("/", [Literal(1), Literal(4)])) == 0.25
    assert _constant(MapJoin("/", [Literal(1.0), Literal(0)])) == float("inf")
    assert np.isnan(_constant(MapJoin("/", [Literal(0), Literal(0)])))
    assert _constant(MapJoin("-", [Literal(1), MapJoin("*", [Literal(2), Literal(3)])])) == -5
    assert _constant(Literal(True)) is None


@pytest.mark.parametrize("src", [
    "s .= 0; for j=_, i=_; s[i, j] = w[j] / A[i, j] end",           # a sparse divisor
    "s .= 1; for j=_, i=_; s[i, j] = A[i, j] / w[j] end",           # a non-zero fill
    "s .= 0; for j=_, i=_; s[i, j] = A[i, j] + w[j] end",           # + is not a scale
    "s .= 0; for j=_, i=_; s[j, i] = A[i, j] / w[j] end",           # transposed output
    "s .= 0; for j=_, i=_; if w[i] > 0; s[i, j] = A[i, j] / w[j] end end",  # another condition
    "s .= 0; for j=_, i=_; s[i, j] = A[i, j] / A[i, j] end",        # no vector
])
def test_masked_scale_refuses_other_programs(src):
    assert programs.match_masked_scale(notation.parse(src)) is None


def test_masked_scale_variants_match():
    m = programs.match_masked_scale(notation.parse("t .= 0.0; for j=_, i=_; t[i, j] = d[i] * G[i, j] end"))
    assert m["op"] == "*" and m["by_axis"] == "row" and m["keep"] is None and m["edges"] == "G"
    m = programs.match_masked_scale(notation.parse(
        "t .= 0; for j=_, i=_; if k[j] != 0; t[i, j] = G[i, j] / d[i] end end"))
    assert m["keep_axis"] == "col" and m["by_axis"] == "row"


def _power_iteration(g, nsteps, damp):
    n = g.ncols
    A = (g.todense() != 0).astype(np.float64)
    d = A.sum(axis=0)
    P = np.where(d[None, :] > 0, A / np.where(d == 0, 1.0, d)[None, :], 0.0)
    P[d == 0, :] = 0.0  # pagerank.jl keeps row i only where out_degree[i] != 0
    r = np.full(n, 1.0 / n)
    for _ in range(nsteps):
        r = (1 - damp) / n + damp * (P @ r)
    return r


@pytest.mark.parametrize("n,p,seed", [(30, 0.5, 1), (300, 0.05, 2)])
def test_oracle_pagerank_equals_power_iteration(n, p, seed):
    g = fsprand(np.random.default_rng(seed), n, n, p)
    assert (np.diff(g.ptr) > 0).all()
    r = oracle.pagerank(n, g.ptr, g.idx, None, 20, 0.85)
    np.testing.assert_allclose(r, _power_iteration(g, 20, 0.85), rtol=1e-13, atol=0)
    assert abs(r.sum() - 1.0) < 1e-12  # no vertex without out-edges: rank is conserved


def test_oracle_pagerank_with_a_vertex_without_out_edges_is_nan():
    """Finch's nest writes 0 / out_degree[j] across the fill region: a zero
    out-degree puts NaN into every kept row."""
    g = fsprand(np.random.default_rng(4), 50, 50, 0.02)
    deg = np.diff(g.ptr)
    assert (deg == 0).any()
    r = oracle.pagerank(50, g.ptr, g.idx, None, 5, 0.85)
    assert np.isnan(r[deg != 0]).all() and np.isfinite(r[deg == 0]).all()
