"""The cost-based planner (finchgb.galley) on the host: which elimination
order and which kernels it chooses for sum-product queries, its sparsity
estimates, and the queries it rejects.  No kernel runs here."""
import numpy as np
import pytest

from finchgb import Dense, Element, SparseList, Tensor, lazy
from finchgb.galley import Stats, galley_scheduler, optimize, query_of, spgemm_estimate
from finchgb.logic import Reorder
from finchgb.scheduler import FinchGBUnsupported
from finchgb.workloads import SparseBuffers, fsprand


def sparse(m, n, nnz, seed):
    rng = np.random.default_rng(seed)
    return Tensor.from_buffers(Dense(SparseList(Element(0.0))), fsprand(rng, m, n, 0.0, nnz=nnz))


def dense(*shape):
    fmt = Dense(Element(0.0)) if len(shape) == 1 else Dense(Dense(Element(0.0)))
    return Tensor(fmt, np.ones(shape))


def plan_of(expr):
    q = query_of(Reorder(expr.node, expr.idxs))
    assert q is not None
    return q, optimize(q)


def test_matrix_chain_times_vector_runs_right_to_left():
    """A * B * x (Julia's left-to-right product) is planned as A * (B * x):
    two SpMVs instead of an SpGEMM and an SpMV."""
    A, B, x = sparse(2000, 2000, 40000, 1), sparse(2000, 2000, 40000, 2), dense(2000)
    q, p = plan_of(lazy(A) @ lazy(B) @ lazy(x))
    assert [s.kind for s in p.steps] == ["spmv", "spmv"]
    first = p.steps[0]
    assert set(first.inputs) == {"t1", "t2"}  # B and x
    assert p.steps[-1].fmt == "dense"


def test_sparse_chain_order_follows_the_sparsest_product():
    """(A B) C when A is far sparser than B and C: the first SpGEMM joins A
    and B (few products), not B and C."""
    A = sparse(3000, 3000, 60, 3)
    B = sparse(3000, 3000, 90000, 4)
    C = sparse(3000, 3000, 90000, 5)
    q, p = plan_of(lazy(A) @ lazy(B) @ lazy(C))
    assert [s.kind for s in p.steps] == ["spgemm", "spgemm"]
    assert set(p.steps[0].inputs) == {"t0", "t1"}
    assert p.steps[0].fmt == "sparse"
    # the other association is costed higher
    A2 = sparse(3000, 3000, 90000, 6)
    C2 = sparse(3000, 3000, 60, 7)
    q2, p2 = plan_of(lazy(A2) @ lazy(B) @ lazy(C2))
    assert set(p2.steps[0].inputs) == {"t1", "t2"}


def test_bilinear_form_is_spmv_then_dot():
    A, x, y = sparse(500, 400, 3000, 8), dense(500), dense(400)
    q, p = plan_of((lazy(x) * (lazy(A) @ lazy(y))).sum())
    assert [s.kind for s in p.steps] == ["spmv", "dot"]
    assert p.steps[-1].fmt == "scalar"


def test_triangle_sum_is_spgemm_then_masked_reduce():
    A = sparse(800, 800, 6000, 9)
    a = lazy(A)
    q, p = plan_of((a * (a @ a)).sum())
    assert [s.kind for s in p.steps] == ["spgemm", "ewise_reduce"]
    assert p.steps[-1].fmt == "scalar"
    assert len(q.red) == 3


def test_plain_spmm_and_dense_contraction():
    A, D = sparse(600, 500, 4000, 10), dense(500, 32)
    q, p = plan_of(lazy(A) @ lazy(D))
    assert [s.kind for s in p.steps] == ["spmm"]
    with pytest.raises(FinchGBUnsupported):
        plan_of(lazy(dense(40, 30)) @ lazy(dense(30, 20)))


def test_degree_constraints_bound_skewed_products():
    """One full column of A against one full row of B: the uniform estimate
    sees n products, the degree-constraint bound the true n^2."""
    n = 1000
    a = Stats({"i": n, "j": n}, n, False, {"i": 1.0, "j": float(n)})
    b = Stats({"j": n, "k": n}, n, False, {"j": float(n), "k": 1.0})
    p_uni, _, _ = spgemm_estimate(a, ("i", "j"), b, ("j", "k"), "j", "uniform")
    p_dc, nnz_dc, _ = spgemm_estimate(a, ("i", "j"), b, ("j", "k"), "j", "dc")
    assert p_uni == pytest.approx(n)
    assert p_dc == pytest.approx(n * n)
    assert nnz_dc == pytest.approx(n * n * -np.expm1(-1.0))


def test_stats_of_swizzled_and_dense_operands():
    from finchgb import swizzle

    buf = SparseBuffers(3, 4, np.array([1, 3, 3, 4, 5]), np.array([1, 3, 2, 2]), np.ones(4), "csc")
    t = Tensor.from_buffers(Dense(SparseList(Element(0.0))), buf)
    lt = lazy(t)
    q = query_of(Reorder(lt.node, lt.idxs))
    s = q.factors[0].stats
    i, j = q.factors[0].idxs
    assert s.nnz == 4 and s.deg[i] == 2 and s.deg[j] == 2  # row 2 holds two; column 1 holds two
    st = swizzle(t, 2, 1)
    ls = lazy(st)
    qs = query_of(Reorder(ls.node, ls.idxs))
    ss = qs.factors[0].stats
    a, b = qs.factors[0].idxs
    assert ss.dims[a] == 4 and ss.dims[b] == 3


def test_non_sum_product_plans_go_to_the_kernel_matcher():
    A, x = sparse(50, 40, 200, 11), dense(40)
    from finchgb.logic import minimum

    lx = lazy(x)
    mn = minimum(lx, lx)
    assert query_of(Reorder(mn.node, mn.idxs)) is None
    g = galley_scheduler()
    assert g.estimator == "dc"
    with pytest.raises(ValueError):
        galley_scheduler(estimator="exact")


@pytest.mark.parametrize("nnz,fmt,kind", [(2000, "sparse", "spgemm"), (60000, "dense", "spgemm_dense")])
def test_spgemm_output_format_follows_estimated_density(nnz, fmt, kind):
    """format-selector.jl:27-65: a product whose estimated density passes
    one half is built dense, a sparse one as a sparse list."""
    A, B = sparse(300, 300, nnz, 11), sparse(300, 300, nnz, 12)
    q, p = plan_of(lazy(A) @ lazy(B))
    assert [s.kind for s in p.steps] == [kind]
    assert p.steps[0].fmt == fmt


def test_select_output_format_thresholds():
    from finchgb.galley import select_output_format

    assert select_output_format(0.6 * 100 * 100, 100, 100, 8) == "dense"
    assert select_output_format(0.4 * 100 * 100, 100, 100, 8) == "sparse"
    assert select_output_format(0.9 * 4e5 * 1e5, 4e5, 1e5, 8) == "sparse"  # a dense copy above 3e10 cells
