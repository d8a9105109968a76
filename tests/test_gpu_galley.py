"""Plans of the cost-based scheduler run on the GPU: every step is a
library kernel, intermediates stay in HBM, and the results equal the dense
products (exactly where the values are small integers, within FP64 rounding
otherwise).  Also the sparse-by-sparse product rule of the kernel matcher."""
import numpy as np
import pytest

from finchgb import Dense, Element, SparseList, Tensor, compute, galley_scheduler, get_scheduler, lazy
from finchgb.scheduler import Scalar
from finchgb.workloads import fsprand

pytestmark = pytest.mark.gpu


def sparse(m, n, nnz, seed, ints=False):
    rng = np.random.default_rng(seed)
    b = fsprand(rng, m, n, 0.0, nnz=nnz)
    if ints:
        b.val = rng.integers(1, 4, size=b.nnz).astype(np.float64)
    t = Tensor.from_buffers(Dense(SparseList(Element(0.0))), b)
    return t, t.todense()


def vec(n, seed):
    x = np.random.default_rng(seed).standard_normal(n)
    return Tensor(Dense(Element(0.0)), x), x


def host(t):
    if isinstance(t, Scalar):
        return float(t)
    return np.asarray(t.todense())


def test_chain_times_vector(gpu_lib):
    (A, Ah), (B, Bh), (x, xh) = sparse(900, 700, 8000, 1), sparse(700, 800, 9000, 2), vec(800, 3)
    g = galley_scheduler()
    y = compute(lazy(A) @ lazy(B) @ lazy(x), ctx=g)
    assert [s.kind for s in g.last_plan.steps] == ["spmv", "spmv"]
    assert g.last_kernel.startswith("galley:")
    np.testing.assert_allclose(host(y), Ah @ (Bh @ xh), rtol=1e-12, atol=1e-12)


def test_sparse_times_sparse_matcher_and_chain(gpu_lib):
    (A, Ah), (B, Bh), (C, Ch) = (sparse(300, 400, 900, 4, ints=True), sparse(400, 350, 5000, 5, ints=True),
                                 sparse(350, 200, 4000, 6, ints=True))
    s = get_scheduler()
    AB = compute(lazy(A) @ lazy(B))
    assert s.last_kernel == "fgb_spgemm"
    assert np.array_equal(host(AB), Ah @ Bh)  # small integers: exact in any order
    g = galley_scheduler()
    ABC = compute(lazy(A) @ lazy(B) @ lazy(C), ctx=g)
    # the second product is estimated past half dense: built as a dense array
    assert [st.kind for st in g.last_plan.steps] == ["spgemm", "spgemm_dense"]
    assert np.array_equal(host(ABC), Ah @ Bh @ Ch)


def test_bilinear_form_and_triangles(gpu_lib):
    (A, Ah), (x, xh), (y, yh) = sparse(500, 400, 3000, 7), vec(500, 8), vec(400, 9)
    g = galley_scheduler()
    s = compute((lazy(x) * (lazy(A) @ lazy(y))).sum(), ctx=g)
    assert isinstance(s, Scalar)
    assert host(s) == pytest.approx(xh @ Ah @ yh, rel=1e-12)
    (T, Th) = sparse(600, 600, 5000, 10, ints=True)
    t = lazy(T)
    tri = compute((t * (t @ t)).sum(), ctx=g)
    assert [st.kind for st in g.last_plan.steps] == ["spgemm", "ewise_reduce"]
    assert host(tri) == float(np.sum(Th * (Th @ Th)))


def test_sparse_times_dense_matrix(gpu_lib):
    (A, Ah), (B, Bh) = sparse(700, 500, 6000, 11), sparse(500, 300, 4000, 12)
    D = np.random.default_rng(13).standard_normal((300, 16))
    Dt = Tensor(Dense(Dense(Element(0.0))), D)
    g = galley_scheduler()
    out = compute(lazy(A) @ lazy(B) @ lazy(Dt), ctx=g)
    kinds = [st.kind for st in g.last_plan.steps]
    assert kinds in (["spmm", "spmm"], ["spgemm", "spmm"])
    np.testing.assert_allclose(host(out), Ah @ Bh @ D, rtol=1e-11, atol=1e-11)


@pytest.mark.parametrize("nnz", [1500, 40000])
def test_spgemm_format_selection_on_device(gpu_lib, nnz):
    """A sparse product runs as a sparse-list SpGEMM, a dense-ish one into a
    dense array; both equal the dense product exactly (small integers), and
    the dense build equals the sparse SpGEMM's values bit for bit."""
    (A, Ah), (B, Bh) = sparse(250, 200, nnz, 21, ints=True), sparse(200, 230, nnz, 22, ints=True)
    g = galley_scheduler()
    C = compute(lazy(A) @ lazy(B), ctx=g)
    kinds = [s.kind for s in g.last_plan.steps]
    assert kinds == (["spgemm_dense"] if nnz == 40000 else ["spgemm"])
    assert np.array_equal(host(C), Ah @ Bh)
    from finchgb import device as dev
    from finchgb.scheduler import sparse_operand

    Ad = sparse_operand(A, ("i", "j"), ("i", "j"))
    Bd = sparse_operand(B, ("i", "j"), ("i", "j"))
    D = dev.spgemm_dense(Ad, Bd).cpu().numpy()
    S = dev.spgemm(Ad, Bd)
    ptr, idx, val = S.to_host()
    Sd = np.zeros_like(D)
    f = np.repeat(np.arange(S.ncols if S.orient == "csc" else S.nrows), np.diff(ptr))
    if S.orient == "csc":
        Sd[idx - 1, f] = val
    else:
        Sd[f, idx - 1] = val
    assert D.tobytes() == Sd.tobytes()
