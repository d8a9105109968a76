"""The Finch-facing API on the GPU: @einsum, lazy/compute and @finch
programs matched onto kernels, checked against the oracle and against
Finch's known answers.  Mirrors test/suites/interface_tests.jl."""
import json
from pathlib import Path

import numpy as np
import pytest

import finchgb as F
import oracle
from finchgb.workloads import csr_from_dense

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "finch_kats.json").read_text())["kats"]


def csc(A, fill=0):
    A = np.asarray(A)
    return F.Tensor(F.Dense(F.SparseList(F.Element(np.asarray(fill, A.dtype)[()], A.dtype))), A)


def vec(x):
    x = np.asarray(x)
    return F.Tensor(F.Dense(F.Element(np.zeros((), x.dtype)[()], x.dtype)), x)


def dense2(B):
    B = np.asarray(B)
    return F.Tensor(F.Dense(F.Dense(F.Element(np.zeros((), B.dtype)[()], B.dtype))), B)


def sprand_int(rng, m, n, p):
    return np.where(rng.random((m, n)) < p, rng.integers(-50, 50, (m, n)), 0).astype(np.int64)


def test_finch_program_spmv_kat(gpu_lib):
    k = KATS["spmv_csc"]
    A = csc(np.array(k["A"]), 0.0)
    x = vec(np.array(k["x"], dtype=np.float64))
    out = F.finch("""
        y .= 0
        for j = _, i = _
            y[i] += A[i, j] * x[j]
        end""", A=A, x=x)
    assert out["y"].todense().tolist() == k["y"]  # bit-exact with Finch's nest


def test_finch_program_accumulates_without_init(gpu_lib):
    A = csc(np.array([[1.0, 2.0], [0.0, 3.0]]), 0.0)
    x = vec(np.array([1.0, 1.0]))
    y = F.transfer(F.gpu(), vec(np.array([10.0, 20.0])))
    out = F.finch("for j=_, i=_; y[i] += A[i, j] * x[j] end", A=A, x=x, y=y)
    assert out["y"].todense().tolist() == [13.0, 23.0]


def test_einsum_spmv_and_transposed(gpu_lib):
    rng = np.random.default_rng(0)
    S = sprand_int(rng, 10, 10, 0.3)
    v = rng.integers(-100, 100, 10).astype(np.int64)
    w = F.einsum("w[i] += S[i,k] * v[k]", S=csc(S), v=vec(v))
    assert w.todense().tolist() == (S @ v).tolist()
    x = F.einsum("x[k] += T[j,k] * u[j]", T=csc(S), u=vec(v))
    assert x.todense().tolist() == (S.T @ v).tolist()


def test_einsum_matmul_kat(gpu_lib):
    k = KATS["einsum_matmul"]
    A = csc(np.array(k["A"], dtype=np.int64).astype(np.float64), 0.0)
    B = dense2(np.array(k["B"], dtype=np.float64))
    C = F.einsum("C[i,j] += A[i,k] * B[k,j]", A=A, B=B)
    assert C.todense().tolist() == k["C"]
    assert int(np.abs(C.todense()).sum()) == k["s_abs"]


def test_einsum_elementwise_sparse(gpu_lib):
    rng = np.random.default_rng(1)
    H = sprand_int(rng, 5, 5, 0.6).astype(np.float64)
    I = sprand_int(rng, 5, 5, 0.6).astype(np.float64)
    J = F.einsum("J[i,j] = H[i,j] * I[i,j]", H=csc(H), I=csc(I))
    assert J == H * I
    assert F.einsum("J[i,j] <<overwrite>>= H[i,j] * I[i,j]", H=csc(H), I=csc(I)) == H * I
    K = F.compute(F.lazy(csc(H)) + F.lazy(csc(I)))
    assert K == H + I


def test_semiring_einsum(gpu_lib):
    """Max- and min-plus SpMV over tensors whose fill (-Inf, +Inf)
    annihilates +, so skipping unstored entries is Finch's own result; a fill
    of 0 would make Finch fold 0 + q[k] for every unstored k, which no kernel
    here does, so that program is refused."""
    rng = np.random.default_rng(2)
    P = np.where(rng.random((30, 30)) < 0.2, rng.integers(1, 9, (30, 30)), 0).astype(np.float64)
    q = rng.integers(0, 9, 30).astype(np.float64)
    R = F.einsum("R[i] <<max>>= P[i,k] + q[k]", P=csc(np.where(P != 0, P, -np.inf), -np.inf), q=vec(q))
    want = np.array([max([P[i, k] + q[k] for k in range(30) if P[i, k] != 0], default=-np.inf)
                     for i in range(30)])
    assert R.todense().tolist() == want.tolist()
    Rmin = F.einsum("R[i] <<min>>= P[i,k] + q[k]", P=csc(np.where(P != 0, P, np.inf), np.inf), q=vec(q))
    want = np.array([min([P[i, k] + q[k] for k in range(30) if P[i, k] != 0], default=np.inf)
                     for i in range(30)])
    assert Rmin.todense().tolist() == want.tolist()
    with pytest.raises(F.FinchGBUnsupported):
        F.einsum("R[i] <<max>>= P[i,k] + q[k]", P=csc(P, 0.0), q=vec(q))
    Bp = F.Tensor(F.Dense(F.SparseList(F.Pattern())), P != 0)
    f = vec((rng.random(30) < 0.3).astype(np.bool_))
    reach = F.einsum("y[i] |= A[i,j] & f[j]", A=Bp, f=f)
    want = ((P != 0).astype(int) @ f.todense().astype(int)) > 0
    assert reach.todense().astype(bool).tolist() == want.tolist()


def test_lazy_spmm_sddmm_reduce(gpu_lib):
    rng = np.random.default_rng(3)
    D = np.where(rng.random((60, 40)) < 0.1, rng.standard_normal((60, 40)), 0.0)
    A = F.csr(D)
    B = dense2(rng.standard_normal((40, 16)))
    C = F.compute(F.lazy(A) @ F.lazy(B))
    np.testing.assert_allclose(C.todense(), D @ B.todense(), rtol=1e-12, atol=1e-12)
    X = dense2(rng.standard_normal((60, 8)))
    Y = dense2(rng.standard_normal((40, 8)))
    S = F.compute(F.lazy(A) * (F.lazy(X) @ F.lazy(Y).T))
    np.testing.assert_allclose(S.todense(), D * (X.todense() @ Y.todense().T), rtol=1e-12,
                               atol=1e-12)
    E = F.csr(np.where(rng.random((60, 40)) < 0.5, rng.standard_normal((60, 40)), 0.0))
    rs = F.compute((F.lazy(A) * F.lazy(E)).sum(dims=2))
    np.testing.assert_allclose(rs.todense(), (D * E.todense()).sum(axis=1), rtol=1e-12,
                               atol=1e-12)
    cs = F.compute(F.lazy(A).sum(dims=1))
    np.testing.assert_allclose(cs.todense(), D.sum(axis=0), rtol=1e-12, atol=1e-12)


class GraphAlgebra(F.DefaultAlgebra):
    """typemax(Int32) is "no edge": declared an annihilator of +, as a Finch
    program over Int32 weights must declare it (Finch's default algebra
    treats only infinities as annihilators of +, src/symbolic/symbolic.jl)."""

    def isannihilator(self, op, x):
        if op == "+" and x == np.iinfo(np.int32).max:
            return True
        return super().isannihilator(op, x)


def test_bellman_ford_in_einsum(gpu_lib):
    from finchgb.scheduler import get_scheduler
    from finchgb.workloads import random_graph

    rng = np.random.default_rng(4)
    n = 5000
    g = random_graph(rng, n, 6.0)
    A = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(np.int32(2**31 - 1), np.int32))), g)
    x = vec(np.where(np.arange(n) == 0, 0, 2**30).astype(np.int32))
    xh = x.todense().copy()
    with pytest.raises(F.FinchGBUnsupported):  # the default algebra cannot skip typemax
        F.einsum("y[i] <<min>>= A[i,j] + x[j]", A=A, x=x)
    sched = get_scheduler().set_options(algebra=GraphAlgebra())
    kernels = []
    for _ in range(10):
        y = F.einsum("y[i] <<min>>= A[i,j] + x[j]", A=A, x=x, ctx=sched)
        kernels.append(sched.last_kernel)
        x = F.einsum("x[i] = min(x[i], y[i])", x=x, y=y)
        yh = oracle.spmv_csc(oracle.SR_MINP, n, n, g.ptr, g.idx, g.val, xh)
        xh = np.minimum(xh, yh)
    assert np.array_equal(x.todense(), xh)
    # the CSC operand is pushed once, then pulled through its CSR copy
    assert kernels[0].endswith(",csc]") and all(k.endswith(",csr]") for k in kernels[1:])


def test_cg_in_einsum_small(gpu_lib):
    from finchgb.workloads import poisson2d

    b0 = poisson2d(16)
    A = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))),
                              F.workloads.SparseBuffers(b0.nrows, b0.ncols, b0.ptr, b0.idx,
                                                        b0.val, "csc"))  # symmetric
    rng = np.random.default_rng(5)
    bh = rng.uniform(-1, 1, b0.nrows)
    x = vec(np.zeros(b0.nrows))
    r = vec(bh.copy())
    p = vec(bh.copy())
    rr = F.einsum("s[] += r[i] * r[i]", r=r)
    for _ in range(200):
        q = F.einsum("q[i] += A[i,j] * p[j]", A=A, p=p)
        pq = F.einsum("s[] += p[i] * q[i]", p=p, q=q)
        alpha = F.einsum("a[] = rr[] / pq[]", rr=rr, pq=pq)
        x = F.einsum("x[i] = x[i] + alpha[] * p[i]", x=x, alpha=alpha, p=p)
        r = F.einsum("r[i] = r[i] - alpha[] * q[i]", r=r, alpha=alpha, q=q)
        rr_new = F.einsum("s[] += r[i] * r[i]", r=r)
        beta = F.einsum("b[] = n[] / o[]", n=rr_new, o=rr)
        p = F.einsum("p[i] = r[i] + beta[] * p[i]", r=r, beta=beta, p=p)
        rr = rr_new
        if rr.value < 1e-24:
            break
    D = b0.todense()
    np.testing.assert_allclose(D @ x.todense(), bh, atol=1e-9)


def test_unsupported_plan_raises(gpu_lib):
    D = F.Tensor(F.Dense(F.Dense(F.Element(0.0))), np.eye(4))
    with pytest.raises(F.FinchGBUnsupported):
        F.einsum("C[i,j] += A[i,k] * B[k,j]", A=D, B=D)  # dense GEMM: no kernel here


def test_einsum_sparse_times_sparse_is_spgemm(gpu_lib):
    rng = np.random.default_rng(21)
    Ad = np.where(rng.random((30, 20)) < 0.2, rng.integers(1, 5, (30, 20)), 0).astype(np.float64)
    Bd = np.where(rng.random((20, 25)) < 0.2, rng.integers(1, 5, (20, 25)), 0).astype(np.float64)
    C = F.einsum("C[i,j] += A[i,k] * B[k,j]", A=csc(Ad), B=csc(Bd))
    assert F.get_scheduler().last_kernel == "fgb_spgemm"
    assert np.array_equal(C.todense(), Ad @ Bd)


@pytest.mark.parametrize("n,p,seed", [(3, 0.7, 0), (3, 0.7, 1), (40, 0.3, 2)])
def test_einsum_max_plus_product(gpu_lib, n, p, seed):
    """test/suites/interface_tests.jl:72-82 restated: P and Q are
    Dense(SparseList(Element(-Inf))) with random integer-valued entries, and
    `@einsum init=-Inf R[i,j] <<max>>= P[i,k] + Q[k,j]` equals the triple
    loop R_ref[i,j] = max(R_ref[i,j], P[i,k] + Q[k,j]) exactly."""
    rng = np.random.default_rng(seed)

    def rand_tensor():
        D = np.where(rng.random((n, n)) < p, rng.integers(-1000, 1000, (n, n)).astype(np.float64), -np.inf)
        return D, F.Tensor(F.Dense(F.SparseList(F.Element(-np.inf))), D)

    Pd, P = rand_tensor()
    Qd, Q = rand_tensor()
    R = F.einsum("R[i,j] <<max>>= P[i,k] + Q[k,j]", init=-np.inf, P=P, Q=Q)
    R_ref = np.full((n, n), -np.inf)
    for i in range(n):
        for j in range(n):
            for k in range(n):
                R_ref[i, j] = max(R_ref[i, j], Pd[i, k] + Qd[k, j])
    assert np.array_equal(R.todense(), R_ref)
    # min-plus over a dense right operand, and or-and over Bool
    Md = np.where(rng.random((n, n)) < p, rng.integers(0, 50, (n, n)).astype(np.float64), np.inf)
    M = F.Tensor(F.Dense(F.SparseList(F.Element(np.inf))), Md)
    X = rng.integers(0, 50, (n, 5)).astype(np.float64)
    S = F.einsum("S[i,j] <<min>>= M[i,k] + X[k,j]", init=np.inf, M=M, X=dense2(X))
    assert np.array_equal(S.todense(), np.min(Md[:, :, None] + X[None, :, :], axis=1))
    Bd = rng.random((n, n)) < p
    Bt = F.Tensor(F.Dense(F.SparseList(F.Element(False))), Bd)
    Y = rng.random((n, 4)) < 0.5
    O = F.einsum("O[i,j] |= B[i,k] & Y[k,j]", B=Bt, Y=dense2(Y))
    assert np.array_equal(O.todense().astype(bool), (Bd.astype(int) @ Y.astype(int)) > 0)


def test_einsum_max_plus_needs_the_annihilating_fill(gpu_lib):
    D = np.array([[1.0, 0.0], [0.0, 2.0]])
    P = F.Tensor(F.Dense(F.SparseList(F.Element(0.0))), D)  # fill 0 is not max-plus's annihilator
    with pytest.raises(F.FinchGBUnsupported):
        F.einsum("R[i,j] <<max>>= P[i,k] + Q[k,j]", init=-np.inf, P=P, Q=dense2(D))


def test_eager_operations(gpu_lib):
    """The eager forms of test/suites/interface_tests.jl (A * B == C * D,
    A * x == C * x; src/interface/eager.jl:82-143), with Julia's `*`
    between tensors written `@` and Python's `*` as Julia's `.*`."""
    rng = np.random.default_rng(12)
    A = np.where(rng.random((5, 5)) < 0.5, rng.random((5, 5)), 0.0)
    B = np.where(rng.random((5, 5)) < 0.5, rng.random((5, 5)), 0.0)
    x = rng.random(5)
    C, D = csc(A), csc(B)
    np.testing.assert_allclose((C @ D).todense(), A @ B, rtol=1e-12, atol=1e-300)  # SpGEMM
    np.testing.assert_allclose((C @ x).todense(), A @ x, rtol=1e-12, atol=1e-300)  # SpMV, numpy operand
    np.testing.assert_allclose((C @ vec(x)).todense(), A @ x, rtol=1e-12, atol=1e-300)
    W = rng.random((5, 3))
    np.testing.assert_allclose((C @ W).todense(), A @ W, rtol=1e-12, atol=1e-300)  # SpMM
    np.testing.assert_allclose((F.csr(A) @ W).todense(), A @ W, rtol=1e-12, atol=1e-300)
    assert (C + D) == A + B and (C * D) == A * B
    y = vec(x)
    assert np.array_equal((y * 2.0).todense(), x * 2.0) and np.array_equal((2.0 * y).todense(), 2.0 * x)
    assert np.array_equal((y + 1.5).todense(), x + 1.5) and np.array_equal((y - 1.5).todense(), x - 1.5)
    assert np.array_equal((1.5 - y).todense(), 1.5 - x)
    assert np.array_equal((y + y).todense(), x + x)
    np.testing.assert_allclose(C.sum(dims=1).todense(), A.sum(axis=0), rtol=1e-12, atol=0)
    np.testing.assert_allclose(F.csr(A).sum(dims=2).todense(), A.sum(axis=1), rtol=1e-12, atol=0)
    np.testing.assert_allclose(float(C.sum().value), A.sum(), rtol=1e-12)
