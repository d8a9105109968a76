"""Mixed-precision CG on the GPU: FP32/BF16-valued SpMV summed in FP32, FP64
or pairs of FP32 numbers, with FP64 reliable residual replacement, reaches
the same FP64 tolerance as FP64 CG; residuals are checked on the host in FP64
against the oracle's SpMV."""
import numpy as np
import pytest
import torch

import finchgb as F
import oracle
from finchgb import cg
from finchgb import device as dev
from finchgb.workloads import poisson2d

pytestmark = pytest.mark.gpu


def true_residual(A, x, b):
    ax = oracle.spmv_csr(oracle.SR_PT, A.nrows, A.ncols, A.ptr, A.idx, A.val, x)
    return np.linalg.norm(b - ax) / np.linalg.norm(b)


@pytest.mark.parametrize("precision", ["f64", "f32", "bf16"])
@pytest.mark.parametrize("N", [32, 96])
def test_cg_reaches_fp64_tolerance(gpu_lib, precision, N):
    A = poisson2d(N)
    rng = np.random.default_rng(N)
    b = rng.uniform(-1, 1, A.nrows)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    x, res = cg.cg_solve(Ad, torch.from_numpy(b).cuda(), precision=precision, rtol=1e-10,
                         chunk=16, replace_every=64)
    xh = x.cpu().numpy()
    assert res.converged
    assert res.true_rel_residual <= 1e-10
    assert true_residual(A, xh, b) <= 1.2e-10  # recomputed independently in FP64
    np.testing.assert_allclose(xh, np.linalg.solve(A.todense(), b), rtol=0, atol=1e-6)


def test_cg_deterministic_and_warm_start(gpu_lib):
    A = poisson2d(48)
    b = np.cos(np.arange(A.nrows))
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    x1, r1 = cg.cg_solve(Ad, bd, precision="f32", chunk=8)
    x2, r2 = cg.cg_solve(Ad, bd, precision="f32", chunk=8)
    assert torch.equal(x1, x2) and r1.iterations == r2.iterations
    x3, r3 = cg.cg_solve(Ad, bd, x=x1.clone(), precision="f32", chunk=8)
    assert r3.converged and r3.iterations == 0  # already at tolerance


def test_cg_rejects_bad_options(gpu_lib):
    A = poisson2d(8)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    with pytest.raises(F.FinchGBError):
        cg.cg_solve(Ad, torch.ones(A.nrows, dtype=torch.float64, device="cuda"), chunk=7)


def test_cg_finch_program_matches_native(gpu_lib):
    A = poisson2d(24)
    b = np.sin(np.arange(A.nrows) * 0.1) + 0.5
    At = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Element(0.0))),
                               F.workloads.SparseBuffers(A.nrows, A.ncols, A.ptr, A.idx, A.val,
                                                         "csc"))  # symmetric: CSR == CSC
    bt = F.Tensor(F.Dense(F.Element(0.0)), b)
    x, it = cg.cg_finch(At, bt, rtol=1e-10)
    assert true_residual(A, x.todense(), b) <= 1e-9
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    xn, res = cg.cg_solve(Ad, torch.from_numpy(b).cuda(), precision="f64", chunk=2)
    np.testing.assert_allclose(x.todense(), xn.cpu().numpy(), rtol=0, atol=1e-8)


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_cg_fp64_accumulation_equals_fp64(gpu_lib, precision):
    """Poisson values (4, -1) are exact in FP32 and BF16: widened to FP64 and
    summed in FP64, the low-precision SpMV gives the FP64 iterates bit for
    bit, so the solve takes the FP64 iteration count; the banded matrix is
    read through 16-bit column offsets."""
    A = poisson2d(64)
    b = np.random.default_rng(5).uniform(-1, 1, A.nrows)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    x64, r64 = cg.cg_solve(Ad, bd, precision="f64", chunk=16, replace_every=64)
    xl, rl = cg.cg_solve(Ad, bd, precision=precision, accumulate="f64", chunk=16, replace_every=64)
    assert r64.compact_index and rl.compact_index
    assert rl.iterations == r64.iterations and torch.equal(xl, x64)
    assert rl.converged and true_residual(A, xl.cpu().numpy(), b) <= 1.2e-10


@pytest.mark.parametrize("acc", ["pair", "spmv_pair"])
@pytest.mark.parametrize("precision", ["f32", "bf16"])
@pytest.mark.parametrize("N", [32, 96])
def test_cg_pair_sums_reach_fp64_tolerance(gpu_lib, precision, N, acc):
    """Pair arithmetic (about 48 bits) for the SpMV sums (spmv_pair: FP64
    vectors, dots and updates; pair: those too in pairs): the FP64
    tolerance, and no more than a few percent more iterations than FP64
    CG, deterministically."""
    A = poisson2d(N)
    b = np.random.default_rng(N + 1).uniform(-1, 1, A.nrows)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    _, r64 = cg.cg_solve(Ad, bd, precision="f64", rtol=1e-10, chunk=16, replace_every=64)
    x, res = cg.cg_solve(Ad, bd, precision=precision, accumulate=acc, rtol=1e-10, chunk=16,
                         replace_every=64)
    assert res.converged and res.true_rel_residual <= 1e-10
    assert true_residual(A, x.cpu().numpy(), b) <= 1.2e-10
    assert res.iterations <= int(1.05 * r64.iterations) + 16
    x2, res2 = cg.cg_solve(Ad, bd, precision=precision, accumulate=acc, rtol=1e-10, chunk=16,
                           replace_every=64)
    assert torch.equal(x, x2) and res2.iterations == res.iterations


def test_cg_pair_sums_wide_matrix_and_warm_start(gpu_lib):
    """The int32 index path of the pair SpMV, a warm start that is already
    converged (x untouched), and the option checks."""
    n = 70000  # couplings 40,000 apart: no 16-bit column offsets
    rng = np.random.default_rng(12)
    far = rng.integers(0, n, 1000)
    rows = np.concatenate([np.arange(n), np.arange(n - 1), np.arange(1, n), far, (far + 40000) % n])
    cols = np.concatenate([np.arange(n), np.arange(1, n), np.arange(n - 1), (far + 40000) % n, far])
    vals = np.concatenate([np.full(n, 2.5), np.full(2 * (n - 1), -1.0), np.full(2000, -0.1)])
    from finchgb.workloads import coo_to_csr

    A = coo_to_csr(n, n, rows + 1, cols + 1, vals)
    b = rng.uniform(-1, 1, n)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    for acc in ("pair", "spmv_pair"):
        x, res = cg.cg_solve(Ad, bd, precision="f32", accumulate=acc, rtol=1e-10, chunk=8)
        assert res.converged and not res.compact_index
        assert true_residual(A, x.cpu().numpy(), b) <= 1.2e-10
    x0 = x.clone()
    x3, r3 = cg.cg_solve(Ad, bd, x=x0, precision="bf16", accumulate="pair", chunk=8)
    assert r3.converged and r3.iterations == 0 and torch.equal(x3, x)
    for acc in ("pair", "spmv_pair"):
        with pytest.raises(F.FinchGBError):  # FP64 values have no pair mode
            cg.cg_solve(Ad, bd, precision="f64", accumulate=acc, chunk=8)


def test_cg_wide_matrix_keeps_the_int32_index(gpu_lib):
    """Columns farther than 32,767 from the diagonal: no compact index, same
    tolerance reached (a diagonally dominant SPD matrix with far couplings)."""
    n = 70000
    rng = np.random.default_rng(9)
    far = rng.integers(0, n, 2000)
    rows = np.concatenate([np.arange(n), np.arange(n - 1), np.arange(1, n), far, (far + 40000) % n])
    cols = np.concatenate([np.arange(n), np.arange(1, n), np.arange(n - 1), (far + 40000) % n, far])
    vals = np.concatenate([np.full(n, 6.0), np.full(2 * (n - 1), -1.0), np.full(4000, -0.5)])
    from finchgb.workloads import coo_to_csr

    A = coo_to_csr(n, n, rows + 1, cols + 1, vals)
    b = rng.uniform(-1, 1, n)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    for precision in ("f64", "f32"):
        x, res = cg.cg_solve(Ad, torch.from_numpy(b).cuda(), precision=precision, rtol=1e-10, chunk=8)
        assert res.converged and not res.compact_index
        assert true_residual(A, x.cpu().numpy(), b) <= 1.2e-10
