"""Mixed-precision CG on the GPU: FP32/BF16-valued SpMV with FP64 dots,
updates and reliable residual replacement reaches the same FP64 tolerance as
FP64 CG; residuals are checked on the host in FP64 against the oracle's SpMV."""
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
