"""GPU parity of SpGEMM (fgb_spgemm_symbolic/numeric) against the oracle's
Gustavson nest: bit-exact structure and values for F64 and F32, fused and
unfused, CSR and CSC (Finch's column form), rows of both tiers (shared-
memory hash and global hash), empty rows and touched zero sums."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import coo_to_csr, csr_from_dense
from helpers import upload

pytestmark = pytest.mark.gpu


def rand_csr(rng, m, n, p, dtype, heavy_rows=()):
    D = np.where(rng.random((m, n)) < p, rng.standard_normal((m, n)), 0.0)
    for r in heavy_rows:
        D[r, : n // 2] = rng.standard_normal(n // 2)
    b = csr_from_dense(D)
    b.val = b.val.astype(dtype)
    return b


def check(A_b, B_b, orient, dtype, fma):
    A = upload(A_b)
    B = upload(B_b)
    C = dev.spgemm(A, B, flags=0 if fma else L.NO_FMA)
    torch.cuda.synchronize()
    if orient == "csr":
        want = oracle.spgemm_csr(A_b.nrows, B_b.ncols, A_b.ptr, A_b.idx, A_b.val, B_b.ptr, B_b.idx,
                                 B_b.val, fma=fma)
    else:  # column form = row form of the transposed problem
        want = oracle.spgemm_csr(B_b.ncols, A_b.nrows, B_b.ptr, B_b.idx, B_b.val, A_b.ptr, A_b.idx,
                                 A_b.val, fma=fma)
    assert np.array_equal(C.ptr.cpu().numpy(), want[0])
    assert np.array_equal(C.idx.cpu().numpy().astype(np.int64), want[1])
    assert C.val.cpu().numpy().tobytes() == want[2].tobytes()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("fma", [True, False])
def test_csr_both_tiers(gpu_lib, dtype, fma):
    rng = np.random.default_rng(21)
    A_b = rand_csr(rng, 400, 300, 0.02, dtype, heavy_rows=(3, 250))  # 2 rows with ub >> 256
    B_b = rand_csr(rng, 300, 500, 0.03, dtype, heavy_rows=(7,))
    A_b.val[::17] = 0.0  # products that touch a coordinate with zero
    check(A_b, B_b, "csr", dtype, fma)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_csc_column_form(gpu_lib, dtype):
    rng = np.random.default_rng(22)
    from finchgb.workloads import csc_from_dense

    Da = np.where(rng.random((350, 280)) < 0.03, rng.standard_normal((350, 280)), 0.0)
    Db = np.where(rng.random((280, 310)) < 0.03, rng.standard_normal((280, 310)), 0.0)
    Da[:, 5] = rng.standard_normal(350)  # a dense column of A: long rows of A^T
    A_b, B_b = csc_from_dense(Da), csc_from_dense(Db)
    A_b.val, B_b.val = A_b.val.astype(dtype), B_b.val.astype(dtype)
    check(A_b, B_b, "csc", dtype, True)


def test_poisson_square_and_errors(gpu_lib):
    from finchgb.workloads import poisson2d

    P = poisson2d(40)  # 1600 x 1600 5-point stencil; A*A is the 13-point one
    check(P, P, "csr", np.float64, True)
    A = upload(P)
    Bad = upload(csr_from_dense(np.ones((7, 3))))
    with pytest.raises(L.FinchGBError) as e:
        dev.spgemm(A, Bad)
    assert e.value.status == L.EINVAL
