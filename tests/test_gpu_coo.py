"""GPU parity of fgb_coo_assemble (fsparse + copy into Dense(SparseList), in
HBM) against the oracle: bit-exact coordinates and values for every value
type and combine, both orientations, both coordinate widths and bases."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import Dense, Element, SparseList, Tensor, compute, einsum, fsparse, gpu, lazy, transfer
from finchgb import device as dev
from helpers import to_host

pytestmark = pytest.mark.gpu

COMBINE = {"+": L.COMBINE_ADD, "|": L.COMBINE_OR, "min": L.COMBINE_MIN, "max": L.COMBINE_MAX,
           "last": L.COMBINE_LAST}


def check(m, n, I, J, V, orient="csc", combine="+", idx_dtype=torch.int64, base=1):
    Id = torch.from_numpy(np.asarray(I) - 1 + base).to(idx_dtype).cuda()
    Jd = torch.from_numpy(np.asarray(J) - 1 + base).to(idx_dtype).cuda()
    Vd = None if V is None else torch.from_numpy(V if V.dtype != np.bool_ else V.astype(np.uint8)).cuda()
    A = dev.coo_assemble(m, n, Id, Jd, Vd, orient=orient, combine=COMBINE[combine], in_base=base)
    ptr, idx, val = oracle.coo_assemble(m, n, I, J, V, csc=orient == "csc", combine=COMBINE[combine])
    torch.cuda.synchronize()
    assert np.array_equal(A.ptr.cpu().numpy().astype(np.int64), ptr)
    assert np.array_equal(A.idx.cpu().numpy().astype(np.int64), idx)
    if V is not None:
        got = A.val.cpu().numpy()
        want = val.astype(np.uint8) if val.dtype == np.bool_ else val
        assert got.tobytes() == want.tobytes()  # bit for bit (NaN, -0.0 included)
    return A


@pytest.mark.parametrize("orient", ["csc", "csr"])
@pytest.mark.parametrize("dtype,combine", [(np.float64, "+"), (np.float32, "+"), (np.int32, "+"),
                                           (np.int64, "min"), (np.float64, "max"),
                                           (np.bool_, "|"), (np.float32, "last")])
def test_random_with_duplicates(gpu_lib, orient, dtype, combine):
    rng = np.random.default_rng(hash((orient, combine, np.dtype(dtype).name)) % 2**32)
    m, n, k = 700, 500, 40000  # ~11% of the coordinates repeat
    I, J = rng.integers(1, m + 1, k), rng.integers(1, n + 1, k)
    if dtype == np.bool_:
        V = rng.random(k) < 0.3
    elif np.dtype(dtype).kind == "f":
        V = rng.standard_normal(k).astype(dtype) * 10.0 ** rng.integers(-8, 9, k)
        V[::97] = -0.0
        V[::89] = 0.0
    else:
        info = np.iinfo(dtype)
        V = rng.integers(info.min // 2, info.max // 2, size=k, dtype=dtype)  # + wraps
    check(m, n, I, J, V, orient, combine)


@pytest.mark.parametrize("idx_dtype,base", [(torch.int32, 1), (torch.int64, 0), (torch.int32, 0)])
def test_coordinate_types_and_bases(gpu_lib, idx_dtype, base):
    rng = np.random.default_rng(3)
    I, J = rng.integers(1, 301, 5000), rng.integers(1, 201, 5000)
    check(300, 200, I, J, rng.standard_normal(5000), idx_dtype=idx_dtype, base=base)


def test_pattern_empty_and_errors(gpu_lib):
    rng = np.random.default_rng(4)
    I, J = rng.integers(1, 50, 300), rng.integers(1, 9000, 300)  # most columns empty
    check(49, 9000, I, J, None)
    A = check(10, 7, np.zeros(0, np.int64), np.zeros(0, np.int64), np.zeros(0))
    assert A.nnz == 0 and A.ptr.cpu().tolist() == [1] * 8
    with pytest.raises(L.FinchGBError) as e:
        check(10, 7, np.array([11]), np.array([1]), np.array([1.0]))
    assert e.value.status == L.EINVAL
    with pytest.raises(L.FinchGBError) as e:
        check(10, 7, np.array([1]), np.array([1]), np.array([1.0]), combine="|")
    assert e.value.status == L.EUNSUPPORTED


def test_fsparse_transfer_then_spmv(gpu_lib):
    """Tensor(fsparse(...)) moved to the GPU is assembled in HBM and computes
    through the scheduler like any Dense(SparseList) tensor."""
    rng = np.random.default_rng(9)
    m, n = 400, 300
    I, J = rng.integers(1, m + 1, 6000), rng.integers(1, n + 1, 6000)
    V = rng.integers(-9, 10, 6000).astype(np.float64)
    A = transfer(gpu(), fsparse(I, J, V, (m, n)))
    assert A.dsparse is not None and A.dsparse.orient == "csc"
    x = Tensor(Dense(Element(0.0)), rng.integers(-5, 6, n).astype(np.float64))
    y = einsum("y[i] += A[i,j]*x[j]", A=A, x=transfer(gpu(), x))
    ptr, idx, val = oracle.coo_assemble(m, n, I, J, V)
    want = oracle.spmv_csc(0, m, n, ptr, idx, val, x.todense())
    assert np.array_equal(y.todense(), want)  # small integers: exact in any order
