"""fread(..., device) puts level buffers straight into HBM: a binsparse CSC
is uploaded as stored, a MatrixMarket file's coordinates are assembled on
the device; both then compute like any resident tensor."""
import numpy as np
import pytest

import oracle
from finchgb import Dense, Element, SparseList, Tensor, einsum, fread, fwrite, gpu, transfer
from finchgb.workloads import fsprand

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ext", [".bspnpy", ".mtx"])
def test_fread_to_device_then_spmv(gpu_lib, tmp_path, ext):
    rng = np.random.default_rng(17)
    b = fsprand(rng, 700, 500, 0.01)
    b.val = rng.integers(-9, 10, b.nnz).astype(np.float64)
    t = Tensor.from_buffers(Dense(SparseList(Element(0.0))), b)
    f = str(tmp_path / f"A{ext}")
    fwrite(f, t)
    A = fread(f, device=gpu())
    assert A.on_device if not hasattr(A, "body") else A.body.on_device
    x = transfer(gpu(), Tensor(Dense(Element(0.0)), rng.integers(-5, 6, 500).astype(np.float64)))
    y = einsum("y[i] += A[i,j]*x[j]", A=A, x=x)
    want = oracle.spmv_csc(0, 700, 500, b.ptr, b.idx, b.val, x.todense())
    assert np.array_equal(y.todense(), want)  # small integers: exact in any order
