"""Per-call SpMM and SDDMM with no schedule given.  Large problems (B or Y
larger than 64 MB, at least 2^20 entries) take the virtual-row slab
schedules built for the call (for SpMM with two column bands),
bit-identical to asking for them explicitly.
While the stream is being captured into a CUDA graph those schedules, whose
build reads sizes back, are not taken: the capture succeeds and replays the
same product within tolerance."""
import numpy as np
import pytest
import torch

from finchgb import device as dev
from finchgb.workloads import zipf_csr
from helpers import RTOL, to_host, upload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big():
    rng = np.random.default_rng(77)
    n = 600_000
    A = zipf_csr(rng, n, n, mean=4.0, a=1.5, cap=2000, dtype=np.float32)
    assert A.nnz >= 1 << 20
    return A


def test_spmm_default_is_the_slab_schedule_and_capture_safe(gpu_lib, big):
    A = upload(big)
    B = torch.randn((big.ncols, 32), dtype=torch.float32, device="cuda")  # 77 MB
    C_def = to_host(dev.spmm(A, B))
    assert np.array_equal(C_def, to_host(dev.spmm(A, B, lanes=8, path=256, variant=3, bands=2)))
    C = torch.empty((big.nrows, 32), dtype=torch.float32, device="cuda")
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        dev.spmm(A, B, C)  # warm-up outside capture
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=s):
            dev.spmm(A, B, C)
    C.zero_()
    g.replay()
    got = to_host(C)
    absA = upload(big.__class__(big.nrows, big.ncols, big.ptr, big.idx, np.abs(big.val), big.orient))
    scale = to_host(dev.spmm(absA, B.abs(), lanes=8, path=128, variant=3))
    assert (np.abs(got - C_def) <= 2 * RTOL[np.dtype(np.float32)] * scale + 1e-30).all()


def test_sddmm_default_is_the_slab_schedule(gpu_lib, big):
    A = upload(big)
    X = torch.randn((big.nrows, 32), dtype=torch.float32, device="cuda")
    Y = torch.randn((big.ncols, 32), dtype=torch.float32, device="cuda")  # 77 MB
    o_def = to_host(dev.sddmm(A, X, Y))
    assert np.array_equal(o_def, to_host(dev.sddmm(A, X, Y, chunk=256, variant=2)))
