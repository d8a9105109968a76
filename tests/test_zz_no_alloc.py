"""fgb_spmm_noalloc: SpMM for callers that cannot allocate device memory.

A host whose device memory is owned by another allocator (for instance a
Julia process using CUDA.jl's pool), or a serving loop that must not enter an
allocator on its hot path, calls this entry point instead of fgb_spmm.  It
takes the scratch of the load-balanced schedule from one fixed device array
and allocates nothing.

The GPU tests call it through the C ABI and check its output against
fgb_spmm's on two calls in a row, the second on a different matrix and width
(the array keeps the previous call's contents, so nothing stale may leak
through), within the tolerance the other SpMM tests use; in FP32, FP64 and
with BF16 values; on a matrix large enough that the default item length does
not fit the array; and with the stream-ordered pool's high-water mark and the
device's free memory read around the call, to show it allocated nothing
(after one first call has loaded the library's device code and the array).
The decision that rejects a schedule too large for the array is checked on
the CPU, through the header that fgb_spmm_noalloc itself uses, so no test
hands the GPU an address it does not own.  The file is collected last and
passes both alone and after the other tests.
"""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest
import torch

from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import zipf_csr

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "finch.jl_gb300" / "csrc"
LIMIT = 16 * 1024 * 1024  # FGB_NOALLOC_SCRATCH_BYTES
RTOL = {L.F32: 2e-5, L.F64: 1e-12}  # |got - want| <= RTOL * sum_j |A[i,j] B[j,k]|

SHIM = r"""
#include "spmm_noalloc_plan.h"
extern "C" int pick(long long nrows, long long nnz, long long nk, long long esz, long long limit,
                    long long* path, long long* need) {
  int64_t p = 0;
  size_t n = 0;
  const bool ok = fgb::noalloc_pick_path(nrows, nnz, nk, (size_t)esz, (size_t)limit, &p, &n);
  *path = p;
  *need = n > (size_t)0x7fffffffffffffffLL ? -1 : (long long)n;
  return ok ? 1 : 0;
}
extern "C" long long need_at(long long nrows, long long nnz, long long nk, long long esz, long long path) {
  const size_t n = fgb::merge_scratch_bytes(nrows, nnz, nk, (size_t)esz, path);
  return n > (size_t)0x7fffffffffffffffLL ? -1 : (long long)n;
}
"""


@pytest.fixture(scope="module")
def plan_shim(tmp_path_factory):
    d = tmp_path_factory.mktemp("noalloc_shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "shim.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", "-I", str(CSRC), str(d / "shim.cpp"),
                    "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    lib.pick.argtypes = [ctypes.c_longlong] * 5 + [ctypes.POINTER(ctypes.c_longlong)] * 2
    lib.pick.restype = ctypes.c_int
    lib.need_at.argtypes = [ctypes.c_longlong] * 5
    lib.need_at.restype = ctypes.c_longlong

    def pick(nrows, nnz, nk, esz, limit=LIMIT):
        p, n = ctypes.c_longlong(), ctypes.c_longlong()
        ok = lib.pick(nrows, nnz, nk, esz, limit, ctypes.byref(p), ctypes.byref(n))
        return bool(ok), p.value, n.value

    pick.need_at = lib.need_at
    return pick


def test_noalloc_sizing_on_cpu(plan_shim):
    # a small matrix keeps the default item length
    ok, path, need = plan_shim(30000, 480000, 128, 4)
    assert ok and path == 256 and 0 < need <= LIMIT
    # 600K rows with mean 16: the default items need ~21 MB, so items lengthen to 512
    ok, path, need = plan_shim(600_000, 9_600_000, 128, 4)
    assert ok and path == 512 and need <= LIMIT
    assert plan_shim.need_at(600_000, 9_600_000, 128, 4, 256) > LIMIT
    # every chosen length fits, and half of it would not
    for nrows, nnz, nk, esz in [(10**6, 16 * 10**6, 128, 4), (10**7, 10**8, 64, 8), (5, 7, 4, 4)]:
        ok, path, need = plan_shim(nrows, nnz, nk, esz)
        assert ok and need <= LIMIT and need == plan_shim.need_at(nrows, nnz, nk, esz, path)
        if path > 256:
            assert plan_shim.need_at(nrows, nnz, nk, esz, path // 2) > LIMIT
    # far too large even at 2^24-step items: rejected (the entry point returns
    # EINVAL on this decision before any device access)
    ok, path, need = plan_shim(2**45, 0, 2**20, 4)
    assert not ok and path == 2**24 and (need == -1 or need > LIMIT)
    assert not plan_shim(2**40, 2**40, 2**12, 8)[0]
    assert plan_shim.need_at(2**62, 2**62, 2**30, 8, 256) == -1  # saturates, no wrap-around


# ---- GPU: through the C ABI -------------------------------------------------

class _Pool:
    """The device's current stream-ordered pool, read through the driver API:
    its used-memory high-water mark shows any stream-ordered allocation made
    in between, even one freed again before the call returned."""
    USED_CURRENT, USED_HIGH = 7, 8  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT / _HIGH

    def __init__(self, device: int):
        self.cu = ctypes.CDLL("libcuda.so.1")
        d = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(d), device) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), d) == 0

    def _get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        z = ctypes.c_uint64(0)  # resets the high-water mark to the current use
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_HIGH, ctypes.byref(z)) == 0

    def used(self):
        return self._get(self.USED_CURRENT)

    def high(self):
        return self._get(self.USED_HIGH)

    def free_bytes(self):
        f, t = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.cu.cuMemGetInfo_v2(ctypes.byref(f), ctypes.byref(t)) == 0
        return f.value


def _call(fn, A, B, C, dtype):
    d = A.desc()
    return getattr(L.load(), fn)(dev.context(), ctypes.byref(d), B.data_ptr(), B.stride(0), B.shape[1],
                                 C.data_ptr(), C.stride(0), dtype, 0, dev.stream_ptr())


def _matrix(rng, m, val):
    h = zipf_csr(rng, m, m, mean=16, cap=50_000)
    vd = {"f32": None, "f64": torch.float64, "bf16": torch.bfloat16}[val]
    vals = h.val.astype(np.float64) if val == "f64" else h.val
    A = dev.DeviceSparse.from_host(h.nrows, h.ncols, h.ptr, h.idx, vals, orient="csr", val_dtype=vd)
    absA = dev.DeviceSparse.from_host(h.nrows, h.ncols, h.ptr, h.idx, np.abs(vals.astype(np.float64)),
                                      orient="csr")
    return A, absA


def _check_pair(rng, A, absA, m, nk, dtype, pool):
    tdt = torch.float64 if dtype == L.F64 else torch.float32
    B = torch.from_numpy(rng.standard_normal((m, nk))).to(tdt).cuda()
    C_ref = torch.empty((m, nk), dtype=tdt, device="cuda")
    C_na = torch.full((m, nk), float("nan"), dtype=tdt, device="cuda")
    L.check(_call("fgb_spmm", A, B, C_ref, dtype), "fgb_spmm")
    torch.cuda.synchronize()
    pool.reset_high()
    used0, free0 = pool.used(), pool.free_bytes()
    L.check(_call("fgb_spmm_noalloc", A, B, C_na, dtype), "fgb_spmm_noalloc")
    torch.cuda.synchronize()
    assert pool.high() == used0, "fgb_spmm_noalloc allocated from the stream-ordered pool"
    assert pool.free_bytes() >= free0, "fgb_spmm_noalloc left device memory allocated"
    scale = dev.spmm(absA, B.abs().double(), flags=L.FINCH_ORDER)
    torch.cuda.synchronize()
    assert torch.isfinite(C_na).all(), "output not fully written"
    diff = (C_na.double() - C_ref.double()).abs()
    assert (diff <= RTOL[dtype] * scale + 1e-30).all(), diff.max().item()


@pytest.fixture(scope="module")
def pool(gpu_lib):
    """The pool reader, after one small call has loaded the library's device
    code and its fixed scratch array on this device (the array is held from
    then until the process exits; loading it is the only device memory the
    entry point ever causes to be taken, and it happens once)."""
    p = _Pool(torch.cuda.current_device())
    rng = np.random.default_rng(1)
    A, _ = _matrix(rng, 500, "f32")
    B = torch.ones((500, 8), dtype=torch.float32, device="cuda")
    C = torch.empty((500, 8), dtype=torch.float32, device="cuda")
    free0 = p.free_bytes()
    L.check(_call("fgb_spmm_noalloc", A, B, C, L.F32), "fgb_spmm_noalloc")
    torch.cuda.synchronize()
    assert free0 - p.free_bytes() <= LIMIT + (64 << 20)  # the array (and device code), once
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("val,dtype", [("f32", L.F32), ("bf16", L.F32), ("f64", L.F64)])
def test_noalloc_matches_spmm_two_calls(gpu_lib, pool, val, dtype):
    rng = np.random.default_rng(7)
    # call 1 and call 2 differ in matrix, width and item count, so plan and
    # carry words left in the array by call 1 would show in call 2's output
    for m, nk in ((30000, 128), (21000, 32 if dtype == L.F32 else 16)):
        A, absA = _matrix(rng, m, val)
        _check_pair(rng, A, absA, m, nk, dtype, pool)


@pytest.mark.gpu
def test_noalloc_lengthened_items(gpu_lib, pool):
    # 600K rows with mean 16 at nk = 128: the default 256-step items need
    # ~21 MB of scratch, above the array, so the entry point lengthens them
    rng = np.random.default_rng(11)
    m = 600_000
    A, absA = _matrix(rng, m, "f32")
    for nk in (128, 64):
        _check_pair(rng, A, absA, m, nk, L.F32, pool)
