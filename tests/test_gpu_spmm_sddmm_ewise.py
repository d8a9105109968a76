"""GPU parity of SpMM, SDDMM, elementwise merges and elementwise+reduce
(through the C ABI) against the oracle."""
import ctypes
import json
from pathlib import Path

import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import SparseBuffers, csr_from_dense, fsprand, zipf_csr
from helpers import assert_close, bf16_bits, to_dev, to_host, upload

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "finch_kats.json").read_text())["kats"]


def csr_rand(rng, m, n, p, dtype):
    D = np.where(rng.random((m, n)) < p, rng.standard_normal((m, n)), 0.0)
    r = csr_from_dense(D)
    r.val = r.val.astype(dtype)
    return r


def spmm_scale(r: SparseBuffers, B):
    return oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, np.abs(r.val).astype(np.float64),
                           np.abs(B).astype(np.float64))


def test_kat_einsum_matmul(gpu_lib):
    k = KATS["einsum_matmul"]
    r = csr_from_dense(np.array(k["A"]))
    A = upload(r)
    C = to_host(dev.spmm(A, to_dev(np.array(k["B"]))))
    assert C.tolist() == k["C"]


@pytest.mark.parametrize("dtype,bf16", [(np.float32, False), (np.float64, False), (np.float32, True)])
@pytest.mark.parametrize("nk", [128, 32, 64, 20, 3, 200])
def test_spmm_csr_bit_exact(gpu_lib, dtype, bf16, nk):
    """With FGB_FINCH_ORDER every C[i,k] is one running sum over j ascending,
    like Finch's nest: the result equals the oracle's nest bit for bit.  The
    default load-balanced schedule is within tolerance."""
    rng = np.random.default_rng(nk)
    r = csr_rand(rng, 257, 300, 0.05, dtype)
    B = rng.standard_normal((300, nk)).astype(dtype)
    A = upload(r, as_bf16=bf16)
    val = bf16_bits(r.val) if bf16 else r.val
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, val, B, bf16=bf16)
    C = to_host(dev.spmm(A, to_dev(B)))
    assert_close(C, want, spmm_scale(r, B), dtype)
    C1 = to_host(dev.spmm(A, to_dev(B), flags=L.FINCH_ORDER))
    assert np.array_equal(C1, want)
    C2 = to_host(dev.spmm(A, to_dev(B), flags=L.FINCH_ORDER | L.NO_FMA))
    want2 = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, val, B, fma=False, bf16=bf16)
    assert np.array_equal(C2, want2)


def test_spmm_accumulate_and_strides(gpu_lib):
    rng = np.random.default_rng(1)
    r = csr_rand(rng, 100, 80, 0.1, np.float32)
    Bfull = rng.standard_normal((80, 160)).astype(np.float32)
    A = upload(r)
    Bd = to_dev(Bfull)[:, :128]  # ldb = 160
    C0 = rng.standard_normal((100, 136)).astype(np.float32)
    Cd = to_dev(C0)
    dev.spmm(A, Bd, Cd[:, :128], flags=L.ACCUMULATE)
    want = oracle.spmm_csr(100, 80, r.ptr, r.idx, r.val, np.ascontiguousarray(Bfull[:, :128]),
                           C=np.ascontiguousarray(C0[:, :128]), init=False)
    got = to_host(Cd)
    scale = spmm_scale(r, np.ascontiguousarray(Bfull[:, :128])) + np.abs(C0[:, :128])
    assert_close(got[:, :128], want, scale, np.float32)
    assert np.array_equal(got[:, 128:], C0[:, 128:])  # untouched beyond nk


def test_spmm_csc_push(gpu_lib):
    rng = np.random.default_rng(2)
    D = np.where(rng.random((120, 90)) < 0.08, rng.standard_normal((120, 90)), 0.0)
    from finchgb.workloads import csc_from_dense

    b = csc_from_dense(D)
    b.val = b.val.astype(np.float32)
    B = rng.standard_normal((90, 48)).astype(np.float32)
    C = to_host(dev.spmm(upload(b), to_dev(B)))
    r = csr_from_dense(D)
    r.val = r.val.astype(np.float32)
    want = oracle.spmm_csr(120, 90, r.ptr, r.idx, r.val, B)
    assert_close(C, want, spmm_scale(r, B), np.float32)


def test_spmm_zipf_rows(gpu_lib):
    rng = np.random.default_rng(4)
    r = zipf_csr(rng, 20000, 20000, mean=16, cap=50_000)
    B = rng.standard_normal((20000, 128)).astype(np.float32)
    A = upload(r)
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, B, nthreads=oracle.max_threads())
    C = to_host(dev.spmm(A, to_dev(B), flags=L.FINCH_ORDER))
    assert np.array_equal(C, want)
    scale = spmm_scale(r, B)
    for lanes, variant in [(2, 0), (4, 0), (8, 0), (16, 0), (32, 0), (32, 1)]:
        for path in (1, 7, 64, 256, 4096):
            C1 = to_host(dev.spmm(A, to_dev(B), lanes=lanes, path=path, variant=variant))
            assert_close(C1, want, scale, np.float32)
            C2 = to_host(dev.spmm(A, to_dev(B), lanes=lanes, path=path, variant=variant))
            assert np.array_equal(C1, C2)  # deterministic carry fix-up
    flag = ctypes.c_int(1)
    L.call("fgb_ctx_device_error", dev.context(), ctypes.byref(flag))
    assert flag.value == 0  # no bounded wait ran out


@pytest.mark.parametrize("nk", [128, 64, 32, 20, 256])
def test_spmm_tma_stage_ring(gpu_lib, nk):
    """B rows staged through shared memory by TMA gather4: same results as
    the register-gather schedule within tolerance, for every slab width."""
    rng = np.random.default_rng(nk + 17)
    r = zipf_csr(rng, 9000, 7000, mean=16, cap=5000)
    B = rng.standard_normal((7000, nk)).astype(np.float32)
    A = upload(r)
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, B, nthreads=oracle.max_threads())
    C = to_host(dev.spmm(A, to_dev(B), lanes=32, path=300, variant=1))
    assert_close(C, want, spmm_scale(r, B), np.float32)
    flag = ctypes.c_int(1)
    L.call("fgb_ctx_device_error", dev.context(), ctypes.byref(flag))
    assert flag.value == 0


@pytest.mark.parametrize("nk", [128, 20, 36, 256])
def test_spmm_virtual_rows(gpu_lib, nk):
    """Variant 2 (column slabs over length-sorted virtual rows): within
    tolerance of the oracle for both slab widths and several virtual-row
    lengths (long rows split into partial sums), deterministic, and the same
    with 64-bit row pointers."""
    rng = np.random.default_rng(nk + 5)
    r = zipf_csr(rng, 12000, 9000, mean=16, cap=5000)
    B = rng.standard_normal((9000, nk)).astype(np.float32)
    A = upload(r)
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, B, nthreads=oracle.max_threads())
    scale = spmm_scale(r, B)
    Bd = to_dev(B)
    for lanes in (2, 4, 8):
        for T in (8, 64, 200):
            C1 = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=2))
            assert_close(C1, want, scale, np.float32)
            C2 = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=2))
            assert np.array_equal(C1, C2)
            # gathers staged in shared memory by cp.async: the same sums, bit for bit
            C4 = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=3))
            assert np.array_equal(C4, C1)
    A64 = dev.DeviceSparse(A.nrows, A.ncols, torch.from_numpy(r.ptr.astype(np.int64)).cuda(), A.idx,
                           A.val, "csr", 1)
    C3 = to_host(dev.spmm(A64, Bd, lanes=4, path=64, variant=2))
    assert np.array_equal(C3, to_host(dev.spmm(A, Bd, lanes=4, path=64, variant=2)))
    assert np.array_equal(C3, to_host(dev.spmm(A64, Bd, lanes=4, path=64, variant=3)))


def test_spmm_virtual_rows_accumulate_strides_empty(gpu_lib):
    rng = np.random.default_rng(31)
    D = np.zeros((500, 300))
    D[5, :] = rng.standard_normal(300)  # one row split into many virtual rows
    D[7, 3] = 1.5
    D[100:140] = np.where(rng.random((40, 300)) < 0.1, rng.standard_normal((40, 300)), 0.0)
    r = csr_from_dense(D)
    r.val = r.val.astype(np.float32)
    Bfull = rng.standard_normal((300, 72)).astype(np.float32)
    C0 = rng.standard_normal((500, 72)).astype(np.float32)
    A = upload(r)
    Cd = to_dev(C0)
    dev.spmm(A, to_dev(Bfull)[:, :48], Cd[:, :48], flags=L.ACCUMULATE, lanes=8, path=16, variant=2)
    B48 = np.ascontiguousarray(Bfull[:, :48])
    want = oracle.spmm_csr(500, 300, r.ptr, r.idx, r.val, B48, C=np.ascontiguousarray(C0[:, :48]),
                           init=False)
    got = to_host(Cd)
    assert_close(got[:, :48], want, spmm_scale(r, B48) + np.abs(C0[:, :48]), np.float32)
    assert np.array_equal(got[:, 48:], C0[:, 48:])  # untouched beyond nk
    Cd3 = to_dev(C0)
    dev.spmm(A, to_dev(Bfull)[:, :48], Cd3[:, :48], flags=L.ACCUMULATE, lanes=8, path=16, variant=3)
    assert np.array_equal(to_host(Cd3), got)
    empty = upload(csr_from_dense(np.zeros((40, 30), dtype=np.float32)))
    Ce = dev.spmm(empty, to_dev(rng.standard_normal((30, 16)).astype(np.float32)), variant=2)
    assert not to_host(Ce).any()
    with pytest.raises(L.FinchGBError):
        dev.spmm(A, to_dev(B48), flags=L.FINCH_ORDER, variant=2)


def test_spmm_merge_accumulate_and_empty(gpu_lib):
    rng = np.random.default_rng(8)
    D = np.zeros((300, 200))
    D[5, :] = rng.standard_normal(200)  # one dense row spanning many items
    D[7, 3] = 1.5
    r = csr_from_dense(D)
    r.val = r.val.astype(np.float32)
    B = rng.standard_normal((200, 64)).astype(np.float32)
    C0 = rng.standard_normal((300, 64)).astype(np.float32)
    A = upload(r)
    Cd = to_dev(C0)
    dev.spmm(A, to_dev(B), Cd, flags=L.ACCUMULATE, lanes=4, path=16)
    want = oracle.spmm_csr(300, 200, r.ptr, r.idx, r.val, B, C=C0.copy(), init=False)
    assert_close(to_host(Cd), want, spmm_scale(r, B) + np.abs(C0), np.float32)
    empty = upload(csr_from_dense(np.zeros((40, 30), dtype=np.float32)))
    assert not to_host(dev.spmm(empty, to_dev(rng.standard_normal((30, 8)).astype(np.float32)))).any()


@pytest.mark.parametrize("k", [64, 16, 7, 100])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sddmm(gpu_lib, k, dtype):
    rng = np.random.default_rng(k)
    r = zipf_csr(rng, 3000, 2500, mean=12, cap=2000, dtype=dtype)
    X = rng.standard_normal((3000, k)).astype(dtype)
    Y = rng.standard_normal((2500, k)).astype(dtype)
    A = upload(r)
    out = to_host(dev.sddmm(A, to_dev(X), to_dev(Y)))
    want = oracle.sddmm_csr(r.nrows, r.ptr, r.idx, r.val, X, Y, acc64=True)
    scale = np.abs(r.val.astype(np.float64)) * oracle.sddmm_csr(
        r.nrows, r.ptr, r.idx, np.ones(r.nnz), np.abs(X).astype(np.float64),
        np.abs(Y).astype(np.float64))
    assert_close(out, want, scale, dtype)
    # Finch order: sequential dot, then the product with A -- bit-exact
    out2 = to_host(dev.sddmm(A, to_dev(X), to_dev(Y), flags=L.FINCH_ORDER))
    assert np.array_equal(out2, oracle.sddmm_csr(r.nrows, r.ptr, r.idx, r.val, X, Y))
    # column slabs (dots accumulated across launches) and explicit schedules
    vn = 4 if dtype == np.float32 else 1
    for slab in (vn * 4, 32 // (8 // np.dtype(dtype).itemsize), k):
        for lanes in (4, 8, 32):
            out3 = to_host(dev.sddmm(A, to_dev(X), to_dev(Y), lanes=lanes, chunk=200, slab=slab))
            assert_close(out3, want, scale, dtype)
    # virtual rows (X's row held in registers): F32, k a multiple of 4 up to 128
    if dtype == np.float32 and k % 4 == 0:
        for T in (8, 64, 200):
            out4 = to_host(dev.sddmm(A, to_dev(X), to_dev(Y), chunk=T, variant=1))
            assert_close(out4, want, scale, dtype)
            out5 = to_host(dev.sddmm(A, to_dev(X), to_dev(Y), chunk=T, variant=1, slab=32))
            assert_close(out5, want, scale, dtype)
            assert np.array_equal(out4, to_host(dev.sddmm(A, to_dev(X), to_dev(Y), chunk=T, variant=1)))
            # gathers of Y staged in shared memory by cp.async: identical results
            assert np.array_equal(out4, to_host(dev.sddmm(A, to_dev(X), to_dev(Y), chunk=T, variant=2)))
            out6 = to_host(dev.sddmm(A, to_dev(X), to_dev(Y), chunk=T, variant=2, slab=32))
            assert np.array_equal(out5, out6)
    else:
        with pytest.raises(L.FinchGBError):
            dev.sddmm(A, to_dev(X), to_dev(Y), chunk=64, variant=1)
        with pytest.raises(L.FinchGBError):
            dev.sddmm(A, to_dev(X), to_dev(Y), chunk=64, variant=2)


def test_sddmm_csc_swaps_roles(gpu_lib):
    rng = np.random.default_rng(9)
    D = np.where(rng.random((60, 50)) < 0.1, rng.standard_normal((60, 50)), 0.0)
    from finchgb.workloads import csc_from_dense

    b = csc_from_dense(D)
    X = rng.standard_normal((60, 32))
    Y = rng.standard_normal((50, 32))
    out = to_host(dev.sddmm(upload(b), to_dev(X), to_dev(Y)))
    f = np.repeat(np.arange(50), np.diff(b.ptr))
    want = b.val * np.einsum("ek,ek->e", X[b.idx - 1], Y[f])
    np.testing.assert_allclose(out, want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("op", [L.EW_MUL, L.EW_ADD])
def test_ewise_merge(gpu_lib, dtype, op):
    rng = np.random.default_rng(op * 10 + np.dtype(dtype).itemsize)
    m, n = 400, 350
    ra = csr_rand(rng, m, n, 0.05, np.float64)
    rb = csr_rand(rng, m, n, 0.05, np.float64)
    ra.val = (ra.val * 100).astype(dtype)
    rb.val = (rb.val * 100).astype(dtype)
    C = dev.ewise(op, upload(ra), upload(rb))
    ptr, idx, val = C.to_host()
    wp, wi, wv = oracle.ewise(op, m, ra.ptr, ra.idx, ra.val, rb.ptr, rb.idx, rb.val)
    assert np.array_equal(ptr, wp) and np.array_equal(idx, wi) and np.array_equal(val, wv)


def test_ewise_kat_twofinger(gpu_lib):
    k = KATS["merge_twofinger_add"]
    x, y, z = k["x"], k["y"], k["z"]
    def vec(d):  # a SparseList vector as a 1 x n CSR matrix
        return SparseBuffers(1, d["n"], np.array(d["ptr"], np.int64), np.array(d["idx"], np.int64),
                             np.array(d["val"]), "csr")
    C = dev.ewise(L.EW_ADD, upload(vec(x)), upload(vec(y)))
    ptr, idx, val = C.to_host()
    assert ptr.tolist() == z["ptr"] and idx.tolist() == z["idx"] and val.tolist() == z["val"]


@pytest.mark.parametrize("dims", [0, 1, 2])
@pytest.mark.parametrize("sparse_b", [True, False])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_ewise_reduce(gpu_lib, dims, sparse_b, dtype):
    rng = np.random.default_rng(dims + 3 * sparse_b)
    m, n = 500, 300
    ra = csr_rand(rng, m, n, 0.06, dtype)
    A = upload(ra)
    if sparse_b:
        rb = csr_rand(rng, m, n, 0.3, dtype)
        y = to_host(dev.ewise_reduce(dims, A, B=upload(rb)))
        want = oracle.ewise_reduce(dims, m, n, ra.ptr, ra.idx, ra.val, rb.ptr, rb.idx, rb.val)
        scale = oracle.ewise_reduce(dims, m, n, ra.ptr, ra.idx, np.abs(ra.val), rb.ptr, rb.idx,
                                    np.abs(rb.val))
    else:
        Bd = rng.standard_normal((m, n)).astype(dtype)
        y = to_host(dev.ewise_reduce(dims, A, B_dense=to_dev(Bd)))
        want = oracle.ewise_reduce(dims, m, n, ra.ptr, ra.idx, ra.val, Bd=Bd)
        scale = oracle.ewise_reduce(dims, m, n, ra.ptr, ra.idx, np.abs(ra.val), Bd=np.abs(Bd))
    assert_close(y, want, scale, dtype)


def test_kat_reduce(gpu_lib):
    k = KATS["reduce"]
    A = upload(csr_from_dense(np.array(k["A"])))
    ones = to_dev(np.ones((4, 3)))
    np.testing.assert_allclose(to_host(dev.ewise_reduce(1, A, B_dense=ones)), k["dims1"], rtol=1e-15)
    np.testing.assert_allclose(to_host(dev.ewise_reduce(2, A, B_dense=ones)), k["dims2"], rtol=1e-15)
    np.testing.assert_allclose(to_host(dev.ewise_reduce(0, A, B_dense=ones)), [k["all"]], rtol=1e-15)


@pytest.mark.parametrize("npanels", [1, 2, 7, 16])
@pytest.mark.parametrize("nk", [128, 32])
def test_spmm_column_panels(gpu_lib, npanels, nk):
    """Panelled SpMM (L2-resident slice of B per panel) equals the oracle
    within tolerance, is deterministic, and accumulates correctly."""
    rng = np.random.default_rng(npanels * 100 + nk)
    r = zipf_csr(rng, 30000, 25000, mean=16, cap=50_000)
    B = rng.standard_normal((25000, nk)).astype(np.float32)
    A = upload(r)
    pn = dev.Panels(A, npanels)
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, B, nthreads=oracle.max_threads())
    scale = spmm_scale(r, B)
    Bd = to_dev(B)
    C1 = to_host(pn.spmm(Bd))
    assert_close(C1, want, scale, np.float32)
    C2 = to_host(pn.spmm(Bd))  # second call reuses the item boundaries
    assert np.array_equal(C1, C2)
    C0 = rng.standard_normal((30000, nk)).astype(np.float32)
    Cd = to_dev(C0)
    pn.spmm(Bd, Cd, flags=L.ACCUMULATE, path=128)
    assert_close(to_host(Cd), want + C0, scale + np.abs(C0), np.float32)
    C3 = to_host(pn.spmm(Bd, variant=1, path=256))  # TMA stage ring per panel
    assert_close(C3, want, scale, np.float32)
    pn.close()
