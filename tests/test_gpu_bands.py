"""GPU parity of the column-band schedules: SpMM and SDDMM over virtual rows
with A's columns cut into bands, each band's entries in launches of their
own so a launch gathers from a fraction of B (or Y).

Bands change only where a heavy row's chunks are cut, so: results lie within
the float tolerance of the oracle; they are deterministic; the register and
cp.async builds agree bit for bit; a row of at most T entries (one running
sum, continued from C band after band) equals the unbanded schedule's bit
for bit; SDDMM entries do not combine, so banded SDDMM equals unbanded."""
import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb import device as dev
from finchgb.workloads import csr_from_dense, zipf_csr
from helpers import assert_close, to_dev, to_host, upload

pytestmark = pytest.mark.gpu


def spmm_scale(r, B):
    return oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, np.abs(r.val).astype(np.float64),
                           np.abs(B).astype(np.float64))


@pytest.mark.parametrize("nk", [128, 36])
def test_spmm_bands(gpu_lib, nk):
    rng = np.random.default_rng(nk + 11)
    r = zipf_csr(rng, 12000, 9000, mean=16, cap=5000)
    B = rng.standard_normal((9000, nk)).astype(np.float32)
    A = upload(r)
    want = oracle.spmm_csr(r.nrows, r.ncols, r.ptr, r.idx, r.val, B, nthreads=oracle.max_threads())
    scale = spmm_scale(r, B)
    lens = np.diff(r.ptr)
    Bd = to_dev(B)
    for lanes in (4, 8):
        for T in (8, 64, 200):
            flat = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=3))
            short = lens <= T
            for bands in (2, 3, 8):
                C1 = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=3, bands=bands))
                assert_close(C1, want, scale, np.float32)
                assert np.array_equal(C1, to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=3,
                                                           bands=bands)))
                C2 = to_host(dev.spmm(A, Bd, lanes=lanes, path=T, variant=2, bands=bands))
                assert np.array_equal(C1, C2)
                assert np.array_equal(C1[short], flat[short])


def test_spmm_bands_accumulate_strides_empty(gpu_lib):
    rng = np.random.default_rng(41)
    D = np.zeros((500, 300))
    D[5, :] = rng.standard_normal(300)  # one row across every band, split into chunks
    D[7, 3] = 1.5
    D[9, 299] = -2.0  # only in the last band
    D[100:140] = np.where(rng.random((40, 300)) < 0.1, rng.standard_normal((40, 300)), 0.0)
    r = csr_from_dense(D)
    r.val = r.val.astype(np.float32)
    Bfull = rng.standard_normal((300, 72)).astype(np.float32)
    C0 = rng.standard_normal((500, 72)).astype(np.float32)
    A = upload(r)
    B48 = np.ascontiguousarray(Bfull[:, :48])
    want = oracle.spmm_csr(500, 300, r.ptr, r.idx, r.val, B48, C=np.ascontiguousarray(C0[:, :48]),
                           init=False)
    for bands, variant in ((2, 3), (4, 3), (8, 3), (4, 2)):
        Cd = to_dev(C0)
        dev.spmm(A, to_dev(Bfull)[:, :48], Cd[:, :48], flags=L.ACCUMULATE, lanes=8, path=16, variant=variant,
                 bands=bands)
        got = to_host(Cd)
        assert_close(got[:, :48], want, spmm_scale(r, B48) + np.abs(C0[:, :48]), np.float32)
        assert np.array_equal(got[:, 48:], C0[:, 48:])  # untouched beyond nk
        Cw = to_host(dev.spmm(A, to_dev(B48), lanes=8, path=16, variant=variant, bands=bands))
        assert_close(Cw, oracle.spmm_csr(500, 300, r.ptr, r.idx, r.val, B48), spmm_scale(r, B48), np.float32)
        assert not Cw[np.diff(r.ptr) == 0].any()  # empty rows written as zeros
    empty = upload(csr_from_dense(np.zeros((40, 30), dtype=np.float32)))
    for variant in (2, 3):
        Ce = dev.spmm(empty, to_dev(rng.standard_normal((30, 16)).astype(np.float32)), variant=variant, bands=4)
        assert not to_host(Ce).any()


def test_spmm_bands_rejects(gpu_lib):
    rng = np.random.default_rng(3)
    r = zipf_csr(rng, 200, 100, mean=4, cap=50)
    A = upload(r)
    Bd = to_dev(rng.standard_normal((100, 32)).astype(np.float32))
    for kw in ({"variant": 3, "bands": 9}, {"variant": 3, "bands": -1}, {"variant": 0, "bands": 2},
               {"variant": 4}):
        with pytest.raises(L.FinchGBError) as e:
            dev.spmm(A, Bd, lanes=8, path=64, **kw)
        assert e.value.status == L.EINVAL


def test_sddmm_bands(gpu_lib):
    rng = np.random.default_rng(5)
    r = zipf_csr(rng, 6000, 7000, mean=16, cap=3000)
    X = rng.standard_normal((6000, 64)).astype(np.float32)
    Y = rng.standard_normal((7000, 64)).astype(np.float32)
    A = upload(r)
    Xd, Yd = to_dev(X), to_dev(Y)
    want = oracle.sddmm_csr(r.nrows, r.ptr, r.idx, r.val, X, Y, acc64=True)
    scale = oracle.sddmm_csr(r.nrows, r.ptr, r.idx, np.abs(r.val), np.abs(X), np.abs(Y), acc64=True)
    for variant in (1, 2):
        for slab in (0, 32):
            flat = to_host(dev.sddmm(A, Xd, Yd, chunk=128, variant=variant, slab=slab))
            assert_close(flat, want, scale, np.float32)
            for bands in (2, 5, 8):
                got = to_host(dev.sddmm(A, Xd, Yd, chunk=128, variant=variant, slab=slab, bands=bands))
                assert np.array_equal(got, flat)
