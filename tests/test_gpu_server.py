"""Serving: continuous batching on the device loop.  Each request's result is
bit-identical alone (per-call mode) and in the mix (batched mode), matches
the oracle within tolerance, admission by HBM footprint queues what does not
fit, and bounded waits report timeouts instead of hanging."""
import time

import numpy as np
import pytest
import torch

import oracle
from finchgb import _lib as L
from finchgb.server import Server, random_csr

pytestmark = pytest.mark.gpu


def host_csr(A):
    torch.cuda.synchronize()
    return (A.ptr.cpu().numpy().astype(np.int64) + 1, A.idx.cpu().numpy().astype(np.int64) + 1,
            A.val.cpu().numpy())


def make_requests(rng, mats, partners, count, pinned=True):
    """Pinned outputs are written in place by the device; pageable ones go
    through pool memory and a copy back, so both paths are exercised."""
    pin = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    reqs = []
    for t in range(count):
        k = int(rng.integers(len(mats)))
        A = mats[k]
        op = ("spmv", "spmm", "masked_mul")[t % 3]
        if op == "spmv":
            inp = pin(torch.from_numpy(rng.standard_normal(A.ncols).astype(np.float32)))
            out = pin(torch.empty(A.nrows, dtype=torch.float32))
            reqs.append((op, k, inp, out, -1, 0))
        elif op == "spmm":
            inp = pin(torch.from_numpy(rng.standard_normal((A.ncols, 32)).astype(np.float32)))
            out = pin(torch.empty((A.nrows, 32), dtype=torch.float32))
            reqs.append((op, k, inp, out, -1, 32))
        else:
            out = pin(torch.empty(A.nnz, dtype=torch.float32))
            reqs.append((op, k, None, out, 1, 0))  # 1: use the partner of matrix k
    return reqs


@pytest.fixture(scope="module")
def library(gpu_lib):
    rng = np.random.default_rng(0)
    mats, partners = [], []
    for k in range(12):
        n = int(np.exp(rng.uniform(np.log(64), np.log(2048))))
        p = float(rng.uniform(0.005, 0.05))
        mats.append(random_csr(1000 + k, n, n, p))
        partners.append(random_csr(5000 + k, n, n, p))
    return mats, partners


def run(server_mode, mats, partners, reqs, batch=False, tuning=None, **kw):
    with Server(mode=server_mode, **kw) as srv:
        ids = [srv.register(A) for A in mats]
        pids = [srv.register(B) for B in partners]
        if tuning is not None:
            srv.set_tuning(tuning)
        if batch:
            recs = [srv.request(op, ids[k], inp, out, matrix_b=pids[k] if kb >= 0 else -1, nk=nk)
                    for op, k, inp, out, kb, nk in reqs]
            tickets = srv.submit_batch(recs)
            lat = srv.wait_batch(tickets)
        else:
            tickets = []
            for op, k, inp, out, kb, nk in reqs:
                tickets.append(srv.submit(op, ids[k], inp, out,
                                          matrix_b=pids[k] if kb >= 0 else -1, nk=nk))
            lat = [srv.wait(t) for t in tickets]
        st = srv.stats()
    return lat, st


def test_same_alone_and_in_the_mix(library):
    mats, partners = library
    rng = np.random.default_rng(1)
    reqs = make_requests(rng, mats, partners, 60)
    run("batched", mats, partners, reqs)
    mixed = [r[3].clone() for r in reqs]
    for r in reqs:
        r[3].fill_(float("nan"))
    run("per_call", mats, partners, reqs)
    alone = [r[3].clone() for r in reqs]
    for a, b in zip(mixed, alone):
        assert torch.equal(a, b)  # bit-identical
    # and against the oracle
    for (op, k, inp, out, kb, nk), got in zip(reqs, mixed):
        ptr, idx, val = host_csr(mats[k])
        A = mats[k]
        if op == "spmv":
            want = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, val.astype(np.float64),
                                   inp.numpy().astype(np.float64))
            scale = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, np.abs(val).astype(np.float64),
                                    np.abs(inp.numpy()).astype(np.float64))
        elif op == "spmm":
            want = oracle.spmm_csr(A.nrows, A.ncols, ptr, idx, val.astype(np.float64),
                                   inp.numpy().astype(np.float64))
            scale = oracle.spmm_csr(A.nrows, A.ncols, ptr, idx, np.abs(val).astype(np.float64),
                                    np.abs(inp.numpy()).astype(np.float64))
        else:
            bp, bi, bv = host_csr(partners[k])
            Db = np.zeros((A.nrows, A.ncols))
            f = np.repeat(np.arange(A.nrows), np.diff(bp))
            Db[f, bi - 1] = bv
            fa = np.repeat(np.arange(A.nrows), np.diff(ptr))
            want = val.astype(np.float64) * Db[fa, idx - 1]
            scale = np.abs(want)
        assert (np.abs(got.numpy().astype(np.float64) - want) <= 2e-5 * scale + 1e-30).all()


def test_tuned_shapes_same_alone_and_in_the_mix(library):
    """The autotuner picks a shape per size class; both modes then compute
    every row at that shape, so results stay bit-identical between them and
    within the tolerance of the oracle."""
    mats, partners = library
    with Server(mode="batched") as srv:
        for A in mats + partners:
            srv.register(A)
        t = srv.tune(reps=2)
        shapes = Server.shapes(t)
    assert sum(x["matrices"] for x in shapes) == len(mats) + len(partners)
    for x in shapes:
        assert x["lanes"] in (2, 4, 8, 16, 32) and x["rows_per_item"] in (32, 64, 128, 256)
        assert 0 < x["ms"] and 0 < x["ms_default"]
    # and shapes unlike the default in every class, so each lane-group width runs
    forced = L.FgbServerTuning()
    for c in range(L.SERVER_CLASSES):
        forced.cls[c].lanes, forced.cls[c].rows_per_item = (2, 4, 8, 16)[c % 4], (32, 256)[c % 2]
    rng = np.random.default_rng(9)
    for tuning in (t, forced):
        reqs = make_requests(rng, mats, partners, 45)
        run("batched", mats, partners, reqs, tuning=tuning)
        mixed = [r[3].clone() for r in reqs]
        for r in reqs:
            r[3].fill_(float("nan"))
        run("per_call", mats, partners, reqs, tuning=tuning)
        for (op, k, inp, out, kb, nk), a in zip(reqs, mixed):
            assert torch.equal(a, out)
            if op == "spmv":
                ptr, idx, val = host_csr(mats[k])
                A = mats[k]
                want = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, val.astype(np.float64),
                                       inp.numpy().astype(np.float64))
                scale = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, np.abs(val).astype(np.float64),
                                        np.abs(inp.numpy()).astype(np.float64))
                assert (np.abs(a.numpy().astype(np.float64) - want) <= 2e-5 * scale + 1e-30).all()
    bad = L.FgbServerTuning()
    for c in range(L.SERVER_CLASSES):
        bad.cls[c].lanes, bad.cls[c].rows_per_item = 3, 64  # not a power of two
    with Server(mode="batched") as srv:
        with pytest.raises(L.FinchGBError) as e:
            srv.set_tuning(bad)
        assert e.value.status == L.EINVAL


def test_tune_edge_cases(library):
    """No matrices: every class empty, nothing changes.  A per-call server
    tunes too, and a matrix registered after tuning takes its class's
    shape."""
    mats, partners = library
    with Server(mode="batched") as srv:
        t = srv.tune(reps=1)
        assert all(c.matrices == 0 for c in t.cls) and Server.shapes(t) == []
    with Server(mode="per_call") as srv:
        ids = [srv.register(A) for A in mats[:4]]
        t = srv.tune(reps=1)
        assert sum(x["matrices"] for x in Server.shapes(t)) == 4
        late = srv.register(mats[4])  # registered after tuning: its class's tuned shape
        rng = np.random.default_rng(3)
        for k, mid in list(enumerate(ids)) + [(4, late)]:
            A = mats[k]
            x = torch.from_numpy(rng.standard_normal(A.ncols).astype(np.float32)).pin_memory()
            y = torch.empty(A.nrows, dtype=torch.float32).pin_memory()
            srv.wait(srv.submit("spmv", mid, x, y))
            ptr, idx, val = host_csr(A)
            want = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, val.astype(np.float64), x.numpy().astype(np.float64))
            scale = oracle.spmv_csr(0, A.nrows, A.ncols, ptr, idx, np.abs(val).astype(np.float64),
                                    np.abs(x.numpy()).astype(np.float64))
            assert (np.abs(y.numpy().astype(np.float64) - want) <= 2e-5 * scale + 1e-30).all()


def test_admission_queues_when_pool_is_small(library):
    mats, partners = library
    rng = np.random.default_rng(2)
    reqs = make_requests(rng, mats, partners, 30, pinned=False)
    need = max(r[3].numel() * 4 + (0 if r[2] is None else r[2].numel() * 4) for r in reqs)
    lat, st = run("batched", mats, partners, reqs, pool_bytes=2 * need + 4096, max_inflight=4)
    assert st["completed"] == 30 and st["pool_used"] == 0
    assert st["batches_published"] >= 8  # admitted a few at a time
    got = [r[3].clone() for r in reqs]
    for r in reqs:
        r[3].fill_(float("nan"))
    run("per_call", mats, partners, reqs)
    for a, r in zip(got, reqs):
        assert torch.equal(a, r[3])


def test_batch_submit_matches_single_submit(library):
    mats, partners = library
    rng = np.random.default_rng(3)
    reqs = make_requests(rng, mats, partners, 90)
    lat, st = run("batched", mats, partners, reqs, batch=True)
    assert st["completed"] == 90 and len(lat) == 90 and min(lat) >= 0
    got = [r[3].clone() for r in reqs]
    for r in reqs:
        r[3].fill_(float("nan"))
    run("batched", mats, partners, reqs)
    for a, r in zip(got, reqs):
        assert torch.equal(a, r[3])


def test_oversized_request_and_bad_ids(library):
    mats, partners = library
    with Server(pool_bytes=1 << 12) as srv:
        big = max(mats, key=lambda A: A.nrows)
        mid = srv.register(big)
        x = torch.zeros(big.ncols, dtype=torch.float32).pin_memory()
        y = torch.zeros(big.nrows, dtype=torch.float32).pin_memory()
        with pytest.raises(L.FinchGBError) as e:
            srv.submit("spmm", mid, torch.zeros((big.ncols, 128), dtype=torch.float32),
                       torch.zeros((big.nrows, 128), dtype=torch.float32), nk=128)
        assert e.value.status == L.ENOMEM
        with pytest.raises(L.FinchGBError) as e:
            srv.submit("spmv", mid + 7, x, y)
        assert e.value.status == L.EINVAL
        with pytest.raises(L.FinchGBError) as e:
            srv.submit("spmm", mid, x, y, nk=6)
        assert e.value.status == L.EUNSUPPORTED
        with pytest.raises(L.FinchGBError) as e:
            srv.wait(123456, timeout_ms=10)
        assert e.value.status == L.EINVAL


def test_device_loop_exits_when_idle_and_relaunches(library):
    mats, partners = library
    A = mats[0]
    with Server(idle_exit_us=2000) as srv:
        mid = srv.register(A)
        x = torch.ones(A.ncols, dtype=torch.float32).pin_memory()
        y1 = torch.empty(A.nrows, dtype=torch.float32).pin_memory()
        srv.wait(srv.submit("spmv", mid, x, y1))
        time.sleep(0.05)  # the loop exits after 2 ms without work
        y2 = torch.empty(A.nrows, dtype=torch.float32).pin_memory()
        srv.wait(srv.submit("spmv", mid, x, y2))
        assert torch.equal(y1, y2)
        assert srv.stats()["launches"] >= 2


def test_wait_is_bounded(library):
    mats, partners = library
    A = max(mats, key=lambda M: M.nnz)
    with Server() as srv:
        mid = srv.register(A)
        ts = []
        for _ in range(20):
            inp = torch.ones((A.ncols, 128), dtype=torch.float32).pin_memory()
            out = torch.empty((A.nrows, 128), dtype=torch.float32).pin_memory()
            ts.append(srv.submit("spmm", mid, inp, out, nk=128))
        try:
            srv.wait(ts[-1], timeout_ms=0)
        except L.FinchGBError as e:
            assert e.status == L.ETIMEOUT  # not done yet: a status, not a hang
        for t in ts[:-1]:
            srv.wait(t)
