"""Calls from several host threads at once.  Finch calls can arrive from any
Julia task or thread.  The tests cover three cases:
- per-call kernels, each thread on its own stream;
- plans built and run from several threads, which share the autotuning
  cache;
- concurrent submits to one server.
Every result must equal the same call made alone.  ctypes releases the
interpreter lock around each library call, so the threads really are inside
the library together."""
import threading

import numpy as np
import pytest
import torch

from finchgb import device as dev
from finchgb.plan import Plan
from finchgb.server import Server, random_csr
from finchgb.workloads import SparseBuffers, zipf_csr
from helpers import upload

pytestmark = pytest.mark.gpu

THREADS = 4


def run_threads(fns):
    results, errors = [None] * len(fns), []

    def wrap(k, fn):
        try:
            results[k] = fn()
        except BaseException as e:  # re-raised in the main thread
            errors.append(e)

    ts = [threading.Thread(target=wrap, args=(k, f)) for k, f in enumerate(fns)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in ts)
    if errors:
        raise errors[0]
    return results


def small_int_csr(seed, m, n):
    """Zipf row lengths with small integer values: every FP32 sum of a few
    thousand such products is exact, so any schedule gives the same bits."""
    b = zipf_csr(np.random.default_rng(seed), m, n, mean=8.0, a=1.5, cap=400, dtype=np.float32)
    vals = np.random.default_rng(seed + 1).integers(-3, 4, b.nnz).astype(np.float32)
    return SparseBuffers(b.nrows, b.ncols, b.ptr, b.idx, vals, b.orient)


def int_tensor(seed, shape):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randint(-3, 4, shape, generator=g).to(torch.float32).cuda()


def test_per_call_kernels_from_threads(gpu_lib):
    A = upload(small_int_csr(11, 30_000, 30_000))
    xs = [int_tensor(k, (30_000,)) for k in range(THREADS)]
    Bs = [int_tensor(10 + k, (30_000, 32)) for k in range(THREADS)]
    Xs = [int_tensor(20 + k, (30_000, 16)) for k in range(THREADS)]
    Ys = [int_tensor(30 + k, (30_000, 16)) for k in range(THREADS)]
    want = [(dev.spmv(A, xs[k]).cpu(), dev.spmm(A, Bs[k]).cpu(), dev.sddmm(A, Xs[k], Ys[k]).cpu())
            for k in range(THREADS)]
    torch.cuda.synchronize()

    def work(k):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            for _ in range(8):
                out = (dev.spmv(A, xs[k]), dev.spmm(A, Bs[k]), dev.sddmm(A, Xs[k], Ys[k]))
            s.synchronize()
            return tuple(o.cpu() for o in out)

    got = run_threads([lambda k=k: work(k) for k in range(THREADS)])
    for g, w in zip(got, want):
        for a, b in zip(g, w):
            assert torch.equal(a, b)


def test_plans_built_and_run_from_threads(gpu_lib):
    A = upload(small_int_csr(12, 40_000, 40_000))
    B = int_tensor(40, (40_000, 64))
    want = dev.spmm(A, B).cpu()
    torch.cuda.synchronize()

    def work(k):
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            C = torch.empty((40_000, 64), dtype=torch.float32, device="cuda")
            p = Plan.spmm(A, B, C, tune_reps=1)
            for _ in range(4):
                C.zero_()
                p.execute()
            s.synchronize()
            return C.cpu()

    for got in run_threads([lambda k=k: work(k) for k in range(THREADS)]):
        assert torch.equal(got, want)


def test_server_submits_from_threads(gpu_lib):
    mats = [random_csr(300 + k, 512 + 64 * k, 512 + 64 * k, 0.02) for k in range(6)]
    rng = np.random.default_rng(5)
    jobs = []  # per thread: (op, matrix, input, output, nk)
    for t in range(THREADS):
        mine = []
        for r in range(40):
            k = int(rng.integers(len(mats)))
            A = mats[k]
            if r % 2:
                inp = torch.from_numpy(rng.standard_normal((A.ncols, 16)).astype(np.float32)).pin_memory()
                mine.append(("spmm", k, inp, torch.empty((A.nrows, 16)).pin_memory(), 16))
            else:
                inp = torch.from_numpy(rng.standard_normal(A.ncols).astype(np.float32)).pin_memory()
                mine.append(("spmv", k, inp, torch.empty(A.nrows).pin_memory(), 0))
        jobs.append(mine)
    with Server(mode="per_call") as srv:  # reference: one request at a time
        ids = [srv.register(A) for A in mats]
        for mine in jobs:
            for op, k, inp, out, nk in mine:
                srv.wait(srv.submit(op, ids[k], inp, out, nk=nk))
    want = [[out.clone() for *_, out, _nk in mine] for mine in jobs]
    for mine in jobs:
        for *_, out, _nk in mine:
            out.fill_(float("nan"))
    with Server(mode="batched") as srv:
        ids = [srv.register(A) for A in mats]

        def work(t):
            tickets = [srv.submit(op, ids[k], inp, out, nk=nk) for op, k, inp, out, nk in jobs[t]]
            for tk in tickets:
                srv.wait(tk)
            return len(tickets)

        assert run_threads([lambda t=t: work(t) for t in range(THREADS)]) == [40] * THREADS
    for mine, w in zip(jobs, want):
        for (*_, out, _nk), ref in zip(mine, w):
            assert torch.equal(out, ref)  # bit-identical to the request alone
