"""Serving compute() calls on resident tensors with continuous batching.

`Server` wraps fgb_server_*: matrices are registered once and stay in HBM;
requests (SpMV, SpMM, masked elementwise multiply on a resident matrix)
are admitted by HBM footprint and run either by the persistent device loop
(mode "batched") or one launch at a time (mode "per_call", the plain GPU
path).  Both modes compute every row the same way, so results are
bit-identical between them.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib as L
from . import device as dev

OPS = {"spmv": L.REQ_SPMV, "spmm": L.REQ_SPMM, "masked_mul": L.REQ_MASKED_MUL}


def random_csr(seed: int, m: int, n: int, p: float, device: int | None = None) -> dev.DeviceSparse:
    """fsprand-distributed m x n CSR generated on the device (FP32 N(0,1))."""
    ctx = dev.context(device)
    d = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    ptr = torch.empty(m + 1, dtype=torch.int32, device=d)
    nnz = ctypes.c_int64()
    L.call("fgb_random_csr", ctx, seed, m, n, p, L.F32, ptr.data_ptr(), None, None,
           ctypes.byref(nnz), dev.stream_ptr())
    idx = torch.empty(max(nnz.value, 1), dtype=torch.int32, device=d)[: nnz.value]
    val = torch.empty(max(nnz.value, 1), dtype=torch.float32, device=d)[: nnz.value]
    L.call("fgb_random_csr", ctx, seed, m, n, p, L.F32, ptr.data_ptr(),
           idx.data_ptr() if nnz.value else 1, val.data_ptr() if nnz.value else 1,
           ctypes.byref(nnz), dev.stream_ptr())
    return dev.DeviceSparse(m, n, ptr, idx, val, "csr", 0)


class Server:
    def __init__(self, pool_bytes: int = 1 << 30, max_inflight: int = 1024,
                 rows_per_item: int = 64, blocks_per_sm: int = 4, idle_exit_us: int = 20000,
                 mode: str = "batched", device: int | None = None):
        self.ctx = dev.context(device)
        cfg = L.FgbServerConfig(pool_bytes, max_inflight, rows_per_item, blocks_per_sm,
                                idle_exit_us, L.SERVE_BATCHED if mode == "batched" else L.SERVE_PER_CALL,
                                0)
        h = ctypes.c_void_p()
        L.call("fgb_server_create", self.ctx, ctypes.byref(cfg), ctypes.byref(h))
        self.h = h
        self.lib = L.load()
        self.matrices: list[dev.DeviceSparse] = []
        self._pending: dict[int, tuple] = {}

    def register(self, A: dev.DeviceSparse) -> int:
        """Registers a resident CSR (int32 ptr/idx, FP32 values); returns its id."""
        mid = ctypes.c_int32()
        d = A.desc()
        L.call("fgb_server_register", self.h, ctypes.byref(d), ctypes.byref(mid))
        self.matrices.append(A)
        return mid.value

    def submit(self, op: str, matrix: int, inp: np.ndarray | torch.Tensor | None,
               out: np.ndarray | torch.Tensor, matrix_b: int = -1, nk: int = 0) -> int:
        """Queues a request on host buffers (pinned torch tensors are fastest)."""
        req = L.FgbRequest(OPS[op], matrix, matrix_b, nk, _hptr(inp), _hptr(out))
        t = ctypes.c_uint64()
        rc = self.lib.fgb_server_submit(self.h, ctypes.byref(req), ctypes.byref(t))
        L.check(rc, "fgb_server_submit")
        self._pending[t.value] = (inp, out)  # keep the buffers alive
        return t.value

    @staticmethod
    def request(op: str, matrix: int, inp, out, matrix_b: int = -1, nk: int = 0) -> L.FgbRequest:
        return L.FgbRequest(OPS[op], matrix, matrix_b, nk, _hptr(inp), _hptr(out))

    def submit_batch(self, reqs) -> list[int]:
        """Queues a ctypes array (or list) of FgbRequest under one lock."""
        n = len(reqs)
        arr = reqs if isinstance(reqs, ctypes.Array) else (L.FgbRequest * n)(*reqs)
        tickets = (ctypes.c_uint64 * n)()
        acc = ctypes.c_int32()
        rc = self.lib.fgb_server_submit_batch(self.h, arr, n, tickets, ctypes.byref(acc))
        L.check(rc, "fgb_server_submit_batch")
        return list(tickets)

    def wait_batch(self, tickets, timeout_ms: int = 60_000) -> list[float]:
        n = len(tickets)
        t = (ctypes.c_uint64 * n)(*tickets)
        lat = (ctypes.c_double * n)()
        rc = self.lib.fgb_server_wait_batch(self.h, t, n, timeout_ms, lat)
        L.check(rc, "fgb_server_wait_batch")
        for x in tickets:
            self._pending.pop(x, None)
        return list(lat)

    def wait(self, ticket: int, timeout_ms: int = 60_000) -> float:
        """Waits for a ticket; returns its submit-to-result latency in seconds."""
        lat = ctypes.c_double()
        rc = self.lib.fgb_server_wait(self.h, ticket, timeout_ms, ctypes.byref(lat))
        if rc != L.ETIMEOUT:
            self._pending.pop(ticket, None)
        L.check(rc, "fgb_server_wait")
        return lat.value

    def tune(self, reps: int = 3) -> L.FgbServerTuning:
        """Runs the serving autotuner (fgb_server_tune) on the registered
        matrices and applies its choice; returns the per-class shapes."""
        t = L.FgbServerTuning()
        L.call("fgb_server_tune", self.h, reps, ctypes.byref(t))
        return t

    def set_tuning(self, t: L.FgbServerTuning):
        """Applies per-class shapes (e.g. another server's tune() result)."""
        L.call("fgb_server_set_tuning", self.h, ctypes.byref(t))

    @staticmethod
    def shapes(t: L.FgbServerTuning) -> list[dict]:
        return [{"class": c, "matrices": x.matrices, "lanes": x.lanes, "rows_per_item": x.rows_per_item,
                 "ms": round(x.ms, 4), "ms_default": round(x.ms_default, 4)}
                for c, x in enumerate(t.cls) if x.matrices > 0]

    def stats(self) -> dict:
        s = L.FgbServerStats()
        L.call("fgb_server_stats_get", self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in L.FgbServerStats._fields_}

    def close(self):
        if self.h:
            L.call("fgb_server_destroy", self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _hptr(a):
    if a is None:
        return None
    if isinstance(a, torch.Tensor):
        assert a.device.type == "cpu" and a.is_contiguous()
        return a.data_ptr()
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data
