"""N > 1 host logic on CPU: world-size-2 gloo ranks (one process each,
127.0.0.1 rendezvous).  Each rank computes its nnz-balanced row block of a
CSR SpMV with the oracle, the blocks are gathered, and the per-rank timing
is reduced to the maximum -- what a row-sharded multi-GPU run does around
its kernels."""
import os
import socket

import numpy as np
import pytest

from finchgb.replicas import row_blocks
from finchgb.workloads import zipf_csr


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    import oracle
    from finchgb.replicas import gather_rows, max_over_ranks, row_blocks

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(12)
        A = zipf_csr(rng, 5000, 4000, mean=12, cap=2000, dtype=np.float64)
        x = rng.standard_normal(4000)
        b = row_blocks(A.ptr, world)
        lo, hi = int(b[rank]), int(b[rank + 1])
        ptr = A.ptr[lo:hi + 1] - A.ptr[lo] + 1
        idx = A.idx[A.ptr[lo] - 1:A.ptr[hi] - 1]
        val = A.val[A.ptr[lo] - 1:A.ptr[hi] - 1]
        y = oracle.spmv_csr(0, hi - lo, A.ncols, ptr, idx, val, x)
        full = gather_rows(y, b)
        t = max_over_ranks(10.0 * (rank + 1))
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.r_[full, t])
    finally:
        dist.destroy_process_group()


def test_row_blocks_balance():
    rng = np.random.default_rng(1)
    A = zipf_csr(rng, 20000, 20000, mean=16, cap=5000)
    for parts in (1, 2, 3, 8):
        b = row_blocks(A.ptr, parts)
        assert b[0] == 0 and b[-1] == A.nrows and np.all(np.diff(b) >= 0)
        work = np.diff(b) + np.diff(A.ptr[b])
        total = A.nrows + A.nnz
        # every block holds its share of rows + entries, give or take one row
        assert work.max() <= total / parts + A.ptr[1:].__sub__(A.ptr[:-1]).max() + 1


def test_two_gloo_ranks_shard_and_gather(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import oracle

    world = 2
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    rng = np.random.default_rng(12)
    A = zipf_csr(rng, 5000, 4000, mean=12, cap=2000, dtype=np.float64)
    x = rng.standard_normal(4000)
    want = oracle.spmv_csr(0, A.nrows, A.ncols, A.ptr, A.idx, A.val, x)
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert np.array_equal(got[:-1], want)  # the same row order of sums as unsharded
        assert got[-1] == 20.0  # max over ranks
