"""Host logic for one process per GPU.

Every box in this build has one GPU, so the benchmark runs N independent
replicas (no data-path collective) and reports the whole job's throughput
over the slowest rank's time.  The same helpers shard one matrix by row
blocks balanced on rows + stored entries (the merge-path split of ptr), the
natural partition of SpMV/SpMM/SDDMM, and gather a row-sharded result.
"""
from __future__ import annotations

import os

import numpy as np


def rank_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def row_blocks(ptr: np.ndarray, nparts: int) -> np.ndarray:
    """Row boundaries b[0] = 0 <= ... <= b[nparts] = m cutting the CSR walk
    (m rows + nnz entries, ptr 1-based or 0-based) into nparts equal pieces."""
    ptr = np.asarray(ptr, dtype=np.int64)
    m = ptr.size - 1
    work = np.arange(m + 1, dtype=np.int64) + (ptr - ptr[0])  # rows + entries before row r
    targets = (np.arange(nparts + 1, dtype=np.float64) * work[-1] / nparts)
    b = np.searchsorted(work, targets, side="left").astype(np.int64)
    b[0], b[-1] = 0, m
    return np.maximum.accumulate(b)


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of a per-rank number (e.g. elapsed ms) over all ranks."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_rows(local: np.ndarray, blocks: np.ndarray) -> np.ndarray:
    """All ranks' row blocks of a result, concatenated in rank order."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size()
    width = int(np.max(np.diff(blocks)))
    buf = torch.zeros((width,) + local.shape[1:], dtype=torch.from_numpy(local[:0]).dtype)
    buf[: local.shape[0]] = torch.from_numpy(np.ascontiguousarray(local))
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf)
    return np.concatenate([parts[r][: blocks[r + 1] - blocks[r]].numpy() for r in range(world)])
