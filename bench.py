"""Benchmark of the GB300 SpMM path on the 1M x 1M power-law configuration.

Workload (one step = one SpMM C = A @ B over the whole matrix):
  A: 1,000,000 x 1,000,000 CSR, Zipf(1.5) row lengths capped at 50,000 and
     rescaled to exactly 16,000,000 stored entries; columns uniform; FP32
     values N(0,1).  B: 1,000,000 x 128 FP32 N(0,1), row-major.  Seeded.
Metric: algorithmic HBM bytes per step (A ptr+idx+val, B, C once each)
divided by time, in GB/s, and that figure against the measured HBM peak.

Arms:
  default            the CUDA path; `value` = device-resident inputs,
                     `e2e` = host buffers through the public API (pinned H2D
                     of A and B, SpMM, D2H of C inside the timed region).
  --impl reference   Finch's CPU nest (the oracle's C restatement, all host
                     threads) on a bounded row sample of the same workload.

Multi-GPU (torchrun): replicas -- every rank runs the same workload on its
own GPU, no data-path collective; value = all ranks' bytes / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "finch.jl_gb300"))
sys.path.insert(0, str(ROOT))

M = N_COLS = 1_000_000
NNZ_MEAN = 16.0
NK = 128
SEED = 20261203
WORKLOAD = "spmm_csr_zipf1.5_1Mx1M_nnz16M_k128_fp32"


def algorithmic_bytes(nrows: int, nnz: int, nk: int, ncols_b: int, ptr_bytes: int = 4) -> int:
    """A ptr + idx (int32) + val (fp32), B (ncols_b x nk), C (nrows x nk), each once."""
    return ptr_bytes * (nrows + 1) + 8 * nnz + 4 * ncols_b * nk + 4 * nrows * nk


def make_inputs():
    from finchgb.workloads import zipf_csr

    rng = np.random.default_rng(SEED)
    A = zipf_csr(rng, M, N_COLS, mean=NNZ_MEAN, a=1.5, cap=50_000, dtype=np.float32)
    B = rng.standard_normal((N_COLS, NK), dtype=np.float32)
    return A, B


def load_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic() -> int | None:
    """Per-launch DRAM bytes of the SpMM kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "spmm_csr_pull_zipf1M_k128.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return int(float(line.split(":", 1)[1].strip()))
    return None


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 6:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[2:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k, v in enumerate(r) if v == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_reference_run(A, B, rows: int, threads: int) -> tuple[float, float]:
    """Finch's row-parallel CPU nest over the first `rows` rows of A.

    Returns (seconds for the sample, seconds scaled to the whole matrix by
    the fraction of stored entries the sample holds)."""
    import oracle

    p = A.ptr[: rows + 1]
    nnz = int(p[-1] - 1)
    idx = A.idx[:nnz]
    val = A.val[:nnz]
    C = np.empty((rows, NK), dtype=np.float32)
    t0 = time.perf_counter()
    oracle.spmm_csr(rows, A.ncols, p, idx, val, B, C=C, nthreads=threads)
    dt = time.perf_counter() - t0
    return dt, dt * (A.nnz / max(nnz, 1))


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle

    A, B = make_inputs()
    threads = oracle.max_threads()
    rows = 100_000  # bounded sample: ~10% of the rows
    for _ in range(max(args.warmup, 0)):
        cpu_reference_run(A, B, rows // 10, threads)
    nbytes = algorithmic_bytes(M, A.nnz, NK, N_COLS)
    times, full = [], []
    for _ in range(args.steps):
        dt, dt_full = cpu_reference_run(A, B, rows, threads)
        times.append(dt)
        full.append(dt_full)
    total = sum(full)
    value = nbytes * args.steps / total / 1e9
    line = {"impl": "reference", "metric": "spmm_gbps_algorithmic", "value": round(value, 3),
            "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
            "sample_ms_per_step": round(1e3 * sum(times) / args.steps, 3),
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "sample": f"first {rows} of {M} rows",
                       "parallelism": f"cpu{threads}"},
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                             "kind": "port",
                             "sample": f"Finch's row-parallel SpMM nest (oracle C restatement, "
                                       f"static split) over rows 1..{rows} of A; time scaled "
                                       f"to the whole matrix by stored entries"},
            "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = torch.device("cuda", torch.cuda.current_device())
    from finchgb import _lib as L
    from finchgb import build
    from finchgb import device as dev

    build.build()
    A_h, B_h = make_inputs()
    nbytes = algorithmic_bytes(M, A_h.nnz, NK, N_COLS)

    # ---- value: device-resident inputs
    A = dev.DeviceSparse.from_host(A_h.nrows, A_h.ncols, A_h.ptr, A_h.idx, A_h.val, orient="csr")
    B = torch.from_numpy(B_h).to(device)
    C = torch.empty((M, NK), dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream()

    def step():
        dev.spmm(A, B, C)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    with ClockSampler(device.index) as clk:
        barrier()
        t_start.record(stream)
        for k in range(args.steps):
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        t_end.record(stream)
        barrier()
    total_ms = t_start.elapsed_time(t_end)
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    if world > 1:
        t = torch.tensor([total_ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nbytes * args.steps * world / (total_ms / 1e3) / 1e9

    # ---- e2e: host buffers -> public API -> host result
    ptr32 = torch.from_numpy(A_h.ptr.astype(np.int32)).pin_memory()
    idx32 = torch.from_numpy(A_h.idx.astype(np.int32)).pin_memory()
    val_h = torch.from_numpy(A_h.val).pin_memory()
    B_pin = torch.from_numpy(B_h).pin_memory()
    C_pin = torch.empty((M, NK), dtype=torch.float32).pin_memory()
    d_ptr = torch.empty_like(ptr32, device=device)
    d_idx = torch.empty_like(idx32, device=device)
    d_val = torch.empty_like(val_h, device=device)
    d_B = torch.empty_like(B_pin, device=device)
    d_C = torch.empty((M, NK), dtype=torch.float32, device=device)
    A_e = dev.DeviceSparse(M, N_COLS, d_ptr, d_idx, d_val, "csr", 1)
    h2d = sum(t.numel() * t.element_size() for t in (ptr32, idx32, val_h, B_pin))
    d2h = C_pin.numel() * C_pin.element_size()

    def e2e_step():
        d_ptr.copy_(ptr32, non_blocking=True)
        d_idx.copy_(idx32, non_blocking=True)
        d_val.copy_(val_h, non_blocking=True)
        d_B.copy_(B_pin, non_blocking=True)
        dev.spmm(A_e, d_B, d_C)
        C_pin.copy_(d_C, non_blocking=True)

    for _ in range(3):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_steps = max(3, args.steps // 4)
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([e2e_ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = nbytes * e2e_steps * world / (e2e_ms / 1e3) / 1e9
    ok = np.allclose(C_pin[:1000].numpy(), C[:1000].cpu().numpy(), rtol=0, atol=0)

    # ---- roofline of the dominant kernel (one SpMM launch per step)
    peak, peak_kind = load_peaks()
    avg_kernel_ms = sum(kernel_ms) / len(kernel_ms)
    achieved = nbytes / (avg_kernel_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": load_traffic(), "kernel": "spmm_csr_pull<float,float,int,32,4>",
                "algorithmic_bytes_per_launch": nbytes}

    cpu_base = None
    if rank == 0 and not args.skip_cpu_baseline:
        import oracle

        threads = oracle.max_threads()
        rows = 60_000
        dt, dt_full = cpu_reference_run(A_h, B_h, rows, threads)
        cpu_base = {"value": round(nbytes / dt_full / 1e9, 3), "unit": "GB/s", "cores": threads,
                    "kind": "port",
                    "sample": f"Finch's row-parallel SpMM nest (oracle C restatement) over rows "
                              f"1..{rows} of A, {threads} threads, {dt:.2f} s; time scaled to "
                              f"the whole matrix by stored entries"}

    if rank == 0:
        line = {"metric": "spmm_gbps_algorithmic", "value": round(value, 1), "unit": "GB/s",
                "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded PCG64)",
                "config": {"workload": WORKLOAD, "nnz": int(A_h.nnz), "k": NK,
                           "algorithmic_bytes_per_step": nbytes,
                           "l2": "inputs larger than L2 (1.16 GB per step vs 129 MB)",
                           "parallelism": f"replicas{world}"},
                "e2e": {"value": round(e2e_value, 1), "unit": "GB/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "steps": e2e_steps,
                        "ms_per_step": round(e2e_ms / e2e_steps, 3), "result_matches": bool(ok)},
                "roofline": roofline, "cpu_baseline": cpu_base,
                "gpu_launches": args.steps, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
