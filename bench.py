"""Benchmark of the GB300 SpMM path on the 1M x 1M power-law configuration.

Workload (one step = one SpMM C = A @ B over the whole matrix):
  A: 1,000,000 x 1,000,000 CSR, Zipf(1.5) row lengths capped at 50,000 and
     rescaled to exactly 16,000,000 stored entries; columns uniform; FP32
     values N(0,1).  B: 1,000,000 x 128 FP32 N(0,1), row-major.  Seeded.
Metric: algorithmic HBM bytes per step (A ptr+idx+val, B, C once each)
divided by time, in GB/s, and that figure against the measured HBM peak.

Arms:
  default            the CUDA path; `value` = device-resident inputs,
                     `e2e` = host buffers through the C ABI (pinned H2D of
                     A and B with fgb_upload, fgb_spmm_ex, D2H of C with
                     fgb_download, all inside the timed region).
  --impl reference   Finch's CPU nest (the oracle's C restatement, all host
                     threads) over the same matrix.

The schedule (lanes per row group = column slab, merge-path item length) is
picked by a short autotune on the same inputs before the timed region.

Multi-GPU (torchrun): replicas -- every rank runs the same workload on its
own GPU, no data-path collective; value = all ranks' bytes / max time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "finch.jl_gb300"))
sys.path.insert(0, str(ROOT))

NNZ_MEAN = 16.0
NK = 128
SEED = 20261203


def workload_name(rows: int) -> str:
    return f"spmm_csr_zipf1.5_{rows // 1000}Kx{rows // 1000}K_nnz{int(rows * NNZ_MEAN) // 1000}K_k{NK}_fp32"


def algorithmic_bytes(nrows: int, nnz: int, nk: int, ncols_b: int, ptr_bytes: int = 4) -> int:
    """A ptr + idx (int32) + val (fp32), B (ncols_b x nk), C (nrows x nk), each once."""
    return ptr_bytes * (nrows + 1) + 8 * nnz + 4 * ncols_b * nk + 4 * nrows * nk


def make_inputs(rows: int):
    from finchgb.workloads import zipf_csr

    rng = np.random.default_rng(SEED)
    A = zipf_csr(rng, rows, rows, mean=NNZ_MEAN, a=1.5, cap=50_000, dtype=np.float32)
    B = rng.standard_normal((rows, NK), dtype=np.float32)
    return A, B


def load_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic() -> tuple[int | None, str | None]:
    """Per-step DRAM bytes of the SpMM kernels from the committed ncu summary."""
    p = ROOT / "profiles" / "spmm_merge_zipf1M_k128.md"
    if not p.exists():
        return None, None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_step:"):
            return int(float(line.split(":", 1)[1].strip())), str(p.relative_to(ROOT))
    return None, None


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = ""

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
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons, "samples": len(rows)}


def dist_setup():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def cpu_reference_pass(A, B, threads: int) -> float:
    """One pass of Finch's row-parallel CPU SpMM nest over the whole matrix."""
    import oracle

    C = np.empty((A.nrows, NK), dtype=np.float32)
    t0 = time.perf_counter()
    oracle.spmm_csr(A.nrows, A.ncols, A.ptr, A.idx, A.val, B, C=C, nthreads=threads)
    return time.perf_counter() - t0


def cpu_baseline(A, B, nbytes: int, min_seconds: float = 10.0, max_passes: int = 30) -> dict:
    import oracle

    threads = oracle.max_threads()
    cpu_reference_pass(A, B, threads)  # warm caches and page in
    times = []
    while sum(times) < min_seconds and len(times) < max_passes:
        times.append(cpu_reference_pass(A, B, threads))
    t = statistics.median(times)
    return {"value": round(nbytes / t / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"whole matrix, {len(times)} passes ({sum(times):.1f} s) of Finch's "
                      f"row-parallel SpMM nest (oracle C restatement, static split), median "
                      f"{1e3 * t:.1f} ms"}


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle

    A, B = make_inputs(args.rows)
    threads = oracle.max_threads()
    nbytes = algorithmic_bytes(A.nrows, A.nnz, NK, A.ncols)
    for _ in range(max(args.warmup, 0)):
        cpu_reference_pass(A, B, threads)
    times = [cpu_reference_pass(A, B, threads) for _ in range(args.steps)]
    total = sum(times)
    value = nbytes * args.steps / total / 1e9
    line = {"impl": "reference", "metric": "spmm_gbps_algorithmic", "value": round(value, 3),
            "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * total / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": workload_name(args.rows), "parallelism": f"cpu{threads}"},
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                             "kind": "port",
                             "sample": "whole matrix per step: Finch's row-parallel SpMM nest "
                                       "(oracle C restatement, static split)"},
            "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def autotune(A, B, C, reps: int = 3, verbose: bool = False):
    """Times each (lanes, path) schedule on the real inputs; returns the best
    and the table (ms per SpMM)."""
    import torch

    from finchgb import device as dev

    table = {}
    for lanes in (2, 4, 8, 16, 32):
        for path in (128, 256, 512, 1024):
            dev.spmm(A, B, C, lanes=lanes, path=path)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(reps):
                dev.spmm(A, B, C, lanes=lanes, path=path)
            e1.record()
            torch.cuda.synchronize()
            table[(lanes, path)] = e0.elapsed_time(e1) / reps
            if verbose:
                print(f"  lanes={lanes:2d} path={path:5d}: {table[(lanes, path)]:.3f} ms",
                      file=sys.stderr)
    best = min(table, key=table.get)
    return best, table


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
    A_h, B_h = make_inputs(args.rows)
    M = A_h.nrows
    nbytes = algorithmic_bytes(M, A_h.nnz, NK, A_h.ncols)

    # ---- value: device-resident inputs
    A = dev.DeviceSparse.from_host(A_h.nrows, A_h.ncols, A_h.ptr, A_h.idx, A_h.val, orient="csr")
    B = torch.from_numpy(B_h).to(device)
    C = torch.empty((M, NK), dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream()
    if args.schedule:
        lanes, path = (int(v) for v in args.schedule.split(","))
        table = {}
    else:
        (lanes, path), table = autotune(A, B, C, verbose=args.sweep)
    slabs = -(-NK // (4 * lanes))
    launches_per_step = 1 + slabs + 1  # merge plan + one launch per slab + carry fix-up

    def step():
        dev.spmm(A, B, C, lanes=lanes, path=path)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    warmup = max(args.warmup, 3)
    for _ in range(warmup):
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
    step_ms = [a.elapsed_time(b) for a, b in ev]
    if world > 1:
        t = torch.tensor([total_ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nbytes * args.steps * world / (total_ms / 1e3) / 1e9

    line = {"metric": "spmm_gbps_algorithmic", "value": round(value, 1), "unit": "GB/s",
            "n_gpus": world, "steps": args.steps, "warmup": warmup,
            "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded PCG64)",
            "config": {"workload": workload_name(args.rows), "nnz": int(A_h.nnz), "k": NK,
                       "algorithmic_bytes_per_step": nbytes,
                       "schedule": {"lanes": lanes, "column_slab": 4 * lanes,
                                    "merge_path_item": path,
                                    "autotune_ms": {f"{k[0]}x{k[1]}": round(v, 4)
                                                    for k, v in table.items()}},
                       "l2": "inputs larger than L2 (1.16 GB per step vs 129 MB)",
                       "parallelism": f"replicas{world}"},
            "gpu_launches": args.steps * launches_per_step}

    # ---- e2e: host buffers through the C ABI -> host result
    if not args.no_e2e:
        ctx = dev.context()
        lib = L.load()
        ptr32 = torch.from_numpy(A_h.ptr.astype(np.int32)).pin_memory()
        idx32 = torch.from_numpy(A_h.idx.astype(np.int32)).pin_memory()
        val_h = torch.from_numpy(A_h.val).pin_memory()
        B_pin = torch.from_numpy(B_h).pin_memory()
        C_pin = torch.empty((M, NK), dtype=torch.float32).pin_memory()
        d_ptr = torch.empty(ptr32.shape, dtype=torch.int32, device=device)
        d_idx = torch.empty(idx32.shape, dtype=torch.int32, device=device)
        d_val = torch.empty(val_h.shape, dtype=torch.float32, device=device)
        d_B = torch.empty(B_pin.shape, dtype=torch.float32, device=device)
        d_C = torch.empty((M, NK), dtype=torch.float32, device=device)
        A_e = dev.DeviceSparse(M, A_h.ncols, d_ptr, d_idx, d_val, "csr", 1)
        desc = A_e.desc()
        tune = L.FgbSpmmTuning(lanes, 0, path)
        h2d_pairs = [(d_ptr, ptr32), (d_idx, idx32), (d_val, val_h), (d_B, B_pin)]
        h2d = sum(h.numel() * h.element_size() for _, h in h2d_pairs)
        d2h = C_pin.numel() * C_pin.element_size()

        def e2e_step():
            s = dev.stream_ptr()
            for d, h in h2d_pairs:
                L.check(lib.fgb_upload(ctx, d.data_ptr(), h.data_ptr(), h.numel() * h.element_size(), s))
            L.check(lib.fgb_spmm_ex(ctx, ctypes.byref(desc), d_B.data_ptr(), NK, NK, d_C.data_ptr(),
                                    NK, L.F32, 0, ctypes.byref(tune), s))
            L.check(lib.fgb_download(ctx, C_pin.data_ptr(), d_C.data_ptr(), d2h, s))

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
        ok = bool(np.array_equal(C_pin[:2000].numpy(), C[:2000].cpu().numpy()))
        line["e2e"] = {"value": round(nbytes * e2e_steps * world / (e2e_ms / 1e3) / 1e9, 1),
                       "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "steps": e2e_steps, "ms_per_step": round(e2e_ms / e2e_steps, 3),
                       "result_matches_device_run": ok}
        line["gpu_launches"] += (e2e_steps) * launches_per_step

    # ---- roofline of the SpMM (plan + per-slab merge kernels + fix-up)
    peak, peak_kind = load_peaks()
    avg_ms = sum(step_ms) / len(step_ms)
    achieved = nbytes / (avg_ms / 1e3) / 1e9
    traffic, traffic_src = load_traffic()
    line["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(achieved / peak, 4),
                        "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                        "traffic": traffic, "traffic_source": traffic_src,
                        "kernel": f"spmm_merge_k x{slabs} slabs + merge_plan_k + spmm_fixup_k",
                        "algorithmic_bytes_per_launch": nbytes,
                        "avg_launch_ms": round(avg_ms, 4)}
    line["cpu_baseline"] = None
    if rank == 0 and not args.skip_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(A_h, B_h, nbytes)
    line["clocks"] = clk.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rows", type=int, default=1_000_000,
                    help="rows = columns of A (16 stored entries per row on average)")
    ap.add_argument("--skip-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--sweep", action="store_true", help="print the autotune table to stderr")
    ap.add_argument("--schedule", default="", help="fixed LANES,PATH instead of the autotune")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
