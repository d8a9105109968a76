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
NSETS = 2  # e2e pipeline depth (3 measured no faster): buffer sets (device A, B, C and page-locked C) in rotation
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


def load_traffic(schedule: str) -> tuple[int | None, str | None]:
    """Per-step DRAM bytes of the SpMM kernels from the committed ncu summary
    of the same schedule (None when the run chose a schedule no summary
    covers).  `schedule` is "lanes=L path=T variant=V bands=P"."""
    for p in sorted((ROOT / "profiles").glob("spmm_*zipf1M_k128*.md")):
        lines = p.read_text().splitlines()
        sched = [ln.split(":", 1)[1].strip() for ln in lines if ln.startswith("schedule:")]
        if not sched or sched[0] != schedule:
            continue
        for line in lines:
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
    from finchgb.replicas import rank_env

    return rank_env()


def cpu_reference_pass(A, B, threads: int) -> float:
    """One pass of Finch's row-parallel CPU SpMM nest over the whole matrix."""
    import oracle

    C = np.empty((A.nrows, NK), dtype=np.float32)
    t0 = time.perf_counter()
    oracle.spmm_csr(A.nrows, A.ncols, A.ptr, A.idx, A.val, B, C=C, nthreads=threads, fast=True)
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
                      f"row-parallel SpMM nest (oracle C restatement, static split, built "
                      f"-O3 -ffast-math -funroll-loops), median {1e3 * t:.1f} ms"}


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
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64)",
            "config": {"workload": workload_name(args.rows), "nnz": int(A.nnz), "k": NK,
                       "algorithmic_bytes_per_step": nbytes, "parallelism": f"cpu{threads}"},
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                             "kind": "port",
                             "sample": "whole matrix per step: Finch's row-parallel SpMM nest "
                                       "(oracle C restatement, static split, built -O3 -ffast-math "
                                       "-funroll-loops)"},
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


def rows_of(A, rows: np.ndarray):
    """The CSR sub-matrix of the given rows (host, 1-based buffers)."""
    from finchgb.workloads import SparseBuffers

    lens = (A.ptr[rows + 1] - A.ptr[rows]).astype(np.int64)
    ptr = np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int64)
    sel = np.concatenate([np.arange(A.ptr[r] - 1, A.ptr[r + 1] - 1) for r in rows])
    return SparseBuffers(len(rows), A.ncols, ptr, A.idx[sel], A.val[sel], "csr")


def spmm_fp64_error(A_h, B_h, C_host: np.ndarray, n: int = 4000, longest: int = 20) -> dict:
    """max |gpu - FP64 oracle| / sum_j |A[i,j] B[j,k]| over sampled rows of C
    (the longest rows included), every column."""
    import oracle

    lens = np.diff(A_h.ptr)
    rng = np.random.default_rng(SEED + 99)
    rows = np.unique(np.concatenate([rng.choice(A_h.nrows, n, replace=False), np.argsort(lens)[-longest:]]))
    sub = rows_of(A_h, rows)
    nt = oracle.max_threads()
    B64 = B_h.astype(np.float64)
    want = oracle.spmm_csr(sub.nrows, sub.ncols, sub.ptr, sub.idx, sub.val.astype(np.float64), B64, nthreads=nt)
    scale = oracle.spmm_csr(sub.nrows, sub.ncols, sub.ptr, sub.idx, np.abs(sub.val).astype(np.float64),
                            np.abs(B64), nthreads=nt)
    err = np.abs(C_host[rows].astype(np.float64) - want)
    rel = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0), np.where(err > 0, np.inf, 0.0))
    return {"max_rel_err_vs_fp64": float(rel.max()), "tolerance": 2e-5,
            "norm": "|gpu - fp64| / sum_j |A[i,j] B[j,k]|",
            "checked": f"{rows.size} rows ({longest} longest, {int(lens[rows].sum())} stored entries) x {NK} columns"}


def e2e_api(A_h, B_h, nbytes: int, steps: int) -> dict:
    """The plugin API end to end: host Finch tensors in, compute(lazy(A) @
    lazy(B)) (transfer, matcher, fgb_spmm), host C out, every step."""
    import torch

    import finchgb as F
    from finchgb.workloads import SparseBuffers

    fmtA = F.Dense(F.SparseList(F.Element(np.float32(0.0))))
    fmtB = F.Dense(F.Dense(F.Element(np.float32(0.0))))
    At = SparseBuffers(A_h.ncols, A_h.nrows, A_h.ptr, A_h.idx, A_h.val, "csc")  # CSC of A^T = CSR of A

    def one():
        A = F.swizzle(F.Tensor.from_buffers(fmtA, At), 2, 1)  # fresh host tensors: every step uploads
        B = F.Tensor(fmtB, B_h)
        return F.compute(F.lazy(A) @ F.lazy(B)).todense()

    C = one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        C = one()
    dt = (time.perf_counter() - t0) / steps
    h2d = A_h.ptr.nbytes + A_h.idx.nbytes + A_h.val.nbytes + B_h.nbytes
    return {"value": round(nbytes / dt / 1e9, 1), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(C.nbytes), "steps": steps, "ms_per_step": round(1e3 * dt, 3),
            "call": "compute(lazy(swizzle(Tensor(Dense(SparseList(Element(0f))), A^T), 2, 1)) @ "
                    "lazy(Tensor(Dense(Dense(Element(0f))), B))).todense()",
            "timing": "host wall clock per call (synchronous), Finch's Int64 ptr/idx uploaded and narrowed"}, C


def spmv_config1() -> dict:
    """Configuration 1 in the default run: y[i] += A[i,j]*x[j], A 10,000^2
    CSC (fsprand p = 0.001), FP64; the three device schedules replayed as
    graphs, their results against the oracle's FP64 nest (Finch order
    bit-exact), and Finch's serial nest timed on one core."""
    import torch

    import oracle
    from finchgb import _lib as L
    from finchgb import device as dev
    from finchgb.workloads import fsprand

    rng = np.random.default_rng(SEED + 1)
    n = 10_000
    A = fsprand(rng, n, n, 0.001)
    x = rng.random(n)
    Ad = dev.DeviceSparse.from_host(n, n, A.ptr, A.idx, A.val, orient="csc")
    Ar = Ad.transposed_storage()
    xd = torch.from_numpy(x).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    nbytes = 12 * A.nnz + 4 * (n + 1) + 16 * n
    want = oracle.spmv_csc(oracle.SR_PT, n, n, A.ptr, A.idx, A.val, x)
    scale = oracle.spmv_csc(oracle.SR_PT, n, n, A.ptr, A.idx, np.abs(A.val), np.abs(x))
    out = {"metric": "spmv_latency_us", "unit": "us", "higher_is_better": False, "dtype": "f64",
           "config": {"workload": "fsprand 10000x10000 p=0.001 CSC, x U[0,1), FP64", "nnz": int(A.nnz)},
           "cpu_baseline": {"value": round(_cpu_time(lambda: oracle.spmv_csc(0, n, n, A.ptr, A.idx, A.val, x))
                                           * 1e6, 3), "unit": "us", "cores": 1, "kind": "port",
                            "sample": "whole matrix, Finch's serial CSC nest (oracle)"}}
    for name, fn in (("csc_push_atomic", lambda: dev.spmv(Ad, xd, y)),
                     ("csr_pull_finch_order", lambda: dev.spmv(Ar, xd, y, flags=L.FINCH_ORDER | L.FMA)),
                     ("csr_pull", lambda: dev.spmv(Ar, xd, y))):
        ms = _graph_ms(fn)
        fn()
        got = y.cpu().numpy()
        err = float(np.max(np.abs(got - want) / (scale + 1e-300)))
        out[name] = {"us": round(ms * 1e3, 3), "roofline": _roof(nbytes, ms), "max_rel_err_vs_fp64": err,
                     "bit_exact_vs_finch_nest": bool(np.array_equal(got, want))}
    return out


def suite_block(A_h, Ad) -> dict:
    """Compact lines for the other configurations: the FP64 SpMV of
    configuration 1, SDDMM (k = 64) on the headline matrix, 20 Bellman-Ford
    min-plus rounds on the 4M-node graph, and CG on the 2048^2 Poisson
    matrix in every arithmetic mode."""
    import torch

    import oracle
    from finchgb import _lib as L
    from finchgb import cg
    from finchgb import device as dev
    from finchgb.plan import Plan
    from finchgb.workloads import poisson2d, random_graph

    out = {"spmv_fp64_10k": spmv_config1()}
    m = A_h.nrows
    rng = np.random.default_rng(SEED + 1)
    X = rng.standard_normal((m, 64), dtype=np.float32)
    Y = rng.standard_normal((m, 64), dtype=np.float32)
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    o = torch.empty(A_h.nnz, dtype=torch.float32, device="cuda")
    plan = Plan.sddmm(Ad, Xd, Yd, o, tune_reps=3)
    ms = _timed_ms(plan.execute, reps=10)
    nbytes = 4 * (m + 1) + 8 * A_h.nnz + 2 * 4 * m * 64 + 4 * A_h.nnz
    e = np.random.default_rng(2).choice(A_h.nnz, 200_000, replace=False)
    rows = np.searchsorted(A_h.ptr - 1, e, side="right") - 1
    cols = A_h.idx[e] - 1
    oh = o.cpu().numpy()
    want = A_h.val[e].astype(np.float64) * np.einsum("ij,ij->i", X[rows].astype(np.float64), Y[cols].astype(np.float64))
    scl = np.abs(A_h.val[e]).astype(np.float64) * np.einsum("ij,ij->i", np.abs(X[rows]).astype(np.float64),
                                                             np.abs(Y[cols]).astype(np.float64))
    rel = np.abs(oh[e] - want) / np.maximum(scl, 1e-300)
    out["sddmm_1M_k64"] = {"metric": "sddmm_gbps_algorithmic", "value": round(nbytes / (ms / 1e3) / 1e9, 1),
                           "unit": "GB/s", "ms_per_call": round(ms, 4), "roofline": _roof(nbytes, ms),
                           "schedule": plan.info(), "max_rel_err_vs_fp64": float(rel.max()),
                           "checked": "200,000 sampled entries, |gpu - fp64| / sum_k |a x_ik y_jk|"}
    del Xd, Yd, o, plan
    # Bellman-Ford: 20 min-plus rounds, pull over a CSR copy, autotuned plan
    g = random_graph(np.random.default_rng(SEED + 3), 4_000_000, 8.0)
    n = g.nrows
    Gd = dev.DeviceSparse.from_host(n, n, g.ptr, g.idx, g.val, orient="csc")
    Gr = Gd.transposed_storage()
    x0 = torch.full((n,), 2**30, dtype=torch.int32, device="cuda")
    x0[0] = 0
    xp, yp = x0.clone(), torch.empty_like(x0)
    pmp = Plan.spmv(Gr, xp, yp, semiring=L.MIN_PLUS)

    def rounds():
        xp.copy_(x0)
        for _ in range(20):
            pmp.execute()
            dev.dense_map(L.MAP_MIN, xp, yp, xp)

    ms20 = _timed_ms(rounds, reps=3, warm=1)
    rounds()
    per_round = 8 * g.nnz + 4 * (n + 1) + 3 * 4 * n + 2 * 4 * n
    # one more round against the oracle's nest on sampled rows: bit-exact (integers)
    ptr, idx, val = Gr.to_host()
    from finchgb.workloads import SparseBuffers

    csr = SparseBuffers(n, n, ptr, idx, val, "csr")
    xcur = xp.cpu().numpy()
    y1 = dev.spmv(Gr, xp, semiring=L.MIN_PLUS).cpu().numpy()
    srows = np.unique(np.random.default_rng(3).choice(n, 3000, replace=False))
    sub = rows_of(csr, srows)
    exact = bool(np.array_equal(y1[srows], oracle.spmv_csr(oracle.SR_MINP, sub.nrows, n, sub.ptr, sub.idx,
                                                            sub.val, xcur)))
    out["bellman_ford_minplus_4M"] = {
        "metric": "minplus_round_gbps", "value": round(20 * per_round / (ms20 / 1e3) / 1e9, 1), "unit": "GB/s",
        "ms_per_20_rounds": round(ms20, 3), "roofline": _roof(20 * per_round, ms20),
        "lanes_per_row": pmp.info()["lanes"], "bit_exact_vs_oracle_on_3000_rows": exact}
    del Gd, Gr, xp, yp, pmp, x0
    # CG: FP64, FP32 and BF16 SpMV to a true relative residual of 1e-10
    P = poisson2d(2048)
    b = np.random.default_rng(SEED + 4).uniform(-1, 1, P.nrows)
    Pd = dev.DeviceSparse.from_host(P.nrows, P.ncols, P.ptr, P.idx, P.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    out["cg_poisson2048"] = {"metric": "cg_seconds", "unit": "s", "higher_is_better": False,
                             **cg_lines(P, Pd, bd)}
    return out


def cg_lines(P, Pd, bd) -> dict:
    """CG to a true relative residual of 1e-10: FP64, and FP32/BF16-valued
    SpMVs summed in FP32, (values widened) in FP64, or with the whole
    iteration in pairs of FP32 numbers.  Per-iteration bytes: the SpMV's ptr,
    index (2-byte offsets when compact) and values, p and q, and the updates'
    r, q, x, p traffic (80 bytes per row)."""
    from finchgb import cg

    lines = {}
    for prec, acc in (("f64", "f64"), ("f32", "f32"), ("bf16", "f32"), ("f32", "f64"), ("bf16", "f64"),
                      ("f32", "spmv_pair"), ("bf16", "spmv_pair"), ("f32", "pair"), ("bf16", "pair")):
        x, res = cg.cg_solve(Pd, bd, precision=prec, rtol=1e-10, max_iter=60_000, accumulate=acc)
        vb = {"f64": 8, "f32": 4, "bf16": 2}[prec]
        ib = 2 if res.compact_index else 4
        # vectors per row: SpMV p, q; r update q, r, r; x/p update p, r, x, x, p
        # (8-byte elements: FP64 or pairs); FP32 sums add p's FP32 copy (write
        # and read)
        per_it = P.nnz * (ib + vb) + 4 * (P.nrows + 1) + 80 * P.nrows + (8 * P.nrows if acc == "f32" else 0)
        ms_it = 1e3 * res.seconds / max(res.iterations, 1)
        key = prec if prec == "f64" else f"{prec}_values_{acc}_sums"
        lines[key] = {"seconds": round(res.seconds, 4), "iterations": res.iterations,
                      "replacements": res.replacements, "true_rel_residual": res.true_rel_residual,
                      "converged": bool(res.converged), "compact_index": bool(res.compact_index),
                      "ms_per_iteration": round(ms_it, 4), "roofline": _roof(per_it, ms_it)}
    f64 = lines["f64"]["seconds"]
    for k, v in lines.items():
        v["speedup_vs_f64"] = round(f64 / v["seconds"], 3) if v["seconds"] > 0 else None
    return lines


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
    fixed_variant = fixed_bands = 0
    if args.schedule:  # fixed schedule LANES,PATH[,VARIANT[,BANDS]] through fgb_spmm_ex (profiling)
        vals = [int(v) for v in args.schedule.split(",")]
        lanes, path = vals[0], vals[1]
        fixed_variant = vals[2] if len(vals) > 2 else 0
        fixed_bands = vals[3] if len(vals) > 3 else 0
        table, plan, npanels = {}, None, 1
    else:
        # the plain schedules' table (for the e2e leg and the record), then the
        # library autotuner, whose search space adds column panels
        (lanes, path), table = autotune(A, B, C, verbose=args.sweep)
        from finchgb.plan import Plan

        plan = Plan.spmm(A, B, C, tune_reps=3)
        info = plan.info()
        npanels = info["panels"]
    variant = info["variant"] if plan is not None else fixed_variant
    bands = max(1, info["bands"] if plan is not None else fixed_bands)
    plan_path = info["path"] if plan is not None else path
    # lanes 0 in a fixed schedule is the library's own default; for this
    # workload that is the 32-column slab schedule (8 lanes)
    plan_lanes = info["lanes"] if plan is not None else (lanes if lanes > 0 else 8)
    slabs = -(-NK // (4 * plan_lanes))
    if plan is None and lanes == 0 and path == 0 and variant == 0:
        variant = 3  # the library's default for a B far larger than L2
    vrow = variant in (2, 3, 4)
    if plan is None and vrow:
        # schedule built per call: count, 5 scans (2 kernels each), fill, a
        # 3-kernel radix sort and the gather, then the slab x band launches
        # and at most 2 fix-up passes (profiling runs only)
        launches_per_step = 16 + slabs * bands + 2
    elif plan is None:
        launches_per_step = 1 + slabs + 1  # merge plan + one launch per slab + carry fix-up
    else:  # the plan's captured graph: its kernel nodes (slab x band launches + fix-up passes)
        launches_per_step = info["launches"]

    def step():
        if plan is not None:
            plan.execute()
        else:
            dev.spmm(A, B, C, lanes=lanes, path=path, variant=fixed_variant, bands=fixed_bands)

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
                       "schedule": ({"autotuner": "fgb_plan_create (tune_reps=3), graph replay",
                                     **plan.info()} if plan is not None else
                                    {"lanes": lanes, "merge_path_item": path}),
                       "plain_schedules_ms": {f"{k[0]}x{k[1]}": round(v, 4)
                                              for k, v in table.items()},
                       "l2": "inputs larger than L2 (1.16 GB per step vs 129 MB)",
                       "parallelism": f"replicas{world}"},
            "gpu_launches": args.steps * launches_per_step}

    # ---- e2e: host buffers through the C ABI -> host result.  NSETS buffer
    # sets with a plan each (the others' schedules come from the tune cache);
    # every step uploads A and B from pinned memory, runs the plan and reads
    # C back, and later steps' uploads overlap earlier steps' SpMM and
    # read-back (copy-in, compute and copy-out streams).
    if not args.no_e2e:
        ctx = dev.context()
        lib = L.load()
        host_A = [torch.from_numpy(A_h.ptr.astype(np.int32)).pin_memory(),
                  torch.from_numpy(A_h.idx.astype(np.int32)).pin_memory(),
                  torch.from_numpy(A_h.val).pin_memory()]
        B_pin = torch.from_numpy(B_h).pin_memory()
        C_pin = [torch.empty((M, NK), dtype=torch.float32).pin_memory() for _ in range(NSETS)]
        sets = []
        for b in range(NSETS):
            if b == 0 and plan is not None:
                A_b, B_b, C_b, plan_b = A, B, C, plan
            else:
                A_b = dev.DeviceSparse.from_host(A_h.nrows, A_h.ncols, A_h.ptr, A_h.idx, A_h.val,
                                                 orient="csr")
                B_b = torch.empty_like(B)
                C_b = torch.empty_like(C)
                B_b.copy_(B)
                if plan is not None:
                    plan_b = Plan.spmm(A_b, B_b, C_b, tune_reps=3)
                else:
                    plan_b = None
            assert A_b.ptr.dtype == torch.int32 and A_b.base == 1
            sets.append((A_b, B_b, C_b, plan_b))
        h2d = sum(h.numel() * h.element_size() for h in host_A) + B_pin.numel() * B_pin.element_size()
        d2h = C_pin[0].numel() * C_pin[0].element_size()
        s_in, s_comp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in range(NSETS)]
        ev_comp = [torch.cuda.Event() for _ in range(NSETS)]
        ev_out = [torch.cuda.Event() for _ in range(NSETS)]
        for b in range(NSETS):  # all events start signalled
            for ev in (ev_in[b], ev_comp[b], ev_out[b]):
                ev.record(stream)

        def e2e_step(i):
            b = i % NSETS
            A_b, B_b, C_b, plan_b = sets[b]
            s_in.wait_event(ev_comp[b])  # the SpMM NSETS steps back has read this set
            for d, h in zip((A_b.ptr, A_b.idx, A_b.val, B_b), (*host_A, B_pin)):
                L.check(lib.fgb_upload(ctx, d.data_ptr(), h.data_ptr(), h.numel() * h.element_size(),
                                       s_in.cuda_stream))
            ev_in[b].record(s_in)
            s_comp.wait_event(ev_in[b])
            s_comp.wait_event(ev_out[b])  # C of NSETS steps back has been read out
            with torch.cuda.stream(s_comp):
                if plan_b is not None:
                    plan_b.execute()
                else:
                    dev.spmm(A_b, B_b, C_b, lanes=lanes, path=path, variant=fixed_variant, bands=fixed_bands)
            ev_comp[b].record(s_comp)
            s_out.wait_event(ev_comp[b])
            L.check(lib.fgb_download(ctx, C_pin[b].data_ptr(), C_b.data_ptr(), d2h, s_out.cuda_stream))
            ev_out[b].record(s_out)

        for i in range(NSETS + 1):
            e2e_step(i)
        for st in (s_in, s_comp, s_out):
            stream.wait_stream(st)
        barrier()
        e2e_steps = max(4, args.steps // 2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s_in.wait_stream(stream)
        for i in range(e2e_steps):
            e2e_step(i)
        for st in (s_in, s_comp, s_out):
            stream.wait_stream(st)
        e1.record(stream)
        barrier()
        e2e_ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([e2e_ms], device=device)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_ms = float(t.item())
        last = (e2e_steps - 1) % NSETS
        ok = bool(np.array_equal(C_pin[last].numpy(), C.cpu().numpy()))
        line["e2e"] = {"value": round(nbytes * e2e_steps * world / (e2e_ms / 1e3) / 1e9, 1),
                       "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "steps": e2e_steps, "ms_per_step": round(e2e_ms / e2e_steps, 3),
                       "pipeline": f"{NSETS} buffer sets; copy-in / SpMM / copy-out streams overlap",
                       "result_matches_device_run": ok, "gpu_launches": e2e_steps * launches_per_step}

    # ---- roofline of the SpMM (plan + per-slab merge kernels + fix-up)
    peak, peak_kind = load_peaks()
    avg_ms = sum(step_ms) / len(step_ms)
    achieved = nbytes / (avg_ms / 1e3) / 1e9
    sched = f"lanes={plan_lanes} path={plan_path} variant={variant} bands={bands}"
    traffic, traffic_src = load_traffic(sched)
    line["roofline"] = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(achieved / peak, 4),
                        "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                        "traffic": traffic, "traffic_source": traffic_src,
                        "schedule": sched,
                        "kernel": (f"spmm_vrow_k x{slabs} column slabs x{bands} bands + vrow_fixup_seg_k + vrow_fixup_rows_k" if variant == 2 else
                                   f"spmm_vrow_async_k x{slabs} column slabs x{bands} bands + vrow_fixup_seg_k + vrow_fixup_rows_k" if variant == 3 else
                                   f"spmm_vrow_pipe_k x{slabs} column slabs x{bands} bands + vrow_fixup_seg_k + vrow_fixup_rows_k" if variant == 4 else
                                   f"{npanels} column panels x (spmm_merge_k + spmm_fixup_k)"
                                   if plan is not None and npanels > 1 else
                                   f"spmm_merge_k x{slabs} slabs + spmm_fixup_k"),
                        "algorithmic_bytes_per_launch": nbytes,
                        "avg_launch_ms": round(avg_ms, 4)}
    if traffic:
        # the DRAM bytes ncu counted for one step, over this run's step time:
        # how busy HBM is, against the compulsory-byte fraction above
        line["roofline"]["traffic_gbs"] = round(traffic / (avg_ms / 1e3) / 1e9, 1)
        line["roofline"]["traffic_frac"] = round(traffic / (avg_ms / 1e3) / 1e9 / peak, 4)
    # The slab kernel gathers a 4*lanes-column piece of one B row per stored
    # entry and slab: nnz * NK * 4 bytes per step, from a working set of one
    # slab of B.  Its ceiling is the random-gather rate at that width and
    # working set, measured here on the same device.
    if vrow:
        gbytes = 16 * plan_lanes
        ws = -(-A_h.ncols // bands) * gbytes  # one band of one slab of B per launch
        ceiling = dev.gather_ceiling(ws, gbytes)
        gathered = A_h.nnz * NK * 4
        g_achieved = gathered / (avg_ms / 1e3) / 1e9
        line["gather_ceiling"] = {"gathered_bytes_per_step": gathered, "gather_bytes": gbytes,
                                  "working_set_bytes": ws,
                                  "achieved": round(g_achieved, 1), "ceiling": round(ceiling, 1),
                                  "unit": "GB/s", "frac": round(g_achieved / ceiling, 4)}
    line["clocks"] = clk.summary()
    if rank == 0:
        # the result of the timed steps against the oracle in FP64
        line["max_rel_err_vs_fp64"] = spmm_fp64_error(A_h, B_h, C.cpu().numpy())
    if rank == 0 and not args.no_e2e:
        # the plugin API from host tensors (transfer + matcher + per-call SpMM + host result)
        line["e2e_api"], C_api = e2e_api(A_h, B_h, nbytes, steps=max(3, min(args.steps, 8)))
        line["e2e_api"]["max_rel_err_vs_fp64"] = spmm_fp64_error(A_h, B_h, C_api)["max_rel_err_vs_fp64"]
        # per call, at most: 2 index narrowings, the 16-kernel schedule build,
        # 4 slabs x 2 bands, 2 fix-up passes
        line["e2e_api"]["gpu_launches_at_most"] = line["e2e_api"]["steps"] * (2 + 16 + 4 * 2 + 2)
        del C_api
    line["cpu_baseline"] = None
    if rank == 0 and not args.skip_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(A_h, B_h, nbytes)
    if rank == 0 and not args.headline_only:
        torch.cuda.empty_cache()
        for key, fn in (("suite", lambda: suite_block(A_h, A)), ("served", served_block)):
            try:
                line[key] = fn()
            except Exception as e:  # a failed block is reported, the headline stands
                line[key] = {"error": repr(e)}
            torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------- the other configurations

def _timed_ms(fn, reps: int = 20, warm: int = 3) -> float:
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _graph_ms(fn, reps: int = 200) -> float:
    """Device time per call with `reps` calls captured in one CUDA graph (the
    launch-latency-free figure for microsecond kernels), median of 5 replays."""
    import torch

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        fn()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            for _ in range(reps):
                fn()
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    times = []
    for _ in range(5):  # the median of 5 replays: one disturbed replay does not set the figure
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / reps)
    return float(np.median(times))


def _cpu_time(fn, min_seconds: float = 2.0, max_reps: int = 1000) -> float:
    fn()
    t, n = 0.0, 0
    while t < min_seconds and n < max_reps:
        t0 = time.perf_counter()
        fn()
        t += time.perf_counter() - t0
        n += 1
    return t / n


def _roof(nbytes: int, ms: float) -> dict:
    peak, kind = load_peaks()
    ach = nbytes / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 4), "peak_kind": kind, "algorithmic_bytes": nbytes,
            "ms": round(ms, 5)}


def suite_spmv_fp64() -> list[dict]:
    """y[i] += A[i,j]*x[j], A 10,000^2 CSC (fsprand 0.001), FP64 throughout."""
    import torch

    import oracle
    from finchgb import _lib as L
    from finchgb import device as dev
    from finchgb.workloads import fsprand

    rng = np.random.default_rng(SEED + 1)
    n = 10_000
    A = fsprand(rng, n, n, 0.001)
    x = rng.random(n)
    Ad = dev.DeviceSparse.from_host(n, n, A.ptr, A.idx, A.val, orient="csc")
    Ar = Ad.transposed_storage()
    xd = torch.from_numpy(x).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    nbytes = 12 * A.nnz + 4 * (n + 1) + 16 * n
    out = []
    threads = oracle.max_threads()
    t_serial = _cpu_time(lambda: oracle.spmv_csc(0, n, n, A.ptr, A.idx, A.val, x))
    for name, fn in (("csc_push_atomic", lambda: dev.spmv(Ad, xd, y)),
                     ("csr_pull_finch_order", lambda: dev.spmv(Ar, xd, y, flags=L.FINCH_ORDER)),
                     ("csr_pull", lambda: dev.spmv(Ar, xd, y))):
        ms_launch = _timed_ms(fn, reps=200)
        ms_graph = _graph_ms(fn)
        out.append({"suite": "spmv_fp64_10k", "variant": name, "metric": "spmv_latency_us",
                    "value": round(ms_graph * 1e3, 3), "unit": "us", "higher_is_better": False,
                    "per_call_launch_us": round(ms_launch * 1e3, 3), "dtype": "f64",
                    "config": {"workload": "fsprand 10000x10000 p=0.001 CSC, x U[0,1)",
                               "nnz": int(A.nnz)},
                    "roofline": _roof(nbytes, ms_graph),
                    "cpu_baseline": {"value": round(t_serial * 1e6, 3), "unit": "us", "cores": 1,
                                     "kind": "port",
                                     "sample": "whole matrix, Finch's serial CSC nest (oracle)"}})
    return out


def suite_sddmm() -> list[dict]:
    """out[e] = A[i,j] * <X[i,:], Y[j,:]>, A the 1M^2 power-law CSR, k = 64, FP32."""
    import torch

    import oracle
    from finchgb import device as dev
    from finchgb.workloads import zipf_csr

    rng = np.random.default_rng(SEED)
    m = 1_000_000
    A = zipf_csr(rng, m, m, mean=NNZ_MEAN, a=1.5, cap=50_000, dtype=np.float32)
    X = rng.standard_normal((m, 64), dtype=np.float32)
    Y = rng.standard_normal((m, 64), dtype=np.float32)
    Ad = dev.DeviceSparse.from_host(m, m, A.ptr, A.idx, A.val, orient="csr")
    Xd, Yd = torch.from_numpy(X).cuda(), torch.from_numpy(Y).cuda()
    outd = torch.empty(A.nnz, dtype=torch.float32, device="cuda")
    nbytes = 4 * (m + 1) + 8 * A.nnz + 2 * 4 * m * 64 + 4 * A.nnz
    from finchgb.plan import Plan

    schedules = {"library_default_per_call": _timed_ms(lambda: dev.sddmm(Ad, Xd, Yd, outd), reps=10),
                 "one_pass_default": _timed_ms(lambda: dev.sddmm(Ad, Xd, Yd, outd, slab=0), reps=10),
                 "slab32_lanes8": _timed_ms(lambda: dev.sddmm(Ad, Xd, Yd, outd, lanes=8, slab=32),
                                            reps=10)}
    plan = Plan.sddmm(Ad, Xd, Yd, outd, tune_reps=3)
    schedules["plan"] = _timed_ms(plan.execute, reps=10)
    ms = schedules["plan"]
    rows = 100_000
    p = A.ptr[: rows + 1]
    nnz_s = int(p[-1] - 1)
    threads = oracle.max_threads()
    t = _cpu_time(lambda: oracle.sddmm_csr(rows, p, A.idx[:nnz_s], A.val[:nnz_s], X[:rows], Y,
                                           nthreads=threads), min_seconds=3.0)
    t_full = t * A.nnz / max(nnz_s, 1)
    # virtual-row plans gather one slab of a Y row per stored entry and slab
    info = plan.info()
    gather = None
    if info["variant"] in (3, 4):
        gbytes = 16 * info["lanes"] if info["lanes"] > 0 else 4 * 64
        gathered = A.nnz * 64 * 4
        ceiling = dev.gather_ceiling(m * gbytes, gbytes)
        g_ach = gathered / (ms / 1e3) / 1e9
        gather = {"gathered_bytes_per_call": gathered, "gather_bytes": gbytes,
                  "working_set_bytes": m * gbytes, "achieved": round(g_ach, 1),
                  "ceiling": round(ceiling, 1), "unit": "GB/s", "frac": round(g_ach / ceiling, 4)}
    return [{"suite": "sddmm_1M_k64", "metric": "sddmm_gbps_algorithmic",
             "value": round(nbytes / (ms / 1e3) / 1e9, 1), "unit": "GB/s", "dtype": "f32",
             "ms_per_call": round(ms, 4),
             "schedules_ms": {k: round(v, 4) for k, v in schedules.items()},
             "plan_choice": info,
             "config": {"workload": "zipf1.5 1Mx1M nnz 16M CSR, X/Y 1Mx64 N(0,1)"},
             "roofline": _roof(nbytes, ms), "gather_ceiling": gather,
             "cpu_baseline": {"value": round(nbytes / t_full / 1e9, 3), "unit": "GB/s",
                              "cores": threads, "kind": "port",
                              "sample": f"rows 1..{rows}, time scaled by stored entries"}}]


def suite_semiring() -> list[dict]:
    """Bellman-Ford min-plus (Int32) and or-and reachability on a 4M-node graph."""
    import torch

    import oracle
    from finchgb import _lib as L
    from finchgb import device as dev
    from finchgb.workloads import random_graph

    rng = np.random.default_rng(SEED + 3)
    n = 4_000_000
    g = random_graph(rng, n, 8.0)
    Ad = dev.DeviceSparse.from_host(n, n, g.ptr, g.idx, g.val, orient="csc")
    Ap = dev.DeviceSparse(n, n, Ad.ptr, Ad.idx, None, "csc", Ad.base)
    sentinel = 2**30
    x0 = torch.full((n,), sentinel, dtype=torch.int32, device="cuda")
    x0[0] = 0

    def rounds(nr=20):
        x = x0.clone()
        y = torch.empty_like(x)
        for _ in range(nr):
            dev.spmv(Ad, x, y, semiring=L.MIN_PLUS)
            dev.dense_map(L.MAP_MIN, x, y, x)
        return x

    ms20 = _timed_ms(lambda: rounds(20), reps=3, warm=1)
    x_push = rounds(20)
    per_round_bytes = 8 * g.nnz + 4 * (n + 1) + 3 * 4 * n + 2 * 4 * n
    # pull over a CSR copy built once on the device (rows = targets: no atomics)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Ar = Ad.transposed_storage()
    torch.cuda.synchronize()
    ms_transpose = 1e3 * (time.perf_counter() - t0)
    Arp = dev.DeviceSparse(n, n, Ar.ptr, Ar.idx, None, "csr", Ar.base)

    from finchgb.plan import Plan

    xp = x0.clone()
    yp = torch.empty_like(xp)
    plan_mp = Plan.spmv(Ar, xp, yp, semiring=L.MIN_PLUS)  # autotuned lanes per row, graph replay

    def rounds_pull(nr=20):
        xp.copy_(x0)
        for _ in range(nr):
            plan_mp.execute()
            dev.dense_map(L.MAP_MIN, xp, yp, xp)
        return xp

    ms20_pull = _timed_ms(lambda: rounds_pull(20), reps=3, warm=1)
    same = bool(torch.equal(rounds_pull(20), x_push))
    # or-and reachability, y = A x over (|, &), for a one-vertex frontier and a
    # frontier of a quarter of the vertices.  The push skips columns whose
    # x[j] is false and the pull stops a row at its first true product, so
    # each line's bytes are the ones that frontier requires: push = y fill,
    # x scan, ptr and entries of the true columns (+ their y writes); pull =
    # the whole matrix, x and y (a row's entries share one 32-byte sector).
    deg = np.diff(g.ptr)
    or_bytes = 4 * g.nnz + 4 * (n + 1) + 2 * n
    frontiers = {"one_vertex": np.zeros(n, dtype=np.uint8),
                 "quarter": (rng.random(n) < 0.25).astype(np.uint8)}
    frontiers["one_vertex"][0] = 1
    or_lines = []
    for fname, fh in frontiers.items():
        fx = torch.from_numpy(fh).cuda()
        y_push, y_pull = torch.empty_like(fx), torch.empty_like(fx)
        ms_push = _timed_ms(lambda: dev.spmv(Ap, fx, y_push, semiring=L.OR_AND), reps=20)
        plan_or = Plan.spmv(Arp, fx, y_pull, semiring=L.OR_AND)
        ms_pull = _timed_ms(plan_or.execute, reps=20)
        active = fh.astype(bool)
        e_active = int(deg[active].sum())
        push_bytes = 2 * n + 8 * int(active.sum()) + 5 * e_active
        same_or = bool(torch.equal(y_push, y_pull))
        common = {"suite": "reachability_or_and_4M", "metric": "or_and_spmv_gbps", "unit": "GB/s",
                  "dtype": "bool", "frontier": fname, "frontier_vertices": int(active.sum()),
                  "equal_push_pull": same_or}
        or_lines.append({**common, "variant": "csc_push",
                         "value": round(push_bytes / (ms_push / 1e3) / 1e9, 1),
                         "ms_per_call": round(ms_push, 4), "entries_touched": e_active,
                         "config": {"workload": "same graph, Pattern level, CSC (columns = sources)"},
                         "roofline": _roof(push_bytes, ms_push)})
        or_lines.append({**common, "variant": "csr_pull",
                         "value": round(or_bytes / (ms_pull / 1e3) / 1e9, 1),
                         "ms_per_call": round(ms_pull, 4), "lanes_per_row": plan_or.info()["lanes"],
                         "config": {"workload": "same graph, Pattern level, CSR copy"},
                         "roofline": _roof(or_bytes, ms_pull)})
    # The pull SpMVs gather one x value per stored entry (a 32-byte sector
    # request each) from an L2-resident x: their ceiling is the device's
    # random-gather request rate over x's working set.
    def gather_line(gathers_per_call, ms_call, x_bytes):
        rate = dev.gather_ceiling(x_bytes, 4) / 4  # gathers per second (GB/s of 4-byte words / 4)
        achieved = gathers_per_call / (ms_call / 1e3)
        return {"gathers_per_call": int(gathers_per_call), "achieved_g_per_s": round(achieved / 1e9, 1),
                "ceiling_g_per_s": round(rate, 1), "working_set_bytes": int(x_bytes),
                "frac": round(achieved / 1e9 / rate, 4)}

    mp_gather = gather_line(g.nnz, ms20_pull / 20, 4 * n)
    for line in or_lines:
        if line["variant"] == "csr_pull":
            line["gather_ceiling"] = gather_line(g.nnz, line["ms_per_call"], n)
    threads = oracle.max_threads()
    xh = np.full(n, sentinel, dtype=np.int32)
    xh[0] = 0
    t_round = _cpu_time(lambda: oracle.spmv_csc(oracle.SR_MINP, n, n, g.ptr, g.idx, g.val, xh),
                        min_seconds=3.0, max_reps=5)
    return [{"suite": "bellman_ford_minplus_4M", "metric": "minplus_round_gbps",
             "value": round(20 * per_round_bytes / (ms20 / 1e3) / 1e9, 1), "unit": "GB/s",
             "dtype": "i32", "ms_per_20_rounds": round(ms20, 3),
             "config": {"workload": "4M nodes, Poisson(8) out-degree, Int32 weights U{1..1000}",
                        "nnz": int(g.nnz)},
             "roofline": _roof(20 * per_round_bytes, ms20),
             "cpu_baseline": {"value": round(per_round_bytes / t_round / 1e9, 3), "unit": "GB/s",
                              "cores": 1, "kind": "port",
                              "sample": "one round: Finch's serial CSC min-plus nest (oracle)"}},
            {"suite": "bellman_ford_minplus_4M", "variant": "csr_pull", "metric": "minplus_round_gbps",
             "value": round(20 * per_round_bytes / (ms20_pull / 1e3) / 1e9, 1), "unit": "GB/s",
             "dtype": "i32", "ms_per_20_rounds": round(ms20_pull, 3),
             "one_time_csr_copy_ms": round(ms_transpose, 3), "equal_to_push": same,
             "lanes_per_row": plan_mp.info()["lanes"],
             "config": {"workload": "same graph; CSR copy built once on the device"},
             "roofline": _roof(20 * per_round_bytes, ms20_pull), "gather_ceiling": mp_gather}] + or_lines


def suite_cg() -> list[dict]:
    """CG on the 2048^2 5-point Poisson matrix: FP64, FP32 and BF16 SpMV."""
    import torch

    from finchgb import cg
    from finchgb import device as dev
    from finchgb.workloads import poisson2d

    A = poisson2d(2048)
    rng = np.random.default_rng(SEED + 4)
    b = rng.uniform(-1, 1, A.nrows)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    return [{"suite": "cg_poisson2048", "variant": k, "metric": "cg_seconds", "value": v["seconds"], "unit": "s",
             "higher_is_better": False, **v} for k, v in cg_lines(A, Ad, bd).items()]


def suite_cg_probe() -> list[dict]:
    """Two 16-iteration chunks of CG on the 2048^2 Poisson matrix in FP64, in
    BF16 pair mode and in BF16 SpMV-pair mode: a short run of the iteration
    kernels (for ncu)."""
    import torch

    from finchgb import cg
    from finchgb import device as dev
    from finchgb.workloads import poisson2d

    A = poisson2d(2048)
    b = np.random.default_rng(SEED + 4).uniform(-1, 1, A.nrows)
    Ad = dev.DeviceSparse.from_host(A.nrows, A.ncols, A.ptr, A.idx, A.val, orient="csr")
    bd = torch.from_numpy(b).cuda()
    out = []
    for prec, acc in (("f64", "f64"), ("bf16", "pair"), ("bf16", "spmv_pair")):
        _, res = cg.cg_solve(Ad, bd, precision=prec, accumulate=acc, rtol=1e-10, max_iter=32, chunk=16)
        torch.cuda.synchronize()
        out.append({"suite": "cg_probe", "variant": f"{prec}_{acc}", "iterations": res.iterations,
                    "seconds": round(res.seconds, 4)})
    return out


def suite_spmv_adaptive() -> list[dict]:
    """The per-call CSR SpMV (no plan), FP64, on the 1M x 1M Zipf matrix
    (16M entries) and on 4M rows of Poisson(8) entries: at these row counts
    the library's default is the adaptive pull (one lane per row of at most
    32 entries, a warp per longer row).  Device time per call from CUDA-graph
    replays, and the plan autotuner's choice over 1, 4, 8 or 32 lanes per
    row and the adaptive pull (lanes 2) with its time."""
    import torch

    from finchgb import _lib as L
    from finchgb import device as dev
    from finchgb.plan import Plan
    from finchgb.workloads import _fibers_from_lengths, _ptr, zipf_csr

    rng = np.random.default_rng(SEED + 7)
    z = zipf_csr(rng, 1_000_000, 1_000_000, mean=16, a=1.5, cap=50_000, dtype=np.float64)
    lengths = rng.poisson(8.0, 4_000_000).astype(np.int64)
    cols = _fibers_from_lengths(rng, lengths, 4_000_000)
    out = []
    for name, (m, n, ptr, idx, val) in (
            ("zipf1.5_1Mx1M_nnz16M", (z.nrows, z.ncols, z.ptr, z.idx, z.val)),
            ("poisson8_4Mx4M", (4_000_000, 4_000_000, _ptr(lengths), cols + 1, rng.random(int(lengths.sum()))))):
        A = dev.DeviceSparse.from_host(m, n, ptr, idx, val, orient="csr")
        x = torch.rand(n, dtype=torch.float64, device="cuda")
        y = torch.empty(m, dtype=torch.float64, device="cuda")
        ms = _graph_ms(lambda: dev.spmv(A, x, y), reps=20)
        nbytes = 4 * (m + 1) + 12 * A.nnz + 8 * n + 8 * m
        plan = Plan.spmv(A, x, y, tune_reps=5)
        out.append({"suite": "spmv_adaptive", "workload": name, "nnz": int(A.nnz), "dtype": "f64",
                    "us_per_call": round(ms * 1e3, 1), "roofline": _roof(nbytes, ms),
                    "plan_lanes": plan.info()["lanes"], "plan_us": round(plan.info()["tuned_ms"] * 1e3, 1)})
        del A, plan
        torch.cuda.empty_cache()
    return out


def suite_pagerank() -> list[dict]:
    """PageRank (docs/examples/pagerank.jl) through finch() on a 4M-vertex
    Pattern graph with out-degree 1 + Poisson(7) (every vertex has an
    out-edge, which the example needs): the time per step (Finch-order SpMV
    + fused affine map) from the difference of 21- and 1-step runs, the
    setup (out-degree counts, the masked transition matrix, its CSR copy),
    and the 21-step result against an independent power iteration in
    scipy."""
    import torch

    import finchgb as F
    from finchgb import examples
    from finchgb.workloads import SparseBuffers, _fibers_from_lengths, _ptr

    rng = np.random.default_rng(SEED + 6)
    n = 4_000_000
    lengths = (1 + rng.poisson(7.0, n)).astype(np.int64)
    rows = _fibers_from_lengths(rng, lengths, n)
    g = SparseBuffers(n, n, _ptr(lengths), rows + 1, None, "csc")
    edges = F.Tensor.from_buffers(F.Dense(F.SparseList(F.Pattern())), g)
    F.transfer(F.gpu(), edges)
    examples.pagerank(edges, nsteps=2)  # warm-up: contexts, pools
    torch.cuda.synchronize()

    def wall(k):
        t0 = time.perf_counter()
        r = examples.pagerank(edges, nsteps=k)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r

    import scipy.sparse as sp

    t1 = min(wall(1)[0] for _ in range(2))
    runs = [wall(21) for _ in range(2)]
    t21, r = min(runs, key=lambda x: x[0])
    per_step = (t21 - t1) / 20
    setup = t1 - per_step  # out-degrees, transition matrix and its CSR copy
    got = r.todense()
    P = sp.csc_matrix((np.repeat(1.0 / lengths, lengths), rows, g.ptr - 1), shape=(n, n))
    ref = np.full(n, 1.0 / n)
    for _ in range(21):
        ref = (1 - 0.85) / n + 0.85 * (P @ ref)
    nnz = int(lengths.sum())
    step_bytes = 4 * (n + 1) + 12 * nnz + 8 * n * 4  # CSR copy, r read, rank written/read, r written
    return [{"suite": "pagerank", "metric": "pagerank_ms_per_step", "value": round(per_step * 1e3, 3),
             "unit": "ms", "higher_is_better": False,
             "config": {"workload": "Pattern graph, 4M vertices, out-degree 1 + Poisson(7)", "nnz": nnz,
                        "steps": 21, "damp": 0.85},
             "setup_ms": round(setup * 1e3, 2), "total_ms_21_steps": round(t21 * 1e3, 2),
             "roofline_per_step": _roof(step_bytes, per_step * 1e3),
             "max_rel_err_vs_power_iteration": float(np.max(np.abs(got - ref)) / np.max(ref)),
             "timing": "host wall clock around finch() calls, synchronised"}]


def serve_library(n_mats: int = 4096, n_partners: int = 512):
    """4,096 resident CSR matrices, rows log-uniform in [64, 8192], square,
    density U[0.5%, 5%], FP32 N(0,1), generated on the device; the first
    n_partners also get a same-shape partner for masked multiplies."""
    from finchgb.server import random_csr

    rng = np.random.default_rng(SEED + 5)
    ns = np.exp(rng.uniform(np.log(64), np.log(8192), n_mats)).astype(int)
    ps = rng.uniform(0.005, 0.05, n_mats)
    mats = [random_csr(SEED + 10 * k, int(n), int(n), float(p)) for k, (n, p) in enumerate(zip(ns, ps))]
    partners = [random_csr(SEED + 10 * k + 7, int(ns[k]), int(ns[k]), float(ps[k]))
                for k in range(n_partners)]
    return mats, partners


def serve_layout(plan, mats, arena_floats):
    """Places the requests' host buffers in a pinned arena used as a ring.

    Request i gets [off[i], off[i] + need[i]) (input then output, or the
    masked product's values); a request that would cross the end starts the
    next lap at 0.  dep[i] is the last earlier request whose range may share
    memory with request i: it must be complete before i is submitted."""
    need = np.array([mats[k].nnz if op == "masked_mul" else (mats[k].ncols + mats[k].nrows) * max(nk, 1)
                     for op, k, nk in plan], dtype=np.int64)
    need = (need + 3) // 4 * 4  # 16-byte aligned starts
    assert need.max() <= arena_floats
    virt = np.empty(len(plan), dtype=np.int64)
    v = 0
    for i, n in enumerate(need):
        if v % arena_floats + n > arena_floats:
            v += arena_floats - v % arena_floats
        virt[i] = v
        v += n
    dep = np.searchsorted(virt, virt + need - arena_floats, side="left") - 1
    return virt % arena_floats, dep


def serve_tune(mats, partners):
    """The serving autotuner on the library: per-class SpMV shapes, applied
    to every server of the run (both modes compute rows the same way at a
    given shape)."""
    from finchgb.server import Server

    with Server(mode="batched", pool_bytes=64 << 20, max_inflight=64) as srv:
        for A in mats + partners:
            srv.register(A)
        t = srv.tune(reps=3)
    return t, Server.shapes(t)


def serve_run(mode, mats, partners, plan, arena, window, arrivals=None, batch=128, tuning=None):
    """Runs the request plan through a server; returns (seconds, latencies, stats).

    The FgbRequest records (pointers into a pinned arena) are built before the
    clock starts, the same for both modes.  Closed loop: requests go in groups
    of `batch` through fgb_server_submit_batch, at most `window` in flight.
    Open loop: every request whose Poisson arrival time has passed is
    submitted as one group."""
    from finchgb import _lib as L
    from finchgb.server import Server

    off, dep = serve_layout(plan, mats, arena.numel())
    lat = []
    with Server(mode=mode, pool_bytes=4 << 30, max_inflight=min(window, 4096)) as srv:
        ids = [srv.register(A) for A in mats]
        pids = [srv.register(B) for B in partners]
        if tuning is not None:
            srv.set_tuning(tuning)
        reqs = (L.FgbRequest * len(plan))()
        for i, (op, k, nk) in enumerate(plan):
            A = mats[k]
            base = int(off[i])
            if op == "spmv":
                reqs[i] = srv.request(op, ids[k], arena[base: base + A.ncols],
                                      arena[base + A.ncols: base + A.ncols + A.nrows])
            elif op == "spmm":
                reqs[i] = srv.request(op, ids[k], arena[base: base + A.ncols * nk],
                                      arena[base + A.ncols * nk: base + (A.ncols + A.nrows) * nk], nk=nk)
            else:
                reqs[i] = srv.request(op, ids[k], None, arena[base: base + A.nnz], matrix_b=pids[k])
        size = ctypes.sizeof(L.FgbRequest)
        base_addr = ctypes.addressof(reqs)
        tickets: list[int] = []
        t_submit = t_wait = 0.0
        waited = 0
        n = len(plan)
        t0 = time.perf_counter()
        i = 0
        while i < n:
            if arrivals is None:
                j = min(n, i + batch)
            else:
                now = time.perf_counter() - t0
                while arrivals[i] > now:
                    now = time.perf_counter() - t0
                j = i + 1
                while j < n and arrivals[j] <= now and j - i < batch:
                    j += 1
            while j > i + 1 and dep[i:j].max() >= i:  # no overlap inside a group
                j -= 1
            # at most `window` requests in flight, and none whose arena range
            # the group reuses
            upto = max(j - window, int(dep[i:j].max()) + 1)
            if upto > waited:
                tw = time.perf_counter()
                lat.extend(srv.wait_batch(tickets[waited:upto]))
                t_wait += time.perf_counter() - tw
                waited = upto
            grp = (L.FgbRequest * (j - i)).from_address(base_addr + i * size)
            ts = time.perf_counter()
            tickets.extend(srv.submit_batch(grp))
            t_submit += time.perf_counter() - ts
            i = j
        tw = time.perf_counter()
        lat.extend(srv.wait_batch(tickets[waited:]))
        t_wait += time.perf_counter() - tw
        dt = time.perf_counter() - t0
        st = srv.stats()
        st["client_submit_s"] = round(t_submit, 4)
        st["client_wait_s"] = round(t_wait, 4)
    return dt, np.array(lat), st


def run_serve(args):
    """Config 5: batched/served requests vs the plain per-call GPU path."""
    import torch

    from finchgb import build

    build.build()
    mats, partners = serve_library()
    rng = np.random.default_rng(SEED + 6)
    n_req = args.requests
    plan = []
    for _ in range(n_req):
        op = ("spmv", "spmm", "masked_mul")[int(rng.integers(3))]
        k = int(rng.integers(len(partners) if op == "masked_mul" else len(mats)))
        plan.append((op, k, 32 if op == "spmm" else 0))
    # compulsory bytes per request: the matrix once (ptr int32, idx int32,
    # val fp32; the partner too for a masked multiply), the input read once
    # and the output written once -- inputs and outputs live in page-locked
    # host memory, so they also cross the host link
    def req_bytes(op, k, nk):
        A = mats[k]
        mat = 4 * (A.nrows + 1) + 8 * A.nnz
        if op == "masked_mul":  # A .* partner, written on A's pattern
            P = partners[k]
            return mat + 4 * (P.nrows + 1) + 8 * P.nnz + 4 * A.nnz, 4 * A.nnz
        io = 4 * (A.ncols + A.nrows) * max(nk, 1)
        return mat + io, io

    rb = [req_bytes(*r) for r in plan]
    total_bytes = float(sum(b for b, _ in rb))
    link_bytes = float(sum(l for _, l in rb))
    # the closed loop measures capacity: as many requests in flight as the
    # server has slots (4,096).  With 1,024 the loop was latency-bound at
    # 256 K requests/s; 2,048 gave 330 K, 4,096 about 345 K.
    window = 4096
    arena = torch.empty(512 << 20, dtype=torch.float32).pin_memory()  # 2 GiB ring
    torch.cuda.synchronize()
    out = {"suite": "served_4096_csr", "requests": n_req, "mix": "1/3 SpMV, 1/3 SpMM(32), 1/3 masked multiply",
           "closed_loop_in_flight": window,
           "matrices": len(mats), "stored_entries": int(sum(A.nnz for A in mats)),
           "config": {"workload": "4096 CSR, rows log-uniform [64, 8192], density U[0.5%, 5%], FP32"}}
    # closed loop (saturation): up to `window` requests in flight
    for mode in ("batched", "per_call"):
        dt, lat, st = serve_run(mode, mats, partners, plan, arena, window)
        out[mode] = {"ops_per_s": round(n_req / dt, 1), "seconds": round(dt, 3),
                     "compulsory_gbps": round(total_bytes / dt / 1e9, 1),
                     "host_link_gbps": round(link_bytes / dt / 1e9, 1),
                     "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                     "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
                     "launches": st["launches"], "batches": st["batches_published"],
                     "dispatcher_ms": {k: round(st[k] / 1e6, 2) for k in
                                       ("admit_ns", "scan_ns", "finish_ns", "queue_ns", "service_ns")
                                       if k in st},
                     "client_submit_s": st["client_submit_s"], "client_wait_s": st["client_wait_s"]}
    out["throughput_ratio_batched_vs_per_call"] = round(
        out["batched"]["ops_per_s"] / out["per_call"]["ops_per_s"], 2)
    # open loop: Poisson arrivals at half of each mode's capacity
    for mode in ("batched", "per_call"):
        lam = 0.5 * out[mode]["ops_per_s"]
        arr = np.cumsum(rng.exponential(1.0 / lam, n_req))
        dt, lat, st = serve_run(mode, mats, partners, plan, arena, window, arrivals=arr)
        out[mode]["poisson_rate_per_s"] = round(lam, 1)
        out[mode]["poisson_p50_ms"] = round(1e3 * float(np.percentile(lat, 50)), 3)
        out[mode]["poisson_p99_ms"] = round(1e3 * float(np.percentile(lat, 99)), 3)
    print(json.dumps(out), flush=True)


def _serve_plan(rng, n_req, mats, partners):
    plan = []
    for _ in range(n_req):
        op = ("spmv", "spmm", "masked_mul")[int(rng.integers(3))]
        k = int(rng.integers(len(partners) if op == "masked_mul" else len(mats)))
        plan.append((op, k, 32 if op == "spmm" else 0))
    return plan


def serve_check(mats, partners, n: int = 48, tuning=None) -> dict:
    """Served results against the FP64 oracle: n mixed requests through the
    batched server; SpMV/SpMM as |got - fp64| / sum|terms|, masked multiply
    (one product per entry) exact."""
    import torch

    import oracle
    from finchgb.server import Server
    from finchgb.workloads import SparseBuffers

    rng = np.random.default_rng(SEED + 8)
    worst, exact = 0.0, True
    with Server(mode="batched", pool_bytes=1 << 30, max_inflight=256) as srv:
        ids = [srv.register(A) for A in mats]
        pids = [srv.register(B) for B in partners]
        if tuning is not None:
            srv.set_tuning(tuning)
        todo = []
        for q in range(n):
            op = ("spmv", "spmm", "masked_mul")[q % 3]
            k = int(rng.integers(len(partners) if op == "masked_mul" else len(mats)))
            A = mats[k]
            if op == "masked_mul":
                out = torch.empty(A.nnz, dtype=torch.float32).pin_memory()
                todo.append((op, k, None, out, srv.submit(op, ids[k], None, out, matrix_b=pids[k])))
                continue
            nk = 32 if op == "spmm" else 1
            inp = torch.from_numpy(rng.standard_normal((A.ncols, nk), dtype=np.float32)).pin_memory()
            out = torch.empty((A.nrows, nk), dtype=torch.float32).pin_memory()
            if op == "spmv":
                inp, out = inp.view(-1), out.view(-1)
            todo.append((op, k, inp, out, srv.submit(op, ids[k], inp, out, nk=nk if op == "spmm" else 0)))
        for op, k, inp, out, t in todo:
            srv.wait(t)
            ptr, idx, val = mats[k].to_host()
            A = SparseBuffers(mats[k].nrows, mats[k].ncols, ptr, idx, val, "csr")
            if op == "masked_mul":
                pp, pi, pv = partners[k].to_host()
                D = np.zeros((A.nrows, A.ncols), np.float32)
                D[np.repeat(np.arange(A.nrows), np.diff(pp)), pi - 1] = pv
                want = val * D[np.repeat(np.arange(A.nrows), np.diff(ptr)), idx - 1]
                exact &= bool(np.array_equal(out.numpy(), want))
                continue
            X = inp.numpy().reshape(A.ncols, -1).astype(np.float64)
            w = oracle.spmm_csr(A.nrows, A.ncols, A.ptr, A.idx, A.val.astype(np.float64), X)
            sc = oracle.spmm_csr(A.nrows, A.ncols, A.ptr, A.idx, np.abs(A.val).astype(np.float64), np.abs(X))
            err = np.abs(out.numpy().reshape(A.nrows, -1) - w) / np.maximum(sc, 1e-300)
            worst = max(worst, float(err.max()))
    return {"requests": n, "max_rel_err_vs_fp64": worst, "masked_mul_exact": exact,
            "norm": "|served - fp64| / sum_j |A[i,j] x[j]|"}


def served_block(min_seconds: float = 1.0) -> dict:
    """Configuration 5 inside the default run: closed-loop capacity of the
    batched server and of the plain per-call path (at least min_seconds of
    requests each), then Poisson arrivals at the same rates for both modes
    (half and nine tenths of the per-call capacity) and at half the batched
    capacity for the batched mode, p50/p99 of the median of three runs;
    clocks sampled; a sample
    of served results against the FP64 oracle.  Every server uses the SpMV
    shapes the serving autotuner picked for the library's size classes."""
    import torch

    mats, partners = serve_library()
    rng = np.random.default_rng(SEED + 6)
    arena = torch.empty(512 << 20, dtype=torch.float32).pin_memory()  # 2 GiB ring
    window = 4096
    out = {"mix": "1/3 SpMV, 1/3 SpMM(32), 1/3 masked multiply", "matrices": len(mats),
           "stored_entries": int(sum(A.nnz for A in mats)), "closed_loop_in_flight": window,
           "config": {"workload": "4096 CSR, rows log-uniform [64, 8192], square, density U[0.5%, 5%], FP32 N(0,1)"}}

    def lat_stats(lat):
        return {"p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3)}

    tuning, shapes = serve_tune(mats, partners)
    out["spmv_shapes"] = shapes
    with ClockSampler(torch.cuda.current_device()) as clk:
        cap = {}
        for mode, n0 in (("batched", 400_000), ("per_call", 40_000)):
            plan = _serve_plan(rng, n0, mats, partners)
            dt, lat, st = serve_run(mode, mats, partners, plan, arena, window, tuning=tuning)
            if dt < min_seconds:  # too short: again with enough requests
                plan = _serve_plan(rng, int(n0 * 1.3 * min_seconds / dt), mats, partners)
                dt, lat, st = serve_run(mode, mats, partners, plan, arena, window, tuning=tuning)
            cap[mode] = len(plan) / dt
            out[mode] = {"closed_loop": {"ops_per_s": round(cap[mode], 1), "requests": len(plan),
                                         "seconds": round(dt, 3), **lat_stats(lat),
                                         "launches": st["launches"]}}
        out["throughput_ratio_batched_vs_per_call"] = round(cap["batched"] / cap["per_call"], 2)
        rates = [("0.5x_per_call_capacity", 0.5 * cap["per_call"], ("batched", "per_call")),
                 ("0.9x_per_call_capacity", 0.9 * cap["per_call"], ("batched", "per_call")),
                 ("0.5x_batched_capacity", 0.5 * cap["batched"], ("batched",))]
        for name, lam, modes in rates:
            n_req = max(5000, int(lam * 1.2 * min_seconds))
            plan = _serve_plan(rng, n_req, mats, partners)
            arr = np.cumsum(rng.exponential(1.0 / lam, n_req))
            for mode in modes:
                # three runs of the same arrivals; the run with the median p99 is
                # reported, every run's p99 beside it
                runs = []
                for _ in range(3):
                    dt, lat, st = serve_run(mode, mats, partners, plan, arena, window, arrivals=arr, tuning=tuning)
                    runs.append((float(np.percentile(lat, 99)), dt, lat))
                runs.sort(key=lambda r: r[0])
                _, dt, lat = runs[1]
                out[mode][f"poisson_{name}"] = {"rate_per_s": round(lam, 1), "requests": n_req,
                                                "seconds": round(dt, 3), **lat_stats(lat),
                                                "p99_ms_of_3_runs": [round(1e3 * r[0], 3) for r in runs]}
    out["clocks"] = clk.summary()
    out["oracle_check"] = serve_check(mats, partners, tuning=tuning)
    return out


def suite_coo() -> list[dict]:
    """fsparse assembly in HBM: 16M random (row, col) Int64 triplets, FP32
    values, about 0.01 % duplicates, into a 1M x 1M Dense(SparseList)."""
    import torch

    import oracle
    from finchgb import _lib as L
    from finchgb import device as dev

    rng = np.random.default_rng(SEED + 7)
    m = n = 1_000_000
    k = 16_000_000
    I = rng.integers(1, m + 1, k)
    J = rng.integers(1, n + 1, k)
    V = rng.standard_normal(k, dtype=np.float32)
    Id, Jd = torch.from_numpy(I).cuda(), torch.from_numpy(J).cuda()
    Vd = torch.from_numpy(V).cuda()
    A = dev.coo_assemble(m, n, Id, Jd, Vd, orient="csc")  # warm-up (and the stored count)
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        dev.coo_assemble(m, n, Id, Jd, Vd, orient="csc")  # synchronous: returns the count
    ms = 1e3 * (time.perf_counter() - t0) / reps
    nbytes = k * (8 + 8 + 4) + A.nnz * (4 + 4) + 4 * (n + 1)
    sample = 2_000_000
    t_cpu = _cpu_time(lambda: oracle.coo_assemble(m, n, I[:sample], J[:sample], V[:sample]),
                      min_seconds=2.0, max_reps=3)
    cpu_bytes = sample * (8 + 8 + 4) + sample * (4 + 4) + 4 * (n + 1)
    return [{"suite": "coo_assemble_16M", "metric": "coo_assemble_gbps", "unit": "GB/s",
             "value": round(nbytes / (ms / 1e3) / 1e9, 1), "ms_per_call": round(ms, 3),
             "triplets": k, "stored": int(A.nnz), "dtype": "f32",
             "config": {"workload": "1M x 1M, 16M uniform Int64 (row, col) triplets, N(0,1) FP32, + on duplicates"},
             "timing": "host wall time of the synchronous call (sort, fold, ptr, count readback)",
             "roofline": _roof(nbytes, ms),
             "cpu_baseline": {"value": round(cpu_bytes / t_cpu / 1e9, 3), "unit": "GB/s", "cores": 1,
                              "kind": "port",
                              "sample": "first 2M triplets, fsparse contract (oracle stable merge sort + fold)"}}]


def suite_spgemm() -> list[dict]:
    """C = A * A for the 2048^2 5-point Poisson matrix (FP64, CSR), Gustavson."""
    import torch

    import oracle
    from finchgb import device as dev
    from finchgb.workloads import poisson2d

    P = poisson2d(2048)
    A = dev.DeviceSparse.from_host(P.nrows, P.ncols, P.ptr, P.idx, P.val, orient="csr")
    C = dev.spgemm(A, A)
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        dev.spgemm(A, A)  # synchronous: symbolic, allocation, numeric, row sort
    ms = 1e3 * (time.perf_counter() - t0) / reps
    products = int(np.sum(np.diff(P.ptr)[P.idx - 1] * 1))  # sum over entries of |row k|
    nbytes = 2 * (12 * P.nnz + 8 * (P.nrows + 1)) + 12 * C.nnz + 8 * (P.nrows + 1)
    rows = 200_000
    t = _cpu_time(lambda: oracle.spgemm_csr(rows, P.ncols, P.ptr[: rows + 1], P.idx, P.val, P.ptr,
                                            P.idx, P.val), min_seconds=2.0, max_reps=3)
    t_full = t * P.nrows / rows
    return [{"suite": "spgemm_poisson2048_squared", "metric": "spgemm_products_per_s", "unit": "Gproducts/s",
             "value": round(products / (ms / 1e3) / 1e9, 3), "ms_per_call": round(ms, 3),
             "products": products, "nnz_A": int(P.nnz), "nnz_C": int(C.nnz), "dtype": "f64",
             "config": {"workload": "2048^2 5-point Poisson CSR (FP64) times itself"},
             "timing": "host wall time of the synchronous symbolic + numeric calls",
             "roofline": _roof(nbytes, ms),
             "cpu_baseline": {"value": round(products / t_full / 1e9, 4), "unit": "Gproducts/s",
                              "cores": 1, "kind": "port",
                              "sample": "rows 1..200000 (Gustavson nest, oracle), scaled by rows"}}]


def run_suite(args):
    from finchgb import build

    build.build()
    for fn in (suite_spmv_fp64, suite_semiring, suite_cg, suite_sddmm, suite_coo, suite_spgemm, suite_cg_probe,
               suite_pagerank, suite_spmv_adaptive):
        if args.suite_only and fn.__name__ not in args.suite_only.split(","):
            continue
        try:
            for line in fn():
                print(json.dumps(line), flush=True)
        except Exception as e:  # report and continue with the next configuration
            print(json.dumps({"suite": fn.__name__, "error": repr(e)}), flush=True)


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
    ap.add_argument("--headline-only", action="store_true",
                    help="only the SpMM line: no suite or served blocks")
    ap.add_argument("--sweep", action="store_true", help="print the autotune table to stderr")
    ap.add_argument("--schedule", default="", help="fixed LANES,PATH instead of the autotune")
    ap.add_argument("--suite", action="store_true",
                    help="measure the other configurations (one JSON line each) instead")
    ap.add_argument("--suite-only", default="", help="comma-separated suite function names")
    ap.add_argument("--serve", action="store_true", help="the batched/served configuration")
    ap.add_argument("--requests", type=int, default=20000)
    args = ap.parse_args()
    if args.serve:
        run_serve(args)
    elif args.suite:
        run_suite(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
