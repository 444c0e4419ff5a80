#!/usr/bin/env python3
"""Benchmark of the GB300 LBL path on the symmetric-indefinite KKT workload
K = [H A^T; A -1e-8 I], H = 3D 7-point Laplacian on 64^3 (n = 262,144), A =
20,000 x n with 6 random N(0,1) entries per row, rhs ~ N(0,1) (N = 282,144),
seeded synthetic data.

One step = one KKT solve to a relative residual below 1e-10: numeric
supernodal Bunch-Kaufman LDL^T factorization (FP32 factor, diagonal floor for
FP32) + supernodal solves + FP64 GMRES refinement on the unperturbed matrix.
The symbolic analysis (ordering, supernodes) is per sparsity pattern and runs
once, outside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput (matrix
values and rhs already in HBM); `e2e` is the same through the C ABI with host
buffers (matrix values and rhs copied in, solution copied out, every step);
`plain_fp64` is the FP64 factorization path on the same GPU; `cpu_baseline`
is the oracle restatement (reference algorithm over OpenBLAS) on the host
cores.  For N > 1 (torchrun) every rank solves its own replica: the path has
no data exchange to shard.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QP solves/sec at 1e-8 KKT tol: mixed+batched+warm-start vs plain GPU FP64"
GRID, MCON, PER_ROW, DELTA, SEED = 64, 20000, 6, 1e-8, 0
SAMPLE_GRID, SAMPLE_M = 48, 8000          # CPU baseline sample of the same family (~9% of the flops)
TARGET_RELRES = 1e-10
# DRAM bytes (read + write) per launch of the dominant kernel classes, scaled
# from one ncu capture of the 48^3 / m=8000 case of this workload family (see
# profiles/); None where no capture exists yet
NCU_TRAFFIC = {}
INNER = 8  # cap on the FGMRES inner steps of the refinement (one restart)
STOP_REL = 1e-12  # FGMRES stops once its residual estimate is below STOP_REL * ||b|| (100x under the target)


def workload_name(g, m):
    return f"lbl_kkt_lap3d_{g}cube_m{m}"


def sym_spmv(K, x):
    cols = np.repeat(np.arange(K.ncol), np.diff(K.p))
    y = np.zeros(K.ncol)
    np.add.at(y, K.i, K.x * x[cols])
    off = K.i != cols
    np.add.at(y, cols[off], K.x[off] * x[K.i[off]])
    return y


def relres(K, x, b):
    return float(np.linalg.norm(b - sym_spmv(K, x)) / np.linalg.norm(b))


def factor_flops(sym):
    w = np.diff(sym.super).astype(np.float64)
    r = np.diff(sym.lpi).astype(np.float64)
    # sum over supernodes of sum_{k<w} (r-k)^2
    return float(np.sum(w * r * r - r * w * (w - 1) + (w - 1) * w * (2 * w - 1) / 6.0))


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample():
    """Oracle restatement on the sample instance with all host threads."""
    from nasoq_gb300 import Symbolic
    from nasoq_gb300 import problems as P
    from oracle import port

    K, rhs = P.lbl_kkt(seed=SEED, grid3d=SAMPLE_GRID, m=SAMPLE_M, per_row=PER_ROW, delta=DELTA)
    sym = Symbolic(K.ncol, K.p, K.i)
    ax = K.x.copy()
    dg = K.p[:-1]
    ax[dg] = np.where(np.abs(ax[dg]) < 1e-9, 1e-9, ax[dg])
    threads = os.cpu_count() or 1
    port.set_threads(threads)
    t0 = time.perf_counter()
    out = port.solve(K.ncol, K.p, K.i, ax, K.x, sym, rhs, req_ref_iter=2, max_inner_iter=2)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "flops": factor_flops(sym), "threads": threads, "N": K.ncol,
            "relres": relres(K, out["x"], rhs), "factor_s": out["factor_s"], "solve_s": out["solve_s"]}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    from nasoq_gb300 import Symbolic
    from nasoq_gb300 import problems as P

    Kc, _ = P.lbl_kkt(seed=SEED, grid3d=args.grid, m=args.mcon, per_row=PER_ROW, delta=DELTA)
    F_full = factor_flops(Symbolic(Kc.ncol, Kc.p, Kc.i))
    for _ in range(args.warmup):
        cpu_sample()
    times, samples = [], []
    for _ in range(args.steps):
        s = cpu_sample()
        samples.append(s)
        times.append(s["seconds"])
    tot = sum(times)
    # flop-scaled to the full workload: seconds per full solve = F_full / (F_sample / t_sample)
    sec_full = statistics.median(times) * F_full / samples[0]["flops"]
    value = 1.0 / sec_full
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.grid, args.mcon), "N": Kc.ncol},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": samples[0]["threads"], "kind": "port",
                         "sample": f"each step: full factor + refined solve of the same KKT family at "
                                   f"{SAMPLE_GRID}^3 grid, m={SAMPLE_M} (N={samples[0]['N']}, "
                                   f"F={samples[0]['flops']:.3e}); value scaled to the full workload by "
                                   f"F_full={F_full:.3e}",
                         "sample_gflops": samples[0]["flops"] / statistics.median(times) / 1e9},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU comparison step")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--grid", type=int, default=GRID, help="Laplacian grid edge (smaller cases for profiler captures)")
    ap.add_argument("--mcon", type=int, default=MCON, help="constraint rows")
    ap.add_argument("--profile-once", action="store_true",
                    help="analysis + exactly one timed step and nothing else (for profiler launch lists)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    import nasoq_gb300 as nq
    from nasoq_gb300 import problems as P

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()

    K, rhs = P.lbl_kkt(seed=SEED, grid3d=args.grid, m=args.mcon, per_row=PER_ROW, delta=DELTA)
    n = K.ncol
    # FGMRES residual estimates are of the true residual b - K x: stop at
    # STOP_REL * ||b|| (tol_rel = 1 leaves the absolute bound in charge)
    st32 = nq.default_settings(precision=nq.NQG_FP32, solve_precision=nq.NQG_FP32, req_ref_iter=1,
                               max_inner_iter=INNER, tol_abs=STOP_REL * float(np.linalg.norm(rhs)), tol_rel=1.0,
                               reg_diag=1e-9)
    t0 = time.perf_counter()
    plan = nq.Plan(n, K.p, K.i, K.x, settings=st32)
    analysis_s = time.perf_counter() - t0
    plan.set_stream(stream.cuda_stream)
    F = factor_flops(plan.symbolic)
    d_rhs = torch.from_numpy(rhs).cuda()
    d_x = torch.empty(n, dtype=torch.float64, device="cuda")

    def step():
        plan.factor()
        plan.solve_device(d_rhs.data_ptr(), d_x.data_ptr())

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    if args.profile_once:
        barrier()
        t1 = time.perf_counter()
        step()
        barrier()
        print(json.dumps({"profile_once_step_s": time.perf_counter() - t1, "launches": plan.launch_count()}))
        plan.close()
        return 0
    for _ in range(args.warmup):
        step()
    barrier()
    l0 = plan.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    launches = (plan.launch_count() - l0) / max(args.steps, 1)
    t_ms = ev0.elapsed_time(ev1)
    if world > 1:
        tt = torch.tensor([t_ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(tt.item())
    value = world * args.steps / (t_ms / 1000.0)
    x32 = d_x.cpu().numpy()
    rr32 = relres(K, x32, rhs)
    inner_used = plan.timings().num_ref_iter

    # end to end through the C ABI with host buffers (values + rhs in, x out)
    ax = np.ascontiguousarray(K.x)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plan.set_values(ax)
    plan.factor()
    xh = plan.solve(rhs)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        plan.set_values(ax)
        plan.factor()
        xh = plan.solve(rhs)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_value = world * args.steps / (e2e_ms / 1000.0)

    # per-kernel-class device time over identical steps (CUDA events per launch)
    plan.set_profiling(True)
    for _ in range(2):
        step()
    stats = plan.kernel_stats()
    plan.set_profiling(False)
    torch.cuda.synchronize()

    # plain FP64 factorization path on the same GPU
    fp64 = None
    if not args.no_fp64:
        st64 = nq.default_settings(precision=nq.NQG_FP64, req_ref_iter=1, max_inner_iter=2, tol_abs=0.0,
                                   tol_rel=0.0, reg_diag=1e-9)
        p64 = nq.Plan(n, K.p, K.i, K.x, settings=st64)
        p64.set_stream(stream.cuda_stream)
        d_x64 = torch.empty(n, dtype=torch.float64, device="cuda")
        p64.factor()
        p64.solve_device(d_rhs.data_ptr(), d_x64.data_ptr())
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        p64.factor()
        p64.solve_device(d_rhs.data_ptr(), d_x64.data_ptr())
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1)
        x64 = d_x64.cpu().numpy()
        fp64 = {"value": 1000.0 / ms64, "unit": "solves/s", "ms_per_step": ms64, "relres": relres(K, x64, rhs),
                "steps": 1}
        err_vs_fp64 = float(np.linalg.norm(x32 - x64) / np.linalg.norm(x64))
        p64.close()
        del d_x64
    else:
        err_vs_fp64 = None

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    dom = max(stats, key=lambda k: stats[k]["total_ms"])
    ds = stats[dom]
    avg_ms = ds["total_ms"] / max(ds["launches"], 1)
    if dom in ("solve", "spmv", "pack"):
        ach = ds["alg_bytes"] / (ds["total_ms"] / 1000.0) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak}
    else:
        ach = ds["alg_flops"] / (ds["total_ms"] / 1000.0) / 1e12
        # FP32 CUDA-core work measured against the measured dense bf16 tensor peak
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s", "frac": ach / bf16_peak,
                "fp32_cuda_core_nominal_tflops": 80.5, "frac_of_fp32_nominal": ach / 80.5}
    roof.update({"kernel": dom, "launches_per_step": ds["launches"] / 2, "avg_launch_ms": avg_ms,
                 "traffic": NCU_TRAFFIC.get(dom), "peak_source": "MEASURED_PEAKS.json" if peaks else "fallback"})
    # every class: factor classes against the measured tensor peak (the tcgen05
    # classes do 3 split-TF32 MMAs per useful multiply-add), solves and SpMV
    # against the measured copy bandwidth
    by_class = {}
    for k, v in stats.items():
        sec = v["total_ms"] / 1000.0
        if sec <= 0:
            continue
        if k in ("solve", "spmv", "pack"):
            a = v["alg_bytes"] / sec / 1e9
            by_class[k] = {"bound": "hbm", "achieved": a, "unit": "GB/s", "frac": a / hbm_peak}
        else:
            a = v["alg_flops"] / sec / 1e12
            e = {"bound": "tensor", "achieved": a, "unit": "TFLOP/s", "frac": a / bf16_peak}
            if k in ("update", "wide_trailing"):
                e["mma_tflops"] = 3 * a
            by_class[k] = e
    roof["by_class"] = by_class
    kinfo = {k: {"ms_per_step": v["total_ms"] / 2, "launches_per_step": v["launches"] / 2} for k, v in stats.items()}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            s = cpu_sample()
            sec_full = s["seconds"] * F / s["flops"]
            cpu = {"value": 1.0 / sec_full, "unit": "solves/s", "cores": s["threads"], "kind": "port",
                   "sample": f"full factor + refined solve of the same KKT family at {SAMPLE_GRID}^3 grid, "
                             f"m={SAMPLE_M} (N={s['N']}, F={s['flops']:.3e}) in {s['seconds']:.2f}s; value "
                             f"scaled to the full workload by F_full={F:.3e}",
                   "sample_gflops": s["flops"] / s["seconds"] / 1e9, "sample_relres": s["relres"]}
        except Exception as e:  # the CPU baseline must not hide the GPU line
            cpu = {"value": None, "unavailable": str(e)[:200]}

    if rank == 0:
        h2d = K.x.nbytes + rhs.nbytes
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32-factor+fp64-refine", "data": "synthetic",
            "config": {"workload": workload_name(args.grid, args.mcon), "N": n, "nnz_K_lower": int(K.nnz),
                       "seed": SEED, "delta": DELTA, "factor_flops": F, "precision": "fp32 factor and triangular solves, fp64 flexible GMRES-IR",
                       "refinement": f"FGMRES, 1 restart, stop at residual {STOP_REL:g}*||b|| (at most {INNER} "
                                     f"inner steps; {inner_used} used)", "target_relres": TARGET_RELRES,
                       "l2": "inputs larger than L2 (FP32 factor 4 GB)", "analysis_s": analysis_s,
                       "parallelism": f"replicas x{world}"},
            "relres": rr32, "meets_target": bool(rr32 <= TARGET_RELRES), "error_vs_fp64_gpu": err_vs_fp64,
            "plain_fp64": fp64,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(n * 8), "ms_per_step": e2e_ms / args.steps},
            "roofline": roof, "kernels": kinfo, "cpu_baseline": cpu, "clocks": clk.summary(),
            "gpu_launches": int(round(launches)),
        }
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
