#!/usr/bin/env python3
"""Benchmark: QP solves/s at a 1e-8 KKT tolerance of the mixed-precision,
batched, learned-warm-start NASOQ path on one GB300, against the plain FP64
GPU path and the reference's CPU method.

Workload (seeded synthetic; the reference's benchmark suites are not
available): the parametric MPC family at horizon 50 (n = 450, 300 equality
rows, 900 box rows), q = P theta, box shifts S theta, theta in R^32 ~ N(0, I),
P and S dense N(0, 0.1) (nasoq_gb300.problems.mpc_parametric).  One step = one
batch of 4096 fresh theta: model logits on the GPU, warm-start sets, and the
batched NASOQ solve (one CTA per QP; the batch's QPs share one cold
factorization of their common KKT matrix), FP32 factorization with FP64
flexible GMRES refinement, every QP checked at eps_abs = 1e-8 and only those
that meet it counted.  The active-set model is
trained at start-up by the library's own kernels on plain-NASOQ solves of
200k random theta (outside the timed region; reported).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value`: device-resident throughput (theta,
q and d already in HBM; model forward, warm start and solve timed with CUDA
events); `e2e`: the same through the C ABI from host buffers (q, d computed
from theta on the host and copied in, x copied out, every step);
`plain_fp64_batched`: the same batches solved by the plain FP64 path (FP64
factor, the reference's refinement schedule, cold start) on the same GPU;
`plain_fp64_single`: the per-QP FP64 GPU path (one problem at a time, host
loop over the C ABI) on a sample; `cpu_baseline`: the oracle restatement of
the reference's method on the host cores.  Secondary sections: `c3`, the
uneven MPC batch (4096 problems, horizons 10..100, launch shape from the
autotuner), `lbl_c2`, the symmetric-indefinite KKT solve of the 64^3
Laplacian workload, and `c5`, the 400 x 400 bounded bilaplacian QP through
the single-QP path (time-boxed; --c5-full solves it to the end).  For N > 1
(torchrun) every rank solves its own batches (no data exchange).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
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
BATCH = 4096
EPS = 1e-8
N_TRAIN = 200_000
REFINE_TOL = 1e-10  # FGMRES target of the mixed path: swept 1e-12..1e-10, every QP Optimal, max lag ~1e-9
THETA_SEED = 20261204
WS_THRESHOLD = 1.5  # logit above which a constraint is proposed (swept 0..5: 1.0-1.5 fastest, every QP optimal)
TRAIN_EPOCHS = 60   # swept 20 / 60: 60 epochs (10 s) cut warm-start drops from 5.0 to 2.9 per QP
CPU_SAMPLE_PER_PROC = 48
# DRAM bytes (read + write) of one batch-kernel launch on this workload, from
# an ncu capture of the measured step of --profile-once (4096 QPs):
# profiles/dram_k_nasoq_batch_mpc50_warm4096.md
NCU_BATCH_TRAFFIC = 3_725_971_200 + 2_870_434_304
# LBL section: K = [H A^T; A -1e-8 I], H 3D 7-point Laplacian on 64^3, A 20000 x n, 6 N(0,1) per row
GRID, MCON, PER_ROW, DELTA, SEED = 64, 20000, 6, 1e-8, 0
TARGET_RELRES = 1e-10
LBL_INNER, LBL_STOP_REL = 8, 1e-12


# ---------------------------------------------------------------------------
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
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "MEASURED_PEAKS.json"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def thetas_for(step, rank):
    return np.random.default_rng([THETA_SEED, rank, step]).standard_normal((BATCH, 32))


def set_batch(b):
    global BATCH
    BATCH = int(b)


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement of the reference's method (cold start),
# one single-threaded process per host core, each on its own slice.
def _cpu_worker(args):
    start, count, step = args
    import nasoq_gb300 as nq
    from nasoq_gb300 import problems as P
    from oracle import port

    port.set_threads(1)
    fam = P.mpc_parametric(0)
    th = np.random.default_rng([THETA_SEED, 7777, step]).standard_normal((start + count, 32))[start:]
    N, Kp, Ki, _ = port.super_kkt(fam.base)
    ex = np.zeros(N, np.int32)
    ex[fam.base.n + fam.base.A.nrow:] = 1
    sym = nq.Symbolic(N, Kp, Ki, extra_cols=ex)
    t0 = time.perf_counter()
    ok = 0
    iters = 0
    for t in th:
        qp = P.QP(fam.base.H, fam.q_of(t), fam.base.A, fam.base.b, fam.base.C, fam.d_of(t))
        r = port.qp_solve(qp, variant=0, eps_abs=EPS, sym=sym)
        ok += r["status"] == 1
        iters += r["num_iter"]
    return time.perf_counter() - t0, ok, iters


def cpu_qp_sample(step=0, per_proc=CPU_SAMPLE_PER_PROC):
    procs = os.cpu_count() or 1
    jobs = [(i * per_proc, per_proc, step) for i in range(procs)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_worker, jobs)
    wall = time.perf_counter() - t0
    n = procs * per_proc
    slowest = max(r[0] for r in res)
    return {"value": n / slowest, "unit": "QP solves/s", "cores": procs, "kind": "port", "wall_seconds": wall,
            "sample": f"{n} QPs of the same family ({per_proc} per process, fresh theta), one single-threaded "
                      f"process per host core, cold start (the reference's method), eps_abs={EPS:g}; value = "
                      f"QPs / solve time of the slowest process ({slowest:.2f}s; {wall:.2f}s with process start)",
            "optimal_fraction": sum(r[1] for r in res) / n, "mean_iterations": sum(r[2] for r in res) / n,
            "per_process_seconds": max(r[0] for r in res)}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    for w in range(args.warmup):
        cpu_qp_sample(step=1000 + w, per_proc=8)
    vals, samples = [], []
    for k in range(args.steps):
        s = cpu_qp_sample(step=k)
        samples.append(s)
        vals.append(s["value"])
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "QP solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * statistics.mean(s["wall_seconds"] for s in samples),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "qp_mpc50_parametric_theta32", "batch": BATCH, "eps_abs": EPS,
                       "variant": "Fixed", "warm_start": "none (the reference's method)"},
            "cpu_baseline": dict(samples[0], value=value),
            "e2e": {"value": value, "unit": "QP solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def qp_section(args, world, rank, local, torch, nq, P, learn, pk, pk_src):
    fam = P.mpc_parametric(0)
    n, mi = fam.base.n, fam.base.C.nrow
    # model: trained on plain-NASOQ solves (outside the timed region), or
    # weights saved by an earlier run (profiler captures skip the training)
    if args.load_model:
        z = np.load(args.load_model)
        model = nq.MLP(tuple(int(v) for v in z["sizes"]))
        model.set_weights(z["w"], z["b"])
        rep = learn.TrainReport(int(z["n_train"]), 0.0, 0.0, [float(v) for v in z["losses"]], float(z["active"]))
    else:
        model, rep = learn.train_model(fam, n_train=args.n_train, seed=11 + rank, epochs=TRAIN_EPOCHS, batch=1024,
                                       lr=1e-3,
                                       solver=dict(variant=0, eps_abs=EPS, precision=nq.NQG_FP32, refine=1,
                                                   refine_tol=REFINE_TOL))
        if args.save_model and rank == 0:
            w, b = model.get_weights()
            np.savez(args.save_model, sizes=np.array(model.sizes), w=w, b=b, n_train=rep.n_train,
                     losses=np.array(rep.losses), active=rep.active_mean)
    mixed = dict(variant=0, eps_abs=EPS, precision=nq.NQG_FP32, refine=1, refine_tol=REFINE_TOL)
    batch = learn.family_batch(fam, BATCH, **mixed)
    ws = learn.WarmStarter(batch, model, fam, threshold=WS_THRESHOLD)
    bstream = torch.cuda.ExternalStream(batch.stream())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def device_step(thetas):
        """Inputs made resident first (untimed), then forward + warm start + solve timed on the batch stream."""
        learn.set_theta(batch, fam, thetas)
        ws.d_theta.copy_(torch.from_numpy(np.ascontiguousarray(thetas, np.float32)))
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(bstream)
        model.forward_device(BATCH, ws.d_theta.data_ptr(), ws.d_logits.data_ptr(), stream=batch.stream())
        batch.warm_start_from_scores(ws.d_logits.data_ptr(), mi, WS_THRESHOLD)
        batch.solve_async()
        e1.record(bstream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    def e2e_step(thetas):
        """Host theta in, host x out, through the C ABI."""
        t0 = time.perf_counter()
        learn.set_theta(batch, fam, thetas)           # q, d from theta on the host, copied in
        ws.propose(thetas)                            # theta copied in, model logits, warm-start sets
        batch.solve()
        x, _, z, st = batch.results()                 # x, z and statistics copied out
        return (time.perf_counter() - t0) * 1e3, x, z, st

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for w in range(args.warmup):
        device_step(thetas_for(10_000 + w, rank))
    barrier()
    if args.profile_once:  # exactly one measured step, for profiler launch lists
        ms1 = device_step(thetas_for(0, rank))
        print(json.dumps({"profile_once_ms": ms1, "batch": BATCH}), flush=True)
        return None
    with ClockSampler(local) as clk:
        barrier()
        ms, solved = [], 0
        for k in range(args.steps):
            ms.append(device_step(thetas_for(k, rank)))
            # QPs that met the tolerance (read after the timed region of the step)
            solved += sum(1 for s in batch.stats() if s.status == 1)
        barrier()
    t_ms = float(sum(ms))
    if world > 1:
        tt = torch.tensor([t_ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(tt.item())
        ts = torch.tensor([float(solved)], device="cuda")
        torch.distributed.all_reduce(ts)  # sum over ranks
        solved = int(ts.item())
    # solves/s counts only the QPs that met eps_abs
    value = solved / (t_ms / 1e3)
    _, _, _, st = batch.results()
    kernel_ms = batch.info().last_ms

    # end to end, one step at a time
    e2e_step(thetas_for(20_000, rank))
    e2e_ms, warm_stats = [], None
    for k in range(args.steps):
        ms_k, xw, zw, warm_stats = e2e_step(thetas_for(k, rank))
        e2e_ms.append(ms_k)
    e2e_seq_value = BATCH / (statistics.median(e2e_ms) / 1e3) * world

    # end to end, pipelined: two batches alternate, so that one step's host
    # work (q, d from theta) and copies (vectors and theta in, x, z and
    # statistics out) overlap the other's solve; page-locked host buffers per
    # batch, reused only after that batch's results were read
    batch2 = learn.family_batch(fam, BATCH, **mixed)
    ws2 = learn.WarmStarter(batch2, model, fam, threshold=WS_THRESHOLD)
    model2 = nq.MLP(tuple(model.sizes))  # one model per stream: the forward's activations are per model
    model2.set_weights(*model.get_weights())
    slots = []
    for bt, wst, mdl in ((batch, ws, model), (batch2, ws2, model2)):
        slots.append({"b": bt, "ws": wst, "model": mdl, "stream": torch.cuda.ExternalStream(bt.stream()),
                      "q": torch.empty((BATCH, n), dtype=torch.float64, pin_memory=True).numpy(),
                      "d": torch.empty((BATCH, mi), dtype=torch.float64, pin_memory=True).numpy(),
                      "th": torch.empty((BATCH, fam.P.shape[1]), dtype=torch.float32, pin_memory=True)})

    def submit(sl, thetas):
        np.matmul(thetas, fam.P.T, out=sl["q"])
        np.matmul(thetas, fam.S.T, out=sl["d"])
        sl["d"] += fam.d0[None, :]
        sl["b"].set_vectors_async(q_all=sl["q"].reshape(-1), d_all=sl["d"].reshape(-1))
        sl["th"].numpy()[:] = thetas
        with torch.cuda.stream(sl["stream"]):
            sl["ws"].d_theta.copy_(sl["th"], non_blocking=True)
        sl["model"].forward_device(BATCH, sl["ws"].d_theta.data_ptr(), sl["ws"].d_logits.data_ptr(),
                                   stream=sl["b"].stream())
        sl["b"].warm_start_from_scores(sl["ws"].d_logits.data_ptr(), mi, WS_THRESHOLD)
        sl["b"].solve_async()

    def pipelined(ks):
        ths = [thetas_for(k, rank) for k in ks]
        barrier()
        t0 = time.perf_counter()
        submit(slots[0], ths[0])
        out = None
        for j in range(1, len(ks)):
            submit(slots[j % 2], ths[j])
            out = slots[(j - 1) % 2]["b"].results()
        out = slots[(len(ks) - 1) % 2]["b"].results()
        return (time.perf_counter() - t0) * 1e3, out

    pipelined([30_000, 30_001, 30_002])  # warm-up: both batches' graphs captured
    kp = max(args.steps, 4)
    pipe_ms, (_, _, _, pipe_stats) = pipelined(list(range(kp)))
    pipe_ok = sum(1 for s_ in pipe_stats if s_.status == 1)
    e2e_value = BATCH * kp / (pipe_ms / 1e3) * world
    # page-locked buffers go before the second batch's stream: torch's host
    # allocator records the streams a buffer was copied on
    torch.cuda.synchronize()
    slots.clear()
    batch2.close()
    del ws2, model2
    th_last = thetas_for(args.steps - 1, rank)
    warm_it = np.array([s.num_iter for s in warm_stats])
    warm_ok = np.mean([s.status == 1 for s in warm_stats])
    lag_max = max(s.lag_res for s in warm_stats)
    cons_max = max(s.cons_sat_norm for s in warm_stats)
    compl_max = max(s.complementarity_infn for s in warm_stats)

    # the same batch cold (mixed precision), and plain FP64 batched (reference schedule, cold)
    def cold_run(settings):
        b = learn.family_batch(fam, BATCH, **settings)
        learn.set_theta(b, fam, th_last)
        b.solve()
        times = []
        for _ in range(2):
            b.solve()
            times.append(b.info().last_ms)
        x, _, z, s = b.results()
        b.close()
        return min(times), x, z, s

    cold_ms, xc, zc, sc = cold_run(mixed)
    # the plain FP64 GPU path: FP64 factor, the reference's refinement schedule,
    # cold start, every QP factoring its own KKT matrix
    f64_ms, x64, z64, s64 = cold_run(dict(variant=0, eps_abs=EPS, precision=nq.NQG_FP64, refine=0,
                                          share_factor=0))
    xr = np.abs(xw - x64).reshape(BATCH, n).max(axis=1) / np.maximum(np.abs(x64).reshape(BATCH, n).max(axis=1), 1)

    # plain FP64 single-QP path (host loop over the C ABI) on a sample
    single = None
    if not args.no_single:
        st64 = nq.qp_settings(variant=0, eps_abs=EPS, precision=nq.NQG_FP64)
        ns_ = args.single_sample
        t0 = time.perf_counter()
        its = []
        for t in th_last[:ns_]:
            x1, y1, z1, a1, r1 = nq.qp_solve(fam.base.H, fam.q_of(t), fam.base.A, fam.base.b, fam.base.C,
                                            fam.d_of(t), settings=st64)
            its.append(r1.num_iter)
        dt = time.perf_counter() - t0
        single = {"value": ns_ / dt, "unit": "QP solves/s", "sample": ns_, "mean_iterations": float(np.mean(its)),
                  "path": "nqg_qp_solve: host active-set loop, GPU FP64 factor / refactor / solve per iteration"}

    # error against the oracle (the reference's method restated, FP64) on a few problems
    oracle_err = None
    if rank == 0 and not args.no_cpu:
        try:
            from oracle import port
            N, Kp, Ki, _ = port.super_kkt(fam.base)
            ex = np.zeros(N, np.int32)
            ex[n + fam.base.A.nrow:] = 1
            sym = nq.Symbolic(N, Kp, Ki, extra_cols=ex)
            errs = []
            for i in range(8):
                t = th_last[i]
                qp = P.QP(fam.base.H, fam.q_of(t), fam.base.A, fam.base.b, fam.base.C, fam.d_of(t))
                r = port.qp_solve(qp, variant=0, eps_abs=EPS, sym=sym)
                xi = xw[i * n:(i + 1) * n]
                errs.append(float(np.linalg.norm(xi - r["x"]) / max(np.linalg.norm(r["x"]), 1e-300)))
            oracle_err = {"max_rel_x_error": max(errs), "problems": 8}
        except Exception as e:
            oracle_err = {"unavailable": str(e)[:200]}

    # roofline of the batch kernel: algorithmic bytes = factor entries read by
    # the triangular solves (forward + backward per preconditioner
    # application) plus the factor written by each refactorization
    batch.set_profiling(True)
    device_step(th_last)
    prof = batch.profile()
    batch.set_profiling(False)
    _, _, _, stp = batch.results()
    elt = 4  # FP32 factor
    sym_fam = _family_symbolic(nq, fam)
    xsize = int(sym_fam.colp[-1])
    applications = sum(s.solves + s.refine_steps for s in stp)
    sn_factored = prof["supernodes"]
    avg_sn_bytes = xsize * elt / max(len(sym_fam.super) - 1, 1)
    alg_bytes = applications * 2 * xsize * elt + sn_factored * avg_sn_bytes
    ach = alg_bytes / (batch.info().last_ms / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": ach, "peak": pk.get("hbm_gbs", 6800.0), "unit": "GB/s",
            "frac": ach / pk.get("hbm_gbs", 6800.0), "traffic": NCU_BATCH_TRAFFIC, "kernel": "k_nasoq_batch<float>",
            "launches_per_step": 1, "avg_launch_ms": batch.info().last_ms, "peak_source": pk_src,
            "algorithmic_bytes_per_launch": alg_bytes,
            "note": "one CTA per QP runs its whole active-set loop; bound by dependent on-chip latency, not DRAM",
            "phase_share": {k: prof[k] / max(prof["total"], 1) for k in
                            ("setup", "refactor", "precond", "spmv", "refine", "select", "update")}}
    out = {
        "value": value, "ms_per_step": t_ms / args.steps,
        "e2e": {"value": e2e_value, "unit": "QP solves/s",
                # in: q, d (FP64), theta (FP32), segment offsets; out: x, y, z (FP64) and the statistics
                "h2d_bytes_per_step": int(BATCH * ((n + mi) * 8 + 32 * 4 + 3 * 8)),
                "d2h_bytes_per_step": int(BATCH * ((n + fam.base.A.nrow + mi) * 8 + 88)),
                "ms_per_step": pipe_ms / kp, "steps": kp,
                "mode": "two batches alternating (one step's host work and copies overlap the other's solve)",
                "last_step_optimal": pipe_ok,
                "sequential": {"value": e2e_seq_value, "ms_per_step": statistics.median(e2e_ms),
                               "mode": "one step at a time: theta in, solve, x and z out"}},
        "check": {"optimal_fraction": float(warm_ok), "max_lag_res": lag_max, "max_cons_sat": cons_max,
                  "max_complementarity": compl_max, "eps_abs": EPS,
                  "max_rel_x_error_vs_fp64_gpu": float(xr.max()), "error_vs_oracle": oracle_err},
        "iterations": {"warm_mean": float(warm_it.mean()), "warm_max": int(warm_it.max()),
                       "cold_mean": float(np.mean([s.num_iter for s in sc])),
                       "warm_dropped_mean": float(np.mean([s.warm_dropped for s in warm_stats]))},
        "mixed_cold_batched": {"value": BATCH / (cold_ms / 1e3), "unit": "QP solves/s",
                               "optimal_fraction": float(np.mean([s.status == 1 for s in sc]))},
        "plain_fp64_batched": {"value": BATCH / (f64_ms / 1e3), "unit": "QP solves/s",
                               "optimal_fraction": float(np.mean([s.status == 1 for s in s64])),
                               "precision": "FP64 factor and solves, the reference's GMRES schedule, cold start, "
                                            "one factorization per QP (share_factor=0)"},
        "plain_fp64_single": single,
        "model": {"sizes": list(model.sizes), "n_train": rep.n_train, "label_seconds": rep.label_seconds,
                  "train_seconds": rep.train_seconds, "loss_first": rep.losses[0], "loss_last": rep.losses[-1],
                  "active_fraction": rep.active_mean},
        "roofline": roof, "clocks": clk.summary(), "kernel_ms": kernel_ms,
        "gpu_launches": 1 + (len(model.sizes) - 1) + 1,
    }
    batch.close()
    model.close()
    return out


def _family_symbolic(nq, fam):
    from nasoq_gb300 import problems as P  # noqa: F401
    b = fam.base
    n, meq, mi = b.n, b.A.nrow, b.C.nrow
    N = n + meq + mi
    cols = []
    for j in range(n):
        r = list(b.H.i[b.H.p[j]:b.H.p[j + 1]]) + [n + i for i in b.A.i[b.A.p[j]:b.A.p[j + 1]]] + \
            [n + meq + i for i in b.C.i[b.C.p[j]:b.C.p[j + 1]]]
        cols.append(r)
    for k in range(n, N):
        cols.append([k])
    Kp = np.cumsum([0] + [len(c) for c in cols]).astype(np.int32)
    Ki = np.concatenate([np.asarray(c, np.int32) for c in cols])
    ex = np.zeros(N, np.int32)
    ex[n + meq:] = 1
    return nq.Symbolic(N, Kp, Ki, extra_cols=ex)


def c3_section(nq, P):
    from nasoq_gb300 import tune
    qps = P.mpc_batch(BATCH, seed=0)
    probs = [(q.H, q.q, q.A, q.b, q.C, q.d) for q in qps]
    out = {"workload": "qp_mpc_uneven_horizon10-100_b4096"}
    for name, kw in (("mixed", dict(precision=nq.NQG_FP32, refine=1, refine_tol=REFINE_TOL)),
                     ("plain_fp64", dict(precision=nq.NQG_FP64, refine=0))):
        # launch shape from the autotuner (timed on this batch, or the choice
        # cached under the user's cache directory)
        tuned, trep = tune.autotune_batch(probs, variant=0, eps_abs=EPS, **kw)
        t0 = time.perf_counter()
        b = nq.QPBatch(probs, settings=tuned)
        fin = time.perf_counter() - t0
        b.solve()
        b.solve()
        ms = b.info().last_ms
        _, _, _, st = b.results()
        out[name] = {"value": BATCH / (ms / 1e3), "unit": "QP solves/s", "ms": ms,
                     "optimal_fraction": float(np.mean([s.status == 1 for s in st])),
                     "iterations_total": int(sum(s.num_iter for s in st)), "patterns": b.info().npatterns,
                     "setup_seconds": fin,
                     "launch": {"threads": tuned.threads, "stage": tuned.stage, "cached": trep["cached"],
                                "trials": trep.get("trials")}}
        b.close()
    return out


def c5_section(args, nq, P):
    """The large bounded QP: 400 x 400 jittered bilaplacian, 2000 pins, box
    rows (n = 160,000, 2000 equalities, 320,000 inequalities), through the
    single-QP path (host loop, every factorization / partial refactorization
    / solve on the GPU, FP64).  The reference's method adds one bound per
    iteration, so the full solve takes thousands of iterations: by default
    the run is time-boxed at --c5-iters iterations and reports the rate;
    --c5-full runs it to the end."""
    t0 = time.perf_counter()
    qp = P.bilaplacian_bounded(seed=0)
    gen_s = time.perf_counter() - t0
    out = {"workload": "bilaplacian_400x400_jitter0.2_pins2000_box", "n": qp.H.ncol, "meq": qp.A.nrow,
           "mineq": qp.C.nrow, "generate_seconds": gen_s}

    def run(cap):
        st = nq.qp_settings(variant=0, eps_abs=EPS, precision=nq.NQG_FP64, max_iter_nas=cap)
        t = time.perf_counter()
        x, y, z, act, r = nq.qp_solve(qp.H, qp.q, qp.A, qp.b, qp.C, qp.d, settings=st)
        wall = time.perf_counter() - t
        return {"iterations": r.num_iter, "seconds": wall, "status": r.status,
                "ms_per_iteration": 1e3 * wall / max(r.num_iter, 1), "gpu_factor_solve_seconds": r.factor_seconds,
                "active_set": r.active_size, "lag_res": r.lag_res, "cons_sat_norm": r.cons_sat_norm}

    # setup (analysis, first factorization, one iteration) and a time-boxed
    # run; the per-iteration time is the difference between the two
    first = run(0)
    boxed = run(args.c5_iters)
    boxed["ms_per_active_set_iteration"] = 1e3 * (boxed["seconds"] - first["seconds"]) / max(
        boxed["iterations"] - first["iterations"], 1)
    boxed["setup_seconds"] = first["seconds"]
    boxed["note"] = "stopped by max_iter_nas (the reference reports such a stop as status 0)"
    out["gpu_time_boxed"] = boxed
    if args.c5_full:
        out["gpu_full"] = run(200000)
    if args.c5_cpu_iters > 0:
        # the reference's method restated on the host (oracle), same start, time-boxed
        try:
            from oracle import port

            def cpu(cap):
                t = time.perf_counter()
                r = port.qp_solve(qp, variant=0, eps_abs=EPS, max_iter_nas=cap)
                return int(r["num_iter"]), time.perf_counter() - t

            i0, t0c = cpu(0)
            i1, t1c = cpu(args.c5_cpu_iters)
            out["cpu_time_boxed"] = {"iterations": i1, "seconds": t1c, "setup_seconds": t0c,
                                     "ms_per_active_set_iteration": 1e3 * (t1c - t0c) / max(i1 - i0, 1),
                                     "kind": "port", "threads": "OpenBLAS default"}
        except Exception as e:
            out["cpu_time_boxed"] = {"unavailable": str(e)[:200]}
    return out


def lbl_section(args, torch, nq, P, pk):
    """The symmetric-indefinite KKT solve (FP32 factor + FP64 FGMRES-IR)."""
    grid, mcon = args.lbl_grid, args.lbl_mcon
    K, rhs = P.lbl_kkt(seed=SEED, grid3d=grid, m=mcon, per_row=PER_ROW, delta=DELTA)
    n = K.ncol
    st32 = nq.default_settings(precision=nq.NQG_FP32, solve_precision=nq.NQG_FP32, req_ref_iter=1,
                               max_inner_iter=LBL_INNER, tol_abs=LBL_STOP_REL * float(np.linalg.norm(rhs)),
                               tol_rel=1.0, reg_diag=1e-9)
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    plan = nq.Plan(n, K.p, K.i, K.x, settings=st32)
    analysis_s = time.perf_counter() - t0
    plan.set_stream(stream.cuda_stream)
    d_rhs = torch.from_numpy(rhs).cuda()
    d_x = torch.empty(n, dtype=torch.float64, device="cuda")

    def step():
        plan.factor()
        plan.solve_device(d_rhs.data_ptr(), d_x.data_ptr())

    # the first factorization of a fresh plan starts from the fill-reducing
    # order (pivots not yet folded into it), as every step of the reference does
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan.factor()
    torch.cuda.synchronize()
    cold_factor_ms = 1000.0 * (time.perf_counter() - t0)
    plan.solve_device(d_rhs.data_ptr(), d_x.data_ptr())
    step()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = args.lbl_steps
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    x32 = d_x.cpu().numpy()
    cols = np.repeat(np.arange(n), np.diff(K.p))
    y = np.zeros(n)
    np.add.at(y, K.i, K.x * x32[cols])
    off = K.i != cols
    np.add.at(y, cols[off], K.x[off] * x32[K.i[off]])
    rr = float(np.linalg.norm(rhs - y) / np.linalg.norm(rhs))
    ref_iter = int(plan.timings().num_ref_iter)
    plan.set_profiling(True)
    step()
    stats = plan.kernel_stats()
    plan.set_profiling(False)
    oracle = None
    if args.lbl_oracle:
        # the reference's FP64 method (oracle restatement, all host cores) on
        # the same system, same ordering and supernodes; outside the timed region
        try:
            from oracle import port
            port.set_threads(os.cpu_count() or 1)
            diag = K.p[:-1]
            axp, axr = K.x.copy(), K.x.copy()
            small = np.abs(K.x[diag]) < 1e-9
            axp[diag[small]] = 1e-9
            axr[diag[small]] = 0.0
            t = time.perf_counter()
            o = port.solve(n, K.p, K.i, axp, axr, plan.symbolic, rhs, req_ref_iter=2, max_inner_iter=2)
            oracle = {"max_rel_x_error": float(np.linalg.norm(x32 - o["x"]) / np.linalg.norm(o["x"])),
                      "oracle_seconds": time.perf_counter() - t, "threads": os.cpu_count()}
        except Exception as e:
            oracle = {"unavailable": str(e)[:200]}
    plan.close()
    return {"workload": f"lbl_kkt_lap3d_{grid}cube_m{mcon}", "N": n, "value": 1000.0 / ms, "unit": "solves/s",
            "ms_per_step": ms, "relres": rr, "meets_target": bool(rr <= TARGET_RELRES), "analysis_s": analysis_s,
            "refine_iterations": ref_iter, "cold_factor_ms": cold_factor_ms,
            "operand_split": "tf32" if os.environ.get("NASOQ_GB300_SPLIT") == "tf32" else "bf16",
            "error_vs_oracle": oracle, "kernels_ms": {k: v["total_ms"] for k, v in stats.items()}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n-train", type=int, default=N_TRAIN)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-single", action="store_true", help="skip the single-QP FP64 sample")
    ap.add_argument("--single-sample", type=int, default=32)
    ap.add_argument("--no-c3", action="store_true")
    ap.add_argument("--no-lbl", action="store_true")
    ap.add_argument("--lbl-steps", type=int, default=3)
    ap.add_argument("--lbl-oracle", action="store_true",
                    help="also solve the LBL system with the oracle (FP64, host cores, ~1-2 min) for its error")
    ap.add_argument("--lbl-only", action="store_true", help="run the LBL section alone")
    ap.add_argument("--lbl-grid", type=int, default=GRID, help="LBL system: grid points per axis of the 3-D Laplacian")
    ap.add_argument("--lbl-mcon", type=int, default=MCON, help="LBL system: constraint rows")
    ap.add_argument("--batch", type=int, default=BATCH, help="QPs per step (smaller cases for profiler captures)")
    ap.add_argument("--profile-once", action="store_true",
                    help="train, then exactly one measured step and nothing else (profiler launch lists)")
    ap.add_argument("--no-c5", action="store_true")
    ap.add_argument("--c5-iters", type=int, default=150, help="active-set iterations of the time-boxed C5 run")
    ap.add_argument("--c5-full", action="store_true", help="also solve C5 to the end")
    ap.add_argument("--c5-cpu-iters", type=int, default=0, help="time-boxed oracle iterations on C5 (0: skip)")
    ap.add_argument("--c5-only", action="store_true", help="run the C5 section alone")
    ap.add_argument("--save-model", default=None, help="write the trained model's weights (.npz)")
    ap.add_argument("--load-model", default=None, help="use saved weights instead of training")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    import torch

    import nasoq_gb300 as nq
    from nasoq_gb300 import learn
    from nasoq_gb300 import problems as P

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pk, pk_src = peaks()
    set_batch(args.batch)
    if args.c5_only:
        if rank == 0:
            print(json.dumps({"c5": c5_section(args, nq, P)}), flush=True)
        return 0
    if args.lbl_only:
        if rank == 0:
            print(json.dumps({"lbl_c2": lbl_section(args, torch, nq, P, pk)}), flush=True)
        return 0
    qp = qp_section(args, world, rank, local, torch, nq, P, learn, pk, pk_src)
    if qp is None:
        return 0
    c3 = None if args.no_c3 else c3_section(nq, P)
    lbl = None if args.no_lbl else lbl_section(args, torch, nq, P, pk)
    c5 = None if args.no_c5 else c5_section(args, nq, P)
    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = cpu_qp_sample(step=0)
        except Exception as e:  # the CPU baseline must not hide the GPU line
            cpu = {"value": None, "unavailable": str(e)[:200]}
    if rank == 0:
        line = {
            "metric": METRIC, "value": qp["value"], "unit": "QP solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": qp["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32-factor+fp64-refine", "data": "synthetic",
            "config": {"workload": "qp_mpc50_parametric_theta32", "batch": BATCH, "n": 450, "meq": 300,
                       "mineq": 900, "eps_abs": EPS, "variant": "Fixed",
                       "precision": f"FP32 factor and triangular solves, FP64 flexible GMRES to {REFINE_TOL:g} relative "
                                    "residual, final polish on the active set",
                       "warm_start": f"learned (MLP 32-256-256-900, BF16 weights, FP32 accumulation; logit > "
                                     f"{WS_THRESHOLD:g} proposes a constraint)",
                       "l2": "256 MB written between timed steps (L2 flush)", "parallelism": f"replicas x{world}"},
            "e2e": qp["e2e"], "check": qp["check"], "iterations": qp["iterations"],
            "mixed_cold_batched": qp["mixed_cold_batched"], "plain_fp64_batched": qp["plain_fp64_batched"],
            "plain_fp64_single": qp["plain_fp64_single"], "model": qp["model"], "roofline": qp["roofline"],
            "cpu_baseline": cpu, "clocks": qp["clocks"], "gpu_launches": qp["gpu_launches"], "c3": c3,
            "lbl_c2": lbl, "c5": c5,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
