"""Learned active-set warm start for parametric QP families.

A family min 1/2 x'Hx + q(theta)'x s.t. Ax = b, Cx <= d(theta) keeps one
sparsity pattern; its plain NASOQ solves (the batched GPU solver, cold start)
label which inequalities are active at the optimum.  An MLP (nasoq_gb300.MLP,
the library's own CUDA kernels) learns theta -> active-set logits; for fresh
theta its logits seed the batched solve (nqg_batch_warm_start_from_scores),
whose active-set iteration corrects the guess and still decides the final
tolerance (reference Nasoq::set_warm_start, src/nasoq.cpp:413-436, is the
entry such a guess replaces).

Device buffers for theta and the logits are torch tensors (plumbing only).
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

import nasoq_gb300 as nq
from nasoq_gb300 import problems as P


def family_batch(fam: P.ParametricQP, count: int, **settings) -> nq.QPBatch:
    """A batch of `count` copies of the family's base problem (one pattern);
    its q / d are set per solve from theta."""
    b = fam.base
    one = (b.H, b.q, b.A, b.b, b.C, b.d)
    return nq.QPBatch([one] * count, settings=nq.batch_settings(**settings))


def set_theta(batch: nq.QPBatch, fam: P.ParametricQP, thetas: np.ndarray):
    """q = P theta, d = d0 + S theta for every problem of the batch."""
    q = thetas @ fam.P.T
    d = fam.d0[None, :] + thetas @ fam.S.T
    batch.set_vectors(q_all=q.ravel(), d_all=d.ravel())


def active_labels(z_all: np.ndarray, count: int, mineq: int) -> np.ndarray:
    """1 where the constraint's multiplier is positive at the optimum."""
    return (z_all.reshape(count, mineq) > 0.0).astype(np.float32)


def solve_labels(fam: P.ParametricQP, thetas: np.ndarray, chunk: int = 4096, **settings):
    """Plain NASOQ (cold start) on every theta; returns labels and statistics."""
    n_all = thetas.shape[0]
    chunk = min(chunk, n_all)
    batch = family_batch(fam, chunk, **settings)
    mineq = fam.base.C.nrow
    labels = np.zeros((n_all, mineq), np.float32)
    iters = np.zeros(n_all, np.int64)
    status = np.zeros(n_all, np.int64)
    for s0 in range(0, n_all, chunk):
        th = thetas[s0:s0 + chunk]
        if th.shape[0] < chunk:  # last partial chunk: pad with repeats
            th = np.concatenate([th, np.repeat(th[-1:], chunk - th.shape[0], axis=0)])
        set_theta(batch, fam, th)
        batch.solve()
        _, _, z, st = batch.results()
        m = min(chunk, n_all - s0)
        labels[s0:s0 + m] = active_labels(z, chunk, mineq)[:m]
        iters[s0:s0 + m] = [st[i].num_iter for i in range(m)]
        status[s0:s0 + m] = [st[i].status for i in range(m)]
    batch.close()
    return labels, iters, status


@dataclass
class TrainReport:
    n_train: int
    label_seconds: float
    train_seconds: float
    losses: list
    active_mean: float


def train_model(fam: P.ParametricQP, n_train: int, seed: int = 0, hidden=(256, 256), epochs: int = 20,
                batch: int = 1024, lr: float = 1e-3, pos_weight: float | None = None, solver=None):
    """Labels n_train random theta ~ N(0, I) with plain NASOQ and trains the
    MLP on them.  Returns (model, report)."""
    rng = np.random.default_rng(seed)
    p = fam.P.shape[1]
    thetas = rng.standard_normal((n_train, p)).astype(np.float64)
    t0 = time.time()
    labels, iters, status = solve_labels(fam, thetas, **(solver or dict(variant=0, eps_abs=1e-8)))
    t1 = time.time()
    keep = status == 1
    x, y = thetas[keep].astype(np.float32), labels[keep]
    if pos_weight is None:  # active constraints are rare: weight them by the class ratio (capped)
        pr = max(float(y.mean()), 1e-6)
        pos_weight = float(min((1.0 - pr) / pr, 50.0))
    model = nq.MLP((p,) + tuple(hidden) + (fam.base.C.nrow,), seed=seed)
    losses = model.fit(x, y, epochs=epochs, batch=batch, lr=lr, pos_weight=pos_weight, seed=seed)
    t2 = time.time()
    return model, TrainReport(int(keep.sum()), t1 - t0, t2 - t1, [float(v) for v in losses], float(y.mean()))


class WarmStarter:
    """Device buffers and calls of one warm-started batched solve: theta ->
    (model logits on the GPU) -> warm-start sets -> solve."""

    def __init__(self, batch: nq.QPBatch, model: nq.MLP, fam: P.ParametricQP, threshold: float = 0.0):
        import torch

        self.torch = torch
        self.batch, self.model, self.fam, self.threshold = batch, model, fam, float(threshold)
        n = len(batch)
        self.d_theta = torch.zeros((n, fam.P.shape[1]), dtype=torch.float32, device="cuda")
        self.d_logits = torch.zeros((n, fam.base.C.nrow), dtype=torch.float32, device="cuda")

    def propose(self, thetas: np.ndarray):
        """Model logits for thetas (host array), then the warm-start sets."""
        torch = self.torch
        self.d_theta.copy_(torch.from_numpy(np.ascontiguousarray(thetas, np.float32)))
        torch.cuda.synchronize()
        self.model.forward_device(thetas.shape[0], self.d_theta.data_ptr(), self.d_logits.data_ptr())
        self.batch.warm_start_from_scores(self.d_logits.data_ptr(), self.d_logits.shape[1], self.threshold)

    def solve(self, thetas: np.ndarray, warm: bool = True):
        set_theta(self.batch, self.fam, thetas)
        if warm:
            self.propose(thetas)
        else:
            self.batch.clear_warm_starts()
        self.batch.solve()
        return self.batch.results()
