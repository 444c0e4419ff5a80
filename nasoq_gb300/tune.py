"""Launch-shape autotuner of the batched QP solver.

The batched kernel's CTA size (`threads`) and shared-memory staging
(`stage`) trade per-QP parallelism against resident CTAs per SM, and the
best choice depends on the problem sizes in the batch.  `autotune_batch`
times a solve of the actual batch under each candidate shape, keeps the
fastest one that solves every QP as well as the best-solving candidate, and
caches the choice on disk under a key made of the batch's size profile
(pattern sizes bucketed by powers of two) and the numeric settings, so the
next batch with the same profile reuses it without timing.
"""
from __future__ import annotations

import hashlib
import json
import math
import os
from collections import Counter

import nasoq_gb300 as nq

CANDIDATES = ((128, 0), (64, 0), (256, 0), (128, 1))
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "nasoq_gb300", "batch_tune.json")


def _bucket(v: int) -> int:
    return 0 if v <= 0 else 1 << int(math.ceil(math.log2(v)))


def profile_key(problems, settings: nq.BatchSettings) -> str:
    """Size profile of a batch (count of problems per bucketed (n, meq,
    mineq, nnz) tuple) plus the settings that change the work per QP."""
    prof = Counter()
    for (H, q, A, b, Cm, d) in problems:
        prof[(_bucket(H.ncol), _bucket(A.nrow), _bucket(Cm.nrow), _bucket(int(H.p[-1]) + int(A.p[-1]) + int(Cm.p[-1])))] += 1
    qs = settings.qp
    blob = json.dumps({"profile": sorted((list(k), v) for k, v in prof.items()),
                       "precision": qs.precision, "variant": qs.variant, "eps_abs": qs.eps_abs,
                       "refine": settings.refine, "refine_tol": settings.refine_tol}, sort_keys=True)
    return hashlib.sha1(blob.encode()).hexdigest()


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, table):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _time_batch(problems, settings, repeats=2):
    """(best kernel ms over `repeats` solves after one warm-up, Optimal count)."""
    b = nq.QPBatch(problems, settings=settings)
    try:
        b.solve()
        ms = []
        for _ in range(repeats):
            b.solve()
            ms.append(b.info().last_ms)
        _, _, _, st = b.results()
        return min(ms), sum(1 for s in st if s.status == 1)
    finally:
        b.close()


def autotune_batch(problems, settings: nq.BatchSettings | None = None, cache: str | None = DEFAULT_CACHE,
                   candidates=CANDIDATES, timer=_time_batch, **kw):
    """Returns (settings with the chosen threads / stage, report dict).

    `timer(problems, settings) -> (ms, optimal_count)` measures one
    candidate (replaceable for tests); `cache=None` disables the disk cache.
    """
    base = settings if settings is not None else nq.batch_settings(**kw)
    key = profile_key(problems, base)
    table = _load(cache) if cache else {}
    if key in table:
        hit = table[key]
        chosen = nq.batch_settings()
        _copy(base, chosen)
        chosen.threads, chosen.stage = int(hit["threads"]), int(hit["stage"])
        return chosen, {"key": key, "cached": True, **hit}
    trials = []
    for threads, stage in candidates:
        s = nq.batch_settings()
        _copy(base, s)
        s.threads, s.stage = threads, stage
        ms, ok = timer(problems, s)
        trials.append({"threads": threads, "stage": stage, "ms": float(ms), "optimal": int(ok)})
    best_ok = max(t["optimal"] for t in trials)
    pick = min((t for t in trials if t["optimal"] == best_ok), key=lambda t: t["ms"])
    chosen = nq.batch_settings()
    _copy(base, chosen)
    chosen.threads, chosen.stage = pick["threads"], pick["stage"]
    entry = {"threads": pick["threads"], "stage": pick["stage"], "ms": pick["ms"], "trials": trials}
    if cache:
        table[key] = entry
        _store(cache, table)
    return chosen, {"key": key, "cached": False, **entry}


def _copy(src: nq.BatchSettings, dst: nq.BatchSettings):
    for name, _ in nq.BatchSettings._fields_:
        if name == "qp":
            for qn, _ in nq.QPSettings._fields_:
                setattr(dst.qp, qn, getattr(src.qp, qn))
        else:
            setattr(dst, name, getattr(src, name))
