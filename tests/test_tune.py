"""The batched solver's launch-shape autotuner (host logic, no GPU): it picks
the fastest candidate among those that solve as many QPs as the best one,
stores the choice under the batch's size profile, and reuses it."""
import json

import pytest

import nasoq_gb300 as nq
from nasoq_gb300 import problems as P
from nasoq_gb300 import tune


def _probs(horizons):
    out = []
    for k, N in enumerate(horizons):
        q = P.qp_mpc(seed=k, horizon=N)
        out.append((q.H, q.q, q.A, q.b, q.C, q.d))
    return out


def test_autotune_picks_fastest_complete_candidate_and_caches(tmp_path):
    probs = _probs([10, 12, 30])
    cache = str(tmp_path / "tune.json")
    table = {(128, 0): (5.0, 3), (64, 0): (3.0, 2), (256, 0): (4.0, 3), (128, 1): (6.0, 3)}
    calls = []

    def timer(problems, s):
        calls.append((s.threads, s.stage))
        return table[(s.threads, s.stage)]

    s, rep = tune.autotune_batch(probs, cache=cache, timer=timer, variant=0, eps_abs=1e-8,
                                 precision=nq.NQG_FP32, refine=1)
    # (64, 0) is fastest but solved fewer QPs
    assert (s.threads, s.stage) == (256, 0) and not rep["cached"]
    assert s.qp.precision == nq.NQG_FP32 and s.refine == 1 and s.qp.eps_abs == 1e-8
    assert len(calls) == 4
    saved = json.load(open(cache))
    assert saved[rep["key"]]["threads"] == 256

    def no_timer(problems, s):
        raise AssertionError("cached choice must not be timed again")

    s2, rep2 = tune.autotune_batch(probs, cache=cache, timer=no_timer, variant=0, eps_abs=1e-8,
                                   precision=nq.NQG_FP32, refine=1)
    assert rep2["cached"] and (s2.threads, s2.stage) == (256, 0)
    # another size profile or other settings: another key
    assert tune.profile_key(_probs([10, 12, 60]), s) != rep["key"]
    assert tune.profile_key(probs, nq.batch_settings(precision=nq.NQG_FP64)) != rep["key"]


@pytest.mark.gpu
def test_autotune_times_real_candidates(tmp_path):
    probs = _probs([10, 20, 40, 80] * 16)
    s, rep = tune.autotune_batch(probs, cache=str(tmp_path / "t.json"), variant=0, eps_abs=1e-8,
                                 precision=nq.NQG_FP32, refine=1, refine_tol=1e-12)
    assert len(rep["trials"]) == len(tune.CANDIDATES)
    assert all(t["optimal"] == len(probs) for t in rep["trials"])
    b = nq.QPBatch(probs, settings=s)
    b.solve()
    assert all(st.status == 1 for st in b.results()[-1])
    assert b.info().threads == s.threads
    b.close()
