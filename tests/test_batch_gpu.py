"""Batched QP solves (nqg_batch_*) against the reference NASOQ solving the
same problems one by one (tests/golden/batch_mixed.nqa, made by
tests/golden/gen_batch_golden.py): 64 MPC problems of uneven horizon
(10..100), 16 small random convex QPs whose iterations drop constraints, and
16 instances of the parametric MPC family sharing one sparsity pattern.  The
reference's Fixed variant at eps_abs = 1e-8.

FP64 with the reference's refinement schedule replays the reference's
decisions: the same status, iteration count and active set; x, y, z within
1e-7 (relative), the objective within 1e-9, KKT norms within eps_abs.  The
mixed-precision path (FP32 factorization and triangular solves, FP64 flexible
GMRES to a 1e-12 relative residual) must reach the same status with KKT
norms within eps_abs and x, z within 1e-6 of the reference; its iteration
counts are reported beside the reference's."""
import os

import numpy as np
import pytest

import nqa
import nasoq_gb300 as nq
from nasoq_gb300 import problems as P

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "batch_mixed.nqa")
KIND_MPC, KIND_RANDOM, KIND_PARAM = 0, 1, 2


def fixture():
    d = nqa.load(GOLD)
    sp = d["spec"].reshape(-1, 5)
    fam = P.mpc_parametric(0)
    qps = []
    for kind, a, b, c, e in sp.tolist():
        if kind == KIND_MPC:
            qp = P.qp_mpc(a, b)
        elif kind == KIND_RANDOM:
            qp = P.qp_random_convex(seed=a, grid=b, meq=c, mineq=e)
        else:
            th = np.random.default_rng(a).standard_normal(32)
            qp = P.QP(fam.base.H, fam.q_of(th), fam.base.A, fam.base.b, fam.base.C, fam.d_of(th))
        qps.append(qp)
    return d, qps


def part(d, name, i):
    p = d[name + "_ptr"]
    return d[name][p[i]:p[i + 1]]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / (nb if nb > 0 else 1.0)


def settings_of(d, **kw):
    return nq.batch_settings(variant=int(d["set_variant"][0]), eps_abs=float(d["set_eps_abs"][0]),
                             diag_perturb=float(d["set_diag_perturb"][0]), max_iter=int(d["set_max_iter"][0]),
                             stop_tol=float(d["set_stop_tol"][0]), max_iter_nas=int(d["set_max_iter_nas"][0]), **kw)


def test_batch_fixture_inputs_reproduce():
    """The seeded generators still produce the inputs the reference solved."""
    d, qps = fixture()
    for i, qp in enumerate(qps):
        assert P.qp_checksum(qp) == pytest.approx(float(d["checksum"][i]), rel=1e-13), f"problem {i}"


def _run(d, qps, **kw):
    b = nq.QPBatch([(q.H, q.q, q.A, q.b, q.C, q.d) for q in qps], settings=settings_of(d, **kw))
    b.solve()
    return b


@pytest.mark.gpu
@pytest.mark.parametrize("factor_path", ["auto", "warp", "cta"])
def test_batch_fp64_matches_reference(factor_path, monkeypatch):
    """The reference's status, iteration count, active set and solution for
    every problem of the batch fixture, with the supernodes factored by the
    launch's choice, level by level a warp each, or one at a time by the CTA."""
    if factor_path != "auto":
        monkeypatch.setenv("NASOQ_GB300_BATCH_WARP_FACTOR", "1" if factor_path == "warp" else "0")
    d, qps = fixture()
    b = _run(d, qps, precision=nq.NQG_FP64, refine=0)
    if factor_path != "auto":
        assert b.info().warp_factor == (1 if factor_path == "warp" else 0)
    eps = float(d["set_eps_abs"][0])
    assert b.info().npatterns < len(qps)  # the parametric instances share one pattern
    for i in range(len(qps)):
        x, y, z, act, res = b.result(i)
        assert res.status == int(d["status"][i]), f"problem {i}"
        assert res.num_iter == int(d["num_iter"][i]), f"problem {i}"
        assert sorted(act.tolist()) == sorted(part(d, "act", i).tolist()), f"problem {i}"
        assert rel(x, part(d, "x", i)) <= 1e-7, f"problem {i}"
        assert rel(z, part(d, "z", i)) <= 1e-7, f"problem {i}"
        if len(y):
            assert rel(y, part(d, "y", i)) <= 1e-7, f"problem {i}"
        ob = float(d["objective"][i])
        assert abs(res.objective - ob) <= 1e-9 * max(abs(ob), 1.0), f"problem {i}"
        assert res.lag_res <= eps and res.cons_sat_norm <= eps and res.non_negativity_infn <= eps
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("factor_path", ["auto", "warp", "cta"])
def test_batch_mixed_precision_meets_tolerance(factor_path, record_property, monkeypatch):
    if factor_path != "auto":
        monkeypatch.setenv("NASOQ_GB300_BATCH_WARP_FACTOR", "1" if factor_path == "warp" else "0")
    d, qps = fixture()
    b = _run(d, qps, precision=nq.NQG_FP32, refine=1, refine_tol=1e-12)
    eps = float(d["set_eps_abs"][0])
    differ = 0
    for i in range(len(qps)):
        x, y, z, act, res = b.result(i)
        assert res.status == int(d["status"][i]), f"problem {i}"
        assert res.lag_res <= eps and res.cons_sat_norm <= eps and res.non_negativity_infn <= eps, f"problem {i}"
        assert rel(x, part(d, "x", i)) <= 1e-6, f"problem {i}"
        assert rel(z, part(d, "z", i)) <= 1e-6, f"problem {i}"
        differ += res.num_iter != int(d["num_iter"][i])
    record_property("iteration_counts_differing", differ)
    print(f"mixed precision: {differ} of {len(qps)} iteration counts differ from the reference's")
    b.close()


@pytest.mark.gpu
def test_batch_repeat_and_new_vectors():
    """A second solve (graph replay) makes the same decisions (iteration
    counts) and the same solution to 1e-12 (the triangular solves push with
    atomics, so the last bits may differ between runs); new q / d for the
    parametric instances give the results of a batch built with them."""
    d, qps = fixture()
    sel = [q for q, k in zip(qps, d["spec"].reshape(-1, 5)[:, 0]) if k == KIND_PARAM]
    b = _run(d, sel, precision=nq.NQG_FP64, refine=0)
    x1, y1, z1, s1 = b.results()
    b.solve()
    x2, y2, z2, s2 = b.results()
    assert [s.num_iter for s in s1] == [s.num_iter for s in s2]
    assert rel(x2, x1) <= 1e-12 and rel(z2, z1) <= 1e-12
    fam = P.mpc_parametric(0)
    ths = [np.random.default_rng(5000 + t).standard_normal(32) for t in range(len(sel))]
    b.set_vectors(q_all=np.concatenate([fam.q_of(t) for t in ths]), d_all=np.concatenate([fam.d_of(t) for t in ths]))
    b.solve()
    x3, _, z3, s3 = b.results()
    fresh = [P.QP(fam.base.H, fam.q_of(t), fam.base.A, fam.base.b, fam.base.C, fam.d_of(t)) for t in ths]
    b2 = _run(d, fresh, precision=nq.NQG_FP64, refine=0)
    x4, _, z4, s4 = b2.results()
    assert rel(x3, x4) <= 1e-12 and rel(z3, z4) <= 1e-12
    assert [s.num_iter for s in s3] == [s.num_iter for s in s4]
    b.close()
    b2.close()


@pytest.mark.gpu
def test_batch_warm_start_from_solution():
    """Warm start from each problem's own final active set: the solution is
    reached again in (almost) no iterations, with the same x."""
    d, qps = fixture()
    b = _run(d, qps, precision=nq.NQG_FP64, refine=0)
    for i in range(len(qps)):
        b.set_warm_start(i, part(d, "act", i))
    b.solve()
    eps = float(d["set_eps_abs"][0])
    for i in range(len(qps)):
        x, y, z, act, res = b.result(i)
        assert res.status == 1, f"problem {i}"
        assert res.num_iter <= 1, f"problem {i}: {res.num_iter} iterations after a warm start at the solution"
        assert rel(x, part(d, "x", i)) <= 1e-7, f"problem {i}"
        assert res.lag_res <= eps and res.cons_sat_norm <= eps
    b.close()


@pytest.mark.gpu
def test_batch_set_vectors_async_matches_sync():
    """New vectors enqueued without waiting, from page-locked arrays, and an
    asynchronous solve give the synchronous update's results: every problem
    Optimal, x and z within rounding of the summation order."""
    torch = pytest.importorskip("torch")
    fam = P.mpc_parametric(0)
    thetas = np.random.default_rng(5).standard_normal((64, fam.P.shape[1]))
    base = fam.base
    one = (base.H, base.q, base.A, base.b, base.C, base.d)
    b = nq.QPBatch([one] * len(thetas), settings=nq.batch_settings(variant=0, eps_abs=1e-8, precision=nq.NQG_FP32,
                                                                    refine=1, refine_tol=1e-10))
    q = thetas @ fam.P.T
    d = fam.d0[None, :] + thetas @ fam.S.T
    b.set_vectors(q_all=q.ravel(), d_all=d.ravel())
    b.solve()
    x0, _, z0, s0 = b.results()
    b.set_vectors(q_all=(2.0 * q).ravel(), d_all=d.ravel())  # other vectors in between
    b.solve()
    qp = torch.empty(q.shape, dtype=torch.float64, pin_memory=True).numpy()
    dp = torch.empty(d.shape, dtype=torch.float64, pin_memory=True).numpy()
    qp[:] = q
    dp[:] = d
    b.set_vectors_async(q_all=qp.reshape(-1), d_all=dp.reshape(-1))
    b.solve_async()
    x1, _, z1, s1 = b.results()
    assert all(a.status == 1 and c.status == 1 for a, c in zip(s0, s1))
    assert rel(x1, x0) <= 1e-8 and rel(z1, z0) <= 1e-8
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [nq.NQG_FP64, nq.NQG_FP32])
def test_shared_factorization_matches_private(precision):
    """Problems with identical matrices start from one shared factorization
    (share_factor = 1) and refactor only their active rows' paths: the same
    status, iteration counts and solutions as factoring each KKT matrix
    privately, cold and warm-started."""
    fam = P.mpc_parametric(0)
    thetas = np.random.default_rng(77).standard_normal((96, fam.P.shape[1]))
    base = fam.base
    one = (base.H, base.q, base.A, base.b, base.C, base.d)
    kw = dict(variant=0, eps_abs=1e-8, precision=precision)
    if precision == nq.NQG_FP32:
        kw.update(refine=1, refine_tol=1e-12)
    runs = {}
    for share in (0, 1):
        b = nq.QPBatch([one] * len(thetas), settings=nq.batch_settings(share_factor=share, **kw))
        b.set_vectors(q_all=(thetas @ fam.P.T).ravel(), d_all=(fam.d0[None, :] + thetas @ fam.S.T).ravel())
        b.solve()
        cold = b.results()
        # warm: every other problem starts from its own optimal active set
        for i in range(0, len(thetas), 2):
            act = b.result(i)[3]
            b.set_warm_start(i, act)
        b.solve()
        warm = b.results()
        runs[share] = (cold, warm)
        b.close()
    tol = 1e-9 if precision == nq.NQG_FP64 else 1e-6
    for phase in (0, 1):
        x0, _, z0, s0 = runs[0][phase]
        x1, _, z1, s1 = runs[1][phase]
        assert all(a.status == 1 and c.status == 1 for a, c in zip(s0, s1))
        if precision == nq.NQG_FP64:
            assert [a.num_iter for a in s0] == [c.num_iter for c in s1]
        assert rel(x1, x0) <= tol and rel(z1, z0) <= tol
