"""Failure paths, driven only by inputs and settings that cannot hang or
fault a GPU:

  * a cross-CTA wait whose poll limit is set to one poll gives up, the call
    returns NQG_ERR_TIMEOUT, and the plan solves correctly again once the
    default limit is back;
  * an exactly singular pivot block makes the factorization return
    NQG_WARN_ZERO_PIVOT (the reference's BK leaves a zero D entry there);
  * a NaN among the matrix values makes it return NQG_WARN_NONFINITE, and a
    batched QP with NaN data is flagged non-finite and never Optimal;
  * an active-set iteration cap below what a problem needs ends the NASOQ
    loop unconverged, which the reference reports as Infeasible (status 0:
    numeric_QP returns is_converged = 0 at the cap, src/nasoq.cpp:488-491, and
    check_solve_status maps that to Infeasible, :712-716)."""
import os

import numpy as np
import pytest

import nqa
import nasoq_gb300 as nq
from nasoq_gb300.problems import CSC

GOLD = os.path.join(os.path.dirname(__file__), "golden")
WIDE_ENV = {"NASOQ_GB300_WIDE_MIN": "12", "NASOQ_GB300_WIDE_NB": "8", "NASOQ_GB300_SOLVE_SMALL": "0,0"}


def tridiag(n, diag=4.0, off=-1.0):
    """Lower CSC of a symmetric tridiagonal matrix (every entry stored)."""
    Ap, Ai, Ax = [0], [], []
    for j in range(n):
        Ai.append(j)
        Ax.append(diag)
        if j + 1 < n:
            Ai.append(j + 1)
            Ax.append(off)
        Ap.append(len(Ai))
    return np.array(Ap, np.int32), np.array(Ai, np.int32), np.array(Ax, np.float64)


@pytest.mark.gpu
def test_wait_limit_gives_up_then_plan_recovers(monkeypatch):
    for k, v in WIDE_ENV.items():
        monkeypatch.setenv(k, v)
    d = nqa.load(os.path.join(GOLD, "lbl_kkt3d_mid.nqa"))
    n = len(d["in_rhs"])
    st = nq.default_settings(req_ref_iter=0, reg_diag=float(d.get("in_reg_diag", [1e-9])[0]))
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=st)
    assert plan.factor() == nq.NQG_OK
    x0 = plan.solve(d["in_rhs"])
    xr = d["out_x_noref"]
    assert np.linalg.norm(x0 - xr) <= 1e-6 * np.linalg.norm(xr)
    # one poll: every block that waits for an earlier block of its supernode gives up
    plan.set_wait_limit(1)
    with pytest.raises(nq.NasoqError, match=r"\(-5\)"):
        plan.solve(d["in_rhs"])
    plan.set_wait_limit(0)
    x1 = plan.solve(d["in_rhs"])
    # the off-diagonal block products are summed by atomics: equal up to rounding
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
    assert np.linalg.norm(x1 - xr) <= 1e-6 * np.linalg.norm(xr)
    assert plan.factor() == nq.NQG_OK
    x2 = plan.solve(d["in_rhs"])
    assert np.linalg.norm(x2 - xr) <= 1e-6 * np.linalg.norm(xr)


@pytest.mark.gpu
def test_singular_block_warns_zero_pivot():
    n = 40
    Ap, Ai, Ax = tridiag(n)
    # column 7 (and its row) exactly zero: a 1x1 pivot of 0 with nothing to swap in
    for j in (6, 7):
        for q in range(Ap[j], Ap[j + 1]):
            if Ai[q] == 7 or j == 7:
                Ax[q] = 0.0
    # reg_diag 0: no diagonal is perturbed (|a_jj| < 0 never holds)
    plan = nq.Plan(n, Ap, Ai, Ax, settings=nq.default_settings(reg_diag=0.0, req_ref_iter=0))
    assert plan.factor() == nq.NQG_WARN_ZERO_PIVOT
    # the same matrix with the default perturbation (reg_diag on tiny diagonals) factors cleanly
    plan2 = nq.Plan(n, Ap, Ai, Ax, settings=nq.default_settings())
    assert plan2.factor() == nq.NQG_OK


@pytest.mark.gpu
def test_nonfinite_values_warn():
    n = 40
    Ap, Ai, Ax = tridiag(n)
    Ax[Ap[11]] = np.nan  # diagonal of column 11
    plan = nq.Plan(n, Ap, Ai, Ax, settings=nq.default_settings(req_ref_iter=0))
    assert plan.factor() == nq.NQG_WARN_NONFINITE
    # finite values again: the same plan factors and solves
    Ax[Ap[11]] = 4.0
    plan.set_values(Ax)
    assert plan.factor() == nq.NQG_OK
    b = np.arange(1.0, n + 1.0)
    x = plan.solve(b)
    K = np.zeros((n, n))
    for j in range(n):
        for q in range(Ap[j], Ap[j + 1]):
            K[Ai[q], j] = K[j, Ai[q]] = Ax[q]
    assert np.linalg.norm(K @ x - b) <= 1e-12 * np.linalg.norm(b)


def _qp_fixture(name):
    d = nqa.load(os.path.join(GOLD, name))
    n = len(d["in_Hp"]) - 1
    meq, mineq = int(d["in_meq"][0]), int(d["in_mineq"][0])
    H = CSC(n, n, d["in_Hp"], d["in_Hi"], d["in_Hx"])
    A = CSC(meq, n, d["in_Ap"], d["in_Ai"], d["in_Ax"])
    Cm = CSC(mineq, n, d["in_Cp"], d["in_Ci"], d["in_Cx"])
    return d, (H, d["in_q"], A, d["in_b"], Cm, d["in_d"])


@pytest.mark.gpu
def test_iteration_cap_ends_with_not_converged():
    d, qp = _qp_fixture("qp_mpc_N25.nqa")
    ref_iters = int(d["out_num_iter"][0])
    assert ref_iters > 3
    kw = dict(variant=int(d["in_variant"][0]), eps_abs=float(d["in_eps_abs"][0]),
              diag_perturb=float(d["in_diag_perturb"][0]), max_iter=int(d["in_max_iter"][0]))
    *_, res = nq.qp_solve(*qp, settings=nq.qp_settings(max_iter_nas=2, **kw))
    assert res.status == 0  # the reference's status for a loop stopped by the cap
    assert res.num_iter <= 3
    b = nq.QPBatch([qp] * 3, settings=nq.batch_settings(max_iter_nas=2, **kw))
    b.solve()
    for i in range(3):
        r = b.result(i)[-1]
        assert r.status == 0 and r.num_iter <= 3
    b.close()
    # without the cap the same batch converges, with the reference's count
    b = nq.QPBatch([qp], settings=nq.batch_settings(**kw))
    b.solve()
    r = b.result(0)[-1]
    assert r.status == 1 and r.num_iter == ref_iters
    b.close()


@pytest.mark.gpu
def test_batch_nonfinite_data_flagged():
    d, (H, q, A, bb, Cm, dd) = _qp_fixture("qp_mpc_N10.nqa")
    q_bad = np.array(q, np.float64)
    q_bad[3] = np.nan
    b = nq.QPBatch([(H, q, A, bb, Cm, dd), (H, q_bad, A, bb, Cm, dd)],
                   settings=nq.batch_settings(variant=int(d["in_variant"][0]), eps_abs=float(d["in_eps_abs"][0]),
                                              diag_perturb=float(d["in_diag_perturb"][0]),
                                              max_iter=int(d["in_max_iter"][0])))
    b.solve()
    ok, bad = b.results()[-1]
    assert ok.status == 1
    assert bad.status != 1
    assert bad.flags & 2  # non-finite
    b.close()
