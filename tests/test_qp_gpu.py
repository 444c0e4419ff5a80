"""GPU parity of the NASOQ QP solve (Nasoq::solve(), src/nasoq.cpp:656-710)
against the reference on its own known-answer problems (tests/1.json and
data/*.yml with data/out_correct.csv) and on seeded QPs.

The active-set loop is replayed with the same decisions, so status, the
number of iterations and the final active set must be identical (with Ruiz
equilibration too, on the qp_scaled_* fixtures); primal and
dual solutions agree to 1e-7 relative (the refinement-free PREDET settings of
tests/1.json reach 1e-12), the objective to 1e-9 relative, and the KKT norms
must meet eps_abs."""
import glob
import os

import numpy as np
import pytest

import nqa
import nasoq_gb300 as nq
from nasoq_gb300.problems import CSC

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(glob.glob(os.path.join(GOLD, "qp_*.nqa")))


def load_qp(d):
    n = len(d["in_Hp"]) - 1
    meq, mineq = int(d["in_meq"][0]), int(d["in_mineq"][0])
    H = CSC(n, n, d["in_Hp"], d["in_Hi"], d["in_Hx"])
    A = CSC(meq, n, d["in_Ap"], d["in_Ai"], d["in_Ax"])
    Cm = CSC(mineq, n, d["in_Cp"], d["in_Ci"], d["in_Cx"])
    return H, d["in_q"], A, d["in_b"], Cm, d["in_d"]


def run(d, precision=nq.NQG_FP64):
    st = nq.qp_settings(variant=int(d["in_variant"][0]), eps_abs=float(d["in_eps_abs"][0]),
                        diag_perturb=float(d["in_diag_perturb"][0]),
                        max_iter=int(d["in_max_iter"][0]),
                        stop_tol=float(d.get("in_stop_tol", [1e-15])[0]),
                        max_iter_nas=int(d.get("in_max_iter_nas", [200000])[0]), precision=precision,
                        scaling=int(d.get("in_scaling", [0])[0]))
    return nq.qp_solve(*load_qp(d), settings=st)


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_qp_matches_reference(path):
    check_against_reference(nqa.load(path), os.path.basename(path))


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_qp_block_solves(path, monkeypatch):
    """Every supernode through the flag-driven block solve kernels (the
    masked solves of the active-set loop included): same bars."""
    monkeypatch.setenv("NASOQ_GB300_SOLVE_SMALL", "0,0")
    check_against_reference(nqa.load(path), os.path.basename(path))


# Families whose most-violated-row choices meet exact ties (the bounded
# bilaplacian: q = 0, box rows of equal violation at mirrored vertices): the
# rounding of one FP64 sum can pick the other row of a tie, so the trajectory
# may differ by a step; the solution may not.
TIE_PRONE = ("qp_bilap_",)


def check_against_reference(d, name=""):
    x, y, z, act, res = run(d)
    assert res.status == int(d["out_status"][0])
    ref_it = int(d["out_num_iter"][0])
    if name.startswith(TIE_PRONE):
        assert abs(res.num_iter - ref_it) <= max(2, ref_it // 100)
        assert len(set(act.tolist()) ^ set(d["out_active_set"].tolist())) <= 2
    else:
        assert res.num_iter == ref_it
        assert sorted(act.tolist()) == sorted(d["out_active_set"].tolist())
    assert rel(x, d["out_x"]) <= 1e-7
    assert rel(z, d["out_z"]) <= 1e-7
    if "out_y" in d:
        assert rel(y, d["out_y"]) <= 1e-7
    ob = float(d["out_objective"][0])
    assert abs(res.objective - ob) <= 1e-9 * max(abs(ob), 1.0)
    eps = float(d["in_eps_abs"][0])
    assert res.cons_sat_norm <= eps and res.non_negativity_infn <= eps


@pytest.mark.gpu
def test_qp_test1json_known_answer():
    """tests/1.json of the reference: x, y, z to Eigen's isApprox (1e-12)."""
    d = nqa.load(os.path.join(GOLD, "qp_test1json.nqa"))
    x, y, z, act, res = run(d)
    assert res.status == 1 and res.num_iter == 23
    assert rel(x, d["out_json_x"]) <= 1e-12
    assert rel(z, d["out_json_z"]) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_qp_fp32_factor_matches_reference(path, record_property):
    """The mixed-precision path (FP32 factorization, FP64 flexible GMRES
    refinement) on every QP fixture: the reference's status, KKT norms within
    the fixture's eps_abs, and x, z within max(1e-6, 10 eps_abs) (relative)
    of the reference's FP64 solution.  The active-set iteration count is recorded beside the
    reference's; the rounding of the FP32 factor may change a decision at a
    near-tie, so it is reported rather than required equal."""
    d = nqa.load(path)
    if int(d["out_status"][0]) != 1:
        pytest.skip("FP32 parity is pinned on the problems the reference solves to Optimal")
    if os.path.basename(path).startswith("qp_bilap_"):
        # kappa(K) of the bilaplacian KKT grows like grid^4 (~1e9 at 80^2): an
        # FP32 factor is too weak a preconditioner for the refinement to reach
        # the 1e-8 decisions; this family runs in FP64
        pytest.skip("the bilaplacian family is beyond the FP32 factor's conditioning")
    x, y, z, act, res = run(d, precision=nq.NQG_FP32)
    ref_it = int(d["out_num_iter"][0])
    record_property("iterations_fp32", res.num_iter)
    record_property("iterations_reference", ref_it)
    print(f"{os.path.basename(path)}: iterations FP32 {res.num_iter}, reference {ref_it}")
    assert res.status == int(d["out_status"][0])
    eps = float(d["in_eps_abs"][0])
    assert res.cons_sat_norm <= eps and res.non_negativity_infn <= eps
    if res.status == 1:
        assert res.lag_res <= eps
    # two solutions meeting eps_abs can differ by about eps_abs
    tol = max(1e-6, 10 * eps)
    assert rel(x, d["out_x"]) <= tol
    assert rel(z, d["out_z"]) <= tol
    if "out_y" in d:
        assert rel(y, d["out_y"]) <= tol
