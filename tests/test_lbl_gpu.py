"""GPU parity of the LBL flow (SolverSettings symbolic_analysis ->
numerical_factorization -> solve_only, examples/lbl_main.cpp:34-43) against
the reference's FP64 outputs in the golden fixtures.

Tolerances: the FP64 factor matches the reference factor to 1e-10 relative
(max-abs over entries) whenever Bunch-Kaufman chose the same pivots; FP64
solutions match to 1e-9 relative 2-norm.  The FP32 factor with FP64 GMRES
refinement must reach a relative residual of 1e-10 with enough refinement
steps."""
import glob
import os

import numpy as np
import pytest

import nqa
import nasoq_gb300 as nq
from nasoq_gb300.problems import CSC

GOLD = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(glob.glob(os.path.join(GOLD, "lbl_*.nqa")))


def _settings(d, **over):
    kw = dict(req_ref_iter=int(d.get("in_req_ref_iter", [2])[0]),
              max_inner_iter=int(d.get("in_max_inner_iter", [2])[0]),
              reg_diag=float(d.get("in_reg_diag", [1e-9])[0]))
    kw.update(over)
    return nq.default_settings(**kw)


def sym_matvec(n, Ap, Ai, Ax, x):
    y = np.zeros(n)
    for j in range(n):
        for q in range(Ap[j], Ap[j + 1]):
            i = Ai[q]
            y[i] += Ax[q] * x[j]
            if i != j:
                y[j] += Ax[q] * x[i]
    return y


def relres(d, x):
    n = len(d["in_rhs"])
    r = d["in_rhs"] - sym_matvec(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], x)
    return np.linalg.norm(r) / np.linalg.norm(d["in_rhs"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp64_factor_and_solve(path):
    d = nqa.load(path)
    n = len(d["in_rhs"])
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d, req_ref_iter=0))
    rc = plan.factor()
    assert rc == 0, f"factor status {rc}"
    vals, dv, perm, ls = plan.factor_arrays()
    same_pivots = np.array_equal(perm, d["out_fac_Perm"])
    if same_pivots:
        assert np.array_equal(ls, d["out_fac_s"]), "row lists after pivoting differ"
        ref = d["out_valL"]
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(vals - ref).max() <= 1e-10 * scale
        refd = d["out_d_val"]
        assert np.abs(dv - refd).max() <= 1e-10 * max(np.abs(refd).max(), 1.0)
    x0 = plan.solve(d["in_rhs"])
    xr = d["out_x_noref"]
    assert np.linalg.norm(x0 - xr) <= 1e-9 * max(np.linalg.norm(xr), 1e-300), "unrefined solve differs"
    plan.close()
    # with the reference's refinement settings
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-9 * np.linalg.norm(xr)
    assert relres(d, x) <= max(10 * relres(d, xr), 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp32_factor_gmres_ir(path):
    d = nqa.load(path)
    n = len(d["in_rhs"])
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"],
                   settings=_settings(d, precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6,
                                      tol_abs=1e-13, tol_rel=1e-13))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)
