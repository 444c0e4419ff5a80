"""Hard pivots at production thresholds: a strongly indefinite KKT system
(2500 zero-diagonal constraint columns, as many negative eigenvalues,
kappa ~ 1.2e4, N = 6596) whose supernodes reach 2545 columns and whose
Bunch-Kaufman factorization takes 2x2 pivots (tests/golden/lblw_kkt3d_hard.nqa,
made by tests/golden/gen_golden.py from the reference).  The multi-CTA
kernels run at their default widths (192-column threshold, 64-column
panels), FP64 and every FP32 variant:

  * FP64: 2x2 pivots found, solutions within max(1e-9, 1e-14 kappa,
    1e-15 g) of the reference's, g its largest factor entry (without and with
    refinement);
  * FP32 factor (tcgen05 on split-BF16 or split-TF32 operands, per-tile
    tcgen05, mma.sync, SIMT trailing updates;
    FP64 or FP32 triangular solves, level or block kernels) with FP64
    refinement: relative residual 1e-10 and x within 1e-6 of the reference."""
import os

import numpy as np
import pytest

import nqa
import nasoq_gb300 as nq

PATH = os.path.join(os.path.dirname(__file__), "golden", "lblw_kkt3d_hard.nqa")


def relres(d, x):
    n = len(d["in_rhs"])
    Ap, Ai, Ax = d["in_Ap"], d["in_Ai"], d["in_Ax"]
    cols = np.repeat(np.arange(n), np.diff(Ap))
    y = np.zeros(n)
    np.add.at(y, Ai, Ax * x[cols])
    off = Ai != cols
    np.add.at(y, cols[off], Ax[off] * x[Ai[off]])
    return np.linalg.norm(d["in_rhs"] - y) / np.linalg.norm(d["in_rhs"])


def _plan(d, **kw):
    n = len(d["in_rhs"])
    st = nq.default_settings(reg_diag=float(d["in_reg_diag"][0]), **kw)
    return nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=st)


@pytest.mark.gpu
def test_fp64_hard_pivots_default_thresholds():
    d = nqa.load(PATH)
    kappa = float(d["out_kappa"][0])
    assert int(d["out_n2x2"][0]) > 0 and int(d["out_sym_max_sup_wid"][0]) > 192
    plan = _plan(d, req_ref_iter=0)
    assert plan.factor() == nq.NQG_OK
    assert plan.timings().num_2x2 > 0
    # unrefined solutions differ by rounding amplified by the element growth
    # that block-restricted pivoting leaves (pivots as small as reg_diag)
    tol = max(1e-9, 1e-14 * kappa, 1e-15 * float(d["out_gmax"][0]))
    x0 = plan.solve(d["in_rhs"])
    xr = d["out_x_noref"]
    assert np.linalg.norm(x0 - xr) <= tol * np.linalg.norm(xr)
    plan.close()
    plan = _plan(d, req_ref_iter=int(d["in_req_ref_iter"][0]))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    assert np.linalg.norm(x - d["out_x"]) <= tol * np.linalg.norm(d["out_x"])
    assert relres(d, x) <= 1e-12
    plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("trailing", ["tcgen05", "tcgen05-tf32", "tile", "mma", "simt"])
@pytest.mark.parametrize("solves", ["fp64", "fp32-level", "fp32-block"])
def test_fp32_hard_pivots_default_thresholds(trailing, solves, monkeypatch):
    if trailing == "tcgen05-tf32":
        monkeypatch.setenv("NASOQ_GB300_SPLIT", "tf32")
    elif trailing != "tcgen05":
        monkeypatch.setenv("NASOQ_GB300_TRAILING", trailing)
    if solves == "fp32-block":
        monkeypatch.setenv("NASOQ_GB300_SOLVE_SMALL", "0,0")
    d = nqa.load(PATH)
    sp = nq.NQG_FP64 if solves == "fp64" else nq.NQG_FP32
    plan = _plan(d, precision=nq.NQG_FP32, solve_precision=sp, req_ref_iter=6, max_inner_iter=6, tol_abs=1e-13,
                 tol_rel=1e-13)
    rc = plan.factor()
    assert rc in (nq.NQG_OK, nq.NQG_WARN_ZERO_PIVOT)
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)
    plan.close()
