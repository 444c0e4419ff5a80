"""GPU parity of the LBL flow (SolverSettings symbolic_analysis ->
numerical_factorization -> solve_only, examples/lbl_main.cpp:34-43) against
the reference's FP64 outputs in the golden fixtures.

Tolerances (kappa = 2-norm condition number of the perturbed matrix, g =
largest |L| entry of the reference factor, i.e. the element growth that
pivoting restricted to supernode diagonal blocks allows):
  * factor backward error  max|P K P^T - L D L^T| <= 1e-13 max(|L||D||L|^T)
    (FP64), computed densely from the GPU factor;
  * when Bunch-Kaufman chose the same pivots as the reference, the row lists
    after pivoting are identical and the D / L values agree to
    max(1e-9, 1e-15 kappa, 1e-14 g) relative to their largest entry;
  * FP64 solutions (with and without refinement) agree with the reference's
    to max(1e-9, 1e-14 kappa, 1e-15 g) relative 2-norm;
  * the FP32 factor with FP64 GMRES refinement reaches a relative residual
    of 1e-10 whenever kappa < 1e8 (beyond that FP32 cannot carry the
    factor and the FP64 path is the one to use)."""
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


def dense_sym(n, Ap, Ai, Ax):
    K = np.zeros((n, n))
    for j in range(n):
        for q in range(Ap[j], Ap[j + 1]):
            K[Ai[q], j] = Ax[q]
            K[j, Ai[q]] = Ax[q]
    return K


def dense_factor(sym, vals, dv, ls):
    """Dense unit-lower L and block-diagonal D from the supernodal arrays."""
    n = sym.info.n
    Ld = np.eye(n)
    for s in range(sym.info.nsuper):
        c0, c1 = sym.super[s], sym.super[s + 1]
        rows = ls[sym.lpi[s]:sym.lpi[s + 1]]
        nr = len(rows)
        base = sym.colp[c0]
        blk = vals[base:base + nr * (c1 - c0)].reshape(c1 - c0, nr).T
        for c in range(c1 - c0):
            for r in range(c + 1, nr):
                Ld[rows[r], c0 + c] = blk[r, c]
    Dd = np.diag(dv[:n])
    for i in range(n - 1):
        if dv[n + i] != 0:
            Dd[i + 1, i] = Dd[i, i + 1] = dv[n + i]
    return Ld, Dd


_COND = {}


def cond_of(path, d):
    if path not in _COND:
        n = len(d["in_rhs"])
        _COND[path] = np.linalg.cond(dense_sym(n, d["in_Ap"], d["in_Ai"], d["out_Ax_perturbed"]))
    return _COND[path]


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_spmv_matches_reference_sweep(path):
    """nqg_spmv_device (rows of the full symmetric CSR, FP64) against the
    oracle's restatement of the reference's column sweep over the lower
    triangle (spmv_csc_sym_one_int, src/matrixVector/spmv_CSC.cpp:26-102) on
    the fixture's matrix and a seeded x: entrywise within the bound of a
    different summation order, nnz_i 2^-52 (|K| |x|)_i."""
    torch = pytest.importorskip("torch")
    from oracle import port
    d = nqa.load(path)
    n = len(d["in_rhs"])
    Ap, Ai, Ax = d["in_Ap"], d["in_Ai"], d["in_Ax"]
    plan = nq.Plan(n, Ap, Ai, Ax, settings=_settings(d))
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    x = np.random.default_rng(n).standard_normal(n)
    dx = torch.from_numpy(x).cuda()
    dy = torch.full_like(dx, float("nan"))
    plan.spmv_device(dx.data_ptr(), dy.data_ptr())
    torch.cuda.synchronize()
    y = dy.cpu().numpy()
    plan.close()
    yr = port.spmv(n, Ap, Ai, Ax, x)
    mag = port.spmv(n, Ap, Ai, np.abs(Ax), np.abs(x))
    cols = np.repeat(np.arange(n), np.diff(Ap))
    nnz_row = np.bincount(Ai, minlength=n) + np.bincount(cols[Ai != cols], minlength=n)
    assert np.all(np.isfinite(y))
    assert np.all(np.abs(y - yr) <= nnz_row * 2.0 ** -52 * mag)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp64_factor_and_solve(path):
    d = nqa.load(path)
    n = len(d["in_rhs"])
    kappa = cond_of(path, d)
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d, req_ref_iter=0))
    rc = plan.factor()
    assert rc == 0, f"factor status {rc}"
    vals, dv, perm, ls = plan.factor_arrays()
    # backward error of the GPU factor against the perturbed, permuted matrix
    Kp = dense_sym(n, d["in_Ap"], d["in_Ai"], d["out_Ax_perturbed"])[np.ix_(perm, perm)]
    Ld, Dd = dense_factor(plan.symbolic, vals, dv, ls)
    R = Kp - Ld @ Dd @ Ld.T
    mag = np.abs(Ld) @ np.abs(Dd) @ np.abs(Ld).T
    assert np.abs(R).max() <= 1e-13 * mag.max(), "factor backward error too large"
    g = np.abs(d["out_valL"]).max()
    tol = max(1e-9, 1e-15 * kappa)
    if np.array_equal(perm, d["out_fac_Perm"]):
        assert np.array_equal(ls, d["out_fac_s"]), "row lists after pivoting differ"
    if np.array_equal(perm, d["out_fac_Perm"]) and g < 1e6:
        # entry-wise comparison is only meaningful without large element growth;
        # with growth the backward error above is the parity criterion
        ref = d["out_valL"]
        assert np.abs(vals - ref).max() <= tol * max(np.abs(ref).max(), 1.0)
        refd = d["out_d_val"]
        assert np.abs(dv - refd).max() <= tol * max(np.abs(refd).max(), 1.0)
    xtol = max(1e-9, 1e-14 * kappa, 1e-15 * g)
    x0 = plan.solve(d["in_rhs"])
    xr = d["out_x_noref"]
    assert np.linalg.norm(x0 - xr) <= xtol * np.linalg.norm(xr), "unrefined solve differs"
    plan.close()
    # with the reference's refinement settings
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    xr = d["out_x"]
    if relres(d, xr) > 1e-8:
        # the refinement matrix (tiny diagonals set to 0 as the reference's
        # set_diags(0) does) is singular here: the reference's own refined
        # vector does not solve the system, so there is nothing to match
        return
    assert np.linalg.norm(x - xr) <= xtol * np.linalg.norm(xr)
    assert relres(d, x) <= max(10 * relres(d, xr), 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp32_factor_gmres_ir(path):
    d = nqa.load(path)
    n = len(d["in_rhs"])
    if cond_of(path, d) > 1e8:
        pytest.skip("kappa * u_fp32 >= 1: FP64 factorization territory")
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"],
                   settings=_settings(d, precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6,
                                      tol_abs=1e-13, tol_rel=1e-13))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("force_blk", [False, True], ids=["level", "block"])
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp32_factor_fp32_solves(path, force_blk, monkeypatch):
    """FP32 factor with the triangular solves in FP32 (solve_precision) and
    flexible GMRES in FP64 around them: relative residual 1e-10 whenever
    kappa < 1e8, through the per-supernode level kernels and through the
    flag-driven block kernels."""
    if force_blk:
        monkeypatch.setenv("NASOQ_GB300_SOLVE_SMALL", "0,0")
    d = nqa.load(path)
    n = len(d["in_rhs"])
    if cond_of(path, d) > 1e8:
        pytest.skip("kappa * u_fp32 >= 1: FP64 factorization territory")
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"],
                   settings=_settings(d, precision=nq.NQG_FP32, solve_precision=nq.NQG_FP32, req_ref_iter=6,
                                      max_inner_iter=6, tol_abs=1e-13, tol_rel=1e-13))
    plan.factor()
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)


WIDE_ENV = {"NASOQ_GB300_WIDE_MIN": "12", "NASOQ_GB300_WIDE_NB": "8", "NASOQ_GB300_SOLVE_SMALL": "0,0"}


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp64_blocked_wide_kernels(path, monkeypatch):
    """Every supernode wider than 12 columns goes through the blocked
    multi-CTA Bunch-Kaufman (panels of 8 columns) and every supernode through
    the flag-driven block solves: same parity bars as the single-CTA
    kernels."""
    for k, v in WIDE_ENV.items():
        monkeypatch.setenv(k, v)
    d = nqa.load(path)
    n = len(d["in_rhs"])
    kappa = cond_of(path, d)
    g = np.abs(d["out_valL"]).max()
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d, req_ref_iter=0))
    assert plan.factor() == 0
    vals, dv, perm, ls = plan.factor_arrays()
    Kp = dense_sym(n, d["in_Ap"], d["in_Ai"], d["out_Ax_perturbed"])[np.ix_(perm, perm)]
    Ld, Dd = dense_factor(plan.symbolic, vals, dv, ls)
    R = Kp - Ld @ Dd @ Ld.T
    mag = np.abs(Ld) @ np.abs(Dd) @ np.abs(Ld).T
    assert np.abs(R).max() <= 1e-13 * mag.max(), "blocked factor backward error too large"
    xtol = max(1e-9, 1e-14 * kappa, 1e-15 * g)
    x0 = plan.solve(d["in_rhs"])
    xr = d["out_x_noref"]
    assert np.linalg.norm(x0 - xr) <= xtol * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("trailing", ["tcgen05", "tcgen05-tf32", "tcgen05-depth1", "tcgen05-depth2", "tcgen05-tile",
                                      "mma", "simt", "general-panels"])
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp32_blocked_wide_kernels(path, trailing, monkeypatch):
    """FP32 factor with every supernode wider than 12 columns in the blocked
    kernels (fast panels where no pivot search is needed, or every panel on
    the general kernel), trailing updates on the tcgen05 tensor cores (one,
    two or four panels per delayed update; the persistent kernel on packed
    split-BF16 or split-TF32 operands, or one CTA per tile with split TF32)
    or with mma.sync (split TF32) or on CUDA cores:
    the refined solution meets the FP32 bar of the single-CTA kernels."""
    for k, v in WIDE_ENV.items():
        monkeypatch.setenv(k, v)
    if trailing == "tcgen05-tf32":
        monkeypatch.setenv("NASOQ_GB300_SPLIT", "tf32")
    elif trailing == "general-panels":
        monkeypatch.setenv("NASOQ_GB300_PANEL", "general")
    elif trailing.startswith("tcgen05-depth"):
        monkeypatch.setenv("NASOQ_GB300_WIDE_DEPTH", trailing[-1])
    elif trailing == "tcgen05-tile":
        monkeypatch.setenv("NASOQ_GB300_TRAILING", "tile")
    else:
        monkeypatch.setenv("NASOQ_GB300_TRAILING", trailing)
    d = nqa.load(path)
    n = len(d["in_rhs"])
    if cond_of(path, d) > 1e8:
        pytest.skip("kappa * u_fp32 >= 1: FP64 factorization territory")
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"],
                   settings=_settings(d, precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6,
                                      tol_abs=1e-13, tol_rel=1e-13))
    assert plan.factor() == 0
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("update", ["tcgen05", "tcgen05-persistent", "tcgen05-persistent-tf32", "simt"])
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_fp32_update_kernels(path, update, monkeypatch):
    """FP32 factor with every Schur update between supernodes on the tcgen05
    tiles (any descendant width), every one as a persistent tcgen05 launch
    on packed split-BF16 or split-TF32 operands, or every one on the
    CUDA-core tiles: the refined solution meets the FP32 bar."""
    if update == "tcgen05":
        monkeypatch.setenv("NASOQ_GB300_UPDATE_TC_MIN", "1")
        monkeypatch.setenv("NASOQ_GB300_UPDATE_PERSIST_MIN", "-1")
    elif update.startswith("tcgen05-persistent"):
        monkeypatch.setenv("NASOQ_GB300_UPDATE_TC_MIN", "1")
        monkeypatch.setenv("NASOQ_GB300_UPDATE_PERSIST_MIN", "0")
        if update.endswith("tf32"):
            monkeypatch.setenv("NASOQ_GB300_SPLIT", "tf32")
    else:
        monkeypatch.setenv("NASOQ_GB300_UPDATE", "simt")
    d = nqa.load(path)
    n = len(d["in_rhs"])
    if cond_of(path, d) > 1e8:
        pytest.skip("kappa * u_fp32 >= 1: FP64 factorization territory")
    plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"],
                   settings=_settings(d, precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6,
                                      tol_abs=1e-13, tol_rel=1e-13))
    assert plan.factor() == 0
    x = plan.solve(d["in_rhs"])
    assert relres(d, x) <= 1e-10
    xr = d["out_x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_panel_rows_kernels(path, monkeypatch):
    """Supernodes wider than 4 columns through k_bk_global, the rows below
    each diagonal block solved by the multi-CTA kernel or by the per-row
    substitution inside k_bk_global: both FP64 factors pass the backward
    error bar.  (Two factorizations are not compared bit for bit: the Schur
    updates scatter with atomics, so summation order varies run to run.)"""
    monkeypatch.setenv("NASOQ_GB300_BK_SMALL", "4")
    d = nqa.load(path)
    n = len(d["in_rhs"])
    for mode in ("split", "serial"):
        monkeypatch.setenv("NASOQ_GB300_PANEL_ROWS", mode)
        plan = nq.Plan(n, d["in_Ap"], d["in_Ai"], d["in_Ax"], settings=_settings(d, req_ref_iter=0))
        assert plan.factor() == 0
        vals, dv, perm, ls = plan.factor_arrays()
        Kp = dense_sym(n, d["in_Ap"], d["in_Ai"], d["out_Ax_perturbed"])[np.ix_(perm, perm)]
        Ld, Dd = dense_factor(plan.symbolic, vals, dv, ls)
        R = Kp - Ld @ Dd @ Ld.T
        mag = np.abs(Ld) @ np.abs(Dd) @ np.abs(Ld).T
        assert np.abs(R).max() <= 1e-13 * mag.max(), mode
        plan.close()


def _dense_lower_csc(M):
    n = M.shape[0]
    Ap = np.zeros(n + 1, np.int32)
    Ap[1:] = np.cumsum(np.arange(n, 0, -1))
    Ai = np.concatenate([np.arange(j, n, dtype=np.int32) for j in range(n)])
    Ax = np.concatenate([M[j:, j] for j in range(n)])
    return Ap, Ai, Ax


@pytest.mark.gpu
@pytest.mark.parametrize("n,pivots", [(900, False), (900, True), (1201, True)])
def test_fast_panel_kernels_agree(n, pivots, monkeypatch):
    """One dense FP32 supernode through the wide kernels (no atomics, so the
    factor is deterministic): the block-first fast panel (one exchange per
    panel) and the grouped one (four columns per exchange) apply the same
    FMAs in the same order and stop at the same columns, so the factors are
    identical bit for bit (compared from the same settled pivot order); with
    small diagonals scattered through the matrix the general kernel takes
    over after every stop.  The refined solution
    meets the FP32 bar."""
    rng = np.random.default_rng(n + pivots)
    M = rng.standard_normal((n, n))
    M = (M + M.T) / 2
    dg = rng.uniform(0.5 * n, n, n) * rng.choice([-1.0, 1.0], n)
    if pivots:
        dg[rng.choice(n, n // 40, replace=False)] = 1e-3
    M[np.diag_indices(n)] = dg
    Ap, Ai, Ax = _dense_lower_csc(M)
    st = nq.default_settings(precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6, tol_abs=1e-13,
                             tol_rel=1e-13, reg_diag=0.0)
    plan = nq.Plan(n, Ap, Ai, Ax, settings=st)
    assert plan.symbolic.info.nsuper == 1
    # the first factorization settles the pivot order that later ones start from
    monkeypatch.setenv("NASOQ_GB300_PANEL", "group")
    assert plan.factor() == 0
    out = {}
    for mode in ("group", "block"):
        if mode == "group":
            monkeypatch.setenv("NASOQ_GB300_PANEL", "group")
        else:
            monkeypatch.delenv("NASOQ_GB300_PANEL", raising=False)
        assert plan.factor() == 0
        out[mode] = plan.factor_arrays()
    for a, b in zip(out["group"], out["block"]):
        assert np.array_equal(a, b)
    rhs = rng.standard_normal(n)
    x = plan.solve(rhs)
    assert np.linalg.norm(rhs - M @ x) <= 1e-10 * np.linalg.norm(rhs)
    plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n,pivots", [(1024, False), (1100, True)])
def test_trailing_kernels_agree(n, pivots, monkeypatch):
    """One dense FP32 supernode: the persistent tcgen05 trailing update on
    packed split-TF32 operands (NASOQ_GB300_SPLIT=tf32) against the
    one-CTA-per-tile kernel that splits its operands while loading them.  With full 64-column panels both
    sum the same products in the same chunks of 32, so the factors agree bit
    for bit; with pivot searches (panels of any width, padded chunks) both
    factors reach a backward error of 1e-4 max(|L||D||L|^T) (no diagonal
    floor) and the refined solution the FP32 bar.  The persistent kernel on
    split-BF16 operands (the default, 64 K entries per chunk) reaches 1e-4
    too."""
    rng = np.random.default_rng(7 * n + pivots)
    M = rng.standard_normal((n, n))
    M = (M + M.T) / 2
    dg = rng.uniform(0.5 * n, n, n) * rng.choice([-1.0, 1.0], n)
    if pivots:
        dg[rng.choice(n, n // 40, replace=False)] = 1e-3
    M[np.diag_indices(n)] = dg
    Ap, Ai, Ax = _dense_lower_csc(M)
    st = nq.default_settings(precision=nq.NQG_FP32, req_ref_iter=6, max_inner_iter=6, tol_abs=1e-13,
                             tol_rel=1e-13, reg_diag=0.0, reg_diag_fp32=1e-30)
    plan = nq.Plan(n, Ap, Ai, Ax, settings=st)
    assert plan.symbolic.info.nsuper == 1
    monkeypatch.setenv("NASOQ_GB300_TRAILING", "tile")
    assert plan.factor() == 0
    out = {}
    monkeypatch.setenv("NASOQ_GB300_SPLIT", "tf32")
    for mode in ("tile", "persistent", "persistent-bf16"):
        if mode == "tile":
            monkeypatch.setenv("NASOQ_GB300_TRAILING", "tile")
        else:
            monkeypatch.delenv("NASOQ_GB300_TRAILING", raising=False)
        if mode == "persistent-bf16":
            monkeypatch.delenv("NASOQ_GB300_SPLIT", raising=False)
        assert plan.factor() == 0
        out[mode] = plan.factor_arrays()
        vals, dv, perm, ls = out[mode]
        Ld, Dd = dense_factor(plan.symbolic, vals, dv, ls)
        R = M[np.ix_(perm, perm)] - Ld @ Dd @ Ld.T
        mag = np.abs(Ld) @ np.abs(Dd) @ np.abs(Ld).T
        assert np.abs(R).max() <= 1e-4 * mag.max(), mode
    if not pivots:
        for a, b in zip(out["tile"], out["persistent"]):
            assert np.array_equal(a, b)
    rhs = rng.standard_normal(n)
    x = plan.solve(rhs)
    assert np.linalg.norm(rhs - M @ x) <= 1e-10 * np.linalg.norm(rhs)
    plan.close()
