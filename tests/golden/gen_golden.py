"""Generates the golden fixtures in this directory by running the reference
NASOQ library (built out-of-tree by oracle/Makefile into oracle/_ref/) on
seeded inputs and on the reference's own known-answer problems.

Run in the development container, where the reference sources live:

    make -C oracle && python tests/golden/gen_golden.py [/path/to/reference]

(the reference path defaults to $NASOQ_REFERENCE, else /root/reference)

Each fixture <case>.nqa holds the inputs (prefix ``in_``) and everything the
reference produced (prefix ``out_``).  The reference runs single-threaded
(OMP_NUM_THREADS=1) so its sums are in a fixed order.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import nqa  # noqa: E402
from nasoq_gb300 import problems as P  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
ONLY = None  # --only PREFIX: regenerate just the cases whose name starts with it


def run(cmd, inp, extra_env=None):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    if extra_env:
        env.update(extra_env)
    with tempfile.TemporaryDirectory() as td:
        src = inp
        if isinstance(inp, dict):
            src = os.path.join(td, "in.nqa")
            nqa.save(src, inp)
        out = os.path.join(td, "out.nqa")
        subprocess.run([REF_DUMP, cmd, src, out], check=True, env=env)
        return nqa.load(out)


def wanted(name):
    return ONLY is None or name.startswith(ONLY)


def save_case(name, inp, out):
    arrs = {"in_" + k: np.asarray(v) for k, v in inp.items()}
    arrs.update({"out_" + k: np.asarray(v) for k, v in out.items()})
    nqa.save(os.path.join(HERE, name + ".nqa"), arrs)
    print(f"{name}: {sum(a.nbytes for a in arrs.values()) / 1024:.1f} KiB")


def lbl_case(name, K, rhs, **settings):
    if not wanted(name):
        return
    inp = {"Ap": K.p, "Ai": K.i, "Ax": K.x, "rhs": rhs}
    for k, v in settings.items():
        inp[k] = np.array([float(v)])
    out = run("lbl", inp)
    save_case(name, inp, out)


def lbl_case_light(name, K, rhs, **settings):
    """An LBL case too large to keep the reference's factor: inputs, the
    reference's solutions, the perturbed values, and the condition number and
    2x2-pivot count of the reference's factorization."""
    if not wanted(name):
        return
    inp = {"Ap": K.p, "Ai": K.i, "Ax": K.x, "rhs": rhs}
    for k, v in settings.items():
        inp[k] = np.array([float(v)])
    out = run("lbl", inp)
    n = K.ncol
    Kd = np.zeros((n, n))
    for j in range(n):
        for q in range(K.p[j], K.p[j + 1]):
            Kd[K.i[q], j] = Kd[j, K.i[q]] = out["Ax_perturbed"][q]
    ev = np.abs(np.linalg.eigvalsh(Kd))
    keep = {k: out[k] for k in ("x", "x_noref", "Ax_perturbed", "num_ref_iter", "sym_max_sup_wid")}
    keep["kappa"] = np.array([ev.max() / ev.min()])
    keep["n2x2"] = np.array([float(np.count_nonzero(out["d_val"][n:]))])
    keep["gmax"] = np.array([float(np.abs(out["valL"]).max())])  # element growth of the factor
    save_case(name, inp, keep)


def qp_inputs(qp: P.QP, **settings):
    inp = {
        "Hp": qp.H.p, "Hi": qp.H.i, "Hx": qp.H.x, "q": qp.q,
        "Ap": qp.A.p, "Ai": qp.A.i, "Ax": qp.A.x, "b": qp.b,
        "Cp": qp.C.p, "Ci": qp.C.i, "Cx": qp.C.x, "d": qp.d,
        "meq": np.array([float(qp.A.nrow)]), "mineq": np.array([float(qp.C.nrow)]),
    }
    for k, v in settings.items():
        inp[k] = np.array([float(v)])
    return inp


def qp_case(name, qp, **settings):
    if not wanted(name):
        return
    inp = qp_inputs(qp, **settings)
    out = run("qp", inp)
    save_case(name, inp, out)


def smp_qp(path):
    d = run("smp", path)
    n = len(d["q"])
    mk = lambda pfx, m: P.CSC(m, n, d[pfx + "p"], d[pfx + "i"], d[pfx + "x"])
    meq, mineq = int(d["meq"][0]), int(d["mineq"][0])
    return P.QP(mk("H", n), d["q"], mk("A", meq), d["b"], mk("C", mineq), d["d"])


def json_qp(path):
    """tests/1.json of the reference (Eigen sparse matrices as JSON)."""
    with open(path) as f:
        js = json.load(f)

    def sp(o):
        rows, cols = int(o["rows"]), int(o["cols"])
        return P.CSC(rows, cols, np.asarray(o["outer_starts"], np.int32),
                     np.asarray(o["inner_indices"], np.int32), np.asarray(o["values"], np.float64))

    def vec(o):
        return np.asarray(o["values"] if isinstance(o, dict) else o, np.float64).ravel()

    H = sp(js["H"])
    qp = P.QP(H, vec(js["q"]), sp(js["A"]), vec(js["b"]), sp(js["C"]), vec(js["d"]))
    return qp, vec(js["x"]), vec(js["y"]), vec(js["z"])


def main(ref):
    # --- LBL (SolverSettings mode 0), examples/lbl_main.cpp:34-43 ---------------
    ex = P.CSC(2, 2, np.array([0, 1, 2], np.int32), np.array([0, 1], np.int32), np.array([2.0, 2.0]))
    lbl_case("lbl_example", ex, np.array([-4.0, -4.0]), req_ref_iter=2, reg_diag=1e-9)
    rng = np.random.default_rng(1)
    H = P.laplacian2d(12, 0.5)
    lbl_case("lbl_lap2d", H, rng.standard_normal(H.ncol), req_ref_iter=2, reg_diag=1e-9)
    rng = np.random.default_rng(2)
    H = P.laplacian2d(10)
    A = P.random_rows(15, H.ncol, 3, rng)
    K = P.kkt_lower(H, A, 1e-8)
    lbl_case("lbl_kkt2d", K, rng.standard_normal(K.ncol), req_ref_iter=2, reg_diag=1e-9)
    K, rhs = P.lbl_kkt(seed=3, grid3d=8, m=40, per_row=6)
    lbl_case("lbl_kkt3d", K, rhs, req_ref_iter=2, reg_diag=1e-9)
    K, rhs = P.lbl_kkt(seed=4, grid3d=12, m=150, per_row=6)
    lbl_case("lbl_kkt3d_mid", K, rhs, req_ref_iter=3, max_inner_iter=3, reg_diag=1e-9)
    # zero diagonal entries that the perturbation rule (|a_jj| < reg_diag) replaces
    rng = np.random.default_rng(5)
    H = P.laplacian2d(6)
    A = P.random_rows(10, H.ncol, 4, rng)
    K = P.kkt_lower(H, A, 0.0)
    lbl_case("lbl_kkt_zero_diag", K, rng.standard_normal(K.ncol), req_ref_iter=2, reg_diag=1e-9)

    # symmetric indefinite matrices with zero diagonals: 2x2 pivots
    K = P.sym_indefinite(seed=6, n=40, density=1.0)
    lbl_case("lbl_indef_dense", K, np.random.default_rng(6).standard_normal(40), req_ref_iter=2, reg_diag=1e-9)
    K = P.sym_indefinite(seed=8, n=300, density=0.02)
    lbl_case("lbl_indef_sparse", K, np.random.default_rng(8).standard_normal(300), req_ref_iter=3,
             max_inner_iter=3, reg_diag=1e-9)

    # strongly indefinite KKT (2500 zero-diagonal constraint columns, 2500
    # negative eigenvalues), kappa ~ 1e4, 2x2 pivots inside supernodes up to
    # 2545 columns wide: the FP32 multi-CTA kernels at their default thresholds
    K, rhs = P.lbl_kkt(seed=22, grid3d=16, m=2500, per_row=4, delta=0.0)
    lbl_case_light("lblw_kkt3d_hard", K, rhs, req_ref_iter=2, reg_diag=1e-9)

    # --- NASOQ QPs ---------------------------------------------------------------
    for pname in ("matt_qp1", "test05_0"):
        qp = smp_qp(os.path.join(ref, "data", pname + ".yml"))
        # data/out_correct.csv rows: NASOQ-Fixed and NASOQ (PREDET) at eps 1e-3
        qp_case(f"qp_{pname}_fixed", qp, variant=0, eps_abs=1e-3, max_iter=2, diag_perturb=1e-9)
        qp_case(f"qp_{pname}_predet", qp, variant=3, eps_abs=1e-3, max_iter=2, diag_perturb=1e-9)
    if wanted("qp_test1json"):
        qp, x, y, z = json_qp(os.path.join(ref, "tests", "1.json"))
        inp = qp_inputs(qp, variant=3, eps_abs=1e-3, max_iter=0, diag_perturb=1e-9, stop_tol=1e-15,
                        max_iter_nas=4000)
        out = run("qp", inp)
        out.update({"json_x": x, "json_y": y, "json_z": z})
        save_case("qp_test1json", inp, out)
    qp = P.qp_random_convex(seed=0)
    qp_case("qp_random_c1_predet", qp, variant=3, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)
    qp_case("qp_random_c1_fixed", qp, variant=0, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)
    qp = P.qp_random_convex(seed=7, grid=12, meq=20, mineq=120)
    qp_case("qp_random_small", qp, variant=3, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)
    for N in (10, 25):
        qp = P.qp_mpc(seed=11 + N, horizon=N)
        qp_case(f"qp_mpc_N{N}", qp, variant=3, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)

    # Ruiz equilibration (Nasoq::scaling > 0, src/nasoq.cpp:1352-1483)
    qp = P.qp_ill_scaled(seed=21)
    qp_case("qp_scaled_ill_ruiz", qp, variant=3, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9, scaling=10)
    qp_case("qp_scaled_ill_none", qp, variant=3, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)
    qp = P.qp_random_convex(seed=7, grid=12, meq=20, mineq=120)
    qp_case("qp_scaled_random_ruiz", qp, variant=0, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9, scaling=5)

    # the large bounded bilaplacian QP family at a size the reference solves in a second
    qp = P.bilaplacian_bounded(seed=0, grid=40, pins=20)
    qp_case("qp_bilap_g40", qp, variant=0, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)
    # supernodes wider than the 192-column multi-CTA threshold
    qp = P.bilaplacian_bounded(seed=1, grid=80, pins=80)
    qp_case("qp_bilap_g80", qp, variant=0, eps_abs=1e-8, max_iter=2, diag_perturb=1e-9)


if __name__ == "__main__":
    args = sys.argv[1:]
    if "--only" in args:
        k = args.index("--only")
        ONLY = args[k + 1]
        del args[k:k + 2]
    main(args[0] if args else os.environ.get("NASOQ_REFERENCE", "/root/reference"))
