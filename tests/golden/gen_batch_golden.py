"""Generates tests/golden/batch_mixed.nqa: the reference NASOQ library
(built out-of-tree by oracle/Makefile into oracle/_ref/) solving a mixed batch
of QPs one by one -- uneven MPC problems, small random convex QPs (these take
dual steps that drop constraints), and instances of the parametric MPC family
(one sparsity pattern shared by many problems).

The inputs are not stored: the parity test rebuilds them from the recorded
generator parameters (seeded numpy generators in nasoq_gb300.problems) and
checks each problem's input checksum first.  Run in the development
container, where the reference sources live:

    make -C oracle && python tests/golden/gen_batch_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import gen_golden as G  # noqa: E402
import nqa  # noqa: E402
from nasoq_gb300 import problems as P  # noqa: E402

SETTINGS = dict(variant=0, eps_abs=1e-8, diag_perturb=1e-9, max_iter=2, stop_tol=1e-15, max_iter_nas=200000)

# kind 0: qp_mpc(a, b); kind 1: qp_random_convex(seed=a, grid=b, meq=c, mineq=d);
# kind 2: mpc_parametric(0) at theta = default_rng(a).standard_normal(32)
KIND_MPC, KIND_RANDOM, KIND_PARAM = 0, 1, 2


def specs():
    out = [(KIND_MPC, s, h, 0, 0) for s, h in P.mpc_batch_specs(64, seed=11)]
    rng = np.random.default_rng(12)
    for t in range(16):
        grid = int(rng.integers(5, 10))
        meq = int(rng.integers(3, 15))
        mineq = int(rng.integers(20, 90))
        out.append((KIND_RANDOM, 500 + t, grid, meq, mineq))
    out += [(KIND_PARAM, 900 + t, 0, 0, 0) for t in range(16)]
    return out


def build(spec, fam=None):
    kind, a, b, c, d = spec
    if kind == KIND_MPC:
        return P.qp_mpc(a, b)
    if kind == KIND_RANDOM:
        return P.qp_random_convex(seed=a, grid=b, meq=c, mineq=d)
    fam = fam or P.mpc_parametric(0)
    th = np.random.default_rng(a).standard_normal(32)
    return P.QP(fam.base.H, fam.q_of(th), fam.base.A, fam.base.b, fam.base.C, fam.d_of(th))


def main():
    fam = P.mpc_parametric(0)
    sp = specs()
    rec = {k: [] for k in ("status", "num_iter", "active_size", "objective", "lag_res", "cons_sat", "checksum")}
    xs, ys, zs, acts = [], [], [], []
    for t, spec in enumerate(sp):
        qp = build(spec, fam)
        out = G.run("qp", G.qp_inputs(qp, **SETTINGS))
        rec["status"].append(int(out["status"][0]))
        rec["num_iter"].append(int(out["num_iter"][0]))
        rec["active_size"].append(len(out["active_set"]))
        rec["objective"].append(float(out["objective"][0]))
        rec["lag_res"].append(float(out["lag_res"][0]))
        rec["cons_sat"].append(float(out["cons_sat_norm"][0]))
        rec["checksum"].append(P.qp_checksum(qp))
        xs.append(out["x"])
        ys.append(out["y"] if "y" in out else np.zeros(0))
        zs.append(out["z"])
        acts.append(np.asarray(out["active_set"], np.int32))
        print(t, spec, "status", rec["status"][-1], "iter", rec["num_iter"][-1], "active", rec["active_size"][-1])
    arrs = {"spec": np.asarray(sp, np.int64).reshape(-1)}
    for k, v in rec.items():
        arrs[k] = np.asarray(v, np.float64 if k in ("objective", "lag_res", "cons_sat", "checksum") else np.int32)
    for name, lst in (("x", xs), ("y", ys), ("z", zs), ("act", acts)):
        arrs[name + "_ptr"] = np.concatenate([[0], np.cumsum([len(a) for a in lst])]).astype(np.int64)
        arrs[name] = np.concatenate(lst) if lst else np.zeros(0)
    for k, v in SETTINGS.items():
        arrs["set_" + k] = np.array([float(v)])
    nqa.save(os.path.join(HERE, "batch_mixed.nqa"), arrs)
    print("saved", sum(a.nbytes for a in arrs.values()) / 1024, "KiB")


if __name__ == "__main__":
    main()
