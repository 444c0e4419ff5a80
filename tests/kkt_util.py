"""Test helpers: the QP super-KKT matrix exactly as the reference's
build_super_matrix forms it (src/QP/linear_solver_wrapper.cpp:246-350)."""
import numpy as np

from nasoq_gb300.problems import CSC


def super_kkt(Hp, Hi, Hx, Ap, Ai, Ax, Cp, Ci, Cx, meq, mineq):
    """Columns 0..n-1: H's lower column, then the equality rows (n + i) with
    their values, then the inequality rows (n + meq + i) with value 0;
    columns n..N-1: a single zero diagonal.  Returns (K, extra_cols, base)."""
    n = len(Hp) - 1
    N = n + meq + mineq
    p = [0]
    rows, vals = [], []
    for j in range(n):
        r = list(Hi[Hp[j]:Hp[j + 1]])
        v = list(Hx[Hp[j]:Hp[j + 1]])
        if meq > 0:
            r += [n + int(i) for i in Ai[Ap[j]:Ap[j + 1]]]
            v += list(Ax[Ap[j]:Ap[j + 1]])
        if mineq > 0:
            r += [n + meq + int(i) for i in Ci[Cp[j]:Cp[j + 1]]]
            v += [0.0] * (Cp[j + 1] - Cp[j])
        rows += r
        vals += v
        p.append(len(rows))
    for k in range(n, N):
        rows.append(k)
        vals.append(0.0)
        p.append(len(rows))
    K = CSC(N, N, np.asarray(p, np.int32), np.asarray(rows, np.int32), np.asarray(vals, np.float64))
    base = n + meq
    extra = np.zeros(N, np.int32)
    extra[base:] = 1
    return K, extra, base
