"""ctypes binding of the oracle restatement (oracle/port/ldlt_port.cpp).
Checker and CPU baseline only."""
import ctypes as C
import glob
import os

import numpy as np

from . import build as _build

_lib = None


def openblas_path():
    import scipy
    d = os.path.realpath(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs"))
    c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    if not c:
        raise RuntimeError("SciPy's bundled OpenBLAS was not found")
    return c[0]


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build())
        L.nqp_init.argtypes = [C.c_char_p]
        L.nqp_set_threads.argtypes = [C.c_int]
        L.nqp_spmv.argtypes = [C.c_int] + [C.c_void_p] * 5
        L.nqp_solve.argtypes = [C.c_int] + [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 8 + \
            [C.c_int, C.c_int, C.c_double, C.c_double] + [C.c_void_p] * 7
        rc = L.nqp_init(openblas_path().encode())
        if rc != 0:
            raise RuntimeError(f"oracle: OpenBLAS symbols not resolved ({rc})")
        _lib = L
    return _lib


def set_threads(t):
    lib().nqp_set_threads(int(t))


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def spmv(n, Ap, Ai, Ax, x):
    """y = K x, K symmetric given by its lower triangle in CSC (the
    reference's spmv_csc_sym_one_int, src/matrixVector/spmv_CSC.cpp:26-102,
    with alpha = 1, beta = 0)."""
    a = lambda v, t: np.ascontiguousarray(v, t)
    Ap, Ai, Ax, x = a(Ap, np.int32), a(Ai, np.int32), a(Ax, np.float64), a(x, np.float64)
    y = np.zeros(n)
    if lib().nqp_spmv(int(n), _p(Ap), _p(Ai), _p(Ax), _p(x), _p(y)) != 0:
        raise ValueError("oracle spmv: bad arguments")
    return y


def solve(n, Ap, Ai, Ax, Ax_ref, sym, rhs, req_ref_iter=2, max_inner_iter=2, tol_abs=1e-15, tol_rel=1e-15,
          want_factor=False):
    """sym: object with perm, super, lpi, ls, colp, sparent, col2sup (numpy)."""
    L = lib()
    a = lambda v, t: np.ascontiguousarray(v, t)
    Ap, Ai, Ax, Ax_ref, rhs = a(Ap, np.int32), a(Ai, np.int32), a(Ax, np.float64), a(Ax_ref, np.float64), \
        a(rhs, np.float64)
    perm, sup, lpi, ls = a(sym.perm, np.int32), a(sym.super, np.int32), a(sym.lpi, np.int64), a(sym.ls, np.int32)
    colp, spar, c2s = a(sym.colp, np.int64), a(sym.sparent, np.int32), a(sym.col2sup, np.int32)
    ns = len(sup) - 1
    x = np.zeros(n)
    times = np.zeros(2)
    nit = C.c_int(0)
    Lo = Do = Po = So = None
    if want_factor:
        Lo = np.zeros(max(int(colp[-1]), 1))
        Do = np.zeros(2 * n)
        Po = np.zeros(n, np.int32)
        So = np.zeros(max(int(lpi[-1]), 1), np.int32)
    rc = L.nqp_solve(n, _p(Ap), _p(Ai), _p(Ax), _p(Ax_ref), ns, _p(perm), _p(sup), _p(lpi), _p(ls), _p(colp),
                     _p(spar), _p(c2s), _p(rhs), req_ref_iter, max_inner_iter, tol_abs, tol_rel, _p(x), _p(times),
                     C.byref(nit), _p(Lo), _p(Do), _p(Po), _p(So))
    if rc != 0:
        raise RuntimeError(f"oracle solve failed ({rc})")
    out = {"x": x, "factor_s": times[0], "solve_s": times[1], "num_ref_iter": nit.value}
    if want_factor:
        out.update({"L": Lo[:int(colp[-1])], "D": Do, "perm": Po, "ls": So[:int(lpi[-1])]})
    return out


def qp_settings_resolved(qp, variant=0, eps_abs=1e-8, diag_perturb=1e-9, max_iter=2, stop_tol=1e-15):
    """(reg, outer, inner, tol) as the reference derives them."""
    H = qp.H
    total_nnz = int(H.p[-1]) + int(qp.C.p[-1]) if qp.C.nrow else int(H.p[-1])
    frob, s = 0.0, 0.0
    for j in range(H.ncol):
        for k in range(H.p[j], H.p[j + 1]):
            s = abs(float(H.x[k]))
            frob += s * s if H.i[k] == j else (2 * s * s if H.i[k] > j else 0.0)
    hn = np.sqrt(frob) if np.isfinite(s) else 0.0
    if variant == 0:  # Fixed
        if eps_abs >= 1e-3:
            it = 0
        elif 1e-7 < eps_abs <= 1e-4:
            it = 1
        elif 1e-10 < eps_abs <= 1e-7:
            it = 2
        else:
            it = 4
        if total_nnz <= 20000:
            it = 3
        return (1e-7 if hn < 1 else 1e-9), it, it, 1e-15
    if variant == 1:  # AUTO
        reg, lo, hi, large = 1e-8, 2, 9, 0
        if eps_abs >= 1e-3:
            lo //= 2
            hi //= 2
        elif eps_abs < 1e-8:
            lo *= 2
            large = large * 2 + 1
        it, tol = large, stop_tol
        n, mi = H.ncol, qp.C.nrow
        if total_nnz < 3e5:
            it, tol = lo, 1e-10
            if hn < 1:
                reg, it, tol = 1e-7, lo, 1e-15
            elif mi / n > 2.5:
                reg, tol, it = 1e-10, 1e-16, lo
            elif n > 1e4 and mi >= 1e4:
                reg, it, tol = 1e-11, hi, 1e-15
        elif hn < 1:
            reg, it, tol = 1e-7, 2, 1e-15
        return reg, it, it, tol
    return diag_perturb, max_iter, max_iter, stop_tol


def super_kkt(qp):
    """Lower CSC of [H; A; C] (constraint columns: a zero diagonal) with every
    constraint value present, as the reference's build_super_matrix lays it
    out."""
    n, meq, mi = qp.H.ncol, qp.A.nrow, qp.C.nrow
    N = n + meq + mi
    p, i, x = [0], [], []
    for j in range(n):
        for (M, off) in ((qp.H, 0), (qp.A, n), (qp.C, n + meq)):
            if M.nrow == 0 and M is not qp.H:
                continue
            for k in range(M.p[j], M.p[j + 1]):
                i.append(int(M.i[k]) + off)
                x.append(float(M.x[k]))
        p.append(len(i))
    for k in range(n, N):
        i.append(k)
        x.append(0.0)
        p.append(len(i))
    return N, np.asarray(p, np.int32), np.asarray(i, np.int32), np.asarray(x, np.float64)


def qp_solve(qp, variant=0, eps_abs=1e-8, diag_perturb=1e-9, max_iter=2, stop_tol=1e-15, max_iter_nas=200000,
             sym=None):
    """NASOQ on one QP (CPU restatement).  sym: the symbolic analysis of the
    super-KKT pattern (nasoq_gb300.Symbolic with the constraint columns
    hidden), reused across problems of one pattern."""
    L = lib()
    if not hasattr(L, "_qp_ready"):
        L.nqp_qp_solve.argtypes = [C.c_int] * 4 + [C.c_void_p] * 6 + [C.c_int] + [C.c_void_p] * 7 + \
            [C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double] + [C.c_void_p] * 6
        L._qp_ready = True
    n, meq, mi = qp.H.ncol, qp.A.nrow, qp.C.nrow
    N, Kp, Ki, Kx = super_kkt(qp)
    if sym is None:
        import nasoq_gb300 as nq
        ex = np.zeros(N, np.int32)
        ex[n + meq:] = 1
        sym = nq.Symbolic(N, Kp, Ki, extra_cols=ex)
    reg, outer, inner, tol = qp_settings_resolved(qp, variant, eps_abs, diag_perturb, max_iter, stop_tol)
    a = lambda v, t: np.ascontiguousarray(v, t)
    arrs = dict(perm=a(sym.perm, np.int32), sup=a(sym.super, np.int32), lpi=a(sym.lpi, np.int64),
                ls=a(sym.ls, np.int32), colp=a(sym.colp, np.int64), spar=a(sym.sparent, np.int32),
                c2s=a(sym.col2sup, np.int32))
    q, b, d = a(qp.q, np.float64), a(qp.b if meq else np.zeros(1), np.float64), a(qp.d if mi else np.zeros(1),
                                                                                    np.float64)
    x, y, z = np.zeros(n), np.zeros(max(meq, 1)), np.zeros(max(mi, 1))
    act = np.zeros(max(mi, 1), np.int32)
    info = np.zeros(3, np.int32)
    norms = np.zeros(5)
    rc = L.nqp_qp_solve(N, n, meq, mi, _p(Kp), _p(Ki), _p(Kx), _p(q), _p(b), _p(d), len(arrs["sup"]) - 1,
                        _p(arrs["perm"]), _p(arrs["sup"]), _p(arrs["lpi"]), _p(arrs["ls"]), _p(arrs["colp"]),
                        _p(arrs["spar"]), _p(arrs["c2s"]), reg, outer, inner, tol, eps_abs, max_iter_nas, reg,
                        _p(x), _p(y), _p(z), _p(act), _p(info), _p(norms))
    if rc != 0:
        raise RuntimeError(f"oracle QP solve failed ({rc})")
    return {"x": x, "y": y[:meq], "z": z[:mi], "active": act[:info[2]].copy(), "status": int(info[0]),
            "num_iter": int(info[1]), "objective": norms[0], "lag_res": norms[1], "cons_sat": norms[2],
            "nonneg": norms[3], "compl": norms[4]}
