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
