"""nasoq_gb300: NASOQ's dual active-set QP solver on one GB300 GPU -- batched
QPs with the whole active-set loop on the device (QPBatch), the learned
active-set warm start (MLP), single QPs (qp_solve), SMP files (load_smp) --
over supernodal Bunch-Kaufman LDL^T, supernodal solves and GMRES refinement
of sparse symmetric-indefinite (KKT) systems (Plan).

This module is a thin ctypes binding of the C ABI in include/nasoq_gb300.h
(built in-tree as nasoq_gb300/libnasoq_gb300.so by nasoq_gb300.build).  There
is no CPU fallback: every numeric call runs the CUDA kernels, and importing
the binding without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnasoq_gb300.so")

NQG_OK = 0
NQG_WARN_ZERO_PIVOT = 1
NQG_WARN_NONFINITE = 2
NQG_ERR_TIMEOUT = -5
NQG_FP64 = 0
NQG_FP32 = 1

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


class Settings(C.Structure):
    _fields_ = [("precision", C.c_int), ("req_ref_iter", C.c_int), ("max_inner_iter", C.c_int),
                ("tol_abs", C.c_double), ("tol_rel", C.c_double), ("reg_diag", C.c_double),
                ("regularization", C.c_int), ("n_relax", C.c_int * 3), ("z_relax", C.c_double * 3),
                ("reg_diag_fp32", C.c_double), ("solve_precision", C.c_int), ("perturb_plus_cols", C.c_int)]


class SymbolicInfo(C.Structure):
    _fields_ = [("n", C.c_int), ("nsuper", C.c_int), ("max_sup_wid", C.c_int), ("max_col", C.c_int),
                ("ssize", C.c_int64), ("xsize", C.c_int64), ("metis_seconds", C.c_double),
                ("total_seconds", C.c_double)]


class Timings(C.Structure):
    _fields_ = [("factor_ms", C.c_double), ("solve_ms", C.c_double), ("refine_ms", C.c_double),
                ("num_ref_iter", C.c_int), ("num_pivot_supernodes", C.c_int), ("num_2x2", C.c_int),
                ("last_residual", C.c_double)]


class KernelStats(C.Structure):
    _fields_ = [("launches", C.c_longlong), ("total_ms", C.c_double), ("alg_flops", C.c_double),
                ("alg_bytes", C.c_double)]


KERNEL_CLASSES = {"update": 0, "wide_panel": 1, "wide_trailing": 2, "bk": 3, "solve": 4, "spmv": 5, "other": 6,
                  "wide_pivot": 7, "pack": 8}


class QPSettings(C.Structure):
    _fields_ = [("variant", C.c_int), ("eps_abs", C.c_double), ("diag_perturb", C.c_double),
                ("stop_tol", C.c_double), ("max_iter", C.c_int), ("max_iter_nas", C.c_int), ("precision", C.c_int),
                ("scaling", C.c_int)]


class QPResult(C.Structure):
    _fields_ = [("status", C.c_int), ("num_iter", C.c_int), ("active_size", C.c_int), ("objective", C.c_double),
                ("primal_obj", C.c_double), ("dual_obj", C.c_double), ("lag_res", C.c_double),
                ("cons_sat_norm", C.c_double), ("non_negativity_infn", C.c_double),
                ("complementarity_infn", C.c_double), ("total_seconds", C.c_double),
                ("factor_seconds", C.c_double)]


class BatchSettings(C.Structure):
    _fields_ = [("qp", QPSettings), ("refine", C.c_int), ("refine_tol", C.c_double), ("threads", C.c_int),
                ("use_graph", C.c_int), ("stage", C.c_int), ("share_factor", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("status", C.c_int), ("num_iter", C.c_int), ("active_size", C.c_int), ("flags", C.c_int),
                ("refine_steps", C.c_int), ("solves", C.c_int), ("warm_dropped", C.c_int), ("pad", C.c_int),
                ("objective", C.c_double), ("lag_res", C.c_double), ("cons_sat_norm", C.c_double),
                ("non_negativity_infn", C.c_double), ("complementarity_infn", C.c_double)]


class BatchInfo(C.Structure):
    _fields_ = [("nprob", C.c_int), ("npatterns", C.c_int), ("grid", C.c_int), ("threads", C.c_int),
                ("blocks_per_sm", C.c_int), ("warp_factor", C.c_int), ("smem_bytes", C.c_int64), ("slot_bytes", C.c_int64),
                ("last_ms", C.c_double)]


_lib = None


def lib():
    """Loads libnasoq_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -m nasoq_gb300.build` first")
    L = C.CDLL(LIB_PATH)
    L.nqg_default_settings.argtypes = [C.POINTER(Settings)]
    L.nqg_default_settings.restype = None
    L.nqg_status_str.argtypes = [C.c_int]
    L.nqg_status_str.restype = C.c_char_p
    L.nqg_symbolic_create.argtypes = [C.c_int, _i32p, _i32p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(C.c_void_p)]
    L.nqg_symbolic_get_info.argtypes = [C.c_void_p, C.POINTER(SymbolicInfo)]
    L.nqg_symbolic_export.argtypes = [C.c_void_p] + [C.c_void_p] * 11
    L.nqg_symbolic_destroy.argtypes = [C.c_void_p]
    L.nqg_symbolic_destroy.restype = None
    L.nqg_plan_create.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.POINTER(Settings),
                                  C.POINTER(C.c_void_p)]
    L.nqg_plan_destroy.argtypes = [C.c_void_p]
    L.nqg_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.nqg_set_wait_limit.argtypes = [C.c_void_p, C.c_longlong]
    L.nqg_get_symbolic.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.nqg_set_values.argtypes = [C.c_void_p, _f64p]
    L.nqg_edit_values.argtypes = [C.c_void_p, C.c_int, _i64p, _f64p]
    L.nqg_factor.argtypes = [C.c_void_p]
    L.nqg_refactor.argtypes = [C.c_void_p, C.c_int, _i32p]
    L.nqg_set_visibility.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_solve.argtypes = [C.c_void_p, _f64p, _f64p]
    L.nqg_solve_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_refine_only.argtypes = [C.c_void_p, _f64p, _f64p]
    L.nqg_ldlt_solve_ordered_device.argtypes = [C.c_void_p, C.c_void_p]
    L.nqg_spmv_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_get_timings.argtypes = [C.c_void_p, C.POINTER(Timings)]
    L.nqg_get_factor.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_get_device_status.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    L.nqg_set_profiling.argtypes = [C.c_void_p, C.c_int]
    L.nqg_get_kernel_stats.argtypes = [C.c_void_p, C.c_int, C.POINTER(KernelStats)]
    L.nqg_get_launch_count.argtypes = [C.c_void_p, C.POINTER(C.c_longlong)]
    L.nqg_qp_default_settings.argtypes = [C.POINTER(QPSettings)]
    L.nqg_qp_default_settings.restype = None
    L.nqg_qp_solve.argtypes = [C.c_int] + [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 4 + [C.c_int] + \
        [C.c_void_p] * 4 + [C.POINTER(QPSettings), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(QPResult)]
    L.nqg_batch_default_settings.argtypes = [C.POINTER(BatchSettings)]
    L.nqg_batch_default_settings.restype = None
    L.nqg_batch_create.argtypes = [C.POINTER(BatchSettings), C.POINTER(C.c_void_p)]
    L.nqg_batch_add.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4 + [C.c_int] + \
        [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 4
    L.nqg_batch_finalize.argtypes = [C.c_void_p]
    L.nqg_batch_set_vectors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_batch_set_vectors_async.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_batch_set_warm_start.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.nqg_batch_solve.argtypes = [C.c_void_p]
    L.nqg_batch_solve_async.argtypes = [C.c_void_p]
    L.nqg_batch_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.POINTER(QPResult)]
    L.nqg_batch_get_all.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_batch_get_info.argtypes = [C.c_void_p, C.POINTER(BatchInfo)]
    L.nqg_batch_get_stream.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.nqg_batch_last_error.argtypes = [C.c_void_p]
    L.nqg_batch_last_error.restype = C.c_char_p
    L.nqg_batch_destroy.argtypes = [C.c_void_p]
    L.nqg_batch_warm_start_from_scores.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float]
    L.nqg_batch_clear_warm_starts.argtypes = [C.c_void_p]
    L.nqg_mlp_create.argtypes = [C.c_int, C.c_void_p, C.c_ulonglong, C.POINTER(C.c_void_p)]
    L.nqg_mlp_num_params.argtypes = [C.c_void_p, C.POINTER(C.c_long), C.POINTER(C.c_long)]
    L.nqg_mlp_set_weights.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_mlp_get_weights.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_mlp_forward.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.nqg_mlp_forward_device.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.nqg_mlp_loss_grad.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_float,
                                    C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
    L.nqg_mlp_set_data.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.nqg_mlp_train.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_ulonglong, C.c_void_p]
    L.nqg_mlp_last_error.argtypes = [C.c_void_p]
    L.nqg_mlp_last_error.restype = C.c_char_p
    L.nqg_mlp_destroy.argtypes = [C.c_void_p]
    L.nqg_batch_set_profiling.argtypes = [C.c_void_p, C.c_int]
    L.nqg_batch_get_profile.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    L.nqg_smp_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.nqg_qp_data_error.argtypes = [C.c_void_p]
    L.nqg_qp_data_error.restype = C.c_char_p
    L.nqg_qp_data_description.argtypes = [C.c_void_p]
    L.nqg_qp_data_description.restype = C.c_char_p
    L.nqg_qp_data_sizes.argtypes = [C.c_void_p] + [C.c_void_p] * 4
    L.nqg_qp_data_export.argtypes = [C.c_void_p] + [C.c_void_p] * 12
    L.nqg_qp_data_extras.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    L.nqg_qp_data_destroy.argtypes = [C.c_void_p]
    _lib = L
    return L


class NasoqError(RuntimeError):
    pass


def _check(rc, what):
    if rc < 0:
        raise NasoqError(f"{what}: {lib().nqg_status_str(rc).decode()} ({rc})")
    return rc


def default_settings(**kw) -> Settings:
    s = Settings()
    lib().nqg_default_settings(C.byref(s))
    for k, v in kw.items():
        if k in ("n_relax", "z_relax"):
            getattr(s, k)[:] = v
        else:
            setattr(s, k, v)
    return s


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Symbolic:
    """Host symbolic analysis (no GPU needed)."""

    def __init__(self, n, Ap, Ai, extra_cols=None, n_relax=(4, 16, 48), z_relax=(0.8, 0.1, 0.05)):
        L = lib()
        Ap = np.ascontiguousarray(Ap, np.int32)
        Ai = np.ascontiguousarray(Ai, np.int32)
        ex = None if extra_cols is None else np.ascontiguousarray(extra_cols, np.int32)
        nr = (C.c_int * 3)(*n_relax)
        zr = (C.c_double * 3)(*z_relax)
        h = C.c_void_p()
        _check(L.nqg_symbolic_create(int(n), Ap, Ai, _ptr(ex), C.cast(nr, C.c_void_p), C.cast(zr, C.c_void_p),
                                     C.byref(h)), "symbolic analysis")
        self._h = h
        self._own = True
        self._load()

    @classmethod
    def _wrap(cls, handle):
        self = cls.__new__(cls)
        self._h = handle
        self._own = False
        self._load()
        return self

    def _load(self):
        L = lib()
        info = SymbolicInfo()
        L.nqg_symbolic_get_info(self._h, C.byref(info))
        self.info = info
        n, ns = info.n, info.nsuper
        a = {k: np.zeros(n, np.int32) for k in ("perm", "iperm", "parent", "colcount", "col2sup", "extra_cols")}
        a["super"] = np.zeros(ns + 1, np.int32)
        a["sparent"] = np.zeros(ns, np.int32)
        a["lpi"] = np.zeros(ns + 1, np.int64)
        a["ls"] = np.zeros(max(info.ssize, 1), np.int32)
        a["colp"] = np.zeros(n + 1, np.int64)
        L.nqg_symbolic_export(self._h, *[_ptr(a[k]) for k in ("perm", "iperm", "parent", "colcount", "super",
                                                              "sparent", "col2sup", "lpi", "ls", "colp",
                                                              "extra_cols")])
        a["ls"] = a["ls"][:info.ssize]
        self.__dict__.update(a)

    def __del__(self):
        if getattr(self, "_own", False) and getattr(self, "_h", None):
            lib().nqg_symbolic_destroy(self._h)
            self._h = None


class Plan:
    """A factorization plan on the GPU (symbolic analysis + device buffers)."""

    def __init__(self, n, Ap, Ai, Ax, extra_cols=None, settings: Settings | None = None, **kw):
        L = lib()
        self.n = int(n)
        self.Ap = np.ascontiguousarray(Ap, np.int32)
        self.Ai = np.ascontiguousarray(Ai, np.int32)
        Ax = np.ascontiguousarray(Ax, np.float64)
        ex = None if extra_cols is None else np.ascontiguousarray(extra_cols, np.int32)
        self.settings = settings if settings is not None else default_settings(**kw)
        h = C.c_void_p()
        _check(L.nqg_plan_create(self.n, self.Ap, self.Ai, Ax, _ptr(ex), C.byref(self.settings), C.byref(h)),
               "plan create")
        self._h = h
        sh = C.c_void_p()
        L.nqg_get_symbolic(h, C.byref(sh))
        self.symbolic = Symbolic._wrap(sh)

    def factor(self):
        return _check(lib().nqg_factor(self._h), "factor")

    def refactor(self, snodes):
        sn = np.ascontiguousarray(snodes, np.int32)
        return _check(lib().nqg_refactor(self._h, len(sn), sn), "refactor")

    def set_values(self, Ax):
        _check(lib().nqg_set_values(self._h, np.ascontiguousarray(Ax, np.float64)), "set values")

    def edit_values(self, idx, vals):
        idx = np.ascontiguousarray(idx, np.int64)
        vals = np.ascontiguousarray(vals, np.float64)
        _check(lib().nqg_edit_values(self._h, len(idx), idx, vals), "edit values")

    def set_visibility(self, visible_sn=None, hidden_col=None):
        v = None if visible_sn is None else np.ascontiguousarray(visible_sn, np.uint8)
        hd = None if hidden_col is None else np.ascontiguousarray(hidden_col, np.uint8)
        _check(lib().nqg_set_visibility(self._h, _ptr(v), _ptr(hd)), "set visibility")

    def solve(self, rhs):
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.empty(self.n, np.float64)
        _check(lib().nqg_solve(self._h, rhs, x), "solve")
        return x

    def refine_only(self, rhs):
        """GMRES refinement alone, started from x = rhs (iterative_ref_only)."""
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.empty(self.n, np.float64)
        _check(lib().nqg_refine_only(self._h, rhs, x), "refine only")
        return x

    def solve_device(self, d_rhs_ptr, d_x_ptr):
        _check(lib().nqg_solve_device(self._h, C.c_void_p(d_rhs_ptr), C.c_void_p(d_x_ptr)), "solve")

    def spmv_device(self, d_x_ptr, d_y_ptr):
        """y = K x (original ordering, the values given at creation or by
        set_values, without perturbation); device buffers of n doubles,
        queued on the plan's stream."""
        _check(lib().nqg_spmv_device(self._h, C.c_void_p(d_x_ptr), C.c_void_p(d_y_ptr)), "spmv")

    def set_stream(self, stream_ptr):
        _check(lib().nqg_set_stream(self._h, C.c_void_p(stream_ptr)), "set stream")

    def set_wait_limit(self, polls=0):
        """Polls before a cross-CTA wait gives up (<= 0: the default)."""
        _check(lib().nqg_set_wait_limit(self._h, C.c_longlong(int(polls))), "set wait limit")

    def timings(self) -> Timings:
        t = Timings()
        lib().nqg_get_timings(self._h, C.byref(t))
        return t

    def factor_arrays(self):
        s = self.symbolic
        vals = np.zeros(max(s.info.xsize, 1), np.float64)
        d = np.zeros(2 * self.n, np.float64)
        perm = np.zeros(self.n, np.int32)
        ls = np.zeros(max(s.info.ssize, 1), np.int32)
        _check(lib().nqg_get_factor(self._h, _ptr(vals), _ptr(d), _ptr(perm), _ptr(ls)), "get factor")
        return vals[:s.info.xsize], d, perm, ls[:s.info.ssize]

    def set_profiling(self, on=True):
        _check(lib().nqg_set_profiling(self._h, 1 if on else 0), "set profiling")

    def kernel_stats(self):
        out = {}
        for name, cls in KERNEL_CLASSES.items():
            st = KernelStats()
            _check(lib().nqg_get_kernel_stats(self._h, cls, C.byref(st)), "kernel stats")
            out[name] = {"launches": st.launches, "total_ms": st.total_ms, "alg_flops": st.alg_flops,
                         "alg_bytes": st.alg_bytes}
        return out

    def launch_count(self):
        v = C.c_longlong(0)
        lib().nqg_get_launch_count(self._h, C.byref(v))
        return v.value

    def device_status(self):
        v = C.c_int(0)
        lib().nqg_get_device_status(self._h, C.byref(v))
        return v.value

    def close(self):
        if getattr(self, "_h", None):
            lib().nqg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


VARIANTS = {"fixed": 0, "auto": 1, "tuned": 2, "predet": 3}


def qp_settings(**kw) -> QPSettings:
    s = QPSettings()
    lib().nqg_qp_default_settings(C.byref(s))
    for k, v in kw.items():
        if k == "variant" and isinstance(v, str):
            v = VARIANTS[v.lower()]
        setattr(s, k, v)
    return s


def load_smp(path):
    """Reads an SMP QP file (the reference's smp-format) into a
    problems.QP  min 1/2 x'Hx + q'x  s.t.  A x = b, C x <= d, with the file's
    constant term, stated optimum, primals, duals and description in
    QP.meta.  Two-sided rows l <= c'x <= u become c'x <= u, -c'x <= -l."""
    from nasoq_gb300 import problems as P
    L = lib()
    h = C.c_void_p()
    rc = L.nqg_smp_load(os.fsencode(path), C.byref(h))
    try:
        if rc < 0:
            msg = L.nqg_qp_data_error(h).decode() if h else "cannot open file"
            raise NasoqError(f"load_smp({path}): {msg}")
        n, meq, mineq = C.c_int(), C.c_int(), C.c_int()
        nnz = np.zeros(3, np.int64)
        L.nqg_qp_data_sizes(h, C.byref(n), C.byref(meq), C.byref(mineq), _ptr(nnz))
        n, meq, mineq = n.value, meq.value, mineq.value
        Hp, Ap, Cp = (np.zeros(n + 1, np.int32) for _ in range(3))
        Hi, Ai, Ci = (np.zeros(max(int(k), 1), np.int32) for k in nnz)
        Hx, Ax, Cx = (np.zeros(max(int(k), 1), np.float64) for k in nnz)
        q, b, d = np.zeros(max(n, 1)), np.zeros(max(meq, 1)), np.zeros(max(mineq, 1))
        L.nqg_qp_data_export(h, *[_ptr(a) for a in (Hp, Hi, Hx, q, Ap, Ai, Ax, b, Cp, Ci, Cx, d)])
        fixed, opt = C.c_double(), C.c_double()
        npr, ndu = C.c_int(), C.c_int()
        L.nqg_qp_data_extras(h, C.byref(fixed), C.byref(opt), C.byref(npr), None, C.byref(ndu), None)
        prim, dual = np.zeros(max(npr.value, 1)), np.zeros(max(ndu.value, 1))
        L.nqg_qp_data_extras(h, None, None, None, _ptr(prim), None, _ptr(dual))
        meta = {"kind": "smp", "path": os.fspath(path), "fixed": fixed.value, "optimal_objective": opt.value,
                "primals": prim[:npr.value], "duals": dual[:ndu.value],
                "description": L.nqg_qp_data_description(h).decode()}
    finally:
        if h:
            L.nqg_qp_data_destroy(h)
    k0, k1, k2 = (int(k) for k in nnz)
    return P.QP(P.CSC(n, n, Hp, Hi[:k0], Hx[:k0]), q[:n], P.CSC(meq, n, Ap, Ai[:k1], Ax[:k1]), b[:meq],
                P.CSC(mineq, n, Cp, Ci[:k2], Cx[:k2]), d[:mineq], meta)


def qp_solve(H, q, A, b, Cm, d, settings: QPSettings | None = None, warm=None):
    """Solves min 1/2 x'Hx + q'x s.t. A x = b, Cm x <= d with the NASOQ
    active-set method on the GPU.  H, A, Cm are CSC objects with p/i/x
    arrays (H lower-stored).  warm = (x0, z0, active_set[, y0]) starts from a
    given point and active set.  Returns (x, y, z, active_set, QPResult)."""
    L = lib()
    n = int(H.ncol)
    meq, mineq = int(A.nrow), int(Cm.nrow)
    arr = lambda a, t: np.ascontiguousarray(a, t)
    Hp, Hi, Hx, qv = arr(H.p, np.int32), arr(H.i, np.int32), arr(H.x, np.float64), arr(q, np.float64)
    Ap, Ai, Ax, bv = arr(A.p, np.int32), arr(A.i, np.int32), arr(A.x, np.float64), arr(b, np.float64)
    Cp, Ci, Cx, dv = arr(Cm.p, np.int32), arr(Cm.i, np.int32), arr(Cm.x, np.float64), arr(d, np.float64)
    x = np.zeros(n)
    y = np.zeros(max(meq, 1))
    z = np.zeros(max(mineq, 1))
    act = np.zeros(max(mineq, 1), np.int32)
    res = QPResult()
    st = settings if settings is not None else qp_settings()
    x0 = z0 = y0 = as0 = None
    nas = 0
    if warm is not None:
        x0 = arr(warm[0], np.float64)
        z0 = arr(warm[1], np.float64)
        as0 = arr(warm[2], np.int32)
        nas = len(as0)
        if len(warm) > 3 and warm[3] is not None:
            y0 = arr(warm[3], np.float64)
    rc = L.nqg_qp_solve(n, _ptr(Hp), _ptr(Hi), _ptr(Hx), _ptr(qv), meq, _ptr(Ap), _ptr(Ai), _ptr(Ax), _ptr(bv),
                        mineq, _ptr(Cp), _ptr(Ci), _ptr(Cx), _ptr(dv), C.byref(st), _ptr(x0), _ptr(z0), _ptr(y0),
                        nas, _ptr(as0), _ptr(x), _ptr(y), _ptr(z), _ptr(act), C.byref(res))
    _check(rc, "qp solve")
    return x, y[:meq], z[:mineq], act[:res.active_size].copy(), res


def batch_settings(**kw) -> BatchSettings:
    """Batch settings; QP keys (variant, eps_abs, diag_perturb, stop_tol,
    max_iter, max_iter_nas, precision) go to the embedded QP settings."""
    s = BatchSettings()
    lib().nqg_batch_default_settings(C.byref(s))
    qp_keys = {f for f, _ in QPSettings._fields_}
    for k, v in kw.items():
        if k == "variant" and isinstance(v, str):
            v = VARIANTS[v.lower()]
        if k in qp_keys:
            setattr(s.qp, k, v)
        else:
            setattr(s, k, v)
    return s


class QPBatch:
    """Many QPs solved together on the GPU (nqg_batch_*): each problem runs
    the NASOQ active-set iteration to the end inside one CTA of a persistent
    kernel.  Problems are given as (H, q, A, b, Cm, d) with CSC objects (H
    lower-stored), the same as qp_solve."""

    def __init__(self, problems, settings: BatchSettings | None = None, **kw):
        L = lib()
        self.settings = settings if settings is not None else batch_settings(**kw)
        h = C.c_void_p()
        _check(L.nqg_batch_create(C.byref(self.settings), C.byref(h)), "batch create")
        self._h = h
        self.sizes = []
        arr = lambda a, t: np.ascontiguousarray(a, t)
        for (H, q, A, b, Cm, d) in problems:
            n, meq, mineq = int(H.ncol), int(A.nrow), int(Cm.nrow)
            keep = [arr(H.p, np.int32), arr(H.i, np.int32), arr(H.x, np.float64), arr(q, np.float64),
                    arr(A.p, np.int32), arr(A.i, np.int32), arr(A.x, np.float64), arr(b, np.float64),
                    arr(Cm.p, np.int32), arr(Cm.i, np.int32), arr(Cm.x, np.float64), arr(d, np.float64)]
            rc = L.nqg_batch_add(h, n, *[_ptr(a) for a in keep[:4]], meq, *[_ptr(a) for a in keep[4:8]], mineq,
                                 *[_ptr(a) for a in keep[8:]])
            self._raise(rc, "batch add")
            self.sizes.append((n, meq, mineq))
        self._raise(L.nqg_batch_finalize(h), "batch finalize")
        self.n_tot = sum(s[0] for s in self.sizes)
        self.meq_tot = sum(s[1] for s in self.sizes)
        self.mineq_tot = sum(s[2] for s in self.sizes)

    def _raise(self, rc, what):
        if rc < 0:
            msg = lib().nqg_batch_last_error(self._h).decode()
            raise NasoqError(f"{what}: {lib().nqg_status_str(rc).decode()} ({rc}) {msg}")
        return rc

    def __len__(self):
        return len(self.sizes)

    def set_vectors(self, q_all=None, b_all=None, d_all=None):
        """New q / b / d of every problem, concatenated in problem order."""
        conv = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        q_all, b_all, d_all = conv(q_all), conv(b_all), conv(d_all)
        self._raise(lib().nqg_batch_set_vectors(self._h, _ptr(q_all), _ptr(b_all), _ptr(d_all)), "set vectors")

    def set_vectors_async(self, q_all=None, b_all=None, d_all=None):
        """set_vectors enqueued on the batch's stream without waiting.  Arrays
        in page-locked memory (e.g. numpy views of pinned torch tensors) are
        copied asynchronously: keep them unchanged until the stream has passed
        the copies (results() synchronizes it).  The arrays are referenced
        until then."""
        conv = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        q_all, b_all, d_all = conv(q_all), conv(b_all), conv(d_all)
        self._pending = (q_all, b_all, d_all)
        self._raise(lib().nqg_batch_set_vectors_async(self._h, _ptr(q_all), _ptr(b_all), _ptr(d_all)),
                    "set vectors")

    def set_warm_start(self, i, active_set):
        """Proposed active set of problem i (None: cold start)."""
        if active_set is None:
            self._raise(lib().nqg_batch_set_warm_start(self._h, int(i), -1, None), "warm start")
            return
        a = np.ascontiguousarray(active_set, np.int32)
        self._raise(lib().nqg_batch_set_warm_start(self._h, int(i), len(a), _ptr(a)), "warm start")

    def warm_start_from_scores(self, d_scores_ptr, ld, threshold=0.0):
        """Warm-start sets from device-resident scores (one row of ld floats
        per problem, e.g. model logits)."""
        self._raise(lib().nqg_batch_warm_start_from_scores(self._h, C.c_void_p(d_scores_ptr), int(ld),
                                                           float(threshold)), "warm start from scores")

    def clear_warm_starts(self):
        self._raise(lib().nqg_batch_clear_warm_starts(self._h), "clear warm starts")

    def solve(self):
        self._raise(lib().nqg_batch_solve(self._h), "batch solve")

    def solve_async(self):
        self._raise(lib().nqg_batch_solve_async(self._h), "batch solve")

    def stream(self):
        v = C.c_void_p()
        self._raise(lib().nqg_batch_get_stream(self._h, C.byref(v)), "stream")
        return v.value

    def result(self, i):
        n, meq, mineq = self.sizes[i]
        x = np.zeros(n)
        y = np.zeros(max(meq, 1))
        z = np.zeros(max(mineq, 1))
        act = np.zeros(max(mineq, 1), np.int32)
        res = QPResult()
        self._raise(lib().nqg_batch_get(self._h, int(i), _ptr(x), _ptr(y), _ptr(z), _ptr(act), C.byref(res)),
                    "batch get")
        return x, y[:meq], z[:mineq], act[:res.active_size].copy(), res

    def results(self):
        """(x_all, y_all, z_all, stats) for every problem, concatenated."""
        x = np.zeros(max(self.n_tot, 1))
        y = np.zeros(max(self.meq_tot, 1))
        z = np.zeros(max(self.mineq_tot, 1))
        st = (BatchStats * len(self.sizes))()
        self._raise(lib().nqg_batch_get_all(self._h, _ptr(x), _ptr(y), _ptr(z), C.cast(st, C.c_void_p)), "get all")
        return x[:self.n_tot], y[:self.meq_tot], z[:self.mineq_tot], st

    def stats(self):
        """Per-problem statistics only (status, iterations, KKT norms, ...)."""
        st = (BatchStats * len(self.sizes))()
        self._raise(lib().nqg_batch_get_all(self._h, None, None, None, C.cast(st, C.c_void_p)), "get all")
        return st

    PROFILE_PHASES = ("total", "setup", "refactor", "precond", "spmv", "refine", "select", "update",
                      "supernodes", "iterations", "fwd_wide", "fwd_narrow", "diag", "bwd", "gather", "init_factor",
                      "sn_assemble", "sn_updates", "sn_bk", "sn_rows", "sn_inverse", "sn_store", "rename")

    def set_profiling(self, on=True):
        self._raise(lib().nqg_batch_set_profiling(self._h, 1 if on else 0), "set profiling")

    def profile(self):
        """Per-phase SM cycles summed over problems (and counts), then reset."""
        v = (C.c_ulonglong * len(self.PROFILE_PHASES))()
        self._raise(lib().nqg_batch_get_profile(self._h, C.cast(v, C.c_void_p), len(v)), "get profile")
        return dict(zip(self.PROFILE_PHASES, list(v)))

    def info(self) -> BatchInfo:
        i = BatchInfo()
        lib().nqg_batch_get_info(self._h, C.byref(i))
        return i

    def close(self):
        self._pending = None
        if getattr(self, "_h", None):
            lib().nqg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class MLP:
    """Active-set model (nqg_mlp_*): sizes = (inputs, hidden..., outputs),
    ReLU hidden layers, BF16 weights with FP32 master copies, trained on the
    GPU by the library's own kernels."""

    def __init__(self, sizes, seed=0):
        L = lib()
        self.sizes = tuple(int(v) for v in sizes)
        arr = (C.c_int * len(self.sizes))(*self.sizes)
        h = C.c_void_p()
        _check(L.nqg_mlp_create(len(self.sizes), C.cast(arr, C.c_void_p), int(seed), C.byref(h)), "mlp create")
        self._h = h
        nw, nb = C.c_long(), C.c_long()
        L.nqg_mlp_num_params(h, C.byref(nw), C.byref(nb))
        self.n_weights, self.n_biases = nw.value, nb.value

    def _raise(self, rc, what):
        if rc < 0:
            raise NasoqError(f"{what}: {lib().nqg_status_str(rc).decode()} ({rc}) "
                             f"{lib().nqg_mlp_last_error(self._h).decode()}")

    def get_weights(self):
        w = np.zeros(self.n_weights, np.float32)
        b = np.zeros(self.n_biases, np.float32)
        self._raise(lib().nqg_mlp_get_weights(self._h, _ptr(w), _ptr(b)), "get weights")
        return w, b

    def set_weights(self, w, b):
        w = np.ascontiguousarray(w, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        self._raise(lib().nqg_mlp_set_weights(self._h, _ptr(w), _ptr(b)), "set weights")

    def layers(self):
        """[(W (out x in), b)] of the FP32 master weights."""
        w, b = self.get_weights()
        out, ow, ob = [], 0, 0
        for i, o in zip(self.sizes[:-1], self.sizes[1:]):
            out.append((w[ow:ow + i * o].reshape(o, i), b[ob:ob + o]))
            ow += i * o
            ob += o
        return out

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], self.sizes[-1]), np.float32)
        self._raise(lib().nqg_mlp_forward(self._h, x.shape[0], _ptr(x), _ptr(y)), "forward")
        return y

    def forward_device(self, rows, d_x, d_logits, stream=None):
        self._raise(lib().nqg_mlp_forward_device(self._h, int(rows), C.c_void_p(d_x), C.c_void_p(d_logits),
                                                 C.c_void_p(stream) if stream else None), "forward")

    def loss_grad(self, x, y, pos_weight=1.0):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        gw = np.zeros(self.n_weights, np.float32)
        gb = np.zeros(self.n_biases, np.float32)
        loss = C.c_double()
        self._raise(lib().nqg_mlp_loss_grad(self._h, x.shape[0], _ptr(x), _ptr(y), float(pos_weight),
                                            C.byref(loss), _ptr(gw), _ptr(gb)), "loss grad")
        return loss.value, gw, gb

    def fit(self, x, y, epochs=10, batch=1024, lr=1e-3, pos_weight=1.0, seed=0):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        self._raise(lib().nqg_mlp_set_data(self._h, x.shape[0], _ptr(x), _ptr(y)), "set data")
        losses = np.zeros(epochs)
        self._raise(lib().nqg_mlp_train(self._h, int(epochs), int(batch), float(lr), float(pos_weight), int(seed),
                                        _ptr(losses)), "train")
        return losses

    def close(self):
        if getattr(self, "_h", None):
            lib().nqg_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
