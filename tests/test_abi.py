"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares; host-only calls work without a device."""
import ctypes
import glob
import os
import re

import numpy as np

import nasoq_gb300 as nq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(nqg_\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_exports_every_declared_symbol():
    lib = ctypes.CDLL(nq.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_default_settings_match_reference():
    s = nq.default_settings()
    # src/QP/linear_solver_wrapper.cpp:205-244
    assert s.req_ref_iter == 2 and s.max_inner_iter == 2
    assert s.tol_abs == 1e-15 and s.tol_rel == 1e-15
    assert s.reg_diag == 1e-8 and s.regularization == 1
    assert list(s.n_relax) == [4, 16, 48]
    assert list(s.z_relax) == [0.8, 0.1, 0.05]


def test_status_strings():
    L = nq.lib()
    for code in (0, 1, 2, -1, -2, -3, -4, -5, -6):
        assert len(L.nqg_status_str(code)) > 0


def test_invalid_arguments_rejected():
    L = nq.lib()
    h = ctypes.c_void_p()
    Ap = np.array([0, 2, 3], np.int32)
    Ai = np.array([0, 1, 1], np.int32)
    bad = np.array([0, 1, 2], np.int32)
    bad_i = np.array([0, 0], np.int32)  # column 1 holds row 0: not lower-stored
    assert L.nqg_symbolic_create(2, bad, bad_i, None, None, None, ctypes.byref(h)) == -1
    nodiag_i = np.array([1, 1], np.int32)  # column 0 has no diagonal entry
    assert L.nqg_symbolic_create(2, bad, nodiag_i, None, None, None, ctypes.byref(h)) == -1
    rc = L.nqg_symbolic_create(2, Ap, Ai, None, None, None, ctypes.byref(h))
    assert rc == 0
    L.nqg_symbolic_destroy(h)


def test_build_tracks_included_units_and_headers():
    """The incremental build recompiles an object when a header (.h, .hpp,
    .cuh) or a .cu file it includes changes: batch_fp64.cu compiles batch.cu
    again for the FP64 instantiation."""
    from nasoq_gb300 import build
    csrc = os.path.join(ROOT, "nasoq_gb300", "csrc")
    deps = {os.path.basename(d) for d in build._deps(os.path.join(csrc, "batch_fp64.cu"))}
    assert {"batch_fp64.cu", "batch.cu", "batch.hpp", "bk.cuh", "tcgen05.cuh", "nasoq_gb300.h"} <= deps
    srcs = {os.path.basename(s) for s in build.sources()}
    assert {"batch.cu", "batch_fp64.cu"} <= srcs
