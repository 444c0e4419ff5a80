"""Host symbolic analysis against the reference: every array that
symbolic_analysis_lin_solve produces (src/symbolic/symbolic_phase.cpp:167-890)
must match bit for bit on the golden fixtures (LBL mode-0 systems and the QP
super-KKT matrices with their hidden inequality columns)."""
import glob
import os

import numpy as np
import pytest

import nqa
from nasoq_gb300 import Symbolic

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _lbl_cases():
    return sorted(glob.glob(os.path.join(GOLD, "lbl_*.nqa")))


def _qp_cases():
    return sorted(glob.glob(os.path.join(GOLD, "qp_*.nqa")))


def compare(sym, d, pfx="out_sym_"):
    n = len(d[pfx + "Perm"])
    assert np.array_equal(sym.perm, d[pfx + "Perm"]), "ordering differs"
    assert np.array_equal(sym.iperm, d[pfx + "IPerm"])
    assert np.array_equal(sym.parent, d[pfx + "Parent"]), "etree differs"
    assert np.array_equal(sym.colcount, d[pfx + "ColCount"]), "column counts differ"
    assert np.array_equal(sym.super, d[pfx + "super"]), "supernodes differ"
    assert np.array_equal(sym.sparent, d[pfx + "sParent"]), "assembly tree differs"
    assert np.array_equal(sym.col2sup, d[pfx + "col2Sup"])
    ip = d[pfx + "i_ptr"]
    # reference i_ptr is per column: the row-list start of the column's supernode
    assert np.array_equal(sym.lpi[sym.col2sup], ip[:n])
    assert sym.lpi[-1] == ip[n]
    assert np.array_equal(sym.ls, d[pfx + "s"]), "row structure differs"
    assert np.array_equal(sym.colp, d[pfx + "p"]), "value layout differs"
    assert np.array_equal(sym.extra_cols, d[pfx + "extra_cols"])
    assert sym.info.xsize == int(d[pfx + "xsize"][0])
    assert sym.info.max_sup_wid == int(d[pfx + "max_sup_wid"][0])
    assert sym.info.max_col == int(d[pfx + "max_col"][0])


@pytest.mark.parametrize("path", _lbl_cases(), ids=os.path.basename)
def test_symbolic_lbl(path):
    d = nqa.load(path)
    n = len(d["in_rhs"])
    sym = Symbolic(n, d["in_Ap"], d["in_Ai"])
    compare(sym, d)


def super_kkt_pattern(d):
    """Pattern of the QP super-KKT [H; A; C] that build_super_matrix forms
    (src/QP/linear_solver_wrapper.cpp:246-350) and its hidden-column flags."""
    from kkt_util import super_kkt
    K, extra, _ = super_kkt(d["in_Hp"], d["in_Hi"], d["in_Hx"], d["in_Ap"], d["in_Ai"], d["in_Ax"],
                            d["in_Cp"], d["in_Ci"], d["in_Cx"], int(d["in_meq"][0]), int(d["in_mineq"][0]))
    return K, extra


@pytest.mark.parametrize("path", _qp_cases(), ids=os.path.basename)
def test_symbolic_qp_superkkt(path):
    d = nqa.load(path)
    K, extra = super_kkt_pattern(d)
    sym = Symbolic(K.ncol, K.p, K.i, extra_cols=extra)
    compare(sym, d)
