"""The allocation-free dense Bunch-Kaufman entry point (nqg_dense_ldlt_noalloc)
for callers that cannot allocate GPU memory while running, checked through
the C ABI against the regular plan-based factorization of the same dense
symmetric-indefinite matrix, on two calls in a row (the shared scratch keeps
the previous call's contents, so the second call must not be affected by
them).  Same tolerance style as the other factorization parity tests: the
two paths run the same kernels, so the factor, D and pivots must agree to
1e-12 relative to the largest entry, and the factor's backward error must be
below 1e-13.  A second test factors tall panels (rows below the diagonal
block) of two different matrices in a row, checks them by their defining
equations, and checks that a call leaves the device's free memory unchanged."""
import ctypes

import numpy as np
import pytest

import nasoq_gb300 as nq
from nasoq_gb300.problems import csc_from_coo


def _dense_sym(n, seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n))
    K = np.tril(M) + np.tril(M, -1).T
    np.fill_diagonal(K, rng.standard_normal(n) * 0.1)  # small diagonal: BK takes interchanges and 2x2 pivots
    return K


def _lower_csc(K):
    n = K.shape[0]
    r, c = np.tril_indices(n)
    return csc_from_coo(n, n, r, c, K[r, c])


@pytest.mark.gpu
def test_noalloc_matches_plan_factor_twice():
    torch = pytest.importorskip("torch")
    L = nq.lib()
    L.nqg_dense_ldlt_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    n = 300
    K = _dense_sym(n, seed=12)
    A = _lower_csc(K)
    plan = nq.Plan(n, A.p, A.i, A.x, settings=nq.default_settings(req_ref_iter=0, reg_diag=1e-9))
    sym = plan.symbolic
    assert sym.info.nsuper == 1 and sym.info.max_sup_wid == n  # one dense supernode: the wide kernels
    assert plan.factor() == 0
    vals, dv, perm_comb, _ = plan.factor_arrays()
    Lref = vals.reshape(n, n).T  # column-major n x n
    Kp = K[np.ix_(sym.perm, sym.perm)]
    scale = np.abs(Lref).max()
    for call in range(2):
        dA = torch.from_numpy(np.ascontiguousarray(Kp.T)).cuda()  # column-major copy
        dD = torch.full((2 * n,), 7.0, dtype=torch.float64, device="cuda")
        dP = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        rc = L.nqg_dense_ldlt_noalloc(n, n, dA.data_ptr(), n, dD.data_ptr(), dP.data_ptr(), None)
        assert rc == 0, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        Lna = dA.cpu().numpy().T
        Dna = dD.cpu().numpy()
        Pna = dP.cpu().numpy()
        assert np.array_equal(sym.perm[Pna], perm_comb), f"call {call}: pivot order differs"
        assert np.abs(Lna - Lref).max() <= 1e-12 * scale, f"call {call}: factor differs"
        assert np.abs(Dna - dv).max() <= 1e-12 * np.abs(dv).max(), f"call {call}: D differs"
        # backward error: P A P^T = L D L^T with the local pivot order
        Lu = np.tril(Lna, -1) + np.eye(n)
        Dm = np.diag(Dna[:n]) + np.diag(Dna[n:2 * n - 1], -1) + np.diag(Dna[n:2 * n - 1], 1)
        Kq = Kp[np.ix_(Pna, Pna)]
        R = Kq - Lu @ Dm @ Lu.T
        mag = np.abs(Lu) @ np.abs(Dm) @ np.abs(Lu).T
        assert np.abs(R).max() <= 1e-13 * mag.max()
    plan.close()


def _check_panel(Pn, Ln, Dn, Pm, w):
    """Pn: the nrow x w input panel (diagonal block on top), Ln/Dn/Pm: the
    call's outputs.  P A11 P^T = L11 D L11^T and L21 = A21[:, P] L11^-T D^-1."""
    nrow = Pn.shape[0]
    Lu = np.tril(Ln[:w, :w], -1) + np.eye(w)
    Dm = np.diag(Dn[:w]) + np.diag(Dn[w:2 * w - 1], -1) + np.diag(Dn[w:2 * w - 1], 1)
    A11 = np.tril(Pn[:w, :w]) + np.tril(Pn[:w, :w], -1).T
    Aq = A11[np.ix_(Pm, Pm)]
    R = Aq - Lu @ Dm @ Lu.T
    mag = np.abs(Lu) @ np.abs(Dm) @ np.abs(Lu).T
    assert np.abs(R).max() <= 1e-13 * mag.max()
    if nrow > w:
        A21 = Pn[w:, :][:, Pm]
        L21 = Ln[w:, :]
        # L21 D L11^T must reproduce the permuted rows below
        R2 = A21 - L21 @ Dm @ Lu.T
        mag2 = np.abs(L21) @ np.abs(Dm) @ np.abs(Lu).T
        assert np.abs(R2).max() <= 1e-12 * max(mag2.max(), np.abs(A21).max())


@pytest.mark.gpu
def test_noalloc_tall_panels_differ_and_allocate_nothing():
    torch = pytest.importorskip("torch")
    L = nq.lib()
    L.nqg_dense_ldlt_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    nrow, w = 300, 200
    for call, seed in enumerate((21, 22)):  # two different matrices in a row
        K = _dense_sym(nrow, seed)
        Pn = K[:, :w].copy()  # w x w symmetric block on top of nrow - w rows
        dA = torch.from_numpy(np.ascontiguousarray(Pn.T)).cuda()
        dD = torch.full((2 * w,), 7.0, dtype=torch.float64, device="cuda")
        dP = torch.full((w,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = L.nqg_dense_ldlt_noalloc(nrow, w, dA.data_ptr(), nrow, dD.data_ptr(), dP.data_ptr(), None)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert rc == 0, f"call {call}: status {rc}"
        if call > 0:  # the first call on the device may load the module
            assert free1 == free0, f"call {call}: free device memory changed by {free0 - free1} bytes"
        Pm = dP.cpu().numpy()
        assert sorted(Pm.tolist()) == list(range(w))
        _check_panel(Pn, dA.cpu().numpy().T, dD.cpu().numpy(), Pm, w)


@pytest.mark.gpu
def test_noalloc_rejects_oversize():
    L = nq.lib()
    L.nqg_dense_ldlt_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]
    # beyond the 8192-row capacity of the fixed scratch: refused before any device work
    dummy = ctypes.c_void_p(16)
    assert L.nqg_dense_ldlt_noalloc(8193, 16, dummy, 8193, dummy, dummy, None) == -6
