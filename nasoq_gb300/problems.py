"""Seeded synthetic problem generators for the workloads this library is
measured on (numpy only, no GPU).

Conventions follow the reference's inputs (include/nasoq/common/def.h:73-122):
symmetric matrices are lower-stored CSC with sorted rows and the diagonal
entry first in every column; constraint matrices are m-by-n CSC (columns are
variables), as `Nasoq(n, Hp, Hi, Hx, q, A..., C...)` takes them
(include/nasoq/nasoq.h:129-133).

All generators draw from ``numpy.random.default_rng(seed)``; the public
benchmark suites the reference was evaluated on are not available, so these
seeded stand-ins reproduce the shapes, sparsity and value distributions of the
workloads named by the benchmark definitions instead.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class CSC:
    """Compressed sparse column matrix (0-based, int32 indices, float64 values)."""

    nrow: int
    ncol: int
    p: np.ndarray
    i: np.ndarray
    x: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.p[-1])

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.nrow, self.ncol))
        for j in range(self.ncol):
            for k in range(self.p[j], self.p[j + 1]):
                d[self.i[k], j] += self.x[k]
        return d


def _from_cols(nrow, ncol, cols):
    """cols: list of (rows, vals) per column; rows are sorted here."""
    p = np.zeros(ncol + 1, dtype=np.int32)
    ii, xx = [], []
    for j, (r, v) in enumerate(cols):
        r = np.asarray(r, dtype=np.int64)
        v = np.asarray(v, dtype=np.float64)
        o = np.argsort(r, kind="stable")
        ii.append(r[o])
        xx.append(v[o])
        p[j + 1] = p[j] + len(r)
    i = np.concatenate(ii).astype(np.int32) if ii else np.zeros(0, np.int32)
    x = np.concatenate(xx) if xx else np.zeros(0)
    return CSC(nrow, ncol, p, i, x)


def csc_from_coo(nrow, ncol, rows, cols, vals):
    """Builds a CSC from triplets (duplicates are summed, rows sorted)."""
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    key = cols * nrow + rows
    order = np.argsort(key, kind="stable")
    key, vals = key[order], vals[order]
    uk, start = np.unique(key, return_index=True)
    sums = np.add.reduceat(vals, start) if len(vals) else vals
    c = uk // nrow
    r = uk % nrow
    p = np.zeros(ncol + 1, dtype=np.int64)
    np.add.at(p, c + 1, 1)
    p = np.cumsum(p).astype(np.int32)
    return CSC(nrow, ncol, p, r.astype(np.int32), sums.astype(np.float64))


def lower_of(full: CSC) -> CSC:
    """Lower triangle (diagonal included) of a square CSC, diagonal first."""
    rows, cols, vals = [], [], []
    for j in range(full.ncol):
        for k in range(full.p[j], full.p[j + 1]):
            if full.i[k] >= j:
                rows.append(full.i[k])
                cols.append(j)
                vals.append(full.x[k])
    return csc_from_coo(full.nrow, full.ncol, rows, cols, vals)


def laplacian2d(k: int, shift: float = 0.0) -> CSC:
    """5-point Laplacian on a k-by-k grid (diagonal 4, off-diagonals -1) plus
    shift*I, lower-stored."""
    n = k * k
    rows, cols, vals = [], [], []
    for y in range(k):
        for x in range(k):
            v = y * k + x
            rows.append(v); cols.append(v); vals.append(4.0 + shift)
            if x + 1 < k:
                rows.append(v + 1); cols.append(v); vals.append(-1.0)
            if y + 1 < k:
                rows.append(v + k); cols.append(v); vals.append(-1.0)
    return csc_from_coo(n, n, rows, cols, vals)


def laplacian3d(k: int, shift: float = 0.0) -> CSC:
    """7-point Laplacian on a k^3 grid (diagonal 6), lower-stored."""
    n = k ** 3
    idx = np.arange(n).reshape(k, k, k)
    rows = [idx.ravel()]
    cols = [idx.ravel()]
    vals = [np.full(n, 6.0 + shift)]
    for ax in range(3):
        a = np.moveaxis(idx, ax, 0)
        lo = a[:-1].ravel()
        hi = a[1:].ravel()
        rows.append(hi); cols.append(lo); vals.append(np.full(lo.size, -1.0))
    return csc_from_coo(n, n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def random_rows(m: int, n: int, per_row: int, rng) -> CSC:
    """m-by-n matrix with `per_row` distinct uniform-random columns in every
    row and N(0,1) values."""
    rows = np.repeat(np.arange(m), per_row)
    cols = np.empty(m * per_row, dtype=np.int64)
    for r in range(m):
        cols[r * per_row:(r + 1) * per_row] = rng.choice(n, size=per_row, replace=False)
    vals = rng.standard_normal(m * per_row)
    return csc_from_coo(m, n, rows, cols, vals)


def kkt_lower(H: CSC, A: CSC, delta: float) -> CSC:
    """K = [H A^T; A -delta*I], lower-stored: columns 0..n-1 hold H's lower
    part and A's column, columns n..n+m-1 the -delta diagonal."""
    n, m = H.ncol, A.nrow
    rows, cols, vals = [], [], []
    for j in range(n):
        for k in range(H.p[j], H.p[j + 1]):
            rows.append(H.i[k]); cols.append(j); vals.append(H.x[k])
        for k in range(A.p[j], A.p[j + 1]):
            rows.append(n + A.i[k]); cols.append(j); vals.append(A.x[k])
    for r in range(m):
        rows.append(n + r); cols.append(n + r); vals.append(-delta)
    return csc_from_coo(n + m, n + m, rows, cols, vals)


def kkt_lower_fast(H: CSC, A: CSC, delta: float) -> CSC:
    """Vectorised kkt_lower for large systems."""
    n, m = H.ncol, A.nrow
    hc = np.repeat(np.arange(n), np.diff(H.p))
    ac = np.repeat(np.arange(n), np.diff(A.p))
    rows = np.concatenate([H.i.astype(np.int64), n + A.i.astype(np.int64), n + np.arange(m)])
    cols = np.concatenate([hc, ac, n + np.arange(m)])
    vals = np.concatenate([H.x, A.x, np.full(m, -delta)])
    return csc_from_coo(n + m, n + m, rows, cols, vals)


@dataclass
class QP:
    """min 1/2 x'Hx + q'x  s.t.  A x = b,  C x <= d   (H lower-stored)."""

    H: CSC
    q: np.ndarray
    A: CSC
    b: np.ndarray
    C: CSC
    d: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n(self):
        return self.H.ncol


def empty_rows(n: int) -> CSC:
    return CSC(0, n, np.zeros(n + 1, np.int32), np.zeros(0, np.int32), np.zeros(0))


def qp_random_convex(seed: int = 0, grid: int = 45, meq: int = 200, mineq: int = 1000,
                     eq_per_row: int = 5, ineq_per_row: int = 4) -> QP:
    """Random convex QP: H = 2D 5-point Laplacian on grid x grid + 1e-3 I,
    q ~ N(0,1); A (meq x n, eq_per_row nnz/row, N(0,1)), b = A x0 with
    x0 ~ U(-1,1); C (mineq x n, ineq_per_row nnz/row, N(0,1)),
    d = C x0 + U(0, 0.5).  grid=45, meq=200, mineq=1000 is the n=2025
    single-QP workload."""
    rng = np.random.default_rng(seed)
    H = laplacian2d(grid, 1e-3)
    n = H.ncol
    q = rng.standard_normal(n)
    x0 = rng.uniform(-1.0, 1.0, n)
    A = random_rows(meq, n, eq_per_row, rng) if meq > 0 else empty_rows(n)
    b = _matvec(A, x0)
    C = random_rows(mineq, n, ineq_per_row, rng)
    d = _matvec(C, x0) + rng.uniform(0.0, 0.5, mineq)
    return QP(H, q, A, b, C, d, {"kind": "random_convex", "seed": seed})


def _scale_csc(M: CSC, row: np.ndarray | None, col: np.ndarray | None) -> CSC:
    x = np.array(M.x, np.float64)
    cols = np.repeat(np.arange(M.ncol), np.diff(M.p))
    if row is not None:
        x *= row[M.i]
    if col is not None:
        x *= col[cols]
    return CSC(M.nrow, M.ncol, M.p, M.i, x)


def qp_ill_scaled(seed: int = 0, grid: int = 12, meq: int = 20, mineq: int = 120, spread: float = 3.0) -> QP:
    """qp_random_convex with its variables and rows rescaled by factors
    10^U(-spread, spread): x = S x', H' = S H S, q' = S q, A' = E A S,
    C' = F C S, b' = E b, d' = F d.  The same optimum (through S) with data
    spanning about 10^(4 spread) in magnitude: the case Ruiz equilibration is
    for."""
    base = qp_random_convex(seed, grid=grid, meq=meq, mineq=mineq)
    rng = np.random.default_rng(seed + 1000)
    n = base.H.ncol
    sv = 10.0 ** rng.uniform(-spread, spread, n)
    se = 10.0 ** rng.uniform(-spread, spread, base.A.nrow)
    sf = 10.0 ** rng.uniform(-spread, spread, base.C.nrow)
    H = _scale_csc(base.H, sv, sv)
    A = _scale_csc(base.A, se, sv)
    C = _scale_csc(base.C, sf, sv)
    return QP(H, base.q * sv, A, base.b * se, C, base.d * sf,
              {"kind": "ill_scaled", "seed": seed, "spread": spread})


def bilaplacian_bounded(seed: int = 0, grid: int = 400, pins: int = 2000, jitter: float = 0.2) -> QP:
    """Large bounded QP of biharmonic-weights type on a grid x grid mesh.

    Vertices sit at (i h, j h) moved by U(-jitter, jitter) h in each
    coordinate.  L is the 5-point Laplacian of the moved vertices with
    dimensionless weights h^2 / |p_a - p_b|^2 between grid neighbours (row
    sums on the diagonal, about 4 on the unjittered grid), M the lumped
    vertex areas (products of the half spacings), and H = L M^-1 L, a
    13-point bilaplacian (lower-stored).  q = 0.  `pins` random vertices
    are fixed to values in {0, 1} (equality rows), and 0 <= x <= 1 on every
    vertex becomes two inequality rows per vertex, x_i <= 1 then -x_i <= 0
    (the bounds-to-rows rule of the SMP converter): n = grid^2 variables,
    `pins` equalities, 2 n inequalities."""
    rng = np.random.default_rng(seed)
    g = grid
    n = g * g
    h = 1.0 / (g - 1)
    jx = rng.uniform(-jitter, jitter, (g, g)) * h
    jy = rng.uniform(-jitter, jitter, (g, g)) * h
    X = np.arange(g)[:, None] * h + jx  # X[i, j]: vertex (i, j), index i * g + j
    Y = np.arange(g)[None, :] * h + jy
    idx = np.arange(n).reshape(g, g)
    rows, cols, w = [], [], []
    for di, dj in ((1, 0), (0, 1)):
        a = idx[:g - di, :g - dj].ravel()
        b = idx[di:, dj:].ravel()
        dx = X.ravel()[b] - X.ravel()[a]
        dy = Y.ravel()[b] - Y.ravel()[a]
        rows.append(a)
        cols.append(b)
        w.append(h * h / (dx * dx + dy * dy))
    a = np.concatenate(rows)
    b = np.concatenate(cols)
    w = np.concatenate(w)
    diag = np.zeros(n)
    np.add.at(diag, a, w)
    np.add.at(diag, b, w)
    import scipy.sparse as sp
    Lm = sp.coo_matrix((np.concatenate([-w, -w, diag]), (np.concatenate([a, b, np.arange(n)]),
                                                          np.concatenate([b, a, np.arange(n)]))), shape=(n, n)).tocsr()
    # lumped areas: half the spacing to each neighbour in both directions
    Xr = X.ravel()
    Yr = Y.ravel()
    ii, jj = np.divmod(np.arange(n), g)
    up = np.where(ii < g - 1, Xr[np.minimum(idx.ravel() + g, n - 1)] - Xr, 0.0)
    dn = np.where(ii > 0, Xr - Xr[np.maximum(idx.ravel() - g, 0)], 0.0)
    rt = np.where(jj < g - 1, Yr[np.minimum(idx.ravel() + 1, n - 1)] - Yr, 0.0)
    lf = np.where(jj > 0, Yr - Yr[np.maximum(idx.ravel() - 1, 0)], 0.0)
    area = 0.25 * (up + dn) * (rt + lf)
    Hm = (Lm @ sp.diags(1.0 / area) @ Lm).tocsc()
    Hl = sp.tril(Hm).tocsc()
    Hl.sort_indices()
    H = CSC(n, n, Hl.indptr.astype(np.int32), Hl.indices.astype(np.int32), Hl.data.astype(np.float64))
    pin = np.sort(rng.choice(n, size=pins, replace=False))
    vals = rng.integers(0, 2, size=pins).astype(np.float64)
    A = csc_from_coo(pins, n, np.arange(pins), pin, np.ones(pins))
    r = np.arange(2 * n)
    C = csc_from_coo(2 * n, n, r, r // 2, np.where(r % 2 == 0, 1.0, -1.0))
    d = np.where(r % 2 == 0, 1.0, 0.0)
    return QP(H, np.zeros(n), A, vals, C, d, {"kind": "bilaplacian_bounded", "seed": seed, "grid": grid,
                                              "pins": pins, "jitter": jitter})


def _matvec(M: CSC, x: np.ndarray) -> np.ndarray:
    y = np.zeros(M.nrow)
    cols = np.repeat(np.arange(M.ncol), np.diff(M.p))
    np.add.at(y, M.i, M.x * x[cols])
    return y


def lbl_kkt(seed: int = 0, grid3d: int = 64, m: int = 20000, per_row: int = 6, delta: float = 1e-8):
    """Symmetric-indefinite KKT system K = [H A^T; A -delta I] with H the 3D
    7-point Laplacian on grid3d^3 and A (m x n) with per_row random columns per
    row, N(0,1) values; rhs ~ N(0,1).  grid3d=64, m=20000 is the n=262144
    (N=282144) LBL workload."""
    rng = np.random.default_rng(seed)
    H = laplacian3d(grid3d)
    A = random_rows_fast(m, H.ncol, per_row, rng)
    K = kkt_lower_fast(H, A, delta)
    rhs = rng.standard_normal(K.ncol)
    return K, rhs


def random_rows_fast(m: int, n: int, per_row: int, rng) -> CSC:
    """Vectorised random_rows (distinct columns per row via rejection)."""
    cols = rng.integers(0, n, size=(m, per_row))
    for _ in range(64):
        s = np.sort(cols, axis=1)
        dup = np.any(s[:, 1:] == s[:, :-1], axis=1)
        if not dup.any():
            break
        cols[dup] = rng.integers(0, n, size=(int(dup.sum()), per_row))
    rows = np.repeat(np.arange(m), per_row)
    vals = rng.standard_normal(m * per_row)
    return csc_from_coo(m, n, rows, cols.ravel(), vals)


def qp_mpc(seed: int, horizon: int, nx: int = 6, nu: int = 3, q_scale: float = 10.0) -> QP:
    """MPC-structured QP over `horizon` steps: variables (x_1..x_N, u_0..u_{N-1}),
    n = (nx+nu)*N.  H = blkdiag(Q, R) with Q, R diagonal U(0.1, 10); dynamics
    x_{k+1} = A_k x_k + B_k u_k (A_k, B_k entries N(0, 0.3), x_0 given) are
    nx*N equality rows; box bounds |u| <= 1, |x| <= 5 become two inequality
    rows each (18N rows for nx=6, nu=3)."""
    rng = np.random.default_rng(seed)
    N = horizon
    nxs, nus = nx * N, nu * N
    n = nxs + nus
    diag = np.concatenate([rng.uniform(0.1, 10.0, nxs), rng.uniform(0.1, 10.0, nus)])
    H = csc_from_coo(n, n, np.arange(n), np.arange(n), diag)
    q = q_scale * rng.standard_normal(n)
    x0 = rng.standard_normal(nx)
    rows, cols, vals = [], [], []
    b = np.zeros(nxs)
    for k in range(N):
        Ak = rng.normal(0.0, 0.3, (nx, nx))
        Bk = rng.normal(0.0, 0.3, (nx, nu))
        for r in range(nx):
            row = k * nx + r
            rows.append(row); cols.append(k * nx + r); vals.append(1.0)  # x_{k+1}
            if k > 0:
                for c in range(nx):
                    rows.append(row); cols.append((k - 1) * nx + c); vals.append(-Ak[r, c])
            else:
                b[row] = Ak[r] @ x0
            for c in range(nu):
                rows.append(row); cols.append(nxs + k * nu + c); vals.append(-Bk[r, c])
    A = csc_from_coo(nxs, n, rows, cols, vals)
    crow, ccol, cval, d = [], [], [], []
    r = 0
    for v in range(n):
        bound = 5.0 if v < nxs else 1.0
        crow += [r, r + 1]; ccol += [v, v]; cval += [1.0, -1.0]
        d += [bound, bound]
        r += 2
    C = csc_from_coo(r, n, crow, ccol, cval)
    return QP(H, q, A, b, C, np.asarray(d), {"kind": "mpc", "seed": seed, "horizon": N})


def sym_indefinite(seed: int, n: int, density: float, zero_diag: bool = True) -> CSC:
    """Random sparse symmetric indefinite matrix (lower-stored), N(0,1)
    off-diagonals, zero (or N(0,1)) diagonal entries stored explicitly so that
    Bunch-Kaufman must take 2x2 pivots."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for j in range(n):
        rows.append(j); cols.append(j); vals.append(0.0 if zero_diag else rng.standard_normal())
        for i in range(j + 1, n):
            if rng.random() < density:
                rows.append(i); cols.append(j); vals.append(rng.standard_normal())
    return csc_from_coo(n, n, rows, cols, vals)


def mpc_batch_specs(count: int, seed: int = 0, horizons=(10, 100)):
    """(seed, horizon) of each problem of an uneven MPC batch: horizons drawn
    uniformly from [horizons[0], horizons[1]], problem seeds seed*100003+i.
    count=4096 with horizons (10, 100) is the batched MPC workload."""
    rng = np.random.default_rng(seed)
    hz = rng.integers(horizons[0], horizons[1] + 1, size=count)
    return [(seed * 100003 + i, int(hz[i])) for i in range(count)]


def mpc_batch(count: int, seed: int = 0, horizons=(10, 100)):
    """The QPs of mpc_batch_specs (see qp_mpc)."""
    return [qp_mpc(s, h) for s, h in mpc_batch_specs(count, seed, horizons)]


@dataclass
class ParametricQP:
    """min 1/2 x'Hx + (P theta)'x  s.t.  A x = b,  C x <= d0 + S theta."""

    base: QP
    P: np.ndarray   # n x p
    d0: np.ndarray  # mineq
    S: np.ndarray   # mineq x p

    def q_of(self, theta):
        return self.P @ theta

    def d_of(self, theta):
        return self.d0 + self.S @ theta


def mpc_parametric(seed: int = 0, horizon: int = 50, p: int = 32, scale: float = 0.1) -> ParametricQP:
    """Parametric QP family on the MPC structure (qp_mpc at the given horizon;
    horizon 50: n = 450, 300 equalities, 900 inequalities): q = P theta and
    d = d0 + S theta, theta in R^p ~ N(0, I), P dense N(0, scale) (standard
    deviation `scale`).  S moves each variable's box as a whole: a dense
    N(0, scale) shift s_v = (G theta)_v enters the two rows of the box of
    variable v with opposite signs (x_v <= ub + s_v, -x_v <= ub - s_v), so the
    box [-ub + s_v, ub + s_v] is never empty; independent perturbations of the
    two rows would make some instances infeasible."""
    base = qp_mpc(seed, horizon)
    rng = np.random.default_rng(seed + 7919)
    n = base.n
    P = rng.normal(0.0, scale, (n, p))
    G = rng.normal(0.0, scale, (n, p))
    S = np.empty((base.C.nrow, p))
    S[0::2] = G
    S[1::2] = -G
    return ParametricQP(base, P, base.d.copy(), S)


def qp_checksum(qp: QP) -> float:
    """Sum of |entries| of every input array: detects a change of a generator."""
    return float(sum(np.abs(np.asarray(a, np.float64)).sum()
                     for a in (qp.H.x, qp.q, qp.A.x, qp.b, qp.C.x, qp.d)))
