"""CPU oracle for GaDE's Crank-Nicolson step — TEST INFRASTRUCTURE ONLY.

A numpy/scipy restatement of the reference CPU build of ``dirac_solver``
(tools/ built with USE_MPI, one rank).  It is the checker for the GB300
product path: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it.  The product never routes
through this module.

Parity pin: this restatement is checked against the reference C sources
themselves, compiled in place with single-rank MPI/BLAS/SuperLU shims by
``oracle/build_ref.py`` (outputs in ``oracle/_ref/``), on generated inputs;
the comparison outputs are committed under ``tests/golden/``.

Functions follow, line by line:
  * f(t) pulse factors      tools/solver_common.c:53-65
  * kappa of an index       tools/solver_common.c:30-37
  * set-up                  tools/dirac_solver.c:223-431
  * unblocked CSR + map     tools/csr.c:653-743
  * stationary matrices     tools/solver.c:409-458
  * preconditioner (ILU)    tools/solver.c:460-485, tools/superlu.c:154-266
  * time-dependent matrix   tools/solver.c:196-407
  * rhs and operator        tools/dirac_solver.c:115-131, 553-562
  * BiCGSTAB                tools/bicgstab.c:125-295
  * time loop               tools/dirac_solver.c:496-636
"""
from __future__ import annotations

import dataclasses
import math
import os
import sys
import time as _time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))
from dirac_hydrogen_code_gb300.formats import csr_read, vec_read  # noqa: E402

SOL = 137.035999084


def ik(i: int) -> int:
    """tools/solver_common.c:30-37."""
    ii = i // 4
    abskappa = int(0.5 * (math.sqrt(8.0 * ii + 1.0) - 1.0)) + 1
    sgnmod = max(4, abskappa * 4)
    sgnfloor = 2.0 * abskappa * (abskappa - 1)
    q = (i - sgnfloor) / sgnmod
    return abskappa * ((q >= 0.5) - (q < 0.5))


def pulse(E0: float, omega: float, cycles: float, t: float) -> np.ndarray:
    """beoyndDipolePulse_axialPart, tools/solver_common.c:53-65 (phi=-pi/2)."""
    T = cycles * 2 * math.pi / omega
    phi = -math.pi / 2
    a = E0 / (4 * omega)
    b = E0 / (2 * omega)
    return np.array([
        -a * math.cos(phi + t * (2 * math.pi / T + omega)),
        -a * math.sin(phi + t * (2 * math.pi / T + omega)),
        -a * math.cos(-phi + t * (2 * math.pi / T - omega)),
        a * math.sin(-phi + t * (2 * math.pi / T - omega)),
        b * math.cos(phi + t * omega),
        b * math.sin(phi + t * omega),
    ], dtype=complex)


@dataclasses.dataclass
class Problem:
    lmax: int
    nblk: int
    blkdim: int
    blk_nnz: int
    Hall: sp.csr_matrix            # block pattern (compact numbering)
    perm: np.ndarray               # compact -> original angular index
    kappa: np.ndarray              # kappa of each compact block row
    H0: np.ndarray                 # (nnz(Hall), lmax) angular couplings
    H1: np.ndarray
    g: np.ndarray                  # (6, lmax, 4, blk_nnz)
    gt: np.ndarray                 # conjugate transposes on the same pattern
    h0: np.ndarray                 # (4, blk_nnz)
    s0: np.ndarray                 # (3, blk_nnz)
    sub_Ap: np.ndarray             # base pattern
    sub_Ai: np.ndarray
    psi0: np.ndarray
    xperm: np.ndarray
    # unblocked structure
    A_indptr: np.ndarray = None
    A_indices: np.ndarray = None
    sub_map: np.ndarray = None     # (nnz(Hall), blk_nnz) -> position in A
    sub_inv: np.ndarray = None     # position in A -> flat index into (nnz(Hall), blk_nnz)
    S_indptr: np.ndarray = None
    S_indices: np.ndarray = None
    S_map: np.ndarray = None       # (nblk, blk_nnz)

    @property
    def n(self) -> int:
        return self.nblk * self.blkdim


def _conj_transpose_on_pattern(Ap, Ai, Ax):
    """csr_conj_transpose (tools/csr.c:963-972): gt(c, r) = conj(g(r, c)),
    stored on the (symmetric) pattern of g."""
    n = len(Ap) - 1
    rows = np.repeat(np.arange(n), np.diff(Ap))
    # position of (c, r) in the pattern
    key = rows.astype(np.int64) * n + Ai
    order = np.argsort(key)
    tkey = Ai.astype(np.int64) * n + rows
    pos = np.searchsorted(key[order], tkey)
    if np.any(pos >= len(key)) or np.any(key[order][np.minimum(pos, len(key) - 1)] != tkey):
        raise ValueError("cant set matrix value: pattern is not symmetric")
    dst = order[pos]
    out = np.zeros_like(Ax)
    out[dst] = np.conj(Ax)
    return out


def load_problem(workdir: str, lmax: int, unblock: bool = True) -> Problem:
    """Reads every input like tools/dirac_solver.c:223-388.  unblock=False
    skips the unblocked CSR of the whole operator (tools/csr.c:653-743),
    which only ``timedep``/``stationary``/``run`` need; ``apply_block_rows``
    works without it."""
    j = lambda f: os.path.join(workdir, f)
    Hall = csr_read(j("H.csr"))
    if Hall.perm is None:
        raise ValueError("H.csr has no permutation trailer")
    nblk = Hall.n
    H = []
    for l in range(lmax):
        H.append((csr_read(j(f"H0l{l}.csr")).to_scipy(), csr_read(j(f"H1l{l}.csr")).to_scipy()))
    g0 = csr_read(j("g0a0l0.csr"))
    blkdim, blk_nnz = g0.n, g0.nnz
    g = np.zeros((6, lmax, 4, blk_nnz), complex)
    gt = np.zeros_like(g)
    for a in range(6):
        for l in range(lmax):
            for gi in range(4):
                m = csr_read(j(f"g{gi}a{a}l{l}.csr"))
                if m.nnz != blk_nnz:
                    raise ValueError("g matrices must share the base pattern")
                g[a, l, gi] = m.Ax
                gt[a, l, gi] = _conj_transpose_on_pattern(m.Ap, m.Ai, m.Ax)
    h0 = np.stack([csr_read(j(f"h0{i}.csr")).Ax for i in range(4)])
    s0 = np.stack([csr_read(j(f"s{i}.csr")).Ax for i in range(3)])
    psi, xperm = vec_read(j("psi0.vec"))
    perm = Hall.perm
    kappa = np.array([ik(int(p)) for p in perm], np.int64)
    hall = Hall.to_scipy()
    rows = np.repeat(np.arange(nblk), np.diff(Hall.Ap))
    orig_r, orig_c = perm[rows], perm[Hall.Ai]
    H0 = np.zeros((Hall.nnz, lmax), complex)
    H1 = np.zeros((Hall.nnz, lmax), complex)
    for l in range(lmax):
        H0[:, l] = np.asarray(H[l][0][orig_r, orig_c]).ravel()
        H1[:, l] = np.asarray(H[l][1][orig_r, orig_c]).ravel()
    p = Problem(lmax, nblk, blkdim, blk_nnz, hall, perm, kappa, H0, H1, g, gt, h0, s0,
                g0.Ap, g0.Ai, psi, xperm)
    if unblock:
        _unblock(p)
    return p


def _unblock(p: Problem) -> None:
    """csr_unblock_matrix (tools/csr.c:653-743) for Hfull and S."""
    Ap, Ai = p.Hall.indptr, p.Hall.indices
    bd, sAp, sAi = p.blkdim, p.sub_Ap, p.sub_Ai
    srow_nnz = np.diff(sAp)
    # row r*bd+rb has sum over blocks in row r of srow_nnz[rb] entries
    blk_per_row = np.diff(Ap)
    row_len = (blk_per_row[:, None] * srow_nnz[None, :]).ravel()
    indptr = np.zeros(p.nblk * bd + 1, np.int64)
    np.cumsum(row_len, out=indptr[1:])
    nnz = int(indptr[-1])
    indices = np.empty(nnz, np.int32)
    sub_map = np.empty((len(Ai), p.blk_nnz), np.int64)
    sub_rows = np.repeat(np.arange(bd), srow_nnz)           # sub-row of each base nz
    for r in range(p.nblk):
        cols = Ai[Ap[r]:Ap[r + 1]]
        nb = len(cols)
        for rb in range(bd):
            lo, hi = sAp[rb], sAp[rb + 1]
            dst0 = indptr[r * bd + rb]
            cc = (cols[:, None] * bd + sAi[None, lo:hi]).ravel()
            indices[dst0:dst0 + nb * (hi - lo)] = cc
            # block k of this row, base entry e -> dst0 + k*(hi-lo) + (e-lo)
            sub_map[Ap[r]:Ap[r + 1], lo:hi] = dst0 + np.arange(nb)[:, None] * (hi - lo) + np.arange(hi - lo)[None, :]
    p.A_indptr, p.A_indices, p.sub_map = indptr, indices, sub_map
    # the inverse map (position in A -> flat (pair, base entry)): filling A is
    # then a gather, split over the host threads like the reference's
    # OpenMP-parallel assembly
    p.sub_inv = np.empty(nnz, np.int64)
    p.sub_inv[sub_map.ravel()] = np.arange(nnz, dtype=np.int64)
    # S: block diagonal
    s_indptr = np.zeros(p.nblk * bd + 1, np.int64)
    np.cumsum(np.tile(srow_nnz, p.nblk), out=s_indptr[1:])
    s_indices = (np.arange(p.nblk)[:, None] * bd + sAi[None, :]).ravel().astype(np.int32)
    p.S_indptr, p.S_indices = s_indptr, s_indices
    p.S_map = np.arange(p.nblk * p.blk_nnz).reshape(p.nblk, p.blk_nnz)
    del sub_rows


def stationary(p: Problem, dt: float, h: float = 1.0):
    """compute_stationary_matrices (tools/solver.c:409-458): S and Hst values
    in the unblocked block-diagonal CSR."""
    ihdt = 1j * h * dt / 2
    k = p.kappa[:, None].astype(float)
    S = p.s0[0][None] + p.s0[1][None] * k + p.s0[2][None] * k * k
    Hst = ihdt * (p.h0[0][None] + p.h0[1][None] * k + p.h0[2][None] * k * k + p.h0[3][None] * k * k * k)
    n = p.n
    Sm = sp.csr_matrix((S.ravel(), p.S_indices, p.S_indptr), shape=(n, n))
    Hm = sp.csr_matrix((Hst.ravel(), p.S_indices, p.S_indptr), shape=(n, n))
    return Sm, Hm


def pgsums(p: Problem, dt: float, ft: np.ndarray, h: float = 1.0):
    """G-sums of tools/solver.c:246-286."""
    ihdt = 1j * h * dt / 2
    pg = np.zeros((p.lmax, 4, p.blk_nnz), complex)
    pgt = np.zeros_like(pg)
    for l in range(p.lmax):
        for a in range(6):
            if a % 2 != l % 2:
                c = SOL * ihdt * ft[a]
                pg[l] += c * p.g[a, l]
                pgt[l] += c * p.gt[a, l]
    return pg, pgt


def timedep(p: Problem, dt: float, ft: np.ndarray, h: float = 1.0) -> sp.csr_matrix:
    """compute_timedep_matrices (tools/solver.c:196-407): Hfull values.

    Each block (r,c) is ihdt*h0(k_r) on the diagonal plus
    sum_l H0l (pg_l0 + k_r pg_l1 + k_c pg_l2 + k_r k_c pg_l3)
        + H1l (pgt_l0 + k_c pgt_l1 + k_r pgt_l2 + k_r k_c pgt_l3);
    the sum over (l, q) is evaluated for all blocks at once as one matrix
    product (same terms, BLAS summation order)."""
    ihdt = 1j * h * dt / 2
    pg, pgt = pgsums(p, dt, ft, h)
    Ap, Ai = p.Hall.indptr, p.Hall.indices
    rows = np.repeat(np.arange(p.nblk), np.diff(Ap))
    ki = p.kappa[rows].astype(float)[:, None]
    kj = p.kappa[Ai].astype(float)[:, None]
    diag = p.perm[rows] == p.perm[Ai]
    nb, L = len(Ai), p.lmax
    coef = np.empty((nb, L, 8), complex)
    coef[:, :, 0] = p.H0
    coef[:, :, 1] = p.H0 * ki
    coef[:, :, 2] = p.H0 * kj
    coef[:, :, 3] = p.H0 * ki * kj
    coef[:, :, 4] = p.H1
    coef[:, :, 5] = p.H1 * kj
    coef[:, :, 6] = p.H1 * ki
    coef[:, :, 7] = p.H1 * ki * kj
    tab = np.concatenate([pg, pgt], axis=1)            # (L, 8, blk_nnz)
    sub = coef.reshape(nb, L * 8) @ tab.reshape(L * 8, p.blk_nnz)
    kd = ki[diag]
    sub[diag] += ihdt * (p.h0[0][None] + p.h0[1][None] * kd + p.h0[2][None] * kd * kd
                         + p.h0[3][None] * kd * kd * kd)
    data = _gather(sub.ravel(), p.sub_inv)
    return sp.csr_matrix((data, p.A_indices, p.A_indptr), shape=(p.n, p.n))


_POOL = None


def _gather(src: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """src[idx], split over the host threads (numpy releases the GIL)."""
    global _POOL
    out = np.empty(idx.size, src.dtype)
    nthr = os.cpu_count() or 1
    if idx.size < (1 << 20) or nthr == 1:
        np.take(src, idx, out=out)
        return out
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor
        _POOL = ThreadPoolExecutor(nthr)

    def part(k):
        lo, hi = k * idx.size // nthr, (k + 1) * idx.size // nthr
        np.take(src, idx[lo:hi], out=out[lo:hi])
    list(_POOL.map(part, range(nthr)))
    return out


def apply_block_rows(p: Problem, dt: float, ft: np.ndarray, x: np.ndarray, rows, h: float = 1.0):
    """S x and Hfull x on the listed block rows only, with the block values
    of ``timedep`` (tools/solver.c:196-407) and ``stationary``
    (tools/solver.c:409-458): for block row r, Hx_r = sum over the coupled
    blocks c of block(r, c) @ x_c, block(r, c) on the base pattern.  Needs no
    unblocked CSR, so it serves the largest configurations.  Returns two
    arrays [len(rows), blkdim]."""
    ihdt = 1j * h * dt / 2
    pg, pgt = pgsums(p, dt, ft, h)
    tab = np.concatenate([pg, pgt], axis=1).reshape(p.lmax * 8, p.blk_nnz)
    Ap, Ai = p.Hall.indptr, p.Hall.indices
    bd = p.blkdim
    base_rows = np.repeat(np.arange(bd), np.diff(p.sub_Ap))
    X = x.reshape(p.nblk, bd)
    Hx = np.zeros((len(rows), bd), complex)
    Sx = np.zeros((len(rows), bd), complex)
    for j, r in enumerate(rows):
        kr = float(p.kappa[r])
        for e in range(Ap[r], Ap[r + 1]):
            c = Ai[e]
            kc = float(p.kappa[c])
            coef = np.concatenate([p.H0[e][:, None] * np.array([1.0, kr, kc, kr * kc])[None, :],
                                   p.H1[e][:, None] * np.array([1.0, kc, kr, kr * kc])[None, :]], axis=1)
            vals = coef.reshape(p.lmax * 8) @ tab
            if p.perm[r] == p.perm[c]:
                vals = vals + ihdt * (p.h0[0] + p.h0[1] * kr + p.h0[2] * kr * kr + p.h0[3] * kr * kr * kr)
                svals = p.s0[0] + p.s0[1] * kr + p.s0[2] * kr * kr
                Sx[j] += _rowsum(base_rows, svals * X[c][p.sub_Ai], bd)
            Hx[j] += _rowsum(base_rows, vals * X[c][p.sub_Ai], bd)
    return Sx, Hx


def _rowsum(rows, v, n):
    out = np.zeros(n, complex)
    np.add.at(out, rows, v)
    return out


def overlap_from_files(workdir: str) -> sp.csr_matrix:
    """S in the solver order from the input files alone: block r is
    s0 + k s1 + k^2 s2 with k the kappa of block row r (tools/solver.c:428-432,
    block diagonal)."""
    from dirac_hydrogen_code_gb300.formats import csr_read as _read
    hall = _read(os.path.join(workdir, "H.csr"))
    s = [_read(os.path.join(workdir, f"s{i}.csr")).to_scipy() for i in range(3)]
    blocks = {}
    out = []
    for orig in hall.perm:
        k = ik(int(orig))
        if k not in blocks:
            blocks[k] = (s[0] + k * s[1] + k * k * s[2]).tocsr()
        out.append(blocks[k])
    return sp.block_diag(out, format="csr")


class IluPrecond:
    """SuperLU ILU of the preconditioner matrix with the reference options
    (tools/superlu.c:218-230).  The CSR arrays of P = S + Hst are handed to
    SuperLU as a CSC matrix (tools/superlu.c:142-152), so the factorised
    matrix is P^T; solve() applies (ILU(P^T))^{-1} like slu_lu_solve."""

    def __init__(self, S: sp.csr_matrix, Hst: sp.csr_matrix):
        P = S.data + Hst.data
        A = sp.csc_matrix((P, S.indices, S.indptr), shape=S.shape)
        self.lu = spla.spilu(A, drop_tol=1e-6, fill_factor=2.0, drop_rule="basic",
                             permc_spec="NATURAL", diag_pivot_thresh=0.0,
                             options=dict(Equil=False, RowPerm="NOROWPERM", ILU_MILU="SILU"))

    def solve(self, b):
        return self.lu.solve(b)


class BlockLuPrecond:
    """Exact LU of each diagonal block of P^T (one factorisation per distinct
    kappa).  The GB300 product path uses this preconditioner; the oracle
    offers it so that the product is checked with identical arithmetic."""

    def __init__(self, p: Problem, S: sp.csr_matrix, Hst: sp.csr_matrix):
        import scipy.linalg as sl
        self.p = p
        bd = p.blkdim
        self.fac = {}
        P = (S + Hst).tocsr()
        for r in range(p.nblk):
            k = int(p.kappa[r])
            if k in self.fac:
                continue
            blk = P[r * bd:(r + 1) * bd, r * bd:(r + 1) * bd].toarray().T
            self.fac[k] = sl.lu_factor(blk)

    def solve(self, b):
        import scipy.linalg as sl
        bd = self.p.blkdim
        out = np.empty_like(b)
        for r in range(self.p.nblk):
            out[r * bd:(r + 1) * bd] = sl.lu_solve(self.fac[int(self.p.kappa[r])], b[r * bd:(r + 1) * bd])
        return out


class Workspace:
    """Persistent BiCGSTAB vectors (solver_workspace_t): p and v survive from
    one call to the next exactly as in tools/bicgstab.c:28-31,136-153."""

    def __init__(self, n):
        self.v = np.zeros(n, complex)
        self.p = np.zeros(n, complex)


def bicgstab(matvec, rhs, x, psolve, wsp: Workspace, maxit: int, tol: float):
    """tools/bicgstab.c:125-295 (single rank).  Returns (iters, tol_error)."""
    n = len(rhs)
    rho = alpha = w = 1.0 + 0j
    v, p = wsp.v, wsp.p
    r = rhs - matvec(x)
    r0 = r.copy()
    r0_sqnorm = np.vdot(r0, r0).real
    rhs_sqnorm = np.vdot(rhs, rhs).real
    if rhs_sqnorm == 0:
        x[:] = 0
        return 0, 0.0
    tol2 = tol * tol * rhs_sqnorm
    eps2 = 1e-12 * 1e-12
    if r0_sqnorm < tol2:
        return 0, math.sqrt(r0_sqnorm / rhs_sqnorm)
    i = 0
    while i < maxit:
        rho_old = rho
        rho = np.vdot(r0, r)
        # fabs() of a C double complex takes the real part
        if abs(rho.real) < eps2 * r0_sqnorm:
            # The CPU build calls spmv(mat, x, r) without zeroing r first
            # (tools/bicgstab.c:217), so r = rhs - (r + A x).
            r = rhs - (r + matvec(x))
            r0 = r.copy()
            r0_sqnorm = np.vdot(r, r).real
            rho = r0_sqnorm + 0j
        beta = (rho / rho_old) * (alpha / w)
        p[:] = r + beta * (p - w * v)
        y = psolve(p)
        v[:] = matvec(y)
        alpha = rho / np.vdot(r0, v)
        s = r - alpha * v
        z = psolve(s)
        t = matvec(z)
        tmp = np.vdot(t, t).real
        w = np.vdot(t, s) / tmp if tmp > 0 else 0j
        x += alpha * y + w * z
        r = s - w * t
        tmp = np.vdot(r, r).real
        if tmp < tol2:
            break
        i += 1
    return i, math.sqrt(np.vdot(r, r).real / rhs_sqnorm)


@dataclasses.dataclass
class StepRecord:
    step: int
    time: float
    iters: int
    tol_error: float
    elapsed: float = 0.0          # wall seconds of the step (assembly + rhs + solve)


def run(workdir: str, maxtime: float, lmax: int, E0: float, omega: float, cycles: float,
        ntime: float, tol: float = 1e-16, maxit: int = 500, start_iter: int = 1,
        precond: str = "ilu", max_steps: int | None = None, psi=None, h: float = 1.0,
        problem: Problem | None = None, callback=None):
    """The time loop of tools/dirac_solver.c:496-636 (CPU build).

    Returns (x, records) with x in the solver's (permuted) order."""
    p = problem if problem is not None else load_problem(workdir, lmax)
    dt = maxtime / ntime
    S, Hst = stationary(p, dt, h)
    if not isinstance(precond, str):
        M = precond                      # a preconditioner built beforehand (same dt)
    else:
        M = IluPrecond(S, Hst) if precond == "ilu" else BlockLuPrecond(p, S, Hst)
    x = (p.psi0 if psi is None else psi).astype(complex).copy()
    wsp = Workspace(p.n)
    it = start_iter
    t = dt * (it - 1)
    recs = []
    while t <= maxtime:
        if max_steps is not None and len(recs) >= max_steps:
            break
        t = t + dt
        t0 = _time.perf_counter()
        ft = pulse(E0, omega, cycles, t)
        H = timedep(p, dt, ft, h)
        rhs = -(H @ x) + S @ x
        mv = lambda y: H @ y + S @ y
        iters, tol_err = bicgstab(mv, rhs, x, M.solve, wsp, maxit, tol)
        recs.append(StepRecord(it, t, iters, tol_err, _time.perf_counter() - t0))
        if callback is not None:
            callback(it, t, x)
        it += 1
    return x, recs, p


def s_norm(p: Problem, x: np.ndarray) -> float:
    """psi^H S psi with the overlap blocks of each kappa."""
    S, _ = stationary(p, 0.0)
    return float(np.vdot(x, S @ x).real)
