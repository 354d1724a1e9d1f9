"""Per-pulse inputs of batched runs.

Pulses that differ in Omega or Cycles differ only in the radial tables g
(Bessel arguments k = omega/SoL and 2 pi/(SoL T) +- k, src/potential.h:471-500)
and in dt = T/Ntime; the angular tables, h0 and S are shared.
``pulse_tables`` computes one pulse's g directly in the layout that
``gade_batch_create`` takes, without writing 24*lmax files per pulse: the
quadrature integrals are assembled interval by interval (every B-spline lives
on SPLINE_DEG+1 knot intervals), which gives the same values as the dense
products that ``dump_couplings`` writes, up to summation order.
"""
from __future__ import annotations

import math
import os

import numpy as np
from scipy.special import spherical_jn

from .couplings import GL_ORDER, SOL, RadialBasis


class _Local:
    """Active basis columns of every knot interval of a RadialBasis."""

    def __init__(self, rb: RadialBasis):
        nint = len(rb.t) - 1
        ncol = rb.P0.shape[1]
        nz = (rb.P0 != 0) | (rb.Pk != 0) | (rb.Q0 != 0) | (rb.Qk != 0)
        act = nz.reshape(nint, GL_ORDER, ncol).any(axis=1)
        K = int(act.sum(axis=1).max())
        cols = np.zeros((nint, K), np.int64)
        mask = np.zeros((nint, K))
        for e in range(nint):
            c = np.nonzero(act[e])[0]
            cols[e, :len(c)] = c
            mask[e, :len(c)] = 1.0
        self.nint, self.ncol, self.cols, self.mask = nint, ncol, cols, mask
        self.gather = cols[:, None, :].repeat(GL_ORDER, axis=1)
        self.w = rb.w.reshape(nint, GL_ORDER)

    def local(self, a: np.ndarray) -> np.ndarray:
        a3 = a.reshape(self.nint, GL_ORDER, self.ncol)
        return np.take_along_axis(a3, self.gather, axis=2) * self.mask[:, None, :]

    def scatter(self, rows: np.ndarray, cidx: np.ndarray):
        """Sparse map from the interval-local products (e, i, j) to the
        base-pattern positions they add to."""
        import scipy.sparse as sp
        K = self.cols.shape[1]
        pos = {(int(r), int(c)): k for k, (r, c) in enumerate(zip(rows, cidx))}
        src, dst = [], []
        for e in range(self.nint):
            for i in range(K):
                if not self.mask[e, i]:
                    continue
                for j in range(K):
                    if not self.mask[e, j]:
                        continue
                    k = pos.get((int(self.cols[e, i]), int(self.cols[e, j])))
                    if k is not None:
                        src.append((e * K + i) * K + j)
                        dst.append(k)
        self.S = sp.csr_matrix((np.ones(len(src)), (dst, src)), shape=(len(rows), self.nint * K * K))

    def glint(self, A: np.ndarray, cw: np.ndarray, Bm: np.ndarray) -> np.ndarray:
        """Pattern values of sum_p a_i(p) cw_c(p) b_j(p) for every weight
        function c: cw [C, nint, GL_ORDER] -> [C, pattern nnz]."""
        tmp = cw[:, :, :, None] * A[None]                          # c e p i
        loc = np.matmul(tmp.transpose(0, 1, 3, 2), Bm[None])         # c e i j
        return (self.S @ loc.reshape(cw.shape[0], -1).T).T


def pulse_tables(params: dict, omega: float, cycles: float, rb: RadialBasis | None = None,
                 _cache: dict = {}) -> np.ndarray:
    """Radial tables of one pulse: complex128 [6, lmax, 4, blk_nnz] with
    [a, l, q] = the values of g<q>a<a>l<l>.csr in the base pattern's CSR
    order (src/dkbbasis.cpp:780-822 with the pulse factors of
    src/potential.h:471-500)."""
    ns_, nk, nl = int(params["Nsplines"]), int(params["Nkappa"]), int(params["Nl"])
    rbox = float(params["rBox"])
    lmax = nl if nl != 0 else 2 * nk + 1
    key = (ns_, rbox)
    if key not in _cache:
        b = rb if rb is not None else RadialBasis(ns_, rbox)
        loc = _Local(b)
        pat = b.base_pattern()
        rows = np.repeat(np.arange(pat.shape[0]), np.diff(pat.indptr))
        mats = [loc.local(m) for m in (b.P0, b.Pk, b.Q0, b.Qk)]
        loc.scatter(rows, pat.indices)
        _cache.clear()
        _cache[key] = (b, loc, rows, pat.indices.astype(np.int64), mats)
    b, loc, rows, cidx, (P0, Pk, Q0, Qk) = _cache[key]
    T = cycles * 2 * math.pi / omega
    k = omega / SOL
    q = 2 * math.pi / (SOL * T)
    kvec = [q + k, q + k, -(q - k), -(q - k), k, k]
    out = np.zeros((6, lmax, 4, len(rows)), np.complex128)
    x = b.x.reshape(loc.nint, GL_ORDER)
    cw = np.stack([loc.w * spherical_jn(l, kvec[a] * x) for a in range(6) for l in range(lmax)])
    for n, (A, Bm) in enumerate(((P0, Q0), (Pk, Q0), (P0, Qk), (Pk, Qk))):
        out[:, :, n, :] = loc.glint(A, cw, Bm).reshape(6, lmax, -1)
    return out


def draw_pulses(n: int, seed: int) -> list[dict]:
    """Seeded pulse set of the batched workload: Intensity log-uniform in
    [1, 100], Omega uniform in [10, 100], Cycles uniform in {1, 2, 3},
    Ntime = 500 * Cycles, maxtime = Cycles * 2 pi / Omega."""
    rng = np.random.default_rng(seed)
    E0 = np.exp(rng.uniform(np.log(1.0), np.log(100.0), n))
    omega = rng.uniform(10.0, 100.0, n)
    cycles = rng.integers(1, 4, n)
    return [dict(E0=float(E0[i]), omega=float(omega[i]), cycles=int(cycles[i]), ntime=500 * int(cycles[i]),
                 maxtime=int(cycles[i]) * 2 * math.pi / float(omega[i])) for i in range(n)]


def _tables_job(args):
    params, omega, cycles = args
    return pulse_tables(params, omega, cycles)


def pulse_tables_many(params: dict, pulses: list[dict], workers: int | None = None) -> np.ndarray:
    """[npulse, 6, lmax, 4, blk_nnz] radial tables of many pulses, computed in
    a pool of fresh (spawned) worker processes: safe after the parent has
    initialised a GPU."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    jobs = [(params, p["omega"], p["cycles"]) for p in pulses]
    workers = workers or min(len(jobs), os.cpu_count() or 1)
    if workers <= 1 or len(jobs) <= 1:
        return np.stack([_tables_job(j) for j in jobs])
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return np.stack(list(ex.map(_tables_job, jobs, chunksize=max(1, len(jobs) // (4 * workers)))))
