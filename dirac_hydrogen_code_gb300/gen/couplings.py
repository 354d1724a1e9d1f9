"""Restatement of ``dumpCouplings`` (src/dumpBdpCouplings.cpp:129-328).

Produces, in the reference file formats, every input the Crank-Nicolson
solver reads: the angular coupling matrices ``H0l<l>.csr``/``H1l<l>.csr``,
the radial Bessel coupling matrices ``g<n>a<alpha>l<l>.csr``, the stationary
Hamiltonian parts ``h0<n>.csr``, the overlap parts ``s<n>.csr`` and the
ground state ``psi0``.  The single-partition part of ``tools/main.py`` lives
in :mod:`.structure`.

Radial basis (src/splinehandler.cpp:25-60, 382-445; src/dkbbasis.cpp:100-330):
degree-7 B-splines on the uniform knots ``t_i = rBox*i/N`` padded with 7
copies of each end point, first and last spline dropped, so ``Ns = N+5``.
Integrals use 8-point Gauss-Legendre per knot interval.  The dual kinetic
balance (DKB) functions are

    P(k) = [B,  (-B' + k B/r) / 2c]      Q(k) = [(B' + k B/r) / 2c,  B]

split as ``P = P0 + k Pk``, ``Q = Q0 + k Qk`` (block ``blkdim = 2 Ns``).
Every radial matrix is stored through its kappa polynomial coefficients.

Angular basis (src/spnrbasis.cpp:50-93, 395-600): spinor states indexed by
``ik``/``imu``; couplings ``bdpK/L/M/N`` built from Wigner 3j symbols.

Everything here is CPU set-up tooling, computed in float64 (the reference
uses long double for the radial quadrature; results agree to ~1e-15
relative, well inside any tolerance used downstream).
"""
from __future__ import annotations

import functools
import json
import math
import os
from fractions import Fraction

import numpy as np
import scipy.linalg
import scipy.sparse as sp
from scipy.interpolate import BSpline
from scipy.special import spherical_jn

from ..formats import Csr, csr_write, dense_write

SOL = 137.035999084          # src/defs.h:35, tools/solver_common.h:37
SPLINE_DEG = 7               # src/dumpBdpCouplings.cpp:220
GL_ORDER = SPLINE_DEG + 1    # src/splinehandler.cpp:391 (l = splinedeg + 1)


# --------------------------------------------------------------------------
# angular index maps (tools/solver_common.c:30-44, src/spnrbasis.cpp:603-640)
# --------------------------------------------------------------------------
def ik(i: int) -> int:
    ii = i // 4
    abskappa = int(0.5 * (math.sqrt(8.0 * ii + 1.0) - 1.0)) + 1
    sgnmod = max(4, abskappa * 4)
    sgnfloor = 2.0 * abskappa * (abskappa - 1)
    q = (i - sgnfloor) / sgnmod
    return abskappa * ((q >= 0.5) - (q < 0.5))


def imu(i: int) -> float:
    abskappa = abs(ik(i))
    kmod = max(2, 2 * abskappa)
    return i % kmod - abskappa + 0.5


def n_angular(kmax: int) -> int:
    """spnrbasis::aqn (src/spnrbasis.cpp:84-90)."""
    return 4 if kmax == 1 else 2 * (kmax + 1) * kmax


# --------------------------------------------------------------------------
# Wigner 3j for integer arguments (Racah formula, exact rational arithmetic)
# --------------------------------------------------------------------------
@functools.lru_cache(maxsize=None)
def wigner3j(j1: int, j2: int, j3: int, m1: int, m2: int, m3: int) -> float:
    if m1 + m2 + m3 != 0:
        return 0.0
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return 0.0
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    f = math.factorial
    pref = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    pref *= f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3)
    kmin = max(0, j2 - j3 - m1, j1 - j3 + m2)
    kmax = min(j1 + j2 - j3, j1 - m1, j2 + m2)
    s = Fraction(0)
    for k in range(kmin, kmax + 1):
        den = (f(k) * f(j3 - j2 + k + m1) * f(j3 - j1 + k - m2) * f(j1 + j2 - j3 - k)
               * f(j1 - k - m1) * f(j2 - k + m2))
        s += Fraction((-1) ** k, den)
    sign = -1 if (j1 - j2 - m3) % 2 else 1
    # sqrt(pref) * s, evaluated so that the only rounding is in the final sqrt
    val = s * s * pref
    r = math.sqrt(val.numerator) / math.sqrt(val.denominator)
    return float(sign * (1 if s >= 0 else -1) * r)


def _ipow(n: int) -> complex:
    return (1, 1j, -1, -1j)[n % 4]


def _sgn(v: float) -> int:
    return (v > 0) - (v < 0)


def _bdp_term(ki, kj, mui, muj, l, which):
    """bdpK/bdpL/bdpM/bdpN of src/spnrbasis.cpp:523-600."""
    if which in "KL":
        a2, b2 = abs(ki + 0.5), abs(kj - 0.5)
    else:
        a2, b2 = abs(ki - 0.5), abs(kj + 0.5)
    if which in "KM":
        if int(2 * muj) != int(2 * mui) - 2:
            return 0.0
    else:
        if int(2 * muj) != int(2 * mui) + 2:
            return 0.0
    if not (abs(a2 - b2) <= l <= a2 + b2 - 1):
        return 0.0
    ja, jb = int(round(a2 - 0.5)), int(round(b2 - 0.5))
    ph = _ipow(int(2 * mui + l))
    w0 = wigner3j(ja, jb, l, 0, 0, 0)
    if which == "K":
        ph *= _sgn(ki)
        amp = math.sqrt(abs(ki + 0.5 - mui) * abs(kj - 0.5 - muj))
        w1 = wigner3j(ja, jb, l, int(round(-mui + 0.5)), int(round(muj + 0.5)), 0)
    elif which == "L":
        ph *= _sgn(kj)
        amp = math.sqrt(abs(ki + 0.5 + mui) * abs(kj - 0.5 + muj))
        w1 = wigner3j(ja, jb, l, int(round(-mui - 0.5)), int(round(muj - 0.5)), 0)
    elif which == "M":
        ph *= _sgn(ki)
        amp = math.sqrt(abs(ki - 0.5 + mui) * abs(kj + 0.5 + muj))
        w1 = wigner3j(ja, jb, l, int(round(-mui + 0.5)), int(round(muj + 0.5)), 0)
    else:
        ph *= _sgn(kj)
        amp = math.sqrt(abs(ki - 0.5 - mui) * abs(kj + 0.5 - muj))
        w1 = wigner3j(ja, jb, l, int(round(-mui - 0.5)), int(round(muj - 0.5)), 0)
    return ph * (2.0 * l + 1.0) * amp * w0 * w1


def angular_coupling(kmax: int, mumax: int, ul: int, l: int) -> sp.csr_matrix:
    """spnrbasis::bdpalphsigmaXmat(ul, l) (src/spnrbasis.cpp:395-470)."""
    nth = n_angular(kmax)
    kap = [ik(i) for i in range(nth)]
    mu = [imu(i) for i in range(nth)]
    rows, cols, vals = [], [], []
    pair = ("K", "L") if ul == 1 else ("M", "N")
    for i in range(nth):
        for j in range(nth):
            # src/spnrbasis.cpp:418 and :438: only |mu| < mumax couples
            if mumax != 0 and (abs(mu[i]) >= mumax or abs(mu[j]) >= mumax):
                continue
            if abs(abs(mu[i] - mu[j]) - 1.0) > 1e-9:
                continue
            x1 = _bdp_term(kap[i], kap[j], mu[i], mu[j], l, pair[0])
            x2 = _bdp_term(kap[i], kap[j], mu[i], mu[j], l, pair[1])
            if x1 != 0 or x2 != 0:
                v = (1j if l % 2 == 1 else -1.0) * (x1 + x2)
                rows.append(i); cols.append(j); vals.append(v)
    m = sp.csr_matrix((np.array(vals, complex), (rows, cols)), shape=(nth, nth))
    m.sort_indices()
    return m


# --------------------------------------------------------------------------
# radial DKB basis
# --------------------------------------------------------------------------
class RadialBasis:
    """Dual-kinetic-balance B-spline basis evaluated at the quadrature points."""

    def __init__(self, nsplines: int, rbox: float):
        t = np.array([rbox / nsplines * i for i in range(nsplines + 1)])
        self.t = t
        z, wz = np.polynomial.legendre.leggauss(GL_ORDER)
        h = np.diff(t)
        self.x = (t[:-1, None] + (1.0 + z[None, :]) * h[:, None] / 2).ravel()
        self.w = (wz[None, :] * h[:, None] / 2).ravel()
        tpad = np.concatenate([[t[0]] * SPLINE_DEG, t, [t[-1]] * SPLINE_DEG])
        nspl = len(tpad) - 1 - SPLINE_DEG
        spl = BSpline(tpad, np.eye(nspl), SPLINE_DEG, extrapolate=False)
        B = np.nan_to_num(spl(self.x, 0))[:, 1:-1]
        dB = np.nan_to_num(spl(self.x, 1))[:, 1:-1]
        d2B = np.nan_to_num(spl(self.x, 2))[:, 1:-1]
        self.ns = B.shape[1]
        c2 = 1.0 / (2 * SOL)
        ix = 1.0 / self.x
        Z = np.zeros_like(B)
        Bx = B * ix[:, None]
        dBx = dB * ix[:, None] - B * (ix ** 2)[:, None]
        self.P0 = np.hstack([B, -c2 * dB]); self.Pk = np.hstack([Z, c2 * Bx])
        self.Q0 = np.hstack([c2 * dB, B]);  self.Qk = np.hstack([c2 * Bx, Z])
        self.dP0 = np.hstack([dB, -c2 * d2B]); self.dPk = np.hstack([Z, c2 * dBx])
        self.dQ0 = np.hstack([c2 * d2B, dB]);  self.dQk = np.hstack([c2 * dBx, Z])
        self.blkdim = 2 * self.ns

    @staticmethod
    def glint(a, w, b):
        return a.T @ (w[:, None] * b)

    def _fact(self, f):
        """kappa-factorised integral (src/dkbbasis.cpp:89-100)."""
        m0 = f(self.P0, self.Q0, self.P0, self.Q0)
        mk = f(self.P0, self.Q0, self.Pk, self.Qk) + f(self.Pk, self.Qk, self.P0, self.Q0)
        mkk = f(self.Pk, self.Qk, self.Pk, self.Qk)
        return m0, mk, mkk

    def overlap(self):
        w, g = self.w, self.glint
        return self._fact(lambda aP, aQ, bP, bQ: g(aP, w, bP) + g(aQ, w, bQ))

    def stationary(self, Z: int):
        """h0..h3 of DiracBDP::H0radprep (src/hamiltonian.h:617-638)."""
        w, g, c = self.w, self.glint, SOL
        wv = w * (-Z / self.x)
        kw = w / self.x
        E = self._fact(lambda aP, aQ, bP, bQ: g(aP, wv, bP) + g(aQ, wv, bQ))
        ulc = self._fact(lambda aP, aQ, bP, bQ: g(aQ, w, bQ))
        K = self._fact(lambda aP, aQ, bP, bQ: g(aQ, kw, bP) + g(aP, kw, bQ))
        # derivative matrix, symmetrised as in src/dkbbasis.cpp:473-480
        f = lambda aP, aQ, bP, bQ: g(aQ, w, bP) - g(aP, w, bQ)
        dd0 = f(self.P0, self.Q0, self.dP0, self.dQ0)
        ddk = f(self.P0, self.Q0, self.dPk, self.dQk) + f(self.Pk, self.Qk, self.dP0, self.dQ0)
        ddkk = f(self.Pk, self.Qk, self.dPk, self.dQk)
        dd = [(m + m.T) / 2 for m in (dd0, ddk, ddkk)]
        h0 = c * dd[0] + E[0] - 2 * c * c * ulc[0]
        h1 = c * (dd[1] + K[0]) + E[1] - 2 * c * c * ulc[1]
        h2 = c * (dd[2] + K[1]) + E[2] - 2 * c * c * ulc[2]
        h3 = c * K[2]
        return h0, h1, h2, h3

    def bessel_couplings(self, l: int, omega: float, cycles: float):
        """g_{n,alpha,l} for n = p00, p0k, pk0, pkk (src/dkbbasis.cpp:780-822)
        with the radial pulse factors of src/potential.h:471-500."""
        T = cycles * 2 * math.pi / omega
        k = omega / SOL
        q = 2 * math.pi / (SOL * T)
        kvec = [q + k, q + k, -(q - k), -(q - k), k, k]
        out = []
        g = self.glint
        for a in range(6):
            cw = self.w * spherical_jn(l, kvec[a] * self.x)
            out.append([g(self.P0, cw, self.Q0), g(self.Pk, cw, self.Q0),
                        g(self.P0, cw, self.Qk), g(self.Pk, cw, self.Qk)])
        return out  # out[alpha][n]

    def base_pattern(self) -> sp.csr_matrix:
        """Union pattern of all radial matrices: 2x2 blocks, each banded
        with the B-spline overlap half-width SPLINE_DEG."""
        ns = self.ns
        i = np.arange(2 * ns)
        d = np.abs((i % ns)[:, None] - (i % ns)[None, :]) <= SPLINE_DEG
        return sp.csr_matrix(d.astype(float))


def _pattern_csr(dense: np.ndarray, pat: sp.csr_matrix) -> Csr:
    rows = np.repeat(np.arange(pat.shape[0]), np.diff(pat.indptr))
    vals = dense[rows, pat.indices].astype(complex)
    return Csr(pat.shape[0], pat.indptr.astype(np.int32), pat.indices.astype(np.int32), vals)


def ground_state(h: tuple, s: tuple, Z: int, kappa: int = -1):
    """Lowest bound state of kappa=-1 (src/hamiltonian.h:872-960,1373-1395)."""
    H = h[0] + kappa * h[1] + kappa ** 2 * h[2] + kappa ** 3 * h[3]
    S = s[0] + kappa * s[1] + kappa ** 2 * s[2]
    evals, evecs = scipy.linalg.eigh(H, S)
    e0 = -Z * Z / 2.0
    idx = int(np.argmin(np.abs(evals - e0)))
    v = evecs[:, idx].copy()
    vv = np.max(np.abs(v))
    j = int(np.argmax(np.abs(v) * 100 > vv))
    if v[j] < 0:
        v = -v
    return evals[idx], v


def dump_couplings(params: dict, outdir: str, verbose: bool = False) -> dict:
    """Write all dumpCouplings outputs for ``params`` into ``outdir``.

    ``params`` uses the JSON keys of src/dumpBdpCouplings.cpp:156-165.
    Returns a summary dict (sizes, ground-state energy).
    """
    ns_, nk, nmu = int(params["Nsplines"]), int(params["Nkappa"]), int(params["Nmu"])
    nl = int(params["Nl"])
    rbox, omega, cycles = float(params["rBox"]), float(params["Omega"]), float(params["Cycles"])
    Z = int(params["Z"])
    lmax = nl if nl != 0 else 2 * nk + 1           # spnrbasis::bdplmax, src/basis.h:607-611
    os.makedirs(outdir, exist_ok=True)

    for l in range(lmax):
        csr_write(os.path.join(outdir, f"H0l{l}.csr"), Csr.from_scipy(angular_coupling(nk, nmu, 1, l)))
        csr_write(os.path.join(outdir, f"H1l{l}.csr"), Csr.from_scipy(angular_coupling(nk, nmu, -1, l)))

    rb = RadialBasis(ns_, rbox)
    pat = rb.base_pattern()
    for l in range(lmax):
        gl = rb.bessel_couplings(l, omega, cycles)
        for a in range(6):
            for n in range(4):
                csr_write(os.path.join(outdir, f"g{n}a{a}l{l}.csr"), _pattern_csr(gl[a][n], pat))
    h = rb.stationary(Z)
    for n in range(4):
        csr_write(os.path.join(outdir, f"h0{n}.csr"), _pattern_csr(h[n], pat))
    s = rb.overlap()
    for n in range(3):
        csr_write(os.path.join(outdir, f"s{n}.csr"), _pattern_csr(s[n], pat))
    e0, v0 = ground_state(h, s, Z)
    nth = n_angular(nk)
    psi = np.zeros((rb.blkdim, nth), complex)
    psi[:, 0] = v0          # index 0 is (kappa=-1, mu=-1/2)
    dense_write(os.path.join(outdir, "psi0"), psi.reshape(-1, order="F"))
    info = dict(lmax=lmax, blkdim=rb.blkdim, blk_nnz=int(pat.nnz), n_angular=nth, e0=float(e0))
    if verbose:
        print(json.dumps(info))
    return info
