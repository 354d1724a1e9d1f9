"""CPU check of the block-LU sweep form that k_precond_tma runs.

Each sweep over the 32-row chunks of a block row is split into the
inverse-diagonal-block products of every chunk (two chunks' triangles packed
per lane so that lane i runs 33 products: row i of chunk 2p, then row 31-i
of chunk 2p+1) and a chain through the neighbour blocks
G_c = -Linv_c Lband_c (U: GU_c = -Uinv_c Uband_c).  This test restates the
packing of pack_factors and the index arithmetic of the kernel in numpy, for
band paddings 16 and 32, for chunk counts with an unpaired last chunk and
padded rows, and for 4 and 8 warps per block row (with 8, two warps split a
lane's 33 products at 17 and the chain's columns spread over 8 partial
sums), and compares the result with a direct LU solve.  (The kernel
itself is compared with the oracle's block LU on the GPU in
tests/test_gpu_parity.py.)
"""
import numpy as np
import pytest

TP = 33 * 32


def _pack(L, U, B, bw, bwp):
    nch = (B + 31) // 32
    Bp = 32 * nch
    Lp = np.eye(Bp, dtype=complex)
    Lp[:B, :B] = L
    Up = np.eye(Bp, dtype=complex)
    Up[:B, :B] = U
    Linv = [np.linalg.inv(Lp[32 * c:32 * c + 32, 32 * c:32 * c + 32]) for c in range(nch)]
    Uinv = [np.linalg.inv(Up[32 * c:32 * c + 32, 32 * c:32 * c + 32]) for c in range(nch)]
    npair = (nch + 1) // 2
    TL = np.zeros((npair, 33, 32), complex)
    TU = np.zeros((npair, 33, 32), complex)
    q = np.arange(33)[:, None]
    i = np.arange(32)[None, :]
    for p in range(npair):
        c0, c1 = 2 * p, 2 * p + 1
        first_l, first_u = q <= i, q <= 31 - i
        TL[p] = np.where(first_l, Linv[c0][i, np.minimum(q, 31)], 0)
        TU[p] = np.where(first_u, Uinv[c0][i, np.minimum(i + q, 31)], 0)
        if c1 < nch:
            TL[p] += np.where(first_l, 0, Linv[c1][31 - i, np.clip(q - i - 1, 0, 31)])
            TU[p] += np.where(first_u, 0, Uinv[c1][31 - i, np.clip(q - 1, 0, 31)])
    GL = np.zeros((nch, bwp, 32), complex)
    GU = np.zeros((nch, bwp, 32), complex)
    for c in range(nch):
        rows = np.arange(32 * c, min(32 * c + 32, B))
        m = rows - 32 * c
        for col in range(bwp):
            cl = 32 * c - bwp + col
            if c > 0 and cl >= 0:
                d = rows - cl
                ok = (d >= 1) & (d <= bw)
                band = np.where(ok, L[rows, cl], 0)
                GL[c, col] = -(Linv[c][:, m] @ band)
            cu = 32 * (c + 1) + col
            if c + 1 < nch and cu < B:
                d = cu - rows
                ok = (d >= 1) & (d <= bw)
                band = np.where(ok, U[rows, cu], 0)
                GU[c, col] = -(Uinv[c][:, m] @ band)
    return nch, Bp, npair, TL, TU, GL, GU


def _triangle_part(T, buf, p, lane, c0, c1, has1, up, q0, q1):
    """pc_triangle_part: products q0..q1-1 of one lane, split into the part
    of row c0 (products up to sw) and the part of row c1."""
    sw = 31 - lane if up else lane
    acc = sav = 0
    for q in range(q0, q1):
        if not up:
            src = 32 * c0 + q if q <= lane else (32 * c1 + q - lane - 1 if has1 else 0)
        else:
            src = 32 * c0 + lane + q if q <= 31 - lane else (32 * c1 + q - 1 if has1 else 0)
        acc += T[p, q, lane] * buf[src]
        if q == sw:
            sav, acc = acc, 0
    if sw >= q1:
        return acc, 0
    if sw >= q0:
        return sav, acc
    return 0, acc


def _sweeps(b, nch, npair, TL, TU, GL, GU, bwp, nw=4):
    """k_precond_tma with nw warps per block row: with 8, warps w and w + 4
    split a pair's 33 products per lane (0-16, 17-32) and the chain's
    columns are spread over 8 warps."""
    halves = [(0, 33)] if nw == 4 else [(0, 17), (17, 33)]
    cpw = bwp // nw
    buf = b.copy()
    for up in (0, 1):
        T, G = (TU, GU) if up else (TL, GL)
        for p in range(npair):
            c0, c1 = 2 * p, 2 * p + 1
            has1 = c1 < nch
            out0 = np.zeros(32, complex)
            out1 = np.zeros(32, complex)
            for lane in range(32):
                for q0, q1 in halves:
                    a0, a1 = _triangle_part(T, buf, p, lane, c0, c1, has1, up, q0, q1)
                    out0[lane] += a0
                    out1[lane] += a1
            buf[32 * c0:32 * c0 + 32] = out0
            if has1:
                buf[32 * c1:32 * c1 + 32] = out1[::-1]
        for c in (range(nch - 1, -1, -1) if up else range(nch)):
            if (up and c == nch - 1) or (not up and c == 0):
                continue
            base = 32 * (c + 1) if up else 32 * c - bwp
            parts = []
            for w in range(nw):
                t = buf[32 * c:32 * c + 32].copy() if w == 0 else np.zeros(32, complex)
                for col in range(w * cpw, (w + 1) * cpw):
                    t += G[c, col] * buf[base + col]
                parts.append(t)
            buf[32 * c:32 * c + 32] = sum(parts)
    return buf


@pytest.mark.parametrize("nw", [4, 8])
@pytest.mark.parametrize("B,bw,bwp", [(130, 15, 16), (96, 20, 32), (33, 3, 16), (200, 31, 32)])
def test_sweep_form_solves_lu(B, bw, bwp, nw):
    rng = np.random.default_rng(B + bw)
    A = np.zeros((B, B), complex)
    for r in range(B):
        lo, hi = max(0, r - bw), min(B, r + bw + 1)
        A[r, lo:hi] = rng.standard_normal(hi - lo) + 1j * rng.standard_normal(hi - lo)
        A[r, r] += 4 * bw
    # banded LU without pivoting, unit lower L (as gade_setup_build factors)
    L = np.eye(B, dtype=complex)
    U = A.copy()
    for k in range(B):
        for r in range(k + 1, min(B, k + bw + 1)):
            L[r, k] = U[r, k] / U[k, k]
            U[r, :] -= L[r, k] * U[k, :]
    U = np.triu(U)
    nch, Bp, npair, TL, TU, GL, GU = _pack(L, U, B, bw, bwp)
    b = np.zeros(Bp, complex)
    b[:B] = rng.standard_normal(B) + 1j * rng.standard_normal(B)
    x = _sweeps(b, nch, npair, TL, TU, GL, GU, bwp, nw)
    ref = np.linalg.solve(U, np.linalg.solve(L, b[:B]))
    assert np.abs(x[:B] - ref).max() < 1e-13 * np.abs(ref).max()
    assert not np.any(x[B:])
