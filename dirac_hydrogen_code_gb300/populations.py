"""Bound and ionised populations of a state (the reference's
``dumpEigvals`` + ``processOutput``, src/dumpEigvals.cpp:131-269,
src/process_output.cpp:168-399, src/hamiltonian.h:872-983,1246-1330).

For every kappa the radial field-free problem H0(k) v = E S(k) v is solved
once (H0(k) = h00 + k h01 + k^2 h02 + k^3 h03, S(k) = s0 + k s1 + k^2 s2 from
the problem's ``h0<n>.csr`` / ``s<n>.csr``; real symmetric, S-orthonormal
eigenvectors with the reference's sign convention).  A state's projection on
eigenvector j of block row r is c_j = x_r^H S(k_r) v_j, and its population
|c_j|^2.  Eigenvalues (rest energy subtracted) split the spectrum into the
negative-energy states (E < -c^2), the bound states (-c^2 <= E < 0) and the
continuum (E >= 0, ionised).  The projection runs on the host (numpy) or on
the GPU (``gade_eigproj``, FP64), both from the same eigenpairs.

CLI: ``python -m dirac_hydrogen_code_gb300.populations WORKDIR LMAX x<iter>.out``
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import scipy.linalg

from .formats import csr_read, out_read
from .gen.couplings import SOL

E_NEG = -SOL * SOL          # below: negative-energy (Dirac sea) states


def _dense(workdir: str, name: str) -> np.ndarray:
    return csr_read(os.path.join(workdir, name)).to_scipy().toarray().real


class Eigenbasis:
    """Eigenpairs of every kappa that occurs in a problem's block rows."""

    def __init__(self, workdir: str, kappa_of_block: np.ndarray):
        h = [_dense(workdir, f"h0{n}.csr") for n in range(4)]
        s = [_dense(workdir, f"s{n}.csr") for n in range(3)]
        self.kappas = sorted({int(k) for k in kappa_of_block})
        kidx = {k: i for i, k in enumerate(self.kappas)}
        self.block_kidx = np.array([kidx[int(k)] for k in kappa_of_block], np.int32)
        B = h[0].shape[0]
        self.B = B
        self.evals = np.zeros((len(self.kappas), B))
        self.W = np.zeros((len(self.kappas), B, B))        # S(k) V(k), [i][j]
        for i, k in enumerate(self.kappas):
            H = h[0] + k * h[1] + k ** 2 * h[2] + k ** 3 * h[3]
            S = s[0] + k * s[1] + k ** 2 * s[2]
            E, V = scipy.linalg.eigh(H, S)
            # sign convention of src/hamiltonian.h:960-983: the first entry
            # larger than 1% of the largest magnitude is positive
            vmax = np.max(np.abs(V), axis=0)
            first = np.argmax(np.abs(V) * 100 > vmax[None, :], axis=0)
            sign = np.sign(V[first, np.arange(B)])
            sign[sign == 0] = 1.0
            V = V * sign[None, :]
            self.evals[i] = E
            self.W[i] = S @ V
        self._dev = None

    def project(self, x: np.ndarray) -> np.ndarray:
        """c[r][j] = x_r^H S(k_r) v_j for a state x (solver order, nblk*B)."""
        X = x.reshape(-1, self.B)
        out = np.empty(X.shape, np.complex128)
        for r in range(X.shape[0]):
            out[r] = X[r].conj() @ self.W[self.block_kidx[r]]
        return out

    def classes(self, c: np.ndarray) -> np.ndarray:
        """[nblk][4]: population of negative-energy, bound and continuum
        states, and the total (= x_r^H S x_r), per block row."""
        p = np.abs(c) ** 2
        E = self.evals[self.block_kidx]
        out = np.zeros((c.shape[0], 4))
        out[:, 0] = np.where(E < E_NEG, p, 0).sum(1)
        out[:, 1] = np.where((E >= E_NEG) & (E < 0), p, 0).sum(1)
        out[:, 2] = np.where(E >= 0, p, 0).sum(1)
        out[:, 3] = p.sum(1)
        return out

    def populations(self, x: np.ndarray) -> dict:
        return summary(self.classes(self.project(x)))

    def populations_device(self, x_ptr: int, ld: int, npulse: int, stream: int = 0) -> list[dict]:
        """The same on the GPU for npulse states at device address x_ptr
        (complex128, pulse stride ld elements)."""
        import torch
        from . import native
        if self._dev is None:
            self._dev = dict(W=torch.from_numpy(self.W).cuda(), E=torch.from_numpy(self.evals).cuda(),
                             kidx=torch.from_numpy(self.block_kidx).cuda())
        d = self._dev
        nblk = len(self.block_kidx)
        cls = torch.empty(npulse, nblk, 4, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        native.call("gade_eigproj", npulse, nblk, self.B, d["kidx"].data_ptr(), d["W"].data_ptr(),
                    d["E"].data_ptr(), E_NEG, int(x_ptr), int(ld), None, cls.data_ptr(), stream)
        torch.cuda.synchronize()
        return [summary(c) for c in cls.cpu().numpy()]


def summary(classes: np.ndarray) -> dict:
    tot = classes.sum(0)
    return {"negative": float(tot[0]), "bound": float(tot[1]), "continuum": float(tot[2]), "norm": float(tot[3])}


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 3:
        print("usage: python -m dirac_hydrogen_code_gb300.populations WORKDIR LMAX x<iter>.out", file=sys.stderr)
        return 1
    from .native import Problem
    workdir, lmax, fname = argv[0], int(argv[1]), argv[2]
    prob = Problem(workdir, lmax)
    kap, _ = prob.blocks()
    _, xperm = prob.psi0()
    xorig = out_read(fname)
    x = xorig[xperm]                       # x[i] = xorig[xperm[i]] (tools/dirac_solver.c:600-606)
    print(json.dumps(Eigenbasis(workdir, kap).populations(x)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
