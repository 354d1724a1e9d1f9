"""CPU oracle of the eigenstate projection — TEST INFRASTRUCTURE ONLY.

A numpy/scipy restatement of what the reference does with a state written
by ``dirac_solver``: ``dumpEigvals`` (src/dumpEigvals.cpp:131-269) solves,
for every kappa, the radial field-free generalised eigenproblem and writes
``evl<kappa>.mat``/``evc<kappa>.mat``; ``processOutput``
(src/process_output.cpp:168-399) reads ``x<iter>.out`` and projects every
angular block of the state on the eigenvectors of its kappa
(``savePsievs`` -> ``eigProj``).  Only ``tests/`` may import this module;
the product's projection (``gade_eigproj`` and
``dirac_hydrogen_code_gb300.populations``) is checked against it.

Followed line by line:
  * eigenpairs per kappa     src/hamiltonian.h:872-958 (prepeigsLowMem: the
    kappas -1, 1, -2, 2, ..., each H0(k) v = E S(k) v with Eigen's
    generalised self-adjoint solver: ascending eigenvalues, S-orthonormal
    eigenvectors; the radial matrices of a kappa are the kappa polynomials
    the generator writes, h0<n>.csr and s<n>.csr, src/dumpBdpCouplings.cpp)
  * sign convention          src/hamiltonian.h:960-983 (the first entry whose
    magnitude times 100 exceeds the column's largest magnitude is positive)
  * projection               src/hamiltonian.h:1246-1300 (eigProj: for block
    th with kappa k, psiev = psiseg^H [S v_0, S v_1, ...])
The energy classes (negative-energy E < -c^2, bound -c^2 <= E < 0,
continuum E >= 0) are the reading of the written eigenvalues that the
populations are built from; the reference leaves it to its analysis
scripts.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.linalg

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(_HERE))
sys.path.insert(0, _HERE)
from dirac_hydrogen_code_gb300.formats import csr_read  # noqa: E402
from oracle import SOL, ik  # noqa: E402


def _radial(workdir: str):
    h = [csr_read(os.path.join(workdir, f"h0{n}.csr")).to_scipy().toarray().real for n in range(4)]
    s = [csr_read(os.path.join(workdir, f"s{n}.csr")).to_scipy().toarray().real for n in range(3)]
    return h, s


def eigenpairs(workdir: str, kappamax: int):
    """{kappa: (evals, evecs)} for kappa = -1, 1, ..., -kappamax, kappamax
    (src/hamiltonian.h:913-958), with the sign convention of
    src/hamiltonian.h:960-983 applied column by column."""
    h, s = _radial(workdir)
    out = {}
    for kappa in range(1, kappamax + 1):
        for k in (-kappa, kappa):
            H0 = h[0] + k * h[1] + k * k * h[2] + k * k * k * h[3]
            S = s[0] + k * s[1] + k * k * s[2]
            evals, evecs = scipy.linalg.eigh(H0, S)
            for i in range(evecs.shape[1]):
                col = evecs[:, i]
                vv = max(abs(col.max()), abs(col.min()))
                j = 0
                while not abs(col[j] * 100) > vv:
                    j += 1
                if col[j] < 0:
                    evecs[:, i] = -col
            out[k] = (evals, evecs)
    return out


def psiev(workdir: str, x: np.ndarray, kappamax: int) -> tuple[list, list]:
    """The projections of a state x (solver order: block rows of H.csr, each
    blkdim radial coefficients) and the eigenvalues of each block's kappa:
    lists over block rows of psiev[th] = x_th^H [S v_j]_j and evl[th]
    (src/hamiltonian.h:1246-1300, 1333-1370)."""
    _, s = _radial(workdir)
    hall = csr_read(os.path.join(workdir, "H.csr"))
    pairs = eigenpairs(workdir, kappamax)
    B = s[0].shape[0]
    X = x.reshape(-1, B)
    projs, evls = [], []
    skev_cache = {}
    for th in range(X.shape[0]):
        k = ik(int(hall.perm[th]))
        evals, evecs = pairs[k]
        if k not in skev_cache:
            S = s[0] + k * s[1] + k * k * s[2]
            skev = np.empty((B, evecs.shape[1]))
            for j in range(evecs.shape[1]):
                skev[:, j] = S @ evecs[:, j]          # matfree<S> of eigenvector j
            skev_cache[k] = skev
        projs.append(X[th].conj() @ skev_cache[k])
        evls.append(evals)
    return projs, evls


def populations(workdir: str, x: np.ndarray, kappamax: int) -> dict:
    """Summed |psiev|^2 over the negative-energy (E < -c^2), bound
    (-c^2 <= E < 0) and continuum (E >= 0) eigenstates, and in total."""
    projs, evls = psiev(workdir, x, kappamax)
    out = {"negative": 0.0, "bound": 0.0, "continuum": 0.0, "norm": 0.0}
    for c, e in zip(projs, evls):
        p = np.abs(c) ** 2
        out["negative"] += float(p[e < -SOL * SOL].sum())
        out["bound"] += float(p[(e >= -SOL * SOL) & (e < 0)].sum())
        out["continuum"] += float(p[e >= 0].sum())
        out["norm"] += float(p.sum())
    return out
