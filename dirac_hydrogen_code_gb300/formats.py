"""Readers and writers for GaDE's binary file formats.

All formats are little-endian, native to the reference tools:

* ``*.csr`` — ``int32 n, int32 nnz, int32 Ap[n+1], int32 Ai[nnz],
  complex128 Ax[nnz]`` and, for ``H.csr`` only, a trailer
  ``int32 perm[n], int32 npart, int32 row_cpu_dist[npart+1]``
  (tools/csr.c:262-318 reads it, tools/main.py:158-171 writes it).
* ``psi0`` — ``int64 rows, int64 cols, complex128 data[rows*cols]``
  (src/dumpBdpCouplings.cpp:84-108, read by tools/main.py:42-48).
* ``psi0.vec`` — ``int32 n, complex128 psi[n], int32 perm[n]``
  (tools/main.py:151-155, read by tools/dirac_solver.c:68-108).
* ``x<step>.out`` — ``int32 nrows, int32 ncols=1, complex128 x[nrows]``
  (tools/dirac_solver.c:616-621).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

IDX = np.dtype("<i4")
CPLX = np.dtype("<c16")


@dataclasses.dataclass
class Csr:
    """A square CSR matrix as stored in a GaDE ``.csr`` file."""

    n: int
    Ap: np.ndarray
    Ai: np.ndarray
    Ax: np.ndarray
    perm: np.ndarray | None = None
    row_cpu_dist: np.ndarray | None = None

    @property
    def nnz(self) -> int:
        return int(self.Ap[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.Ax, self.Ai, self.Ap), shape=(self.n, self.n))

    @staticmethod
    def from_scipy(m, perm=None, row_cpu_dist=None) -> "Csr":
        m = m.tocsr()
        m.sort_indices()
        return Csr(m.shape[0], np.asarray(m.indptr, IDX), np.asarray(m.indices, IDX),
                   np.asarray(m.data, CPLX), perm, row_cpu_dist)


def csr_read(path: str | os.PathLike) -> Csr:
    """Read a ``.csr`` file; mirrors the checks of tools/csr.c:262-318."""
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 8:
        raise ValueError(f"wrong file format in {path}")
    n, nnz = np.frombuffer(raw, IDX, 2)
    n, nnz = int(n), int(nnz)
    off = 8
    need = off + 4 * (n + 1) + 4 * nnz + 16 * nnz
    if n < 0 or nnz < 0 or len(raw) < need:
        raise ValueError(f"wrong file format in {path}")
    Ap = np.frombuffer(raw, IDX, n + 1, off).copy(); off += 4 * (n + 1)
    if Ap[n] != nnz:
        raise ValueError(f"wrong file format (nnz) in {path}: nrows {n} nnz {nnz} Ap {Ap[n]}")
    Ai = np.frombuffer(raw, IDX, nnz, off).copy(); off += 4 * nnz
    Ax = np.frombuffer(raw, CPLX, nnz, off).copy(); off += 16 * nnz
    perm = dist = None
    if len(raw) >= off + 4 * n and n > 0:
        perm = np.frombuffer(raw, IDX, n, off).copy(); off += 4 * n
        if len(raw) < off + 4:
            raise ValueError(f"wrong file format in {path}: partitioning info not found")
        npart = int(np.frombuffer(raw, IDX, 1, off)[0]); off += 4
        if npart < 1 or len(raw) < off + 4 * (npart + 1):
            raise ValueError(f"wrong file format in {path}: partitioning info inconsistent")
        dist = np.frombuffer(raw, IDX, npart + 1, off).copy()
    return Csr(n, Ap, Ai, Ax, perm, dist)


def csr_write(path: str | os.PathLike, m: Csr) -> None:
    """Write a ``.csr`` file (with the partition trailer when ``m.perm`` is set)."""
    with open(path, "wb") as f:
        np.array([m.n, m.nnz], IDX).tofile(f)
        np.asarray(m.Ap, IDX).tofile(f)
        np.asarray(m.Ai, IDX).tofile(f)
        np.asarray(m.Ax, CPLX).tofile(f)
        if m.perm is not None:
            np.asarray(m.perm, IDX).tofile(f)
            dist = m.row_cpu_dist if m.row_cpu_dist is not None else np.array([0, m.n], IDX)
            np.array([len(dist) - 1], IDX).tofile(f)
            np.asarray(dist, IDX).tofile(f)


def dense_write(path, v: np.ndarray) -> None:
    """Write ``psi0``: int64 rows, int64 cols, complex128 column-major data."""
    v = np.asarray(v, CPLX)
    if v.ndim == 1:
        v = v[:, None]
    with open(path, "wb") as f:
        np.array(v.shape, "<i8").tofile(f)
        np.asfortranarray(v).T.tofile(f)


def dense_read(path) -> np.ndarray:
    with open(path, "rb") as f:
        rows, cols = np.fromfile(f, "<i8", 2)
        data = np.fromfile(f, CPLX, int(rows) * int(cols))
    return data


def vec_write(path, psi: np.ndarray, perm: np.ndarray) -> None:
    """Write ``psi0.vec``: int32 n, complex128 psi[n], int32 perm[n]."""
    with open(path, "wb") as f:
        np.array([len(psi)], IDX).tofile(f)
        np.asarray(psi, CPLX).tofile(f)
        np.asarray(perm, IDX).tofile(f)


def vec_read(path) -> tuple[np.ndarray, np.ndarray]:
    """Read ``psi0.vec`` -> (psi, perm); tools/dirac_solver.c:68-108."""
    with open(path, "rb") as f:
        raw = f.read()
    n = int(np.frombuffer(raw, IDX, 1)[0])
    if n < 0 or len(raw) < 4 + 16 * n + 4 * n:
        raise ValueError(f"wrong file format in {path}")
    psi = np.frombuffer(raw, CPLX, n, 4).copy()
    perm = np.frombuffer(raw, IDX, n, 4 + 16 * n).copy()
    return psi, perm


def out_write(path, x: np.ndarray) -> None:
    """Write ``x<step>.out``: int32 nrows, int32 ncols=1, complex128 x."""
    with open(path, "wb") as f:
        np.array([len(x), 1], IDX).tofile(f)
        np.asarray(x, CPLX).tofile(f)


def out_read(path) -> np.ndarray:
    with open(path, "rb") as f:
        nrows, ncols = np.fromfile(f, IDX, 2)
        return np.fromfile(f, CPLX, int(nrows) * int(ncols))
