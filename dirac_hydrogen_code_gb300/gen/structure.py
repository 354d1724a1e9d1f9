"""Single-partition restatement of tools/main.py:50-171.

Builds the block coupling pattern ``H.csr`` (pattern of sum_l H0l + H1l with
the empty rows/columns removed, plus the identity) and the permuted initial
state ``psi0.vec``.  METIS partitioning (tools/main.py:85-112) is multi-rank
only and is not restated: one GPU runs the whole problem.
"""
from __future__ import annotations

import glob
import os

import numpy as np
import scipy.sparse as sp

from ..formats import Csr, csr_read, csr_write, dense_read, vec_write


def build_structure(workdir: str) -> dict:
    n_l = len(glob.glob(os.path.join(workdir, "H0l*.csr")))
    if n_l == 0:
        raise FileNotFoundError("Did not find any H*csr files")
    res = None
    for l in range(n_l):
        for kind in ("H0l", "H1l"):
            m = csr_read(os.path.join(workdir, f"{kind}{l}.csr")).to_scipy()
            res = m if res is None else res + m
    # non-empty columns of the summed pattern (tools/main.py:73); the
    # structure is symmetric so rows and columns coincide
    colsum = np.asarray(res.sum(axis=0)).ravel()
    nzc = np.nonzero(colsum)[0].astype(np.int32)
    res_full = res + sp.identity(res.shape[0], format="csr")
    hall = res_full[nzc[:, None], nzc].tocsr()
    hall.sort_indices()
    nblk = len(nzc)

    g0 = csr_read(os.path.join(workdir, "g0a0l0.csr"))
    blkdim = g0.n
    psi_full = dense_read(os.path.join(workdir, "psi0"))
    # tools/main.py:141-147: the block permutation of a single partition is
    # the identity, so psi0.vec holds the first nblk*blkdim entries
    perm = np.arange(nblk * blkdim, dtype=np.int32)
    psi0 = psi_full[perm]
    vec_write(os.path.join(workdir, "psi0.vec"), psi0, perm)

    out = Csr(nblk, hall.indptr.astype(np.int32), hall.indices.astype(np.int32),
              hall.data.astype(complex), perm=nzc, row_cpu_dist=np.array([0, nblk], np.int32))
    csr_write(os.path.join(workdir, "H.csr"), out)
    return dict(nblk=nblk, hall_nnz=int(hall.nnz), blkdim=blkdim, lmax=n_l,
                n=nblk * blkdim, nnz_full=int(hall.nnz) * int(g0.nnz))
