"""Cases of the golden fixtures (tests/golden/*.npz) produced by the reference
CPU build; shared by make_golden.py and the tests."""
import os

import numpy as np

from dirac_hydrogen_code_gb300.formats import csr_read

TINY_DIPOLE = dict(Nsplines=20, Ntime=40, Nkappa=2, Nmu=0, Nl=1, rBox=30.0,
                   Intensity=10, Omega=50.0, Cycles=1, Z=1)
TINY_NONDIPOLE = dict(Nsplines=24, Ntime=60, Nkappa=3, Nmu=2, Nl=0, rBox=30.0,
                      Intensity=10, Omega=50.0, Cycles=2, Z=1)
DIPOLE_SMALL = dict(Nsplines=100, Ntime=500, Nkappa=4, Nmu=0, Nl=1, rBox=30.0,
                    Intensity=10, Omega=50.0, Cycles=1, Z=1)
NONDIPOLE_MEDIUM = dict(Nsplines=250, Ntime=1500, Nkappa=8, Nmu=4, Nl=0, rBox=30.0,
                        Intensity=10, Omega=50.0, Cycles=3, Z=1)

CASES = {
    "tiny_dipole": dict(params=TINY_DIPOLE, tol=1e-12, maxit=500),
    "tiny_nondipole": dict(params=TINY_NONDIPOLE, tol=1e-12, maxit=500),
    # the reference's hard-coded tolerance and cap (tools/dirac_solver.c:506-507)
    "tiny_dipole_tol16": dict(params=TINY_DIPOLE, tol=1e-16, maxit=500, max_steps=12),
    "dipole_small": dict(params=DIPOLE_SMALL, tol=1e-12, maxit=500),
    "nondipole_medium_20": dict(params=NONDIPOLE_MEDIUM, tol=1e-12, maxit=500, max_steps=20, sample=True),
}


def fingerprint(workdir: str, lmax: int) -> np.ndarray:
    """L1 norms of the radial and angular inputs, to detect a generator drift."""
    vals = []
    for name in ["s0.csr", "s2.csr", "h00.csr", "h03.csr", "g0a0l0.csr", "g3a5l0.csr",
                 f"H0l{lmax - 1}.csr", f"H1l{lmax - 1}.csr"]:
        m = csr_read(os.path.join(workdir, name))
        vals.append(np.abs(m.Ax).sum())
    return np.array(vals)
