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
NONDIPOLE_LARGE = dict(Nsplines=300, Ntime=4000, Nkappa=16, Nmu=8, Nl=10, rBox=30.0,
                       Intensity=10, Omega=50.0, Cycles=5, Z=1)

# Rows of the random sketch of a state: a seeded complex Gaussian matrix R
# scaled so that E|R e|^2 = |e|^2; |R (x - x_ref)| estimates |x - x_ref|
# (relative spread ~1/sqrt(2 SKETCH_ROWS)) from SKETCH_ROWS numbers.
SKETCH_ROWS = 64
SKETCH_SEED = 777

CASES = {
    "tiny_dipole": dict(params=TINY_DIPOLE, tol=1e-12, maxit=500),
    "tiny_nondipole": dict(params=TINY_NONDIPOLE, tol=1e-12, maxit=500),
    # the reference's hard-coded tolerance and cap (tools/dirac_solver.c:506-507)
    "tiny_dipole_tol16": dict(params=TINY_DIPOLE, tol=1e-16, maxit=500, max_steps=12),
    "dipole_small": dict(params=DIPOLE_SMALL, tol=1e-12, maxit=500),
    "nondipole_medium_20": dict(params=NONDIPOLE_MEDIUM, tol=1e-12, maxit=500, max_steps=20, sample=True),
    # the whole 1500-step pulse of the nondipole medium configuration: final
    # state entire, a sketch of the state every 150 steps
    "nondipole_medium_full": dict(params=NONDIPOLE_MEDIUM, tol=1e-12, maxit=500, snap_every=150),
    # the first 20 steps of the NKappa=16 configuration (N = 244,000): sketches
    # every 5 steps and of the final state
    "nondipole_large_20": dict(params=NONDIPOLE_LARGE, tol=1e-12, maxit=500, max_steps=20, snap_every=5,
                               sketch_only=True),
}


def sketch(x: np.ndarray) -> np.ndarray:
    """R x for the seeded sketch matrix R (SKETCH_ROWS x len(x)), generated
    row by row so that large states need no dense R."""
    rng = np.random.default_rng(SKETCH_SEED)
    out = np.empty(SKETCH_ROWS, np.complex128)
    scale = 1.0 / np.sqrt(2.0 * SKETCH_ROWS)
    for k in range(SKETCH_ROWS):
        r = rng.standard_normal(len(x)) + 1j * rng.standard_normal(len(x))
        out[k] = scale * (r @ x)
    return out


def fingerprint(workdir: str, lmax: int) -> np.ndarray:
    """L1 norms of the radial and angular inputs, to detect a generator drift."""
    vals = []
    for name in ["s0.csr", "s2.csr", "h00.csr", "h03.csr", "g0a0l0.csr", "g3a5l0.csr",
                 f"H0l{lmax - 1}.csr", f"H1l{lmax - 1}.csr"]:
        m = csr_read(os.path.join(workdir, name))
        vals.append(np.abs(m.Ax).sum())
    return np.array(vals)
