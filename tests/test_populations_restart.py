"""CPU tests of the populations (eigenstate projection, host side) and of
the restart converters between x<iter>.out and psi0.vec."""
import json
import os
import subprocess
import sys

import numpy as np

from dirac_hydrogen_code_gb300 import formats
from dirac_hydrogen_code_gb300.populations import Eigenbasis
from dirac_hydrogen_code_gb300.restart import out_to_vec, vec_to_out

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _basis(workdirs, name):
    from dirac_hydrogen_code_gb300.native import Problem
    d, params, info = workdirs[name]
    prob = Problem(d, info["lmax"])
    kap, ang = prob.blocks()
    return d, info, prob, Eigenbasis(d, kap), kap


def test_blocks_follow_angular_indices(workdirs, native_lib):
    from dirac_hydrogen_code_gb300.gen.couplings import ik
    d, info, prob, eb, kap = _basis(workdirs, "tiny_nondipole")
    perm = formats.csr_read(os.path.join(d, "H.csr")).perm
    assert kap.tolist() == [ik(int(i)) for i in perm]


def test_ground_state_is_bound(workdirs, native_lib):
    d, info, prob, eb, kap = _basis(workdirs, "dipole_small")
    psi, _ = prob.psi0()
    pop = eb.populations(psi)
    assert abs(pop["bound"] - 1.0) < 1e-10 and pop["continuum"] < 1e-12 and pop["negative"] < 1e-12
    # the population sits in the 1s state: eigenvalue -0.5000067 of kappa = -1
    c = eb.project(psi)
    r = int(np.argmax(np.abs(c).max(1)))
    j = int(np.argmax(np.abs(c[r])))
    assert kap[r] == -1 and abs(eb.evals[eb.block_kidx[r], j] + 0.5000067) < 1e-6


def test_projection_is_complete(workdirs, native_lib):
    """sum_j |c_j|^2 = x_r^H S(k_r) x_r for any state (S-orthonormal eigenvectors)."""
    import oracle as O
    d, info, prob, eb, kap = _basis(workdirs, "tiny_nondipole")
    rng = np.random.default_rng(4)
    x = rng.standard_normal(prob.n) + 1j * rng.standard_normal(prob.n)
    cls = eb.classes(eb.project(x))
    p = O.load_problem(d, info["lmax"])
    S, _ = O.stationary(p, 0.0)
    X = x.reshape(-1, eb.B)
    Sx = (S @ x).reshape(-1, eb.B)
    assert np.allclose(cls[:, 3], np.einsum("ri,ri->r", X.conj(), Sx).real, rtol=1e-10)
    assert np.allclose(cls[:, :3].sum(1), cls[:, 3], rtol=1e-12)
    # the spectrum has all three classes
    assert eb.evals.min() < -2e4 and eb.evals.max() > 0 and ((eb.evals < 0) & (eb.evals > -2e4)).any()


def test_host_populations_match_oracle(workdirs, native_lib):
    """The product's host projection against the oracle restatement of the
    reference's dumpEigvals + processOutput (oracle/populations.py), on the
    ground state and on a seeded random state: every block's projections
    and the class populations."""
    import populations as OP
    d, info, prob, eb, kap = _basis(workdirs, "tiny_nondipole")
    kmax = int(np.abs(kap).max())
    rng = np.random.default_rng(12)
    psi, _ = prob.psi0()
    for x in (psi, rng.standard_normal(prob.n) + 1j * rng.standard_normal(prob.n)):
        c = eb.project(x)
        projs, evls = OP.psiev(d, x, kmax)
        scale = max(np.abs(c).max(), 1e-300)
        for r in range(len(projs)):
            assert np.abs(c[r] - projs[r]).max() <= 1e-12 * scale, r
            assert np.array_equal(eb.evals[eb.block_kidx[r]], evls[r])
        ref = OP.populations(d, x, kmax)
        got = eb.populations(x)
        for key in ref:
            assert abs(got[key] - ref[key]) <= 1e-12 * ref["norm"], key


def test_populations_cli(workdirs, native_lib, tmp_path):
    d, info, prob, eb, kap = _basis(workdirs, "tiny_dipole")
    psi, perm = prob.psi0()
    f = str(tmp_path / "x7.out")
    formats.out_write(f, vec_to_out(psi, perm))
    res = subprocess.run([sys.executable, "-m", "dirac_hydrogen_code_gb300.populations", d, str(info["lmax"]), f],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    pop = json.loads(res.stdout.strip().splitlines()[-1])
    assert abs(pop["bound"] - eb.populations(psi)["bound"]) < 1e-14


def test_restart_round_trip(tmp_path):
    rng = np.random.default_rng(8)
    n = 500
    perm = rng.permutation(n).astype(np.int32)
    psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    xorig = vec_to_out(psi, perm)
    assert np.array_equal(xorig[perm], psi)
    assert np.array_equal(out_to_vec(xorig, perm), psi)
    # CLI: psi0.vec -> x.out -> psi0.vec
    v0, o, v1 = (str(tmp_path / f) for f in ("a.vec", "x.out", "b.vec"))
    formats.vec_write(v0, psi, perm)
    m = [sys.executable, "-m", "dirac_hydrogen_code_gb300.restart"]
    assert subprocess.run(m + ["to-out", v0, "-o", o], cwd=ROOT).returncode == 0
    assert subprocess.run(m + ["to-vec", o, "--perm", v0, "-o", v1], cwd=ROOT).returncode == 0
    psi1, perm1 = formats.vec_read(v1)
    assert np.array_equal(psi1, psi) and np.array_equal(perm1, perm)
    assert np.array_equal(formats.out_read(o), xorig)
