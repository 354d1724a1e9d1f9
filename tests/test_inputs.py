"""CPU tests: file formats, the input generator, structure step and the
oracle's internal consistency."""
import math
import os

import numpy as np
import pytest

from dirac_hydrogen_code_gb300 import formats
from dirac_hydrogen_code_gb300.gen import couplings


def test_csr_roundtrip(tmp_path):
    import scipy.sparse as sp
    m = sp.random(7, 7, density=0.4, random_state=1, format="csr") * (1 + 2j)
    c = formats.Csr.from_scipy(m)
    formats.csr_write(tmp_path / "a.csr", c)
    r = formats.csr_read(tmp_path / "a.csr")
    assert r.perm is None
    assert np.array_equal(r.Ap, c.Ap) and np.array_equal(r.Ai, c.Ai) and np.array_equal(r.Ax, c.Ax)
    c.perm = np.arange(7, dtype=np.int32)[::-1].copy()
    formats.csr_write(tmp_path / "b.csr", c)
    r = formats.csr_read(tmp_path / "b.csr")
    assert np.array_equal(r.perm, c.perm) and list(r.row_cpu_dist) == [0, 7]


def test_csr_read_rejects_bad_nnz(tmp_path):
    with open(tmp_path / "bad.csr", "wb") as f:
        np.array([2, 3], "<i4").tofile(f)
        np.array([0, 1, 2], "<i4").tofile(f)     # Ap[n] != nnz
        np.array([0, 1, 1], "<i4").tofile(f)
        np.zeros(3, "<c16").tofile(f)
    with pytest.raises(ValueError, match="nnz"):
        formats.csr_read(tmp_path / "bad.csr")


def test_vec_and_out_roundtrip(tmp_path):
    psi = np.arange(6) * (1 - 1j)
    perm = np.array([5, 4, 3, 2, 1, 0], np.int32)
    formats.vec_write(tmp_path / "p.vec", psi, perm)
    a, b = formats.vec_read(tmp_path / "p.vec")
    assert np.array_equal(a, psi) and np.array_equal(b, perm)
    formats.out_write(tmp_path / "x.out", psi)
    assert np.array_equal(formats.out_read(tmp_path / "x.out"), psi)


def test_kappa_mu_maps():
    # |kappa|=1: i=0,1 -> -1 ; i=2,3 -> +1 ; |kappa|=2 spans 8 states
    assert [couplings.ik(i) for i in range(12)] == [-1, -1, 1, 1, -2, -2, -2, -2, 2, 2, 2, 2]
    assert [couplings.imu(i) for i in range(4)] == [-0.5, 0.5, -0.5, 0.5]
    assert couplings.n_angular(4) == 40 and couplings.n_angular(1) == 4


def test_wigner3j_known_values():
    w = couplings.wigner3j
    assert w(1, 1, 0, 0, 0, 0) == pytest.approx(-1 / math.sqrt(3), abs=1e-15)
    assert w(1, 1, 2, 0, 0, 0) == pytest.approx(math.sqrt(2 / 15), abs=1e-15)
    assert w(2, 2, 2, 1, -1, 0) == pytest.approx(math.sqrt(1 / 70), abs=1e-15)
    assert w(1, 1, 1, 0, 0, 0) == 0.0            # odd j-sum with m=0
    assert w(1, 1, 3, 0, 0, 0) == 0.0            # triangle rule


def test_generator_physics(workdirs):
    d, params, info = workdirs["dipole_small"]
    # relativistic 1s energy of hydrogen (src/dumpBdpCouplings.cpp:310-320)
    assert info["e0"] == pytest.approx(-0.500006656, abs=2e-8)
    assert (info["nblk"], info["blkdim"], info["blk_nnz"], info["hall_nnz"]) == (40, 210, 6076, 200)
    s0 = formats.csr_read(os.path.join(d, "s0.csr"))
    g = formats.csr_read(os.path.join(d, "g1a4l0.csr"))
    assert np.array_equal(s0.Ap, g.Ap) and np.array_equal(s0.Ai, g.Ai)    # shared base pattern
    assert np.all(g.Ax.imag == 0)                                        # radial couplings real
    h = formats.csr_read(os.path.join(d, "H0l0.csr"))
    assert np.all(h.Ax.real == 0) and np.all(h.Ax.imag != 0)             # angular couplings imaginary
    hall = formats.csr_read(os.path.join(d, "H.csr"))
    assert hall.perm is not None and list(hall.row_cpu_dist) == [0, hall.n]
    psi, perm = formats.vec_read(os.path.join(d, "psi0.vec"))
    assert np.array_equal(perm, np.arange(len(psi)))


def test_generator_sizes_nondipole(workdirs):
    d, params, info = workdirs["tiny_nondipole"]
    assert info["lmax"] == 2 * params["Nkappa"] + 1                    # Nl=0 -> 2*Nkappa+1
    for l in range(info["lmax"]):
        for kind in ("H0l", "H1l"):
            assert os.path.exists(os.path.join(d, f"{kind}{l}.csr"))
    assert info["nblk"] < couplings.n_angular(params["Nkappa"])        # |mu| >= Nmu removed


def test_oracle_stationary_symmetric(workdirs):
    import oracle as O
    d, params, info = workdirs["tiny_nondipole"]
    p = O.load_problem(d, info["lmax"])
    S, H = O.stationary(p, 0.01)
    P = (S + H).tocsr()
    assert abs(P - P.T).max() < 1e-12 * abs(P).max()


def test_oracle_preconditioners_agree(workdirs):
    """ILU(1e-6) of the reference and the exact block LU give the same
    iteration counts and final state to roundoff on the small dipole case."""
    import oracle as O
    d, params, info = workdirs["tiny_dipole"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    p = O.load_problem(d, info["lmax"])
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    x1, r1, _ = O.run(*args, tol=1e-12, precond="ilu", problem=p)
    x2, r2, _ = O.run(*args, tol=1e-12, precond="blocklu", problem=p)
    assert [r.iters for r in r1] == [r.iters for r in r2]
    assert np.linalg.norm(x1 - x2) / np.linalg.norm(x1) < 1e-12
    assert len(r1) in (params["Ntime"], params["Ntime"] + 1)
