"""The allocation-free entry point gade_solver_apply_dot_noalloc.

It serves callers that may not allocate device memory while running (a
framework owning all GPU memory through its own pool, or a pipelined loop
that cannot afford cudaMalloc's implicit synchronisation).  Its reduction
scratch is a fixed array inside the library.  Checked through the C ABI
against the existing entry point (gade_solver_apply_device) and a host dot
product, on two calls in a row so that the shared scratch is reused, with
each of the two operators (matrix-free and assembled) forced; a problem
with more work units than the fixed array holds is rejected.
This file is collected last on purpose.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_MAX_UNITS = 16384        # reduction slots of the library's fixed scratch array


@pytest.mark.parametrize("op", [0, 1])
def test_apply_dot_noalloc_matches_existing_entry_point(tmp_path, op):
    import torch
    from dirac_hydrogen_code_gb300 import build, native
    from dirac_hydrogen_code_gb300.cn import pulse
    from dirac_hydrogen_code_gb300.gen import generate

    if build.is_stale():
        build.build()
    params = dict(Nsplines=24, Ntime=60, Nkappa=3, Nmu=2, Nl=0, rBox=30.0,
                  Intensity=10, Omega=50.0, Cycles=2, Z=1)
    info = generate(params, str(tmp_path))
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    prob = native.Problem(str(tmp_path), info["lmax"])
    sol = native.Solver(prob, T / params["Ntime"])
    sol.set_operator(op)
    sol.set_time(pulse(params["Intensity"], params["Omega"], params["Cycles"], 0.3 * T))
    assert sol.operator()["assembled"] == op
    n = prob.n
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(5)
    for call in range(2):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        r0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        xt = torch.from_numpy(x).to(dev)
        r0t = torch.from_numpy(r0).to(dev)
        y_ref = torch.empty_like(xt)
        y_new = torch.empty_like(xt)
        dot = torch.zeros(2, dtype=torch.float64, device=dev)
        sol.apply_device(xt.data_ptr(), y_ref.data_ptr(), stream)
        sol.apply_dot_noalloc(xt.data_ptr(), r0t.data_ptr(), y_new.data_ptr(), dot.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        yr, yn = y_ref.cpu().numpy(), y_new.cpu().numpy()
        assert np.linalg.norm(yn - yr) / np.linalg.norm(yr) <= 1e-13, f"call {call}"
        d = complex(*dot.cpu().numpy())
        d_ref = np.vdot(r0, yr)
        assert abs(d - d_ref) / abs(d_ref) <= 1e-12, f"call {call}"
    with pytest.raises(native.GadeError) as e:
        sol.apply_dot_noalloc(0, 0, 0, 0, stream)
    assert e.value.code == 4


def _many_block_problem(workdir: str, nang: int):
    """A valid problem with `nang` angular blocks: the radial files of a
    small generated dipole problem and synthetic angular couplings (purely
    imaginary, nearest-neighbour, one Bessel order), so that the block count
    exceeds the fixed scratch array without the cost of the generator's
    angular tables."""
    import scipy.sparse as sp
    from dirac_hydrogen_code_gb300.formats import Csr, csr_write, dense_write
    from dirac_hydrogen_code_gb300.gen import generate
    from dirac_hydrogen_code_gb300.gen.structure import build_structure
    params = dict(Nsplines=20, Ntime=40, Nkappa=2, Nmu=0, Nl=1, rBox=30.0,
                  Intensity=10, Omega=50.0, Cycles=1, Z=1)
    info = generate(params, workdir)
    i = np.arange(nang - 1)
    vals = 1j * (0.1 + 0.01 * (i % 7))
    h = sp.coo_matrix((np.r_[vals, vals], (np.r_[i, i + 1], np.r_[i + 1, i])), shape=(nang, nang)).tocsr()
    h.sort_indices()
    for kind in ("H0l0", "H1l0"):
        csr_write(os.path.join(workdir, f"{kind}.csr"), Csr.from_scipy(h))
    psi = np.zeros((info["blkdim"], nang), complex)
    psi[:, 0] = 1.0 / math.sqrt(info["blkdim"])
    dense_write(os.path.join(workdir, "psi0"), psi.reshape(-1, order="F"))
    build_structure(workdir)
    return info["lmax"]


def test_apply_dot_noalloc_rejects_problems_beyond_its_scratch(tmp_path):
    import torch
    from dirac_hydrogen_code_gb300 import build, native
    from dirac_hydrogen_code_gb300.cn import pulse

    if build.is_stale():
        build.build()
    nang = NOALLOC_MAX_UNITS + 360
    lmax = _many_block_problem(str(tmp_path), nang)
    prob = native.Problem(str(tmp_path), lmax)
    assert prob.info["nblk"] > NOALLOC_MAX_UNITS
    sol = native.Solver(prob, 1e-3)
    sol.set_time(pulse(10.0, 50.0, 1.0, 0.01))
    dev = torch.device("cuda:0")
    x = torch.zeros(prob.n, dtype=torch.complex128, device=dev)
    y = torch.empty_like(x)
    dot = torch.zeros(2, dtype=torch.float64, device=dev)
    with pytest.raises(native.GadeError) as e:
        sol.apply_dot_noalloc(x.data_ptr(), x.data_ptr(), y.data_ptr(), dot.data_ptr())
    assert e.value.code == 4 and "16384" in str(e.value)
    # the allocating entry point serves the same problem
    sol.apply_device(x.data_ptr(), y.data_ptr())
    torch.cuda.synchronize(dev)
    assert float(y.abs().max()) == 0.0
