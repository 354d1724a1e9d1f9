"""GPU: eigenstate projection (populations) against the oracle restatement
of the reference's dumpEigvals + processOutput (oracle/populations.py) and
against the host path, and a drop-in run restarted from its own
x<iter>.out against an uninterrupted run."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from dirac_hydrogen_code_gb300 import build, formats
from dirac_hydrogen_code_gb300.cn import run_batch, step_times
from dirac_hydrogen_code_gb300.native import Problem
from dirac_hydrogen_code_gb300.populations import Eigenbasis

pytestmark = pytest.mark.gpu


def test_device_projection_matches_oracle(workdirs, native_lib):
    """gade_eigproj on batched pulse states: every block's projections on
    the eigenstates of its kappa and the class populations, against the
    oracle (src/hamiltonian.h:872-983, 1246-1300)."""
    import populations as OP
    import torch
    from dirac_hydrogen_code_gb300 import native
    from dirac_hydrogen_code_gb300.populations import E_NEG
    d, params, info = workdirs["tiny_nondipole"]
    prob = Problem(d, info["lmax"])
    kap, _ = prob.blocks()
    kmax = int(np.abs(kap).max())
    eb = Eigenbasis(d, kap)
    pulses = [dict(E0=e, omega=params["Omega"], cycles=params["Cycles"], ntime=params["Ntime"]) for e in (5.0, 60.0)]
    xs, _, b = run_batch(prob, pulses, None, tol=1e-12)
    xptr, ld = b.state_device()
    nblk, B = len(kap), eb.B
    W = torch.from_numpy(eb.W).cuda()
    E = torch.from_numpy(eb.evals).cuda()
    kidx = torch.from_numpy(eb.block_kidx).cuda()
    coef = torch.empty(len(pulses), nblk, B, dtype=torch.complex128, device="cuda")
    cls = torch.empty(len(pulses), nblk, 4, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    native.call("gade_eigproj", len(pulses), nblk, B, kidx.data_ptr(), W.data_ptr(), E.data_ptr(), E_NEG,
                int(xptr), int(ld), coef.data_ptr(), cls.data_ptr(), 0)
    torch.cuda.synchronize()
    coef, cls = coef.cpu().numpy(), cls.cpu().numpy()
    for k in range(len(pulses)):
        projs, evls = OP.psiev(d, xs[k], kmax)
        scale = np.abs(coef[k]).max()
        for r in range(nblk):
            assert np.abs(coef[k][r] - projs[r]).max() <= 1e-12 * scale, (k, r)
        ref = OP.populations(d, xs[k], kmax)
        tot = cls[k].sum(0)
        for j, key in enumerate(("negative", "bound", "continuum", "norm")):
            assert abs(tot[j] - ref[key]) <= 1e-12 * ref["norm"], key
    assert OP.populations(d, xs[1], kmax)["continuum"] > OP.populations(d, xs[0], kmax)["continuum"]


def test_device_populations_match_host(workdirs, native_lib):
    d, params, info = workdirs["tiny_nondipole"]
    prob = Problem(d, info["lmax"])
    kap, _ = prob.blocks()
    eb = Eigenbasis(d, kap)
    pulses = [dict(E0=e, omega=params["Omega"], cycles=params["Cycles"], ntime=params["Ntime"]) for e in (5.0, 60.0)]
    xs, _, b = run_batch(prob, pulses, None, tol=1e-12)
    xptr, ld = b.state_device()
    dev = eb.populations_device(xptr, ld, len(pulses))
    for k in range(len(pulses)):
        host = eb.populations(xs[k])
        for key in ("negative", "bound", "continuum", "norm"):
            assert abs(dev[k][key] - host[key]) <= 1e-12 * max(host["norm"], 1e-300) + 1e-300, key
        assert host["continuum"] > 0 and abs(host["norm"] - 1.0) < 1e-6
    assert dev[1]["continuum"] > dev[0]["continuum"]      # a stronger pulse ionises more


def test_restart_continues_the_run(workdirs, native_lib, tmp_path):
    d, params, info = workdirs["tiny_dipole"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    n = params["Ntime"]
    exe = build.solver_path()
    base = [exe, "-l", str(info["lmax"]), "-i", str(params["Intensity"]), "-o", str(params["Omega"]),
            "-c", str(params["Cycles"]), "--tol", "1e-12", "--final-dump"]
    full, half = str(tmp_path / "full"), str(tmp_path / "half")
    shutil.copytree(d, full)
    shutil.copytree(d, half)
    r = subprocess.run(base + ["-t", repr(T), "-n", str(n)], cwd=full, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    nfull = len(step_times(T, n)[1])
    # first half: the same dt (T/2 over n/2 steps), then continue with -s
    r = subprocess.run(base + ["-t", repr(T / 2), "-n", str(n // 2)], cwd=half, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    nhalf = len(step_times(T / 2, n // 2)[1])
    r = subprocess.run(base + ["-t", repr(T), "-n", str(n), "-s", str(nhalf + 1), "--restart", f"x{nhalf}.out"],
                       cwd=half, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    xa = formats.out_read(os.path.join(full, f"x{nfull}.out"))
    xb = formats.out_read(os.path.join(half, f"x{nfull}.out"))
    assert np.linalg.norm(xa - xb) / np.linalg.norm(xa) < 1e-10
