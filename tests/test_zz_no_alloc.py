"""The allocation-free entry point gade_solver_apply_dot_noalloc.

It serves callers that may not allocate device memory while running (a
framework owning all GPU memory through its own pool, or a pipelined loop
that cannot afford cudaMalloc's implicit synchronisation).  Its reduction
scratch is a fixed array inside the library.  Checked through the C ABI
against the existing entry point (gade_solver_apply_device) and a host dot
product, on two calls in a row so that the shared scratch is reused.
This file is collected last on purpose.
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_apply_dot_noalloc_matches_existing_entry_point(tmp_path):
    import torch
    from dirac_hydrogen_code_gb300 import build, native
    from dirac_hydrogen_code_gb300.cn import pulse
    from dirac_hydrogen_code_gb300.gen import generate

    if not os.path.exists(build.library_path()):
        build.build()
    params = dict(Nsplines=24, Ntime=60, Nkappa=3, Nmu=2, Nl=0, rBox=30.0,
                  Intensity=10, Omega=50.0, Cycles=2, Z=1)
    info = generate(params, str(tmp_path))
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    prob = native.Problem(str(tmp_path), info["lmax"])
    sol = native.Solver(prob, T / params["Ntime"])
    sol.set_time(pulse(params["Intensity"], params["Omega"], params["Cycles"], 0.3 * T))
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
