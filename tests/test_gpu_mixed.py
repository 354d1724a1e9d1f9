"""Mixed precision (GADE_PREC_MIXED): complex64 inner BiCGSTAB inside FP64
iterative refinement.  Whole pulses against the FP64 path; the stated error
is the relative S-norm (physical L2 norm of the wavefunction) and the
relative L2 norm of the coefficient vector."""
import math

import numpy as np
import pytest

import oracle as O
from dirac_hydrogen_code_gb300.cn import run

pytestmark = pytest.mark.gpu


def _errors(p, x, xref):
    S, _ = O.stationary(p, 0.0)
    e = x - xref
    s_err = math.sqrt(abs(np.vdot(e, S @ e).real) / abs(np.vdot(xref, S @ xref).real))
    return s_err, float(np.linalg.norm(e) / np.linalg.norm(xref))


@pytest.mark.parametrize("name", ["tiny_nondipole", "dipole_small"])
def test_mixed_whole_pulse(workdirs, native_lib, name):
    d, params, info = workdirs[name]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    x64, r64, _ = run(*args, tol=1e-12, write_outputs=False)
    xm, rm, _ = run(*args, tol=1e-10, precision="mixed", write_outputs=False)
    p = O.load_problem(d, info["lmax"])
    s_err, l2_err = _errors(p, xm, x64)
    assert s_err <= 1e-8, s_err
    assert l2_err <= 1e-6, l2_err
    assert all(r["true_residual"] <= 1e-10 for r in rm)
    assert sum(r["refinements"] for r in rm) >= len(rm)            # at least one FP64 residual per step
    # norm conservation check (FP64 x^H S x before every step)
    sn = np.array([r["snorm"] for r in rm])
    assert np.all(np.abs(sn - sn[0]) < 1e-7)


def test_mixed_matches_fp64_tight_tolerance(workdirs, native_lib):
    d, params, info = workdirs["tiny_dipole"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    x64, _, _ = run(*args, tol=1e-12, write_outputs=False)
    xm, rm, _ = run(*args, tol=1e-12, precision="mixed", write_outputs=False)
    p = O.load_problem(d, info["lmax"])
    s_err, l2_err = _errors(p, xm, x64)
    assert s_err <= 1e-11 and l2_err <= 1e-10, (s_err, l2_err)
