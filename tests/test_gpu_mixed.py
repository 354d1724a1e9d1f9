"""Mixed precision (GADE_PREC_MIXED): complex64 inner BiCGSTAB inside FP64
iterative refinement, over whole pulses, against the reference CPU build
(the golden fixtures of tests/golden/, made by tools/ compiled in place).

The bound is the relative L2 error of the final wavefunction, <= 1e-8, with
the refinement tolerance 1e-12, the tolerance of the plain FP64 runs.  The
tolerance, not the precision, sets the error: over the whole 1500-step pulse
of the nondipole medium configuration a residual bound of 1e-10 leaves
2.0e-8 in plain FP64 and 1.6e-8 in mixed precision, and 1e-11 still 1.5e-8
(the residual of every step, times the operator's inverse, accumulates).  At
the equal residual 1e-10 the mixed path is checked to be no less accurate
than the plain FP64 path.
"""
import math
import os

import numpy as np
import pytest

from dirac_hydrogen_code_gb300.cn import run
from dirac_hydrogen_code_gb300.gen import generate
from tests.golden.cases import CASES, sketch

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MIXED_TOL = 1e-12          # refinement tolerance that keeps whole pulses within 1e-8
ERR_BOUND = 1e-8


@pytest.fixture(scope="module")
def golden_case(tmp_path_factory):
    cache = {}

    def get(name):
        if name not in cache:
            spec = CASES[name]
            d = str(tmp_path_factory.mktemp(name))
            info = generate(spec["params"], d)
            cache[name] = (d, info, spec, dict(np.load(os.path.join(GOLDEN, f"{name}.npz"))))
        return cache[name]
    return get


def _args(d, info, params):
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    return (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])


def _err(x, g):
    if "x" in g:
        return float(np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]))
    return float(np.linalg.norm(sketch(x) - g["x_sketch"]) / g["x_norm"])


@pytest.mark.parametrize("name", ["tiny_nondipole", "dipole_small", "nondipole_medium_full", "nondipole_large_20"])
def test_mixed_whole_pulse_matches_reference_build(golden_case, native_lib, name):
    d, info, spec, g = golden_case(name)
    xm, rm, _ = run(*_args(d, info, spec["params"]), tol=MIXED_TOL, precision="mixed",
                    max_steps=spec.get("max_steps"), write_outputs=False)
    assert len(rm) == len(g["iters"])
    err = _err(xm, g)
    assert err <= ERR_BOUND, err
    assert all(r["refinements"] >= 1 for r in rm)             # an FP64 residual pass every step
    # norm conservation check (FP64 x^H S x before every step)
    sn = np.array([r["snorm"] for r in rm])
    assert np.all(np.abs(sn - sn[0]) <= 1e-7 * sn[0])


def test_mixed_at_equal_residual_as_accurate_as_fp64(golden_case, native_lib):
    """At the refinement tolerance 1e-10 over the whole 1500-step pulse the
    mixed path's error against the reference is within 2x the plain FP64
    path's at the same tolerance."""
    d, info, spec, g = golden_case("nondipole_medium_full")
    args = _args(d, info, spec["params"])
    x64, _, _ = run(*args, tol=1e-10, write_outputs=False)
    xm, _, _ = run(*args, tol=1e-10, precision="mixed", write_outputs=False)
    e64, em = _err(x64, g), _err(xm, g)
    assert em <= 2 * e64 + 1e-10, (em, e64)


def test_mixed_matches_fp64_tight_tolerance(workdirs, native_lib):
    d, params, info = workdirs["tiny_dipole"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    x64, _, _ = run(*args, tol=1e-12, write_outputs=False)
    xm, rm, _ = run(*args, tol=1e-12, precision="mixed", write_outputs=False)
    assert np.linalg.norm(xm - x64) / np.linalg.norm(x64) <= 1e-10


@pytest.mark.parametrize("name", ["tiny_nondipole", "nondipole_large_20"])
def test_double_float_residual_agrees_with_fp64_residual(golden_case, native_lib, name):
    """The refinement residual in double-float on the FP32 units (the
    default on the matrix-free operator) against the same pass on the FP64
    units: the refinement passes and inner iterations within 2 and 4 in
    total over the steps (a residual near the tolerance may decide either
    way), the initial residuals within 1e-6 relative of each other (a
    residual of ~1e-6 |b| computed to ~1e-14 |b|), and final states within
    1e-10 (both solve to the same residual tolerance)."""
    from dirac_hydrogen_code_gb300.native import Solver
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    d, info, spec, g = golden_case(name)
    params = spec["params"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    dt, steps = step_times(T, params["Ntime"])
    nsteps = min(len(steps), 20)
    from dirac_hydrogen_code_gb300.native import Problem
    prob = Problem(d, info["lmax"])
    psi, _ = prob.psi0()
    out = []
    for mode in (0, 1):
        sol = Solver(prob, dt, precision="mixed")
        sol.set_operator(0)
        sol.set_residual_precision(mode)
        assert sol.residual_precision()["double_float_in_use"] == bool(mode)
        sol.set_x(psi)
        recs = [sol.step(pulse(params["Intensity"], params["Omega"], params["Cycles"], t), 500, 1e-12)
                for _, t in steps[:nsteps]]
        out.append((sol.get_x(), recs))
        sol.close()
    (x64, r64), (xdd, rdd) = out
    assert sum(abs(a["refinements"] - b["refinements"]) for a, b in zip(r64, rdd)) <= 2
    assert sum(abs(a["inner_iters"] - b["inner_iters"]) for a, b in zip(r64, rdd)) <= 4
    for a, b in zip(r64, rdd):
        assert abs(a["init_residual"] - b["init_residual"]) <= 1e-6 * a["init_residual"] + 1e-15
    assert np.linalg.norm(xdd - x64) / np.linalg.norm(x64) <= 1e-10


def test_fp64_apply_after_double_float_steps(golden_case, native_lib):
    """Mixed steps with the double-float residual pass leave the FP64 radial
    tables out; the next FP64 apply rebuilds them from the step's pulse
    factors: the same result as setting the time again."""
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    from dirac_hydrogen_code_gb300.native import Problem, Solver
    d, info, spec, g = golden_case("tiny_nondipole")
    params = spec["params"]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    dt, steps = step_times(T, params["Ntime"])
    prob = Problem(d, info["lmax"])
    sol = Solver(prob, dt, precision="mixed")
    sol.set_operator(0)
    assert sol.residual_precision()["double_float_in_use"]
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps[:5]]
    for ft in fts:
        sol.step(ft, 500, 1e-12)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(prob.n) + 1j * rng.standard_normal(prob.n)
    y_after_step = sol.apply(x)
    sol.set_time(fts[-1])
    assert np.array_equal(y_after_step, sol.apply(x))
