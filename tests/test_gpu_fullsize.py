"""Size-independent properties at the largest configuration (NKappa=16,
NMu=8, NSplines=300, lmax 10; N = 244k), where the oracle's assembled
operator would be too large to build in a test: linearity of the operator,
Hermiticity of S and anti-Hermiticity of the time-dependent part (the
reference's Hfull carries the factor i h dt/2 of a Hermitian H), and the
Crank-Nicolson step's norm conservation and agreement between precisions."""

import math

import numpy as np
import pytest

from dirac_hydrogen_code_gb300.cn import pulse, step_times
from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
from dirac_hydrogen_code_gb300.native import Problem, Solver

pytestmark = pytest.mark.gpu

NAME = "nondipole_large"


@pytest.fixture(scope="module")
def large(tmp_path_factory, native_lib):
    params = CONFIGS[NAME]
    d = str(tmp_path_factory.mktemp(NAME))
    info = generate(params, d)
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    dt, steps = step_times(T, params["Ntime"])
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps[:40]]
    prob = Problem(d, info["lmax"])
    yield prob, dt, fts
    prob.close()


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def test_operator_linearity_and_symmetry(large):
    prob, dt, fts = large
    sol = Solver(prob, dt)
    sol.set_time(fts[17])
    n = prob.n
    x, y = _rand(n, 1), _rand(n, 2)
    a, b = 0.3 - 1.1j, -2.0 + 0.25j
    ax, sx, hx = sol.apply(x, parts=True)
    ay, sy, hy = sol.apply(y, parts=True)
    # y = S x + H x with the parts returned separately
    assert np.linalg.norm(ax - (sx + hx)) <= 1e-14 * np.linalg.norm(ax)
    # linearity of the whole operator
    lin = sol.apply(a * x + b * y)
    assert np.linalg.norm(lin - (a * ax + b * ay)) <= 1e-13 * np.linalg.norm(lin)
    # S Hermitian, Hfull = i h dt/2 H(t) anti-Hermitian (normwise bounds)
    nx, ny = np.linalg.norm(x), np.linalg.norm(y)
    assert abs(np.vdot(y, sx) - np.conj(np.vdot(x, sy))) <= 1e-12 * ny * np.linalg.norm(sx)
    assert abs(np.vdot(y, hx) + np.conj(np.vdot(x, hy))) <= 1e-12 * ny * np.linalg.norm(hx)
    # x^H S x real and positive, x^H Hfull x imaginary
    sxx, hxx = np.vdot(x, sx), np.vdot(x, hx)
    assert sxx.real > 0 and abs(sxx.imag) <= 1e-12 * abs(sxx)
    assert abs(hxx.real) <= 1e-12 * nx * np.linalg.norm(hx)
    sol.close()


def test_cn_steps_conserve_norm_and_agree_across_precisions(large):
    prob, dt, fts = large
    psi, _ = prob.psi0()
    nsteps = 30
    out = {}
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-10)):
        sol = Solver(prob, dt, precision=prec)
        sol.set_x(psi)
        recs = [sol.step(ft, maxit=500, tol=tol) for ft in fts[:nsteps]]
        x = sol.get_x()
        _, s0, _ = sol.apply(psi, parts=True)
        _, sxn, _ = sol.apply(x, parts=True)
        out[prec] = (x, recs, np.vdot(psi, s0).real, np.vdot(x, sxn).real)
        sol.close()
    x64, recs64, n0, n1 = out["fp64"]
    # Crank-Nicolson is unitary in the S-norm: drift at the solver tolerance
    assert abs(n1 - n0) / n0 <= 1e-10
    assert max(r["iters"] for r in recs64) <= 5
    assert all(r["tol_error"] < 1e-12 for r in recs64)
    x32, recs32, _, m1 = out["mixed"]
    assert abs(m1 - n0) / n0 <= 1e-9
    assert np.linalg.norm(x32 - x64) / np.linalg.norm(x64) <= 1e-8
