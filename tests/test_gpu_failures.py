"""Failure paths of the step, made on the host (no GPU fault, trap or hang).

* A non-finite state (a NaN planted in psi0 on the host) makes the
  right-hand side non-finite: the step returns GADE_ERR_NUMERIC, for a
  single pulse (FP64 and mixed precision) and for the failing pulse of a
  batch, and the solver steps normally once the state is set again.
* A preconditioner stage wait that runs out (the kernel is told to withhold
  one stage copy, and the wait is limited to a few polls) ends the step with
  GADE_ERR_CUDA; the device stays usable and the next step, from a state set
  again, equals a new solver's first step.

The reference records only non-convergence (tools/bicgstab.c:196-226) and
exits on other errors; these are the status codes of include/gade.h.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GADE_ERR_CUDA = 3
GADE_ERR_NUMERIC = 5


def _setup(workdirs, name="tiny_dipole"):
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    from dirac_hydrogen_code_gb300.native import Problem
    d, params, info = workdirs[name]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    dt, steps = step_times(T, params["Ntime"])
    prob = Problem(d, info["lmax"])
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps]
    return prob, dt, fts


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_state_returns_numeric(workdirs, native_lib, precision):
    from dirac_hydrogen_code_gb300.native import GadeError, Solver
    prob, dt, fts = _setup(workdirs)
    tol = 1e-12 if precision == "fp64" else 1e-10
    psi, _ = prob.psi0()
    bad = psi.copy()
    bad[len(bad) // 3] = complex(np.nan, 0.0)
    sol = Solver(prob, dt, precision=precision)
    sol.set_operator(0)
    sol.set_x(bad)
    with pytest.raises(GadeError) as e:
        sol.step(fts[0], 500, tol)
    assert e.value.code == GADE_ERR_NUMERIC
    # the solver recovers once the state is set again
    sol.set_x(psi)
    st = sol.step(fts[0], 500, tol)
    fresh = Solver(prob, dt, precision=precision)
    fresh.set_operator(0)
    st_ref = fresh.step(fts[0], 500, tol)
    x, x_ref = sol.get_x(), fresh.get_x()
    assert np.all(np.isfinite(x))
    assert st["iters"] == st_ref["iters"]
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e-14


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_pulse_of_batch_returns_numeric(workdirs, native_lib, precision):
    from dirac_hydrogen_code_gb300.native import Batch, GadeError
    prob, dt, fts = _setup(workdirs)
    tol = 1e-12 if precision == "fp64" else 1e-10
    psi, _ = prob.psi0()
    b = Batch(prob, [dt, dt], precision=precision, chunk_splines=16)
    b.set_operator(0)
    bad = psi.copy()
    bad[7] = complex(0.0, np.inf)
    b.set_x(1, bad)
    ft = np.stack([fts[0], fts[0]])
    with pytest.raises(GadeError) as e:
        b.step(ft, maxit=500, tol=tol)
    assert e.value.code == GADE_ERR_NUMERIC
    assert "pulse 1" in str(e.value)
    # pulse 1 steps normally once its state is set again: as in a new batch
    # (it never iterated in the failed step, so nothing of it carries over)
    b.set_x(1, psi)
    b.step(ft, maxit=500, tol=tol)
    fresh = Batch(prob, [dt, dt], precision=precision, chunk_splines=16)
    fresh.set_operator(0)
    fresh.step(ft, maxit=500, tol=tol)
    x1 = b.get_x(1)
    assert np.all(np.isfinite(x1)) and np.array_equal(x1, fresh.get_x(1))


@pytest.mark.parametrize("stage", [0, 1])
def test_preconditioner_wait_limit_returns_cuda_error(workdirs, native_lib, stage):
    from dirac_hydrogen_code_gb300.native import GadeError, Solver
    prob, dt, fts = _setup(workdirs, "tiny_nondipole")
    psi, _ = prob.psi0()
    sol = Solver(prob, dt)
    sol.set_operator(0)
    sol.set_wait_limit(1000)
    sol.inject_wait_timeout(stage)
    with pytest.raises(GadeError) as e:
        sol.step(fts[0], 500, 1e-12)
    assert e.value.code == GADE_ERR_CUDA
    # also through the preconditioner entry point alone
    with pytest.raises(GadeError) as e:
        sol.precond(psi)
    assert e.value.code == GADE_ERR_CUDA
    # the device and the solver stay usable
    sol.inject_wait_timeout(-1)
    sol.set_wait_limit(0)
    sol.set_x(psi)
    recs = [sol.step(ft, 500, 1e-12) for ft in fts[:3]]
    fresh = Solver(prob, dt)
    fresh.set_operator(0)
    recs_ref = [fresh.step(ft, 500, 1e-12) for ft in fts[:3]]
    assert [r["iters"] for r in recs] == [r["iters"] for r in recs_ref]
    x, x_ref = sol.get_x(), fresh.get_x()
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) <= 1e-14
    z = sol.precond(psi)
    assert np.array_equal(z, fresh.precond(psi))
