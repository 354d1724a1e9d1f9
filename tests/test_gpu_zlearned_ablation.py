"""Ablation of the learned initial guess (GPU): a network trained on the
solver's own trajectories of seeded training pulses, evaluated on held-out
pulses against the same mixed-precision solver without it.

Stated per run: mean relative FP64 residual of the initial guess, inner
iterations per step and the final-state error against an FP64 run at tol
1e-12.  The learned guess must lower the mean initial residual by at least
10% and must not make the final state worse: its relative L2 error stays
within 1e-7 of the FP64 reference and within 1.5x of the plain guess's
(both solves stop at the same FP64 residual, 1e-10, every step)."""
import json
import os

import numpy as np
import pytest

from dirac_hydrogen_code_gb300 import learned as L
from dirac_hydrogen_code_gb300.gen import CONFIGS
from dirac_hydrogen_code_gb300.native import Problem

pytestmark = pytest.mark.gpu


def test_learned_guess_ablation(workdirs, native_lib):
    d, params, info = workdirs["dipole_small"]
    prob = Problem(d, info["lmax"])
    nsteps = 200
    mk = lambda n, seed: L.intensity_pulses(n, seed, params["Omega"], params["Cycles"], params["Ntime"])  # noqa
    train, held = mk(16, 101), mk(4, 202)
    model = L.build_model(prob, train, nsteps, rank=64, nsnap=200, pod_pulses=8, epochs=30, seed=1)
    xr, _, _ = L.run_held_out(prob, held, nsteps, 1e-12, "fp64", None)
    out = {}
    for label, mdl in [("extrapolation", None), ("learned", model)]:
        xs, st, ms = L.run_held_out(prob, held, nsteps, 1e-10, "mixed", mdl)
        ini = np.array([[s["init_residual"] for s in row] for row in st])[L.K_HIST:]
        its = np.array([[s["inner_iters"] for s in row] for row in st])
        err = np.linalg.norm(xs - xr, axis=1) / np.linalg.norm(xr, axis=1)
        out[label] = dict(init_residual=float(ini.mean()), inner_iters=float(its.mean()), max_err=float(err.max()),
                          ms=ms)
    print(json.dumps(out))
    assert out["learned"]["init_residual"] < 0.9 * out["extrapolation"]["init_residual"], out
    assert out["learned"]["max_err"] <= 1e-7, out
    assert out["learned"]["max_err"] <= 1.5 * out["extrapolation"]["max_err"], out
