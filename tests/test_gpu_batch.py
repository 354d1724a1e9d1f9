"""Batched pulses on the GPU (gade_batch_*), through the C ABI.

  * every pulse of a batch against the CPU oracle run on that pulse's own
    generated inputs (same block-LU preconditioner): relative L2 of x
    <= 1e-10 after the pulse's whole time grid, BiCGSTAB iterations within
    +-1 per step (the batch's radial tables come from gen.pulse_tables, which
    sums the quadrature in a different order than the files: ~1e-16)
  * a batch of several pulses against one-pulse batches of the same pulses:
    bit-identical states (the per-pulse work and reduction order do not
    depend on the other pulses), with and without CUDA graphs
  * uneven lengths: a pulse whose time grid ended keeps its final state and
    leaves the launch list
"""
import math
import os

import numpy as np
import pytest

import oracle as O
from dirac_hydrogen_code_gb300.cn import pulse, run, run_batch, step_times
from dirac_hydrogen_code_gb300.gen import generate
from dirac_hydrogen_code_gb300.gen.pulses import pulse_tables
from dirac_hydrogen_code_gb300.native import Batch, GadeError, Problem

pytestmark = pytest.mark.gpu

PULSES = [dict(E0=10.0, omega=50.0, cycles=2, ntime=20),
          dict(E0=30.0, omega=35.0, cycles=1, ntime=13),
          dict(E0=3.0, omega=80.0, cycles=3, ntime=27)]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def batch_case(workdirs, tmp_path_factory):
    d, params, info = workdirs["tiny_nondipole"]
    prob = Problem(d, info["lmax"])
    tables = np.stack([pulse_tables(params, p["omega"], p["cycles"]) for p in PULSES])
    dirs = []
    for k, p in enumerate(PULSES):
        dk = str(tmp_path_factory.mktemp(f"pulse{k}"))
        generate(dict(params, Omega=p["omega"], Cycles=p["cycles"], Ntime=p["ntime"]), dk)
        dirs.append(dk)
    return d, params, info, prob, tables, dirs


def test_batch_matches_oracle_per_pulse(batch_case, native_lib):
    d, params, info, prob, tables, dirs = batch_case
    xs, recs, b = run_batch(prob, PULSES, tables, tol=1e-12, maxit=500)
    for k, p in enumerate(PULSES):
        T = p["cycles"] * 2 * math.pi / p["omega"]
        xo, ro, _ = O.run(dirs[k], T, info["lmax"], p["E0"], p["omega"], p["cycles"], p["ntime"],
                          tol=1e-12, maxit=500, precond="blocklu")
        assert len(recs[k]) == len(ro) == len(step_times(T, p["ntime"])[1])
        assert max(abs(a.iters - r["iters"]) for a, r in zip(ro, recs[k])) <= 1
        assert _rel(xs[k], xo) < 1e-10, k
    inf = b.info()
    assert inf["npulse"] == 3 and inf["steps"] == max(len(r) for r in recs)
    assert inf["chunk_splines"] in inf["tune_cs"]


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("graphs", [True, False])
def test_batch_bit_identical_to_single_pulse_batches(batch_case, native_lib, graphs, op):
    """With the same operator (matrix-free 0, assembled 1) a pulse's bits do
    not depend on the other pulses of its batch."""
    d, params, info, prob, tables, dirs = batch_case
    cs = 16
    xs, recs, _ = run_batch(prob, PULSES, tables, tol=1e-12, chunk_splines=cs, use_graphs=graphs, operator=op)
    for k in range(len(PULSES)):
        x1, r1, _ = run_batch(prob, [PULSES[k]], tables[k:k + 1], tol=1e-12, chunk_splines=cs,
                              use_graphs=True, iters_per_launch=2, operator=op)
        assert np.array_equal(xs[k], x1[0]), k
        assert [r["iters"] for r in recs[k]] == [r["iters"] for r in r1[0]]


def test_batch_matches_single_solver(workdirs, native_lib):
    """With the problem's own radial tables a batch pulse is the solver's run."""
    d, params, info = workdirs["tiny_nondipole"]
    prob = Problem(d, info["lmax"])
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    p = dict(E0=params["Intensity"], omega=params["Omega"], cycles=params["Cycles"], ntime=params["Ntime"])
    xs, recs, _ = run_batch(prob, [p, dict(p, E0=2 * p["E0"])], None, tol=1e-12, max_steps=12)
    x1, r1, _ = run(d, T, info["lmax"], p["E0"], p["omega"], p["cycles"], p["ntime"], tol=1e-12, max_steps=12,
                    write_outputs=False, problem=prob)
    assert _rel(xs[0], x1) < 1e-13
    assert [r["iters"] for r in recs[0]] == [r["iters"] for r in r1]
    assert _rel(xs[1], x1) > 1e-6          # the second pulse is a different pulse


def test_batch_retires_finished_pulses(batch_case, native_lib):
    d, params, info, prob, tables, dirs = batch_case
    seen = []

    def cb(j, b):
        seen.append(b.info()["active"])
    xs, recs, b = run_batch(prob, PULSES, tables, tol=1e-12, callback=cb)
    n = [len(r) for r in recs]
    assert seen == [sum(1 for m in n if j < m) for j in range(max(n))]
    # the state of a retired pulse is its state after its last step
    x_short, _, _ = run_batch(prob, [PULSES[1]], tables[1:2], tol=1e-12)
    assert _rel(xs[1], x_short[0]) < 1e-13


def test_batch_maxit_and_edge_cases(batch_case, native_lib):
    d, params, info, prob, tables, dirs = batch_case
    dts = [p["cycles"] * 2 * math.pi / p["omega"] / p["ntime"] for p in PULSES]
    b = Batch(prob, dts, tables)
    ft = np.stack([pulse(p["E0"], p["omega"], p["cycles"], 0.3) for p in PULSES])
    st = b.step(ft, maxit=1, tol=1e-30)
    assert [s["iters"] for s in st] == [1, 1, 1]
    # zero state: x = 0, no iterations (tools/bicgstab.c:173-179)
    b.set_x(1, np.zeros(prob.n, complex))
    st = b.step(ft, maxit=500, tol=1e-12)
    assert st[1]["iters"] == 0 and st[1]["tol_error"] == 0.0 and np.all(b.get_x(1) == 0)
    assert st[0]["iters"] > 0
    # inactive pulses are untouched
    x2 = b.get_x(2)
    st = b.step(ft, active=[1, 1, 0], maxit=500, tol=1e-12)
    assert st[2]["iters"] == 0 and np.array_equal(b.get_x(2), x2)
    assert b.info()["active"] == 2
    with pytest.raises(GadeError) as e:
        b.step(ft, maxit=-1)
    assert e.value.code == 4
    with pytest.raises(GadeError):
        b.set_x(5, np.zeros(prob.n, complex))


def test_mixed_batch_matches_oracle(batch_case, native_lib):
    """complex64 inner solves in FP64 refinement, batched: every pulse
    against the CPU oracle's FP64 run on its own inputs, relative L2 of the
    final state <= 1e-8 at the refinement tolerance 1e-11."""
    d, params, info, prob, tables, dirs = batch_case
    xm, rm, b = run_batch(prob, PULSES, tables, tol=1e-11, precision="mixed")
    for k, pk in enumerate(PULSES):
        T = pk["cycles"] * 2 * math.pi / pk["omega"]
        xo, _, _ = O.run(dirs[k], T, info["lmax"], pk["E0"], pk["omega"], pk["cycles"], pk["ntime"],
                         tol=1e-12, maxit=500, precond="ilu")
        assert _rel(xm[k], xo) <= 1e-8, k
        assert all(r["refinements"] >= 1 for r in rm[k])
        sn = np.array([r["snorm"] for r in rm[k]])
        assert np.all(np.abs(sn - sn[0]) < 1e-7)


def test_mixed_batch_matches_single_pulse_mixed(batch_case, native_lib):
    """A batched mixed pulse follows the single-pulse mixed solver's rules:
    same refinement passes and inner iterations on the pulse's own inputs."""
    d, params, info, prob, tables, dirs = batch_case
    xm, rm, _ = run_batch(prob, PULSES, tables, tol=1e-10, precision="mixed")
    for k, pk in enumerate(PULSES):
        T = pk["cycles"] * 2 * math.pi / pk["omega"]
        xs, rs, _ = run(dirs[k], T, info["lmax"], pk["E0"], pk["omega"], pk["cycles"], pk["ntime"], tol=1e-10,
                        precision="mixed", write_outputs=False)
        assert _rel(xm[k], xs) < 1e-8, k
        assert sum(abs(a["refinements"] - r["refinements"]) for a, r in zip(rm[k], rs)) <= 2
        assert sum(abs(a["inner_iters"] - r["inner_iters"]) for a, r in zip(rm[k], rs)) <= 4


@pytest.mark.parametrize("op", [0, 1])
def test_mixed_batch_bit_identical_to_single_pulse_batches(batch_case, native_lib, op):
    d, params, info, prob, tables, dirs = batch_case
    xs, recs, _ = run_batch(prob, PULSES, tables, tol=1e-10, precision="mixed", chunk_splines=16, operator=op)
    for k in range(len(PULSES)):
        x1, r1, _ = run_batch(prob, [PULSES[k]], tables[k:k + 1], tol=1e-10, precision="mixed", chunk_splines=16,
                              iters_per_launch=3, operator=op)
        assert np.array_equal(xs[k], x1[0]), k
        assert [r["inner_iters"] for r in recs[k]] == [r["inner_iters"] for r in r1[0]]


@pytest.mark.parametrize("shared_tables", [False, True])
def test_batch_operators_agree(batch_case, native_lib, shared_tables):
    """The assembled operator of a batch (per-pulse values; one set of
    unit-factor values when the pulses share their radial tables) gives the
    matrix-free batch's iterations and states."""
    d, params, info, prob, tables, dirs = batch_case
    pulses = PULSES
    if shared_tables:
        pulses = [dict(p, omega=params["Omega"], cycles=params["Cycles"]) for p in PULSES]
    tab = None if shared_tables else tables
    out = []
    for op in (0, 1):
        xs, recs, b = run_batch(prob, pulses, tab, tol=1e-12, maxit=500, operator=op)
        assert b.operator()["assembled"] == op
        out.append((xs, [[r["iters"] for r in rk] for rk in recs]))
        b.close()
    assert out[1][1] == out[0][1]
    for k in range(len(pulses)):
        assert _rel(out[1][0][k], out[0][0][k]) < 1e-12, k
