"""GPU parity tests: the CUDA path, called through the C ABI
(libgade_gb300.so), against the CPU oracle on identical generated inputs.

Tolerances (FP64 everywhere):
  * operator parts S x, H(t) x       relative L2  <= 1e-13
  * preconditioner P^T z = b          relative residual <= 1e-11
  * one CN step / short runs          relative L2 of x <= 1e-12 vs the oracle
                                      with the same (block-LU) preconditioner
  * full runs vs the oracle with the  relative L2 of x <= 1e-10, BiCGSTAB
    reference SuperLU ILU             iterations within +-1 per step
"""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from dirac_hydrogen_code_gb300 import build, formats
from dirac_hydrogen_code_gb300.cn import pulse, run, step_times
from dirac_hydrogen_code_gb300.native import GadeError, Problem, Solver

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _setup(workdirs, name):
    d, params, info = workdirs[name]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    dt = T / params["Ntime"]
    return d, params, info, T, dt


@pytest.mark.parametrize("op", [0, 1])
@pytest.mark.parametrize("name", ["tiny_dipole", "tiny_nondipole", "dipole_small"])
def test_operator_matches_oracle(workdirs, native_lib, name, op):
    """Matrix-free (0) and assembled (1) operator against the oracle's
    assembly of the reference's matrices."""
    d, params, info, T, dt = _setup(workdirs, name)
    p = O.load_problem(d, info["lmax"])
    prob = Problem(d, info["lmax"])
    assert prob.info["real_coupling"] == 1
    sol = Solver(prob, dt)
    sol.set_operator(op)
    assert sol.operator()["assembled"] == op
    rng = np.random.default_rng(7)
    x = rng.standard_normal(p.n) + 1j * rng.standard_normal(p.n)
    for t in (0.25 * T, 0.8 * T):
        ft = pulse(params["Intensity"], params["Omega"], params["Cycles"], t)
        sol.set_time(ft)
        y, sx, hx = sol.apply(x, parts=True)
        S, _ = O.stationary(p, dt)
        H = O.timedep(p, dt, ft)
        assert _rel(sx, S @ x) < 1e-13
        assert _rel(hx, H @ x) < 1e-13
        assert _rel(y, S @ x + H @ x) < 1e-13
    assert sol.launch_count() > 0


@pytest.mark.parametrize("warps", [8, 4])
@pytest.mark.parametrize("name", ["tiny_dipole", "tiny_nondipole", "dipole_small"])
def test_preconditioner_matches_oracle(workdirs, native_lib, name, warps):
    d, params, info, T, dt = _setup(workdirs, name)
    p = O.load_problem(d, info["lmax"])
    sol = Solver(Problem(d, info["lmax"]), dt)
    sol.set_precond_warps(warps)
    with pytest.raises(GadeError):
        sol.set_precond_warps(6)
    S, Hst = O.stationary(p, dt)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(p.n) + 1j * rng.standard_normal(p.n)
    z = sol.precond(b)
    P = (S + Hst).tocsr()
    assert _rel(P.T @ z, b) < 1e-11
    zo = O.BlockLuPrecond(p, S, Hst).solve(b)
    assert _rel(z, zo) < 1e-11
    # the reference's ILU(1e-6) differs from the exact inverse only slightly
    zi = O.IluPrecond(S, Hst).solve(b)
    assert _rel(z, zi) < 1e-4


@pytest.mark.parametrize("name", ["tiny_dipole", "tiny_nondipole"])
def test_steps_match_oracle_same_preconditioner(workdirs, native_lib, name):
    d, params, info, T, dt = _setup(workdirs, name)
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, p = O.run(*args, tol=1e-12, precond="blocklu", max_steps=12)
    xg, rg, _ = run(*args, tol=1e-12, max_steps=12, write_outputs=False)
    assert [r.iters for r in ro] == [r["iters"] for r in rg]
    assert _rel(xg, xo) < 1e-12


@pytest.mark.parametrize("name", ["tiny_dipole", "tiny_nondipole"])
def test_full_run_matches_reference_semantics(workdirs, native_lib, name):
    """Whole pulse, reference tolerance semantics, ILU oracle."""
    d, params, info, T, dt = _setup(workdirs, name)
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, p = O.run(*args, tol=1e-12, precond="ilu")
    xg, rg, _ = run(*args, tol=1e-12, write_outputs=False)
    assert len(ro) == len(rg) == len(step_times(T, params["Ntime"])[1])
    assert max(abs(a.iters - b["iters"]) for a, b in zip(ro, rg)) <= 1
    assert _rel(xg, xo) <= 1e-10
    drift_o = O.s_norm(p, xo) - O.s_norm(p, p.psi0)
    drift_g = O.s_norm(p, xg) - O.s_norm(p, p.psi0)
    assert abs(drift_o - drift_g) < 1e-11


def test_dipole_small_full_run(workdirs, native_lib):
    """The dipole benchmark configuration (N=8400), whole pulse at tol 1e-12."""
    d, params, info, T, dt = _setup(workdirs, "dipole_small")
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, p = O.run(*args, tol=1e-12, precond="ilu")
    xg, rg, _ = run(*args, tol=1e-12, write_outputs=False)
    assert len(rg) == len(ro)
    diffs = [abs(a.iters - b["iters"]) for a, b in zip(ro, rg)]
    assert max(diffs) <= 1
    assert _rel(xg, xo) <= 1e-10
    drift_o = O.s_norm(p, xo) - O.s_norm(p, p.psi0)
    drift_g = O.s_norm(p, xg) - O.s_norm(p, p.psi0)
    assert abs(drift_o - drift_g) < 1e-11


def test_reference_default_tolerance(workdirs, native_lib):
    """tol=1e-16/maxit=500 as hard-coded in tools/dirac_solver.c:506-507."""
    d, params, info, T, dt = _setup(workdirs, "tiny_dipole")
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, p = O.run(*args, tol=1e-16, maxit=500, precond="blocklu", max_steps=8)
    xg, rg, _ = run(*args, tol=1e-16, maxit=500, max_steps=8, write_outputs=False)
    assert max(abs(a.iters - b["iters"]) for a, b in zip(ro, rg)) <= 1
    assert _rel(xg, xo) < 1e-12


def test_general_complex_coupling(workdirs, native_lib, tmp_path):
    """Inputs whose g tables are complex take the general (non-real) path."""
    d, params, info, T, dt = _setup(workdirs, "tiny_nondipole")
    d2 = str(tmp_path / "cplx")
    shutil.copytree(d, d2)
    rng = np.random.default_rng(11)
    for l in range(info["lmax"]):
        for a in range(6):
            for q in range(4):
                f = os.path.join(d2, f"g{q}a{a}l{l}.csr")
                m = formats.csr_read(f)
                m.Ax = m.Ax + 1e-3j * rng.standard_normal(m.nnz) * np.abs(m.Ax)
                formats.csr_write(f, m)
    prob = Problem(d2, info["lmax"])
    assert prob.info["real_coupling"] == 0
    sol = Solver(prob, dt)
    p = O.load_problem(d2, info["lmax"])
    ft = pulse(params["Intensity"], params["Omega"], params["Cycles"], 0.4 * T)
    sol.set_time(ft)
    x = rng.standard_normal(p.n) + 1j * rng.standard_normal(p.n)
    y, sx, hx = sol.apply(x, parts=True)
    assert _rel(hx, O.timedep(p, dt, ft) @ x) < 1e-13
    args = (d2, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, _ = O.run(*args, tol=1e-12, precond="blocklu", max_steps=5)
    xg, rg, _ = run(*args, tol=1e-12, max_steps=5, write_outputs=False, problem=prob)
    assert _rel(xg, xo) < 1e-12


def test_without_dkb_zero_blocks(workdirs, native_lib, tmp_path):
    """Radial tables that lack the DKB zero blocks take the four-term kernel
    and still match the oracle."""
    d, params, info, T, dt = _setup(workdirs, "tiny_nondipole")
    d2 = str(tmp_path / "full")
    shutil.copytree(d, d2)
    rng = np.random.default_rng(12)
    for l in range(info["lmax"]):
        f = os.path.join(d2, f"g3a1l{l}.csr")          # fill g3's zero quadrants
        m = formats.csr_read(f)
        m.Ax = m.Ax + 1e-4 * rng.standard_normal(m.nnz) * np.max(np.abs(m.Ax))
        formats.csr_write(f, m)
    prob = Problem(d2, info["lmax"])
    assert prob.info["dkb_zero"] == 0 and prob.info["real_coupling"] == 1
    args = (d2, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    sol = Solver(prob, dt)
    p = O.load_problem(d2, info["lmax"])
    ft = pulse(params["Intensity"], params["Omega"], params["Cycles"], 0.4 * T)
    sol.set_time(ft)
    x = rng.standard_normal(p.n) + 1j * rng.standard_normal(p.n)
    _, _, hx = sol.apply(x, parts=True)
    assert _rel(hx, O.timedep(p, dt, ft) @ x) < 1e-13
    xo, ro, _ = O.run(*args, tol=1e-12, precond="blocklu", max_steps=5)
    xg, rg, _ = run(*args, tol=1e-12, max_steps=5, write_outputs=False, problem=prob)
    assert _rel(xg, xo) < 1e-12


def test_edge_cases(workdirs, native_lib):
    d, params, info, T, dt = _setup(workdirs, "tiny_dipole")
    prob = Problem(d, info["lmax"])
    sol = Solver(prob, dt)
    ft = pulse(params["Intensity"], params["Omega"], params["Cycles"], dt)
    psi, _ = prob.psi0()
    # zero state: rhs = 0 -> x set to zero, no iterations (tools/bicgstab.c:173-179)
    sol.set_x(np.zeros(prob.n, complex))
    st = sol.step(ft, maxit=500, tol=1e-12)
    assert st["iters"] == 0 and st["tol_error"] == 0.0
    assert np.all(sol.get_x() == 0)
    # huge tolerance: initial residual already below -> return before iterating
    sol.set_x(psi)
    st = sol.step(ft, maxit=500, tol=1.0)
    assert st["iters"] == 0 and 0 < st["tol_error"] < 1.0
    assert np.array_equal(sol.get_x(), psi)
    # maxit = 0: no iteration, tol_error = initial relative residual
    st = sol.step(ft, maxit=0, tol=1e-12)
    assert st["iters"] == 0 and st["tol_error"] > 0
    # argument errors come back as status codes
    with pytest.raises(ValueError):
        sol.set_x(np.zeros(3, complex))
    with pytest.raises(GadeError) as e:
        sol.step(ft, maxit=-1, tol=1e-12)
    assert e.value.code == 4
    with pytest.raises(GadeError) as e:
        Solver(prob, -1.0)
    assert e.value.code == 4


def test_drop_in_executable(workdirs, native_lib, tmp_path):
    """dirac_solver with the reference CLI on a copy of the inputs."""
    d, params, info, T, dt = _setup(workdirs, "tiny_dipole")
    d2 = str(tmp_path / "run")
    shutil.copytree(d, d2)
    exe = build.solver_path()
    cmd = [exe, "-t", repr(T), "-l", str(info["lmax"]), "-i", str(params["Intensity"]),
           "-o", str(params["Omega"]), "-c", str(params["Cycles"]), "-n", str(params["Ntime"]),
           "--tol", "1e-12", "--final-dump", "--stats", "stats.jsonl"]
    res = subprocess.run(cmd, cwd=d2, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    assert "All matrices read correctly" in res.stdout and "Total runtime" in res.stdout
    nsteps = len(step_times(T, params["Ntime"])[1])
    out = formats.out_read(os.path.join(d2, f"x{nsteps}.out"))
    args = (d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"], params["Ntime"])
    xo, ro, p = O.run(*args, tol=1e-12, precond="ilu")
    xorig = np.empty_like(xo)
    xorig[p.xperm] = xo
    assert _rel(out, xorig) <= 1e-10
    lines = open(os.path.join(d2, "runstats.txt")).read().splitlines()
    assert len(lines) == params["Ntime"]
    assert lines[0].startswith("0, 0.000000e+00, 0")
    # wrong arguments: fewer than 5 -> usage error, as the reference
    res = subprocess.run([exe, "-t", "1"], cwd=d2, capture_output=True, text=True)
    assert res.returncode != 0
    # missing input file -> error message, non-zero exit, no crash
    os.remove(os.path.join(d2, "h02.csr"))
    res = subprocess.run(cmd, cwd=d2, capture_output=True, text=True, timeout=60)
    assert res.returncode == 1 and "h02.csr" in res.stderr


def test_order_split_matches_unsplit(workdirs, native_lib):
    """The operator with 1-4 order splits and with the balanced segments
    (partial sums of a unit's pieces combined by its last piece) gives the
    same steps up to the order of summation."""
    d, params, info, T, dt = _setup(workdirs, "tiny_nondipole")
    prob = Problem(d, info["lmax"])
    psi, _ = prob.psi0()
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in step_times(T, params["Ntime"])[1][:6]]
    ref = None
    for ns in (1, 2, 3, 4, 0):
        sol = Solver(prob, dt)
        sol.set_split(ns)
        assert sol.split()[0] == ns
        if ns == 0:
            bal = sol.balanced()
            # a tiny problem on a whole GPU: units cut into many pieces
            assert bal["segments"] > 0 and bal["pieces"] > prob.info["nblk"]
        sol.set_x(psi)
        its = [sol.step(ft, maxit=500, tol=1e-12)["iters"] for ft in fts]
        x = sol.get_x()
        if ref is None:
            ref = (x, its)
        else:
            assert its == ref[1]
            assert _rel(x, ref[0]) < 1e-13, ns
        sol.close()


def test_balanced_partition_mixed_precision(workdirs, native_lib):
    """Mixed precision with the balanced segments (complex64 operator cut into
    pieces too) reaches the same states as with the plain layout."""
    d, params, info, T, dt = _setup(workdirs, "tiny_nondipole")
    prob = Problem(d, info["lmax"])
    psi, _ = prob.psi0()
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in step_times(T, params["Ntime"])[1][:6]]
    out = []
    for ns in (1, 0):
        sol = Solver(prob, dt, precision="mixed")
        sol.set_split(ns)
        sol.set_x(psi)
        for ft in fts:
            sol.step(ft, maxit=500, tol=1e-10)
        out.append(sol.get_x())
        sol.close()
    assert _rel(out[1], out[0]) < 1e-8


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["tiny_dipole", "tiny_nondipole"])
def test_assembled_operator_steps_match_matrix_free(workdirs, native_lib, name, prec):
    """CN steps with the assembled couplings (sum of unit-factor values
    weighted by the step's pulse factors) match the matrix-free ones: FP64
    with the same iterations and states within summation-order differences;
    mixed precision (complex64 inner solves on the values rounded to float)
    within its tolerance."""
    d, params, info, T, dt = _setup(workdirs, name)
    prob = Problem(d, info["lmax"])
    psi, _ = prob.psi0()
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t)
           for _, t in step_times(T, params["Ntime"])[1][:8]]
    tol = 1e-12 if prec == "fp64" else 1e-10
    out = []
    for op in (0, 1):
        sol = Solver(prob, dt, precision=prec)
        sol.set_operator(op)
        sol.set_x(psi)
        its = [sol.step(ft, maxit=500, tol=tol)["iters"] for ft in fts]
        out.append((sol.get_x(), its))
        sol.close()
    if prec == "fp64":
        assert out[1][1] == out[0][1]
        assert _rel(out[1][0], out[0][0]) < 1e-12
    else:
        assert _rel(out[1][0], out[0][0]) < 1e-8


@pytest.mark.parametrize("name", ["tiny_nondipole", "dipole_small"])
def test_partitions_give_deterministic_applies(workdirs, native_lib, name):
    """Every partition (balanced segments, plain, order split) and both
    operators give the same bits for repeated applies, and A x = S x + H x
    with the parts computed apart (units cut into pieces combine their
    partial sums in a fixed order)."""
    d, params, info, T, dt = _setup(workdirs, name)
    prob = Problem(d, info["lmax"])
    sol = Solver(prob, dt)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(prob.n) + 1j * rng.standard_normal(prob.n)
    ft = pulse(params["Intensity"], params["Omega"], params["Cycles"], 0.4 * T)
    for op, splits in ((0, (0, 1, 2)), (1, (1,))):
        sol.set_operator(op)
        for ns in splits:
            if op == 0:
                sol.set_split(ns)
            sol.set_time(ft)
            y = sol.apply(x)
            _, sx, hx = sol.apply(x, parts=True)
            y3 = sol.apply(x)
            assert np.array_equal(y, y3), (op, ns)
            assert _rel(y, sx + hx) < 1e-14, (op, ns)
    sol.close()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_step_host_matches_step_sequence(workdirs, native_lib, prec):
    """gade_solver_step_host (state in and out through host memory, one
    wait in the common case) gives the same bits as set_x + step + get_x,
    also with the output aliasing the input and when continuing from the
    device state (x_in NULL)."""
    d, params, info, T, dt = _setup(workdirs, "tiny_nondipole")
    prob = Problem(d, info["lmax"])
    psi, _ = prob.psi0()
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t)
           for _, t in step_times(T, params["Ntime"])[1][:6]]
    tol = 1e-12 if prec == "fp64" else 1e-10
    a = Solver(prob, dt, precision=prec)
    b = Solver(prob, dt, precision=prec)
    xa = psi.copy()
    xb = psi.copy()
    for k, ft in enumerate(fts):
        if k < 3:
            a.set_x(xa)
            sb = b.step_host(xb, ft, maxit=500, tol=tol, x_out=xb)      # aliased in/out
        else:
            out = np.empty_like(xb)
            sb = b.step_host(None, ft, maxit=500, tol=tol, x_out=out)   # continue on the device
            xb = out
        sa = a.step(ft, maxit=500, tol=tol)
        xa = a.get_x()
        assert sa["iters"] == sb["iters"], k
        assert np.array_equal(xa, xb), k
    a.close()
    b.close()
