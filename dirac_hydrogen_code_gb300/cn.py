"""Python host mirror of the reference time loop (tools/dirac_solver.c:496-636)
running every step on the GPU through the C ABI; ``run_batch`` advances many
pulses together on one GPU.

``run()`` has the semantics of ``dirac_solver -t maxtime -l lmax -i E0
-o omega -c cycles -n Ntime``: dt = maxtime/Ntime, the loop runs
``while (time <= maxtime)`` with ``time += dt`` accumulated in floating point
(Ntime or Ntime+1 steps), f(t) is evaluated at the new time, and x<iter>.out
plus runstats.txt are written every 2000 steps.
"""
from __future__ import annotations

import math
import os
import time as _time

import numpy as np

from .formats import out_write
from .native import Problem, Solver


def pulse(E0: float, omega: float, cycles: float, t: float) -> np.ndarray:
    """beoyndDipolePulse_axialPart (tools/solver_common.c:53-65)."""
    T = cycles * 2 * math.pi / omega
    phi = -math.pi / 2
    a, b = E0 / (4 * omega), E0 / (2 * omega)
    return np.array([
        -a * math.cos(phi + t * (2 * math.pi / T + omega)),
        -a * math.sin(phi + t * (2 * math.pi / T + omega)),
        -a * math.cos(-phi + t * (2 * math.pi / T - omega)),
        a * math.sin(-phi + t * (2 * math.pi / T - omega)),
        b * math.cos(phi + t * omega),
        b * math.sin(phi + t * omega),
    ], dtype=np.complex128)


def step_times(maxtime: float, ntime: float, start_iter: int = 1):
    """(iter, t) pairs of the reference loop, with its float accumulation."""
    dt = maxtime / ntime
    t = dt * (start_iter - 1)
    it = start_iter
    out = []
    while t <= maxtime:
        t = t + dt
        out.append((it, t))
        it += 1
    return dt, out


def run(workdir: str, maxtime: float, lmax: int, E0: float, omega: float, cycles: float,
        ntime: float, tol: float = 1e-16, maxit: int = 500, start_iter: int = 1,
        precision: str = "fp64", device: int = 0, max_steps: int | None = None,
        write_outputs: bool = True, problem: Problem | None = None, x0: np.ndarray | None = None,
        callback=None, operator: int | None = None):
    """Returns (x, records, solver) with x in the solver (permuted) order.
    ``operator``: force the matrix-free (0) or assembled (1) operator
    instead of the one chosen by timing at creation."""
    prob = problem if problem is not None else Problem(workdir, lmax)
    dt, steps = step_times(maxtime, ntime, start_iter)
    solver = Solver(prob, dt, 1.0, precision=precision, device=device)
    if operator is not None:
        solver.set_operator(operator)
    psi, xperm = prob.psi0()
    solver.set_x(psi if x0 is None else x0)
    nslots = int(ntime) + 4
    itersarr = np.zeros(nslots, np.int32)
    tolsarr = np.zeros(nslots)
    timearr = np.zeros(nslots, np.int64)
    recs = []
    for it, t in steps:
        if max_steps is not None and len(recs) >= max_steps:
            break
        t0 = _time.perf_counter()
        st = solver.step(pulse(E0, omega, cycles, t), maxit=maxit, tol=tol)
        us = int((_time.perf_counter() - t0) * 1e6)
        st.update(iter=it, time=t, us=us)
        recs.append(st)
        if 0 <= it < nslots:
            itersarr[it], tolsarr[it], timearr[it] = st["iters"], st["tol_error"], us
        if callback is not None:
            callback(it, t, solver)
        if write_outputs and it % 2000 == 0:
            x = solver.get_x()
            xorig = np.empty_like(x)
            xorig[xperm] = x
            out_write(os.path.join(workdir, f"x{it}.out"), xorig)
            with open(os.path.join(workdir, "runstats.txt"), "w") as f:
                for i in range(int(ntime)):
                    f.write("%d, %e, %d\n" % (itersarr[i], tolsarr[i], timearr[i]))
    return solver.get_x(), recs, solver


def run_batch(problem: Problem, pulses: list[dict], tables: np.ndarray | None = None, tol: float = 1e-16,
              maxit: int = 500, device: int = 0, max_steps: int | None = None, callback=None,
              operator: int | None = None, **batch_kw):
    """The reference time loop for many pulses at once on one GPU.

    ``pulses``: dicts with E0, omega, cycles, ntime and optionally maxtime
    (default cycles*2*pi/omega), i.e. one ``dirac_solver -t maxtime -i E0 -o
    omega -c cycles -n ntime`` run each.  ``tables``: per-pulse radial tables
    [npulse, 6, lmax, 4, blk_nnz] (``gen.pulse_tables``) or None when every
    pulse has the Omega and Cycles the problem files were made with.  Each
    pulse keeps its own float-accumulated time grid (Ntime or Ntime+1 steps);
    a pulse whose grid has ended leaves the batch.  ``operator``: force the
    matrix-free (0) or assembled (1) operator instead of the timed choice.
    Returns (xs, records, batch): final states (permuted order) and per-pulse
    step records."""
    from .native import Batch
    grids = []
    for p in pulses:
        maxtime = p.get("maxtime", p["cycles"] * 2 * math.pi / p["omega"])
        grids.append(step_times(maxtime, p["ntime"]))
    dts = [g[0] for g in grids]
    batch = Batch(problem, dts, tables, device=device, **batch_kw)
    if operator is not None:
        batch.set_operator(operator)
    nsteps = [len(g[1]) for g in grids]
    total = max(nsteps)
    if max_steps is not None:
        total = min(total, max_steps)
    recs = [[] for _ in pulses]
    ft = np.zeros((len(pulses), 6), np.complex128)
    for j in range(total):
        active = np.array([j < n for n in nsteps], np.int32)
        for k, p in enumerate(pulses):
            if active[k]:
                ft[k] = pulse(p["E0"], p["omega"], p["cycles"], grids[k][1][j][1])
        stats = batch.step(ft, active, maxit=maxit, tol=tol)
        for k in range(len(pulses)):
            if active[k]:
                it, t = grids[k][1][j]
                stats[k].update(iter=it, time=t)
                recs[k].append(stats[k])
        if callback is not None:
            callback(j, batch)
    xs = [batch.get_x(k) for k in range(len(pulses))]
    return xs, recs, batch
