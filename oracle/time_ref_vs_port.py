"""Recipe: per-step wall time of the compiled reference CPU build
(oracle/_ref/dirac_solver_ref, tools/ compiled in place) against the oracle
port (oracle/oracle.py) on the same generated inputs and the same steps of
the same pulse.  Test infrastructure only; it checks that the port timed by
bench.py's CPU legs (the reference sources do not reach every machine) is a
fair stand-in for the reference build.

    python oracle/time_ref_vs_port.py [steps] [skip]

A reference step is timed by the wall clock between the ends of two
consecutive BiCGSTAB calls (the link-time hook logs it), i.e. its assembly,
right-hand side and solve, like the port's per-step timer.  The first `skip`
steps are left out of both means.  OpenMP (the reference's assembly) and the
port's BLAS use every host thread.
"""
import json
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
import oracle as O  # noqa: E402
from dirac_hydrogen_code_gb300.gen import CONFIGS, generate  # noqa: E402

REF = os.path.join(HERE, "_ref", "dirac_solver_ref")


def time_case(name, steps, skip, tol=1e-12):
    params = CONFIGS[name]
    with tempfile.TemporaryDirectory() as d:
        info = generate(params, d)
        T = params["Cycles"] * 2 * math.pi / params["Omega"]
        env = dict(os.environ, GADE_REF_TOL=repr(tol), GADE_REF_MAXIT="500", GADE_REF_LOG=os.path.join(d, "ref.log"),
                   GADE_REF_MAXSTEPS=str(steps + skip), OMP_NUM_THREADS=str(os.cpu_count()),
                   MAT_NUM_THREADS=str(os.cpu_count()))
        cmd = [REF, "-t", repr(T), "-l", str(info["lmax"]), "-i", str(params["Intensity"]), "-o",
               str(params["Omega"]), "-c", str(params["Cycles"]), "-n", str(params["Ntime"])]
        subprocess.run(cmd, cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        log = np.loadtxt(os.path.join(d, "ref.log"), ndmin=2)
        wall = log[:, 4] * 1e-6
        ref_steps = np.diff(wall)[skip - 1:]               # step k ends at wall[k]
        _, recs, _ = O.run(d, T, info["lmax"], params["Intensity"], params["Omega"], params["Cycles"],
                           params["Ntime"], tol=tol, maxit=500, precond="ilu", max_steps=steps + skip)
        port_steps = np.array([r.elapsed for r in recs[skip:]])
        iters_ref = log[skip:, 1].astype(int).tolist()
        iters_port = [r.iters for r in recs[skip:]]
    return {"workload": name, "steps": len(ref_steps), "skip": skip,
            "reference_s_per_step": float(ref_steps.mean()), "port_s_per_step": float(port_steps.mean()),
            "port_over_reference": float(port_steps.mean() / ref_steps.mean()),
            "same_iterations": iters_ref == iters_port, "threads": os.cpu_count()}


if __name__ == "__main__":
    if not os.path.exists(REF):
        sys.exit("build oracle/_ref first: python oracle/build_ref.py")
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 20
    skip = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    for name in ("dipole_small", "nondipole_medium"):
        print(json.dumps(time_case(name, steps, skip)))
