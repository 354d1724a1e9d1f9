"""Generates tests/golden/*.npz from the reference CPU build itself.

For each case the inputs are generated in the reference formats
(dirac_hydrogen_code_gb300.gen) and the reference tools/ solver, compiled in
place by oracle/build_ref.py into oracle/_ref/dirac_solver_ref, runs the time
loop with its own code.  Recorded per case: the BiCGSTAB iterations and
tol_error of every step, and the state after the last step (entire for the
small cases; a seeded sample of 2048 entries, the L2 norm and a seeded
projection for the nondipole medium case).  An input fingerprint guards
against a different generator output on another machine.

Run here (needs /root/reference and a built oracle/_ref):
    python tests/golden/make_golden.py
"""
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from dirac_hydrogen_code_gb300.gen import CONFIGS, generate  # noqa: E402
from tests.golden.cases import CASES, fingerprint  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "dirac_solver_ref")


def run_case(name, spec):
    params = spec["params"]
    with tempfile.TemporaryDirectory() as d:
        info = generate(params, d)
        T = params["Cycles"] * 2 * math.pi / params["Omega"]
        env = dict(os.environ, GADE_REF_TOL=repr(spec["tol"]), GADE_REF_MAXIT=str(spec["maxit"]),
                   GADE_REF_LOG=os.path.join(d, "ref.log"), GADE_REF_XOUT=os.path.join(d, "x.bin"),
                   OMP_NUM_THREADS=str(os.cpu_count()))
        if spec.get("max_steps"):
            env["GADE_REF_MAXSTEPS"] = str(spec["max_steps"])
        cmd = [REF, "-t", repr(T), "-l", str(info["lmax"]), "-i", str(params["Intensity"]),
               "-o", str(params["Omega"]), "-c", str(params["Cycles"]), "-n", str(params["Ntime"])]
        subprocess.run(cmd, cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        log = np.loadtxt(os.path.join(d, "ref.log"), ndmin=2)
        x = np.fromfile(os.path.join(d, "x.bin"), np.complex128)
        out = dict(iters=log[:, 1].astype(np.int32), tol_error=log[:, 2], fingerprint=fingerprint(d, info["lmax"]),
                   x_norm=np.linalg.norm(x), n=len(x))
        rng = np.random.default_rng(1234)
        if spec.get("sample"):
            idx = np.sort(rng.choice(len(x), 2048, replace=False))
            proj = rng.standard_normal(len(x)) + 1j * rng.standard_normal(len(x))
            out.update(x_idx=idx, x_sample=x[idx], x_proj=np.vdot(proj, x))
        else:
            out.update(x=x)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "steps", len(log), "iters", sorted(set(out["iters"].tolist())), "|x|", out["x_norm"])


if __name__ == "__main__":
    if not os.path.exists(REF):
        sys.exit("build oracle/_ref first: python oracle/build_ref.py")
    for name, spec in CASES.items():
        run_case(name, spec)
