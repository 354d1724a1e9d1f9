"""Generates tests/golden/*.npz from the reference CPU build itself.

For each case the inputs are generated in the reference formats
(dirac_hydrogen_code_gb300.gen) and the reference tools/ solver, compiled in
place by oracle/build_ref.py into oracle/_ref/dirac_solver_ref, runs the time
loop with its own code.  Recorded per case: the BiCGSTAB iterations and
tol_error of every step, and the state after the last step (entire for the
small cases and the whole nondipole medium pulse; a seeded sample of 2048
entries, the L2 norm and a seeded projection for its first 20 steps; a
seeded sketch, cases.sketch, where only that is kept).  Cases with
``snap_every`` also keep, every that many steps, the sketch, the L2 norm and
the S-norm x^H S x of the state (S-norm drift through the pulse).  An input
fingerprint guards against a different generator output on another machine.

Run where the reference checkout is present (GADE_REFERENCE, see
oracle/build_ref.py) after building oracle/_ref:
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
from dirac_hydrogen_code_gb300.formats import vec_read  # noqa: E402
from dirac_hydrogen_code_gb300.gen import CONFIGS, generate  # noqa: E402
from tests.golden.cases import CASES, fingerprint, sketch  # noqa: E402

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
        if spec.get("snap_every"):
            env["GADE_REF_XSNAP_EVERY"] = str(spec["snap_every"])
        cmd = [REF, "-t", repr(T), "-l", str(info["lmax"]), "-i", str(params["Intensity"]),
               "-o", str(params["Omega"]), "-c", str(params["Cycles"]), "-n", str(params["Ntime"])]
        subprocess.run(cmd, cwd=d, env=env, check=True, stdout=subprocess.DEVNULL)
        log = np.loadtxt(os.path.join(d, "ref.log"), ndmin=2)
        x = np.fromfile(os.path.join(d, "x.bin"), np.complex128)
        out = dict(iters=log[:, 1].astype(np.int32), tol_error=log[:, 2], fingerprint=fingerprint(d, info["lmax"]),
                   x_norm=np.linalg.norm(x), n=len(x))
        rng = np.random.default_rng(1234)
        if spec.get("snap_every"):
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle as O
            S = O.overlap_from_files(d)
            psi0, _ = vec_read(os.path.join(d, "psi0.vec"))
            steps = list(range(spec["snap_every"], len(log) + 1, spec["snap_every"]))
            snaps = [np.fromfile(os.path.join(d, f"x.bin.{k}"), np.complex128) for k in steps]
            out.update(snap_steps=np.array(steps, np.int32),
                       snap_sketch=np.stack([sketch(v) for v in snaps]),
                       snap_norm=np.array([np.linalg.norm(v) for v in snaps]),
                       snap_snorm=np.array([np.vdot(v, S @ v).real for v in snaps]),
                       snorm0=np.vdot(psi0, S @ psi0).real, snorm_final=np.vdot(x, S @ x).real,
                       x_sketch=sketch(x))
            del S
        if spec.get("sketch_only"):
            pass
        elif spec.get("sample"):
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
    names = sys.argv[1:] or list(CASES)
    for name in names:
        run_case(name, CASES[name])
