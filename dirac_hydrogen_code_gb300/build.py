"""Builds the native parts in-tree, for sm_103a only.

Outputs (git-ignored) in ``dirac_hydrogen_code_gb300/lib/``:

* ``libgade_gb300.so`` — the C ABI of ``include/gade.h`` (host set-up in C,
  kernels in CUDA);
* ``dirac_solver``     — the drop-in executable (same CLI and files as the
  reference tools/dirac_solver).

Translation units are compiled in parallel; a full build takes a few
seconds.  No cmake, no torch extension machinery.  GADE_NVCC_FLAGS adds
flags to the CUDA compilation of the solver (tuning builds, e.g.
-DA32_NST=4 for the stages of the complex64 assembled apply).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the GB300 path")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    bad = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            bad.append(" ".join(c) + "\n" + out)
        elif out.strip():
            sys.stderr.write(out)
    if bad:
        raise RuntimeError("native build failed:\n" + "\n".join(bad))


def library_path() -> str:
    return os.path.join(LIB, "libgade_gb300.so")


def solver_path() -> str:
    return os.path.join(LIB, "dirac_solver")


def is_stale() -> bool:
    """True when the library or the executable is missing or older than a
    source file or header."""
    outs = [library_path(), solver_path()]
    if not all(os.path.exists(o) for o in outs):
        return True
    built = min(os.path.getmtime(o) for o in outs)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(f) > built for f in srcs)


def build(verbose: bool = False) -> str:
    os.makedirs(LIB, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    cuda_lib = os.path.join(_cuda_home(), "lib64")
    objs = {
        "gade_host.o": ["gcc", "-O3", "-std=gnu11", "-fPIC", "-Wall", "-Wno-unused-function",
                        "-I", INCLUDE, "-c", os.path.join(CSRC, "gade_host.c")],
        "gade_cuda.o": [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                        *os.environ.get("GADE_NVCC_FLAGS", "").split(),
                        "-I", INCLUDE, "-c", os.path.join(CSRC, "gade_cuda.cu")],
        "gade_learned.o": [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                           "-I", INCLUDE, "-c", os.path.join(CSRC, "gade_learned.cu")],
        "dirac_solver.o": ["gcc", "-O3", "-std=gnu11", "-Wall", "-I", INCLUDE, "-c",
                           os.path.join(CSRC, "dirac_solver.c")],
    }
    cmds = [c + ["-o", os.path.join(LIB, o)] for o, c in objs.items()]
    _run_all(cmds)
    lib = library_path()
    _run_all([[nvcc, *ARCH, "-shared", "-o", lib, os.path.join(LIB, "gade_host.o"),
               os.path.join(LIB, "gade_cuda.o"), os.path.join(LIB, "gade_learned.o"), "-lcudart", "-lm"]])
    _run_all([["gcc", "-o", solver_path(), os.path.join(LIB, "dirac_solver.o"), "-L", LIB,
               "-lgade_gb300", "-Wl,-rpath,$ORIGIN", "-L", cuda_lib, "-Wl,-rpath," + cuda_lib,
               "-lcudart", "-lm"]])
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)
