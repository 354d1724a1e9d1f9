"""Recipe: compile the reference CPU solver (tools/ with USE_MPI, one rank)
from its own sources, in place under <reference>/tools, into
oracle/_ref/dirac_solver_ref.  Test infrastructure only.  The reference
checkout is taken from the GADE_REFERENCE environment variable or the first
command-line argument (default /root/reference).

The reference needs MPI, SuperLU and a Fortran-ABI BLAS, none of which is
installed, plus an x86-only SSE header.  The shims under oracle/shim/ stand
in for exactly those: a single-rank MPI header, four BLAS1 routines in C,
a prefetch stub, and the four slu_* functions backed by scipy's SuperLU
through embedded CPython (same ILU options).  The reference's own
dirac_solver.c, solver.c, csr.c, bicgstab.c, solver_common.c, utils.c and
sorted_list.c are compiled unchanged; link-time --wrap hooks
(oracle/shim/ref_hooks.c) add per-step logging, a tolerance override and
the padding of an out-of-bounds write in the reference.

Runs only where the reference sources exist (this x86 container); the
binary does not travel to other architectures.
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_tools(root: str | None = None) -> str:
    """tools/ directory of the reference checkout: the argument, else
    $GADE_REFERENCE, else /root/reference."""
    root = root or os.environ.get("GADE_REFERENCE") or "/root/reference"
    return os.path.join(root, "tools")


REF = reference_tools()
OUT = os.path.join(HERE, "_ref")
SRCS = ["dirac_solver.c", "solver.c", "csr.c", "bicgstab.c", "solver_common.c", "utils.c", "sorted_list.c"]


def build(ref: str | None = None) -> str:
    REF = reference_tools(ref) if ref else globals()["REF"]
    if not os.path.isdir(REF):
        raise FileNotFoundError(f"{REF} not present: the pinned reference oracle cannot be built here")
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "dirac_solver_ref")
    pyinc = sysconfig.get_paths()["include"]
    ldflags = subprocess.run(["python3-config", "--embed", "--ldflags"], capture_output=True,
                             text=True, check=True).stdout.split()
    cflags = ["-O2", "-w", "-fopenmp", "-DUSE_MPI", "-I", os.path.join(HERE, "shim"), "-I", REF]
    objs = []
    for src in SRCS:
        o = os.path.join(OUT, src.replace(".c", ".o"))
        subprocess.run(["gcc", *cflags, "-c", os.path.join(REF, src), "-o", o], check=True)
        objs.append(o)
    for src, extra in (("blas1.c", []), ("ref_hooks.c", []), ("slu_embed.c", ["-I", pyinc])):
        o = os.path.join(OUT, src.replace(".c", ".o"))
        subprocess.run(["gcc", *cflags, *extra, "-c", os.path.join(HERE, "shim", src), "-o", o], check=True)
        objs.append(o)
    subprocess.run(["gcc", "-o", exe, *objs, "-fopenmp", "-Wl,--wrap=bicgstab", "-Wl,--wrap=calloc",
                    *ldflags, "-lm"], check=True)
    return exe


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
