"""Restart tooling between the solver's two state formats.

* ``x<iter>.out`` (written every 2000 steps, tools/dirac_solver.c:579-621):
  int32 nrows, int32 ncols = 1, complex128 xorig[nrows] in the compact
  un-permuted order, xorig[xperm[i]] = x[i].
* ``psi0.vec`` (tools/main.py:141-155, read by tools/dirac_solver.c:68-108):
  int32 n, complex128 psi[n] in the solver's (permuted) order, int32 perm[n].

A run continues from step ``iter`` with ``dirac_solver ... -s iter+1`` and
either ``--restart x<iter>.out`` or a ``psi0.vec`` made by ``to-vec``.

CLI::

    python -m dirac_hydrogen_code_gb300.restart to-vec x2000.out --perm psi0.vec -o psi0_2000.vec
    python -m dirac_hydrogen_code_gb300.restart to-out psi0.vec -o x0.out
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from .formats import out_read, out_write, vec_read, vec_write


def out_to_vec(xorig: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """psi in the solver order from an x<iter>.out vector."""
    if len(xorig) != len(perm):
        raise ValueError(f"state has {len(xorig)} entries, the permutation {len(perm)}")
    return np.asarray(xorig)[perm]


def vec_to_out(psi: np.ndarray, perm: np.ndarray) -> np.ndarray:
    """x<iter>.out vector (compact un-permuted order) from psi in the solver order."""
    if len(psi) != len(perm):
        raise ValueError(f"state has {len(psi)} entries, the permutation {len(perm)}")
    xorig = np.empty(len(psi), np.complex128)
    xorig[perm] = psi
    return xorig


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m dirac_hydrogen_code_gb300.restart")
    sub = ap.add_subparsers(dest="cmd", required=True)
    a = sub.add_parser("to-vec", help="x<iter>.out -> psi0.vec")
    a.add_argument("out")
    a.add_argument("--perm", required=True, help="a psi0.vec of the same problem (its permutation is kept)")
    a.add_argument("-o", "--output", required=True)
    b = sub.add_parser("to-out", help="psi0.vec -> x<iter>.out")
    b.add_argument("vec")
    b.add_argument("-o", "--output", required=True)
    args = ap.parse_args(argv)
    if args.cmd == "to-vec":
        _, perm = vec_read(args.perm)
        vec_write(args.output, out_to_vec(out_read(args.out), perm), perm)
    else:
        psi, perm = vec_read(args.vec)
        out_write(args.output, vec_to_out(psi, perm))
    return 0


if __name__ == "__main__":
    sys.exit(main())
