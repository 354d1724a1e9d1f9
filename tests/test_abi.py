"""CPU tests of the C ABI: the library builds/loads, exports every function
include/gade.h declares, reads inputs on the host and reports errors as
status codes.  No compute call is made (no GPU here)."""
import os
import re
import shutil

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header="gade.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gade_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(native_lib):
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(native_lib, n)]
    assert not missing, missing
    from dirac_hydrogen_code_gb300.native import _LEARNED_SIGS, _SIGS
    assert set(_SIGS) == set(names), set(names) ^ set(_SIGS)
    learned = _declared("gade_learned.h")
    assert not [n for n in learned if not hasattr(native_lib, n)]
    assert set(_LEARNED_SIGS) == set(learned), set(learned) ^ set(_LEARNED_SIGS)


def test_learned_plan_layout_matches_header(tmp_path):
    """native.LearnedGuessPlan has gade_learned_guess_plan's size and field
    offsets (a C program compiled against include/gade_learned.h)."""
    import ctypes
    import subprocess
    from dirac_hydrogen_code_gb300.native import LearnedGuessPlan
    names = [f[0] for f in LearnedGuessPlan._fields_]
    prog = ['#include <stdio.h>', '#include <stddef.h>', '#include "gade_learned.h"', 'int main(void) {',
            '  printf("%zu\\n", sizeof(gade_learned_guess_plan));']
    prog += [f'  printf("%zu\\n", offsetof(gade_learned_guess_plan, {n}));' for n in names]
    prog += ['  return 0;', '}']
    (tmp_path / "plan.c").write_text("\n".join(prog) + "\n")
    exe = str(tmp_path / "plan")
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(tmp_path / "plan.c"), "-o", exe], check=True)
    got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(LearnedGuessPlan)] + [getattr(LearnedGuessPlan, n).offset for n in names]
    assert got == want


def test_problem_load_on_host(workdirs, native_lib):
    from dirac_hydrogen_code_gb300 import formats
    from dirac_hydrogen_code_gb300.native import Problem
    d, params, info = workdirs["tiny_nondipole"]
    p = Problem(d, info["lmax"])
    assert p.info["nblk"] == info["nblk"] and p.info["blkdim"] == info["blkdim"]
    assert p.info["nnz_full"] == info["nnz_full"] and p.info["real_coupling"] == 1
    assert p.info["dkb_zero"] == 1          # the generated radial tables have the DKB zero blocks
    psi, perm = p.psi0()
    ref, rperm = formats.vec_read(os.path.join(d, "psi0.vec"))
    assert np.array_equal(psi, ref) and np.array_equal(perm, rperm)


def test_problem_load_errors(workdirs, native_lib, tmp_path):
    from dirac_hydrogen_code_gb300.native import GadeError, Problem
    d, params, info = workdirs["tiny_dipole"]
    with pytest.raises(GadeError) as e:
        Problem(str(tmp_path / "nowhere"), 1)
    assert e.value.code == 1 and "H.csr" in str(e.value)
    with pytest.raises(GadeError) as e:
        Problem(d, info["lmax"] + 1)                    # H0l<lmax>.csr does not exist
    assert e.value.code == 1
    with pytest.raises(GadeError) as e:
        Problem(d, 0)
    assert e.value.code == 4
    d2 = str(tmp_path / "trunc")
    shutil.copytree(d, d2)
    with open(os.path.join(d2, "s1.csr"), "r+b") as f:
        f.truncate(40)                                   # truncated file
    with pytest.raises(GadeError) as e:
        Problem(d2, info["lmax"])
    assert e.value.code == 2 and "s1.csr" in str(e.value)


def test_solver_without_gpu_fails_with_status(workdirs, native_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dirac_hydrogen_code_gb300.native import GadeError, Problem, Solver
    d, params, info = workdirs["tiny_dipole"]
    with pytest.raises(GadeError) as e:
        Solver(Problem(d, info["lmax"]), 1e-3)
    assert e.value.code in (3, 4)
