"""CPU test of the binding a maintainer adds to the reference's host loop
(the C snippet of INTEGRATION.md section 2): the reference's own
tools/dirac_solver.c, with each of its GPU blocks (the
``#if defined USE_CUDA | defined USE_HIP`` sections) replaced by the
include/gade.h calls below, compiles against include/gade.h, links
libgade_gb300.so and the reference's other translation units (built in place
by oracle/build_ref.py), and runs its set-up up to the device: the inputs
load, and without a GPU the solver creation reports the CUDA error through
gade_last_error().  The patched copy lives in a temporary directory; nothing
of the reference is committed.  Skipped where the reference checkout or its
oracle build is absent.
"""
import os
import subprocess
import sys
import sysconfig

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# replacement of each GPU block of tools/dirac_solver.c, in file order
GADE_BLOCKS = [
    # the GPU headers
    '#include "gade.h"\n',
    # gpu_HS_spmv_fun / gpu_LU_precond_fun callbacks: not needed
    '',
    # gpu_init_model_matrices / gpu_compute_row_col: the solver builds its tables itself
    '',
    # GPU set-up after the preconditioner (dt is known)
    '    gade_problem *gp = NULL;\n'
    '    gade_solver *gs = NULL;\n'
    '    if (gade_problem_load(".", lmax, &gp)) ERROR("%s\\n", gade_last_error());\n'
    '    if (gade_solver_create(gp, dt, h, GADE_PREC_FP64, 0, &gs)) ERROR("%s\\n", gade_last_error());\n'
    '    if (gade_solver_set_x(gs, (const double *)(x + csr_local_rowoffset(&Hfull)), csr_nrows(&Hfull)))\n'
    '        ERROR("%s\\n", gade_last_error());\n',
    # the BiCGSTAB workspace: the CPU type stays (unused)
    None,
    # the loop body: assembly, rhs and BiCGSTAB in one call
    '        {\n'
    '            gade_step_stats st;\n'
    '            tic();\n'
    '            if (gade_solver_step(gs, (const double *)ft, iters, tol_error, &st))\n'
    '                ERROR("%s\\n", gade_last_error());\n'
    '            toc_output(&bicgtime);\n'
    '            iters = st.iters;\n'
    '            tol_error = st.tol_error;\n'
    '        }\n',
    # output every 2000 steps
    '            if (gade_solver_get_x(gs, (double *)(x + csr_local_rowoffset(&Hfull)), csr_nrows(&Hfull)))\n'
    '                ERROR("%s\\n", gade_last_error());\n',
]


def patch_gpu_blocks(src: str) -> str:
    """Replaces the i-th GPU block with GADE_BLOCKS[i] (None: keep its
    #else branch)."""
    lines = src.splitlines(keepends=True)
    out, i, nblock = [], 0, 0
    while i < len(lines):
        if lines[i].strip() == "#if defined USE_CUDA | defined USE_HIP":
            depth, j, els = 1, i + 1, None
            while depth:
                t = lines[j].strip()
                if t.startswith("#if"):
                    depth += 1
                elif t.startswith("#endif"):
                    depth -= 1
                elif t.startswith("#else") and depth == 1:
                    els = j
                j += 1
            rep = GADE_BLOCKS[nblock]
            if rep is None:
                out.extend(lines[els + 1:j - 1])
            else:
                out.append(rep)
            nblock += 1
            i = j
            continue
        out.append(lines[i])
        i += 1
    assert nblock == len(GADE_BLOCKS), f"expected {len(GADE_BLOCKS)} GPU blocks, found {nblock}"
    return "".join(out)


def test_reference_loop_binds_the_c_abi(tmp_path, native_lib):
    import build_ref
    tools = build_ref.reference_tools()
    objs_dir = os.path.join(ROOT, "oracle", "_ref")
    others = ["solver.o", "csr.o", "bicgstab.o", "solver_common.o", "utils.o", "sorted_list.o",
              "blas1.o", "slu_embed.o"]
    if not os.path.isdir(tools) or not all(os.path.exists(os.path.join(objs_dir, o)) for o in others):
        pytest.skip("reference checkout or its oracle build absent")
    src = open(os.path.join(tools, "dirac_solver.c")).read()
    patched = tmp_path / "dirac_solver_gade.c"
    patched.write_text(patch_gpu_blocks(src))
    shim = os.path.join(ROOT, "oracle", "shim")
    inc = os.path.join(ROOT, "include")
    lib = os.path.join(ROOT, "dirac_hydrogen_code_gb300", "lib")
    exe = str(tmp_path / "dirac_solver_gade")
    obj = str(tmp_path / "dirac_solver_gade.o")
    cc = subprocess.run(["gcc", "-O1", "-w", "-fopenmp", "-DUSE_MPI", "-I", shim, "-I", inc, "-I", tools, "-c",
                         str(patched), "-o", obj], capture_output=True, text=True)
    assert cc.returncode == 0, cc.stderr[-3000:]
    py_ld = subprocess.run(["python3-config", "--embed", "--ldflags"], capture_output=True, text=True,
                           check=True).stdout.split()
    from dirac_hydrogen_code_gb300 import build
    cuda_lib = os.path.join(build._cuda_home(), "lib64")
    ld = subprocess.run(["gcc", "-o", exe, obj, *[os.path.join(objs_dir, o) for o in others], "-fopenmp",
                         "-L", lib, "-lgade_gb300", f"-Wl,-rpath,{lib}", "-L", cuda_lib, f"-Wl,-rpath,{cuda_lib}",
                         "-lcudart", *py_ld, "-lm"], capture_output=True, text=True)
    assert ld.returncode == 0, ld.stderr[-3000:]
    # run its set-up on a small generated problem
    from dirac_hydrogen_code_gb300.gen import generate
    params = dict(Nsplines=20, Ntime=40, Nkappa=2, Nmu=0, Nl=1, rBox=30.0, Intensity=10, Omega=50.0, Cycles=1, Z=1)
    work = tmp_path / "run"
    info = generate(params, str(work))
    env = dict(os.environ, PYTHONPATH=os.pathsep.join(sys.path), OMP_NUM_THREADS="1")
    r = subprocess.run([exe, "-t", "0.12566370614359174", "-l", str(info["lmax"]), "-i", "10", "-o", "50",
                        "-c", "1", "-n", "40"], cwd=str(work), capture_output=True, text=True, env=env,
                       timeout=300)
    out = r.stdout + r.stderr
    assert "All matrices read correctly" in out, out[-2000:]
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:
        gpu = False
    if not gpu:
        # gade_solver_create reports the missing device through gade_last_error()
        assert r.returncode != 0 and ("CUDA" in out or "cuda" in out), out[-2000:]
