"""ctypes binding of ``libgade_gb300.so`` (include/gade.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared library is missing or does not export the ABI.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import build as _build

GADE_PREC_FP64 = 0
GADE_PREC_MIXED = 1


class GadeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gade error {code}: {msg}")
        self.code = code


class ProblemInfo(C.Structure):
    _fields_ = [("lmax", C.c_int32), ("nblk", C.c_int32), ("blkdim", C.c_int32), ("blk_nnz", C.c_int32),
                ("n", C.c_int64), ("hall_nnz", C.c_int64), ("nnz_full", C.c_int64),
                ("real_coupling", C.c_int32), ("dkb_zero", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("iters", C.c_int32), ("tol_error", C.c_double), ("restarts", C.c_int32),
                ("refinements", C.c_int32), ("inner_iters", C.c_int32), ("true_residual", C.c_double),
                ("snorm", C.c_double), ("init_residual", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class KernelTimes(C.Structure):
    _fields_ = [("apply_launches", C.c_int64), ("apply_ms", C.c_double),
                ("precond_launches", C.c_int64), ("precond_ms", C.c_double),
                ("other_launches", C.c_int64), ("other_ms", C.c_double)]


class BatchOptions(C.Structure):
    _fields_ = [("chunk_splines", C.c_int32), ("iters_per_launch", C.c_int32), ("use_graphs", C.c_int32)]


class BatchInfo(C.Structure):
    _fields_ = [("npulse", C.c_int32), ("active", C.c_int32), ("chunk_splines", C.c_int32),
                ("iters_per_launch", C.c_int32), ("graph_replays", C.c_int64), ("steps", C.c_int64),
                ("ntune", C.c_int32), ("tune_cs", C.c_int32 * 4), ("tune_ms", C.c_float * 4),
                ("apply_flops", C.c_double)]


_LIB = None

# every entry point of include/gade.h with its ctypes signature
_SIGS = {
    "gade_last_error": (C.c_char_p, []),
    "gade_problem_load": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "gade_problem_get_info": (C.c_int, [C.c_void_p, C.POINTER(ProblemInfo)]),
    "gade_problem_get_psi0": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gade_problem_get_blocks": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gade_problem_free": (None, [C.c_void_p]),
    "gade_solver_create": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_void_p)]),
    "gade_solver_free": (None, [C.c_void_p]),
    "gade_solver_set_x": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "gade_solver_get_x": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "gade_solver_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.POINTER(StepStats)]),
    "gade_solver_step_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_void_p,
                                        C.POINTER(StepStats)]),
    "gade_solver_set_time": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gade_solver_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gade_solver_precond": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gade_solver_apply_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gade_solver_launch_count": (C.c_int64, [C.c_void_p]),
    "gade_solver_time_apply": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "gade_solver_time_precond": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "gade_solver_time_apply_mixed": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "gade_solver_stream": (C.c_void_p, [C.c_void_p]),
    "gade_solver_profile": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(KernelTimes)]),
    "gade_probe_fp64_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
    "gade_solver_flops": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gade_solver_split": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]),
    "gade_solver_set_split": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_apply_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "gade_solver_set_operator": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_batch_operator": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]),
    "gade_batch_set_operator": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_assembly_cost": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "gade_solver_operator": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_void_p]),
    "gade_solver_balanced": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "gade_solver_apply_dot_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                                C.c_void_p]),
    "gade_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_double, C.c_int32,
                                    C.c_int32, C.POINTER(BatchOptions), C.POINTER(C.c_void_p)]),
    "gade_batch_free": (None, [C.c_void_p]),
    "gade_batch_set_x": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "gade_batch_get_x": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "gade_batch_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                  C.POINTER(StepStats)]),
    "gade_batch_get_info": (C.c_int, [C.c_void_p, C.POINTER(BatchInfo)]),
    "gade_batch_stream": (C.c_void_p, [C.c_void_p]),
    "gade_batch_state_device": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "gade_batch_guess_buffer": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "gade_batch_use_guess": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_set_wait_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
    "gade_solver_restart": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "gade_solver_inject_wait_timeout": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_set_precond_warps": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_set_residual_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_solver_residual_precision": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "gade_batch_set_residual_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "gade_batch_set_wait_limit": (C.c_int, [C.c_void_p, C.c_uint32]),
}

# include/gade_learned.h (device pointers as integers)
_P = C.c_void_p


class LearnedGuessPlan(C.Structure):
    """gade_learned_guess_plan (include/gade_learned.h), field for field."""
    _fields_ = [("n", C.c_int32), ("R", C.c_int32), ("npulse", C.c_int32), ("K", C.c_int32),
                ("din", C.c_int32), ("dh", C.c_int32), ("dout", C.c_int32),
                ("U", _P), ("hist", _P), ("x", _P), ("ldx", C.c_int64), ("scratch", _P),
                ("scratch_bytes", C.c_int64), ("mu_in", _P), ("sd_in", _P), ("mu_out", _P), ("sd_out", _P),
                ("x16", _P), ("W16", _P * 3), ("bias", _P * 3), ("H1", _P), ("H2", _P), ("out", _P),
                ("H1_16", _P), ("H2_16", _P), ("c", _P), ("scale", _P), ("corr", _P), ("ldcorr", C.c_int64),
                ("limit", C.c_float)]


_LEARNED_SIGS = {
    "gade_gemm_bf16": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, C.c_int64, C.c_int64, _P, C.c_int64,
                                 C.c_int64, _P, _P, C.c_int64, C.c_int32, _P, C.c_int64, _P, C.c_int64, _P]),
    "gade_learned_status": (C.c_int, [C.POINTER(C.c_int32)]),
    "gade_learned_guess_step": (C.c_int, [C.POINTER(LearnedGuessPlan), C.c_int32, _P, _P]),
    "gade_gemm_bf16_path": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, C.c_int64, C.c_int64, _P, C.c_int64,
                                      C.c_int64]),
    "gade_learned_set_gemm_options": (C.c_int, [C.c_int32, C.c_uint32, C.c_int32]),
    "gade_mse_grad": (C.c_int, [C.c_int32, C.c_int32, _P, _P, _P, _P, _P, _P]),
    "gade_colsum": (C.c_int, [C.c_int32, C.c_int32, _P, C.c_int64, _P, _P]),
    "gade_adam": (C.c_int, [C.c_int64, _P, _P, _P, _P, _P, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.c_int32, _P]),
    "gade_to_bf16": (C.c_int, [C.c_int64, _P, _P, _P]),
    "gade_pod_project": (C.c_int, [C.c_int64, C.c_int32, _P, _P, C.c_int64, C.c_int32, _P, _P, C.c_int64, _P]),
    "gade_pod_project_scratch": (C.c_int64, [C.c_int64, C.c_int32, C.c_int32]),
    "gade_pod_project_fp64": (C.c_int, [C.c_int64, C.c_int32, _P, _P, C.c_int64, C.c_int32, _P, _P, C.c_int64, _P]),
    "gade_pod_expand": (C.c_int, [C.c_int64, C.c_int32, _P, _P, _P, C.c_int32, _P, C.c_int64, _P]),
    "gade_learned_features": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P, _P, _P, _P]),
    "gade_learned_outputs": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P, C.c_float,
                                       _P, _P, _P]),
    "gade_eigproj": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, C.c_double, _P, C.c_int64, _P, _P,
                               _P]),
}


def library_path() -> str:
    return _build.library_path()


def load_library() -> C.CDLL:
    """Load libgade_gb300.so; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise GadeError(-1, f"{path} is missing: run dirac_hydrogen_code_gb300.build.build() "
                            "(or __graft_entry__.build()) first; there is no fallback path")
    lib = C.CDLL(path)
    for name, (res, args) in list(_SIGS.items()) + list(_LEARNED_SIGS.items()):
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int):
    if rc != 0:
        msg = load_library().gade_last_error().decode(errors="replace")
        raise GadeError(rc, msg)


def _cbuf(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


class Problem:
    """Host copy of the solver inputs (tools/dirac_solver.c:223-388)."""

    def __init__(self, workdir: str, lmax: int):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.gade_problem_load(os.fsencode(workdir), int(lmax), C.byref(h)))
        self._h = h
        self.workdir = workdir
        info = ProblemInfo()
        _check(lib.gade_problem_get_info(h, C.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in ProblemInfo._fields_}
        self.n = int(info.n)

    def blocks(self) -> tuple[np.ndarray, np.ndarray]:
        """(kappa, original angular index) of every block row."""
        nblk = int(self.info["nblk"])
        kap = np.empty(nblk, np.int32)
        ang = np.empty(nblk, np.int32)
        _check(load_library().gade_problem_get_blocks(self._h, kap.ctypes.data, ang.ctypes.data))
        return kap, ang

    def psi0(self) -> tuple[np.ndarray, np.ndarray]:
        psi = np.empty(self.n, np.complex128)
        perm = np.empty(self.n, np.int32)
        _check(load_library().gade_problem_get_psi0(self._h, psi.ctypes.data, perm.ctypes.data))
        return psi, perm

    def close(self):
        if getattr(self, "_h", None):
            load_library().gade_problem_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Device solver of one pulse; mirrors the reference GPU interface
    (gpu_solver.h, gpu_sparse.h, gpu_bicgstab.h) through include/gade.h."""

    def __init__(self, problem: Problem, dt: float, h: float = 1.0, precision: str = "fp64",
                 device: int = 0):
        lib = load_library()
        prec = {"fp64": GADE_PREC_FP64, "mixed": GADE_PREC_MIXED}[precision]
        hs = C.c_void_p()
        _check(lib.gade_solver_create(problem._h, float(dt), float(h), prec, int(device), C.byref(hs)))
        self._h = hs
        self.n = problem.n
        self.problem = problem

    # gpu_put_vec / gpu_get_vec
    def set_x(self, x: np.ndarray):
        x = _cbuf(x)
        if x.shape != (self.n,):
            raise ValueError(f"state must have {self.n} entries")
        _check(load_library().gade_solver_set_x(self._h, x.ctypes.data, self.n))

    def get_x(self) -> np.ndarray:
        x = np.empty(self.n, np.complex128)
        _check(load_library().gade_solver_get_x(self._h, x.ctypes.data, self.n))
        return x

    def restart(self, x: np.ndarray):
        """New pulse on this solver: state x, nothing carried over from the
        previous steps (BiCGSTAB's p and v, the extrapolation history)."""
        x = _cbuf(x)
        if x.shape != (self.n,):
            raise ValueError(f"state must have {self.n} entries")
        _check(load_library().gade_solver_restart(self._h, x.ctypes.data, self.n))

    # pgsum part of gpu_compute_timedep_matrices
    def set_time(self, ft: np.ndarray):
        ft = _cbuf(ft)
        _check(load_library().gade_solver_set_time(self._h, ft.ctypes.data))

    # gpu_HS_spmv_fun
    def apply(self, x: np.ndarray, parts: bool = False):
        x = _cbuf(x)
        y = np.empty(self.n, np.complex128)
        if parts:
            sx = np.empty(self.n, np.complex128)
            hx = np.empty(self.n, np.complex128)
            _check(load_library().gade_solver_apply(self._h, x.ctypes.data, y.ctypes.data,
                                                    sx.ctypes.data, hx.ctypes.data))
            return y, sx, hx
        _check(load_library().gade_solver_apply(self._h, x.ctypes.data, y.ctypes.data, None, None))
        return y

    # gpu_LU_precond_fun
    def precond(self, b: np.ndarray) -> np.ndarray:
        b = _cbuf(b)
        z = np.empty(self.n, np.complex128)
        _check(load_library().gade_solver_precond(self._h, b.ctypes.data, z.ctypes.data))
        return z

    # loop body of tools/dirac_solver.c:503-551
    def step(self, ft: np.ndarray, maxit: int = 500, tol: float = 1e-16) -> dict:
        ft = _cbuf(ft)
        st = StepStats()
        _check(load_library().gade_solver_step(self._h, ft.ctypes.data, int(maxit), float(tol), C.byref(st)))
        return st.as_dict()

    def step_host(self, x_in, ft: np.ndarray, maxit: int = 500, tol: float = 1e-16, x_out=None) -> dict:
        """One step with the state in host memory: x_in (complex128 [n] or a
        host address, None to continue from the device state) in, the new
        state out to x_out (array or host address, None: not copied)."""
        ft = _cbuf(ft)
        st = StepStats()
        if isinstance(x_in, np.ndarray):
            x_in = _cbuf(x_in)
            if x_in.shape != (self.n,):
                raise ValueError(f"x_in must have {self.n} entries")
        if isinstance(x_out, np.ndarray):
            if x_out.dtype != np.complex128 or x_out.shape != (self.n,) or not x_out.flags.c_contiguous:
                raise ValueError(f"x_out must be a contiguous complex128 array of {self.n} entries")
        pin = x_in.ctypes.data if isinstance(x_in, np.ndarray) else x_in
        pout = x_out.ctypes.data if isinstance(x_out, np.ndarray) else x_out
        _check(load_library().gade_solver_step_host(self._h, pin, ft.ctypes.data, int(maxit), float(tol), pout,
                                                    C.byref(st)))
        return st.as_dict()

    def apply_device(self, x_ptr: int, y_ptr: int, stream: int = 0):
        _check(load_library().gade_solver_apply_device(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr),
                                                       C.c_void_p(stream) if stream else None))

    def apply_dot_noalloc(self, x_ptr: int, r0_ptr: int, y_ptr: int, dot_ptr: int, stream: int = 0):
        """y = (S + H(t)) x and dot = <r0, y> on device buffers, without any
        device allocation (scratch in a fixed array inside the library)."""
        _check(load_library().gade_solver_apply_dot_noalloc(
            self._h, C.c_void_p(x_ptr), C.c_void_p(r0_ptr), C.c_void_p(y_ptr), C.c_void_p(dot_ptr),
            C.c_void_p(stream) if stream else None))

    def launch_count(self) -> int:
        return int(load_library().gade_solver_launch_count(self._h))

    def time_apply(self, reps: int = 20) -> float:
        ms = C.c_double()
        _check(load_library().gade_solver_time_apply(self._h, int(reps), C.byref(ms)))
        return ms.value

    def time_apply_mixed(self, reps: int = 20) -> float:
        """Average ms of the complex64 inner-solve apply (mixed precision)."""
        ms = C.c_double()
        _check(load_library().gade_solver_time_apply_mixed(self._h, int(reps), C.byref(ms)))
        return ms.value

    def time_precond(self, reps: int = 20) -> float:
        ms = C.c_double()
        _check(load_library().gade_solver_time_precond(self._h, int(reps), C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        return int(load_library().gade_solver_stream(self._h) or 0)

    def profile(self, enable: bool = True):
        _check(load_library().gade_solver_profile(self._h, 1 if enable else 0))

    def kernel_times(self) -> dict:
        kt = KernelTimes()
        _check(load_library().gade_solver_kernel_times(self._h, C.byref(kt)))
        return {k: getattr(kt, k) for k, _ in KernelTimes._fields_}

    def split(self) -> tuple[int, list[float]]:
        """(partition of the operator kernel: 0 balanced, 1-4 order split;
        timed apply ms for 1-4 splits)."""
        ns = C.c_int32()
        ms = (C.c_float * 4)()
        _check(load_library().gade_solver_split(self._h, C.byref(ns), ms))
        return int(ns.value), [float(v) for v in ms]

    def set_split(self, nsplit: int):
        _check(load_library().gade_solver_set_split(self._h, int(nsplit)))

    def balanced(self) -> dict:
        """Balanced partition of the FP64 operator: segments (CTAs), pieces, timed ms."""
        seg, pcs, ms, gw = C.c_int32(), C.c_int32(), C.c_float(), C.c_double()
        _check(load_library().gade_solver_balanced(self._h, C.byref(seg), C.byref(pcs), C.byref(ms), C.byref(gw)))
        return {"segments": int(seg.value), "pieces": int(pcs.value), "ms": float(ms.value),
                "gather_weight": float(gw.value)}

    def operator(self) -> dict:
        """Operator in use (0 matrix-free, 1 assembled) and the timed FP64
        applies: matrix-free, assembled with the plain and the balanced partition."""
        a = C.c_int32()
        ms = (C.c_float * 5)()
        _check(load_library().gade_solver_operator(self._h, C.byref(a), ms))
        return {"assembled": int(a.value), "matrix_free_ms": float(ms[0]),
                "assembled_plain_ms": float(ms[1]), "assembled_balanced_ms": float(ms[2]),
                "tables_ms": float(ms[3]), "assembly_ms": float(ms[4])}

    def set_operator(self, assembled: int):
        _check(load_library().gade_solver_set_operator(self._h, int(assembled)))

    def set_wait_limit(self, polls: int = 0):
        """Polls of each preconditioner stage wait before the step gives up
        with GADE_ERR_CUDA (0: the default)."""
        _check(load_library().gade_solver_set_wait_limit(self._h, int(polls)))

    def set_precond_warps(self, warps: int):
        """Warps per block row of the block-LU solves: 8 (default) or 4."""
        _check(load_library().gade_solver_set_precond_warps(self._h, int(warps)))

    def set_residual_precision(self, mode: int):
        """Mixed precision: the refinement residual on the FP64 units (0) or
        in double-float on the FP32 units (1, the default where available)."""
        _check(load_library().gade_solver_set_residual_precision(self._h, int(mode)))

    def residual_precision(self) -> dict:
        m, u = C.c_int32(), C.c_int32()
        _check(load_library().gade_solver_residual_precision(self._h, C.byref(m), C.byref(u)))
        return {"mode": int(m.value), "double_float_in_use": bool(u.value)}

    def inject_wait_timeout(self, stage: int = -1):
        """Tests of the failure path: the preconditioner kernel withholds the
        copy of this stage so that its wait runs out (-1: off)."""
        _check(load_library().gade_solver_inject_wait_timeout(self._h, int(stage)))

    def assembly_cost(self) -> tuple[float, float]:
        """(FP64 flops, compulsory DRAM bytes) of one step's coupling assembly."""
        f, b = C.c_double(), C.c_double()
        _check(load_library().gade_solver_assembly_cost(self._h, C.byref(f), C.byref(b)))
        return float(f.value), float(b.value)

    def apply_bytes(self) -> float:
        """Compulsory DRAM bytes of one FP64 BiCGSTAB operator apply."""
        b = C.c_double()
        _check(load_library().gade_solver_apply_bytes(self._h, C.byref(b)))
        return float(b.value)

    def flops(self) -> tuple[float, float]:
        """(FP64 flops of one operator apply, of one preconditioner solve)."""
        a, b = C.c_double(), C.c_double()
        _check(load_library().gade_solver_flops(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            load_library().gade_solver_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fp64_peak_tflops(device: int = 0) -> float:
    """Measured FP64 FMA throughput (TFLOP/s) of the device."""
    v = C.c_double()
    _check(load_library().gade_probe_fp64_peak(int(device), C.byref(v)))
    return v.value


class Batch:
    """Many pulses on one problem's angular tables, h0 and S (gade_batch_*).

    ``dts``: time step of each pulse; ``g``: None (all pulses use the
    problem's radial tables) or a complex128 array [npulse, 6, lmax, 4,
    blk_nnz] in the loader's layout (see ``gen.pulse_tables``)."""

    def __init__(self, problem: Problem, dts, g: np.ndarray | None = None, h: float = 1.0,
                 precision: str = "fp64", device: int = 0, chunk_splines: int = 0,
                 iters_per_launch: int = 0, use_graphs: bool = True):
        lib = load_library()
        prec = {"fp64": GADE_PREC_FP64, "mixed": GADE_PREC_MIXED}[precision]
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        self.npulse = int(dts.size)
        gp = None
        if g is not None:
            g = _cbuf(g)
            info = problem.info
            want = (self.npulse, 6, info["lmax"], 4, info["blk_nnz"])
            if g.shape != want:
                raise ValueError(f"radial tables must have shape {want}, got {g.shape}")
            gp = g.ctypes.data
        opt = BatchOptions(int(chunk_splines), int(iters_per_launch), 1 if use_graphs else 0)
        hb = C.c_void_p()
        _check(lib.gade_batch_create(problem._h, self.npulse, dts.ctypes.data, gp, float(h), prec, int(device),
                                     C.byref(opt), C.byref(hb)))
        self._h = hb
        self.n = problem.n
        self.problem = problem

    def set_x(self, pulse: int, x: np.ndarray):
        x = _cbuf(x)
        if x.shape != (self.n,):
            raise ValueError(f"state must have {self.n} entries")
        _check(load_library().gade_batch_set_x(self._h, int(pulse), x.ctypes.data, self.n))

    def get_x(self, pulse: int) -> np.ndarray:
        x = np.empty(self.n, np.complex128)
        _check(load_library().gade_batch_get_x(self._h, int(pulse), x.ctypes.data, self.n))
        return x

    def step(self, ft: np.ndarray, active=None, maxit: int = 500, tol: float = 1e-16) -> list[dict]:
        """ft: complex128 [npulse, 6]; active: bool/int [npulse] or None (all)."""
        ft = _cbuf(ft)
        if ft.shape != (self.npulse, 6):
            raise ValueError(f"pulse factors must have shape ({self.npulse}, 6)")
        act = None
        if active is not None:
            act = np.ascontiguousarray(active, dtype=np.int32)
            if act.shape != (self.npulse,):
                raise ValueError("active must have one entry per pulse")
        st = (StepStats * self.npulse)()
        _check(load_library().gade_batch_step(self._h, act.ctypes.data if act is not None else None,
                                              ft.ctypes.data, int(maxit), float(tol), st))
        return [st[k].as_dict() for k in range(self.npulse)]

    def info(self) -> dict:
        bi = BatchInfo()
        _check(load_library().gade_batch_get_info(self._h, C.byref(bi)))
        out = {k: getattr(bi, k) for k, _ in BatchInfo._fields_}
        out["tune_cs"] = list(bi.tune_cs)[:bi.ntune]
        out["tune_ms"] = list(bi.tune_ms)[:bi.ntune]
        return out

    def stream(self) -> int:
        return int(load_library().gade_batch_stream(self._h) or 0)

    def operator(self) -> dict:
        """Operator in use (0 matrix-free, 1 assembled) and the timed batch
        applies (matrix-free, assembled)."""
        a = C.c_int32()
        ms = (C.c_float * 5)()
        _check(load_library().gade_batch_operator(self._h, C.byref(a), ms))
        return {"assembled": int(a.value), "matrix_free_ms": float(ms[0]), "assembled_ms": float(ms[1]),
                "tables_ms": float(ms[3]), "assembly_ms": float(ms[4])}

    def set_operator(self, assembled: int):
        _check(load_library().gade_batch_set_operator(self._h, int(assembled)))

    def set_wait_limit(self, polls: int = 0):
        _check(load_library().gade_batch_set_wait_limit(self._h, int(polls)))

    def set_residual_precision(self, mode: int):
        _check(load_library().gade_batch_set_residual_precision(self._h, int(mode)))

    def state_device(self) -> tuple[int, int]:
        """(device address of the pulse states, per-pulse stride in complex elements)."""
        p, ld = C.c_void_p(), C.c_int64()
        _check(load_library().gade_batch_state_device(self._h, C.byref(p), C.byref(ld)))
        return int(p.value), int(ld.value)

    def guess_buffer(self) -> tuple[int, int]:
        """(device address of the initial-guess corrections, per-pulse stride)."""
        p, ld = C.c_void_p(), C.c_int64()
        _check(load_library().gade_batch_guess_buffer(self._h, C.byref(p), C.byref(ld)))
        return int(p.value), int(ld.value)

    def use_guess(self, enable: bool = True):
        _check(load_library().gade_batch_use_guess(self._h, 1 if enable else 0))

    def close(self):
        if getattr(self, "_h", None):
            load_library().gade_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def call(name: str, *args):
    """Call a device-pointer entry point of include/gade_learned.h; raise on
    a nonzero status."""
    fn = getattr(load_library(), name)
    rc = fn(*args)
    if fn.restype is C.c_int:
        _check(rc)
    return rc
