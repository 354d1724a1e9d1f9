"""Benchmark of the GB300 Crank-Nicolson step (GaDE tools/ solver).

Workload (N=1): the nondipole medium configuration — Z=1, rBox=30,
NSplines=250, NKappa=8, NMu=4, Nl=0 (lmax 17), 3-cycle pulse Omega=50,
E0=10, Ntime=1500, complex128, BiCGSTAB tolerance 1e-12; inputs generated
in the reference file formats (synthetic: there is no dataset).  One "step"
is one full CN step: per-step operator (assembly or radial tables), rhs,
preconditioned BiCGSTAB to tolerance.  The pulse is run whole (1501 steps);
the K timed steps are sampled evenly across it after the W warm-up steps,
so that they follow the envelope through its peak, and each is timed from
the state the pulse reaches there (the steps between run untimed).  Inputs
stay resident in HBM for ``value``; ``e2e`` goes through the C ABI with the
state copied from pinned host memory and back every step.  The reference
arm and the CPU baseline time the CPU restatement of the reference build on
the same sampled steps, each from the pulse's own state there.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N>1) every rank runs an independent replica of the pulse on
its own GPU (the single-pulse solve does not shard; no collectives on the
data path): ``value`` is total steps/s over the ranks, timed as max over
ranks between barriers.

Variants (rank 0, in ``variants``): the single pulse in mixed precision
against plain FP64 at the same residual; 64 seeded pulses of uneven length
batched on one GPU (FP64 and mixed, pulse-steps/s); the learned initial
guess at NKappa=16 against the plain and extrapolated guesses on held-out
pulses (a bounded window of steps per pulse, ``--learned-steps``).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "nondipole_medium"
TOL = 1e-12
MAXIT = 500
METRIC = "CN steps/s (plain FP64, nondipole medium NKappa=8)"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.device = device
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _gen(workdir: str):
    from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
    params = CONFIGS[WORKLOAD]
    info = generate(params, workdir)
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    return params, info, T


def sample_positions(nsteps_pulse: int, k: int, warmup: int) -> list[int]:
    """0-based indices of the k timed steps in the pulse's step order: the
    steps after the `warmup` first ones cut into k equal strata, the middle
    step of each, so that the sample follows the pulse envelope through its
    peak."""
    span = nsteps_pulse - warmup
    if k < 1 or k > span:
        raise ValueError(f"cannot sample {k} steps from {span} steps after {warmup} warm-up steps")
    return [warmup + int((i + 0.5) * span / k) for i in range(k)]


def timed_steps_text(k: int, m: int, w: int) -> str:
    return (f"{k} CN steps sampled evenly across the {m}-step pulse after {w} warm-up steps (the middle step "
            f"of each stratum of {(m - w) / k:.1f} steps), each from the state the pulse reaches there")


def bench_config(info: dict, ws: int, k: int, m: int, w: int) -> dict:
    """The workload description, identical in both arms."""
    return {"workload": WORKLOAD, "N": info["n"], "nnz_equiv": info["nnz_full"], "lmax": info["lmax"], "tol": TOL,
            "timed_steps": timed_steps_text(k, m, w),
            "l2": "GPU arm: flushed (256 MB write) before every timed step, outside its events",
            "parallelism": f"replicas x{ws}",
            "iters_counting": "tools/bicgstab.c: the iteration that meets the tolerance is not counted"}


def cpu_port_time(workdir, lmax: int, sample_file: str) -> float:
    """Mean wall time of one CN step of the CPU restatement of the reference
    build (oracle port: the reference assembly, scipy CSR SpMV and SuperLU
    ILU solves, BiCGSTAB of tools/bicgstab.c; one rank) over the sampled
    steps in sample_file (positions and the state each step starts from),
    after one untimed warm-up step.  Set-up (reads, ILU factorisation) is
    excluded, as in the reference's own per-step timer.  Returns s/step."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from dirac_hydrogen_code_gb300.gen import CONFIGS
    params = CONFIGS[WORKLOAD]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    p = O.load_problem(workdir, lmax)
    S, Hst = O.stationary(p, T / params["Ntime"])
    M = O.IluPrecond(S, Hst)
    data = np.load(sample_file)
    pos, states = data["positions"], data["states"]

    def one(j, x):
        _, recs, _ = O.run(workdir, T, lmax, params["Intensity"], params["Omega"], params["Cycles"],
                           params["Ntime"], tol=TOL, maxit=MAXIT, start_iter=int(j) + 1, precond=M,
                           max_steps=1, psi=x, problem=p)
        return recs[0].elapsed
    one(pos[0], states[0])
    return sum(one(j, x) for j, x in zip(pos, states)) / len(pos)


# one thread per CPU process (the throughput comparison runs one process per core)
CPU_THREAD_ENV = {"OMP_NUM_THREADS": "1", "OPENBLAS_NUM_THREADS": "1", "MKL_NUM_THREADS": "1"}


def cpu_processes(workdir, lmax: int, sample_file: str, nproc: int, one_thread: bool) -> list[float]:
    """s/step of nproc concurrent oracle-port processes, each timing the
    sampled steps of sample_file on its own (started together).  one_thread:
    BLAS and OpenMP limited to one thread per process; else every host thread
    is available to the port (its BLAS-threaded parts use them)."""
    env = dict(os.environ, **CPU_THREAD_ENV) if one_thread else dict(os.environ)
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-worker", workdir, str(lmax), sample_file]
    procs = [subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, env=env) for _ in range(nproc)]
    out = []
    for p in procs:
        o, e = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"CPU worker failed: {e.decode()[-500:]}")
        out.append(float(o.decode().strip().splitlines()[-1]))
    return out


def cpu_worker(argv) -> int:
    workdir, lmax, sample_file = argv
    print(cpu_port_time(workdir, int(lmax), sample_file))
    return 0


def write_sample(path: str, positions, states) -> str:
    import numpy as np
    np.savez(path, positions=np.asarray(positions, np.int64), states=np.stack(states))
    return path


def gpu_states(workdir, info, fts, dt, positions, device=0):
    """The state at the start of each listed step of the pulse, from the
    plain FP64 GPU path (used only to give the CPU steps their starting
    states; nothing of it is timed)."""
    from dirac_hydrogen_code_gb300 import native
    prob = native.Problem(workdir, info["lmax"])
    sol = native.Solver(prob, dt, 1.0, precision="fp64", device=device)
    psi, _ = prob.psi0()
    sol.set_x(psi)
    want, out = set(positions), {}
    for j in range(max(positions) + 1):
        if j in want:
            out[j] = sol.get_x()
        sol.step(fts[j], MAXIT, TOL)
    sol.close()
    prob.close()
    return [out[j] for j in positions]


def run_reference(args):
    """The reference arm: the CPU restatement of the reference build (oracle
    port) on the host cores, on the GPU arm's workload, config and sampled
    steps; each timed step starts from the state the pulse reaches there
    (from the FP64 GPU path when a GPU is present, else psi0)."""
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    import numpy as np
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    with tempfile.TemporaryDirectory() as d:
        params, info, T = _gen(d)
        dt, steps = step_times(T, params["Ntime"])
        fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps]
        pos = sample_positions(len(fts), args.steps, args.warmup)
        have_gpu = False
        try:
            import torch
            have_gpu = torch.cuda.is_available()
        except Exception:
            pass
        if have_gpu:
            states = gpu_states(d, info, fts, dt, pos, device=local)
            start = "the state the FP64 GPU path reaches there (computed beforehand, not timed)"
        else:
            from dirac_hydrogen_code_gb300.formats import vec_read
            psi, _ = vec_read(os.path.join(d, "psi0.vec"))
            states = [psi] * len(pos)
            start = "psi0 (no GPU present to give the pulse's own states)"
        sample = write_sample(os.path.join(d, "sample.npz"), pos, states)
        s_per_step = cpu_processes(d, info["lmax"], sample, 1, False)[0]
        cfg = bench_config(info, ws, args.steps, len(fts), args.warmup)
    v = 1.0 / s_per_step
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": s_per_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (generated dumpCouplings inputs)",
        "config": cfg,
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{timed_steps_text(args.steps, len(fts), args.warmup)}; each step starts from "
                                   f"{start}; one untimed warm-up step; one process (one reference rank) with "
                                   "every host thread available to its BLAS-threaded parts; SpMV and SuperLU "
                                   "solves single-threaded"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def max_over_ranks(t_local: float, dist, device: str) -> float:
    """The job's time: the slowest rank's (every rank gets it)."""
    if dist is None:
        return t_local
    import torch
    tt = torch.tensor([t_local], dtype=torch.float64, device=device if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def walk(sol, fts, positions, tol, stream, l2_flush, torch, states=False, kernel_times=False, quality_at=None):
    """One whole pulse on `sol` (restarted from psi0 by the caller): every
    step's device time with CUDA events on the solver's stream, the L2
    flushed before each step listed in `positions` (outside its events).
    states: keep the state each listed step starts from.  kernel_times: the
    solver's per-kernel event times (direct launches) summed over the listed
    steps.  quality_at: a step after which the true residual of the step is
    measured (outside every timed region).  Returns a dict."""
    import numpy as np
    want = set(positions)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in fts]
    out = {"iters": [], "records": [], "states": {}, "launches": 0, "quality": None}
    kt_sum = {}
    if kernel_times:
        sol.profile(True)
    for j, ft in enumerate(fts):
        if j in want:
            if states:
                out["states"][j] = sol.get_x()
            with torch.cuda.stream(stream):
                l2_flush.add_(1.0)
            if kernel_times:
                sol.kernel_times()                     # waits for the device and resets the sums
            l0 = sol.launch_count()
        x_prev = sol.get_x() if j == quality_at else None
        with torch.cuda.stream(stream):
            ev[j][0].record(stream)
        st = sol.step(ft, MAXIT, tol)
        with torch.cuda.stream(stream):
            ev[j][1].record(stream)
        if j in want:
            out["launches"] += sol.launch_count() - l0
            if kernel_times:
                for k, v in sol.kernel_times().items():
                    kt_sum[k] = kt_sum.get(k, 0) + v
        if x_prev is not None:
            x_new = sol.get_x()
            _, sxp, hxp = sol.apply(x_prev, parts=True)
            b_rhs = sxp - hxp
            out["quality"] = {"step": j + 1, "true_residual": float(np.linalg.norm(b_rhs - sol.apply(x_new))
                                                                     / np.linalg.norm(b_rhs)),
                              "recursive_residual": float(st["tol_error"]), "iters": int(st["iters"])}
        out["iters"].append(int(st["iters"]))
        out["records"].append(st)
    torch.cuda.synchronize()
    if kernel_times:
        sol.profile(False)
    ms = [a.elapsed_time(b) for a, b in ev]
    out["ms"] = ms
    out["ms_timed"] = sum(ms[j] for j in positions)
    out["ms_pulse"] = sum(ms)
    out["kt"] = kt_sum
    return out


def iteration_histogram(iters) -> dict:
    h = {}
    for v in iters:
        h[str(v)] = h.get(str(v), 0) + 1
    return dict(sorted(h.items(), key=lambda kv: int(kv[0])))


def run_ours(args):
    import numpy as np
    import torch
    ws, rank, local = _dist()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local
    torch.cuda.set_device(device)
    from dirac_hydrogen_code_gb300 import native
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    native.load_library()

    tmp = tempfile.TemporaryDirectory()
    params, info, T = _gen(tmp.name)
    prob = native.Problem(tmp.name, info["lmax"])
    dt, steps = step_times(T, params["Ntime"])
    sol = native.Solver(prob, dt, 1.0, precision="fp64", device=device)
    if args.operator != "auto":
        sol.set_operator(1 if args.operator == "assembled" else 0)
    ns, split_ms = sol.split()
    bal = sol.balanced()
    partition = {"chosen": "balanced" if ns == 0 else f"order split {ns}",
                 "apply_ms_timed_at_creation": {"balanced": bal["ms"],
                                                **{f"split{k + 1}": v for k, v in enumerate(split_ms) if v > 0}},
                 "balanced_ctas": bal["segments"], "balanced_pieces": bal["pieces"],
                 "balanced_gather_weight": bal["gather_weight"]}
    psi, _ = prob.psi0()
    stream = torch.cuda.ExternalStream(sol.stream(), device=device)
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{device}")
    fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps]
    M = len(fts)
    pos = sample_positions(M, args.steps, args.warmup)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)

    # timed region: the sampled steps of one whole pulse (the warm-up steps
    # and the steps between the samples run untimed), device time of each
    # with CUDA events on the solver's stream
    hbm_peak, peak_kind = _peaks()
    clocks = Clocks(device)
    sol.restart(psi)
    barrier()
    clocks.start()
    w1 = walk(sol, fts, pos, TOL, stream, l2_flush, torch, states=True)
    barrier()
    clk = clocks.stop()
    launches = w1["launches"]
    t_local = max_over_ranks(w1["ms_timed"] / 1e3, dist, f"cuda:{device}")
    value = ws * args.steps / t_local
    x_end = sol.get_x()

    # per-kernel device times of the sampled steps: a second pulse with event
    # pairs around every launch (direct launches; the timed steps above replay
    # captured graphs), and the step quality near the pulse peak
    sol.restart(psi)
    mid = pos[len(pos) // 2]
    w2 = walk(sol, fts, pos, TOL, stream, l2_flush, torch, kernel_times=True, quality_at=mid)
    kt = w2["kt"]

    # e2e through the C ABI with pinned host buffers: one gade_solver_step_host
    # call per step, the state in from and out to the pinned host buffer, the
    # pulse factors from host memory; the sampled steps timed on the host
    n = prob.n
    hx = torch.empty(2 * n, dtype=torch.float64, pin_memory=True)
    hx.numpy()[:] = psi.view(np.float64)
    lib = native.load_library()
    h = sol._h
    ptr = hx.data_ptr()
    fts_host = [np.ascontiguousarray(f, dtype=np.complex128) for f in fts]
    st_host = native.StepStats()
    sol.restart(psi)
    want = set(pos)
    te = 0.0
    barrier()
    for j in range(M):
        if j in want:
            with torch.cuda.stream(stream):
                l2_flush.add_(1.0)
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            native._check(lib.gade_solver_step_host(h, ptr, fts_host[j].ctypes.data, MAXIT, TOL, ptr,
                                                    native.C.byref(st_host)))
            te += time.perf_counter() - t0
        else:
            native._check(lib.gade_solver_step_host(h, ptr, fts_host[j].ctypes.data, MAXIT, TOL, ptr,
                                                    native.C.byref(st_host)))
    barrier()
    te = max_over_ranks(te, dist, f"cuda:{device}")
    e2e = ws * args.steps / te

    # S-norm drift of the whole pulse: psi^H S psi at the end against psi0's
    _, sx_end, _ = sol.apply(x_end, parts=True)
    _, s_psi0, _ = sol.apply(psi, parts=True)
    sn0 = float(np.vdot(psi, s_psi0).real)
    pulse_info = {
        "steps": M, "iters_histogram": iteration_histogram(w1["iters"]),
        "timed_positions": [j + 1 for j in pos], "timed_iters": [w1["iters"][j] for j in pos],
        "whole_pulse_device_s": w1["ms_pulse"] / 1e3, "whole_pulse_steps_per_s": M / (w1["ms_pulse"] / 1e3),
        "whole_pulse_note": "device time of every step of the pulse, L2 flushed only before the sampled steps",
        "snorm_drift_rel_at_end": abs(float(np.vdot(x_end, sx_end).real) - sn0) / sn0,
        "step_quality_near_peak": w2["quality"],
        "operator_partition": partition,
    }

    # roofline of the dominant kernel (the operator apply)
    apply_ms = kt["apply_ms"] / max(kt["apply_launches"], 1)
    nnz = info["nnz_full"]
    N = info["n"]
    csr_bytes = 20 * nnz + 4 * (N + 1) + 32 * N               # assembled complex128 CSR SpMV
    achieved = csr_bytes / (apply_ms * 1e-3) / 1e9
    fp64_peak = native.fp64_peak_tflops(device)
    mf_flops, pc_flops = sol.flops()
    mf_bytes = sol.apply_bytes()
    opinfo = sol.operator()
    asm_flops, asm_bytes = sol.assembly_cost()
    assembled = bool(opinfo["assembled"])
    roof = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
        "traffic": _ncu_traffic("k_apply_asm" if assembled else "k_apply"), "peak_kind": peak_kind,
        "kernel": ("k_apply_asm (S + H(t) apply with this step's assembled real coupling values)" if assembled
                   else "k_apply (matrix-free S + H(t) apply)"),
        "note": ("achieved = CSR-equivalent bytes of the reference assembled complex128 SpMV "
                 "(20 nnz + 4(N+1) + 32N) / average operator apply time over the sampled steps; the kernel "
                 "stores real coupling values (8 B) and is bound by the FP64 pipe, see fp64" if assembled else
                 "achieved = CSR-equivalent bytes of the reference assembled complex128 SpMV "
                 "(20 nnz + 4(N+1) + 32N) / average k_apply time over the sampled steps; the matrix-free "
                 "kernel moves far fewer bytes and is bound by the FP64 pipe, see fp64"),
        "operator": opinfo,
        "assembly_per_step": {"kernel": "k_assemble", "flops": asm_flops, "bytes": asm_bytes} if assembled else None,
        "fp64": {"achieved_tflops": mf_flops / (apply_ms * 1e-3) / 1e12, "peak_tflops": fp64_peak,
                 "frac": mf_flops / (apply_ms * 1e-3) / 1e12 / fp64_peak, "flops_per_launch": mf_flops,
                 "peak_kind": "measured (own FP64 FMA kernel)"},
        "compulsory_bytes": {"per_launch": mf_bytes,
                             "achieved_gbs": mf_bytes / (apply_ms * 1e-3) / 1e9,
                             "frac": mf_bytes / (apply_ms * 1e-3) / 1e9 / hbm_peak,
                             "formula": ("stored coupling values pairs x W x B x 8 B + diagonal blocks "
                                         "nk x W x B x 16 B + 48 N (x, r0 in; v out)" if assembled else
                                         "table slabs of the used (order, kappa) pairs x W x B x 32 B + "
                                         "diagonal blocks nk x W x B x 16 B + angular terms x 36 B + "
                                         "slot maps + 48 N (x, r0 in; v out)")},
        "apply_ms": apply_ms, "precond_ms": kt["precond_ms"] / max(kt["precond_launches"], 1),
        "kernel_share": {"apply": kt["apply_ms"], "precond": kt["precond_ms"], "other": kt["other_ms"]},
    }

    variants = None
    if rank == 0 and not args.no_variants:
        variants = {"single_pulse_precision": mixed_variant(prob, params, info, T, args, device, torch, native,
                                                            psi, fts, pos, l2_flush)}
        if not args.no_batch:
            variants["batch64"] = batch_variant(prob, params, args, torch)
        if not args.no_large:
            variants["nkappa16_whole_pulse"] = nkappa16_variant(args, torch)
        if not args.no_learned:
            variants["learned_nkappa16"] = learned_variant(args, torch)

    # CPU baseline on a bounded sample of the same sampled steps (rank 0, N=1),
    # each from the state the GPU pulse reached there
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        every = max(1, len(pos) // args.cpu_steps)
        cpos = pos[every // 2::every][:args.cpu_steps]
        sample = write_sample(os.path.join(tmp.name, "cpu_sample.npz"), cpos, [w1["states"][j] for j in cpos])
        s_per_step = cpu_processes(tmp.name, info["lmax"], sample, 1, False)[0]
        cpu = {"value": 1.0 / s_per_step, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{len(cpos)} of the timed steps (pulse steps {[j + 1 for j in cpos]}), each from the "
                         "state the GPU pulse reached there, after one untimed warm-up step (oracle port: "
                         "reference assembly, scipy CSR SpMV, SuperLU ILU, BiCGSTAB at tol 1e-12; one process "
                         "(one reference rank) with every host thread available to its BLAS-threaded parts)"}
        if variants is not None and "batch64" in variants:
            # throughput comparison for the batch: one single-threaded process per host core
            nproc = os.cpu_count() or 1
            per = cpu_processes(tmp.name, info["lmax"], sample, nproc, True)
            variants["batch64"]["cpu_aggregate"] = {
                "value": sum(1.0 / x for x in per), "unit": "pulse-steps/s", "processes": nproc, "cores": nproc,
                "kind": "port", "sample": f"{nproc} concurrent single-threaded processes, each timing the "
                                          f"{len(cpos)} CN steps of the CPU baseline's sample"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_local * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (generated dumpCouplings inputs)",
            "config": bench_config(info, ws, args.steps, M, args.warmup),
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
            "pulse": pulse_info,
            "variants": variants,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    sol.close()
    prob.close()
    tmp.cleanup()
    return 0


def mixed_variant(prob, params, info, T, args, device, torch, native, psi, fts, positions, l2_flush):
    """Mixed precision (complex64 inner BiCGSTAB in FP64 refinement) against
    plain FP64, each over the whole pulse from psi0, timed on the sampled
    steps like the headline, at the residual 1e-10 (both) and at the
    configuration's 1e-12 (both); errors of the final state (relative S-norm
    and L2, populations) against the plain FP64 run at 1e-12."""
    import numpy as np
    from dirac_hydrogen_code_gb300.cn import step_times
    dt, _ = step_times(T, params["Ntime"])
    out = {"timed_steps": timed_steps_text(len(positions), len(fts), args.warmup)}
    finals = {}
    runs = (("fp64", "fp64", TOL), ("fp64_tol1e-10", "fp64", 1e-10), ("mixed_tol1e-10", "mixed", 1e-10),
            ("mixed_tol1e-12", "mixed", 1e-12))
    for tag, prec, tol in runs:
        sol = native.Solver(prob, dt, 1.0, precision=prec, device=device)
        sol.restart(psi)
        stream = torch.cuda.ExternalStream(sol.stream(), device=device)
        w = walk(sol, fts, positions, tol, stream, l2_flush, torch)
        finals[tag] = sol.get_x()
        sol.restart(psi)
        kt = walk(sol, fts, positions, tol, stream, l2_flush, torch, kernel_times=True)["kt"]
        recs = [w["records"][j] for j in positions]
        k = len(positions)
        out[tag] = {"steps_per_s": k / (w["ms_timed"] / 1e3), "ms_per_step": w["ms_timed"] / k,
                    "whole_pulse_steps_per_s": len(fts) / (w["ms_pulse"] / 1e3),
                    "inner_iters_per_step": float(np.mean([r["inner_iters"] for r in recs])),
                    "fp64_residual_passes_per_step": float(np.mean([r["refinements"] for r in recs])),
                    "kernel_ms_per_step": {kk: round(v / k, 4) for kk, v in kt.items() if kk.endswith("_ms")}}
        sol.close()
    ref = finals["fp64"]
    eb = _eigenbasis(prob)
    pref = eb.populations(ref)
    for tag in ("fp64_tol1e-10", "mixed_tol1e-10", "mixed_tol1e-12"):
        out[tag]["population_err_vs_fp64"] = _pop_err(eb.populations(finals[tag]), pref)
    out["fp64"]["populations"] = pref
    chk = native.Solver(prob, dt, 1.0, precision="fp64", device=device)
    chk.set_time(fts[0])
    _, sref, _ = chk.apply(ref, parts=True)
    for tag in ("fp64_tol1e-10", "mixed_tol1e-10", "mixed_tol1e-12"):
        e = finals[tag] - ref
        _, se, _ = chk.apply(e, parts=True)
        out[tag]["err_vs_fp64_whole_pulse"] = {
            "s_norm_rel": float(np.sqrt(abs(np.vdot(e, se).real) / abs(np.vdot(ref, sref).real))),
            "l2_rel": float(np.linalg.norm(e) / np.linalg.norm(ref))}
    chk.close()
    out["speedup_mixed_vs_fp64_at_1e-10"] = out["mixed_tol1e-10"]["steps_per_s"] / out["fp64_tol1e-10"]["steps_per_s"]
    out["speedup_mixed_vs_fp64_at_1e-12"] = out["mixed_tol1e-12"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    return out


BATCH_SEED = 2026


def _eigenbasis(prob):
    from dirac_hydrogen_code_gb300.populations import Eigenbasis
    kap, _ = prob.blocks()
    return Eigenbasis(prob.workdir, kap)


def _pop_err(p, ref):
    """absolute error of the bound and continuum populations"""
    return {"bound_abs": abs(p["bound"] - ref["bound"]), "continuum_abs": abs(p["continuum"] - ref["continuum"]),
            "continuum_rel": abs(p["continuum"] - ref["continuum"]) / max(ref["continuum"], 1e-300)}


def batch_variant(prob, params, args, torch):
    """64 pulses on the nondipole medium matrices (Intensity log-uniform in
    [1, 100], Omega uniform in [10, 100], Cycles in {1, 2, 3}, Ntime =
    500 Cycles; seeded), each with its own radial tables, dt and LU factors,
    advanced together to the end of the longest pulse (a pulse whose time
    grid has ended retires from the batch): plain FP64 at tol 1e-12 and 1e-10
    and mixed precision at 1e-10 and 1e-12.  Timed with CUDA events on the batch's
    stream: the whole run (every pulse-step of every pulse; the batch's
    inputs, 64 pulses' tables and values, are far larger than L2) and, for
    comparison with earlier measurements, the batch steps after warm-up at
    the start of the pulses.  Unit: pulse-steps/s (one CN step of one
    pulse).  Errors of the FP64 run at 1e-10 and of the mixed runs: final
    states of every pulse against the FP64 run at 1e-12."""
    import numpy as np
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    from dirac_hydrogen_code_gb300.gen.pulses import draw_pulses, pulse_tables_many
    from dirac_hydrogen_code_gb300.native import Batch
    pulses = draw_pulses(64, BATCH_SEED)
    t0 = time.perf_counter()
    tables = pulse_tables_many(params, pulses)
    t_tables = time.perf_counter() - t0
    grids = [step_times(p["maxtime"], p["ntime"]) for p in pulses]
    nsteps = [len(g[1]) for g in grids]
    total = max(nsteps)
    first = min(args.warmup + args.batch_steps, total)
    ft = np.zeros((len(pulses), 6), complex)
    out = {"pulses": len(pulses), "seed": BATCH_SEED, "tables_s": t_tables, "unit": "pulse-steps/s",
           "pulse_steps_whole_run": int(sum(nsteps)), "batch_steps_whole_run": total}
    finals = {}
    for tag, prec, tol in (("fp64_tol1e-12", "fp64", 1e-12), ("fp64_tol1e-10", "fp64", 1e-10),
                           ("mixed_tol1e-10", "mixed", 1e-10), ("mixed_tol1e-12", "mixed", 1e-12)):
        b = Batch(prob, [g[0] for g in grids], tables, precision=prec)
        stream = torch.cuda.ExternalStream(b.stream())

        def steps(j0, j1):
            st = []
            for j in range(j0, j1):
                active = np.array([j < n for n in nsteps], np.int32)
                for k, p in enumerate(pulses):
                    if active[k]:
                        ft[k] = pulse(p["E0"], p["omega"], p["cycles"], grids[k][1][j][1])
                rec = b.step(ft, active, maxit=MAXIT, tol=tol)
                st.append([rec[k] for k in range(len(pulses)) if active[k]])
            return st
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        st_w = steps(0, args.warmup)
        ev[1].record(stream)
        st_t = steps(args.warmup, first)
        ev[2].record(stream)
        st_r = steps(first, total)
        ev[3].record(stream)
        ev[3].synchronize()
        ms_first = ev[1].elapsed_time(ev[2])
        ms_whole = ev[0].elapsed_time(ev[3])
        allrec = [r for row in st_w + st_t + st_r for r in row]
        inf = b.info()
        out[tag] = {"pulse_steps_per_s": sum(nsteps) / (ms_whole / 1e3), "whole_run_s": ms_whole / 1e3,
                    "iters_per_step": float(np.mean([r["iters"] for r in allrec])),
                    "fp64_residual_passes_per_step": float(np.mean([r["refinements"] for r in allrec])),
                    "first_steps": {"batch_steps": first - args.warmup,
                                    "pulse_steps_per_s": len(pulses) * (first - args.warmup) / (ms_first / 1e3),
                                    "iters_per_step": float(np.mean([[r["iters"] for r in row] for row in st_t]))},
                    "graph_replays_per_step": inf["graph_replays"] / max(inf["steps"], 1),
                    "operator": "assembled" if b.operator()["assembled"] else "matrix-free",
                    "chunk_splines": inf["chunk_splines"], "autotune_ms": dict(zip(inf["tune_cs"], inf["tune_ms"]))}
        finals[tag] = np.stack([b.get_x(k) for k in range(len(pulses))])
        b.close()
    out["speedup_mixed_vs_fp64"] = out["mixed_tol1e-10"]["pulse_steps_per_s"] / out["fp64_tol1e-12"]["pulse_steps_per_s"]
    out["speedup_mixed_vs_fp64_at_1e-12"] = (out["mixed_tol1e-12"]["pulse_steps_per_s"]
                                             / out["fp64_tol1e-12"]["pulse_steps_per_s"])
    ref = finals["fp64_tol1e-12"]
    eb = _eigenbasis(prob)
    # the plain FP64 run at 1e-10 is there to show what the tolerance alone leaves
    for tag in ("fp64_tol1e-10", "mixed_tol1e-10", "mixed_tol1e-12"):
        mx = finals[tag]
        perr = [_pop_err(eb.populations(mx[k]), eb.populations(ref[k])) for k in range(len(pulses))]
        out[tag]["err_vs_fp64_whole_run"] = {
            "l2_rel_max": float(np.max(np.linalg.norm(mx - ref, axis=1) / np.linalg.norm(ref, axis=1))),
            "bound_abs_max": max(e["bound_abs"] for e in perr),
            "continuum_abs_max": max(e["continuum_abs"] for e in perr)}
    return out


def nkappa16_variant(args, torch):
    """The NKappa=16 configuration (NMu=8, NSplines=300, Nl=10, 5 cycles,
    Ntime=4000, N = 244,000; the matrix-free operator): one whole pulse per
    precision, timed on K steps sampled evenly across it like the headline
    (L2 flushed before each), plain FP64 at tolerance 1e-12 and 1e-10 and
    mixed precision (complex64 inner solve, double-float refinement residual)
    at 1e-10 and 1e-12, and at 1e-10 with the refinement residual on the FP64
    units; final-state errors against the plain FP64 run at 1e-12."""
    import numpy as np
    from dirac_hydrogen_code_gb300 import native
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
    params = CONFIGS["nondipole_large"]
    out = {"workload": "nondipole_large (NKappa=16)", "unit": "steps/s"}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with tempfile.TemporaryDirectory() as d:
        info = generate(params, d)
        prob = native.Problem(d, info["lmax"])
        T = params["Cycles"] * 2 * math.pi / params["Omega"]
        dt, steps = step_times(T, params["Ntime"])
        fts = [pulse(params["Intensity"], params["Omega"], params["Cycles"], t) for _, t in steps]
        pos = sample_positions(len(fts), args.steps, args.warmup)
        out["timed_steps"] = timed_steps_text(len(pos), len(fts), args.warmup)
        psi, _ = prob.psi0()
        finals = {}
        for tag, prec, tol in (("fp64_tol1e-12", "fp64", 1e-12), ("fp64_tol1e-10", "fp64", 1e-10),
                               ("mixed_tol1e-10", "mixed", 1e-10), ("mixed_tol1e-12", "mixed", 1e-12),
                               ("mixed_fp64_residual_tol1e-10", "mixed", 1e-10)):
            sol = native.Solver(prob, dt, 1.0, precision=prec)
            if "fp64_residual" in tag:
                sol.set_residual_precision(0)
            sol.restart(psi)
            stream = torch.cuda.ExternalStream(sol.stream())
            w = walk(sol, fts, pos, tol, stream, flush, torch)
            finals[tag] = sol.get_x().copy()
            recs = [w["records"][j] for j in pos]
            rec = {"steps_per_s": len(pos) / (w["ms_timed"] / 1e3),
                   "whole_pulse_steps_per_s": len(fts) / (w["ms_pulse"] / 1e3),
                   "iters_histogram": iteration_histogram(w["iters"]), "operator": sol.operator()["assembled"]}
            if prec == "mixed":
                rec["fp64_residual_passes_per_step"] = float(np.mean([r["refinements"] for r in recs]))
                rec["inner_iters_per_step"] = float(np.mean([r["inner_iters"] for r in recs]))
                rec["residual_pass"] = ("double-float" if sol.residual_precision()["double_float_in_use"]
                                        else "FP64")
            out[tag] = rec
            sol.close()
        eb = _eigenbasis(prob)
        ref = finals["fp64_tol1e-12"]
        pref = eb.populations(ref)
        for tag in ("fp64_tol1e-10", "mixed_tol1e-10", "mixed_tol1e-12", "mixed_fp64_residual_tol1e-10"):
            out[tag]["l2_err_vs_fp64_tol1e-12"] = float(np.linalg.norm(finals[tag] - ref) / np.linalg.norm(ref))
            out[tag]["population_err_vs_fp64"] = _pop_err(eb.populations(finals[tag]), pref)
        prob.close()
    base12, base10 = out["fp64_tol1e-12"]["steps_per_s"], out["fp64_tol1e-10"]["steps_per_s"]
    out["speedup_mixed_tol1e-10_vs_fp64_tol1e-10"] = out["mixed_tol1e-10"]["steps_per_s"] / base10
    out["speedup_mixed_tol1e-10_vs_fp64_tol1e-12"] = out["mixed_tol1e-10"]["steps_per_s"] / base12
    out["speedup_mixed_tol1e-12_vs_fp64_tol1e-12"] = out["mixed_tol1e-12"]["steps_per_s"] / base12
    out["speedup_mixed_fp64_residual_tol1e-10_vs_fp64_tol1e-12"] = (
        out["mixed_fp64_residual_tol1e-10"]["steps_per_s"] / base12)
    return out


def learned_variant(args, torch):
    """Learned initial guess at NKappa=16, NMu=8, NSplines=300, Nl=10, 5
    cycles, Ntime=4000: POD basis (rank <= 128) from 200 seeded snapshots of
    8 training pulses, MLP 2 x 256 trained on 32 training pulses, evaluated
    on 8 held-out pulses; pulses differ in Intensity only (log-uniform in
    [1, 100], seeded), so they share g, dt and the LU factors.  Bounded
    sample: the first `learned_steps` steps of every pulse.  Compared at the
    same residual 1e-10: plain FP64, mixed precision with the extrapolated
    guess, mixed precision with the learned guess; and the two mixed runs at
    1e-12; errors against an FP64 run at tol 1e-12."""
    import numpy as np
    from dirac_hydrogen_code_gb300 import learned as L
    from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
    from dirac_hydrogen_code_gb300.native import Problem
    params = CONFIGS["nondipole_large"]
    W = args.learned_steps
    out = {"workload": "nondipole_large (NKappa=16)", "steps_per_pulse": W, "unit": "steps/s"}
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        info = generate(params, d)
        out["generate_s"] = time.perf_counter() - t0
        prob = Problem(d, info["lmax"])
        mk = lambda n, seed: L.intensity_pulses(n, seed, params["Omega"], params["Cycles"], params["Ntime"])  # noqa
        train, held = mk(32, 101), mk(8, 202)
        t0 = time.perf_counter()
        model = L.build_model(prob, train, W, rank=128, nsnap=200, pod_pulses=8, epochs=30, seed=1)
        out["build_s"] = time.perf_counter() - t0
        out["model"] = {k: model.history[k] for k in ("rows", "rank", "sv_ratio", "snapshots", "train_s")}
        out["model"]["loss_first_last"] = [model.history["loss"][0], model.history["loss"][-1]]
        xr, _, ms_ref = L.run_held_out(prob, held, W, 1e-12, "fp64", None)
        out["fp64_tol1e-12"] = {"steps_per_s": len(held) * W / (ms_ref / 1e3)}
        eb = _eigenbasis(prob)
        pref = [eb.populations(x) for x in xr]
        out["fp64_tol1e-12_populations_mean"] = {k: float(np.mean([p[k] for p in pref])) for k in pref[0]}
        for tag, prec, mdl, tol in (("fp64_tol1e-10", "fp64", None, 1e-10), ("mixed_tol1e-10", "mixed", None, 1e-10),
                                    ("learned_mixed_tol1e-10", "mixed", model, 1e-10),
                                    ("mixed_tol1e-12", "mixed", None, 1e-12),
                                    ("learned_mixed_tol1e-12", "mixed", model, 1e-12)):
            xs, st, ms = L.run_held_out(prob, held, W, tol, prec, mdl)
            err = np.linalg.norm(xs - xr, axis=1) / np.linalg.norm(xr, axis=1)
            rec = {"steps_per_s": len(held) * W / (ms / 1e3),
                   "iters_per_step": float(np.mean([[r["iters"] for r in row] for row in st])),
                   "final_l2_err_vs_fp64_max": float(err.max())}
            perr = [_pop_err(eb.populations(xs[k]), pref[k]) for k in range(len(held))]
            rec["population_err_vs_fp64_max"] = {"bound_abs": max(e["bound_abs"] for e in perr),
                                                 "continuum_abs": max(e["continuum_abs"] for e in perr)}
            if prec == "mixed":
                ini = np.array([[r["init_residual"] for r in row] for row in st])[L.K_HIST:]
                rec["init_residual_mean"] = float(ini.mean())
                rec["fp64_residual_passes_per_step"] = float(np.mean([[r["refinements"] for r in row] for row in st]))
                rec["inner_iters_per_step"] = float(np.mean([[r["inner_iters"] for r in row] for row in st]))
            out[tag] = rec
        prob.close()
    base = out["fp64_tol1e-10"]["steps_per_s"]
    out["speedup_vs_fp64"] = {k: out[k]["steps_per_s"] / base for k in ("mixed_tol1e-10", "learned_mixed_tol1e-10")}
    base12 = out["fp64_tol1e-12"]["steps_per_s"]
    out["speedup_vs_fp64_tol1e-12"] = {k: out[k]["steps_per_s"] / base12
                                       for k in ("mixed_tol1e-10", "learned_mixed_tol1e-10", "mixed_tol1e-12",
                                                 "learned_mixed_tol1e-12")}
    out["learned_over_extrapolated"] = {t: out[f"learned_mixed_{t}"]["steps_per_s"] / out[f"mixed_{t}"]["steps_per_s"]
                                        for t in ("tol1e-10", "tol1e-12")}
    return out


def _ncu_traffic(kernel: str = "k_apply"):
    """DRAM bytes per launch of the operator kernel (dram__bytes_read.sum +
    dram__bytes_write.sum) from the committed ncu summary of this workload."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{WORKLOAD}.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return int(line.split(":")[1])
    except OSError:
        pass
    return None


def profile_only(args):
    """Warm-up and timed steps of one precision, nothing else: a small,
    deterministic launch sequence for profiler captures."""
    import torch
    from dirac_hydrogen_code_gb300 import native
    from dirac_hydrogen_code_gb300.cn import pulse, step_times
    native.load_library()
    from dirac_hydrogen_code_gb300.gen import CONFIGS, generate
    with tempfile.TemporaryDirectory() as d:
        params = CONFIGS[args.profile_workload]
        info = generate(params, d)
        T = params["Cycles"] * 2 * math.pi / params["Omega"]
        prob = native.Problem(d, info["lmax"])
        dt, steps = step_times(T, params["Ntime"])
        sol = native.Solver(prob, dt, 1.0, precision=args.profile_precision, device=0)
        if args.operator != "auto":
            sol.set_operator(1 if args.operator == "assembled" else 0)
        tol = TOL if args.profile_precision == "fp64" else 1e-10
        first = args.profile_from
        for k in range(first, first + args.warmup + args.steps):
            sol.step(pulse(params["Intensity"], params["Omega"], params["Cycles"], steps[k][1]), MAXIT, tol)
        torch.cuda.synchronize()
        print(json.dumps({"profiled": args.profile_precision, "steps": args.warmup + args.steps,
                          "launches": sol.launch_count()}))
        sol.close()
        prob.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip every variant (precision, batch, learned)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-pulse batch variant")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-guess variant")
    ap.add_argument("--no-large", action="store_true", help="skip the NKappa=16 whole-pulse variant")
    ap.add_argument("--batch-steps", type=int, default=10, help="timed batch steps of the batch variant")
    ap.add_argument("--learned-steps", type=int, default=200, help="steps per pulse of the learned variant")
    ap.add_argument("--operator", default="auto", choices=["auto", "assembled", "matrix-free"],
                    help="operator of the headline solver (auto: chosen by timing at creation; a profiler "
                         "run that distorts that timing names it)")
    ap.add_argument("--profile-precision", default=None, choices=["fp64", "mixed"],
                    help="only run this precision's steps (for profiler captures)")
    ap.add_argument("--profile-workload", default=WORKLOAD, choices=["dipole_small", WORKLOAD, "nondipole_large"],
                    help="workload of the profile-only run")
    ap.add_argument("--profile-from", type=int, default=0,
                    help="profile-only run: first step (0-based) of the pulse to run, from psi0 (e.g. the pulse "
                         "peak, where BiCGSTAB iterates)")
    if len(sys.argv) > 1 and sys.argv[1] == "--cpu-worker":
        return cpu_worker(sys.argv[2:])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_precision:
        return profile_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
