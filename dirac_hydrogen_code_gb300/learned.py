"""Learned initial guess for mixed-precision Crank-Nicolson batches.

The reference starts every BiCGSTAB solve from the previous state
(tools/dirac_solver.c:533-551); the mixed-precision step here starts from the
linear extrapolation x_n + (x_n - x_{n-1}).  The learned guess adds U c:

  * U: a POD basis (rank R, orthonormal rows, complex64 on the GPU) of the
    solver's own second differences x_{n+1} - 2 x_n + x_{n-1}, i.e. of what
    extrapolation misses, from seeded snapshots of training trajectories;
  * c: the output of an MLP (two hidden ReLU layers) whose input is the POD
    projections of the last K = 4 states and the pulse factors f_a(t) of the
    step, trained to predict U^H (x_{n+1} - 2 x_n + x_{n-1}).

Device memory comes from PyTorch; every computation of the network and of
the subspace runs in this package's kernels (include/gade_learned.h): BF16
tensor-core GEMMs with FP32 accumulation for the forward and backward passes,
Adam on FP32 master weights, projection and expansion.  The FP64 refinement
of the mixed step still certifies every step; a prediction larger than the
last state change is dropped on the device (plain extrapolation).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np
import torch

from . import native
from .cn import pulse, step_times
from .native import Batch, Problem

K_HIST = 4


class _Dev:
    """A raw device allocation seen as a tensor (no copy)."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, shape, dtype=torch.complex128) -> torch.Tensor:
    typestr = {torch.complex128: "<c16", torch.complex64: "<c8", torch.float64: "<f8", torch.float32: "<f4"}[dtype]
    return torch.as_tensor(_Dev(ptr, shape, typestr), device="cuda")


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class MLP:
    """din -> dh -> dh -> dout, ReLU hidden layers, BF16 weights (FP32 master
    copies), FP32 accumulation, MSE loss, Adam.  Workspaces hold max_rows
    samples."""

    def __init__(self, din: int, dh: int, dout: int, max_rows: int, seed: int = 0):
        self.din, self.dh, self.dout, self.max_rows = din, dh, dout, max_rows
        g = torch.Generator(device="cpu").manual_seed(seed)
        dims = [(din, dh), (dh, dh), (dh, dout)]
        self.W, self.b = [], []
        for i, (a, bdim) in enumerate(dims):
            std = math.sqrt(2.0 / a) if i < 2 else math.sqrt(1.0 / a)
            self.W.append((torch.randn(a, bdim, generator=g) * std).cuda())
            self.b.append(torch.zeros(bdim, device="cuda"))
        self.params = [t for pair in zip(self.W, self.b) for t in pair]      # W1 b1 W2 b2 W3 b3
        self.W16 = [torch.empty(w.shape, dtype=torch.bfloat16, device="cuda") for w in self.W]
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.step_count = 0
        R = max_rows
        f32 = dict(dtype=torch.float32, device="cuda")
        b16 = dict(dtype=torch.bfloat16, device="cuda")
        self.H1, self.H2 = torch.empty(R, dh, **f32), torch.empty(R, dh, **f32)
        self.H1_16, self.H2_16 = torch.empty(R, dh, **b16), torch.empty(R, dh, **b16)
        self.out = torch.empty(R, dout, **f32)
        self.G3, self.G2, self.G1 = torch.empty(R, dout, **f32), torch.empty(R, dh, **f32), torch.empty(R, dh, **f32)
        self.G3_16, self.G2_16, self.G1_16 = (torch.empty(R, dout, **b16), torch.empty(R, dh, **b16),
                                              torch.empty(R, dh, **b16))
        self.rowloss = torch.empty(R, dtype=torch.float64, device="cuda")
        self.sync_bf16(0)

    def sync_bf16(self, stream: int):
        for w, w16 in zip(self.W, self.W16):
            native.call("gade_to_bf16", w.numel(), w.data_ptr(), w16.data_ptr(), stream)

    def _gemm(self, M, N, K, A, sa0, sa1, B, sb0, sb1, bias, mask, ldm, act, C, ldc, C16, ldc16, stream):
        native.call("gade_gemm_bf16", M, N, K, A, sa0, sa1, B, sb0, sb1, bias, mask, ldm, act, C, ldc, C16,
                    ldc16, stream)

    def forward(self, X16: torch.Tensor, M: int, stream: int) -> torch.Tensor:
        """X16: BF16 [>=M, din] rows; returns the FP32 output rows [M, dout]."""
        assert M <= self.max_rows
        dh, dout, din = self.dh, self.dout, self.din
        W1, W2, W3 = (w.data_ptr() for w in self.W16)
        b1, b2, b3 = (b.data_ptr() for b in self.b)
        self._gemm(M, dh, din, X16.data_ptr(), din, 1, W1, dh, 1, b1, None, 0, 1, self.H1.data_ptr(), dh,
                   self.H1_16.data_ptr(), dh, stream)
        self._gemm(M, dh, dh, self.H1_16.data_ptr(), dh, 1, W2, dh, 1, b2, None, 0, 1, self.H2.data_ptr(), dh,
                   self.H2_16.data_ptr(), dh, stream)
        self._gemm(M, dout, dh, self.H2_16.data_ptr(), dh, 1, W3, dout, 1, b3, None, 0, 0, self.out.data_ptr(),
                   dout, None, 0, stream)
        return self.out[:M]

    def backward(self, X16: torch.Tensor, T: torch.Tensor, M: int, stream: int):
        """Gradients of the mean squared error of the last forward pass."""
        dh, dout, din = self.dh, self.dout, self.din
        W2, W3 = self.W16[1].data_ptr(), self.W16[2].data_ptr()
        gW1, gb1, gW2, gb2, gW3, gb3 = (g.data_ptr() for g in self.grads)
        native.call("gade_mse_grad", M, dout, self.out.data_ptr(), T.data_ptr(), self.G3.data_ptr(),
                    self.G3_16.data_ptr(), self.rowloss.data_ptr(), stream)
        self._gemm(dh, dout, M, self.H2_16.data_ptr(), 1, dh, self.G3_16.data_ptr(), dout, 1, None, None, 0, 0,
                   gW3, dout, None, 0, stream)
        native.call("gade_colsum", M, dout, self.G3.data_ptr(), dout, gb3, stream)
        self._gemm(M, dh, dout, self.G3_16.data_ptr(), dout, 1, W3, 1, dout, None, self.H2.data_ptr(), dh, 0,
                   self.G2.data_ptr(), dh, self.G2_16.data_ptr(), dh, stream)
        self._gemm(dh, dh, M, self.H1_16.data_ptr(), 1, dh, self.G2_16.data_ptr(), dh, 1, None, None, 0, 0,
                   gW2, dh, None, 0, stream)
        native.call("gade_colsum", M, dh, self.G2.data_ptr(), dh, gb2, stream)
        self._gemm(M, dh, dh, self.G2_16.data_ptr(), dh, 1, W2, 1, dh, None, self.H1.data_ptr(), dh, 0,
                   self.G1.data_ptr(), dh, self.G1_16.data_ptr(), dh, stream)
        self._gemm(din, dh, M, X16.data_ptr(), 1, din, self.G1_16.data_ptr(), dh, 1, None, None, 0, 0,
                   gW1, dh, None, 0, stream)
        native.call("gade_colsum", M, dh, self.G1.data_ptr(), dh, gb1, stream)

    def adam(self, lr: float, stream: int):
        self.step_count += 1
        w16 = {0: self.W16[0], 2: self.W16[1], 4: self.W16[2]}
        for i, (p, g, m, v) in enumerate(zip(self.params, self.grads, self.m, self.v)):
            native.call("gade_adam", p.numel(), p.data_ptr(), _p(w16.get(i)), g.data_ptr(), m.data_ptr(),
                        v.data_ptr(), lr, 0.9, 0.999, 1e-8, self.step_count, stream)

    def train_batch(self, X16: torch.Tensor, T: torch.Tensor, M: int, lr: float, stream: int) -> torch.Tensor:
        self.forward(X16, M, stream)
        self.backward(X16, T, M, stream)
        self.adam(lr, stream)
        return self.rowloss[:M]


def pod_basis(snaps: np.ndarray, rank: int) -> tuple[np.ndarray, np.ndarray]:
    """Method of snapshots (Sirovich 1987): rows of ``snaps`` (m x n,
    complex) -> up to ``rank`` orthonormal rows spanning their dominant
    subspace, and the singular values.  FP64 on the host."""
    G = snaps.conj() @ snaps.T
    w, V = np.linalg.eigh(G)
    order = np.argsort(w)[::-1]
    w, V = w[order], V[:, order]
    # eigenvalues of the Gram matrix are squared singular values: below
    # ~1e-13 of the largest they are rounding noise of the Gram product
    keep = [r for r in range(min(rank, len(w))) if w[r] > w[0] * 1e-13]
    U = (V[:, keep].T @ snaps) / np.sqrt(w[keep])[:, None]
    return U, np.sqrt(np.maximum(w, 0))


class LearnedModel:
    """POD basis + normalisation + network of one problem."""

    def __init__(self, U: np.ndarray, mlp: MLP, mu_in, sd_in, mu_out, sd_out, history: dict):
        self.R = U.shape[0]
        self.n = U.shape[1]
        self.U = torch.from_numpy(np.ascontiguousarray(U.astype(np.complex64))).cuda()
        self.mlp = mlp
        self.mu_in, self.sd_in, self.mu_out, self.sd_out = (t.float().cuda().contiguous() for t in
                                                            (mu_in, sd_in, mu_out, sd_out))
        self.history = history


def _pulse_factors(pulses, grids, j):
    """[npulse, 12] reals of f(t) of step j (0-based) of every pulse; zeros
    past a pulse's end."""
    ft = np.zeros((len(pulses), 12))
    for k, p in enumerate(pulses):
        if j < len(grids[k][1]):
            f = pulse(p["E0"], p["omega"], p["cycles"], grids[k][1][j][1])
            ft[k] = np.stack([f.real, f.imag], axis=1).ravel()
    return ft


def _ft_complex(ft_real: np.ndarray) -> np.ndarray:
    return ft_real[:, 0::2] + 1j * ft_real[:, 1::2]


def run_trajectories(problem: Problem, pulses, nsteps: int, tol: float, precision: str = "fp64",
                     on_step=None, **batch_kw):
    """Runs the pulses together for nsteps steps; on_step(j, batch, xview)
    after each step j (0-based).  Returns (batch, grids, stats)."""
    grids = [step_times(p["maxtime"], p["ntime"]) for p in pulses]
    b = Batch(problem, [g[0] for g in grids], None, precision=precision, **batch_kw)
    xptr, ld = b.state_device()
    xview = device_view(xptr, (len(pulses), ld))
    stats = []
    for j in range(nsteps):
        ft = _ft_complex(_pulse_factors(pulses, grids, j))
        stats.append(b.step(ft, maxit=500, tol=tol))
        if on_step is not None:
            on_step(j, b, xview)
    return b, grids, stats


def build_model(problem: Problem, train_pulses, nsteps: int, rank: int = 128, nsnap: int = 200,
                pod_pulses: int = 8, seed: int = 0, hidden: int = 256, epochs: int = 30, batch_rows: int = 512,
                lr: float = 1e-3, tol: float = 1e-10, log=None) -> LearnedModel:
    """Snapshots -> POD basis -> training set -> network, all from the
    solver's own trajectories of the training pulses (plain FP64 steps)."""
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    n = problem.n
    # 1. POD snapshots: seeded (pulse, step) picks among the first pod_pulses
    npod = min(pod_pulses, len(train_pulses))
    picks = sorted(rng.choice(npod * (nsteps - 1), size=min(nsnap, npod * (nsteps - 1)), replace=False))
    want = {}
    for q in picks:
        k, j = divmod(int(q), nsteps - 1)
        want.setdefault(j + 1, []).append(k)        # second difference around state j+1
    snaps = []
    # ring of the last three states of the POD pulses
    ring = []

    def grab_states(j, b, xv):
        # torch works on its own stream only: wait for the batch's work first
        torch.cuda.synchronize()
        ring.append(xv[:npod].clone())
        if len(ring) > 3:
            ring.pop(0)
        # ring[-1] = x_{j+1}, ring[-2] = x_j, ring[-3] = x_{j-1}
        if len(ring) == 3 and j in want:
            d = ring[-1] - 2 * ring[-2] + ring[-3]
            for k in want[j]:
                snaps.append(d[k].cpu().numpy())

    psi, _ = problem.psi0()
    ring.append(torch.from_numpy(np.tile(psi, (npod, 1))).cuda())
    torch.cuda.synchronize()
    b0, _, _ = run_trajectories(problem, train_pulses[:npod], nsteps, tol, on_step=grab_states)
    b0.close()
    S = np.stack(snaps)
    U, sv = pod_basis(S, rank)
    R = U.shape[0]
    if log:
        log(f"POD: {len(snaps)} snapshots, rank {R}, sigma_R/sigma_0 = {sv[R - 1] / sv[0]:.3e}, "
            f"{time.perf_counter() - t0:.1f}s")
    Ud = torch.from_numpy(np.ascontiguousarray(U.astype(np.complex64))).cuda()
    # 2. projections of every training trajectory
    npul = len(train_pulses)
    coef = torch.zeros(nsteps + 1, npul, R, dtype=torch.complex128, device="cuda")
    scratch_b = native.call("gade_pod_project_scratch", n, R, npul)
    scratch = torch.empty(scratch_b, dtype=torch.uint8, device="cuda")
    x0 = torch.from_numpy(np.tile(psi, (npul, 1))).cuda()
    stream0 = torch.cuda.current_stream().cuda_stream
    native.call("gade_pod_project_fp64", n, R, Ud.data_ptr(), x0.data_ptr(), n, npul, coef[0].data_ptr(),
                scratch.data_ptr(), scratch_b, stream0)
    torch.cuda.synchronize()

    def project(j, b, xv):
        st = b.stream()
        native.call("gade_pod_project_fp64", n, R, Ud.data_ptr(), xv.data_ptr(), xv.shape[1], npul,
                    coef[j + 1].data_ptr(), scratch.data_ptr(), scratch_b, st)

    b, grids, _ = run_trajectories(problem, train_pulses, nsteps, tol, on_step=project)
    torch.cuda.synchronize()
    b.close()
    ft_all = torch.from_numpy(np.stack([_pulse_factors(train_pulses, grids, j) for j in range(nsteps)])).cuda()
    # 3. training set: state n >= K-1 predicts x_{n+1} (step n, pulse factors ft[n])
    din = K_HIST * 2 * R + 12
    rows = []
    ones, zeros = torch.ones(din, device="cuda"), torch.zeros(din, device="cuda")
    raw_in = torch.empty((nsteps - K_HIST) * npul, din, dtype=torch.float32, device="cuda")
    dummy16 = torch.empty_like(raw_in, dtype=torch.bfloat16)
    for m, t in enumerate(range(K_HIST - 1, nsteps - 1)):
        # hist slots t-3..t, newest at slot 3; pulse factors of step t+1 (0-based index t)
        native.call("gade_learned_features", npul, R, K_HIST, K_HIST - 1, coef[t - K_HIST + 1].data_ptr(),
                    ft_all[t].data_ptr(), zeros.data_ptr(), ones.data_ptr(),
                    dummy16[m * npul:].data_ptr(), raw_in[m * npul:].data_ptr(), stream0)
        rows.append(t)
    nrow = len(rows) * npul
    raw_in = raw_in[:nrow]
    t_idx = torch.tensor(rows, device="cuda")
    tgt = coef[t_idx + 1] - 2 * coef[t_idx] + coef[t_idx - 1]                 # [T, npul, R]
    raw_out = torch.view_as_real(tgt.reshape(nrow, R)).reshape(nrow, 2 * R).float()
    mu_in, sd_in = raw_in.mean(0), raw_in.std(0)
    sd_in = torch.where(sd_in > 0, sd_in, torch.ones_like(sd_in))
    mu_out, sd_out = raw_out.mean(0), raw_out.std(0)
    sd_out = torch.where(sd_out > 0, sd_out, torch.ones_like(sd_out))
    X32 = ((raw_in - mu_in) / sd_in).contiguous()
    X16 = torch.empty_like(X32, dtype=torch.bfloat16)
    native.call("gade_to_bf16", X32.numel(), X32.data_ptr(), X16.data_ptr(), stream0)
    T32 = ((raw_out - mu_out) / sd_out).contiguous()
    # 4. training on the GPU with the package's kernels
    batch_rows = max(1, min(batch_rows, nrow))
    mlp = MLP(din, hidden, 2 * R, max_rows=batch_rows, seed=seed)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    hist = dict(loss=[], rows=nrow, rank=R, sv_ratio=float(sv[R - 1] / sv[0]), snapshots=len(snaps))
    tr0 = time.perf_counter()
    for ep in range(epochs):
        perm = torch.randperm(nrow, device="cuda", generator=gen)
        tot = torch.zeros((), dtype=torch.float64, device="cuda")
        for s in range(0, nrow - batch_rows + 1, batch_rows):
            idx = perm[s:s + batch_rows]
            xb, tb = X16[idx].contiguous(), T32[idx].contiguous()
            rl = mlp.train_batch(xb, tb, batch_rows, lr * (0.5 ** (ep // max(1, epochs // 4))), stream0)
            tot += rl.sum()
        hist["loss"].append(float(tot) / (nrow // batch_rows * batch_rows * 2 * R))
    torch.cuda.synchronize()
    hist["train_s"] = time.perf_counter() - tr0
    if log:
        log(f"trained {epochs} epochs on {nrow} rows: loss {hist['loss'][0]:.3e} -> {hist['loss'][-1]:.3e}, "
            f"{hist['train_s']:.1f}s")
    return LearnedModel(U, mlp, mu_in, sd_in, mu_out, sd_out, hist)


class LearnedGuess:
    """Drives a mixed-precision batch with the model's guess: after every
    step it projects the new states, runs the network for the next step and
    writes U c into the batch's guess buffer, all in one C-ABI call
    (gade_learned_guess_step) on the batch's stream; torch only allocates.
    The pulse factors of the next step come from device memory, so nothing
    is copied or synchronised between steps."""

    def __init__(self, model: LearnedModel, batch: Batch, limit: float = 1.0):
        self.m, self.b = model, batch
        self.np = batch.npulse
        R, n = model.R, model.n
        mlp = model.mlp
        assert self.np <= mlp.max_rows
        self.hist = torch.zeros(K_HIST, self.np, R, dtype=torch.complex128, device="cuda")
        self.count = 0
        self.head = K_HIST - 1
        self.scratch_b = native.call("gade_pod_project_scratch", n, R, self.np)
        self.scratch = torch.empty(self.scratch_b, dtype=torch.uint8, device="cuda")
        self.x16 = torch.empty(self.np, mlp.din, dtype=torch.bfloat16, device="cuda")
        self.c = torch.empty(self.np, R, dtype=torch.complex64, device="cuda")
        self.scale = torch.empty(self.np, dtype=torch.float32, device="cuda")
        self.ft = torch.empty(self.np, 12, dtype=torch.float64, device="cuda")
        self.corr, self.ld = batch.guess_buffer()
        self.xptr, self.xld = batch.state_device()
        self.limit = limit
        self.used = 0
        self.guess_on = None
        P = native.LearnedGuessPlan()
        P.n, P.R, P.npulse, P.K = n, R, self.np, K_HIST
        P.din, P.dh, P.dout = mlp.din, mlp.dh, mlp.dout
        P.U, P.hist, P.x, P.ldx = model.U.data_ptr(), self.hist.data_ptr(), self.xptr, self.xld
        P.scratch, P.scratch_bytes = self.scratch.data_ptr(), self.scratch_b
        P.mu_in, P.sd_in = model.mu_in.data_ptr(), model.sd_in.data_ptr()
        P.mu_out, P.sd_out = model.mu_out.data_ptr(), model.sd_out.data_ptr()
        P.x16 = self.x16.data_ptr()
        for i in range(3):
            P.W16[i] = mlp.W16[i].data_ptr()
            P.bias[i] = mlp.b[i].data_ptr()
        P.H1, P.H2, P.out = mlp.H1.data_ptr(), mlp.H2.data_ptr(), mlp.out.data_ptr()
        P.H1_16, P.H2_16 = mlp.H1_16.data_ptr(), mlp.H2_16.data_ptr()
        P.c, P.scale, P.corr, P.ldcorr, P.limit = self.c.data_ptr(), self.scale.data_ptr(), self.corr, self.ld, limit
        self.plan = P
        self._lib = native.load_library()

    def _use(self, on: bool):
        if on != self.guess_on:
            self.b.use_guess(on)
            self.guess_on = on

    def advance(self, ft_next_dev: int | None) -> bool:
        """Project the batch's current states into the history and, once K
        states are there and ft_next_dev (device address of the next step's
        [npulse, 12] pulse-factor reals) is given, prepare the guess for the
        next step.  Returns whether the next step uses it."""
        self.head = (self.head + 1) % K_HIST
        self.count += 1
        infer = self.count >= K_HIST and ft_next_dev is not None
        native._check(self._lib.gade_learned_guess_step(native.C.byref(self.plan), self.head,
                                                        ft_next_dev if infer else None, self.b.stream()))
        self._use(infer)
        if infer:
            self.used += 1
        return infer

    def observe(self):
        """Project the batch's current states into the history."""
        self.advance(None)

    def prepare(self, ft_next: np.ndarray) -> bool:
        """Guess for the next step from host pulse factors ft_next ([npulse,
        12] reals), on the newest projection already in the history (after
        observe): the network half of advance, for callers without device
        pulse factors."""
        if self.count < K_HIST:
            self._use(False)
            return False
        m, st = self.m, self.b.stream()
        # a blocking copy on torch's stream: no torch work is ever queued on
        # the batch's stream (the batch owns and destroys it)
        self.ft.copy_(torch.from_numpy(ft_next))
        native.call("gade_learned_features", self.np, m.R, K_HIST, self.head, self.hist.data_ptr(),
                    self.ft.data_ptr(), m.mu_in.data_ptr(), m.sd_in.data_ptr(), self.x16.data_ptr(), None, st)
        out = m.mlp.forward(self.x16, self.np, st)
        native.call("gade_learned_outputs", self.np, m.R, K_HIST, self.head, out.data_ptr(), m.mu_out.data_ptr(),
                    m.sd_out.data_ptr(), self.hist.data_ptr(), self.limit, self.c.data_ptr(),
                    self.scale.data_ptr(), st)
        native.call("gade_pod_expand", m.n, m.R, m.U.data_ptr(), self.c.data_ptr(), self.scale.data_ptr(),
                    self.np, self.corr, self.ld, st)
        self._use(True)
        self.used += 1
        return True


def run_held_out(problem: Problem, pulses, nsteps: int, tol: float, precision: str, model: LearnedModel | None,
                 limit: float = 1.0, **batch_kw):
    """Held-out pulses for nsteps steps: plain (model None) or with the
    learned guess.  Returns (final states [npulse, n] complex128 numpy,
    per-step stats, device ms of the whole run)."""
    grids = [step_times(p["maxtime"], p["ntime"]) for p in pulses]
    b = Batch(problem, [g[0] for g in grids], None, precision=precision, **batch_kw)
    lg = LearnedGuess(model, b, limit=limit) if model is not None else None
    ft_all = [_pulse_factors(pulses, grids, j) for j in range(nsteps + 1)]
    ft_dev = torch.from_numpy(np.stack(ft_all)).cuda() if lg is not None else None   # [nsteps+1][npulse][12]
    if lg is not None:
        lg.advance(None)                                        # x_0
    st = torch.cuda.ExternalStream(b.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    torch.cuda.synchronize()
    e0.record(st)
    for j in range(nsteps):
        stats.append(b.step(_ft_complex(ft_all[j]), maxit=500, tol=tol))
        if lg is not None:
            lg.advance(ft_dev[j + 1].data_ptr())
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    xs = np.stack([b.get_x(k) for k in range(len(pulses))])
    b.close()
    return xs, stats, ms


def intensity_pulses(n: int, seed: int, omega: float, cycles: int, ntime: int) -> list[dict]:
    """Seeded pulses that differ in Intensity only (log-uniform in [1, 100]),
    so that they share g, dt and the preconditioner."""
    rng = np.random.default_rng(seed)
    E0 = np.exp(rng.uniform(0.0, math.log(100.0), n))
    T = cycles * 2 * math.pi / omega
    return [dict(E0=float(e), omega=omega, cycles=cycles, ntime=ntime, maxtime=T) for e in E0]


def experiment(params: dict, nsteps: int, ntrain: int = 32, nheld: int = 8, rank: int = 128, nsnap: int = 200,
               pod_pulses: int = 8, epochs: int = 30, seed: int = 1, tol: float = 1e-10, workdir: str | None = None,
               log=None, limit: float = 1.0) -> dict:
    """The learned-guess protocol: POD + network from `ntrain` seeded training
    pulses (plain FP64 trajectories), then `nheld` seeded held-out pulses run
    four ways for `nsteps` steps: FP64 at tol 1e-12 (reference), plain FP64 at
    `tol`, mixed precision with the extrapolated guess and with the learned
    guess (both at `tol`).  Pulses differ in Intensity only (log-uniform in
    [1, 100]).  Returns steps/s, iterations, initial residuals and final-state
    errors (relative L2, bound and continuum populations) of each run."""
    import tempfile
    from .gen import generate
    from .populations import Eigenbasis
    say = log or (lambda *a: None)
    own = workdir is None
    tmp = tempfile.TemporaryDirectory() if own else None
    d = tmp.name if own else workdir
    if not os.path.exists(os.path.join(d, "H.csr")):
        generate(params, d)
    lmax = params["Nl"] if params["Nl"] else 2 * params["Nkappa"] + 1
    prob = Problem(d, lmax)
    mk = lambda n, s: intensity_pulses(n, s, params["Omega"], params["Cycles"], params["Ntime"])  # noqa: E731
    train, held = mk(ntrain, 100 + seed), mk(nheld, 200 + seed)
    out = {"params": params, "steps_per_pulse": nsteps, "train_pulses": ntrain, "held_out_pulses": nheld,
           "limit": limit,
           "seeds": {"train": 100 + seed, "held_out": 200 + seed, "pod_and_network": seed}, "tol": tol}
    t0 = time.perf_counter()
    model = build_model(prob, train, nsteps, rank=rank, nsnap=nsnap, pod_pulses=pod_pulses, seed=seed,
                        epochs=epochs, tol=tol, log=say)
    out["build_s"] = time.perf_counter() - t0
    out["model"] = {k: model.history[k] for k in ("rows", "rank", "sv_ratio", "snapshots", "train_s")}
    out["model"]["loss_per_epoch"] = model.history["loss"]
    kap, _ = prob.blocks()
    eb = Eigenbasis(d, kap)
    xr, _, ms_ref = run_held_out(prob, held, nsteps, 1e-12, "fp64", None)
    pref = [eb.populations(x) for x in xr]
    out["reference_fp64_tol1e-12"] = {"steps_per_s": nheld * nsteps / (ms_ref / 1e3),
                                      "populations_mean": {k: float(np.mean([p[k] for p in pref])) for k in pref[0]}}
    say("reference done", out["reference_fp64_tol1e-12"])
    for tag, prec, mdl in (("fp64", "fp64", None), ("mixed", "mixed", None), ("learned_mixed", "mixed", model)):
        if prec == "fp64" and tol == 1e-12:
            xs, st, ms = xr, None, ms_ref                       # the reference run itself
        else:
            xs, st, ms = run_held_out(prob, held, nsteps, tol, prec, mdl, limit=limit)
        err = np.linalg.norm(xs - xr, axis=1) / np.linalg.norm(xr, axis=1)
        pops = [eb.populations(x) for x in xs]
        rec = {"steps_per_s": nheld * nsteps / (ms / 1e3),
               "iters_per_step": float(np.mean([[r["iters"] for r in row] for row in st])) if st else None,
               "final_l2_err_max": float(err.max()), "final_l2_err_mean": float(err.mean()),
               "bound_abs_err_max": max(abs(p["bound"] - q["bound"]) for p, q in zip(pops, pref)),
               "continuum_abs_err_max": max(abs(p["continuum"] - q["continuum"]) for p, q in zip(pops, pref))}
        if prec == "mixed":
            ini = np.array([[r["init_residual"] for r in row] for row in st])[K_HIST:]
            rec["init_residual_mean"] = float(ini.mean())
            rec["init_residual_median"] = float(np.median(ini))
            rec["fp64_residual_passes_per_step"] = float(np.mean([[r["refinements"] for r in row] for row in st]))
        out[tag] = rec
        say(tag, rec)
    base = out["fp64"]["steps_per_s"]
    out["speedup_vs_fp64"] = {k: out[k]["steps_per_s"] / base for k in ("mixed", "learned_mixed")}
    prob.close()
    if tmp is not None:
        tmp.cleanup()
    return out


def time_gemm(M: int, N: int, K: int, reps: int = 20, path: int = 0, seed: int = 0) -> dict:
    """CUDA-event time of gade_gemm_bf16 on seeded BF16 operands A (M x K,
    K-contiguous) and B (K x N, N-contiguous), FP32 output: 3 warm-up
    launches, then the average of `reps`; path 1 forces the plain-load
    staging.  Checked against torch's FP32 product of the same operands."""
    import ctypes
    g = torch.Generator(device="cpu").manual_seed(seed)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(K, N, generator=g).to(torch.bfloat16).cuda()
    C = torch.empty(M, N, device="cuda")
    native.call("gade_learned_set_gemm_options", int(path), 0, 0)
    try:
        def go():
            native.call("gade_gemm_bf16", M, N, K, A.data_ptr(), K, 1, B.data_ptr(), N, 1, None, None, 0, 0,
                        C.data_ptr(), N, None, 0, 0)
        for _ in range(3):
            go()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            go()
        e1.record()
        torch.cuda.synchronize()
    finally:
        native.call("gade_learned_set_gemm_options", 0, 0, 0)
    ms = e0.elapsed_time(e1) / reps
    ref = A.float() @ B.float()
    flags = ctypes.c_int32(-1)
    native.call("gade_learned_status", ctypes.byref(flags))
    tma = native.load_library().gade_gemm_bf16_path(M, N, K, A.data_ptr(), K, 1, B.data_ptr(), N, 1)
    return {"M": M, "N": N, "K": K, "staging": "tensor copies" if tma else "plain loads", "us": ms * 1e3,
            "tflops": 2.0 * M * N * K / ms / 1e9, "rel_err": float((C - ref).norm() / ref.norm()),
            "status": flags.value}


def main(argv=None) -> int:
    import argparse
    import json
    import sys
    from .gen import CONFIGS
    if argv is None:
        argv = sys.argv[1:]
    if argv and argv[0] == "--gemm":
        # --gemm M N K [reps [path]]: time one GEMM shape of the learned-guess kernels
        vals = [int(v) for v in argv[1:]]
        print(json.dumps(time_gemm(*vals)))
        return 0
    ap = argparse.ArgumentParser(prog="python -m dirac_hydrogen_code_gb300.learned")
    ap.add_argument("--workload", default="nondipole_large", choices=sorted(CONFIGS))
    ap.add_argument("--steps", type=int, default=0, help="steps per pulse (0: the whole pulse, Ntime+1)")
    ap.add_argument("--train", type=int, default=32)
    ap.add_argument("--held", type=int, default=8)
    ap.add_argument("--rank", type=int, default=128)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--tol", type=float, default=1e-10, help="residual tolerance of the compared runs")
    ap.add_argument("--limit", type=float, default=1.0,
                    help="a prediction is used while |c| <= limit * |projection of the last state change|")
    ap.add_argument("--out", default=None, help="write the result JSON here")
    args = ap.parse_args(argv)
    params = CONFIGS[args.workload]
    T = params["Cycles"] * 2 * math.pi / params["Omega"]
    nsteps = args.steps or len(step_times(T, params["Ntime"])[1])
    res = experiment(params, nsteps, args.train, args.held, rank=args.rank, epochs=args.epochs, tol=args.tol,
                     log=lambda *a: print(*a, file=sys.stderr, flush=True), limit=args.limit)
    res["workload"] = args.workload
    txt = json.dumps(res)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)
    print(txt)
    return 0


if __name__ == "__main__":
    import sys as _sys
    _sys.exit(main())
