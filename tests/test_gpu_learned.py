"""GPU kernels of the learned initial guess against the numpy oracle
(oracle/mlp.py) and numpy linear algebra:

  * BF16 tcgen05 GEMM (every transposition, ragged sizes, bias, ReLU,
    mask): relative error <= 1e-5 against float64 products of the same
    BF16-rounded operands (FP32 accumulation)
  * MLP loss gradients: relative Frobenius error <= 2e-3 per parameter
    against the oracle with the same BF16 rounding points
  * Adam: <= 1e-5 relative against the float64 update
  * POD projection / expansion: <= 1e-6 relative (complex64 basis, FP32
    products), the FP64 projection <= 1e-12
"""
import ctypes

import numpy as np
import pytest
import torch

import mlp as M
from dirac_hydrogen_code_gb300 import native
from dirac_hydrogen_code_gb300.learned import MLP

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _bf(x):
    return torch.from_numpy(np.asarray(x, np.float32)).cuda().to(torch.bfloat16)


def _gemm_options(path=0, wait_limit=0, withhold=0):
    native.call("gade_learned_set_gemm_options", path, wait_limit, withhold)


def _status():
    flags = ctypes.c_int32(-1)
    native.call("gade_learned_status", ctypes.byref(flags))
    return flags.value


def _tma_layout(rows, K, s_row, s_k):
    """Whether an operand (rows x K, element (r, k) at r*s_row + k*s_k) can
    be staged by 2-D tensor copies: unit stride along one dimension and a
    16-byte row stride (free for a single row)."""
    def ok(inner, outer, ld):
        stride = 2 * ld
        if outer == 1 and stride < 2 * inner:
            return True
        return stride % 16 == 0 and stride >= 2 * inner
    if s_k == 1:
        return ok(K, rows, s_row)
    return s_row == 1 and ok(rows, K, s_k)


# (M, N, K): ragged tiles, K blocks past the copy ring's depth, row strides
# of a multiple of 8 elements (tensor copies) and not (plain loads)
@pytest.mark.parametrize("M_,N_,K_", [(1, 8, 16), (37, 70, 45), (130, 256, 1036), (512, 256, 256),
                                      (200, 136, 520)])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_gemm_bf16(native_lib, M_, N_, K_, ta, tb):
    rng = np.random.default_rng(M_ + N_ + K_)
    A = M.bf16(rng.standard_normal((M_, K_)))
    B = M.bf16(rng.standard_normal((K_, N_)))
    bias = rng.standard_normal(N_).astype(np.float32)
    mask = rng.standard_normal((M_, N_)).astype(np.float32)
    Ad = _bf(A.T.copy() if ta else A)
    Bd = _bf(B.T.copy() if tb else B)
    sa = (1, M_) if ta else (K_, 1)
    sb = (1, K_) if tb else (N_, 1)
    lib = native.load_library()
    tma = lib.gade_gemm_bf16_path(M_, N_, K_, Ad.data_ptr(), *sa, Bd.data_ptr(), *sb)
    assert tma == int(_tma_layout(M_, K_, *sa) and _tma_layout(N_, K_, sb[1], sb[0]))
    C = torch.empty(M_, N_, device="cuda")
    C16 = torch.empty(M_, N_, dtype=torch.bfloat16, device="cuda")
    Cld = torch.empty(M_, N_, device="cuda")
    bd, md = torch.from_numpy(bias).cuda(), torch.from_numpy(mask).cuda()
    for act, use_mask in [(0, False), (1, False), (0, True)]:
        args = (M_, N_, K_, Ad.data_ptr(), *sa, Bd.data_ptr(), *sb, bd.data_ptr(),
                md.data_ptr() if use_mask else None, N_, act)
        native.call("gade_gemm_bf16", *args, C.data_ptr(), N_, C16.data_ptr(), N_, 0)
        try:                                    # the same product staged by plain loads
            _gemm_options(path=1)
            native.call("gade_gemm_bf16", *args, Cld.data_ptr(), N_, None, 0, 0)
        finally:
            _gemm_options()
        torch.cuda.synchronize()
        ref = A @ B + bias
        if use_mask:
            ref = ref * (mask > 0)
        if act:
            ref = np.maximum(ref, 0)
        got = C.cpu().numpy().astype(np.float64)
        assert _rel(got, ref) <= 1e-5, (act, use_mask)
        assert np.array_equal(C16.float().cpu().numpy(), M.bf16(got).astype(np.float32))
        assert torch.equal(C, Cld)              # same MMAs in the same order: same bits
    assert _status() == 0                       # no tensor-core wait ran out


def test_gemm_wait_timeout_sets_status(native_lib):
    """The tensor-copy stager withholds its copies (a flag nothing sets): the
    MMA thread's bounded wait runs out, the CTAs free their tensor memory
    and return, the status word says so, and the next GEMM is exact."""
    rng = np.random.default_rng(5)
    M_, N_, K_ = 256, 128, 192
    A = M.bf16(rng.standard_normal((M_, K_)))
    B = M.bf16(rng.standard_normal((K_, N_)))
    Ad, Bd = _bf(A), _bf(B)
    assert native.load_library().gade_gemm_bf16_path(M_, N_, K_, Ad.data_ptr(), K_, 1, Bd.data_ptr(), N_, 1) == 1
    C = torch.full((M_, N_), -7.0, device="cuda")
    assert _status() == 0
    try:
        _gemm_options(wait_limit=1000, withhold=1)
        native.call("gade_gemm_bf16", M_, N_, K_, Ad.data_ptr(), K_, 1, Bd.data_ptr(), N_, 1, None, None, 0, 0,
                    C.data_ptr(), N_, None, 0, 0)
        torch.cuda.synchronize()
        assert _status() == 1
        assert bool(torch.all(C == -7.0))       # no tile written
    finally:
        _gemm_options()
    native.call("gade_gemm_bf16", M_, N_, K_, Ad.data_ptr(), K_, 1, Bd.data_ptr(), N_, 1, None, None, 0, 0,
                C.data_ptr(), N_, None, 0, 0)
    torch.cuda.synchronize()
    assert _status() == 0
    assert _rel(C.cpu().numpy().astype(np.float64), A @ B) <= 1e-5


def test_mlp_gradients_match_oracle(native_lib):
    din, dh, dout, rows = 1036, 256, 256, 192
    mlp = MLP(din, dh, dout, max_rows=rows, seed=3)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((rows, din))
    T = rng.standard_normal((rows, dout))
    with torch.no_grad():
        for i in range(3):
            mlp.b[i].copy_(torch.from_numpy(rng.standard_normal(mlp.b[i].numel()) * 0.1))
    mlp.sync_bf16(0)
    X16 = _bf(X)
    Td = torch.from_numpy(T.astype(np.float32)).cuda()
    out = mlp.forward(X16, rows, 0)
    mlp.backward(X16, Td, rows, 0)
    torch.cuda.synchronize()
    params = dict(W1=mlp.W[0].double().cpu().numpy(), b1=mlp.b[0].double().cpu().numpy(),
                  W2=mlp.W[1].double().cpu().numpy(), b2=mlp.b[1].double().cpu().numpy(),
                  W3=mlp.W[2].double().cpu().numpy(), b3=mlp.b[2].double().cpu().numpy())
    f = M.forward(params, X)
    assert _rel(out.double().cpu().numpy(), f["out"]) <= 1e-3
    loss, g = M.loss_and_grads(params, X, T.astype(np.float32).astype(np.float64))
    assert abs(float(mlp.rowloss[:rows].sum()) / (rows * dout) - loss) <= 1e-4 * loss
    names = ["W1", "b1", "W2", "b2", "W3", "b3"]
    for name, gd in zip(names, mlp.grads):
        assert _rel(gd.double().cpu().numpy(), g[name]) <= 2e-3, name


def test_adam_matches_oracle(native_lib):
    rng = np.random.default_rng(7)
    n = 5000
    w, g = rng.standard_normal(n), rng.standard_normal(n)
    m, v = rng.standard_normal(n) * 0.1, np.abs(rng.standard_normal(n)) * 0.1
    wd, gd, md, vd = (torch.from_numpy(a.astype(np.float32)).cuda() for a in (w, g, m, v))
    w16 = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    native.call("gade_adam", n, wd.data_ptr(), w16.data_ptr(), gd.data_ptr(), md.data_ptr(), vd.data_ptr(),
                1e-3, 0.9, 0.999, 1e-8, 3, 0)
    torch.cuda.synchronize()
    f32 = lambda a: a.astype(np.float32).astype(np.float64)   # noqa: E731
    wr, mr, vr = M.adam(f32(w), f32(g), f32(m), f32(v), 3)
    assert _rel(wd.double().cpu().numpy(), wr) <= 1e-6
    assert _rel(md.double().cpu().numpy(), mr) <= 1e-6 and _rel(vd.double().cpu().numpy(), vr) <= 1e-6
    assert np.array_equal(w16.float().cpu().numpy(), M.bf16(wd.cpu().numpy()).astype(np.float32))


def test_pod_project_and_expand(native_lib):
    rng = np.random.default_rng(9)
    n, R, P = 70001, 48, 5
    U = (rng.standard_normal((R, n)) + 1j * rng.standard_normal((R, n))).astype(np.complex64)
    X = rng.standard_normal((P, n)) + 1j * rng.standard_normal((P, n))
    Ud, Xd = torch.from_numpy(U).cuda(), torch.from_numpy(X).cuda()
    coef = torch.empty(P, R, dtype=torch.complex128, device="cuda")
    sb = native.call("gade_pod_project_scratch", n, R, P)
    scratch = torch.empty(sb, dtype=torch.uint8, device="cuda")
    native.call("gade_pod_project", n, R, Ud.data_ptr(), Xd.data_ptr(), n, P, coef.data_ptr(), scratch.data_ptr(),
                sb, 0)
    torch.cuda.synchronize()
    ref = X @ U.astype(np.complex128).conj().T
    assert _rel(coef.cpu().numpy(), ref) <= 1e-6                # FP32 products and chunk sums
    coef64 = torch.empty_like(coef)
    native.call("gade_pod_project_fp64", n, R, Ud.data_ptr(), Xd.data_ptr(), n, P, coef64.data_ptr(),
                scratch.data_ptr(), sb, 0)
    torch.cuda.synchronize()
    assert _rel(coef64.cpu().numpy(), ref) <= 1e-12             # FP64 (training targets)
    # a state change of 1e-4 projected as the difference of two projections
    # (the plausibility bound of gade_learned_outputs) keeps ~1e-3
    X2 = X + 1e-4 * (rng.standard_normal((P, n)) + 1j * rng.standard_normal((P, n)))
    coef2 = torch.empty_like(coef)
    native.call("gade_pod_project", n, R, Ud.data_ptr(), torch.from_numpy(X2).cuda().data_ptr(), n, P,
                coef2.data_ptr(), scratch.data_ptr(), sb, 0)
    torch.cuda.synchronize()
    dref = (X2 - X) @ U.astype(np.complex128).conj().T
    assert _rel((coef2 - coef).cpu().numpy(), dref) <= 1e-2
    c = (rng.standard_normal((P, R)) + 1j * rng.standard_normal((P, R))).astype(np.complex64)
    scale = np.array([1, 0, 1, 1, 0.5], np.float32)
    cd, sd = torch.from_numpy(c).cuda(), torch.from_numpy(scale).cuda()
    y = torch.empty(P, n, dtype=torch.complex128, device="cuda")
    native.call("gade_pod_expand", n, R, Ud.data_ptr(), cd.data_ptr(), sd.data_ptr(), P, y.data_ptr(), n, 0)
    torch.cuda.synchronize()
    yref = (scale[:, None] * c.astype(np.complex128)) @ U.astype(np.complex128)
    assert _rel(y.cpu().numpy(), yref) <= 1e-6
    assert np.all(y[1].cpu().numpy() == 0)


def test_fused_guess_step_matches_separate_calls(workdirs, native_lib):
    """LearnedGuess.advance (one gade_learned_guess_step per step, pulse
    factors from device memory) and the separate projection / features /
    network / outputs / expansion calls (observe + prepare, pulse factors
    from the host) give bit-identical guesses over a few mixed steps of two
    batches on the same pulses."""
    from dirac_hydrogen_code_gb300 import learned as L
    from dirac_hydrogen_code_gb300.cn import step_times
    from dirac_hydrogen_code_gb300.native import Batch, Problem
    d, params, info = workdirs["tiny_nondipole"]
    prob = Problem(d, info["lmax"])
    pulses = L.intensity_pulses(2, 5, params["Omega"], params["Cycles"], params["Ntime"])
    grids = [step_times(p["maxtime"], p["ntime"]) for p in pulses]
    rng = np.random.default_rng(9)
    R = 6
    Q, _ = np.linalg.qr(rng.standard_normal((prob.n, R)) + 1j * rng.standard_normal((prob.n, R)))
    din = L.K_HIST * 2 * R + 12
    mlp = MLP(din, 32, 2 * R, 8, seed=3)
    ones, zeros = torch.ones, torch.zeros
    model = L.LearnedModel(Q.T.conj(), mlp, zeros(din), ones(din), zeros(2 * R), 1e-3 * ones(2 * R), {})
    nsteps = 8
    ft_all = [L._pulse_factors(pulses, grids, j) for j in range(nsteps + 1)]
    ft_dev = torch.from_numpy(np.stack(ft_all)).cuda()
    runs = []
    for fused in (True, False):
        # fixed operator and chunking: the timed choices may differ between batches
        b = Batch(prob, [g[0] for g in grids], None, precision="mixed", chunk_splines=16)
        b.set_operator(0)
        lg = L.LearnedGuess(model, b, limit=1e30)
        corr_ptr, ld = b.guess_buffer()
        corr = L.device_view(corr_ptr, (2, ld))
        lg.advance(None)
        seen = []
        for j in range(nsteps):
            b.step(L._ft_complex(ft_all[j]), maxit=500, tol=1e-10)
            if fused:
                used = lg.advance(ft_dev[j + 1].data_ptr())
            else:
                lg.observe()
                used = lg.prepare(ft_all[j + 1])
            torch.cuda.synchronize()
            seen.append((used, corr[:, :prob.n].clone().cpu().numpy()))
        runs.append((seen, np.stack([b.get_x(k) for k in range(2)])))
        b.close()
    (sa, xa), (sb, xb) = runs
    assert [u for u, _ in sa] == [u for u, _ in sb]
    assert sum(u for u, _ in sa) == sum(j + 2 >= L.K_HIST for j in range(nsteps))
    for (_, ca), (_, cb) in zip(sa, sb):
        assert np.array_equal(ca, cb)
    assert np.any(sa[-1][1] != 0)
    assert np.array_equal(xa, xb)
