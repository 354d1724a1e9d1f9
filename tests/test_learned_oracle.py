"""CPU checks of the learned guess's oracle and host math: the numpy MLP
oracle's gradients against finite differences, its BF16 rounding against
PyTorch's, and the POD basis of the method of snapshots."""
import numpy as np
import pytest

import mlp as M


def _params(rng, din, dh, dout, scale=0.3):
    return dict(W1=rng.standard_normal((din, dh)) * scale, b1=rng.standard_normal(dh) * 0.1,
                W2=rng.standard_normal((dh, dh)) * scale, b2=rng.standard_normal(dh) * 0.1,
                W3=rng.standard_normal((dh, dout)) * scale, b3=rng.standard_normal(dout) * 0.1)


def test_exact_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng, 7, 6, 5)
    X, T = rng.standard_normal((9, 7)), rng.standard_normal((9, 5))
    _, g = M.loss_and_grads_exact(p, X, T)
    h = 1e-6
    for k in p:
        flat = p[k].reshape(-1)
        for idx in rng.choice(flat.size, size=min(5, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp, _ = M.loss_and_grads_exact(p, X, T)
            flat[idx] = old - h
            lm, _ = M.loss_and_grads_exact(p, X, T)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k].reshape(-1)[idx]) <= 1e-6 * max(1.0, abs(fd)), (k, idx)


def test_rounded_gradients_close_to_exact():
    rng = np.random.default_rng(1)
    p = _params(rng, 40, 32, 16)
    X, T = rng.standard_normal((64, 40)), rng.standard_normal((64, 16))
    _, ge = M.loss_and_grads_exact(p, X, T)
    _, gr = M.loss_and_grads(p, X, T)
    for k in ge:
        assert np.linalg.norm(gr[k] - ge[k]) <= 0.05 * np.linalg.norm(ge[k]), k


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-8, 8, 10000), [0.0, -0.0, 1.0, 3.0]])
    ref = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(M.bf16(x), ref)


def test_pod_basis_orthonormal_and_spanning():
    from dirac_hydrogen_code_gb300.learned import pod_basis
    rng = np.random.default_rng(3)
    n, m, r = 500, 40, 6
    modes = rng.standard_normal((r, n)) + 1j * rng.standard_normal((r, n))
    snaps = (rng.standard_normal((m, r)) + 1j * rng.standard_normal((m, r))) @ modes
    U, sv = pod_basis(snaps, 10)
    assert U.shape[0] == r                      # numerically zero directions are dropped
    assert np.allclose(U @ U.conj().T, np.eye(r), atol=1e-10)
    resid = snaps - (snaps @ U.conj().T) @ U
    assert np.linalg.norm(resid) <= 1e-9 * np.linalg.norm(snaps)
    assert np.all(np.diff(sv[:r]) <= 1e-9 * sv[0])
