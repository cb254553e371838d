"""The FP64 warm-start network of the oracle against finite differences and
torch's bfloat16 rounding (CPU only): the oracle of the CUDA training kernels is
itself checked here."""
import numpy as np
import pytest
import torch

from oracle import mlp_oracle as M


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(M.P_N, np.float64)
    p[M.P_MU:M.P_MU + 5] = rng.normal(size=5)
    p[M.P_IS:M.P_IS + 5] = rng.uniform(0.5, 2.0, size=5)
    p[M.P_W1:M.P_B1] = rng.normal(size=M.H * M.F) * 0.6
    p[M.P_B1:M.P_W2] = rng.normal(size=M.H) * 0.1
    p[M.P_W2:M.P_B2] = rng.normal(size=M.H * M.H) * 0.2
    p[M.P_B2:M.P_W3] = rng.normal(size=M.H) * 0.1
    p[M.P_W3:M.P_B3] = rng.normal(size=M.H) * 0.2
    p[M.P_B3] = 0.3
    p[M.P_YS] = 2.0
    p[M.P_YM] = -1.0
    return p


def test_bf16_round_matches_torch():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=4000) * 10.0 ** rng.integers(-8, 8, size=4000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, -3.5e-3]]).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).float().numpy().astype(np.float64)
    assert np.array_equal(M.bf16_round(x), ref)


@pytest.mark.parametrize("over", [1.0, 6.0])
def test_gradient_matches_finite_differences(over):
    rng = np.random.default_rng(2)
    p = _params()
    X = np.zeros((64, 8))
    X[:, :5] = rng.normal(size=(64, 5))
    T = rng.normal(size=64)
    loss, g = M.loss_and_grad(p, X, T, over_weight=over)
    assert loss > 0
    h = 1e-6
    idx = np.concatenate([rng.choice(np.arange(M.P_W1, M.P_B3 + 1), 60, replace=False), [M.P_B3, M.P_B1, M.P_W3]])
    for k in idx:
        if M.P_W1 <= k < M.P_B1 and (k - M.P_W1) % M.F >= 5:
            continue  # weights of the unused feature slots multiply zero
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_and_grad(pp, X, T, over_weight=over)[0] - M.loss_and_grad(pm, X, T, over_weight=over)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])
    # nothing outside the trained block
    assert np.all(g[:M.P_W1] == 0) and np.all(g[M.P_B3 + 1:] == 0)


def test_predict_units_and_adam_decreases_loss():
    rng = np.random.default_rng(3)
    p = _params(1)
    X = np.zeros((256, 8))
    X[:, :5] = rng.normal(size=(256, 5))
    y = M.forward(p, X)["y"]
    assert np.allclose(M.predict(p, X), y * 2.0 - 1.0)
    T = np.tanh(X[:, 0]) + 0.5 * X[:, 3]
    m = np.zeros(M.P_N)
    v = np.zeros(M.P_N)
    l0 = M.loss_and_grad(p, X, T)[0]
    for s in range(200):
        _, g = M.loss_and_grad(p, X, T)
        M.adam(p, m, v, g, 3e-3, s)
    assert M.loss_and_grad(p, X, T)[0] < 0.25 * l0
