"""FP64 restatement of the warm-start network -- test infrastructure only.

This module is the oracle for the CUDA forward, backward and Adam kernels of the
learned warm start (apbf_gb300/csrc/mlp.cu).  Only tests, the smoke check and the
benchmark's baseline leg may import it; the product never does.  The network has
no counterpart in the reference (cg-tuwien/APBF solves from lambda = 0 in every
Jacobi iteration, source/incompressibility.cpp:24), so there is nothing to pin it
to but its own mathematics: a ReLU perceptron with 8 feature slots (6 used by the
solver), two hidden layers of 64 and one output, on normalised features,
loss = mean over the batch of (y - t)^2.

Parameter vector (float32, offsets in floats): mu[8] @0, inv_sigma[8] @8,
W1[64][8] @16, b1[64] @528, W2[64][64] @592 (row = output), b2[64] @4688,
w3[64] @4752, b3 @4816, y_scale @4817, y_mean @4818, omega_max @4819 (read by the
solver's hook, not by the network), min_neighbors @4820 (likewise), 4821..4823
reserved; 4824 floats.

`bf16=True` rounds the operands of every tensor-core product to bfloat16 (round
to nearest even) where the kernels do, so that the remaining difference is the
FP32 accumulation order; `bf16=False` is the exact FP64 network.
"""
from __future__ import annotations

import numpy as np

P_MU, P_IS, P_W1, P_B1, P_W2, P_B2, P_W3, P_B3, P_YS, P_YM, P_OMEGA, P_NMIN, P_N = (0, 8, 16, 528, 592, 4688, 4752,
                                                                                4816, 4817, 4818, 4819, 4820, 4824)
H, F = 64, 8
TRAINED = slice(P_W1, P_B3 + 1)


def bf16_round(x: np.ndarray) -> np.ndarray:
    """float -> bfloat16 -> float with round-to-nearest-even (finite inputs)."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray) -> dict:
    p = np.asarray(p, dtype=np.float64)
    return {
        "mu": p[P_MU:P_MU + F], "is": p[P_IS:P_IS + F],
        "W1": p[P_W1:P_B1].reshape(H, F), "b1": p[P_B1:P_W2],
        "W2": p[P_W2:P_B2].reshape(H, H), "b2": p[P_B2:P_W3],
        "w3": p[P_W3:P_B3], "b3": p[P_B3], "ys": p[P_YS], "ym": p[P_YM],
    }


def _q(x, on):
    return bf16_round(x) if on else np.asarray(x, np.float64)


def forward(p: np.ndarray, X: np.ndarray, bf16: bool = False) -> dict:
    """Activations of the network on rows X (n x 8 features); y in the normalised space."""
    w = unpack(p)
    X = np.asarray(X, np.float64)
    if bf16:  # the kernel normalises in FP32, then rounds to BF16
        X32 = np.asarray(X, np.float32)
        xn = bf16_round((X32 - w["mu"].astype(np.float32)) * w["is"].astype(np.float32))
    else:
        xn = (X - w["mu"]) * w["is"]
    h1 = np.maximum(_q(xn, False) @ _q(w["W1"], bf16).T + w["b1"], 0.0)
    h2 = np.maximum(_q(h1, bf16) @ _q(w["W2"], bf16).T + w["b2"], 0.0)
    y = h2 @ w["w3"] + w["b3"]
    return {"xn": xn, "h1": h1, "h2": h2, "y": y}


def predict(p: np.ndarray, X: np.ndarray, bf16: bool = False) -> np.ndarray:
    """lambda in physical units: y * y_scale + y_mean."""
    w = unpack(p)
    return forward(p, X, bf16)["y"] * w["ys"] + w["ym"]


def loss_and_grad(p: np.ndarray, X: np.ndarray, T: np.ndarray, bf16: bool = False,
                  over_weight: float = 1.0) -> tuple[float, np.ndarray]:
    """Weighted mean squared error against normalised targets T -- mean of w e^2,
    e = y - T, w = over_weight where e < 0 and 1 elsewhere -- and its gradient
    (4824 floats, zero outside the trained block W1..b3)."""
    w = unpack(p)
    a = forward(p, X, bf16)
    T = np.asarray(T, np.float64)
    n = X.shape[0]
    e = a["y"] - T
    wt = np.where(e < 0, over_weight, 1.0)
    dy = 2.0 * wt * e / n
    dh2 = (a["h2"] > 0) * (dy[:, None] * w["w3"][None, :])
    dh1 = (a["h1"] > 0) * (_q(dh2, bf16) @ _q(w["W2"], bf16))
    g = np.zeros(P_N, np.float64)
    g[P_W1:P_B1] = (_q(dh1, bf16).T @ _q(a["xn"], bf16)).ravel()
    g[P_B1:P_W2] = dh1.sum(0)
    g[P_W2:P_B2] = (_q(dh2, bf16).T @ _q(a["h1"], bf16)).ravel()
    g[P_B2:P_W3] = dh2.sum(0)
    g[P_W3:P_B3] = dy @ a["h2"]
    g[P_B3] = dy.sum()
    return float(np.mean(wt * e * e)), g


def adam(p: np.ndarray, m: np.ndarray, v: np.ndarray, g: np.ndarray, lr: float, step: int,
         b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8) -> None:
    """One Adam update of the trained block in place (step = number of earlier steps)."""
    t = TRAINED
    m[t] = b1 * m[t] + (1 - b1) * g[t]
    v[t] = b2 * v[t] + (1 - b2) * g[t] * g[t]
    mh = m[t] / (1 - b1 ** (step + 1))
    vh = v[t] / (1 - b2 ** (step + 1))
    p[t] = p[t] - lr * mh / (np.sqrt(vh) + eps)
