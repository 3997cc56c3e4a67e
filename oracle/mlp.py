"""CPU restatement of the alpha-guess MLP (test infrastructure only).

Network n_in -> 32 -> 32 -> 1 with tanh hidden layers:
    x~ = x * input_scale
    h1 = tanh(W1 x~ + b1);  h2 = tanh(W2 h1 + b2);  y = w3 . h2 + b3
    guess = 2 + output_scale * y
    loss  = mean((guess - alpha*)^2)
Used to check the CUDA forward/backward (float64 analytic gradients and
central finite differences) and the BF16 tensor-core inference (operands
rounded to bfloat16, products accumulated in float).
"""
from __future__ import annotations

import numpy as np


def forward(m, X):
    x = X * m.input_scale
    h1 = np.tanh(x @ m.w1.T + m.b1)
    h2 = np.tanh(h1 @ m.w2.T + m.b2)
    y = h2 @ m.w3 + m.b3
    return x, h1, h2, y


def loss_and_grad(m, X, t):
    """float64 loss and analytic gradient (dict of arrays)."""
    X = X.astype(np.float64)
    mm = _as64(m)
    x, h1, h2, y = forward(mm, X)
    e = 2.0 + mm.output_scale * y - t
    n = len(t)
    loss = float(np.mean(e * e))
    dy = 2.0 * e * mm.output_scale / n
    g = {"b3": dy.sum(), "w3": dy @ h2}
    dh2 = np.outer(dy, mm.w3) * (1 - h2 ** 2)
    g["w2"] = dh2.T @ h1
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ mm.w2) * (1 - h1 ** 2)
    g["w1"] = dh1.T @ x
    g["b1"] = dh1.sum(0)
    return loss, g


def loss_only(m, X, t):
    mm = _as64(m)
    *_, y = forward(mm, X.astype(np.float64))
    e = 2.0 + mm.output_scale * y - t
    return float(np.mean(e * e))


def bf16(a):
    """Round float32 values to bfloat16 (round to nearest even), as floats."""
    a = np.asarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def predict_bf16(m, X):
    """The fused kernel's inference: BF16 operands, float accumulation."""
    x = bf16(X.astype(np.float32) * m.input_scale.astype(np.float32)).astype(np.float64)
    w1 = bf16(m.w1).astype(np.float64)
    w2 = bf16(m.w2).astype(np.float64)
    h1 = np.tanh(x @ w1.T + m.b1)
    h1 = bf16(h1.astype(np.float32)).astype(np.float64)
    h2 = np.tanh(h1 @ w2.T + m.b2)
    y = h2 @ m.w3.astype(np.float64) + m.b3
    return 2.0 + m.output_scale * y


def _as64(m):
    class M:
        pass
    mm = M()
    for k in ("input_scale", "w1", "b1", "w2", "b2", "w3"):
        setattr(mm, k, np.asarray(getattr(m, k), np.float64))
    mm.b3 = float(m.b3)
    mm.output_scale = float(m.output_scale)
    return mm
