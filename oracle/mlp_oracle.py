"""CPU oracle of the learned-start MLP (TEST INFRASTRUCTURE ONLY).

Float64 numpy restatement of the network that nla3d_gb300.learned trains with
the library's kernels (csrc/mlp.cu): hidden layers y = tanh(x W^T + b), a
linear output layer, weights rounded to BF16 (round to nearest, ties to even)
before every product, mean-squared-error loss.  The GPU gradients are checked
against this, and this against central finite differences.
"""
from __future__ import annotations

import numpy as np


def to_bf16(x: np.ndarray) -> np.ndarray:
    """Round float values to the nearest BF16 (ties to even); returns float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(Ws, bs, X):
    """Activations [X, h1, ..., out] with BF16-rounded weights."""
    acts = [np.asarray(X, dtype=np.float64)]
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = acts[-1] @ to_bf16(W).T + b
        acts.append(np.tanh(z) if l < len(Ws) - 1 else z)
    return acts


def loss_and_grads(Ws, bs, X, T):
    """MSE loss mean((out - T)^2) and its gradients w.r.t. W (through the BF16
    rounding, treated as identity) and b."""
    acts = forward(Ws, bs, X)
    out = acts[-1]
    n = out.size
    loss = float(((out - T) ** 2).sum() / n)
    d = 2.0 * (out - T) / n
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        if l < len(Ws) - 1:
            d = d * (1.0 - acts[l + 1] ** 2)
        gW[l] = d.T @ acts[l]
        gb[l] = d.sum(axis=0)
        d = d @ to_bf16(Ws[l])
    return loss, gW, gb
