"""CPU oracle of the ray -> cluster network (test infrastructure only).

A numpy restatement of the network's math: tanh-form GELU layers, softmax
cross-entropy, and their gradients by the chain rule. `bf16=True` rounds to
bfloat16 (round to nearest even) at the points where the GPU stores bf16:
inputs, weights, pre-activations, activations and back-propagated
gradients; accumulation stays fp32. With bf16=False and float64 the
gradients are checked against finite differences, which pins the math.
"""
from __future__ import annotations

import numpy as np

K_GELU = 0.7978845608028654  # sqrt(2 / pi)


def bf16(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    th = np.tanh(K_GELU * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + th) + 0.5 * x * (1.0 - th * th) * K_GELU * (1.0 + 3.0 * 0.044715 * x * x)


def unpack(p: np.ndarray, layout):
    return {name: p[o:o + int(np.prod(shape))].reshape(shape) for name, o, shape in layout}


def loss_grad(params: np.ndarray, layout, X: np.ndarray, labels: np.ndarray, n_classes: int, bf16_round: bool = True,
              dtype=np.float32):
    """Mean softmax-CE loss over rows with label >= 0 and the gradient of the
    sum of per-row losses divided by the number of such rows."""
    def r(a):  # the GPU's bf16 stores, or nothing
        return bf16(np.asarray(a, np.float32)).astype(dtype) if bf16_round else np.asarray(a, dtype)

    P = unpack(params.astype(dtype), layout)
    Wb = {k: (r(v) if k.startswith("W") else v) for k, v in P.items()}
    h = r(X)
    acts, zs = [h], []
    for k in range(1, 5):
        z = r(h @ Wb[f"W{k}"] + P[f"b{k}"])
        h = r(gelu(z))
        zs.append(z)
        acts.append(h)
    logits = (h @ Wb["W5"] + P["b5"]).astype(dtype)
    valid = labels >= 0
    nv = max(1, int(valid.sum()))
    z = logits[:, :n_classes]
    m = z.max(axis=1, keepdims=True)
    e = np.exp(z - m)
    s = e.sum(axis=1, keepdims=True)
    lab = np.where(valid, labels, 0)
    loss_rows = np.log(s[:, 0]) - (z[np.arange(len(z)), lab] - m[:, 0])
    loss = float(loss_rows[valid].sum() / nv)
    d = np.zeros_like(logits)
    d[:, :n_classes] = e / s
    d[np.arange(len(d)), lab] -= 1.0
    d[~valid] = 0.0
    d = r(d / nv)
    G = {}
    G["W5"] = acts[4].T @ d
    G["b5"] = d.sum(axis=0)
    dh = d @ Wb["W5"].T
    for k in range(4, 0, -1):
        dz = r(dh * gelu_grad(zs[k - 1]))
        G[f"W{k}"] = acts[k - 1].T @ dz
        G[f"b{k}"] = dz.sum(axis=0)
        dh = dz @ Wb[f"W{k}"].T
    g = np.zeros(params.size, dtype)
    for name, o, shape in layout:
        g[o:o + int(np.prod(shape))] = G[name].reshape(-1)
    return loss, g
