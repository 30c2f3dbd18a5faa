"""CPU restatement of the edge-prior MLP (forward and backward) with the
engine's BF16 roundings.  TEST INFRASTRUCTURE ONLY (gradient checks).

The GPU rounds to BF16 exactly these operands of its tensor-core products:
the inputs x, the weights w1 and w2, the layer-1 activations (input of layer
2), the layer-2 gradient dh2 (input of the product with w2 and of dW2), the
layer-1 gradient dh1 (input of dW1).  Everything else is FP32 (here FP64).
"""
from __future__ import annotations

import numpy as np

HIDDEN, IN = 64, 8


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to BF16 (nearest even) and back to float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.view(np.float32).astype(np.float64)


def unpack(p: np.ndarray) -> dict:
    o, out = 0, {}
    for name, shape in (("w1", (HIDDEN, IN)), ("b1", (HIDDEN,)), ("w2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
                        ("w3", (HIDDEN,)), ("b3", (1,))):
        size = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + size], np.float64).reshape(shape)
        o += size
    return out


def forward(p: np.ndarray, x: np.ndarray):
    """x: [E, 8] float values (already BF16-representable)."""
    v = unpack(p)
    w1 = bf16(v["w1"])
    w2 = bf16(v["w2"])
    z1 = x @ w1.T + v["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = bf16(h1) @ w2.T + v["b2"]
    h2 = np.maximum(z2, 0.0)
    z = h2 @ v["w3"] + v["b3"][0]
    return dict(h1=h1, h2=h2, z=z, prob=1.0 / (1.0 + np.exp(-z)))


def gradient(p: np.ndarray, x: np.ndarray, y: np.ndarray):
    """Gradient of the mean binary cross-entropy; returns (grad vector, loss sum)."""
    v = unpack(p)
    f = forward(p, x)
    E = x.shape[0]
    dz = (f["prob"] - y) / E
    loss = np.sum(np.maximum(f["z"], 0) - f["z"] * y + np.log1p(np.exp(-np.abs(f["z"]))))
    dh2 = np.where(f["h2"] > 0, dz[:, None] * v["w3"][None, :], 0.0)
    dh2b = bf16(dh2)
    dh1 = np.where(f["h1"] > 0, dh2b @ bf16(v["w2"]), 0.0)
    g = dict(w3=f["h2"].T @ dz, b3=np.array([dz.sum()]), b2=dh2.sum(0), w2=dh2b.T @ bf16(f["h1"]),
             b1=dh1.sum(0), w1=bf16(dh1).T @ x)
    out = np.zeros(p.size, np.float64)
    o = 0
    for name in ("w1", "b1", "w2", "b2", "w3", "b3"):
        size = g[name].size
        out[o:o + size] = g[name].reshape(-1)
        o += size
    return out, loss
