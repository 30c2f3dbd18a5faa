"""CPU restatement of the edge-prior MLP (forward and backward) with the
engine's BF16 roundings.  TEST INFRASTRUCTURE ONLY (gradient checks).

The GPU rounds to BF16 exactly these operands of its tensor-core products:
the inputs x, the weights w1 and w2, the layer-1 activations h1 (input of
layer 2 and of dW2), the layer-2 activations h2 and the output gradient dz
(the two factors of dw3), the layer-2 gradient dh2 (input of the product
with w2, of dW2 and of db2) and the layer-1 gradient dh1 (input of dW1 and
db1).  The bias gradients db1, db2 are products with a column of ones.
Everything else is FP32 (here FP64).
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
    dh1b = bf16(np.where(f["h1"] > 0, dh2b @ bf16(v["w2"]), 0.0))
    g = dict(w3=bf16(f["h2"]).T @ bf16(dz), b3=np.array([dz.sum()]), b2=dh2b.sum(0), w2=dh2b.T @ bf16(f["h1"]),
             b1=dh1b.sum(0), w1=dh1b.T @ x)
    out = np.zeros(p.size, np.float64)
    o = 0
    for name in ("w1", "b1", "w2", "b2", "w3", "b3"):
        size = g[name].size
        out[o:o + size] = g[name].reshape(-1)
        o += size
    return out, loss


U32 = 2.0 ** -24         # FP32 unit roundoff
BF16_STEP = 2.0 ** -7    # largest spacing of neighbouring BF16 values relative to their size


def forward_bounds(p: np.ndarray, x: np.ndarray):
    """Per-row magnitudes that bound the difference between the GPU's logit
    (FP32 accumulation) and forward()'s (FP64 accumulation), both from the
    same BF16 operand bits:
      scale[e] = |b3| + sum_c |w3_c| (|h2_c| + |b2_c| + sum_i |bf16(h1_i) w2_ci|)
                 -- the summands of z and of each layer-2 pre-activation it
                 uses; FP32 summation error is at most the chain length
                 (64 terms of z plus the layer-2 steps) times U32 times it;
      flip[e]  = BF16_STEP * max_i |h1_i| * sum_c |w3_c w2_ci|  -- the change
                 of z when one layer-1 activation rounds to the neighbouring
                 BF16 value (its FP32 and FP64 values straddle a rounding
                 midpoint).
    """
    v = unpack(p)
    f = forward(p, x)
    w2b = np.abs(bf16(v["w2"]))
    w3 = np.abs(v["w3"])
    h1b = np.abs(bf16(f["h1"]))
    s2 = h1b @ w2b.T + np.abs(v["b2"]) + f["h2"]
    scale = np.abs(v["b3"][0]) + s2 @ w3
    reach = w3 @ w2b                           # sum_c |w3_c w2_ci| per input i
    flip = BF16_STEP * np.max(h1b * reach[None, :], axis=1)
    return scale, flip


def gradient_bounds(p: np.ndarray, x: np.ndarray, y: np.ndarray, chunk: int = 512):
    """Per-entry magnitudes of the gradient sums: for an entry sum_e a_e b_e of
    BF16 operands, S = sum_e |a_e b_e| (the FP32 accumulation error is a
    multiple of U32 * S) and M = max_e |a_e b_e| (one operand that rounds to
    the neighbouring BF16 value moves the entry by at most BF16_STEP * M).
    Returns (S, M) as parameter-shaped vectors."""
    v = unpack(p)
    f = forward(p, x)
    E = x.shape[0]
    dz = (f["prob"] - y) / E
    dh2b = bf16(np.where(f["h2"] > 0, dz[:, None] * v["w3"][None, :], 0.0))
    dh1b = bf16(np.where(f["h1"] > 0, dh2b @ bf16(v["w2"]), 0.0))
    h1b, h2b, dzb = bf16(f["h1"]), bf16(f["h2"]), bf16(dz)
    ones = np.ones((E, 1))
    pairs = dict(w1=(dh1b, x), b1=(dh1b, ones), w2=(dh2b, h1b), b2=(dh2b, ones), w3=(h2b, dzb[:, None]),
                 b3=(dz[:, None], ones))
    S, M = {}, {}
    for name, (a, b) in pairs.items():
        a, b = np.abs(a), np.abs(b)
        S[name] = a.T @ b
        m = np.zeros((a.shape[1], b.shape[1]))
        for s in range(0, E, chunk):
            m = np.maximum(m, np.max(a[s:s + chunk, :, None] * b[s:s + chunk, None, :], axis=0))
        M[name] = m
    shape = dict(w1=(HIDDEN, IN), b1=(HIDDEN,), w2=(HIDDEN, HIDDEN), b2=(HIDDEN,), w3=(HIDDEN,), b3=(1,))
    outS, outM = np.zeros(p.size), np.zeros(p.size)
    o = 0
    for name in ("w1", "b1", "w2", "b2", "w3", "b3"):
        size = int(np.prod(shape[name]))
        outS[o:o + size] = S[name].reshape(-1)[:size] if name != "w3" else S[name][:, 0]
        outM[o:o + size] = M[name].reshape(-1)[:size] if name != "w3" else M[name][:, 0]
        o += size
    return outS, outM
