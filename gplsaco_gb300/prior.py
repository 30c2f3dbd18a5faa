"""Learned edge prior: training data from the engine's own runs, training on
the GPU with the project's forward/backward kernels, and the per-instance
fallback to plain FACO.

Parameters are one FP32 vector (layout in include/faco_gb300.h,
faco_mlp_param_count values).  Edge rows are [E, 8] BF16 bit patterns
(uint16), labels [E] float32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

HIDDEN, IN = 64, 8


def param_count() -> int:
    return int(_lib.load().faco_mlp_param_count())


def unpack(params: np.ndarray) -> dict:
    """Views of the parameter vector: w1 [64,8], b1, w2 [64,64], b2, w3, b3."""
    o = 0
    out = {}
    for name, shape in (("w1", (HIDDEN, IN)), ("b1", (HIDDEN,)), ("w2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
                        ("w3", (HIDDEN,)), ("b3", (1,))):
        size = int(np.prod(shape))
        out[name] = params[o:o + size].reshape(shape)
        o += size
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation."""
    rng = np.random.default_rng(seed)
    p = np.zeros(param_count(), np.float32)
    v = unpack(p)
    v["w1"][:] = rng.normal(0, np.sqrt(2 / IN), (HIDDEN, IN))
    v["w2"][:] = rng.normal(0, np.sqrt(2 / HIDDEN), (HIDDEN, HIDDEN))
    v["w3"][:] = rng.normal(0, np.sqrt(1 / HIDDEN), HIDDEN)
    v["b3"][:] = -2.0   # most candidate edges are not in the best tour
    return p


def to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> BF16 bit patterns, round to nearest even."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounded = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return rounded.astype(np.uint16)


def from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


def forward(params: np.ndarray, x_bits: np.ndarray) -> np.ndarray:
    params = np.ascontiguousarray(params, np.float32)
    x_bits = np.ascontiguousarray(x_bits, np.uint16).reshape(-1, IN)
    prob = np.zeros(x_bits.shape[0], np.float32)
    _lib.check(_lib.load().faco_mlp_forward(params.ctypes.data, x_bits.ctypes.data, x_bits.shape[0],
                                            prob.ctypes.data))
    return prob


def gradient(params: np.ndarray, x_bits: np.ndarray, y: np.ndarray):
    params = np.ascontiguousarray(params, np.float32)
    x_bits = np.ascontiguousarray(x_bits, np.uint16).reshape(-1, IN)
    y = np.ascontiguousarray(y, np.float32)
    grad = np.zeros_like(params)
    loss = np.zeros(1, np.float32)
    _lib.check(_lib.load().faco_mlp_gradient(params.ctypes.data, x_bits.ctypes.data, y.ctypes.data,
                                             x_bits.shape[0], grad.ctypes.data, loss.ctypes.data))
    return grad, float(loss[0])


def train(params: np.ndarray, x_bits: np.ndarray, y: np.ndarray, *, epochs: int = 10, batch: int = 8192,
          lr: float = 2e-3, seed: int = 0):
    """Adam on the GPU; rows are shuffled once on the host (seeded)."""
    params = np.array(params, np.float32, copy=True)
    x_bits = np.ascontiguousarray(x_bits, np.uint16).reshape(-1, IN)
    y = np.ascontiguousarray(y, np.float32)
    order = np.random.default_rng(seed).permutation(y.size)
    xs, ys = np.ascontiguousarray(x_bits[order]), np.ascontiguousarray(y[order])
    losses = np.zeros(epochs, np.float32)
    _lib.check(_lib.load().faco_mlp_train(params.ctypes.data, xs.ctypes.data, ys.ctypes.data, ys.size, epochs,
                                          batch, lr, losses.ctypes.data))
    return params, losses


def _profile_main(argv=None) -> None:
    """A short, self-contained run of the MLP kernels for profiling:
    `python -m gplsaco_gb300.prior --rows R --epochs E --forward-rows F`
    trains on R synthetic rows (features uniform in [0, 1], labels from a
    fixed rule) and runs one forward pass over F rows."""
    import argparse
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--rows", type=int, default=1 << 20)
    ap.add_argument("--epochs", type=int, default=1)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--forward-rows", type=int, default=1 << 22)
    args = ap.parse_args(argv)
    rng = np.random.default_rng(7)
    x = rng.random((args.rows, IN), dtype=np.float32)
    x[:, 6:] = 0.0
    y = ((x[:, 0] < 0.2) | (x[:, 5] > 0.8)).astype(np.float32)
    xb = to_bf16_bits(x)
    t = time.perf_counter()
    params, losses = train(init_params(1), xb, y, epochs=args.epochs, batch=args.batch)
    print(f"train {args.rows} rows x {args.epochs} epochs: {time.perf_counter() - t:.3f} s, loss {losses.tolist()}")
    xf = to_bf16_bits(rng.random((args.forward_rows, IN), dtype=np.float32) * np.array([1, 1, 1, 1, 1, 1, 0, 0],
                                                                                       np.float32))
    t = time.perf_counter()
    p = forward(params, xf)
    print(f"forward {args.forward_rows} rows: {time.perf_counter() - t:.3f} s, mean p {float(p.mean()):.4f}")


if __name__ == "__main__":
    _profile_main()
