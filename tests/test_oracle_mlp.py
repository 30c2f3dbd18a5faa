"""The edge-prior MLP oracle: analytic gradient vs central differences (with
the BF16 roundings switched off, in float64)."""
import numpy as np

from oracle import mlp_oracle


def test_oracle_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(mlp_oracle, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.default_rng(0)
    size = 64 * 8 + 64 + 64 * 64 + 64 + 64 + 1 + 3
    p = rng.normal(0, 0.3, size)
    p[:64 * 8].reshape(64, 8)[:, 6:] = 0.0
    x = rng.random((40, 8))
    y = (rng.random(40) < 0.3).astype(np.float64)
    g, _ = mlp_oracle.gradient(p, x, y)

    def loss(q):
        z = mlp_oracle.forward(q, x)["z"]
        return np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))

    idx = np.concatenate([rng.choice(64 * 6, 20, replace=False),              # w1 (used columns)
                          64 * 8 + rng.choice(64, 5, replace=False),          # b1
                          64 * 8 + 64 + rng.choice(4096, 30, replace=False),  # w2
                          64 * 8 + 64 + 4096 + rng.choice(64 * 2 + 1, 20, replace=False)])
    idx = np.array([i if i >= 64 * 8 or (i % 8) < 6 else i - 2 for i in idx])
    for i in idx:
        e = np.zeros(size); e[i] = 1e-6
        fd = (loss(p + e) - loss(p - e)) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
