"""Learned edge prior on the GPU: tensor-core forward/backward against the
CPU oracle, training, edge data, and the plain-FACO fallback."""
import numpy as np
import pytest

from oracle import mlp_oracle
from tests import _cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prior(engine_lib):
    from gplsaco_gb300 import prior
    return prior


def _data(prior, rng, E):
    x = np.zeros((E, 8), np.float32)
    x[:, :] = rng.random((E, 8), dtype=np.float32)
    x[:, 5] = (rng.random(E) < 0.2).astype(np.float32)
    bits = prior.to_bf16_bits(x)
    y = ((x[:, 0] < 0.3) ^ (x[:, 5] > 0.5)).astype(np.float32)
    return bits, prior.from_bf16_bits(bits).astype(np.float64), y


@pytest.mark.parametrize("E", [1, 15, 64, 1000, 4099, 65536])
def test_forward_matches_oracle(prior, E):
    """Probabilities from the tcgen05 forward pass against the oracle's, per
    row within 1/4 (the sigmoid's slope bound) of the logit bound: FP32
    summation over the logit's chain (64 terms of z, 8 steps of layer 2) on
    the shared BF16 operands, plus one layer-1 activation that rounds to the
    neighbouring BF16 value on one side only."""
    rng = np.random.default_rng(E)
    params = prior.init_params(seed=E)
    bits, x, _ = _data(prior, rng, E)
    got = prior.forward(params, bits)
    want = mlp_oracle.forward(params, x)["prob"]
    scale, flip = mlp_oracle.forward_bounds(params, x)
    bound = 0.25 * (72 * mlp_oracle.U32 * scale + flip)
    assert np.all(np.abs(got - want) <= bound)


@pytest.mark.parametrize("E", [16, 64, 777, 8192, 65536])
def test_gradient_matches_oracle(prior, E):
    """Gradients from the tcgen05 backward pass against the oracle's, entry by
    entry.  Both sides multiply the same BF16 operands; they differ by
    (a) FP32 against FP64 accumulation: at most the chain length times U32
    times S = sum_e |a_e b_e|, the chain being 8 products per 128-row tile,
    the tiles of one CTA, and the CTA partials added in order; (b) an operand
    whose FP32 and FP64 values round to neighbouring BF16 values: BF16_STEP
    times M = max_e |a_e b_e| each, two allowed per entry.  The loss: its
    own chain times U32 times the loss, plus the logit bound of every row."""
    import torch
    rng = np.random.default_rng(100 + E)
    params = prior.init_params(seed=E)
    bits, x, y = _data(prior, rng, E)
    grad, loss = prior.gradient(params, bits, y)
    want, want_loss = mlp_oracle.gradient(params, x, y)
    tiles = -(-E // 128)
    blocks = min(tiles, 2 * torch.cuda.get_device_properties(0).multi_processor_count)
    chain = 8 * -(-tiles // blocks) + blocks + 8
    S, M = mlp_oracle.gradient_bounds(params, x, y)
    bound = chain * mlp_oracle.U32 * S + 2 * mlp_oracle.BF16_STEP * M
    err = np.abs(grad.astype(np.float64) - want)
    assert np.all(err <= bound), int(np.argmax(err - bound))
    scale, flip = mlp_oracle.forward_bounds(params, x)
    assert abs(loss - want_loss) <= (chain + 160) * mlp_oracle.U32 * want_loss + np.sum(72 * mlp_oracle.U32 * scale + flip)


def test_training_reduces_loss(prior):
    rng = np.random.default_rng(7)
    bits, x, y = _data(prior, rng, 50000)
    params = prior.init_params(seed=1)
    trained, losses = prior.train(params, bits, y, epochs=8, batch=4096, lr=3e-3)
    assert losses[-1] < 0.5 * losses[0]
    acc = np.mean((prior.forward(trained, bits) > 0.5) == (y > 0.5))
    assert acc > 0.9
    # the gradient is reduced in a fixed order: training is reproducible bit for bit
    again, again_losses = prior.train(params, bits, y, epochs=8, batch=4096, lr=3e-3)
    assert np.array_equal(np.asarray(again).view(np.uint32), np.asarray(trained).view(np.uint32))
    assert np.array_equal(np.asarray(again_losses), np.asarray(losses))
    g1, l1 = prior.gradient(params, bits, y)
    g2, l2 = prior.gradient(params, bits, y)
    assert np.array_equal(np.asarray(g1).view(np.uint32), np.asarray(g2).view(np.uint32)) and l1 == l2


def test_edge_data_and_fallback(prior):
    import gplsaco_gb300 as g
    from oracle import oracle
    n, ants = 300, 8
    xy = _cases.uniform_instance(n, seed=12)
    settings = g.FixedFacoSettings(ants=ants, retention=0.9)
    keys = np.array([5, 5, 5], np.uint64)
    seeds = np.array([1, 2, 3], np.uint64)
    engine = g.FacoBatchEngine(n, 3, settings)
    engine.register_problem(5, xy.astype(np.float64))
    # plain reference result
    plain = engine.evaluate_faco_evaluations(keys, seeds, ants * 6, 8)
    # features/labels mid-run; prior with every colony disabled == plain FACO bit for bit
    engine.begin(keys, seeds, 8)
    engine.step(3)
    x, y = engine.edge_data()
    assert x.shape == (3 * n * 16, 8) and y.shape == (3 * n * 16,)
    xf = prior.from_bf16_bits(x)
    assert np.array_equal(xf[:, 5], y)                       # in-best-tour flag == label at the same state
    assert np.all((xf >= 0) & (xf <= 1))
    # x7: alpha-nearness over the mean nearest-neighbour length, clipped at 4, / 4
    rows = engine.problem_rows(5)
    alpha = oracle.alpha_nearness(xy, rows["primary"], rows["backup"], rows["ls"])
    mean_nn = np.float32(max(1.0, float(np.mean(oracle.euc2d_matrix(xy)[np.arange(n), rows["ls"][:, 0]]))))
    want7 = (np.minimum(alpha.astype(np.float32) / mean_nn, np.float32(4.0)) * np.float32(0.25)).astype(np.float32)
    want7 = prior.from_bf16_bits(prior.to_bf16_bits(np.tile(want7.reshape(-1), 3)))
    assert np.array_equal(xf[:, 7], want7)
    # x6: rank of i in j's candidate row / (k-1), 1 when absent (mutual nearness)
    primary = engine.problem_rows(5)["primary"].astype(np.int64)
    k = primary.shape[1]
    back = np.ones((n, k), np.float32)
    for i in range(n):
        for r in range(k):
            hit = np.nonzero(primary[primary[i, r]] == i)[0]
            if hit.size:
                back[i, r] = hit[0] / (k - 1)
    want6 = prior.from_bf16_bits(prior.to_bf16_bits(np.tile(back.reshape(-1), 3)))
    assert np.array_equal(xf[:, 6], want6)
    assert np.all(y.reshape(3, n, 16).sum(axis=2) <= 2)     # at most the two tour neighbours per node
    engine.prior_set(prior.init_params(seed=3), np.zeros(3, np.uint8))
    engine.step(3)
    res = engine.finish()
    assert [int(c) for c in res["costs"]] == [it["cost"] for it in plain["items"]]
    # enabled prior: valid tours, exact lengths
    engine.begin(keys, seeds, 8)
    engine.prior_set(prior.init_params(seed=3), np.ones(3, np.uint8), floor=0.05)
    for _ in range(3):
        engine.step(2)
        engine.prior_refresh()
    res = engine.finish()
    m = oracle.euc2d_matrix(xy)
    for c in range(3):
        t = np.asarray(res["tours"][c], np.int64)
        assert np.array_equal(np.sort(t), np.arange(n))
        assert int(np.sum(m[t, np.roll(t, -1)])) == int(res["costs"][c])
    engine.close()


def test_departures_prior(prior):
    """The departures-only prior: disabled on every colony it is plain FACO
    bit for bit; enabled (with and without departures) it gives valid
    tours with exact lengths; a non-bool flag is refused."""
    import gplsaco_gb300 as g
    from oracle import oracle
    n, ants, iterations = 400, 8, 12
    xy = _cases.uniform_instance(n, seed=21)
    settings = g.FixedFacoSettings(ants=ants, primary_width=20, retention=0.98)
    keys = np.array([7, 7], np.uint64)
    seeds = np.array([1, 2], np.uint64)
    engine = g.FacoBatchEngine(n, 2, settings)
    engine.register_problem(7, xy.astype(np.float64))
    plain = engine.evaluate_faco_evaluations(keys, seeds, ants * iterations, 8)
    params = prior.init_params(seed=4)
    engine.begin(keys, seeds, 8)
    engine.prior_set(params, np.zeros(2, np.uint8), 0.05, 2, departures=True)
    engine.step(iterations)
    res = engine.finish()
    assert [int(c) for c in res["costs"]] == [it["cost"] for it in plain["items"]]
    steps = {}
    for departures in (False, True):
        engine.begin(keys, seeds, 8)
        engine.prior_set(params, np.ones(2, np.uint8), 0.05, 2, departures=departures)
        engine.step(iterations)
        res = engine.finish()
        m = oracle.euc2d_matrix(xy)
        for c in range(2):
            t = np.asarray(res["tours"][c], np.int64)
            assert np.array_equal(np.sort(t), np.arange(n))
            assert int(np.sum(m[t, np.roll(t, -1)])) == int(res["costs"][c])
        steps[departures] = res["construction_steps"]
    with pytest.raises(ValueError):
        engine.begin(keys, seeds, 8)
        try:
            engine.prior_set(params, np.ones(2, np.uint8), 0.05, 2, departures=1)
        finally:
            engine.finish()
    engine.close()
    assert steps[True] > 0 and steps[False] > 0
    print("construction steps, prior / departures-only prior:", steps[False], steps[True])
