"""What the trained edge prior gains over plain FACO.

The network is trained on the GPU by the project's own forward/backward
kernels, on labels from runs the engine itself produced (edges of each
colony's best tour after a plain run of a training pool).  Then plain FACO
and prior-reweighted FACO run the same held-out instances (disjoint seeds)
from the same initial tours with the same seeds, ants and MNE target, and
the mean gap to a long plain run's best is compared iteration by iteration.
The prior must reach the target gap in fewer iterations and stay ahead at
every checkpoint after the first batches.  Everything here is deterministic
(bit-exact engine, fixed-order gradient reduction), so the numbers printed
are the ones the assertions see."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_prior_reaches_the_gap_in_fewer_iterations(engine_lib):
    from gplsaco_gb300 import experiments as ex
    cfg = ex.GapConfig(train_pool=16, train_iterations=200, epochs=6, iterations=200, reference_iterations=800,
                       chunk=10)
    x, y = ex.collect_training_data(cfg)
    assert 0.05 < float(np.mean(y)) < 0.15          # about two tour edges per 20 candidates
    params, losses = ex.geometry_model(x, y, cfg)
    assert losses[-1] < losses[0]
    # held out: instance seeds 600-607, disjoint from the training pool (500-515)
    xys = [ex._xy("uniform" if i % 2 == 0 else "clustered", 800, 600 + i) for i in range(8)]
    refs = ex.reference_lengths(cfg, xys)
    plain, _, plain_work = ex.gap_run(cfg, xys, refs, None, mne=8)
    prior, _, prior_work = ex.gap_run(cfg, xys, refs, params, None, floor=0.05, gamma=2, refresh=0, mne=8)
    target = 0.01
    _, it_plain = ex.first_time_below(plain, target)
    _, it_prior = ex.first_time_below(prior, target)
    gaps = {r[0]: (round(r[2], 5), round(p[2], 5)) for r, p in zip(plain, prior)}
    print(f"iterations to a {target:.1%} mean gap: plain {it_plain}, prior {it_prior}; "
          f"mean gap (plain, prior) by iteration {gaps}; work per ant-iteration plain {plain_work}, "
          f"prior {prior_work}")
    assert it_prior is not None and it_plain is not None
    assert it_prior < it_plain
    for it, (gp, gq) in gaps.items():
        if it >= 20:
            assert gq < gp, (it, gp, gq)
