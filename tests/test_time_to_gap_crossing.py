"""The time-to-gap crossing on the host: the first iteration whose mean gap is
at or below the target comes from the per-iteration trace (not from the
chunk readings), and its time is interpolated between the clock readings of
the chunk it falls in; without a trace, the first chunk reading at or below
the target."""
import numpy as np

from gplsaco_gb300 import experiments as ex


def _rows(readings):
    return [(it, sec, gap, None) for it, sec, gap in readings]


def test_per_iteration_gaps_are_means_over_instances():
    refs = np.array([100.0, 200.0])
    best = np.array([[110, 220], [105, 200], [100, 200]])
    np.testing.assert_allclose(ex.per_iteration_gaps(best, refs), [0.1, 0.025, 0.0])


def test_crossing_is_exact_and_interpolated():
    # chunk readings every 16 iterations; the trace crosses 1 % after 21
    readings = [(0, 0.0, 0.05), (16, 1.6, 0.02), (32, 3.6, 0.005)]
    gaps = np.linspace(0.05, 0.0, 32)
    gaps[:20] = np.maximum(gaps[:20], 0.011)
    gaps[20] = 0.0099                                   # iteration 21
    rows = ex.Rows(_rows(readings), gaps)
    seconds, iterations = ex.first_time_below(rows, 0.01)
    assert iterations == 21
    assert abs(seconds - (1.6 + 2.0 * 5 / 16)) < 1e-12   # inside the chunk (16, 32]
    seconds, iterations = ex.first_time_below(rows, 0.01, extra_seconds=0.5)
    assert iterations == 21 and abs(seconds - (2.225 + 0.5)) < 1e-12


def test_crossing_at_the_start_and_never():
    rows = ex.Rows(_rows([(0, 0.0, 0.008), (16, 1.0, 0.007)]), np.full(16, 0.007))
    assert ex.first_time_below(rows, 0.01) == (0.0, 0)
    rows = ex.Rows(_rows([(0, 0.0, 0.05), (16, 1.0, 0.04)]), np.full(16, 0.04))
    assert ex.first_time_below(rows, 0.01) == (None, None)


def test_without_a_trace_the_chunk_reading_decides():
    rows = _rows([(0, 0.0, 0.05), (10, 1.0, 0.02), (20, 2.0, 0.009)])
    assert ex.first_time_below(rows, 0.01) == (2.0, 20)
