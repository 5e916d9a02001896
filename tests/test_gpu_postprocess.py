"""Device-side ensemble statistics (ensemble_mean / ensemble_percentile,
cpp/memilio/data/analyze_result.h:289-338) against the reference's definition
restated in numpy: the mean sums x / runs in run order; a percentile p is the
value at sorted index floor(runs * p). Same values, so the results are equal
exactly."""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("runs", [33, 64])
def test_ensemble_stats_match_reference_definition(runs):
    ctx = N.Context(0)
    graphs = W.ensemble(num_samples=runs, N=20, out_degree=4)
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    b.advance(6.0)
    p = np.array([0.05, 0.25, 0.5, 0.75, 0.95])
    mean, pct = b.ensemble_stats(p)
    x = np.stack(b.states())  # [runs, N, 10G]
    ref_mean = np.zeros_like(x[0])
    for r in range(runs):
        ref_mean += x[r] / runs
    np.testing.assert_array_equal(mean, ref_mean)
    srt = np.sort(x, axis=0)
    for q, pv in enumerate(p):
        np.testing.assert_array_equal(pct[q], srt[int(runs * pv)])
    b.close()
    ctx.close()
