"""Commuter statistics on the device against the oracle.

MobilityEdge::add_mobility_result_time_point
(cpp/memilio/mobility/metapopulation_mobility_instant.h:423-447): at every
departure and every return (after the underflow fix) of an edge, the sums of
the travelers over the save-index sets (here INS + INSC and ISy + ISyC of all
age groups, as cpp/examples/ode_secir_graph.cpp builds them) and their total.
The oracle's recording is pinned to the reference's own test values in
tests/test_oracle_graph.py.

Tolerances: the FP64 solver 1e-10 relative (floor 1e-9 of the edge's total);
the mixed solver 1e-5 relative (floor 1e-6 of the edge's total): the FP32
exchange computes the travelers as FP32 products.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {N.PRECISION_FP64: (1e-10, 1e-9), N.PRECISION_MIXED: (1e-5, 1e-6)}


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def save_sets(G):
    return [[gr * 10 + c for gr in range(G) for c in (L.INS, L.INSC)],
            [gr * 10 + c for gr in range(G) for c in (L.ISY, L.ISYC)]]


@pytest.fixture(scope="module")
def stressed():
    # finite test-and-trace and ICU capacities: the returns need underflow fixes
    g = W.mobility_graph(seed=1, N=120, out_degree=30, stress=True)
    fin, counts, times, values, st = O.graph_run_commuters(g, 0.0, 30.0, save_sets(6), capacity=64)
    assert st["underflow_fixes"] > 0
    return g, fin, counts, times, values


@pytest.mark.parametrize("precision", [N.PRECISION_FP64, N.PRECISION_MIXED])
def test_commuter_stats_match_oracle(ctx, stressed, precision):
    g, fin, counts, times, values = stressed
    other = W.mobility_graph(seed=5, N=20, G=3, out_degree=4)  # in the batch, recording nothing
    b = N.Batch(ctx, [other, g], 0.0, N.solver_opts(precision=precision))
    b.set_commuter_stats(1, save_sets(6), 64)
    for t in (10.0, 20.5, 30.0):  # several advances append to the same series
        b.advance(t)
    c, tt, v = b.commuter_stats(1)
    np.testing.assert_array_equal(c, counts)
    assert (c == 60).all()
    np.testing.assert_allclose(tt[:, :60], times[:, :60], rtol=0, atol=1e-12)
    rtol, floor = TOL[precision]
    den = np.maximum(np.abs(values[:, :60]), floor * values[:, :60, -1:])
    err = np.abs(v[:, :60] - values[:, :60]) / den
    assert err.max() <= rtol, float(err.max())
    # recording leaves the simulation unchanged
    plain = N.Batch(ctx, [other, g], 0.0, N.solver_opts(precision=precision))
    plain.advance(30.0)
    np.testing.assert_array_equal(plain.state_flat(), b.state_flat())
    # a restart starts the series again; switching off stops recording
    b.reset(0.0)
    b.advance(1.0)
    assert (b.commuter_stats(1)[0] == 2).all()
    b.set_commuter_stats(1, [], 0)
    with pytest.raises(N.MgpuError):
        b.commuter_stats(1)
    b.close()
    plain.close()


def test_commuter_stats_capacity_and_arguments(ctx):
    g = W.mobility_graph(seed=7, N=6, G=2, out_degree=2)
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    with pytest.raises(N.MgpuError) as e:
        b.set_commuter_stats(0, [[0, 25]], 8)  # index outside 10 G
    assert e.value.code == 2
    b.set_commuter_stats(0, save_sets(2), 3)
    b.advance(2.0)  # four exchanges, three kept
    with pytest.raises(N.MgpuError) as e:
        b.commuter_stats(0)
    assert e.value.code == 2
    b.close()
    plain = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64_PLAIN))
    with pytest.raises(N.MgpuError) as e:
        plain.set_commuter_stats(0, save_sets(2), 8)
    assert e.value.code == 104
    plain.close()
