"""Flow results of the batched solvers (mgpu_batch_set_flow_recording /
mgpu_batch_get_flows): FlowSimulation::get_flows() of every node of a graph
(cpp/memilio/compartments/flow_simulation.h:36-121; a graph of FlowSimulation
nodes, cpp/tests/test_graph_simulation.cpp:276-340).

  * Isolated nodes: the population change equals the recorded flows scattered
    to their compartments (FlowModel::get_derivatives of the flows,
    flow_simulation_base.h:90-103), to 1e-10 of the age group's population in
    FP64 and 1e-6 in the mixed precision; and the flows agree with the
    oracle's FlowSimulation (whose integrator controls the error of the flows,
    not of the compartments) within 1e-4 relative to the flow, floor 1e-6 of
    the age group's population: the integrator's tolerance, not rounding.
  * A graph with mobility: flows only grow, the FP64 and mixed solvers agree
    to 1e-5 (floor 1e-6), a graph's flows are the same alone and in a batch,
    recording does not change the states, and a reset starts from zero.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SRC = [L.S, L.E, L.INS, L.INS, L.INSC, L.INSC, L.ISY, L.ISY, L.ISYC, L.ISYC, L.ISEV, L.ISEV, L.ISEV, L.ICRI, L.ICRI]
DST = [L.E, L.INS, L.ISY, L.R, L.ISYC, L.R, L.ISEV, L.R, L.ISEV, L.R, L.ICRI, L.R, L.D, L.D, L.R]


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def scatter(F, G):
    """get_derivatives of accumulated flows [.., 15 G]: the population change [.., 10 G]."""
    F = np.asarray(F).reshape(-1, G, 15)
    d = np.zeros((F.shape[0], G, 10))
    for k in range(15):
        d[:, :, SRC[k]] -= F[:, :, k]
        d[:, :, DST[k]] += F[:, :, k]
    return d.reshape(-1, 10 * G)


def run(ctx, graphs, precision, days, record=True):
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=precision))
    if record:
        b.set_flow_recording(True)
    b.advance(days)
    out = (b.states(), b.flows() if record else None)
    b.close()
    return out


@pytest.mark.parametrize("precision,tol", [(N.PRECISION_FP64, 1e-10), (N.PRECISION_MIXED, 1e-6)])
def test_isolated_nodes_flows(ctx, precision, tol):
    g = W.single_node(seed=91, G=6, count=16, stress=True)
    (state,), (F,) = run(ctx, [g], precision, 30.0)
    Ng = g.init_state.reshape(-1, 6, 10).sum(axis=2).repeat(10, axis=1)
    assert np.max(np.abs(state - g.init_state - scatter(F, 6)) / Ng) <= tol
    assert F.min() >= 0.0
    # the reference's FlowSimulation of the same nodes
    worst = 0.0
    for v in range(0, 16, 3):
        _, flows, _, _ = O.simulate_flows(g, v, 0.0, 30.0, 0.1)
        ref = flows[-1].reshape(6, 15)
        n_g = g.init_state[v].reshape(6, 10).sum(axis=1, keepdims=True)
        worst = max(worst, float(np.max(np.abs(F[v].reshape(6, 15) - ref) / np.maximum(ref, 1e-6 * n_g))))
    print("flows vs FlowSimulation, max relative difference", worst)
    assert worst <= 1e-4


def test_graph_flows(ctx):
    g = W.mobility_graph(seed=92, N=40, G=4, out_degree=8)
    other = W.mobility_graph(seed=93, N=12, G=2, out_degree=3)
    b = N.Batch(ctx, [g, other], 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    b.set_flow_recording(True)
    prev = np.zeros((g.num_nodes, 15 * g.num_groups))
    for t in np.arange(1.0, 11.0, 1.0):
        b.advance(float(t))
        F = b.flows()[0]
        assert (F >= prev).all()
        prev = F
    states = b.state_flat()
    b.reset(0.0)
    assert not b.flows()[0].any()
    b.close()
    # alone, and without recording
    (alone,), (F_alone,) = run(ctx, [g], N.PRECISION_MIXED, 10.0)
    np.testing.assert_array_equal(F_alone, prev)
    (plain_state, _), _ = run(ctx, [g, other], N.PRECISION_MIXED, 10.0, record=False)
    np.testing.assert_array_equal(states[:g.num_nodes * g.n], plain_state.ravel())
    # FP64 against mixed
    (_,), (F64,) = run(ctx, [g], N.PRECISION_FP64, 10.0)
    n_g = g.init_state.reshape(-1, 4, 10).sum(axis=2)
    den = np.maximum(F64.reshape(-1, 4, 15), 1e-6 * n_g[:, :, None])
    assert np.max(np.abs(prev.reshape(-1, 4, 15) - F64.reshape(-1, 4, 15)) / den) <= 1e-5
    # the plain per-graph drop-in does not record flows
    pb = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64_PLAIN))
    with pytest.raises(N.MgpuError) as e:
        pb.set_flow_recording(True)
    assert e.value.code == 104
    pb.close()
