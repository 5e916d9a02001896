"""The two forms of the mixed solvers' exchange passes give identical results.

A graph whose departure snapshot records (and return-time rates) fit in
shared memory returns and departs in one CTA per graph, reading them from a
copy there; the other graphs run the node-list passes, which gather the same
records from the global tables. Both compute the same FP32 products and
TwoSum updates over each (node, age group)'s incident edges in the serial
order of MobilityEdge::apply_mobility
(memilio/mobility/metapopulation_mobility_instant.h:544-623), so states,
flows, commuter statistics and counters are bitwise equal between a batch
with every eligible graph staged (mgpu_solver_opts.staged_exchange = 2) and
one without (0); the default (1) stages when the per-graph CTAs fill the GPU.

Cases: the benchmark's 400-node, 6-group graph (commuter compartments S, E,
INS, ISy, R; one fraction per (edge, group)); every compartment mobile with
per-compartment coefficients; the commuter compartments with per-compartment
coefficients; staged, small and edge-damped graphs in one batch; a stressed
graph whose returns take the exact underflow path; flow recording and
commuter statistics; the FP64-control variant. And two graphs that pass the
same coefficient array with different edges run as they do alone (the
in-edge-ordered copy of the coefficients is shared only with the same edges).
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED = [N.PRECISION_MIXED, N.PRECISION_MIXED_FP64_CONTROL]


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def run(ctx, graphs, precision, staged, days, horizons=None, flows=False, stats_graph=None):
    # staged: every eligible graph staged (2), else the node-list passes only (0)
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=precision, staged_exchange=2 if staged else 0))
    if flows:
        b.set_flow_recording(True)
    if stats_graph is not None:
        g = graphs[stats_graph]
        sets = [list(range(0, 10 * g.num_groups, 10)), list(range(3, 10 * g.num_groups, 10))]
        b.set_commuter_stats(stats_graph, sets, 64)
    if horizons is None:
        b.advance(days)
    else:
        b.advance(0.0, horizons)
    out = {"states": [s.copy() for s in b.states()], "stats": b.stats()}
    if flows:
        out["flows"] = [f.copy() for f in b.flows()]
    if stats_graph is not None:
        out["commuters"] = b.commuter_stats(stats_graph)
    b.close()
    return out


def assert_same(a, b):
    for x, y in zip(a["states"], b["states"]):
        np.testing.assert_array_equal(x, y)
    for k in ("accepted_steps", "rejected_steps", "underflow_fixes", "sequential_exchanges", "scan_items"):
        assert a["stats"][k] == b["stats"][k], k
    if "flows" in a:
        for x, y in zip(a["flows"], b["flows"]):
            np.testing.assert_array_equal(x, y)
    if "commuters" in a:
        for x, y in zip(a["commuters"], b["commuters"]):
            np.testing.assert_array_equal(np.asarray(x), np.asarray(y))


def all_mobile(g0, seed):
    # a coefficient on every compartment, different per compartment (no single
    # fraction per (edge, group)): the general compartment mask and records
    rng = np.random.default_rng(seed)
    coeff = g0.edge_coeff_baseline * rng.uniform(0.5, 1.5, g0.edge_coeff_baseline.shape)
    coeff[coeff == 0.0] = rng.uniform(0.001, 0.02, int((coeff == 0.0).sum()))
    return L.GraphArrays(g0.num_groups, g0.params, g0.contact_baseline, g0.contact_minimum, g0.damping_times,
                         g0.damping_values, g0.init_state, g0.edge_src, g0.edge_dst, coeff)


def edge_damped(g0):
    # commuting halved from day 3 (edge dampings: the FP64-coefficient passes)
    E = g0.edge_src.shape[0]
    n = 10 * g0.num_groups
    times = np.broadcast_to(np.array([L.DBL_LOWEST, 3.0, L.DBL_MAX]), (E, 3)).copy()
    vals = np.zeros((E, 3, n))
    vals[:, 1:] = 0.5
    return L.GraphArrays(g0.num_groups, g0.params, g0.contact_baseline, g0.contact_minimum, g0.damping_times,
                         g0.damping_values, g0.init_state, g0.edge_src, g0.edge_dst, g0.edge_coeff_baseline,
                         np.zeros_like(g0.edge_coeff_baseline), times, vals)


@pytest.mark.parametrize("precision", MIXED)
def test_benchmark_graph(ctx, precision):
    ens = W.ensemble(num_samples=3, N=400, G=6, out_degree=30)
    a = run(ctx, ens, precision, True, 12.0)
    b = run(ctx, ens, precision, False, 12.0)
    assert_same(a, b)


@pytest.mark.parametrize("precision", MIXED)
def test_all_compartments_mobile(ctx, precision):
    g = all_mobile(W.mobility_graph(seed=71, N=90, G=6, out_degree=12), 72)
    assert_same(run(ctx, [g], precision, True, 8.0), run(ctx, [g], precision, False, 8.0))


def test_staged_small_and_damped_graphs_in_one_batch(ctx):
    graphs = [W.mobility_graph(seed=81, N=400, G=6, out_degree=30),   # staged
              W.mobility_graph(seed=82, N=20, G=3, out_degree=4),     # too few items: node lists
              W.mobility_graph(seed=83, N=200, G=2, out_degree=10),   # staged, another group count
              edge_damped(W.mobility_graph(seed=84, N=60, G=6, out_degree=8)),  # edge dampings
              W.single_node(seed=85, G=4, count=3)]                   # no edges
    horizons = np.array([9.0, 6.5, 8.0, 7.5, 3.0])
    a = run(ctx, graphs, N.PRECISION_MIXED, True, 0.0, horizons)
    b = run(ctx, graphs, N.PRECISION_MIXED, False, 0.0, horizons)
    assert_same(a, b)
    # per pass, the staged batch launched one per-graph kernel (the 400- and
    # 200-node graphs) and one node list (3 groups) where the other launched
    # three node lists (6, 3 and 2 groups)
    assert a["stats"]["kernel_launches"] < b["stats"]["kernel_launches"]


def test_underflow_fixes(ctx):
    g = W.mobility_graph(seed=1, N=120, G=6, out_degree=30, stress=True)
    a = run(ctx, [g], N.PRECISION_MIXED, True, 30.0)
    b = run(ctx, [g], N.PRECISION_MIXED, False, 30.0)
    assert_same(a, b)
    assert a["stats"]["underflow_fixes"] > 0


def test_flows_and_commuter_statistics(ctx):
    graphs = [W.mobility_graph(seed=91, N=100, G=4, out_degree=10),
              W.mobility_graph(seed=92, N=50, G=6, out_degree=6)]
    a = run(ctx, graphs, N.PRECISION_MIXED, True, 6.0, flows=True, stats_graph=0)
    b = run(ctx, graphs, N.PRECISION_MIXED, False, 6.0, flows=True, stats_graph=0)
    assert_same(a, b)


def test_commuter_mask_with_per_compartment_coefficients(ctx):
    # S, E, INS, ISy, R mobile with a different fraction per compartment: the
    # commuter mask without one value per (edge, group)
    g0 = W.mobility_graph(seed=95, N=100, G=6, out_degree=10)
    rng = np.random.default_rng(96)
    coeff = g0.edge_coeff_baseline * rng.uniform(0.5, 1.5, g0.edge_coeff_baseline.shape)
    g = L.GraphArrays(g0.num_groups, g0.params, g0.contact_baseline, g0.contact_minimum, g0.damping_times,
                      g0.damping_values, g0.init_state, g0.edge_src, g0.edge_dst, coeff)
    assert_same(run(ctx, [g], N.PRECISION_MIXED, True, 8.0), run(ctx, [g], N.PRECISION_MIXED, False, 8.0))


def test_shared_coefficients_with_other_edges(ctx):
    # two graphs pass the same coefficient array with different edges: each keeps
    # its own in-edge order of the coefficients, so each runs as it does alone
    a = W.mobility_graph(seed=97, N=60, G=6, out_degree=8)
    rng = np.random.default_rng(98)
    dst = a.edge_dst.copy()
    for v in range(a.num_nodes):  # other targets, the same number of out-edges per node
        sel = np.nonzero(a.edge_src == v)[0]
        pool = np.setdiff1d(np.arange(a.num_nodes), [v])
        dst[sel] = np.sort(rng.choice(pool, size=sel.size, replace=False))
    b = L.GraphArrays(a.num_groups, a.params, a.contact_baseline, a.contact_minimum, a.damping_times,
                      a.damping_values, a.init_state, a.edge_src, dst, a.edge_coeff_baseline)
    both = run(ctx, [a, b], N.PRECISION_MIXED, True, 6.0)
    alone_a = run(ctx, [a], N.PRECISION_MIXED, True, 6.0)
    alone_b = run(ctx, [b], N.PRECISION_MIXED, True, 6.0)
    np.testing.assert_array_equal(both["states"][0], alone_a["states"][0])
    np.testing.assert_array_equal(both["states"][1], alone_b["states"][0])
