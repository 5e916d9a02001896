"""Oracle graph simulation: the reference's mobility and graph invariants.

Mirrors cpp/tests/test_mobility.cpp (edgeApplyMobility population sums,
compareNoMobilityWithSingleIntegration) and the conservation tests of
cpp/tests/test_odesecir.cpp:126-181."""
import numpy as np

from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W
from oracle import oracle as O
from tests.golden.scenarios import reference_test_model


def two_node_graph(coeff=0.1):
    m = reference_test_model(1, 0.25)
    P = np.repeat(m.params, 2, axis=0)
    # risk 1 as in test_mobility.cpp:168, so every compartment moves by exactly its coefficient
    P[:, L.group_param_index(L.G_RISK_FROM_SYMPTOMATIC, 0, 1)] = 1.0
    P[:, L.group_param_index(L.G_MAX_RISK_FROM_SYMPTOMATIC, 0, 1)] = 1.0
    y = np.repeat(m.init_state, 2, axis=0)
    y[:, :] = [990, 0, 0, 0, 10, 0, 0, 0, 0, 0]
    return L.GraphArrays(1, P, np.repeat(m.contact_baseline, 2, 0), np.repeat(m.contact_minimum, 2, 0),
                         np.repeat(m.damping_times, 2, 0), np.repeat(m.damping_values, 2, 0), y,
                         np.array([0]), np.array([1]), np.full((1, 10), coeff))


def test_edge_mobility_population_sums():
    # test_mobility.cpp:154-215: 10% of every compartment leaves node 1 for node 2
    # (990/10 -> 891/9 and 1089/11), returns (1000/1000), leaves again (900/1100)
    g = two_node_graph(0.1)
    rec, fin, st = O.graph_run(g, 0.0, 1.5, 0.5, 0.1)
    sums = rec.sum(axis=2)
    np.testing.assert_allclose(sums[0], [900, 1100], rtol=1e-12)
    np.testing.assert_allclose(sums[1], [1000, 1000], rtol=1e-12)
    np.testing.assert_allclose(sums[2], [900, 1100], rtol=1e-12)


def test_zero_coefficients_equal_independent_solves():
    # test_mobility.cpp:30-127 (compareNoMobilityWithSingleIntegration)
    g = W.mobility_graph(seed=4, N=6, out_degree=2)
    g0 = L.GraphArrays(g.num_groups, g.params, g.contact_baseline, g.contact_minimum, g.damping_times,
                       g.damping_values, g.init_state, g.edge_src, g.edge_dst, np.zeros_like(g.edge_coeff_baseline))
    _, fin, _ = O.graph_run(g0, 0.0, 5.0)
    for v in range(g.num_nodes):
        t, y, _ = O.simulate(g.subgraph_nodes([v]), 0, 0.0, 5.0, 0.1)
        # the graph restarts every node solve at each exchange boundary, so the
        # step sequences differ: agreement within the integrator tolerance
        np.testing.assert_allclose(fin[v], y[-1], rtol=1e-5, atol=1e-6)


def test_graph_conservation_and_invariants():
    g = W.mobility_graph(seed=1, N=60, out_degree=12)
    rec, fin, st = O.graph_run(g, 0.0, 20.0)
    tot0 = g.init_state.sum()
    assert abs(fin.sum() - tot0) / tot0 < 1e-12
    # per-node population is conserved after every return (odd boundaries come back home)
    homes = g.init_state.sum(axis=1)
    np.testing.assert_allclose(rec[1::2].sum(axis=2), np.broadcast_to(homes, rec[1::2].shape[:2]), rtol=1e-9)
    y = rec.reshape(rec.shape[0], g.num_nodes, g.num_groups, 10)
    assert np.all(np.diff(y[..., L.D], axis=0) >= -1e-9)           # dead never decrease
    assert np.all(np.diff(y[..., L.R].sum(axis=1), axis=0) >= -1e-6)  # recovered (graph total) never decrease
    assert y.min() > -1e-6


def test_ensemble_threads_match_serial():
    ens = W.ensemble(num_samples=3, N=10, out_degree=3)
    res, el, st = O.ensemble_run(ens, 0.0, 3.0, num_threads=3)
    for g, r in zip(ens, res):
        _, fin, _ = O.graph_run(g, 0.0, 3.0, record=False)
        np.testing.assert_array_equal(r, fin)


def test_damping_cache_combines_levels():
    # damping.h:545-600: same level adds, different levels combine as 1-(1-a)(1-b)
    t, m = O.damping_cache(1, 1, [1.0, 2.0, 2.0], [0, 0, 1], [0, 1, 0], [[0.2], [0.3], [0.5]])
    assert list(t[1:-1]) == [1.0, 2.0]
    assert m[1, 0, 0] == 0.2
    np.testing.assert_allclose(m[2, 0, 0], 1 - (1 - 0.5) * (1 - 0.5))


def _commuter_test_graph(insc=0.0, isyc=0.0):
    """Two nodes of the one-group model of the reference's mobility-result test
    (cpp/tests/test_mobility.cpp:217-283) joined by an edge with coefficients 0.1."""
    G = 1
    p = np.zeros(L.param_stride(G))
    p[L.P_ICU_CAPACITY] = L.DBL_MAX
    p[L.P_TNT_CAPACITY] = L.DBL_MAX
    p[L.P_TNT_MAX_RISK] = 5.0
    for k, v in ((L.G_TIME_EXPOSED, 1.0), (L.G_TIME_INS, 1.0), (L.G_TIME_ISY, 1.0), (L.G_TIME_ISEV, 1.0),
                 (L.G_TIME_ICRI, 1.0), (L.G_TRANSMISSION_PROB, 1.0), (L.G_RISK_FROM_SYMPTOMATIC, 1.0),
                 (L.G_MAX_RISK_FROM_SYMPTOMATIC, 1.0), (L.G_REL_TRANSMISSION_NS, 1.0), (L.G_SEVERE_PER_ISY, 0.5)):
        p[L.group_param_index(k, 0, G)] = v
    y = np.zeros(10)
    y[L.INS], y[L.INSC], y[L.ISY], y[L.ISYC] = 10.0, insc, 20.0, isyc
    y[L.S] = 1000.0 - 30.0  # set_difference_from_total(S, 1000) before the confirmed compartments were set
    base = np.full((2, 1, 1, 1), 5.0)
    return L.GraphArrays(G, np.stack([p, p]), base, np.zeros_like(base), np.zeros((2, 1, 0)),
                         np.zeros((2, 1, 0, 1, 1)), np.stack([y, y]), np.array([0], np.int32),
                         np.array([1], np.int32), np.full((1, 10), 0.1))


def test_mobility_results_match_the_reference_test():
    # MobilityEdge::add_mobility_result_time_point (metapopulation_mobility_instant.h:423-447):
    # the save-index sets (INS + INSC, ISy + ISyC) and the total of the departing travelers
    sets = [[L.INS, L.INSC], [L.ISY, L.ISYC]]
    np.testing.assert_allclose(O.departure_commuters(_commuter_test_graph(), 0, 0.0, sets), [1.0, 2.0, 100.0],
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(O.departure_commuters(_commuter_test_graph(100.0, 30.0), 0, 0.0, sets),
                               [11.0, 5.0, 113.0], rtol=0, atol=1e-12)


def test_mobility_results_of_a_graph_run():
    # one time point per departure and per return; the run itself is unchanged by recording
    g = W.mobility_graph(seed=3, N=10, G=2, out_degree=3, stress=True)
    sets = [[L.INS, L.INSC, 10 + L.INS, 10 + L.INSC], [L.ISY, L.ISYC, 10 + L.ISY, 10 + L.ISYC]]
    fin, counts, times, values, st = O.graph_run_commuters(g, 0.0, 5.0, sets, capacity=16)
    _, fin0, _ = O.graph_run(g, 0.0, 5.0, record=False)
    np.testing.assert_array_equal(fin, fin0)
    assert (counts == 10).all()
    np.testing.assert_allclose(times[0, :10], np.arange(1, 11) * 0.5)
    # a departure's total equals the coefficient-weighted source state it took
    assert (values[:, :10, 2] > 0).all() and (values[:, :10, 2] >= values[:, :10, 0] + values[:, :10, 1]).all()
