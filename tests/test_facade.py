"""The C++ facade (memilio_gb300/cpp/miogpu): MEmilio's C++ API over libmiogpu.

Host-only checks (no GPU): the facade's damping cache equals the oracle's
restatement of Dampings::update_cache, and a graph packs into a valid layout
(edges sorted by (src, dst) although added out of order, padded damping
caches, the reference's parameter defaults). GPU checks compare the facade's
Simulation, GraphSimulation and ParameterStudy with the FP64 oracle.
"""
import json
import subprocess

import numpy as np
import pytest

from memilio_gb300 import build as B
from memilio_gb300 import layout as L
from oracle import oracle as O

FP64_TOL = 1e-10  # batched FP64 solver vs oracle, relative to the age group's population
ODE_TOL = 1e-5    # two accurate solutions with different step sequences (the integrator's rel tol)


@pytest.fixture(scope="module")
def programs():
    return B.build_facade()


def run(programs, mode):
    r = subprocess.run([programs["facade_check"], mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def graph_of(d):
    G, N, M, K = d["G"], d["N"], d["M"], d["K"]
    E = d["E"]
    return L.GraphArrays(G, np.array(d["params"]), np.array(d["contact_baseline"]).reshape(N, M, G, G),
                         np.array(d["contact_minimum"]).reshape(N, M, G, G),
                         np.array(d["damping_times"]).reshape(N, M, K),
                         np.array(d["damping_values"]).reshape(N, M, K, G, G),
                         np.array(d["state"]).reshape(N, 10 * G), np.array(d["src"], np.int32),
                         np.array(d["dst"], np.int32), np.array(d["coeff_baseline"]).reshape(E, 10 * G),
                         np.array(d["coeff_minimum"]).reshape(E, 10 * G))


def scaled(a, b, G):
    a = np.asarray(a).reshape(-1, G, 10)
    b = np.asarray(b).reshape(-1, G, 10)
    return float(np.max(np.abs(a - b) / np.maximum(b.sum(axis=2, keepdims=True), 1.0)))


def test_damping_cache_matches_oracle(programs):
    cases = run(programs, "dampings")["cases"]
    assert len(cases) == 5
    for c in cases:
        n = len(c["times"])
        t = np.array(c["cache_times"])
        v = np.array(c["cache_values"]).reshape(-1, 2, 2)
        if n == 0:
            assert t.shape[0] == 2 and np.all(v == 0)
            continue
        ot, ov = O.damping_cache(2, 2, c["times"], np.array(c["levels"], np.int32), np.array(c["types"], np.int32),
                                 np.array(c["matrices"]).reshape(n, 2, 2))
        np.testing.assert_array_equal(t, ot)
        np.testing.assert_allclose(v, ov, rtol=0, atol=1e-15)
    # an equal (time, type, level) key replaces the damping
    assert cases[4]["times"] == [3.0, 3.0] and cases[4]["matrices"][0] == 0.7


def test_graph_packs_into_layout(programs):
    d = run(programs, "pack")
    g = graph_of(d)  # validates shapes and (src, dst) order
    assert list(zip(d["src"], d["dst"])) == [(0, 1), (0, 2), (1, 0), (2, 0)]
    assert g.num_damping_points == d["K"] >= 3
    assert np.all(g.damping_times[:, :, 0] == np.finfo(np.float64).min)
    assert np.all(g.damping_times[:, :, -1] == np.finfo(np.float64).max)
    p = g.params[0]
    assert p[L.P_TNT_MAX_RISK] == 5.0  # the reference's default
    assert np.all(g.init_state >= 0)


@pytest.mark.gpu
def test_simulation_matches_oracle(programs):
    d = run(programs, "simulate")
    G, K, M = d["G"], d["K"], d["M"]
    g = L.GraphArrays(G, np.array(d["params"]), np.array(d["contact_baseline"]).reshape(1, M, G, G),
                      np.array(d["contact_minimum"]).reshape(1, M, G, G), np.array(d["damping_times"]).reshape(1, M, K),
                      np.array(d["damping_values"]).reshape(1, M, K, G, G), np.array(d["state"]).reshape(1, 10 * G),
                      np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 10 * G)))
    t, y, _ = O.simulate(g, 0, 0.0, 12.0, 0.1)
    np.testing.assert_allclose(d["times_whole"], t, rtol=0, atol=1e-6)
    assert scaled(d["last_whole"], y[-1], G) < 1e-8
    # two advance() calls keep the step size: the grid contains the first horizon
    assert 4.0 in d["times_pieces"] and d["dt_mid"] > 0
    assert scaled(d["last_pieces"], y[-1], G) < ODE_TOL
    ref = O.eval_rhs(g, 0, g.init_state[0], g.init_state[0], 5.0)
    np.testing.assert_allclose(d["dydt_t5"], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.gpu
def test_graph_simulation_matches_oracle(programs):
    d = run(programs, "graph")
    g = graph_of(d)
    rec, fin, _ = O.graph_run(g, 0.0, 6.0, record=True)
    assert d["t_end"] == 6.0
    t = np.array(d["t"])
    np.testing.assert_allclose(t, np.arange(0.0, 6.01, 0.5), rtol=0, atol=1e-12)
    states = np.array(d["states"]).reshape(len(t), g.num_nodes, g.n)
    assert scaled(states[0], g.init_state, g.num_groups) == 0.0
    for b in range(1, len(t)):
        assert scaled(states[b], rec[b - 1], g.num_groups) < FP64_TOL, b


@pytest.mark.gpu
def test_parameter_study_matches_oracle(programs):
    runs = run(programs, "study")["runs"]
    assert len(runs) == 4
    finals = []
    for r in runs:
        g = graph_of(r)
        _, fin, _ = O.graph_run(g, 0.0, 5.0, record=False)
        got = np.array(r["final"]).reshape(g.num_nodes, g.n)
        assert scaled(got, fin, g.num_groups) < FP64_TOL
        finals.append(got)
    # the sampled transmission factors differ, so do the results
    assert not np.allclose(finals[0], finals[3])


@pytest.mark.gpu
def test_flow_simulation_matches_oracle(programs):
    d = run(programs, "flows")
    G, K, M = d["G"], d["K"], d["M"]
    g = L.GraphArrays(G, np.array(d["params"]), np.array(d["contact_baseline"]).reshape(1, M, G, G),
                      np.array(d["contact_minimum"]).reshape(1, M, G, G), np.array(d["damping_times"]).reshape(1, M, K),
                      np.array(d["damping_values"]).reshape(1, M, K, G, G), np.array(d["state"]).reshape(1, 10 * G),
                      np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, 10 * G)))
    t, f, y, _ = O.simulate_flows(g, 0, 0.0, 10.0, 0.1)
    np.testing.assert_allclose(d["t"], t, rtol=0, atol=1e-6)
    assert scaled(d["last_pop"], y[-1], G) < 1e-8
    np.testing.assert_allclose(d["last_flows"], f[-1], rtol=1e-8, atol=1e-8 * np.abs(f[-1]).max())


@pytest.mark.gpu
def test_example_program_runs():
    # memilio_gb300/cpp/examples/ode_secir_graph.cpp: two counties, 30 days
    r = subprocess.run([B.build_facade()["ode_secir_graph"]], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("node ")]
    assert len(lines) == 2 and all("t=30.0" in l for l in lines)
    totals = [float(l.split("(total ")[1].split(",")[0]) for l in lines]
    assert abs(sum(totals) - 30000.0) < 1e-6  # 20000 + 10000 residents, conserved by the exchange


def test_interpolate_simulation_result_matches_reference_tests(programs):
    # expectations of cpp/tests/test_analyze_result.cpp:68-175
    d = run(programs, "interpolate")
    near = lambda a, b: np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)
    near(d["simple"]["t"], [0, 1, 2, 3, 4, 5])
    near(d["simple"]["v"], [0.1, 0.25, 0.35, 0.45, 0.55, 0.65])
    near(d["complex"]["t"], [0, 1, 2])
    near(d["complex"]["v"], [1, 2, 1 + 2 * 2 / 3, 2 + 8 * 2 / 3, 3 + 2 * 5 / 6, 10 - 7 * 5 / 6])
    near(d["exact_day"]["t"], [0, 1, 2, 3])
    near(d["exact_day"]["v"][1:3], [2.0, 2.0 + 10 / 11])
    near(d["default_tol"]["t"], [0, 1, 2])
    near(d["given_tol"]["t"], [1, 2])
    near(d["chosen"]["t"], [0.2, 0.6, 1.0, 1.3, 2.4])
    near(d["chosen"]["v"], [1 / 8, 5 / 8, 1.2, 1.8, 2 + 10 / 11])


@pytest.mark.gpu
def test_mobility_results_match_oracle(programs):
    # MobilityEdge::get_mobility_results with save indices through the facade
    # (the reference's cpp/examples/ode_secir_graph.cpp sets), against the oracle
    d = run(programs, "commuters")
    g = graph_of(d)
    G = g.num_groups
    sets = [[gr * 10 + c for gr in range(G) for c in (L.INS, L.INSC)],
            [gr * 10 + c for gr in range(G) for c in (L.ISY, L.ISYC)]]
    _, counts, times, values, _ = O.graph_run_commuters(g, 0.0, 6.0, sets, capacity=16)
    np.testing.assert_array_equal(np.array(d["counts"], int), counts)
    got_t = np.array(d["times"]).reshape(g.num_edges, -1)
    got_v = np.array(d["values"]).reshape(g.num_edges, -1, len(sets) + 1)
    np.testing.assert_allclose(got_t, times[:, :counts[0]], rtol=0, atol=1e-12)
    ref = values[:, :counts[0]]
    assert np.max(np.abs(got_v - ref) / np.maximum(np.abs(ref), 1e-9 * ref[..., -1:])) < 1e-10


def test_graph_builder_sorts_and_deduplicates(programs):
    # GraphBuilder::build(make_unique=true) (cpp/memilio/mobility/graph_builder.h):
    # edges sorted by (start, end); of the two 0 -> 1 edges the one added last
    # (coefficients 0.03) stays, as Graph::add_edge's replacement leaves it
    d = run(programs, "builder")
    assert d["same"] == 1 and d["E"] == 4
    assert list(zip(d["src"], d["dst"])) == [(0, 1), (0, 2), (1, 0), (2, 0)]
    assert abs(d["coeff_baseline"][0] - 0.03) < 1e-15


@pytest.mark.gpu
def test_graph_of_flow_simulations(programs):
    # the reference's consistency test of a graph of FlowSimulation nodes
    # (cpp/tests/test_graph_simulation.cpp:276-340): the same states as a graph
    # of Simulation nodes (to rounding: the FP64 kernel that also sums the flows
    # contracts a few multiply-adds differently), the flows start at zero and
    # only grow
    d = run(programs, "flows_graph")
    G = d["G"]
    P = len(d["t"])
    assert P == 13 and abs(d["t"][-1] - 6.0) < 1e-12
    np.testing.assert_allclose(d["states_flows"], d["states_plain"], rtol=1e-12, atol=1e-12)
    f = np.array(d["flows"]).reshape(3, P, 15 * G)
    assert (f[:, 0] == 0).all() and (np.diff(f, axis=1) >= 0).all() and f[:, -1].max() > 0
