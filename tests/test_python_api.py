"""The Python entry memilio_gb300.simulation(.osecir), mirroring
memilio.simulation(.osecir) (pycode/memilio-simulation): the reference's
example scripts' calls (pycode/examples/simulation/ode_secir_simple.py,
ode_secir_mobility.py) run unchanged apart from the imports. Host-only: the
parameter and population API, the damping cache against the oracle's
restatement of Dampings::update_cache, interpolation against the reference's
tests, GraphParameterStudy's sampled runs. GPU: simulate, MobilitySimulation
and GraphParameterStudy against the FP64 oracle."""
import numpy as np
import pytest

import memilio_gb300.simulation as mio
import memilio_gb300.simulation.osecir as osecir
from memilio_gb300 import layout as L
from oracle import oracle as O

State = osecir.InfectionState


def simple_model(total=83000.0, exposed=100.0):
    # the calls of ode_secir_simple.py
    model = osecir.Model(1)
    A0 = mio.AgeGroup(0)
    model.parameters.TimeExposed[A0] = 3.2
    model.parameters.TimeInfectedNoSymptoms[A0] = 2.
    model.parameters.TimeInfectedSymptoms[A0] = 6.
    model.parameters.TimeInfectedSevere[A0] = 12.
    model.parameters.TimeInfectedCritical[A0] = 8.
    model.populations[A0, State.Exposed] = exposed
    model.populations[A0, State.InfectedNoSymptoms] = 50
    model.populations[A0, State.InfectedSymptoms] = 50
    model.populations[A0, State.InfectedSevere] = 20
    model.populations[A0, State.InfectedCritical] = 10
    model.populations[A0, State.Recovered] = 10
    model.populations.set_difference_from_total((A0, State.Susceptible), total)
    model.parameters.RelativeTransmissionNoSymptoms[A0] = 0.67
    model.parameters.TransmissionProbabilityOnContact[A0] = 1.0
    model.parameters.RecoveredPerInfectedNoSymptoms[A0] = 0.09
    model.parameters.RiskOfInfectionFromSymptomatic[A0] = 0.25
    model.parameters.SeverePerInfectedSymptoms[A0] = 0.2
    model.parameters.CriticalPerSevere[A0] = 0.25
    model.parameters.DeathsPerCritical[A0] = 0.3
    model.parameters.MaxRiskOfInfectionFromSymptomatic[A0] = 0.5
    model.parameters.ContactPatterns.cont_freq_mat[0].baseline = np.ones((1, 1))
    model.parameters.ContactPatterns.cont_freq_mat[0].minimum = np.zeros((1, 1))
    model.parameters.ContactPatterns.cont_freq_mat.add_damping(mio.Damping(coeffs=np.r_[0.9], t=30.0, level=0, type=0))
    model.apply_constraints()
    return model


def test_parameters_and_populations():
    m = simple_model()
    assert m.populations.get_total() == 83000.0
    assert m.parameters.TimeExposed[mio.AgeGroup(0)] == 3.2
    assert m.parameters.ICUCapacity == L.DBL_MAX and m.parameters.TestAndTraceCapacityMaxRisk == 5.0
    m.parameters.Seasonality = 0.7  # out of range: apply_constraints resets it
    assert m.apply_constraints() and m.parameters.Seasonality == 0.0
    m.populations.set_difference_from_group_total_AgeGroup((mio.AgeGroup(0), State.Susceptible), 1000.0)
    assert m.populations.get_group_total_AgeGroup(0) == 1000.0
    with pytest.raises(IndexError):
        m.parameters.TimeExposed[mio.AgeGroup(1)] = 1.0


def test_damping_cache_matches_oracle():
    ds = [mio.Damping(0.4, 6.0), mio.Damping(np.full((2, 2), 0.2), 9.0, level=1),
          mio.Damping(0.1, 9.0, level=1, type=1), mio.Damping(0.3, 12.0), mio.Damping(0.35, 12.0)]
    t, v = mio.damping_cache((2, 2), ds)
    # the last damping replaces the one with the same (time, type, level)
    ot, ov = O.damping_cache(2, 2, [6, 9, 9, 12], [0, 1, 1, 0], [0, 0, 1, 0],
                             np.array([np.full((2, 2), x) for x in (0.4, 0.2, 0.1, 0.35)]))
    np.testing.assert_array_equal(t, ot)
    np.testing.assert_array_equal(v, ov)


def test_interpolation_matches_reference_tests():
    # cpp/tests/test_analyze_result.cpp:150-175 (timePointsCanBeChosen) and :106-121
    ts = mio.TimeSeries(1)
    for t, y in [(0.1, 0.0), (0.9, 1.0), (1.4, 2.0), (2.5, 3.0), (3.0, 4.0)]:
        ts.add_time_point(t, [y])
    r = mio.interpolate_simulation_result(ts, times=[0.2, 0.6, 1.0, 1.3, 2.4])
    np.testing.assert_allclose(r.as_ndarray()[1], [1 / 8, 5 / 8, 1.2, 1.8, 2 + 10 / 11], rtol=0, atol=1e-12)
    ts = mio.TimeSeries(1)
    for t, y in [(0.0, 0.0), (0.5, 1.0), (1.0, 2.0), (2.1, 3.0), (3.0, 4.0)]:
        ts.add_time_point(t, [y])
    r = mio.interpolate_simulation_result(ts)
    np.testing.assert_allclose(r.as_ndarray()[0], [0, 1, 2, 3])
    np.testing.assert_allclose(r.as_ndarray()[1, 1:3], [2.0, 2 + 10 / 11], rtol=0, atol=1e-12)


def test_graph_keeps_edges_sorted():
    g = osecir.MobilityGraph()
    for i in range(3):
        g.add_node(i, simple_model())
    g.add_edge(2, 0, 0.1 * np.ones(10))
    g.add_edge(0, 1, 0.1 * np.ones(10))
    g.add_edge(1, 0, 0.1 * np.ones(10))
    assert [(g.get_edge(i).start_node_idx, g.get_edge(i).end_node_idx) for i in range(3)] == [(0, 1), (1, 0), (2, 0)]


def two_node_graph():
    graph = osecir.MobilityGraph()
    graph.add_node(id=0, model=simple_model(10000.0), t0=0)
    graph.add_node(id=1, model=simple_model(2000.0, exposed=0.0), t0=0)
    coeffs = 0.1 * np.ones(10)
    coeffs[State.Dead] = 0
    graph.add_edge(0, 1, mio.MobilityParameters(coeffs))
    graph.add_edge(1, 0, mio.MobilityParameters(coeffs))
    return graph


def sample_run(graph, run):
    """A seeded stand-in for draw_sample: per run, other initial exposed and exposure times."""
    rng = np.random.default_rng(run)
    for node in (graph.get_node(i) for i in range(graph.num_nodes)):
        m = node.property.model
        m.populations[mio.AgeGroup(0), State.Exposed] = float(rng.uniform(50.0, 150.0))
        m.parameters.TimeExposed[mio.AgeGroup(0)] = float(rng.uniform(2.5, 4.0))


def test_parameter_study_samples_copies():
    graph = two_node_graph()
    study = osecir.GraphParameterStudy(graph, 0.0, 10.0, 0.5, 3, sample=sample_run)
    assert (study.num_runs, study.t0, study.tmax, study.dt) == (3, 0.0, 10.0, 0.5)
    runs = study._sampled_graphs()
    assert len(runs) == 3
    e0 = [r.get_node(0).property.model.populations[mio.AgeGroup(0), State.Exposed] for r in runs]
    assert len(set(e0)) == 3  # every run drew its own values
    # the graph itself is not changed, and each run starts from its sampled populations
    assert graph.get_node(0).property.model.populations[mio.AgeGroup(0), State.Exposed] == 100.0
    for r in runs:
        res = r.get_node(0).property.result
        assert res.get_num_time_points() == 1
        np.testing.assert_array_equal(res.get_last_value(), r.get_node(0).property.model.populations.array())
    again = study._sampled_graphs()  # runs are reproducible
    assert [r.get_node(0).property.model.parameters.TimeExposed[mio.AgeGroup(0)] for r in again] == \
        [r.get_node(0).property.model.parameters.TimeExposed[mio.AgeGroup(0)] for r in runs]
    with pytest.raises(ValueError):
        osecir.GraphParameterStudy(graph, 0.0, 10.0, 0.5, 0)


@pytest.mark.gpu
def test_parameter_study_matches_oracle():
    study = osecir.GraphParameterStudy(two_node_graph(), 0.0, 10.0, 0.5, 3, sample=sample_run)
    seen = []
    study.run(lambda g, r: seen.append((r, g)))
    assert [r for r, _ in seen] == [0, 1, 2]
    expect = study._arrays(study._sampled_graphs())
    for (r, g), a in zip(seen, expect):
        rec, fin, _ = O.graph_run(a, 0.0, 10.0, dt_exchange=0.5, dt0=0.5)
        for v in range(2):
            got = g.get_node(v).property.result
            assert got.get_num_time_points() == 21
            np.testing.assert_allclose(got.get_last_value(), fin[v], rtol=1e-10, atol=1e-10 * fin[v].sum())
            np.testing.assert_allclose(got.get_value(10), rec[9, v], rtol=1e-10, atol=1e-10 * fin[v].sum())
    results = osecir.GraphParameterStudy(two_node_graph(), 0.0, 10.0, 0.5, 2, sample=sample_run).run()
    np.testing.assert_allclose(results[1].get_node(1).property.result.get_last_value(),
                               seen[1][1].get_node(1).property.result.get_last_value(), rtol=1e-12, atol=1e-9)


def sample_model(model, run):
    rng = np.random.default_rng(100 + run)
    model.populations[mio.AgeGroup(0), State.Exposed] = float(rng.uniform(50.0, 150.0))
    model.parameters.TimeInfectedSymptoms[mio.AgeGroup(0)] = float(rng.uniform(5.0, 7.0))


def test_model_parameter_study_samples_copies():
    m = simple_model()
    study = osecir.ParameterStudy(m, 0.0, 20.0, 0.1, 4, sample=sample_model)
    runs = study._sampled_models()
    assert len({r.parameters.TimeInfectedSymptoms[mio.AgeGroup(0)] for r in runs}) == 4
    assert m.populations[mio.AgeGroup(0), State.Exposed] == 100.0
    assert study.parameters is m and study.num_runs == 4


@pytest.mark.gpu
def test_model_parameter_study_matches_oracle():
    study = osecir.ParameterStudy(simple_model(), 0.0, 30.0, 0.1, 4, sample=sample_model)
    sims = study.run()
    for r, (sim, m) in enumerate(zip(sims, study._sampled_models())):
        g = osecir._graph_arrays([m], [m.populations.array()])
        t, y, _ = O.simulate(g, 0, 0.0, 30.0, 0.1)
        got = sim.result
        assert got.get_num_time_points() == t.size
        np.testing.assert_allclose(got.as_ndarray()[0], t, rtol=0, atol=1e-9)
        np.testing.assert_allclose(got.get_last_value(), y[-1], rtol=1e-9, atol=1e-9 * 83000)
        assert sim.model.parameters.TimeInfectedSymptoms[mio.AgeGroup(0)] == \
            m.parameters.TimeInfectedSymptoms[mio.AgeGroup(0)]
    seen = []
    study.run(lambda s, r: seen.append(r))
    assert seen == [0, 1, 2, 3]


@pytest.mark.gpu
def test_simulate_flows_matches_oracle():
    m = simple_model()
    pops, flows = osecir.simulate_flows(0, 30, 0.1, m)
    g = osecir._graph_arrays([m], [m.populations.array()])
    t, f, y, _ = O.simulate_flows(g, 0, 0.0, 30.0, 0.1)
    assert pops.get_num_time_points() == flows.get_num_time_points() == t.size
    np.testing.assert_allclose(flows.as_ndarray()[0], t, rtol=0, atol=1e-9)
    np.testing.assert_allclose(flows.get_last_value(), f[-1], rtol=1e-9, atol=1e-9 * 83000)
    np.testing.assert_allclose(pops.get_last_value(), y[-1], rtol=1e-9, atol=1e-9 * 83000)


@pytest.mark.gpu
def test_simulate_matches_oracle():
    m = simple_model()
    r = osecir.simulate(0, 50, 0.1, m)
    g = osecir._graph_arrays([m], [m.populations.array()])
    t, y, _ = O.simulate(g, 0, 0.0, 50.0, 0.1)
    np.testing.assert_allclose(r.as_ndarray()[0], t, rtol=0, atol=1e-9)
    np.testing.assert_allclose(r.get_last_value(), y[-1], rtol=1e-9, atol=1e-9 * 83000)


@pytest.mark.gpu
def test_mobility_simulation_matches_oracle():
    # the calls of ode_secir_mobility.py
    graph = osecir.MobilityGraph()
    graph.add_node(id=0, model=simple_model(10000.0), t0=0)
    graph.add_node(id=1, model=simple_model(2000.0, exposed=0.0), t0=0)
    coeffs = 0.1 * np.ones(10)
    coeffs[State.Dead] = 0
    graph.add_edge(0, 1, mio.MobilityParameters(coeffs))
    graph.add_edge(1, 0, mio.MobilityParameters(coeffs))
    sim = osecir.MobilitySimulation(graph, 0, dt=0.5)
    sim.advance(20)
    r0 = osecir.interpolate_simulation_result(sim.graph.get_node(0).property.result)
    assert r0.get_num_time_points() == 21
    rec, fin, _ = O.graph_run(sim._g, 0.0, 20.0)
    for v in range(2):
        got = sim.graph.get_node(v).property.result
        assert got.get_num_time_points() == 41
        np.testing.assert_allclose(got.get_last_value(), fin[v], rtol=1e-10, atol=1e-10 * fin[v].sum())
        np.testing.assert_allclose(got.get_value(20), rec[19, v], rtol=1e-10, atol=1e-10 * fin[v].sum())
