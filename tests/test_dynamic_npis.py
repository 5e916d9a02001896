"""Dynamic NPIs (osecir::Simulation::advance, cpp/models/ode_secir/model.h:289-367;
implement_dynamic_npis and DynamicNPIs, cpp/memilio/epidemiology/dynamic_npis.h).

Host-only: the facade's damping lists after implement_dynamic_npis and after the
NPI check of Simulation::advance with the state held fixed equal the
expectations of the reference's tests (cpp/tests/test_dynamic_npis.cpp:
implement_empty :145-170, implement :172-317, secir_threshold_safe :421-450,
secir_threshold_exceeded :452-482, secir_delayed_implementation :484-539). The
oracle's restatement runs a graph without thresholds exactly as without NPIs.
GPU: a graph simulation with NPIs through the facade (device solver, caches
replaced with mgpu_batch_set_damping_cache) against the oracle, with and
without NPIs on the mobility edges (MobilityEdge::apply_mobility,
cpp/memilio/mobility/metapopulation_mobility_instant.h:549-566).
"""
import json
import subprocess

import numpy as np
import pytest

from memilio_gb300 import build as B
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W
from oracle import oracle as O

from tests.test_facade import graph_of, scaled


@pytest.fixture(scope="module")
def programs():
    return B.build_facade()


def run(programs, mode):
    r = subprocess.run([programs["facade_check"], mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def lists(d):
    """[(time, level, type, value)] per matrix, times rounded for comparison."""
    return [[(round(t, 12), lv, ty, round(v, 12)) for t, lv, ty, v in m] for m in d]


def test_implement_dynamic_npis_matches_reference_tests(programs):
    d = run(programs, "npi_logic")
    assert lists(d["implement_empty"]) == [[(0.45, 0, 0, 0.8), (0.6, 0, 0, 0.0)]] * 2
    assert lists(d["implement_first"]) == [
        [(0.3, 0, 0, 0.15), (0.4, 0, 0, 0.2), (0.45, 0, 0, 0.4), (0.5, 0, 1, 0.25), (0.6, 0, 0, 0.2),
         (0.7, 0, 0, 0.35)],
        [(0.45, 0, 0, 0.4), (0.5, 1, 1, 0.25), (0.6, 0, 0, 0.0), (0.9, 0, 0, 0.45)]]
    assert lists(d["implement_second"]) == [
        [(0.3, 0, 0, 0.3), (0.45, 0, 0, 0.4), (0.5, 0, 1, 0.25), (0.6, 0, 0, 0.3), (0.7, 0, 0, 0.35)],
        [(0.45, 0, 0, 0.4), (0.5, 1, 1, 0.25), (0.6, 0, 0, 0.0), (0.9, 0, 0, 0.45)]]


def contact_at(dampings, t, baseline=1.0):
    """ContactMatrixGroup::get_matrix_at of a 1 x 1 matrix with these dampings."""
    if not dampings:
        return baseline
    times = [x[0] for x in dampings]
    ct, cm = O.damping_cache(1, 1, times, [x[1] for x in dampings], [x[2] for x in dampings],
                             np.array([x[3] for x in dampings]).reshape(-1, 1, 1))
    ub = int(np.searchsorted(ct, t, side="right"))
    lo, hi = cm[ub - 1, 0, 0], cm[ub, 0, 0]
    x0, x1 = ct[ub] - 1.0, ct[ub]
    d = lo if t <= x0 else (hi if t >= x1 else 0.5 * (lo - hi) * np.cos(np.pi / (x1 - x0) * (t - x0)) + 0.5 * (lo + hi))
    return baseline - d * baseline


def test_npi_check_matches_reference_tests(programs):
    d = run(programs, "npi_logic")
    assert d["threshold_safe"] == [[]]
    assert len(d["threshold_exceeded"][0]) == 2
    t0 = d["delayed_t0"][0]  # t0 = 0: no delay at the start, full effect at once
    for t in (0.0, 1.0, 3.0):
        assert contact_at(t0, t) == 0.5
    t1 = d["delayed_t1"][0]  # t0 = 1, delay 2: ramp over [3, 4]
    assert contact_at(t1, 3.0) == 1.0 and contact_at(t1, 4.0) == 0.5
    tl = d["delayed_long"][0]  # delay 10: ramp over [11, 12]
    assert contact_at(tl, 11.0) == 1.0 and contact_at(tl, 12.0) == 0.5
    # keep-alive: renewed at expiry without a dip
    ka = d["keep_alive"][0]
    assert all(contact_at(ka, t) == 0.5 for t in np.arange(0.0, 8.01, 0.25))


def test_oracle_without_thresholds_equals_plain_run():
    g = W.mobility_graph(seed=5, N=8, G=2, out_degree=3)
    _, fin0, _ = O.graph_run(g, 0.0, 10.0, record=False)
    fin, cnt, _ = O.graph_run_npi(g, 0.0, 10.0, {"thresholds": []}, [])
    np.testing.assert_array_equal(fin, fin0)
    assert not cnt.any()


def test_oracle_npis_enact_and_conserve():
    g = W.mobility_graph(seed=5, N=8, G=2, out_degree=3)
    npis = {"thresholds": [(1e-6, [(0.5, 0, 0, [0], [1.0, 1.0])])], "duration": 3.0, "delay": 1.0}
    fin, cnt, _ = O.graph_run_npi(g, 0.0, 10.0, npis, [])
    _, fin0, _ = O.graph_run(g, 0.0, 10.0, record=False)
    assert cnt.min() >= 1
    np.testing.assert_allclose(fin.sum(), g.init_state.sum(), rtol=1e-12)
    # fewer contacts, fewer infections
    assert fin.reshape(8, 2, 10)[..., L.S].sum() > fin0.reshape(8, 2, 10)[..., L.S].sum()


def edge_npis_of(G):
    """The edge NPIs of facade_check's npi_edges mode (edge_npis)."""
    ones = [1.0] * G
    return {"thresholds": [(1.0, [(0.5, 0, 0, [0], ones)]), (4.0, [(0.8, 1, 0, [0], ones)])],
            "duration": 2.0, "base_value": 1e5}


def test_oracle_edge_npis():
    g = W.mobility_graph(seed=5, N=8, G=2, out_degree=3)
    fin0, cnt0, _ = O.graph_run_npi(g, 0.0, 10.0, {"thresholds": []}, [])
    # edge NPIs without thresholds: the run without NPIs
    fin, cnt, ecnt, _ = O.graph_run_npi(g, 0.0, 10.0, {"thresholds": []}, [], edge_npis={"thresholds": []})
    np.testing.assert_array_equal(fin, fin0)
    assert not ecnt.any()
    # a threshold every source crosses at once: every edge enacts at the first exchange and, with
    # one-day NPIs, again at every expiry
    ones = [1.0, 1.0]
    enp = {"thresholds": [(1e-9, [(0.6, 0, 0, [0], ones)])], "duration": 1.0}
    fin, cnt, ecnt, _ = O.graph_run_npi(g, 0.0, 10.0, {"thresholds": []}, [], edge_npis=enp)
    assert ecnt.shape == (g.num_edges,) and (ecnt == 10).all()
    np.testing.assert_allclose(fin.sum(), g.init_state.sum(), rtol=1e-12)
    assert np.abs(fin - fin0).max() > 1e-6  # fewer commuters change the epidemic
    # full damping of the commuters: the nodes run as if unconnected
    enp_all = {"thresholds": [(1e-9, [(1.0, 0, 0, [0], ones)])], "duration": 100.0}
    fin, _, ecnt, _ = O.graph_run_npi(g, 0.0, 10.0, {"thresholds": []}, [], edge_npis=enp_all)
    assert (ecnt == 1).all()
    solo = L.GraphArrays(g.num_groups, g.params, g.contact_baseline, g.contact_minimum, g.damping_times,
                         g.damping_values, g.init_state, np.zeros(0, np.int32), np.zeros(0, np.int32),
                         np.zeros((0, g.n)))
    _, fin_solo, _ = O.graph_run(solo, 0.0, 10.0, record=False)
    np.testing.assert_allclose(fin, fin_solo, rtol=1e-9, atol=1e-9)


def npis_of_facade_graph(G):
    """The NPIs of facade_check's npi_graph mode (three_nodes_npi)."""
    ones = [1.0] * G
    return {"thresholds": [(2.0, [(0.5, 0, 0, [0], ones)]), (6.0, [(0.8, 2, 0, [0], ones)])],
            "duration": 3.0, "delay": 1.0, "base_value": 1e5}


@pytest.mark.gpu
def test_graph_simulation_with_npis_matches_oracle(programs):
    d = run(programs, "npi_graph")
    g = graph_of(d)
    G = g.num_groups
    init = [(t, lv, ty, m, np.full((G, G), v)) for m, lst in enumerate(d["initial_dampings"]) for t, lv, ty, v in lst]
    fin, cnt, _ = O.graph_run_npi(g, 0.0, 12.0, npis_of_facade_graph(G), init)
    assert cnt.sum() > 0  # NPIs were enacted in this run
    np.testing.assert_array_equal(np.array(d["enacted_fp64"]), cnt)
    assert scaled(d["final_fp64"], fin, G) < 1e-10
    np.testing.assert_array_equal(np.array(d["enacted_mixed"]), cnt)
    assert scaled(d["final_mixed"], fin, G) < 1e-5


@pytest.mark.gpu
def test_set_damping_cache_between_advances():
    from memilio_gb300 import _native as N
    ctx = N.Context(0)
    g1 = W.mobility_graph(seed=7, N=6, G=2, out_degree=3)
    # g2: a second damping at day 4 on node 2 (same cache as g1 before day 3)
    t1, v1 = g1.damping_times[2, 0], g1.damping_values[2, 0]
    G = g1.num_groups
    t_new = np.array([t1[0], 4.0, t1[1], t1[2]])
    v_new = np.stack([v1[0], np.full((G, G), 0.25), v1[1] + 0.25 - v1[1] * 0.25, v1[2] + 0.25 - v1[2] * 0.25])
    assert t1.size == 3 and t1[1] > 5.0
    K = 4  # room for the extra point: pad every cache by repeating its last point
    pad = lambda g: L.GraphArrays(G, g.params, g.contact_baseline, g.contact_minimum,
                                  np.concatenate([g.damping_times, np.full(g.damping_times.shape[:2] + (1,), L.DBL_MAX)], 2),
                                  np.concatenate([g.damping_values, g.damping_values[:, :, -1:]], 2),
                                  g.init_state, g.edge_src, g.edge_dst, g.edge_coeff_baseline)
    a = pad(g1)
    b = pad(g1)
    b.damping_times[2, 0] = t_new
    b.damping_values[2, 0] = v_new
    for prec in (N.PRECISION_FP64, N.PRECISION_MIXED):
        ba = N.Batch(ctx, [a], 0.0, N.solver_opts(precision=prec))
        bb = N.Batch(ctx, [b], 0.0, N.solver_opts(precision=prec))
        ba.advance(2.0)
        ba.set_damping_cache(0, 2, 0, t_new, v_new)
        ba.advance(8.0)
        bb.advance(8.0)
        if prec == N.PRECISION_FP64:
            np.testing.assert_array_equal(ba.states()[0], bb.states()[0])
        else:
            # (the FP32 contact rows of the two caches round differently before day 3)
            assert scaled(ba.states()[0], bb.states()[0], G) < 1e-6
        with pytest.raises(N.MgpuError):
            ba.set_damping_cache(0, 2, 0, np.zeros(K + 1), np.zeros((K + 1, G, G)))  # more points than room
        ba.close()
        bb.close()
    # a damping cache shared by two graphs of a batch cannot be replaced for one of them
    bs = N.Batch(ctx, [a, a], 0.0, N.solver_opts())
    with pytest.raises(N.MgpuError):
        bs.set_damping_cache(0, 2, 0, t_new, v_new)
    bs.close()
    ctx.close()


@pytest.mark.gpu
def test_graph_simulation_with_edge_npis_matches_oracle(programs):
    d = run(programs, "npi_edges")
    g = graph_of(d)
    G = g.num_groups
    init = [(t, lv, ty, m, np.full((G, G), v)) for m, lst in enumerate(d["initial_dampings"]) for t, lv, ty, v in lst]
    fin, cnt, ecnt, _ = O.graph_run_npi(g, 0.0, 12.0, npis_of_facade_graph(G), init, edge_npis=edge_npis_of(G))
    assert ecnt.sum() > 0  # edge NPIs were enacted in this run
    for tag, tol in (("fp64", 1e-10), ("mixed", 1e-5)):
        np.testing.assert_array_equal(np.array(d["enacted_" + tag]), cnt)
        np.testing.assert_array_equal(np.array(d["edge_enacted_" + tag]), ecnt)
        assert scaled(d["final_" + tag], fin, G) < tol
    # recording only at tmax: the checks read the per-node sums of the device, the same run
    assert d["num_points_norecord"] == 2
    np.testing.assert_array_equal(d["final_norecord"], d["final_fp64"])
    np.testing.assert_array_equal(d["enacted_norecord"], list(d["enacted_fp64"]) + list(d["edge_enacted_fp64"]))


@pytest.mark.gpu
def test_compartment_sums_equal_state_sums():
    from memilio_gb300 import _native as N
    ctx = N.Context(0)
    graphs = [W.mobility_graph(seed=3, N=5, G=2, out_degree=2), W.mobility_graph(seed=4, N=7, G=3, out_degree=3)]
    for prec in (N.PRECISION_FP64, N.PRECISION_MIXED):
        b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=prec))
        b.advance(2.0)
        states = b.states()
        for c in (L.S, L.ISY, L.D):
            want = []
            for g, st in zip(graphs, states):
                for v in range(g.num_nodes):
                    s = 0.0
                    for gr in range(g.num_groups):
                        s += st[v, gr * 10 + c]
                    want.append(s)
            np.testing.assert_array_equal(b.compartment_sums(c), np.array(want))
        with pytest.raises(N.MgpuError):
            b.compartment_sums(10)
        b.close()
    ctx.close()


@pytest.mark.gpu
def test_step_api_order_is_enforced():
    from memilio_gb300 import _native as N
    ctx = N.Context(0)
    g = W.mobility_graph(seed=9, N=4, G=2, out_degree=2)
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64))
    ref = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64))
    with pytest.raises(N.MgpuError):
        b.step_exchange()  # no interval begun
    b.step_nodes(0.5)
    for call in (lambda: b.advance(1.0), lambda: b.step_nodes(0.5), lambda: b.set_state(ref.state_flat())):
        with pytest.raises(N.MgpuError):
            call()
    b.step_exchange()
    b.step_nodes(1.0)
    b.step_exchange()
    ref.advance(1.0)  # two split intervals equal two whole ones
    np.testing.assert_array_equal(b.state_flat(), ref.state_flat())
    b.close()
    ref.close()
    plain = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64_PLAIN))
    with pytest.raises(N.MgpuError):
        plain.step_nodes(0.5)
    plain.close()
    ctx.close()


@pytest.mark.gpu
def test_async_advance_refuses_interleaved_calls():
    # while an advance launched with mgpu_batch_launch is in progress, every call
    # that would change the state, the clock or the caches in between is refused;
    # the advance then completes as one whole mgpu_batch_advance would
    from memilio_gb300 import _native as N
    ctx = N.Context(0)
    g = W.mobility_graph(seed=9, N=6, G=2, out_degree=2)
    for prec in (N.PRECISION_FP64, N.PRECISION_MIXED):
        b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=prec))
        ref = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=prec))
        ref.advance(2.0)
        state0 = ref.state_flat()
        assert b.launch(2.0, 1) == 3  # four intervals, one launched
        times, vals = g.damping_times[0, 0], g.damping_values[0, 0]
        refused = (lambda: b.advance(2.0), lambda: b.reset(0.0), lambda: b.step_nodes(0.5),
                   lambda: b.set_state(state0), lambda: b.set_damping_cache(0, 0, 0, times, vals))
        for call in refused:
            with pytest.raises(N.MgpuError):
                call()
        rem = 3
        while rem:
            rem = b.launch(2.0, 1)
        while not b.query():
            pass
        np.testing.assert_array_equal(b.state_flat(), state0)
        b.close()
        ref.close()
    ctx.close()
