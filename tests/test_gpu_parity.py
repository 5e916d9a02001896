"""GPU parity: libmiogpu (through its C ABI) against the FP64 CPU oracle and
the reference's golden trajectories.

Tolerances (written per test):
  plain and batched FP64 solvers: max |gpu - oracle| / N_group <= 1e-10
  mixed FP32/FP64 solver        : max |gpu - oracle| / N_group <= 1e-5
where N_group is the population of the node's age group the compartment
belongs to. Conservation: every node's population after a return equals its
initial population to 1e-9 relative; the graph total to 1e-9.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W
from oracle import oracle as O
from tests.golden.scenarios import GOLDEN_CASES, golden_case, sum_groups

pytestmark = pytest.mark.gpu

PRECISIONS = [N.PRECISION_FP64_PLAIN, N.PRECISION_FP64, N.PRECISION_MIXED]
TOL = {N.PRECISION_FP64_PLAIN: 1e-10, N.PRECISION_FP64: 1e-10, N.PRECISION_MIXED: 1e-5}


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def group_scaled_error(gpu, ref, G):
    """max |gpu - ref| / (population of the age group), over all compartments."""
    gpu = np.asarray(gpu).reshape(-1, G, 10)
    ref = np.asarray(ref).reshape(-1, G, 10)
    scale = np.maximum(ref.sum(axis=2, keepdims=True), 1e-300)
    return float(np.max(np.abs(gpu - ref) / scale))


# Accepted-step grids. The CPU oracle reproduces the golden files at the
# reference's own tolerance (1e-9/1e-10 absolute) because it repeats the
# reference's rounding. The embedded error estimate is a near-cancellation, so
# rounding-level differences (fused multiply-adds, last-ulp differences of
# pow/sin/cos) move the adaptive step times: the oracle itself moves by
# 6.7e-8 in time and 4e-10 x N_group in value when built with FMA contraction.
# The GPU is held to 25x that spread.
GRID_T_TOL = 1e-6      # absolute, days
GRID_Y_TOL = 1e-8      # relative to the age group's population


@pytest.mark.parametrize("name", sorted(GOLDEN_CASES))
def test_simulate_matches_golden(ctx, name):
    c = golden_case(name)
    (t, y), = ctx.simulate(c["model"], [0], c["t0"], c["tmax"], c["dt"], c["opts"])
    exp = c["expected"]
    assert len(t) == exp.shape[0]
    np.testing.assert_allclose(t, exp[:, 0], rtol=0, atol=GRID_T_TOL)
    ys = sum_groups(y, c["G"])
    scale = exp[:, 1:].sum(axis=1, keepdims=True)
    assert np.max(np.abs(ys - exp[:, 1:]) / scale) < GRID_Y_TOL


def test_simulate_matches_oracle_many_nodes(ctx):
    g = W.single_node(seed=7, G=6, count=64)
    res = ctx.simulate(g, np.arange(64), 0.0, 100.0, 0.1, max_points=2048)
    for v in range(0, 64, 9):
        t_ref, y_ref, _ = O.simulate(g, v, 0.0, 100.0, 0.1)
        t, y = res[v]
        assert len(t) == len(t_ref)
        np.testing.assert_allclose(t, t_ref, rtol=0, atol=GRID_T_TOL)
        assert group_scaled_error(y, y_ref, 6) < GRID_Y_TOL


def test_eval_rhs_matches_oracle(ctx):
    rng = np.random.default_rng(11)
    g = W.single_node(seed=8, G=6, count=16, stress=True)
    nodes = np.arange(16)
    pop = g.init_state * rng.uniform(0.5, 1.5, g.init_state.shape) + rng.uniform(0, 50, g.init_state.shape)
    y = pop * rng.uniform(0.5, 1.0, pop.shape)
    t = rng.uniform(0, 40, 16)
    out = ctx.eval_rhs(g, nodes, pop, y, t)
    for v in nodes:
        ref = O.eval_rhs(g, v, pop[v], y[v], t[v])
        np.testing.assert_allclose(out[v], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def run_graph(ctx, g, precision, days, record=True):
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=precision))
    rec = []
    t = 0.0
    while t < days - 1e-12:
        t += 0.5
        b.advance(t)
        if record:
            rec.append(b.states()[0].copy())
    st = b.stats()
    fin = b.states()[0].copy()
    b.close()
    return (np.array(rec) if record else None), fin, st


@pytest.mark.parametrize("precision", PRECISIONS)
def test_graph_matches_oracle_every_boundary(ctx, precision):
    g = W.mobility_graph(seed=21, N=40, out_degree=8)
    rec_ref, fin_ref, st_ref = O.graph_run(g, 0.0, 10.0)
    rec, fin, st = run_graph(ctx, g, precision, 10.0)
    assert rec.shape == rec_ref.shape
    err = max(group_scaled_error(rec[b], rec_ref[b], g.num_groups) for b in range(rec.shape[0]))
    assert err < TOL[precision], err
    if precision != N.PRECISION_MIXED:
        assert st["accepted_steps"] == st_ref["accepted_steps"]


@pytest.mark.parametrize("precision", PRECISIONS)
def test_graph_all_compartments_mobile(ctx, precision):
    # coefficients on every compartment (not only S, E, INS, ISy, R): the exchange
    # kernels' general compartment mask
    g0 = W.mobility_graph(seed=23, N=30, out_degree=6)
    rng = np.random.default_rng(5)
    coeff = g0.edge_coeff_baseline.copy()
    coeff[coeff == 0.0] = rng.uniform(0.001, 0.02, int((coeff == 0.0).sum()))
    g = L.GraphArrays(g0.num_groups, g0.params, g0.contact_baseline, g0.contact_minimum, g0.damping_times,
                      g0.damping_values, g0.init_state, g0.edge_src, g0.edge_dst, coeff)
    rec_ref, _, _ = O.graph_run(g, 0.0, 6.0)
    rec, _, _ = run_graph(ctx, g, precision, 6.0)
    err = max(group_scaled_error(rec[b], rec_ref[b], g.num_groups) for b in range(rec.shape[0]))
    assert err < TOL[precision], err


@pytest.mark.parametrize("precision", PRECISIONS)
def test_graph_with_underflow_fixes(ctx, precision):
    # stress variant (finite test-and-trace / ICU capacities): the reference's
    # return underflow fix fires; the sequential exact pass must reproduce it
    g = W.mobility_graph(seed=1, N=120, out_degree=30, stress=True)
    _, fin_ref, st_ref = O.graph_run(g, 0.0, 30.0, record=False)
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=precision))
    b.advance(30.0)
    fin = b.states()[0]
    st = b.stats()
    assert group_scaled_error(fin, fin_ref, g.num_groups) < TOL[precision]
    assert st_ref["underflow_fixes"] > 0
    if precision != N.PRECISION_MIXED:
        assert st["underflow_fixes"] == st_ref["underflow_fixes"]


def test_late_epidemic_fixes_take_parallel_exact_path(ctx):
    # late in the epidemic most returns need the underflow fix; the per-node
    # exact scans must reproduce the serial loop (same fixes, same states)
    # without falling back to the per-graph sequential pass
    g = W.mobility_graph(seed=1, N=80, out_degree=20)
    _, fin_ref, st_ref = O.graph_run(g, 0.0, 90.0, record=False)
    assert st_ref["underflow_fixes"] > 20
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64))
    b.advance(90.0)
    st = b.stats()
    assert group_scaled_error(b.states()[0], fin_ref, g.num_groups) < 1e-10
    assert st["underflow_fixes"] == st_ref["underflow_fixes"]
    assert st["sequential_exchanges"] <= 2


@pytest.mark.parametrize("precision", [N.PRECISION_FP64, N.PRECISION_MIXED])
def test_ensemble_matches_oracle(ctx, precision):
    ens = W.ensemble(num_samples=12, N=30, out_degree=6)
    b = N.Batch(ctx, ens, 0.0, N.solver_opts(precision=precision))
    b.advance(20.0)
    got = b.states()
    ref, _, _ = O.ensemble_run(ens, 0.0, 20.0, num_threads=4)
    for gs, rs in zip(got, ref):
        assert group_scaled_error(gs, rs, 6) < TOL[precision]


@pytest.mark.parametrize("precision", PRECISIONS)
def test_edge_cases_in_one_batch(ctx, precision):
    # the largest age-group count, a single node without edges, a graph without
    # edges and a stressed graph (finite capacities) side by side in one batch
    graphs = [W.mobility_graph(seed=61, N=12, G=8, out_degree=3),
              W.single_node(seed=62, G=2, count=1),
              W.single_node(seed=63, G=5, count=4),
              W.mobility_graph(seed=64, N=9, G=3, out_degree=8, stress=True)]
    horizons = np.array([7.0, 3.0, 4.5, 6.0])
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=precision))
    b.advance(0.0, horizons)
    np.testing.assert_allclose(b.times(), horizons, rtol=0, atol=1e-12)
    got = b.states()
    for g, h, gs in zip(graphs, horizons, got):
        _, fin, _ = O.graph_run(g, 0.0, float(h), record=False)
        assert group_scaled_error(gs, fin, g.num_groups) < TOL[precision]
    b.close()


@pytest.mark.parametrize("precision", [N.PRECISION_FP64, N.PRECISION_MIXED])
def test_uneven_batch_matches_oracle(ctx, precision):
    graphs, horizons = W.uneven_batch(num_graphs=24, seed=5, max_nodes=60, max_degree=10, horizon=(2.0, 12.0))
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=precision))
    b.advance(0.0, horizons)
    got = b.states()
    np.testing.assert_allclose(b.times(), horizons, rtol=0, atol=1e-12)
    for g, h, gs in zip(graphs, horizons, got):
        _, fin, _ = O.graph_run(g, 0.0, float(h), record=False)
        assert group_scaled_error(gs, fin, g.num_groups) < TOL[precision]


def test_mixed_conservation_and_monotone(ctx):
    g = W.mobility_graph(seed=31, N=200, out_degree=30)
    rec, fin, st = run_graph(ctx, g, N.PRECISION_MIXED, 30.0)
    homes = g.init_state.sum(axis=1)
    after_return = rec[1::2].sum(axis=2)
    assert np.max(np.abs(after_return - homes) / homes) < 1e-9
    assert abs(fin.sum() - homes.sum()) / homes.sum() < 1e-9
    y = rec.reshape(rec.shape[0], g.num_nodes, g.num_groups, 10)
    assert np.all(np.diff(y[..., L.D], axis=0) >= 0)
    assert np.all(np.diff(y[..., L.R].sum(axis=1), axis=0) >= -1e-6 * homes.sum())
    assert y.min() >= -1e-6


def test_advance_in_pieces_equals_one_call(ctx):
    g = W.mobility_graph(seed=41, N=20, out_degree=4)
    b1 = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64))
    b1.advance(7.0)
    b2 = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64))
    for t in (1.5, 3.0, 7.0):
        b2.advance(t)
    np.testing.assert_array_equal(b1.states()[0], b2.states()[0])


def test_mixed_split_intervals_match_fp64(ctx):
    # Horizons off the half-day grid clip an interval, so a later return falls in
    # an interval that does not start at its departure (the return-side rates are
    # then taken from the saved post-departure state). Both solvers see the same
    # clipped exchange grid.
    g = W.mobility_graph(seed=43, N=30, out_degree=6)
    finals = []
    for precision in (N.PRECISION_FP64, N.PRECISION_MIXED):
        b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=precision))
        for t in (1.25, 3.0, 4.6, 6.0):
            b.advance(t)
        np.testing.assert_allclose(b.times(), [6.0], rtol=0, atol=1e-12)
        finals.append(b.states()[0].copy())
        b.close()
    assert group_scaled_error(finals[1], finals[0], g.num_groups) < TOL[N.PRECISION_MIXED]


def test_cuda_graph_replay_equals_stream_launches(ctx):
    g = W.mobility_graph(seed=42, N=30, out_degree=5)
    outs = []
    for use_graph in (True, False):
        b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_MIXED, use_cuda_graph=use_graph))
        b.advance(6.0)
        outs.append(b.states()[0].copy())
    np.testing.assert_array_equal(outs[0], outs[1])


def test_error_statuses(ctx):
    g = W.mobility_graph(seed=43, N=10, out_degree=3)
    bad = L.GraphArrays(g.num_groups, g.params, g.contact_baseline, g.contact_minimum, g.damping_times,
                        g.damping_values, g.init_state, g.edge_src, g.edge_dst, g.edge_coeff_baseline)
    bad.edge_dst = bad.edge_dst[::-1].copy()
    with pytest.raises(N.MgpuError) as e:
        N.Batch(ctx, [bad], 0.0, N.solver_opts())
    assert e.value.code == 3  # InvalidValue: edges not sorted
    with pytest.raises(N.MgpuError) as e:
        N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_FP64,
                                              integrator=L.integrator_opts(method=L.METHOD_RKF45)))
    assert e.value.code == 104  # Unsupported
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_MIXED, max_steps_per_interval=1))
    with pytest.raises(N.MgpuError) as e:
        b.advance(2.0)
    assert e.value.code == 103  # StepFailed: step cap, reported without faulting the device
    b.close()
    ctx.set_memory_budget(1 << 16)
    with pytest.raises(N.MgpuError) as e:
        N.Batch(ctx, [g], 0.0, N.solver_opts())
    assert e.value.code == 101  # OutOfMemory from the budget
    ctx.set_memory_budget(0)
