"""GPU parity at the benchmark's own configurations, against the FP64 oracle.

  * the 400-node mobility graph of the benchmark (6 age groups, 30 out-edges
    per node, commuter fractions on S, E, INS, ISy, R) over 90 days, every
    0.5-day boundary recorded (GraphSimulation::advance,
    cpp/memilio/mobility/graph_simulation.h:101-120, with
    MobilityEdge::apply_mobility, metapopulation_mobility_instant.h:544-623);
  * the first 16 samples of the benchmark's 1024-sample ensemble of that
    graph over 90 days (ParameterStudy runs, parameter_studies.h:288-345);
  * an uneven batch with a graph of more than 1000 nodes and horizons up to
    90 days.

Error measure (oracle.compartment_error): per compartment,
|gpu - oracle| / max(|oracle|, floor * N_g) with N_g the population of the
compartment's (node, age group).

Tolerances, stated per solver:
  FP64 batched : <= 1e-10 with floor 1e-9 at every boundary; the same
                 accepted-step and underflow-fix counts as the oracle. (The
                 device contracts multiply-adds, the oracle does not; on
                 compartments far below a person that rounding shows up above
                 1e-10 relative, e.g. 1.02e-10 on a value of 1e-7 persons.)
  mixed        : the integrator's rel tol, 1e-5, with floor 1e-6, for the
                 final states and for 99.9 % of the values at every boundary;
                 every value at every boundary within 1e-4. (The values between
                 1e-5 and 1e-4 are compartments that a return empties almost
                 completely, e.g. 10 persons of ISy less 9.94 returning: the
                 remainder keeps the FP32 right-hand side's ~1e-6 relative
                 rounding of the 10 persons.)
  both         : every node's resident population after a return equals its
                 initial population to 1e-9 relative; Dead monotone per
                 (node, age group).
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import replicas as R
from memilio_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DAYS = 90.0
FLOOR_FP64, TOL_FP64 = 1e-9, 1e-10
FLOOR_MIXED, TOL_MIXED, TOL_MIXED_ANY = 1e-6, 1e-5, 1e-4
PRECISIONS = {"fp64": N.PRECISION_FP64, "mixed": N.PRECISION_MIXED}


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def cfg1():
    """The benchmark's base graph and the oracle's states at every boundary."""
    g = W.mobility_graph(seed=1)
    rec, fin, st = O.graph_run(g, 0.0, DAYS)
    return g, rec, st


def run_recorded(ctx, g, precision, days):
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=precision))
    rec, t = [], 0.0
    while t < days - 1e-12:
        t += 0.5
        b.advance(t)
        rec.append(b.states()[0].copy())
    st = b.stats()
    b.close()
    return np.array(rec), st


def check_invariants(g, rec):
    homes = g.init_state.sum(axis=1)
    after_return = rec[1::2].sum(axis=2)
    assert np.max(np.abs(after_return - homes) / homes) < 1e-9
    y = rec.reshape(rec.shape[0], g.num_nodes, g.num_groups, 10)
    assert np.all(np.diff(y[..., L.D], axis=0) >= 0.0)
    assert y.min() >= -1e-6 * homes.max()


@pytest.mark.parametrize("name", ["fp64", "mixed"])
def test_benchmark_graph_every_boundary(ctx, cfg1, name):
    g, rec_ref, st_ref = cfg1
    rec, st = run_recorded(ctx, g, PRECISIONS[name], DAYS)
    assert rec.shape == rec_ref.shape == (180, 400, 60)
    check_invariants(g, rec)
    assert st_ref["underflow_fixes"] > 0  # the exact return path is exercised
    if name == "fp64":
        err = O.compartment_error(rec, rec_ref, 6, FLOOR_FP64)
        assert err.max() <= TOL_FP64, O.error_summary(err)
        assert st["accepted_steps"] == st_ref["accepted_steps"]
        assert st["underflow_fixes"] == st_ref["underflow_fixes"]
    else:
        err = O.compartment_error(rec, rec_ref, 6, FLOOR_MIXED)
        s = O.error_summary(err)
        assert O.compartment_error(rec[-1], rec_ref[-1], 6, FLOOR_MIXED).max() <= TOL_MIXED, s
        assert s["p999"] <= TOL_MIXED and s["max"] <= TOL_MIXED_ANY, s
        # the FP32 return can decide a borderline underflow fix differently
        assert abs(st["underflow_fixes"] - st_ref["underflow_fixes"]) <= max(2, st_ref["underflow_fixes"] // 100)


@pytest.fixture(scope="module")
def ensemble16():
    """The first 16 samples of the benchmark's ensemble, and their oracle runs."""
    ens = R.ensemble_for_rank(16, 0, base=W.mobility_graph(seed=1))
    fins, _, st = O.ensemble_run(ens, 0.0, DAYS, num_threads=os.cpu_count() or 1)
    return ens, fins, st


@pytest.mark.parametrize("name", ["fp64", "mixed"])
def test_benchmark_ensemble_subsample(ctx, ensemble16, name):
    ens, fins, st_ref = ensemble16
    b = N.Batch(ctx, ens, 0.0, N.solver_opts(precision=PRECISIONS[name]))
    b.advance(DAYS)
    got = b.states()
    st = b.stats()
    b.close()
    assert st_ref["underflow_fixes"] > 0
    floor, tol = (FLOOR_FP64, TOL_FP64) if name == "fp64" else (FLOOR_MIXED, TOL_MIXED)
    errs = [O.compartment_error(a, r, 6, floor) for a, r in zip(got, fins)]
    assert max(float(e.max()) for e in errs) <= tol, O.error_summary(errs)
    homes = ens[0].init_state.sum()
    for a in got:
        assert abs(a.sum() - homes) / homes < 1e-9
    if name == "fp64":
        assert st["underflow_fixes"] == st_ref["underflow_fixes"]
        assert st["accepted_steps"] == st_ref["accepted_steps"]


def test_uneven_batch_with_large_graph(ctx):
    # graphs of the uneven distribution (1-6 age groups, out-degree up to 50)
    # plus one of 1200 nodes; horizons up to 90 days
    graphs, horizons = W.uneven_batch(num_graphs=6, seed=17, max_nodes=300, horizon=(30.0, 90.0))
    graphs = graphs + [W.mobility_graph(seed=73, N=1200, G=4, out_degree=25)]
    horizons = np.append(horizons, 90.0)
    with cf.ThreadPoolExecutor(max_workers=min(len(graphs), os.cpu_count() or 1)) as ex:
        refs = list(ex.map(lambda gh: O.graph_run(gh[0], 0.0, float(gh[1]), record=False)[1],
                           zip(graphs, horizons)))
    for name, floor, tol in (("fp64", FLOOR_FP64, TOL_FP64), ("mixed", FLOOR_MIXED, TOL_MIXED)):
        b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=PRECISIONS[name]))
        b.advance(0.0, horizons)
        np.testing.assert_allclose(b.times(), horizons, rtol=0, atol=1e-12)
        for g, got, ref in zip(graphs, b.states(), refs):
            e = O.compartment_error(got, ref, g.num_groups, floor)
            assert e.max() <= tol, (name, g.num_nodes, O.error_summary(e))
        b.close()
