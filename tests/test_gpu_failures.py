"""Failure isolation between the graphs of a batch and the requests of a server.

In the reference every ParameterStudy run is an independent simulation
(cpp/memilio/compartments/parameter_studies.h:288-345) and a failed adaptive
step logs and continues (cpp/memilio/math/integrator.h:236-246). Here a graph
whose node solves hit the step cap or end an interval with a non-finite state
is flagged on its own (mgpu_batch_get_failed); the advance reports
MGPU_STEP_FAILED, and every other graph of the batch (every other request of
the server) completes with the states it has when solved alone, bit for bit.

The failing graphs are made on the host: stay times of 1e-4 days (rates of
1e4 per day need thousands of explicit steps per 0.5-day interval, above a cap
of 100), or a NaN in one initial state. Neither can make a kernel fault or
hang: the step loops are counted, a NaN error norm is accepted by the
controller (the clock stays finite), and no index is computed from a state
value.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CAP = 100  # steps per node and interval; the normal graphs need a handful
DAYS = 3.0
ALL = [N.PRECISION_FP64_PLAIN, N.PRECISION_FP64, N.PRECISION_MIXED, N.PRECISION_MIXED_FP64_CONTROL]


@pytest.fixture(scope="module")
def ctx():
    from memilio_gb300 import build as B
    B.build()
    c = N.Context(0)
    yield c
    c.close()


def with_params(g, P=None, y0=None):
    return L.GraphArrays(g.num_groups, g.params if P is None else P, g.contact_baseline, g.contact_minimum,
                         g.damping_times, g.damping_values, g.init_state if y0 is None else y0, g.edge_src,
                         g.edge_dst, g.edge_coeff_baseline)


def stiff(g):
    P = g.params.copy()
    for k in (L.G_TIME_EXPOSED, L.G_TIME_INS, L.G_TIME_ISY, L.G_TIME_ISEV, L.G_TIME_ICRI):
        i = L.group_param_index(k, 0, g.num_groups)
        P[:, i:i + g.num_groups] = 1e-4
    return with_params(g, P=P)


def with_nan(g):
    y = g.init_state.copy()
    y[1, 2] = np.nan
    return with_params(g, y0=y)


def normal_graphs():
    return W.mobility_graph(seed=81, N=10, G=3, out_degree=3), W.mobility_graph(seed=82, N=7, G=2, out_degree=2)


def solo(ctx, g, opts):
    b = N.Batch(ctx, [g], 0.0, opts)
    b.advance(DAYS)
    out = b.states()[0].copy()
    b.close()
    return out


@pytest.mark.parametrize("precision", ALL)
@pytest.mark.parametrize("kind", ["step_cap", "nonfinite"])
def test_failed_graph_leaves_the_others_intact(ctx, precision, kind):
    a, c = normal_graphs()
    bad = stiff(W.mobility_graph(seed=83, N=6, G=2, out_degree=2)) if kind == "step_cap" else \
        with_nan(W.mobility_graph(seed=84, N=6, G=2, out_degree=2))
    flag = N.FAILED_STEP_CAP if kind == "step_cap" else N.FAILED_NONFINITE
    opts = N.solver_opts(precision=precision, max_steps_per_interval=CAP)
    b = N.Batch(ctx, [a, bad, c], 0.0, opts)
    with pytest.raises(N.MgpuError) as e:
        b.advance(DAYS)
    assert e.value.code == 103  # StepFailed
    assert " 1 (" in str(e.value)  # the message names graph 1
    f = b.failed()
    assert f[0] == 0 and f[2] == 0 and (f[1] & flag)
    np.testing.assert_allclose(b.times(), [DAYS] * 3, rtol=0, atol=1e-12)
    got = b.states()
    np.testing.assert_array_equal(got[0], solo(ctx, a, opts))
    np.testing.assert_array_equal(got[2], solo(ctx, c, opts))
    # a restart clears the flags
    b.reset(0.0)
    assert not b.failed().any()
    b.close()


def test_server_delivers_each_requests_own_status(ctx):
    a, c = normal_graphs()
    bad = stiff(W.mobility_graph(seed=83, N=6, G=2, out_degree=2))
    srv = N.Server(0, N.server_opts(precision=N.PRECISION_MIXED, max_steps_per_interval=CAP))
    ids = {srv.submit(g, 0.0, DAYS): name for name, g in (("a", a), ("bad", bad), ("c", c))}
    results, failed = {}, {}
    for _ in range(100000):
        srv.step()
        while True:
            try:
                t = srv.take()
            except N.MgpuError as e:
                failed[e.args[0]] = e.code
                continue
            if t is None:
                break
            results[ids[t[0]]] = t[1]
        if len(results) + len(failed) == 3:
            break
    srv.close()
    assert sorted(results) == ["a", "c"]
    assert list(failed.values()) == [103]
    opts = N.solver_opts(precision=N.PRECISION_MIXED, max_steps_per_interval=CAP)
    np.testing.assert_array_equal(results["a"], solo(ctx, a, opts))
    np.testing.assert_array_equal(results["c"], solo(ctx, c, opts))


def test_batch_destroyed_after_its_context():
    # a caller (e.g. a garbage-collected wrapper) may destroy a batch after its
    # context: mgpu_destroy releases the context's remaining batches, and a later
    # mgpu_batch_destroy of such a handle, or a second one, does nothing
    import ctypes
    L_ = N.lib()
    h_ctx, h_b = ctypes.c_void_p(), ctypes.c_void_p()
    assert L_.mgpu_create(0, ctypes.byref(h_ctx)) == 0
    g = W.mobility_graph(seed=85, N=5, G=2, out_degree=2)
    arr = L.graphs_as_ctypes([g])
    opts = N.solver_opts()
    assert L_.mgpu_batch_create(h_ctx, arr, 1, 0.0, ctypes.byref(opts), ctypes.byref(h_b)) == 0
    assert L_.mgpu_batch_advance(h_b, 1.0, ctypes.POINTER(ctypes.c_double)()) == 0
    L_.mgpu_destroy(h_ctx)
    L_.mgpu_batch_destroy(h_b)
    L_.mgpu_batch_destroy(h_b)
    # the Python wrapper closes its batches with the context
    ctx2 = N.Context(0)
    b = N.Batch(ctx2, [g], 0.0, opts)
    ctx2.close()
    assert not b._h
    b.close()
