"""Continuous batching (mgpu_server_*) and the asynchronous batch advance it is
built on (mgpu_batch_launch / mgpu_batch_query).

The central property: a request's result is the same whether it is solved
alone or inside the server's mix of overlapping batches. The batched solver
treats every graph independently (per-graph interval clock, per-graph exchange
and underflow handling), so the results are expected to agree to the last
bit; the assertions allow 1e-12 relative to the age group's population.
Against the FP64 oracle the mixed solver's tolerance (1e-5) applies.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIX_TOL = 1e-12
ORACLE_TOL = 1e-5


def scaled_error(a, b, G):
    a = np.asarray(a).reshape(-1, G, 10)
    b = np.asarray(b).reshape(-1, G, 10)
    scale = np.maximum(b.sum(axis=2, keepdims=True), 1.0)
    return float(np.max(np.abs(a - b) / scale))


@pytest.fixture(scope="module")
def ctx():
    c = N.Context(0)
    yield c
    c.close()


def requests(n=24, seed=41):
    return W.uneven_batch(num_graphs=n, seed=seed, max_nodes=80, max_degree=12, horizon=(2.0, 14.0))


def alone(ctx, g, tmax):
    b = N.Batch(ctx, [g], 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    b.advance(float(tmax))
    out = b.graph_state(0)
    b.close()
    return out


def test_async_launch_matches_advance(ctx):
    graphs, horizons = requests(8, seed=43)
    ref = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    ref.advance(0.0, horizons)
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    import ctypes
    rem, done = ctypes.c_int32(), ctypes.c_int32()
    tpg = np.ascontiguousarray(horizons)
    ctx.check(N.lib().mgpu_batch_launch(b._h, 0.0, N._dp(tpg), 3, ctypes.byref(rem)))
    launches = 1
    while True:
        ctx.check(N.lib().mgpu_batch_query(b._h, ctypes.byref(done)))
        if not done.value:
            continue
        if rem.value == 0:
            break
        ctx.check(N.lib().mgpu_batch_launch(b._h, 0.0, N._dp(tpg), 3, ctypes.byref(rem)))
        launches += 1
    assert launches > 1
    np.testing.assert_allclose(b.times(), horizons, rtol=0, atol=1e-12)
    assert np.array_equal(b.state_flat(), ref.state_flat())
    for i, g in enumerate(graphs):
        assert np.array_equal(b.graph_state(i).ravel(), ref.states()[i].ravel())


def test_server_results_equal_alone_and_overlap(ctx):
    graphs, horizons = requests(24)
    # immediate admission, so that every wave becomes its own batch
    srv = N.Server(0, N.server_opts(max_batches=8, phases_per_launch=2, min_batch_graphs=1, max_wait_ms=0.0))
    ids, results, max_batches = {}, {}, 0
    # three waves: later requests arrive while earlier ones are on the device
    waves = [range(0, 8), range(8, 16), range(16, 24)]
    for w, wave in enumerate(waves):
        for i in wave:
            ids[srv.submit(graphs[i], 0.0, horizons[i])] = i
        for _ in range(3):
            srv.step()
            max_batches = max(max_batches, srv.num_batches())
    for _ in range(200000):
        srv.step()
        max_batches = max(max_batches, srv.num_batches())
        while True:
            t = srv.take()
            if t is None:
                break
            rid, state, lat = t
            results[ids[rid]] = state
            assert lat >= 0.0
        if len(results) == len(graphs):
            break
    assert len(results) == len(graphs)
    assert max_batches >= 2, "batches admitted at different times should overlap"
    assert srv.memory_in_use() == 0 and srv.num_batches() == 0
    srv.close()
    for i, g in enumerate(graphs):
        ref = alone(ctx, g, horizons[i])
        assert scaled_error(results[i], ref, g.num_groups) <= MIX_TOL, i
    for i in (0, 9, 23):
        _, fin, _ = O.graph_run(graphs[i], 0.0, float(horizons[i]), record=False)
        assert scaled_error(results[i], fin, graphs[i].num_groups) < ORACLE_TOL


def test_server_admission_waits_for_memory(ctx):
    graphs, horizons = requests(6, seed=47)
    one = max(int(N.lib().mgpu_batch_estimate_bytes(g.as_ctypes(), 1,
                                                    N.solver_opts(precision=N.PRECISION_MIXED))) for g in graphs)
    # room for about one request at a time
    srv = N.Server(0, N.server_opts(memory_budget=int(one * 1.5), max_batches=8))
    for g, h in zip(graphs, horizons):
        srv.submit(g, 0.0, h)
    waited, done = False, 0
    for _ in range(200000):
        _, _, queued = srv.step()
        waited = waited or queued > 0
        assert srv.memory_in_use() <= int(one * 1.5)
        while srv.take() is not None:
            done += 1
        if done == len(graphs):
            break
    assert done == len(graphs) and waited
    srv.close()


def test_server_rejects_request_larger_than_budget(ctx):
    graphs, horizons = requests(1, seed=49)
    srv = N.Server(0, N.server_opts(memory_budget=1024))
    with pytest.raises(N.MgpuError):
        srv.submit(graphs[0], 0.0, horizons[0])
    srv.close()


def test_autotuned_schedule_gives_identical_results(ctx):
    # the schedule only changes which lanes and blocks integrate an instance
    graphs, horizons = requests(12, seed=53)
    a = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    a.advance(0.0, horizons)
    b = N.Batch(ctx, graphs, 0.0, N.solver_opts(precision=N.PRECISION_MIXED))
    tune = b.autotune()
    assert tune["instances_per_block"] > 0
    b.advance(0.0, horizons)
    assert np.array_equal(a.state_flat(), b.state_flat())
    a.close()
    b.close()


def test_server_waits_to_batch_requests_while_busy(ctx):
    # with a batch running, later requests wait for min_batch_graphs or max_wait_ms
    graphs, horizons = requests(10, seed=57)
    srv = N.Server(0, N.server_opts(min_batch_graphs=4, max_wait_ms=1e6))
    srv.submit(graphs[0], 0.0, 60.0)  # a long first request keeps the device busy
    srv.step()
    assert srv.num_batches() == 1
    for i in range(1, 4):
        srv.submit(graphs[i], 0.0, horizons[i])
        srv.step()
        assert srv.num_batches() == 1  # fewer than 4 waiting: no new batch yet
    srv.submit(graphs[4], 0.0, horizons[4])
    srv.step()
    assert srv.num_batches() == 2  # 4 waiting: admitted together
    done = 0
    for _ in range(500000):
        srv.step()
        while srv.take() is not None:
            done += 1
        if done == 5:
            break
    assert done == 5
    srv.close()


@pytest.mark.parametrize("rebatch", [16, 0])
def test_rebatching_merges_running_batches(ctx, rebatch):
    # two waves fill the server's two batch slots while a third waits; once both
    # batches stand between intervals (no travelers away after each pair of
    # intervals) the server merges them into one (mgpu_batch_regroup), which
    # frees a slot for the third wave, and every request still ends exactly as
    # when solved alone
    import time
    graphs, horizons = requests(10, seed=61)
    horizons = np.maximum(horizons, 6.0)
    srv = N.Server(0, N.server_opts(max_batches=2, rebatch_max_graphs=rebatch))
    ids, results = {}, {}
    for i in range(4):
        ids[srv.submit(graphs[i], 0.0, horizons[i])] = i
    srv.step()
    for i in range(4, 8):
        ids[srv.submit(graphs[i], 0.0, horizons[i])] = i
    srv.step()
    assert srv.num_batches() == 2
    for i in range(8, 10):
        ids[srv.submit(graphs[i], 0.0, horizons[i])] = i
    time.sleep(0.3)  # both batches finish the intervals they were given
    _, _, queued = srv.step()
    if rebatch:
        assert srv.num_merges() == 1 and queued == 0 and srv.num_batches() == 2
    else:
        assert srv.num_merges() == 0 and queued == 2
    for _ in range(200000):
        srv.step()
        while True:
            t = srv.take()
            if t is None:
                break
            results[ids[t[0]]] = t[1]
        if len(results) == len(graphs):
            break
    assert srv.memory_in_use() == 0
    srv.close()
    for i, g in enumerate(graphs):
        np.testing.assert_array_equal(results[i], alone(ctx, g, horizons[i]))
