"""The allocation-free single-node simulate, mgpu_simulate_final_noalloc.

Its final states must equal those of mgpu_simulate on the same nodes, on two
calls in a row (the second one in place), and a call larger than the fixed
work space must be rejected before anything is launched. The file name sorts
last, so in a full run these tests run after every other GPU test of the same
process; they also pass alone.
"""
import numpy as np
import pytest

from memilio_gb300 import _native as N
from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# One kernel body and the same compile flags as mgpu_simulate: the states agree
# to the last bit. Asserted within 1e-13 relative (values >= 1) / absolute.
TOL = 1e-13
OUT_OF_RANGE = 2
SCRATCH_BYTES = 4 * 1024 * 1024


@pytest.fixture(scope="module")
def ctx():
    c = N.Context(0)
    yield c
    c.close()


def _device_inputs(torch, g):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to("cuda")
    K = g.damping_times.shape[2]
    return {
        "params": dev(g.params),
        "contact": dev(np.stack([g.contact_baseline, g.contact_minimum], axis=2)),
        "dtimes": dev(g.damping_times) if K else None,
        "dvals": dev(g.damping_values) if K else None,
        "y0": dev(g.init_state),
    }


def _call(ctx, g, d, count, t0, tmax, dt0, opts, y_out, status):
    ptr = lambda t: None if t is None else t.data_ptr()
    return N.lib().mgpu_simulate_final_noalloc(
        ctx.handle, g.num_groups, g.contact_baseline.shape[1], g.damping_times.shape[2], count,
        ptr(d["params"]), ptr(d["contact"]), ptr(d["dtimes"]), ptr(d["dvals"]), ptr(d["y0"]),
        t0, tmax, dt0, opts, ptr(y_out), ptr(status))


@pytest.mark.parametrize("stress", [False, True])
def test_final_states_equal_simulate_on_two_calls(ctx, stress):
    torch = pytest.importorskip("torch")
    g = W.single_node(seed=23, G=6, count=48, stress=stress)
    count = g.num_nodes
    t0, tmax, dt0 = 0.0, 40.0, 0.1
    opts = L.integrator_opts()
    ref = ctx.simulate(g, np.arange(count), t0, tmax, dt0, opts)
    want = np.stack([y[-1] for _, y in ref])
    d = _device_inputs(torch, g)
    for call in range(2):
        if call == 0:
            y_out = torch.full_like(d["y0"], float("nan"))  # separate output
        else:
            y_out = d["y0"].clone()                         # in place
            d = dict(d, y0=y_out)
        status = torch.full((count,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = _call(ctx, g, d, count, t0, tmax, dt0, opts, y_out, status)
        assert rc == 0, N.STATUS_NAMES.get(rc, rc)
        torch.cuda.synchronize()
        assert (status.cpu().numpy() == 0).all()
        got = y_out.cpu().numpy()
        err = np.abs(got - want) / np.maximum(np.abs(want), 1.0)
        assert err.max() <= TOL, (call, float(err.max()))


def test_oversize_call_is_rejected(ctx):
    torch = pytest.importorskip("torch")
    g = W.single_node(seed=5, G=6, count=1)
    d = _device_inputs(torch, g)
    too_many = SCRATCH_BYTES // (640 * g.num_groups) + 1
    y_out = torch.zeros_like(d["y0"])
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = _call(ctx, g, d, too_many, 0.0, 1.0, 0.1, L.integrator_opts(), y_out, status)
    assert rc == OUT_OF_RANGE
    fits = SCRATCH_BYTES // (640 * g.num_groups)
    assert fits >= 1000  # about 1092 nodes at six age groups


def test_without_dampings_null_arrays(ctx):
    # K = 0: the damping arrays are NULL and the contact matrix is constant
    torch = pytest.importorskip("torch")
    g6 = W.single_node(seed=31, G=6, count=24)
    n_nodes = g6.num_nodes
    g = L.GraphArrays(g6.num_groups, g6.params, g6.contact_baseline, g6.contact_minimum,
                      np.zeros((n_nodes, 1, 0)), np.zeros((n_nodes, 1, 0, 6, 6)), g6.init_state,
                      np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, g6.n)))
    t0, tmax, dt0 = 0.0, 30.0, 0.1
    opts = L.integrator_opts()
    ref = ctx.simulate(g, np.arange(n_nodes), t0, tmax, dt0, opts)
    want = np.stack([y[-1] for _, y in ref])
    d = _device_inputs(torch, g)
    assert d["dtimes"] is None and d["dvals"] is None
    y_out = torch.empty_like(d["y0"])
    status = torch.full((n_nodes,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert _call(ctx, g, d, n_nodes, t0, tmax, dt0, opts, y_out, status) == 0
    torch.cuda.synchronize()
    assert (status.cpu().numpy() == 0).all()
    got = y_out.cpu().numpy()
    assert (np.abs(got - want) / np.maximum(np.abs(want), 1.0)).max() <= TOL


def test_non_finite_state_sets_status_bit(ctx):
    # a NaN in one node's initial state: that node reports bit 1 (non-finite),
    # the others are unaffected. (A NaN error norm is accepted by the controller,
    # so the step size and the clock stay finite and the node still reaches tmax.)
    torch = pytest.importorskip("torch")
    g = W.single_node(seed=37, G=6, count=8)
    count = g.num_nodes
    t0, tmax, dt0 = 0.0, 10.0, 0.1
    opts = L.integrator_opts()
    ref = ctx.simulate(g, np.arange(count), t0, tmax, dt0, opts)
    want = np.stack([y[-1] for _, y in ref])
    d = _device_inputs(torch, g)
    d["y0"][3, 1] = float("nan")
    y_out = torch.empty_like(d["y0"])
    status = torch.full((count,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert _call(ctx, g, d, count, t0, tmax, dt0, opts, y_out, status) == 0
    torch.cuda.synchronize()
    st = status.cpu().numpy()
    assert st[3] & 2
    assert (np.delete(st, 3) == 0).all()
    got = np.delete(y_out.cpu().numpy(), 3, axis=0)
    ok = np.delete(want, 3, axis=0)
    assert (np.abs(got - ok) / np.maximum(np.abs(ok), 1.0)).max() <= TOL
