"""ctypes binding of the CPU oracle (oracle/build/libsecir_oracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg. The product (memilio_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from memilio_gb300.layout import (GraphArrays, MgpuGraph, MgpuIntegratorOpts, integrator_opts,
                                  NUM_COMPARTMENTS, NUM_FLOWS)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "libsecir_oracle.so")
_lib = None


class OrcStats(ctypes.Structure):
    _fields_ = [
        ("accepted_steps", ctypes.c_int64),
        ("rejected_steps", ctypes.c_int64),
        ("rhs_evals", ctypes.c_int64),
        ("underflow_fixes", ctypes.c_int64),
        ("failed_steps", ctypes.c_int64),
    ]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, no other dependency)."""
    src = os.path.join(_HERE, "secir_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER
        d = ctypes.c_double
        L.orc_eval_rhs.argtypes = [P(MgpuGraph), ctypes.c_int, P(d), P(d), d, P(d)]
        L.orc_eval_flows.argtypes = [P(MgpuGraph), ctypes.c_int, P(d), P(d), d, P(d)]
        L.orc_simulate.argtypes = [P(MgpuGraph), ctypes.c_int, d, d, d, P(MgpuIntegratorOpts), ctypes.c_int,
                                   P(d), P(d), P(ctypes.c_int), P(OrcStats)]
        L.orc_simulate_flows.argtypes = [P(MgpuGraph), ctypes.c_int, d, d, d, P(MgpuIntegratorOpts), ctypes.c_int,
                                         P(d), P(d), P(d), P(ctypes.c_int), P(OrcStats)]
        L.orc_graph_run.argtypes = [P(MgpuGraph), d, d, d, d, P(MgpuIntegratorOpts), P(d), P(d), P(OrcStats)]
        L.orc_ensemble_run.argtypes = [P(MgpuGraph), ctypes.c_int, d, d, d, d, P(MgpuIntegratorOpts), ctypes.c_int,
                                       P(d), P(d), P(OrcStats)]
        L.orc_damping_cache.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P(d), P(ctypes.c_int32),
                                        P(ctypes.c_int32), P(d), ctypes.c_int, P(d), P(d)]
        i32p = P(ctypes.c_int32)
        L.orc_graph_run_commuters.argtypes = [P(MgpuGraph), d, d, d, d, P(MgpuIntegratorOpts), ctypes.c_int, i32p,
                                              i32p, ctypes.c_int, P(d), i32p, P(d), P(d), P(OrcStats)]
        L.orc_departure_commuters.argtypes = [P(MgpuGraph), ctypes.c_int, d, ctypes.c_int, i32p, i32p, P(d)]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def eval_rhs(g: GraphArrays, node: int, pop, y, t: float) -> np.ndarray:
    pop = np.ascontiguousarray(pop, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros(g.n)
    cg = g.as_ctypes()
    assert lib().orc_eval_rhs(ctypes.byref(cg), node, _p(pop), _p(y), t, _p(out)) == 0
    return out


def eval_flows(g: GraphArrays, node: int, pop, y, t: float) -> np.ndarray:
    pop = np.ascontiguousarray(pop, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    out = np.zeros(g.num_groups * NUM_FLOWS)
    cg = g.as_ctypes()
    assert lib().orc_eval_flows(ctypes.byref(cg), node, _p(pop), _p(y), t, _p(out)) == 0
    return out


def simulate(g: GraphArrays, node: int, t0: float, tmax: float, dt: float, opts=None, max_points: int = 200000):
    """Single-node simulate(): returns (times [P], values [P, 10G], stats)."""
    opts = opts or integrator_opts()
    out_t = np.zeros(max_points)
    out_y = np.zeros((max_points, g.n))
    npts = ctypes.c_int(0)
    st = OrcStats()
    cg = g.as_ctypes()
    rc = lib().orc_simulate(ctypes.byref(cg), node, t0, tmax, dt, ctypes.byref(opts), max_points, _p(out_t),
                            _p(out_y), ctypes.byref(npts), ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("orc_simulate failed (max_points too small?)")
    return out_t[:npts.value].copy(), out_y[:npts.value].copy(), st.as_dict()


def simulate_flows(g: GraphArrays, node: int, t0: float, tmax: float, dt: float, opts=None,
                   max_points: int = 200000):
    """simulate_flows(): returns (times [P], flows [P, 15G], populations [P, 10G], stats)."""
    opts = opts or integrator_opts()
    nf = 15 * g.num_groups
    out_t = np.zeros(max_points)
    out_f = np.zeros((max_points, nf))
    out_y = np.zeros((max_points, g.n))
    npts = ctypes.c_int(0)
    st = OrcStats()
    cg = g.as_ctypes()
    rc = lib().orc_simulate_flows(ctypes.byref(cg), node, t0, tmax, dt, ctypes.byref(opts), max_points, _p(out_t),
                                  _p(out_f), _p(out_y), ctypes.byref(npts), ctypes.byref(st))
    if rc != 0:
        raise RuntimeError("orc_simulate_flows failed (max_points too small?)")
    k = npts.value
    return out_t[:k].copy(), out_f[:k].copy(), out_y[:k].copy(), st.as_dict()


def num_boundaries(t0: float, tmax: float, dt_exchange: float) -> int:
    t, nb = t0, 0
    while t < tmax:
        dt = dt_exchange if t + dt_exchange <= tmax else tmax - t
        t += dt
        nb += 1
    return nb


def graph_run(g: GraphArrays, t0: float, tmax: float, dt_exchange: float = 0.5, dt0: float = 0.1, opts=None,
              record: bool = True):
    """make_mobility_sim(t0, dt_exchange, graph).advance(tmax).

    Returns (boundary_states [B, N, 10G] or None, final [N, 10G], stats)."""
    opts = opts or integrator_opts()
    nb = num_boundaries(t0, tmax, dt_exchange)
    rec = np.zeros((nb, g.num_nodes, g.n)) if record else None
    fin = np.zeros((g.num_nodes, g.n))
    st = OrcStats()
    cg = g.as_ctypes()
    rc = lib().orc_graph_run(ctypes.byref(cg), t0, tmax, dt_exchange, dt0, ctypes.byref(opts),
                             _p(rec) if record else ctypes.POINTER(ctypes.c_double)(), _p(fin), ctypes.byref(st))
    assert rc == 0
    return rec, fin, st.as_dict()


def ensemble_run(graphs, t0: float, tmax: float, dt_exchange: float = 0.5, dt0: float = 0.1, opts=None,
                 num_threads: int = 0):
    """Independent runs of many graphs over `num_threads` host threads.

    Returns (list of final [N_b, 10G], elapsed seconds, stats)."""
    opts = opts or integrator_opts()
    arr = (MgpuGraph * len(graphs))(*[g.as_ctypes() for g in graphs])
    sizes = [g.num_nodes * g.n for g in graphs]
    out = np.zeros(sum(sizes))
    el = ctypes.c_double(0)
    st = OrcStats()
    rc = lib().orc_ensemble_run(arr, len(graphs), t0, tmax, dt_exchange, dt0, ctypes.byref(opts), num_threads,
                                _p(out), ctypes.byref(el), ctypes.byref(st))
    assert rc == 0
    res, off = [], 0
    for g, s in zip(graphs, sizes):
        res.append(out[off:off + s].reshape(g.num_nodes, g.n))
        off += s
    return res, el.value, st.as_dict()


def _sets(save_sets):
    """CSR form (offsets, indices) of a list of index sets."""
    offsets = np.zeros(len(save_sets) + 1, np.int32)
    for i, st in enumerate(save_sets):
        offsets[i + 1] = offsets[i] + len(st)
    indices = np.ascontiguousarray(np.concatenate([np.asarray(st, np.int32) for st in save_sets])
                                   if save_sets else np.zeros(0, np.int32), np.int32)
    return offsets, indices


def graph_run_commuters(g: GraphArrays, t0: float, tmax: float, save_sets, capacity: int = 1024,
                        dt_exchange: float = 0.5, dt0: float = 0.1, opts=None):
    """graph_run recording every edge's mobility results with the given save
    indices (MobilityEdge::add_mobility_result_time_point). Returns (final
    [N, 10G], counts [E], times [E, capacity], values [E, capacity, sets + 1], stats)."""
    L = lib()
    i32p = ctypes.POINTER(ctypes.c_int32)
    opts = opts or integrator_opts()
    offsets, indices = _sets(save_sets)
    S, E = len(save_sets), g.num_edges
    fin = np.zeros((g.num_nodes, g.n))
    counts = np.zeros(max(E, 1), np.int32)
    times = np.zeros((max(E, 1), capacity))
    values = np.zeros((max(E, 1), capacity, S + 1))
    st = OrcStats()
    cg = g.as_ctypes()
    rc = L.orc_graph_run_commuters(ctypes.byref(cg), t0, tmax, dt_exchange, dt0, ctypes.byref(opts), S,
                                   offsets.ctypes.data_as(i32p), indices.ctypes.data_as(i32p), capacity, _p(fin),
                                   counts.ctypes.data_as(i32p), _p(times), _p(values), ctypes.byref(st))
    assert rc == 0
    return fin, counts[:E], times[:E], values[:E], st.as_dict()


def departure_commuters(g: GraphArrays, edge: int, t: float, save_sets) -> np.ndarray:
    """One apply_mobility(t, 0, from, to) of `edge` on the initial states: the
    mobility result it records [sets + 1]."""
    offsets, indices = _sets(save_sets)
    out = np.zeros(len(save_sets) + 1)
    i32p = ctypes.POINTER(ctypes.c_int32)
    cg = g.as_ctypes()
    rc = lib().orc_departure_commuters(ctypes.byref(cg), edge, t, len(save_sets), offsets.ctypes.data_as(i32p),
                                       indices.ctypes.data_as(i32p), _p(out))
    assert rc == 0
    return out


def compartment_error(got, ref, num_groups: int, floor: float = 1e-6) -> np.ndarray:
    """Per-compartment relative error of `got` against the oracle's `ref`:

        |got - ref| / max(|ref|, floor * N_g)

    N_g is the population of the (node, age group) the compartment belongs to
    (the sum of its ten compartments in `ref`), so `floor` is the absolute
    floor as a fraction of the age group. Arrays of any leading shape with
    10 * num_groups values last; the result has shape [..., num_groups, 10]."""
    got = np.asarray(got, np.float64).reshape(-1, num_groups, NUM_COMPARTMENTS)
    ref = np.asarray(ref, np.float64).reshape(-1, num_groups, NUM_COMPARTMENTS)
    n_g = ref.sum(axis=2, keepdims=True)
    den = np.maximum(np.abs(ref), floor * n_g)
    den = np.where(den > 0.0, den, 1.0)  # an empty age group: absolute error
    return np.abs(got - ref) / den


def error_summary(errs) -> dict:
    """max, p99 and p99.9 of compartment_error arrays (one or a list)."""
    e = np.concatenate([np.ravel(x) for x in (errs if isinstance(errs, (list, tuple)) else [errs])])
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)), "p999": float(np.percentile(e, 99.9)),
            "values": int(e.size)}


def damping_cache(rows, cols, times, levels, types, matrices, cap=64):
    times = np.ascontiguousarray(times, np.float64)
    levels = np.ascontiguousarray(levels, np.int32)
    types = np.ascontiguousarray(types, np.int32)
    matrices = np.ascontiguousarray(matrices, np.float64)
    out_t = np.zeros(cap)
    out_m = np.zeros((cap, rows, cols))
    k = lib().orc_damping_cache(rows, cols, len(times), _p(times),
                                levels.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                types.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _p(matrices), cap,
                                _p(out_t), _p(out_m))
    assert k > 0
    return out_t[:k].copy(), out_m[:k].copy()


class OrcNpiSampling(ctypes.Structure):
    _fields_ = [("value", ctypes.c_double), ("level", ctypes.c_int32), ("type", ctypes.c_int32),
                ("num_matrices", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("matrices", ctypes.POINTER(ctypes.c_int32)), ("group_weights", ctypes.POINTER(ctypes.c_double))]


class OrcDynamicNpis(ctypes.Structure):
    _fields_ = [("num_thresholds", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("thresholds", ctypes.POINTER(ctypes.c_double)), ("first", ctypes.POINTER(ctypes.c_int32)),
                ("samplings", ctypes.POINTER(OrcNpiSampling)), ("duration", ctypes.c_double),
                ("delay", ctypes.c_double), ("base_value", ctypes.c_double), ("directive_begin", ctypes.c_double),
                ("directive_end", ctypes.c_double)]


class OrcDamping(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("level", ctypes.c_int32), ("type", ctypes.c_int32),
                ("matrix", ctypes.c_int32), ("pad", ctypes.c_int32), ("coeffs", ctypes.POINTER(ctypes.c_double))]


def _dynamic_npis(npis: dict, keep: list):
    """OrcDynamicNpis of an NPI dict; the arrays it points to are appended to keep."""
    samp, first, thr = [], [0], []
    for threshold, items in npis["thresholds"]:
        thr.append(threshold)
        for value, level, typ, mats, weights in items:
            m = np.ascontiguousarray(mats, np.int32)
            w = np.ascontiguousarray(weights, np.float64)
            keep += [m, w]
            samp.append(OrcNpiSampling(value, level, typ, len(m), 0, m.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                       _p(w)))
        first.append(len(samp))
    thr_a = np.ascontiguousarray(thr, np.float64)
    first_a = np.ascontiguousarray(first, np.int32)
    samp_a = (OrcNpiSampling * max(len(samp), 1))(*samp)
    keep += [thr_a, first_a, samp_a]
    return OrcDynamicNpis(len(thr), 0, _p(thr_a), first_a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), samp_a,
                          npis.get("duration", 14.0), npis.get("delay", 0.0), npis.get("base_value", 1.0),
                          npis.get("directive_begin", np.finfo(np.float64).min),
                          npis.get("directive_end", np.finfo(np.float64).max))


def graph_run_npi(g: GraphArrays, t0: float, tmax: float, npis: dict, dampings, dt_exchange: float = 0.5,
                  dt0: float = 0.1, opts=None, edge_npis: dict = None):
    """make_mobility_sim(...).advance(tmax) with the same dynamic NPIs on every node.

    npis: {"thresholds": [(threshold, [(value, level, type, [matrices], [group weights]), ...]), ...],
           "duration", "delay", "base_value", "directive_begin", "directive_end"};
    dampings: the nodes' initial contact dampings [(time, level, type, matrix, G x G coefficients), ...];
    edge_npis: the same NPIs on every edge (MobilityParameters::get_dynamic_npis_infected; the
    matrices of a sampling are ignored), or None. Returns (final [N, 10G], enactments per node [N],
    stats), and with edge_npis also the enactments per edge [E] after the node counts."""
    L = lib()
    if not hasattr(L.orc_graph_run_npi, "_typed"):
        P = ctypes.POINTER
        d = ctypes.c_double
        L.orc_graph_run_npi.argtypes = [P(MgpuGraph), d, d, d, d, P(MgpuIntegratorOpts), P(OrcDynamicNpis),
                                        ctypes.c_int, P(OrcDamping), P(OrcDynamicNpis), P(d), P(ctypes.c_int32),
                                        P(ctypes.c_int32), P(OrcStats)]
        L.orc_graph_run_npi._typed = True
    opts = opts or integrator_opts()
    keep = []
    p = _dynamic_npis(npis, keep)
    ep = _dynamic_npis(edge_npis, keep) if edge_npis is not None else None
    damp = []
    for time, level, typ, mat, coeffs in dampings:
        c = np.ascontiguousarray(coeffs, np.float64)
        keep.append(c)
        damp.append(OrcDamping(time, level, typ, mat, 0, _p(c)))
    damp_a = (OrcDamping * max(len(damp), 1))(*damp)
    fin = np.zeros((g.num_nodes, g.n))
    cnt = np.zeros(g.num_nodes, np.int32)
    ecnt = np.zeros(max(g.num_edges, 1), np.int32)
    st = OrcStats()
    cg = g.as_ctypes()
    rc = L.orc_graph_run_npi(ctypes.byref(cg), t0, tmax, dt_exchange, dt0, ctypes.byref(opts), ctypes.byref(p),
                             len(damp), damp_a, ctypes.byref(ep) if ep is not None else None, _p(fin),
                             cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                             ecnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(st))
    assert rc == 0
    if edge_npis is not None:
        return fin, cnt, ecnt[:g.num_edges], st.as_dict()
    return fin, cnt, st.as_dict()
