"""ctypes binding of libmiogpu (include/miogpu.h).

The library must be built (memilio_gb300.build.build()); loading fails
loudly otherwise — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from typing import Optional, Sequence

import numpy as np

from .layout import GraphArrays, MgpuGraph, MgpuIntegratorOpts, graphs_as_ctypes, integrator_opts

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("MIOGPU_LIB") or os.path.join(HERE, "lib", "libmiogpu.so")

OK = 0
STATUS_NAMES = {0: "OK", 1: "UnknownError", 2: "OutOfRange", 3: "InvalidValue", 4: "InvalidFileFormat",
                5: "KeyNotFound", 6: "InvalidType", 7: "FileNotFound", 100: "CudaError", 101: "OutOfMemory",
                102: "Timeout", 103: "StepFailed", 104: "Unsupported"}

PRECISION_FP64_PLAIN = 0
PRECISION_FP64 = 1
PRECISION_MIXED = 2
PRECISION_MIXED_FP64_CONTROL = 3
FAILED_STEP_CAP = 1
FAILED_NONFINITE = 2

# every entry point declared in include/miogpu.h
EXPORTED = ["mgpu_default_solver_opts", "mgpu_create", "mgpu_destroy", "mgpu_last_error", "mgpu_set_memory_budget",
            "mgpu_eval_rhs", "mgpu_simulate", "mgpu_batch_create", "mgpu_batch_advance", "mgpu_batch_get_state",
            "mgpu_batch_get_time", "mgpu_batch_set_state", "mgpu_batch_set_damping_cache", "mgpu_batch_set_edge_damping_cache",
            "mgpu_batch_step_nodes", "mgpu_batch_step_exchange", "mgpu_batch_get_compartment_sums", "mgpu_batch_get_stats", "mgpu_batch_get_timing",
            "mgpu_batch_device_bytes", "mgpu_batch_reset", "mgpu_batch_destroy", "mgpu_simulate_final_noalloc",
            "mgpu_batch_launch", "mgpu_batch_query", "mgpu_batch_get_failed", "mgpu_batch_set_commuter_stats",
            "mgpu_batch_get_commuter_stats",
            "mgpu_batch_set_flow_recording", "mgpu_batch_get_flows", "mgpu_batch_regroup", "mgpu_batch_autotune", "mgpu_simulate_dt", "mgpu_simulate_flows", "mgpu_batch_ensemble_stats", "mgpu_batch_get_graph_state", "mgpu_batch_estimate_bytes",
            "mgpu_default_server_opts", "mgpu_server_create", "mgpu_server_destroy", "mgpu_server_submit",
            "mgpu_server_step", "mgpu_server_take", "mgpu_server_memory_in_use", "mgpu_server_num_batches", "mgpu_server_num_merges"]


class MgpuSolverOpts(ctypes.Structure):
    _fields_ = [
        ("integrator", MgpuIntegratorOpts),
        ("dt0", ctypes.c_double),
        ("dt_exchange", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("instances_per_block", ctypes.c_int32),
        ("max_steps_per_interval", ctypes.c_int32),
        ("use_cuda_graph", ctypes.c_int32),
        ("profile", ctypes.c_int32),
        ("staged_exchange", ctypes.c_int32),
    ]


class MgpuServerOpts(ctypes.Structure):
    _fields_ = [
        ("solver", MgpuSolverOpts),
        ("memory_budget", ctypes.c_int64),
        ("max_batches", ctypes.c_int32),
        ("phases_per_launch", ctypes.c_int32),
        ("max_graphs_per_batch", ctypes.c_int32),
        ("min_batch_graphs", ctypes.c_int32),
        ("max_wait_ms", ctypes.c_double),
        ("rebatch_max_graphs", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class MgpuTiming(ctypes.Structure):
    _fields_ = [
        ("advance_ms", ctypes.c_double),
        ("ode_ms", ctypes.c_double),
        ("exchange_ms", ctypes.c_double),
        ("ode_launches", ctypes.c_int64),
        ("attempts", ctypes.c_int64),
        ("prep_ms", ctypes.c_double),
        ("return_ms", ctypes.c_double),
        ("exact_ms", ctypes.c_double),
        ("depart_ms", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: (float(getattr(self, k)) if k.endswith("ms") else int(getattr(self, k))) for k, _ in self._fields_}


class MgpuStats(ctypes.Structure):
    _fields_ = [
        ("accepted_steps", ctypes.c_int64),
        ("rejected_steps", ctypes.c_int64),
        ("failed_steps", ctypes.c_int64),
        ("underflow_fixes", ctypes.c_int64),
        ("sequential_exchanges", ctypes.c_int64),
        ("phases", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("scan_items", ctypes.c_int64),
    ]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class MgpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)} ({code}): {msg}")
        self.code = code


_lib = None


def lib():
    """Load libmiogpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} not built: run memilio_gb300.build.build() (needs nvcc)")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    d = ctypes.c_double
    vp = ctypes.c_void_p
    L.mgpu_default_solver_opts.argtypes = [P(MgpuSolverOpts)]
    L.mgpu_default_solver_opts.restype = None
    L.mgpu_create.argtypes = [ctypes.c_int, P(vp)]
    L.mgpu_destroy.argtypes = [vp]
    L.mgpu_destroy.restype = None
    L.mgpu_last_error.argtypes = [vp]
    L.mgpu_last_error.restype = ctypes.c_char_p
    L.mgpu_set_memory_budget.argtypes = [vp, ctypes.c_int64]
    L.mgpu_eval_rhs.argtypes = [vp, P(MgpuGraph), ctypes.c_int32, P(ctypes.c_int32), P(d), P(d), P(d), P(d)]
    L.mgpu_simulate.argtypes = [vp, P(MgpuGraph), ctypes.c_int32, P(ctypes.c_int32), d, d, d,
                                P(MgpuIntegratorOpts), ctypes.c_int32, P(d), P(d), P(ctypes.c_int32)]
    L.mgpu_simulate_dt.argtypes = [vp, P(MgpuGraph), ctypes.c_int32, P(ctypes.c_int32), d, d, P(d),
                                P(MgpuIntegratorOpts), ctypes.c_int32, P(d), P(d), P(ctypes.c_int32)]
    L.mgpu_simulate_flows.argtypes = [vp, P(MgpuGraph), ctypes.c_int32, P(ctypes.c_int32), d, d, d,
                                      P(MgpuIntegratorOpts), ctypes.c_int32, P(d), P(d), P(d), P(ctypes.c_int32)]
    L.mgpu_batch_create.argtypes = [vp, P(MgpuGraph), ctypes.c_int32, d, P(MgpuSolverOpts), P(vp)]
    L.mgpu_batch_advance.argtypes = [vp, d, P(d)]
    L.mgpu_batch_get_state.argtypes = [vp, P(d)]
    L.mgpu_batch_get_time.argtypes = [vp, P(d)]
    L.mgpu_batch_set_state.argtypes = [vp, P(d)]
    L.mgpu_batch_set_damping_cache.argtypes = [vp] + [ctypes.c_int32] * 4 + [P(d), P(d)]
    L.mgpu_batch_set_edge_damping_cache.argtypes = [vp] + [ctypes.c_int32] * 3 + [P(d), P(d)]
    L.mgpu_batch_step_nodes.argtypes = [vp, d, P(d)]
    L.mgpu_batch_step_exchange.argtypes = [vp]
    L.mgpu_batch_get_compartment_sums.argtypes = [vp, ctypes.c_int32, P(d)]
    L.mgpu_batch_get_stats.argtypes = [vp, P(MgpuStats)]
    L.mgpu_batch_get_timing.argtypes = [vp, P(MgpuTiming)]
    L.mgpu_batch_reset.argtypes = [vp, d]
    i32 = ctypes.c_int32
    # device pointers are passed as integers (void*)
    L.mgpu_simulate_final_noalloc.argtypes = [vp, i32, i32, i32, i32, vp, vp, vp, vp, vp, d, d, d,
                                              P(MgpuIntegratorOpts), vp, vp]
    L.mgpu_batch_launch.argtypes = [vp, d, P(d), i32, P(i32)]
    L.mgpu_batch_query.argtypes = [vp, P(i32)]
    L.mgpu_batch_get_failed.argtypes = [vp, P(i32), P(i32)]
    L.mgpu_batch_set_commuter_stats.argtypes = [vp, i32, i32, P(i32), P(i32), i32]
    L.mgpu_batch_set_flow_recording.argtypes = [vp, i32]
    L.mgpu_batch_regroup.argtypes = [vp, P(MgpuGraph), i32, P(vp), P(i32), P(vp)]
    L.mgpu_batch_get_flows.argtypes = [vp, P(d)]
    L.mgpu_batch_get_commuter_stats.argtypes = [vp, i32, P(i32), P(d), P(d)]
    L.mgpu_batch_autotune.argtypes = [vp, P(i32), P(i32)]
    L.mgpu_batch_ensemble_stats.argtypes = [vp, P(d), i32, P(d), P(d)]
    L.mgpu_batch_get_graph_state.argtypes = [vp, i32, P(d)]
    L.mgpu_batch_estimate_bytes.argtypes = [P(MgpuGraph), i32, P(MgpuSolverOpts)]
    L.mgpu_batch_estimate_bytes.restype = ctypes.c_int64
    L.mgpu_default_server_opts.argtypes = [P(MgpuServerOpts)]
    L.mgpu_default_server_opts.restype = None
    L.mgpu_server_create.argtypes = [ctypes.c_int, P(MgpuServerOpts), P(vp)]
    L.mgpu_server_destroy.argtypes = [vp]
    L.mgpu_server_destroy.restype = None
    L.mgpu_server_submit.argtypes = [vp, P(MgpuGraph), d, d, P(ctypes.c_int64)]
    L.mgpu_server_step.argtypes = [vp, P(i32), P(i32), P(i32)]
    L.mgpu_server_take.argtypes = [vp, P(ctypes.c_int64), P(d), ctypes.c_int64, P(ctypes.c_int64), P(d)]
    L.mgpu_server_memory_in_use.argtypes = [vp]
    L.mgpu_server_memory_in_use.restype = ctypes.c_int64
    L.mgpu_server_num_batches.argtypes = [vp]
    L.mgpu_server_num_batches.restype = ctypes.c_int32
    L.mgpu_server_num_merges.argtypes = [vp]
    L.mgpu_server_num_merges.restype = ctypes.c_int64
    L.mgpu_batch_device_bytes.argtypes = [vp]
    L.mgpu_batch_device_bytes.restype = ctypes.c_int64
    L.mgpu_batch_destroy.argtypes = [vp]
    L.mgpu_batch_destroy.restype = None
    _lib = L
    return L


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def solver_opts(precision=PRECISION_MIXED, dt0=0.1, dt_exchange=0.5, integrator: Optional[MgpuIntegratorOpts] = None,
                instances_per_block=0, max_steps_per_interval=0, use_cuda_graph=True,
                profile=False, staged_exchange=True) -> MgpuSolverOpts:
    o = MgpuSolverOpts()
    lib().mgpu_default_solver_opts(ctypes.byref(o))
    if integrator is not None:
        o.integrator = integrator
    o.dt0 = dt0
    o.dt_exchange = dt_exchange
    o.precision = precision
    o.instances_per_block = instances_per_block
    o.max_steps_per_interval = max_steps_per_interval
    o.use_cuda_graph = 1 if use_cuda_graph else 0
    o.profile = 1 if profile else 0
    o.staged_exchange = int(staged_exchange)  # True/1: when the per-graph CTAs fill the GPU, 2: always
    return o


class Context:
    """One mgpu_context (one CUDA stream on one device)."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        self._batches = weakref.WeakSet()  # batches to close before the context
        rc = lib().mgpu_create(device, ctypes.byref(self._h))
        if rc != OK:
            raise MgpuError(rc, "mgpu_create failed")

    @property
    def handle(self):
        return self._h

    def check(self, rc: int):
        if rc != OK:
            raise MgpuError(rc, lib().mgpu_last_error(self._h).decode())

    def close(self):
        if self._h:
            for b in list(self._batches):
                b.close()
            lib().mgpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_memory_budget(self, nbytes: int):
        self.check(lib().mgpu_set_memory_budget(self._h, int(nbytes)))

    def eval_rhs(self, g: GraphArrays, nodes, pop, y, t) -> np.ndarray:
        nodes = np.ascontiguousarray(nodes, np.int32)
        cnt = nodes.shape[0]
        pop = np.ascontiguousarray(pop, np.float64).reshape(cnt, g.n)
        y = np.ascontiguousarray(y, np.float64).reshape(cnt, g.n)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, np.float64), (cnt,)))
        out = np.zeros((cnt, g.n))
        cg = g.as_ctypes()
        self.check(lib().mgpu_eval_rhs(self._h, ctypes.byref(cg), cnt, _ip(nodes), _dp(pop), _dp(y), _dp(t),
                                       _dp(out)))
        return out

    def simulate_flows(self, g: GraphArrays, nodes, t0: float, tmax: float, dt0: float, opts=None,
                       max_points=4096):
        """Per node: (times [P], flows [P, 15G], populations [P, 10G]) of every accepted step."""
        opts = opts or integrator_opts()
        nodes = np.ascontiguousarray(nodes, np.int32)
        cnt = nodes.shape[0]
        nf = 15 * g.num_groups
        out_t = np.zeros((cnt, max_points))
        out_f = np.zeros((cnt, max_points, nf))
        out_y = np.zeros((cnt, max_points, g.n))
        npts = np.zeros(cnt, np.int32)
        cg = g.as_ctypes()
        self.check(lib().mgpu_simulate_flows(self._h, ctypes.byref(cg), cnt, _ip(nodes), t0, tmax, dt0,
                                             ctypes.byref(opts), max_points, _dp(out_t), _dp(out_f), _dp(out_y),
                                             _ip(npts)))
        return [(out_t[k, :npts[k]].copy(), out_f[k, :npts[k]].copy(), out_y[k, :npts[k]].copy())
                for k in range(cnt)]

    def simulate(self, g: GraphArrays, nodes, t0: float, tmax: float, dt0: float, opts=None, max_points=4096):
        """Per node: (times [P], values [P, 10G]) of every accepted step."""
        opts = opts or integrator_opts()
        nodes = np.ascontiguousarray(nodes, np.int32)
        cnt = nodes.shape[0]
        out_t = np.zeros((cnt, max_points))
        out_y = np.zeros((cnt, max_points, g.n))
        npts = np.zeros(cnt, np.int32)
        cg = g.as_ctypes()
        self.check(lib().mgpu_simulate(self._h, ctypes.byref(cg), cnt, _ip(nodes), t0, tmax, dt0, ctypes.byref(opts),
                                       max_points, _dp(out_t), _dp(out_y), _ip(npts)))
        return [(out_t[k, :npts[k]].copy(), out_y[k, :npts[k]].copy()) for k in range(cnt)]


class Batch:
    """mgpu_batch: graphs simulated together (GraphSimulation per graph)."""

    def __init__(self, ctx: Context, graphs: Sequence[GraphArrays], t0: float = 0.0, opts: MgpuSolverOpts = None):
        self.ctx = ctx
        self.graphs = list(graphs)
        self._arr = graphs_as_ctypes(self.graphs)
        self._h = ctypes.c_void_p()
        opts = opts or solver_opts()
        ctx.check(lib().mgpu_batch_create(ctx.handle, self._arr, len(self.graphs), t0, ctypes.byref(opts),
                                          ctypes.byref(self._h)))
        ctx._batches.add(self)
        self.sizes = [g.num_nodes * g.n for g in self.graphs]
        self.total = int(sum(self.sizes))

    def advance(self, tmax: float, tmax_per_graph=None):
        if tmax_per_graph is not None:
            tpg = np.ascontiguousarray(tmax_per_graph, np.float64)
            assert tpg.shape[0] == len(self.graphs)
            self.ctx.check(lib().mgpu_batch_advance(self._h, float(tmax), _dp(tpg)))
        else:
            self.ctx.check(lib().mgpu_batch_advance(self._h, float(tmax), ctypes.POINTER(ctypes.c_double)()))

    def launch(self, tmax: float, max_phases: int) -> int:
        """mgpu_batch_launch: enqueue up to max_phases intervals of an advance to tmax
        without waiting; returns the intervals still to launch."""
        rem = ctypes.c_int32()
        self.ctx.check(lib().mgpu_batch_launch(self._h, float(tmax), ctypes.POINTER(ctypes.c_double)(),
                                               int(max_phases), ctypes.byref(rem)))
        return rem.value

    def query(self) -> bool:
        """mgpu_batch_query: True when the launched intervals have finished."""
        done = ctypes.c_int32()
        self.ctx.check(lib().mgpu_batch_query(self._h, ctypes.byref(done)))
        return bool(done.value)

    def set_commuter_stats(self, graph: int, save_sets, capacity: int):
        """mgpu_batch_set_commuter_stats: record the edges' mobility results of one
        graph with these sets of flat compartment indices (empty: stop)."""
        off = np.zeros(len(save_sets) + 1, np.int32)
        for i, st in enumerate(save_sets):
            off[i + 1] = off[i] + len(st)
        idx = np.ascontiguousarray(np.concatenate([np.asarray(st, np.int32) for st in save_sets])
                                   if save_sets else np.zeros(1, np.int32), np.int32)
        ip = ctypes.POINTER(ctypes.c_int32)
        self.ctx.check(lib().mgpu_batch_set_commuter_stats(self._h, int(graph), len(save_sets), off.ctypes.data_as(ip),
                                                           idx.ctypes.data_as(ip), int(capacity)))
        self._stats = getattr(self, "_stats", {})
        self._stats[graph] = (len(save_sets), int(capacity))

    def commuter_stats(self, graph: int):
        """mgpu_batch_get_commuter_stats: (counts [E], times [E, capacity],
        values [E, capacity, sets + 1]) of one graph."""
        S, cap = self._stats[graph]
        E = max(self.graphs[graph].num_edges, 1)
        counts = np.zeros(E, np.int32)
        times = np.zeros((E, cap))
        values = np.zeros((E, cap, S + 1))
        self.ctx.check(lib().mgpu_batch_get_commuter_stats(self._h, int(graph),
                                                           counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                           _dp(times), _dp(values)))
        E = self.graphs[graph].num_edges
        return counts[:E], times[:E], values[:E]

    def set_flow_recording(self, on: bool = True):
        """mgpu_batch_set_flow_recording: sum every node's flows from now on (from zero)."""
        self.ctx.check(lib().mgpu_batch_set_flow_recording(self._h, 1 if on else 0))

    def flows(self):
        """mgpu_batch_get_flows: per graph, the accumulated flows [N, 15 G]."""
        nf = [g.num_nodes * 15 * g.num_groups for g in self.graphs]
        out = np.empty(max(sum(nf), 1))
        self.ctx.check(lib().mgpu_batch_get_flows(self._h, _dp(out)))
        res, off = [], 0
        for g, k in zip(self.graphs, nf):
            res.append(out[off:off + k].reshape(g.num_nodes, 15 * g.num_groups))
            off += k
        return res

    def failed(self) -> np.ndarray:
        """mgpu_batch_get_failed: per graph 0, or FAILED_STEP_CAP | FAILED_NONFINITE."""
        f = np.zeros(max(len(self.graphs), 1), np.int32)
        n = ctypes.c_int32()
        self.ctx.check(lib().mgpu_batch_get_failed(self._h, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                   ctypes.byref(n)))
        return f[:len(self.graphs)]

    def state_flat(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.total)
        self.ctx.check(lib().mgpu_batch_get_state(self._h, _dp(out)))
        return out

    def states(self):
        flat = self.state_flat()
        res, off = [], 0
        for g, s in zip(self.graphs, self.sizes):
            res.append(flat[off:off + s].reshape(g.num_nodes, g.n))
            off += s
        return res

    def set_state(self, flat: np.ndarray):
        flat = np.ascontiguousarray(flat, np.float64)
        assert flat.size == self.total
        self.ctx.check(lib().mgpu_batch_set_state(self._h, _dp(flat)))

    def set_edge_damping_cache(self, graph: int, edge: int, times, values):
        """mgpu_batch_set_edge_damping_cache: times [K'], values [K'][10G]."""
        t = np.ascontiguousarray(times, np.float64)
        v = np.ascontiguousarray(values, np.float64)
        self.ctx.check(lib().mgpu_batch_set_edge_damping_cache(self._h, graph, edge, t.shape[0], _dp(t), _dp(v)))

    def step_nodes(self, tmax: float):
        self.ctx.check(lib().mgpu_batch_step_nodes(self._h, float(tmax), ctypes.POINTER(ctypes.c_double)()))

    def step_exchange(self):
        self.ctx.check(lib().mgpu_batch_step_exchange(self._h))

    def compartment_sums(self, compartment: int) -> np.ndarray:
        """mgpu_batch_get_compartment_sums: per node (all graphs), the sum over age groups of one compartment."""
        out = np.zeros(sum(g.num_nodes for g in self.graphs))
        self.ctx.check(lib().mgpu_batch_get_compartment_sums(self._h, compartment, _dp(out)))
        return out

    def set_damping_cache(self, graph: int, node: int, matrix: int, times, values):
        """mgpu_batch_set_damping_cache: times [K'], values [K'][G][G]."""
        t = np.ascontiguousarray(times, np.float64)
        v = np.ascontiguousarray(values, np.float64)
        self.ctx.check(lib().mgpu_batch_set_damping_cache(self._h, graph, node, matrix, t.shape[0], _dp(t), _dp(v)))

    def times(self) -> np.ndarray:
        out = np.zeros(len(self.graphs))
        self.ctx.check(lib().mgpu_batch_get_time(self._h, _dp(out)))
        return out

    def stats(self) -> dict:
        s = MgpuStats()
        self.ctx.check(lib().mgpu_batch_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def reset(self, t0: float = 0.0):
        self.ctx.check(lib().mgpu_batch_reset(self._h, float(t0)))

    def timing(self) -> dict:
        t = MgpuTiming()
        self.ctx.check(lib().mgpu_batch_get_timing(self._h, ctypes.byref(t)))
        return t.as_dict()

    def device_bytes(self) -> int:
        return int(lib().mgpu_batch_device_bytes(self._h))

    def close(self):
        if self._h:
            lib().mgpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ensemble_stats(self, percentiles=(0.05, 0.5, 0.95)):
        """(mean [N, 10G], percentiles [P, N, 10G]) of the current states over the batch's graphs."""
        g = self.graphs[0]
        p = np.ascontiguousarray(percentiles, np.float64)
        mean = np.empty((g.num_nodes, g.n))
        pct = np.empty((p.shape[0], g.num_nodes, g.n))
        self.ctx.check(lib().mgpu_batch_ensemble_stats(self._h, _dp(p), p.shape[0], _dp(mean), _dp(pct)))
        return mean, pct

    def autotune(self) -> dict:
        ipb, grid = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(lib().mgpu_batch_autotune(self._h, ctypes.byref(ipb), ctypes.byref(grid)))
        return {"instances_per_block": ipb.value, "grid_blocks": grid.value}

    def graph_state(self, graph: int) -> np.ndarray:
        g = self.graphs[graph]
        out = np.empty(g.num_nodes * g.n)
        self.ctx.check(lib().mgpu_batch_get_graph_state(self._h, int(graph), _dp(out)))
        return out.reshape(g.num_nodes, g.n)


def server_opts(precision=PRECISION_MIXED, memory_budget=0, max_batches=16, phases_per_launch=2,
                max_graphs_per_batch=4096, min_batch_graphs=1, max_wait_ms=0.0, rebatch_max_graphs=0,
                **solver_kw) -> MgpuServerOpts:
    o = MgpuServerOpts()
    lib().mgpu_default_server_opts(ctypes.byref(o))
    o.solver = solver_opts(precision=precision, **solver_kw)
    o.memory_budget = int(memory_budget)
    o.max_batches = int(max_batches)
    o.phases_per_launch = int(phases_per_launch)
    o.max_graphs_per_batch = int(max_graphs_per_batch)
    o.min_batch_graphs = int(min_batch_graphs)
    o.max_wait_ms = float(max_wait_ms)
    o.rebatch_max_graphs = int(rebatch_max_graphs)
    return o


class Server:
    """mgpu_server: device-resident request loop with continuous batching."""

    def __init__(self, device: int = 0, opts: MgpuServerOpts = None):
        self._h = ctypes.c_void_p()
        rc = lib().mgpu_server_create(device, ctypes.byref(opts or server_opts()), ctypes.byref(self._h))
        if rc != OK:
            raise MgpuError(rc, "mgpu_server_create failed")
        self._graphs = {}  # request id -> graph (keeps the host arrays alive)

    def submit(self, g: GraphArrays, t0: float, tmax: float) -> int:
        rid = ctypes.c_int64()
        rc = lib().mgpu_server_submit(self._h, ctypes.byref(g.as_ctypes()), float(t0), float(tmax),
                                      ctypes.byref(rid))
        if rc != OK:
            raise MgpuError(rc, "mgpu_server_submit failed")
        self._graphs[rid.value] = g
        return rid.value

    def step(self):
        c, r, q = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        rc = lib().mgpu_server_step(self._h, ctypes.byref(c), ctypes.byref(r), ctypes.byref(q))
        if rc != OK:
            raise MgpuError(rc, "mgpu_server_step failed")
        return c.value, r.value, q.value

    def take(self):
        """(request id, final states [N, 10G], latency s) of one completed request, or None."""
        rid, cnt, lat = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        rc = lib().mgpu_server_take(self._h, ctypes.byref(rid), ctypes.POINTER(ctypes.c_double)(), 0,
                                    ctypes.byref(cnt), ctypes.byref(lat))
        if rid.value == 0 and rc == OK:
            return None
        g = self._graphs[rid.value] if rid.value in self._graphs else None
        out = np.empty(max(cnt.value, 1))
        rc = lib().mgpu_server_take(self._h, ctypes.byref(rid), _dp(out), out.shape[0], ctypes.byref(cnt),
                                    ctypes.byref(lat))
        g = self._graphs.pop(rid.value)
        if rc != OK:
            raise MgpuError(rc, f"request {rid.value} failed")
        return rid.value, out[:cnt.value].reshape(g.num_nodes, g.n), lat.value

    def memory_in_use(self) -> int:
        return int(lib().mgpu_server_memory_in_use(self._h))

    def num_batches(self) -> int:
        return int(lib().mgpu_server_num_batches(self._h))

    def num_merges(self) -> int:
        return int(lib().mgpu_server_num_merges(self._h))

    def close(self):
        if self._h:
            lib().mgpu_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
