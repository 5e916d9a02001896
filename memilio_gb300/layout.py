"""Python mirror of include/miogpu_layout.h: the flat-array format of an
age-resolved ODE-SECIR metapopulation graph.

A :class:`GraphArrays` owns the numpy arrays of one graph and hands out a
ctypes ``mgpu_graph`` view of them. Compartment and flow order follow
osecir::InfectionState and the osecir Flows typelist
(models/ode_secir/infection_state.h:33-47, models/ode_secir/model.h:45-59).
"""
from __future__ import annotations

import ctypes
import operator
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

NUM_COMPARTMENTS = 10
NUM_FLOWS = 15
MAX_GROUPS = 8
MAX_CONTACT_MATRICES = 4

S, E, INS, INSC, ISY, ISYC, ISEV, ICRI, R, D = range(10)
COMPARTMENT_NAMES = ["S", "E", "INS", "INSC", "ISy", "ISyC", "ISev", "ICri", "R", "D"]

# scalar parameters (head of each parameter record)
P_START_DAY, P_SEASONALITY, P_ICU_CAPACITY, P_TNT_CAPACITY, P_TNT_MAX_RISK, \
    P_COMMUTER_NONDETECTION, P_START_COMMUTER_DETECTION, P_END_COMMUTER_DETECTION = range(8)
NUM_SCALAR_PARAMS = 8

# per-group parameters
(G_TIME_EXPOSED, G_TIME_INS, G_TIME_ISY, G_TIME_ISEV, G_TIME_ICRI, G_TRANSMISSION_PROB,
 G_REL_TRANSMISSION_NS, G_RECOVERED_PER_INS, G_RISK_FROM_SYMPTOMATIC, G_MAX_RISK_FROM_SYMPTOMATIC,
 G_SEVERE_PER_ISY, G_CRITICAL_PER_SEVERE, G_DEATHS_PER_SEVERE, G_DEATHS_PER_CRITICAL) = range(14)
NUM_GROUP_PARAMS = 14

METHOD_CASH_KARP54 = 0
METHOD_RKF45 = 1

DBL_MAX = float(np.finfo(np.float64).max)
DBL_MIN = float(np.finfo(np.float64).tiny)
DBL_LOWEST = -DBL_MAX

FLOW_SRC = [S, E, INS, INS, INSC, INSC, ISY, ISY, ISYC, ISYC, ISEV, ISEV, ISEV, ICRI, ICRI]
FLOW_DST = [E, INS, ISY, R, ISYC, R, ISEV, R, ISEV, R, ICRI, R, D, D, R]


def param_stride(G: int) -> int:
    return NUM_SCALAR_PARAMS + NUM_GROUP_PARAMS * G


def group_param_index(p: int, g: int, G: int) -> int:
    return NUM_SCALAR_PARAMS + p * G + g


class MgpuGraph(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("num_groups", ctypes.c_int32),
        ("num_edges", ctypes.c_int32),
        ("num_contact_matrices", ctypes.c_int32),
        ("num_damping_points", ctypes.c_int32),
        ("num_edge_damping_points", ctypes.c_int32),
        ("params", ctypes.c_void_p),  # const double*
        ("contact_baseline", ctypes.c_void_p),  # const double*
        ("contact_minimum", ctypes.c_void_p),  # const double*
        ("damping_times", ctypes.c_void_p),  # const double*
        ("damping_values", ctypes.c_void_p),  # const double*
        ("init_state", ctypes.c_void_p),  # const double*
        ("edge_src", ctypes.c_void_p),  # const int32_t*
        ("edge_dst", ctypes.c_void_p),  # const int32_t*
        ("edge_coeff_baseline", ctypes.c_void_p),  # const double*
        ("edge_coeff_minimum", ctypes.c_void_p),  # const double*
        ("edge_damping_times", ctypes.c_void_p),  # const double*
        ("edge_damping_values", ctypes.c_void_p),  # const double*
    ]


class MgpuIntegratorOpts(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("abs_tol", ctypes.c_double),
        ("rel_tol", ctypes.c_double),
        ("dt_min", ctypes.c_double),
        ("dt_max", ctypes.c_double),
    ]


def integrator_opts(method=METHOD_CASH_KARP54, abs_tol=1e-10, rel_tol=1e-5, dt_min=DBL_MIN, dt_max=DBL_MAX):
    """Defaults of ControlledStepperWrapper (memilio/math/stepper_wrapper.h:83-91)."""
    return MgpuIntegratorOpts(method, 0, abs_tol, rel_tol, dt_min, dt_max)


def _addr(a: Optional[np.ndarray], dtype) -> Optional[int]:
    """Address of a C-contiguous array of `dtype` (None for an empty one)."""
    if a is None or a.size == 0:
        return None
    assert a.dtype == dtype and a.flags.c_contiguous
    if a.flags.writeable:
        return ctypes.addressof(ctypes.c_char.from_buffer(a))  # (a faster route to the data pointer)
    return a.__array_interface__["data"][0]


def graphs_as_ctypes(graphs) -> ctypes.Array:
    """An mgpu_graph array of `graphs` (the arrays must outlive its use)."""
    return (MgpuGraph * len(graphs))(*[g.as_ctypes() for g in graphs])


@dataclass
class GraphArrays:
    """Numpy arrays of one graph in the miogpu layout.

    Shapes: params [N, stride(G)], contact_baseline/minimum [N, M, G, G],
    damping_times [N, M, K], damping_values [N, M, K, G, G], init_state
    [N, 10G], edge_src/dst [E] (sorted by (src, dst)), edge_coeff_baseline
    [E, 10G], edge_coeff_minimum [E, 10G] or None, edge_damping_times
    [E, Ke], edge_damping_values [E, Ke, 10G].
    """

    num_groups: int
    params: np.ndarray
    contact_baseline: np.ndarray
    contact_minimum: np.ndarray
    damping_times: np.ndarray
    damping_values: np.ndarray
    init_state: np.ndarray
    edge_src: np.ndarray
    edge_dst: np.ndarray
    edge_coeff_baseline: np.ndarray
    edge_coeff_minimum: Optional[np.ndarray] = None
    edge_damping_times: Optional[np.ndarray] = None
    edge_damping_values: Optional[np.ndarray] = None
    _c: Optional[MgpuGraph] = field(default=None, repr=False)
    _c_src: Optional[tuple] = field(default=None, repr=False, compare=False)

    def __post_init__(self):
        G = self.num_groups
        n = NUM_COMPARTMENTS * G
        f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self.params = f64(self.params).reshape(-1, param_stride(G))
        N = self.params.shape[0]
        self.contact_baseline = f64(self.contact_baseline).reshape(N, -1, G, G)
        M = self.contact_baseline.shape[1]
        self.contact_minimum = f64(self.contact_minimum).reshape(N, M, G, G)
        self.damping_times = f64(self.damping_times).reshape(N, M, -1)
        K = self.damping_times.shape[2]
        self.damping_values = f64(self.damping_values).reshape(N, M, K, G, G)
        self.init_state = f64(self.init_state).reshape(N, n)
        self.edge_src = np.ascontiguousarray(self.edge_src, dtype=np.int32).reshape(-1)
        self.edge_dst = np.ascontiguousarray(self.edge_dst, dtype=np.int32).reshape(-1)
        Ecount = self.edge_src.shape[0]
        self.edge_coeff_baseline = f64(self.edge_coeff_baseline).reshape(Ecount, n)
        if self.edge_coeff_minimum is not None:
            self.edge_coeff_minimum = f64(self.edge_coeff_minimum).reshape(Ecount, n)
        if self.edge_damping_times is None or np.asarray(self.edge_damping_times).size == 0:
            self.edge_damping_times = np.zeros((Ecount, 0))
            self.edge_damping_values = np.zeros((Ecount, 0, n))
        else:
            self.edge_damping_times = f64(self.edge_damping_times).reshape(Ecount, -1)
            Ke = self.edge_damping_times.shape[1]
            self.edge_damping_values = f64(self.edge_damping_values).reshape(Ecount, Ke, n)
        if Ecount:
            key = self.edge_src.astype(np.int64) * max(N, 1) + self.edge_dst
            if np.any(np.diff(key) <= 0):
                raise ValueError("edges must be sorted by (src, dst) without duplicates")

    @property
    def num_nodes(self) -> int:
        return self.params.shape[0]

    @property
    def num_edges(self) -> int:
        return self.edge_src.shape[0]

    @property
    def num_contact_matrices(self) -> int:
        return self.contact_baseline.shape[1]

    @property
    def num_damping_points(self) -> int:
        return self.damping_times.shape[2]

    @property
    def n(self) -> int:
        return NUM_COMPARTMENTS * self.num_groups

    def as_ctypes(self) -> MgpuGraph:
        """The mgpu_graph view of the arrays (they must outlive its use); kept
        while the arrays are the same objects (changes in place need no rebuild,
        an attribute set to another array rebuilds it)."""
        src = (self.params, self.contact_baseline, self.contact_minimum, self.damping_times, self.damping_values,
               self.init_state, self.edge_src, self.edge_dst, self.edge_coeff_baseline, self.edge_coeff_minimum,
               self.edge_damping_times, self.edge_damping_values)
        if self._c is not None and self._c_src is not None and all(map(operator.is_, src, self._c_src)):
            return self._c
        f8, i4 = np.float64, np.int32
        a = _addr
        g = MgpuGraph(self.num_nodes, self.num_groups, self.num_edges, self.num_contact_matrices,
                      self.num_damping_points, self.edge_damping_times.shape[1],
                      a(self.params, f8), a(self.contact_baseline, f8), a(self.contact_minimum, f8),
                      a(self.damping_times, f8), a(self.damping_values, f8), a(self.init_state, f8),
                      a(self.edge_src, i4), a(self.edge_dst, i4), a(self.edge_coeff_baseline, f8),
                      a(self.edge_coeff_minimum, f8), a(self.edge_damping_times, f8),
                      a(self.edge_damping_values, f8))
        self._c = g
        self._c_src = src
        return g

    def subgraph_nodes(self, nodes) -> "GraphArrays":
        """Nodes `nodes` without edges (for single-node checks)."""
        nodes = np.asarray(nodes)
        return GraphArrays(
            self.num_groups, self.params[nodes], self.contact_baseline[nodes], self.contact_minimum[nodes],
            self.damping_times[nodes], self.damping_values[nodes], self.init_state[nodes],
            np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros((0, self.n)))

    def with_init_state(self, state: np.ndarray) -> "GraphArrays":
        return GraphArrays(
            self.num_groups, self.params, self.contact_baseline, self.contact_minimum, self.damping_times,
            self.damping_values, np.asarray(state, np.float64).reshape(self.num_nodes, self.n), self.edge_src,
            self.edge_dst, self.edge_coeff_baseline, self.edge_coeff_minimum, self.edge_damping_times,
            self.edge_damping_values)


def damping_cache_single(G: int, t_damp: float, value: float):
    """Cache of one constant damping at level 0/type 0 (damping.h:570-600):
    points (lowest, 0), (t, value), (max, value)."""
    times = np.array([DBL_LOWEST, t_damp, DBL_MAX])
    vals = np.zeros((3, G, G))
    vals[1] = value
    vals[2] = value
    return times, vals
