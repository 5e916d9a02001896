"""`memilio.simulation.osecir` over libmiogpu (pycode/memilio-simulation's
osecir bindings, bindings/models/osecir.cpp): Model with parameters and
populations, simulate, MobilityGraph and MobilitySimulation
(make_mobility_sim + GraphSimulation), interpolate_simulation_result.
The solves run on the GPU through the C ABI; results are TimeSeries."""
from __future__ import annotations

import enum
from typing import List, Optional

import numpy as np

from .. import _native as N
from .. import layout as L
from . import AgeGroup, Damping, MobilityParameters, TimeSeries, damping_cache, interpolate_simulation_result

__all__ = ["InfectionState", "Parameters", "Populations", "Model", "simulate", "simulate_flows", "MobilityGraph",
           "MobilitySimulation", "ParameterStudy", "GraphParameterStudy", "interpolate_simulation_result"]


class InfectionState(enum.IntEnum):
    """osecir::InfectionState (models/ode_secir/infection_state.h:33-47)."""
    Susceptible = 0
    Exposed = 1
    InfectedNoSymptoms = 2
    InfectedNoSymptomsConfirmed = 3
    InfectedSymptoms = 4
    InfectedSymptomsConfirmed = 5
    InfectedSevere = 6
    InfectedCritical = 7
    Recovered = 8
    Dead = 9
    Count = 10


_SCALARS = {"StartDay": L.P_START_DAY, "Seasonality": L.P_SEASONALITY, "ICUCapacity": L.P_ICU_CAPACITY,
            "TestAndTraceCapacity": L.P_TNT_CAPACITY, "TestAndTraceCapacityMaxRisk": L.P_TNT_MAX_RISK}
_GROUP = {"TimeExposed": L.G_TIME_EXPOSED, "TimeInfectedNoSymptoms": L.G_TIME_INS,
          "TimeInfectedSymptoms": L.G_TIME_ISY, "TimeInfectedSevere": L.G_TIME_ISEV,
          "TimeInfectedCritical": L.G_TIME_ICRI, "TransmissionProbabilityOnContact": L.G_TRANSMISSION_PROB,
          "RelativeTransmissionNoSymptoms": L.G_REL_TRANSMISSION_NS,
          "RecoveredPerInfectedNoSymptoms": L.G_RECOVERED_PER_INS,
          "RiskOfInfectionFromSymptomatic": L.G_RISK_FROM_SYMPTOMATIC,
          "MaxRiskOfInfectionFromSymptomatic": L.G_MAX_RISK_FROM_SYMPTOMATIC,
          "SeverePerInfectedSymptoms": L.G_SEVERE_PER_ISY, "CriticalPerSevere": L.G_CRITICAL_PER_SEVERE,
          "DeathsPerSevere": L.G_DEATHS_PER_SEVERE, "DeathsPerCritical": L.G_DEATHS_PER_CRITICAL}


class _GroupValues:
    def __init__(self, rec, p, G):
        self._rec, self._p, self._G = rec, p, G

    def _i(self, g):
        g = int(g)
        if not 0 <= g < self._G:
            raise IndexError("age group out of range")
        return L.group_param_index(self._p, g, self._G)

    def __getitem__(self, g):
        return float(self._rec[self._i(g)])

    def __setitem__(self, g, v):
        self._rec[self._i(g)] = float(v)


class ContactMatrix:
    """mio.ContactMatrix: baseline, minimum and dampings of one contact matrix."""

    def __init__(self, G: int):
        self.baseline = np.ones((G, G))
        self.minimum = np.zeros((G, G))
        self.dampings: List[Damping] = []

    def add_damping(self, d: Damping):
        self.dampings.append(d)


class ContactMatrixGroup:
    """mio.ContactMatrixGroup: contact matrices that add up."""

    def __init__(self, num_matrices: int, G: int):
        self._m = [ContactMatrix(G) for _ in range(num_matrices)]

    def __getitem__(self, i) -> ContactMatrix:
        return self._m[i]

    def __setitem__(self, i, m: ContactMatrix):
        self._m[i] = m

    def __len__(self):
        return len(self._m)

    def add_damping(self, d: Damping):
        for m in self._m:
            m.add_damping(d)


class _ContactPatterns:
    def __init__(self, G):
        self.cont_freq_mat = ContactMatrixGroup(1, G)


class Parameters:
    """osecir::Parameters with the reference's defaults (parameters.h:399-768)."""

    def __init__(self, G: int):
        object.__setattr__(self, "_G", G)
        rec = np.zeros(L.param_stride(G))
        rec[L.P_ICU_CAPACITY] = L.DBL_MAX
        rec[L.P_TNT_CAPACITY] = L.DBL_MAX
        rec[L.P_TNT_MAX_RISK] = 5.0
        for p in (L.G_TIME_EXPOSED, L.G_TIME_INS, L.G_TIME_ISY, L.G_TIME_ISEV, L.G_TIME_ICRI,
                  L.G_TRANSMISSION_PROB, L.G_REL_TRANSMISSION_NS, L.G_RISK_FROM_SYMPTOMATIC,
                  L.G_MAX_RISK_FROM_SYMPTOMATIC):
            for g in range(G):
                rec[L.group_param_index(p, g, G)] = 1.0
        object.__setattr__(self, "_rec", rec)
        object.__setattr__(self, "ContactPatterns", _ContactPatterns(G))

    def __getattr__(self, name):
        if name in _SCALARS:
            return float(self._rec[_SCALARS[name]])
        if name in _GROUP:
            return _GroupValues(self._rec, _GROUP[name], self._G)
        raise AttributeError(name)

    def __setattr__(self, name, v):
        if name in _SCALARS:
            self._rec[_SCALARS[name]] = float(v)
        elif name == "ContactPatterns":
            object.__setattr__(self, name, v)
        else:
            raise AttributeError(f"{name} cannot be set (per-group parameters are set by age group)")

    def get_num_groups(self) -> int:
        return self._G

    def apply_constraints(self) -> bool:
        """apply_constraints (parameters.h:465-611): corrects out-of-range values."""
        rec, G, fixed = self._rec, self._G, False

        def fix(i, bad, to):
            nonlocal fixed
            if bad:
                rec[i] = to
                fixed = True

        fix(L.P_SEASONALITY, rec[L.P_SEASONALITY] < 0.0 or rec[L.P_SEASONALITY] > 0.5, 0.0)
        for p in (L.P_ICU_CAPACITY, L.P_TNT_CAPACITY, L.P_TNT_MAX_RISK):
            fix(p, rec[p] < 0.0, 0.0)
        for g in range(G):
            gi = lambda p: L.group_param_index(p, g, G)
            for p in (L.G_TIME_EXPOSED, L.G_TIME_INS, L.G_TIME_ISY, L.G_TIME_ISEV, L.G_TIME_ICRI):
                fix(gi(p), rec[gi(p)] < 0.1, 0.1)
            for p in (L.G_TRANSMISSION_PROB, L.G_RECOVERED_PER_INS, L.G_RISK_FROM_SYMPTOMATIC,
                      L.G_SEVERE_PER_ISY, L.G_CRITICAL_PER_SEVERE, L.G_DEATHS_PER_SEVERE):
                fix(gi(p), rec[gi(p)] < 0.0 or rec[gi(p)] > 1.0, 0.0)
            fix(gi(L.G_REL_TRANSMISSION_NS), rec[gi(L.G_REL_TRANSMISSION_NS)] < 0.0, 0.0)
            fix(gi(L.G_DEATHS_PER_SEVERE),
                rec[gi(L.G_CRITICAL_PER_SEVERE)] + rec[gi(L.G_DEATHS_PER_SEVERE)] > 1.0, 0.0)
            fix(gi(L.G_DEATHS_PER_CRITICAL),
                rec[gi(L.G_DEATHS_PER_CRITICAL)] < 0.0 or rec[gi(L.G_DEATHS_PER_CRITICAL)] > 1.0, 0.0)
        return fixed


class Populations:
    """osecir::Model::populations: indexed by (AgeGroup, InfectionState), flat g*10 + c."""

    def __init__(self, G: int):
        self._G = G
        self._v = np.zeros(G * L.NUM_COMPARTMENTS)

    @staticmethod
    def _i(key):
        g, c = key
        return int(g) * L.NUM_COMPARTMENTS + int(c)

    def __getitem__(self, key):
        return float(self._v[self._i(key)])

    def __setitem__(self, key, v):
        self._v[self._i(key)] = float(v)

    def numel(self) -> int:
        return self._v.size

    def get_total(self) -> float:
        return float(self._v.sum())

    def get_group_total_AgeGroup(self, g) -> float:
        g = int(g)
        return float(self._v[g * L.NUM_COMPARTMENTS:(g + 1) * L.NUM_COMPARTMENTS].sum())

    def set_difference_from_total(self, key, total):
        """The entry `key` such that all entries sum to `total`."""
        i = self._i(key)
        self._v[i] = float(total) - (self._v.sum() - self._v[i])

    def set_difference_from_group_total_AgeGroup(self, key, total):
        """The entry `key` such that its age group sums to `total`."""
        i = self._i(key)
        g = int(key[0])
        self._v[i] = float(total) - (self.get_group_total_AgeGroup(g) - self._v[i])

    def apply_constraints(self) -> bool:
        neg = self._v < 0
        self._v[neg] = 0.0
        return bool(neg.any())

    def array(self) -> np.ndarray:
        return self._v


class Model:
    """osecir::Model(num_agegroups)."""

    def __init__(self, num_agegroups: int):
        G = int(num_agegroups)
        if not 1 <= G <= L.MAX_GROUPS:
            raise ValueError(f"1 to {L.MAX_GROUPS} age groups")
        self.parameters = Parameters(G)
        self.populations = Populations(G)

    def apply_constraints(self) -> bool:
        a = self.parameters.apply_constraints()
        b = self.populations.apply_constraints()
        return a or b

    def check_constraints(self) -> bool:
        import copy
        return copy.deepcopy(self).apply_constraints()

    def _num_groups(self) -> int:
        return self.parameters.get_num_groups()

    def _contact_arrays(self, extra_points: int = 0):
        """(baseline [M,G,G], minimum [M,G,G], damping times [M,K], values [M,K,G,G]) of this node."""
        G = self._num_groups()
        cm = self.parameters.ContactPatterns.cont_freq_mat
        base = np.array([np.broadcast_to(cm[m].baseline, (G, G)) for m in range(len(cm))], np.float64)
        mini = np.array([np.broadcast_to(cm[m].minimum, (G, G)) for m in range(len(cm))], np.float64)
        caches = [damping_cache((G, G), cm[m].dampings) if cm[m].dampings else None for m in range(len(cm))]
        if all(c is None for c in caches):
            return base, mini, np.zeros((len(cm), 0)), np.zeros((len(cm), 0, G, G))
        caches = [c if c is not None else damping_cache((G, G), []) for c in caches]
        K = max(c[0].size for c in caches) + extra_points
        times = np.full((len(cm), K), L.DBL_MAX)
        vals = np.zeros((len(cm), K, G, G))
        for m, (t, v) in enumerate(caches):
            times[m, :t.size] = t
            vals[m, :t.size] = v
            vals[m, t.size:] = v[-1]
        return base, mini, times, vals


def _graph_arrays(models: List[Model], states: List[np.ndarray], edges=()) -> L.GraphArrays:
    G = models[0]._num_groups()
    parts = [m._contact_arrays() for m in models]
    K = max(p[2].shape[1] for p in parts)
    M = parts[0][0].shape[0]
    dt, dv = np.full((len(models), M, K), L.DBL_MAX), np.zeros((len(models), M, K, G, G))
    for v, p in enumerate(parts):
        k = p[2].shape[1]
        if k:
            dt[v, :, :k] = p[2]
            dv[v, :, :k] = p[3]
            dv[v, :, k:] = p[3][:, -1:]
        elif K:
            dt[v, :, 0] = L.DBL_LOWEST
    n = G * L.NUM_COMPARTMENTS
    src = np.array([e[0] for e in edges], np.int32)
    dst = np.array([e[1] for e in edges], np.int32)
    coeff = np.array([e[2] for e in edges], np.float64).reshape(len(edges), n)
    return L.GraphArrays(G, np.array([m.parameters._rec for m in models]), np.array([p[0] for p in parts]),
                         np.array([p[1] for p in parts]), dt, dv, np.array(states, np.float64), src, dst, coeff)


_ctx: Optional[N.Context] = None
_OUT_OF_RANGE = 2  # MGPU_OUT_OF_RANGE: more accepted steps than room


def _context() -> N.Context:
    global _ctx
    if _ctx is None:
        _ctx = N.Context(0)
    return _ctx


def simulate(t0: float, tmax: float, dt: float, model: Model) -> TimeSeries:
    """osecir::simulate (models/ode_secir/model.h, simulation.h:99-110): every
    accepted step of the Cash-Karp 5(4) integration, on the GPU."""
    g = _graph_arrays([model], [model.populations.array()])
    cap = 4096
    while True:
        try:
            (t, y), = _context().simulate(g, [0], float(t0), float(tmax), float(dt), max_points=cap)
            break
        except N.MgpuError as e:
            if e.code != _OUT_OF_RANGE or cap >= 1 << 22:
                raise
            cap *= 4
    ts = TimeSeries(g.n)
    for k in range(t.size):
        ts.add_time_point(t[k], y[k])
    return ts


def simulate_flows(t0: float, tmax: float, dt: float, model: Model) -> List[TimeSeries]:
    """osecir::simulate_flows (models/ode_secir/model.h:404-410,
    compartments/flow_simulation.h): [populations, flows] of every accepted step,
    the flows (15 per age group) accumulated from zero; on the GPU."""
    g = _graph_arrays([model], [model.populations.array()])
    cap = 4096
    while True:
        try:
            (t, f, y), = _context().simulate_flows(g, [0], float(t0), float(tmax), float(dt), max_points=cap)
            break
        except N.MgpuError as e:
            if e.code != _OUT_OF_RANGE or cap >= 1 << 22:
                raise
            cap *= 4
    pops, flows = TimeSeries(g.n), TimeSeries(f.shape[1])
    for k in range(t.size):
        pops.add_time_point(t[k], y[k])
        flows.add_time_point(t[k], f[k])
    return [pops, flows]


class _Node:
    def __init__(self, id, model: Model, t0: float):
        self.id = id
        self.property = _NodeProperty(model, t0)


class _NodeProperty:
    """SimulationNode: the node's model and its result (the state at t0 and after
    every exchange interval)."""

    def __init__(self, model: Model, t0: float):
        import copy
        self.model = copy.deepcopy(model)
        self.result = TimeSeries(model.populations.numel())
        self.result.add_time_point(t0, self.model.populations.array())


class _Edge:
    def __init__(self, start, end, params: MobilityParameters):
        self.start_node_idx, self.end_node_idx, self.property = start, end, params


class MobilityGraph:
    """osecir.MobilityGraph: nodes with a model each, edges with mobility
    coefficients, kept sorted by (start, end) as Graph::add_edge does."""

    def __init__(self):
        self._nodes: List[_Node] = []
        self._edges: List[_Edge] = []

    def add_node(self, id, model: Model, t0: float = 0.0, dt: float = 0.1):
        self._nodes.append(_Node(id, model, t0))
        return self._nodes[-1]

    def add_edge(self, start_node_idx: int, end_node_idx: int, params):
        if not isinstance(params, MobilityParameters):
            params = MobilityParameters(params)
        e = _Edge(int(start_node_idx), int(end_node_idx), params)
        keys = [(x.start_node_idx, x.end_node_idx) for x in self._edges]
        k = (e.start_node_idx, e.end_node_idx)
        if k in keys:
            self._edges[keys.index(k)] = e
        else:
            self._edges.append(e)
            self._edges.sort(key=lambda x: (x.start_node_idx, x.end_node_idx))
        return e

    @property
    def num_nodes(self) -> int:
        return len(self._nodes)

    @property
    def num_edges(self) -> int:
        return len(self._edges)

    def get_node(self, i: int) -> _Node:
        return self._nodes[i]

    def get_edge(self, i: int) -> _Edge:
        return self._edges[i]


class MobilitySimulation:
    """osecir.MobilitySimulation(graph, t0, dt): make_mobility_sim + GraphSimulation
    (metapopulation_mobility_instant.h:656-678, graph_simulation.h:101-120) on the
    GPU's batched FP64 solver; node results gain the state after every interval."""

    def __init__(self, graph: MobilityGraph, t0: float = 0.0, dt: float = 0.5,
                 precision: int = N.PRECISION_FP64):
        self.graph = graph
        self.t = float(t0)
        self.dt = float(dt)
        models = [n.property.model for n in graph._nodes]
        states = [n.property.result.get_last_value() for n in graph._nodes]
        edges = [(e.start_node_idx, e.end_node_idx, e.property.coeffs) for e in graph._edges]
        self._g = _graph_arrays(models, states, edges)
        self._batch = N.Batch(_context(), [self._g], self.t,
                              N.solver_opts(precision=precision, dt_exchange=self.dt))

    def advance(self, tmax: float):
        n = self._g.n
        while self.t < tmax:
            t_next = min(self.t + self.dt, tmax)
            if tmax - t_next < 1e-12 * max(1.0, abs(tmax)):
                t_next = tmax
            self._batch.advance(t_next)
            self.t = t_next
            st = self._batch.states()[0]
            for v, node in enumerate(self.graph._nodes):
                node.property.result.add_time_point(self.t, st[v].reshape(n))

    def get_t(self) -> float:
        return self.t


class GraphParameterStudy:
    """osecir.GraphParameterStudy(graph, t0, tmax, dt, num_runs)
    (bindings/compartments/parameter_studies.h:88-122 over ParameterStudy::run_serial,
    cpp/memilio/compartments/parameter_studies.h): num_runs copies of the graph,
    each sampled and simulated from t0 to tmax with exchanges every dt
    (make_sampled_graph_simulation(graph, t0, dt, dt)).

    All runs go to the GPU as ONE batch. `sample` takes draw_sample's place: a
    callable that changes a copy of the graph (its nodes' models and populations,
    its edges' coefficients) in place, given the copy and the run index; without
    it every run simulates the graph as given. (The reference's Random123 draws
    are not reproduced.)"""

    def __init__(self, graph: MobilityGraph, t0: float, tmax: float, dt: float, num_runs: int,
                 sample=None, precision: int = N.PRECISION_FP64):
        if num_runs < 1:
            raise ValueError("num_runs must be at least 1")
        self._graph = graph
        self._t0, self._tmax, self._dt = float(t0), float(tmax), float(dt)
        self._num_runs = int(num_runs)
        self._sample = sample
        self._precision = precision

    @property
    def num_runs(self) -> int:
        return self._num_runs

    @property
    def t0(self) -> float:
        return self._t0

    @property
    def tmax(self) -> float:
        return self._tmax

    @property
    def dt(self) -> float:
        return self._dt

    @property
    def parameters(self) -> MobilityGraph:
        return self._graph

    def _sampled_graphs(self):
        """The sampled copies of the graph, one per run."""
        import copy
        runs = []
        for r in range(self._num_runs):
            g = copy.deepcopy(self._graph)
            if self._sample is not None:
                self._sample(g, r)
            for node in g._nodes:  # each run starts from its sampled populations
                node.property.result = TimeSeries(node.property.model.populations.numel())
                node.property.result.add_time_point(self._t0, node.property.model.populations.array())
            runs.append(g)
        return runs

    def _arrays(self, runs):
        return [_graph_arrays([n.property.model for n in g._nodes],
                              [n.property.result.get_last_value() for n in g._nodes],
                              [(e.start_node_idx, e.end_node_idx, e.property.coeffs) for e in g._edges])
                for g in runs]

    def run(self, handle_result=None):
        """Simulate every run; with handle_result(graph, run_index) each result
        graph is handed over in run order, else the result graphs are returned.
        A result graph's node results hold the state after every exchange."""
        runs = self._sampled_graphs()
        arrays = self._arrays(runs)
        batch = N.Batch(_context(), arrays, self._t0,
                        N.solver_opts(precision=self._precision, dt_exchange=self._dt, dt0=self._dt))
        try:
            t = self._t0
            while t < self._tmax:
                t_next = min(t + self._dt, self._tmax)
                if self._tmax - t_next < 1e-12 * max(1.0, abs(self._tmax)):
                    t_next = self._tmax
                batch.advance(t_next)
                t = t_next
                for g, a, st in zip(runs, arrays, batch.states()):
                    for v, node in enumerate(g._nodes):
                        node.property.result.add_time_point(t, st[v].reshape(a.n))
        finally:
            batch.close()
        if handle_result is None:
            return runs
        for r, g in enumerate(runs):
            handle_result(g, r)
        return None


class _StudySimulation:
    """osecir.Simulation as ParameterStudy.run hands it over: the run's sampled
    model and its result (every accepted step)."""

    def __init__(self, model: Model, result: TimeSeries):
        self._model = model
        self._result = result

    @property
    def model(self) -> Model:
        return self._model

    @property
    def result(self) -> TimeSeries:
        return self._result

    def get_result(self) -> TimeSeries:
        return self._result


class ParameterStudy:
    """osecir.ParameterStudy(model, t0, tmax, dt, num_runs) (bind_OdeParameterStudy,
    bindings/compartments/parameter_studies.h:56-86): num_runs sampled copies of
    one model, each simulated from t0 to tmax with initial step dt; all runs are
    integrated together on the GPU (one lane group per run). `sample(model_copy,
    run_index)` takes draw_sample's place, as for GraphParameterStudy."""

    def __init__(self, model: Model, t0: float, tmax: float, dt: float, num_runs: int, sample=None):
        if num_runs < 1:
            raise ValueError("num_runs must be at least 1")
        self._model = model
        self._t0, self._tmax, self._dt = float(t0), float(tmax), float(dt)
        self._num_runs = int(num_runs)
        self._sample = sample

    @property
    def num_runs(self) -> int:
        return self._num_runs

    @property
    def t0(self) -> float:
        return self._t0

    @property
    def tmax(self) -> float:
        return self._tmax

    @property
    def dt(self) -> float:
        return self._dt

    @property
    def parameters(self) -> Model:
        return self._model

    def _sampled_models(self) -> List[Model]:
        import copy
        runs = []
        for r in range(self._num_runs):
            m = copy.deepcopy(self._model)
            if self._sample is not None:
                self._sample(m, r)
            runs.append(m)
        return runs

    def run(self, handle_result=None):
        """Simulate every run; with handle_result(simulation, run_index) each is
        handed over in run order, else the simulations are returned."""
        models = self._sampled_models()
        g = _graph_arrays(models, [m.populations.array() for m in models])
        cap = 4096
        while True:
            try:
                res = _context().simulate(g, list(range(len(models))), self._t0, self._tmax, self._dt,
                                          max_points=cap)
                break
            except N.MgpuError as e:
                if e.code != _OUT_OF_RANGE or cap >= 1 << 22:
                    raise
                cap *= 4
        sims = []
        for m, (t, y) in zip(models, res):
            ts = TimeSeries(g.n)
            for k in range(t.size):
                ts.add_time_point(t[k], y[k])
            sims.append(_StudySimulation(m, ts))
        if handle_result is None:
            return sims
        for r, s in enumerate(sims):
            handle_result(s, r)
        return None
