"""Seeded synthetic ODE-SECIR workloads in the miogpu layout.

No public benchmark data exists for this path (the German county commuter
matrix is not available offline), so seeded synthetic inputs of the stated
shapes and value ranges stand in for it:

  single_node   : G=6 age groups, N_g ~ U[5e4, 5e5], E and INS ~ U[0, 1e-3] N_g,
                  contacts U[0.5, 10] with one damping 0.3 at day 20, stay
                  times U[2, 8], probabilities U[0.05, 0.5]; optional finite
                  test-and-trace / ICU capacities ("stress").
  mobility_graph: 400 such nodes, ~30 random out-edges per node, commuter
                  fractions min(lognormal(-4, 1), 0.2) per (edge, group) on the
                  mobile compartments S, E, INS, ISy, R.
  ensemble      : samples of one graph; per sample the transmission
                  probabilities, stay times and the damping value scaled by
                  U[0.8, 1.2] factors shared by all nodes of the sample
                  (ParameterStudy: global parameters drawn once per run).
  uneven_batch  : graphs with N ~ logU[1, 2000], G ~ U{1..6}, horizon
                  ~ U[30, 180] days, out-degree ~ U{0..min(50, N-1)}.
"""
from __future__ import annotations

import numpy as np

from . import layout as L

MOBILE = [L.S, L.E, L.INS, L.ISY, L.R]


def node_models(rng: np.random.Generator, G: int, count: int, stress: bool = False, damping_day: float = 20.0,
                damping_value: float = 0.3):
    """Parameters, contacts, damping caches and initial states of `count` nodes."""
    P = np.zeros((count, L.param_stride(G)))
    P[:, L.P_START_DAY] = 0.0
    P[:, L.P_SEASONALITY] = 0.0
    P[:, L.P_ICU_CAPACITY] = L.DBL_MAX
    P[:, L.P_TNT_CAPACITY] = L.DBL_MAX
    P[:, L.P_TNT_MAX_RISK] = 5.0

    def gp(k):
        i = L.group_param_index(k, 0, G)
        return slice(i, i + G)

    for k in (L.G_TIME_EXPOSED, L.G_TIME_INS, L.G_TIME_ISY, L.G_TIME_ISEV, L.G_TIME_ICRI):
        P[:, gp(k)] = rng.uniform(2.0, 8.0, (count, G))
    for k in (L.G_TRANSMISSION_PROB, L.G_REL_TRANSMISSION_NS, L.G_RECOVERED_PER_INS, L.G_RISK_FROM_SYMPTOMATIC,
              L.G_MAX_RISK_FROM_SYMPTOMATIC, L.G_SEVERE_PER_ISY, L.G_CRITICAL_PER_SEVERE, L.G_DEATHS_PER_CRITICAL):
        P[:, gp(k)] = rng.uniform(0.05, 0.5, (count, G))
    P[:, gp(L.G_MAX_RISK_FROM_SYMPTOMATIC)] = np.maximum(P[:, gp(L.G_MAX_RISK_FROM_SYMPTOMATIC)],
                                                         P[:, gp(L.G_RISK_FROM_SYMPTOMATIC)])
    P[:, gp(L.G_DEATHS_PER_SEVERE)] = 0.0

    Ng = rng.uniform(5e4, 5e5, (count, G))
    y = np.zeros((count, G, 10))
    y[:, :, L.E] = rng.uniform(0, 1e-3, (count, G)) * Ng
    y[:, :, L.INS] = rng.uniform(0, 1e-3, (count, G)) * Ng
    y[:, :, L.S] = Ng - y[:, :, L.E] - y[:, :, L.INS]
    if stress:
        total = Ng.sum(axis=1)
        P[:, L.P_TNT_CAPACITY] = 35.0 * total / 1e4
        P[:, L.P_ICU_CAPACITY] = 100.0 * total / 1e4

    base = rng.uniform(0.5, 10.0, (count, 1, G, G))
    mini = np.zeros_like(base)
    times = np.broadcast_to(np.array([L.DBL_LOWEST, damping_day, L.DBL_MAX]), (count, 1, 3)).copy()
    vals = np.zeros((count, 1, 3, G, G))
    vals[:, :, 1:] = damping_value
    return P, base, mini, times, vals, y.reshape(count, 10 * G)


def random_edges(rng: np.random.Generator, N: int, degrees: np.ndarray, exact: bool = False):
    """Directed edges without self-loops, sorted by (src, dst); degrees[v] targets per node."""
    if N < 2:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    degrees = np.minimum(degrees, N - 1)
    if exact:
        src, dst = [], []
        for v in range(N):
            d = int(degrees[v])
            if d == 0:
                continue
            t = rng.choice(N - 1, size=d, replace=False)
            t = t + (t >= v)
            src.append(np.full(d, v))
            dst.append(np.sort(t))
        if not src:
            return np.zeros(0, np.int32), np.zeros(0, np.int32)
        return np.concatenate(src).astype(np.int32), np.concatenate(dst).astype(np.int32)
    src = np.repeat(np.arange(N), degrees)
    t = rng.integers(0, N - 1, src.shape[0])
    dst = t + (t >= src)
    key = np.unique(src.astype(np.int64) * N + dst)
    return (key // N).astype(np.int32), (key % N).astype(np.int32)


MAX_OUT_FRACTION = 0.3


def edge_coefficients(rng: np.random.Generator, E: int, G: int, src: np.ndarray = None):
    """Commuter fractions min(lognormal(-4, 1), 0.2) per (edge, group), on S, E, INS, ISy, R.

    With ~30 out-edges the raw draws send ~90% (often >100%) of a node's
    group away every other half-day, which drives compartments negative in
    the reference semantics as well. The fractions of each (source, group)
    are therefore scaled down so that their sum is at most 0.3."""
    frac = np.minimum(rng.lognormal(-4.0, 1.0, (E, G)), 0.2)
    if src is not None and E:
        tot = np.zeros((int(src.max()) + 1, G))
        np.add.at(tot, src, frac)
        scale = np.minimum(1.0, MAX_OUT_FRACTION / np.maximum(tot, 1e-300))
        frac = frac * scale[src]
    c = np.zeros((E, G, 10))
    for comp in MOBILE:
        c[:, :, comp] = frac
    return c.reshape(E, 10 * G)


def single_node(seed: int = 0, G: int = 6, count: int = 1, stress: bool = False) -> L.GraphArrays:
    rng = np.random.default_rng(seed)
    P, base, mini, times, vals, y = node_models(rng, G, count, stress)
    return L.GraphArrays(G, P, base, mini, times, vals, y, np.zeros(0, np.int32), np.zeros(0, np.int32),
                         np.zeros((0, 10 * G)))


def mobility_graph(seed: int = 1, N: int = 400, G: int = 6, out_degree: int = 30, stress: bool = False
                   ) -> L.GraphArrays:
    rng = np.random.default_rng(seed)
    P, base, mini, times, vals, y = node_models(rng, G, N, stress)
    src, dst = random_edges(rng, N, np.full(N, out_degree), exact=True)
    coeff = edge_coefficients(rng, src.shape[0], G, src)
    return L.GraphArrays(G, P, base, mini, times, vals, y, src, dst, coeff)


def perturb(base: L.GraphArrays, rng: np.random.Generator) -> L.GraphArrays:
    """One ParameterStudy sample: transmission probabilities, stay times and the
    damping value scaled by U[0.8, 1.2], each factor shared by all nodes."""
    G = base.num_groups
    P = base.params.copy()
    f_beta = rng.uniform(0.8, 1.2, G)
    i = L.group_param_index(L.G_TRANSMISSION_PROB, 0, G)
    P[:, i:i + G] *= f_beta
    for k in (L.G_TIME_EXPOSED, L.G_TIME_INS, L.G_TIME_ISY, L.G_TIME_ISEV, L.G_TIME_ICRI):
        i = L.group_param_index(k, 0, G)
        P[:, i:i + G] *= rng.uniform(0.8, 1.2, G)
    f_damp = rng.uniform(0.8, 1.2)
    vals = base.damping_values * f_damp
    return L.GraphArrays(G, P, base.contact_baseline, base.contact_minimum, base.damping_times, vals,
                         base.init_state, base.edge_src, base.edge_dst, base.edge_coeff_baseline,
                         base.edge_coeff_minimum, base.edge_damping_times, base.edge_damping_values)


def ensemble(num_samples: int = 1024, seed: int = 2, N: int = 400, G: int = 6, out_degree: int = 30,
             base: L.GraphArrays = None):
    base = base if base is not None else mobility_graph(seed, N, G, out_degree)
    rng = np.random.default_rng(seed + 1000)
    return [perturb(base, rng) for _ in range(num_samples)]


def uneven_batch(num_graphs: int = 4096, seed: int = 3, max_nodes: int = 2000, max_degree: int = 50,
                 horizon=(30.0, 180.0), max_groups: int = 6):
    """Returns (graphs, horizons)."""
    rng = np.random.default_rng(seed)
    graphs, horizons = [], []
    for _ in range(num_graphs):
        N = int(round(np.exp(rng.uniform(0.0, np.log(max_nodes)))))
        N = max(N, 1)
        G = int(rng.integers(1, max_groups + 1))
        P, base, mini, times, vals, y = node_models(rng, G, N)
        deg = rng.integers(0, min(max_degree, max(N - 1, 0)) + 1, N)
        src, dst = random_edges(rng, N, deg)
        coeff = edge_coefficients(rng, src.shape[0], G, src)
        graphs.append(L.GraphArrays(G, P, base, mini, times, vals, y, src, dst, coeff))
        horizons.append(float(rng.uniform(*horizon)))
    return graphs, np.array(horizons)


def node_days(graphs, horizons) -> float:
    """Work unit of the metric: sum over instances of nodes x simulated days."""
    h = np.broadcast_to(np.asarray(horizons, np.float64), (len(graphs),))
    return float(sum(g.num_nodes * hh for g, hh in zip(graphs, h)))
