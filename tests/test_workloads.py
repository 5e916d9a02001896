"""Synthetic workload generators: shapes, ranges, edge order; the graph view of the arrays."""
import numpy as np

from memilio_gb300 import layout as L
from memilio_gb300 import workloads as W


def test_single_node_ranges():
    g = W.single_node(seed=0, G=6, count=50)
    y = g.init_state.reshape(50, 6, 10)
    Ng = y.sum(axis=2)
    assert np.all((Ng >= 5e4) & (Ng <= 5e5))
    assert np.all(y[:, :, L.E] <= 1e-3 * Ng + 1e-9) and np.all(y[:, :, L.INS] <= 1e-3 * Ng + 1e-9)
    assert np.all(y[:, :, [L.INSC, L.ISY, L.ISYC, L.ISEV, L.ICRI, L.R, L.D]] == 0)
    b = g.contact_baseline
    assert b.min() >= 0.5 and b.max() <= 10
    i = L.group_param_index(L.G_TIME_EXPOSED, 0, 6)
    assert g.params[:, i:i + 30].min() >= 2 and g.params[:, i:i + 30].max() <= 8
    assert list(g.damping_times[0, 0]) == [L.DBL_LOWEST, 20.0, L.DBL_MAX]


def test_graph_edges_sorted_no_self_loops():
    g = W.mobility_graph(seed=1, N=50, out_degree=10)
    key = g.edge_src.astype(np.int64) * 50 + g.edge_dst
    assert np.all(np.diff(key) > 0)
    assert np.all(g.edge_src != g.edge_dst)
    assert np.all(np.bincount(g.edge_src, minlength=50) == 10)


def test_commuter_fractions_bounded():
    g = W.mobility_graph(seed=1, N=100, out_degree=30)
    c = g.edge_coeff_baseline.reshape(-1, 6, 10)
    assert c.max() <= 0.2
    assert np.all(c[:, :, [L.INSC, L.ISYC, L.ISEV, L.ICRI, L.D]] == 0)
    tot = np.zeros((100, 6))
    np.add.at(tot, g.edge_src, c[:, :, L.S])
    assert tot.max() <= W.MAX_OUT_FRACTION + 1e-12


def test_ensemble_shares_topology_and_perturbs():
    ens = W.ensemble(num_samples=4, N=20, out_degree=5)
    assert all(np.shares_memory(e.edge_src, ens[0].edge_src) for e in ens)
    i = L.group_param_index(L.G_TRANSMISSION_PROB, 0, 6)
    assert not np.allclose(ens[0].params[:, i], ens[1].params[:, i])


def test_uneven_batch_distribution():
    graphs, h = W.uneven_batch(num_graphs=64, seed=3)
    assert all(1 <= g.num_nodes <= 2000 for g in graphs)
    assert all(1 <= g.num_groups <= 6 for g in graphs)
    assert np.all((h >= 30) & (h <= 180))


def test_graph_view_follows_its_arrays():
    # the mgpu_graph view is kept while the arrays are the same objects (their
    # contents may change in place) and rebuilt when an array is replaced
    g = W.mobility_graph(seed=7, N=12, G=2, out_degree=3)
    v1 = g.as_ctypes()
    g.init_state[0, 0] += 1.0
    assert g.as_ctypes() is v1
    g.init_state = g.init_state.copy()
    v2 = g.as_ctypes()
    assert v2 is not v1
    assert v2.init_state == g.init_state.ctypes.data
    assert v2.edge_src == v1.edge_src and v2.params == v1.params
