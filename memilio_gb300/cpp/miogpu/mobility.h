/*
 * miogpu/mobility.h — the metapopulation graph with the API of MEmilio's
 * mio::Graph (cpp/memilio/mobility/graph.h:144-303), SimulationNode and
 * MobilityEdge (metapopulation_mobility_instant.h:39-101,106-290,300-623),
 * make_mobility_sim / GraphSimulation (:656-678, graph_simulation.h:63-120)
 * and ParameterStudy (cpp/memilio/compartments/parameter_studies.h:47-374),
 * computing on the GPU through libmiogpu's batches:
 *
 *   GraphSimulation::advance -> mgpu_batch_advance (one batch per graph)
 *   ParameterStudy::run      -> every sampled graph in one batch
 *
 * Node results are recorded at every exchange boundary (every dt of the
 * graph simulation), not at every accepted integrator step.
 */
#ifndef MIOGPU_FACADE_MOBILITY_H
#define MIOGPU_FACADE_MOBILITY_H

#include "osecir.h"

#include <algorithm>
#include <functional>
#include <stdexcept>
#include <type_traits>

namespace miogpu
{

template <class NodePropertyT>
struct Node {
    template <class... Args>
    Node(int node_id, Args&&... args)
        : id(node_id)
        , property(std::forward<Args>(args)...)
    {
    }
    int id;
    NodePropertyT property;
};

template <class EdgePropertyT>
struct Edge {
    template <class... Args>
    Edge(size_t start, size_t end, Args&&... args)
        : start_node_idx(start)
        , end_node_idx(end)
        , property(std::forward<Args>(args)...)
    {
    }
    size_t start_node_idx;
    size_t end_node_idx;
    EdgePropertyT property;
};

/* mio::Graph: nodes in insertion order, edges kept sorted by (start, end);
 * adding an edge that exists replaces its property (graph.h:216-241). */
template <class NodePropertyT, class EdgePropertyT>
class Graph
{
public:
    using NodeProperty = NodePropertyT;
    using EdgeProperty = EdgePropertyT;

    Graph() = default;
    /* Takes nodes and edges as they are (graph.h:154-160); the edges must be
     * sorted by (start, end), as GraphBuilder::build leaves them. */
    Graph(std::vector<Node<NodePropertyT>>&& nodes, std::vector<Edge<EdgePropertyT>>&& edges)
        : m_nodes(std::move(nodes))
        , m_edges(std::move(edges))
    {
    }

    template <class... Args>
    Node<NodePropertyT>& add_node(int id, Args&&... args)
    {
        m_nodes.emplace_back(id, std::forward<Args>(args)...);
        return m_nodes.back();
    }
    template <class... Args>
    Edge<EdgePropertyT>& add_edge(size_t start, size_t end, Args&&... args)
    {
        if (start >= m_nodes.size() || end >= m_nodes.size()) {
            throw std::out_of_range("edge node index out of range");
        }
        Edge<EdgePropertyT> e(start, end, std::forward<Args>(args)...);
        auto it = std::lower_bound(m_edges.begin(), m_edges.end(), e, [](const auto& a, const auto& b) {
            return std::make_pair(a.start_node_idx, a.end_node_idx) < std::make_pair(b.start_node_idx, b.end_node_idx);
        });
        if (it != m_edges.end() && it->start_node_idx == start && it->end_node_idx == end) {
            *it = std::move(e);
            return *it;
        }
        return *m_edges.insert(it, std::move(e));
    }
    std::vector<Node<NodePropertyT>>& nodes()
    {
        return m_nodes;
    }
    const std::vector<Node<NodePropertyT>>& nodes() const
    {
        return m_nodes;
    }
    std::vector<Edge<EdgePropertyT>>& edges()
    {
        return m_edges;
    }
    const std::vector<Edge<EdgePropertyT>>& edges() const
    {
        return m_edges;
    }

private:
    std::vector<Node<NodePropertyT>> m_nodes;
    std::vector<Edge<EdgePropertyT>> m_edges;
};

/* mio::GraphBuilder (mobility/graph_builder.h): collects nodes and edges in any
 * order and builds the Graph in one go, sorting the edges by (start, end) once
 * (stable, so equal pairs keep their insertion order) instead of inserting each
 * edge in place. With make_unique, of several edges between the same nodes the
 * one added last is kept. (A graph with duplicate edges is refused by the
 * device batches, which need one edge per (start, end).) */
template <class NodePropertyT, class EdgePropertyT>
class GraphBuilder
{
public:
    using NodeProperty = NodePropertyT;
    using EdgeProperty = EdgePropertyT;

    GraphBuilder() = default;
    GraphBuilder(size_t num_nodes, size_t num_edges)
    {
        m_nodes.reserve(num_nodes);
        m_edges.reserve(num_edges);
    }
    template <class... Args>
    void add_node(int id, Args&&... args)
    {
        m_nodes.emplace_back(id, std::forward<Args>(args)...);
    }
    template <class... Args>
    void add_edge(size_t start_node_idx, size_t end_node_idx, Args&&... args)
    {
        if (start_node_idx >= m_nodes.size() || end_node_idx >= m_nodes.size()) {
            throw std::out_of_range("edge node index out of range");
        }
        m_edges.emplace_back(start_node_idx, end_node_idx, std::forward<Args>(args)...);
    }
    Graph<NodePropertyT, EdgePropertyT> build(bool make_unique = false) &&
    {
        std::stable_sort(m_edges.begin(), m_edges.end(), [](const auto& a, const auto& b) {
            return a.start_node_idx == b.start_node_idx ? a.end_node_idx < b.end_node_idx
                                                        : a.start_node_idx < b.start_node_idx;
        });
        if (make_unique && !m_edges.empty()) {
            std::vector<Edge<EdgePropertyT>> unique;
            unique.reserve(m_edges.size());
            for (size_t i = 0; i < m_edges.size(); ++i) {
                const bool last_of_pair = i + 1 == m_edges.size() ||
                                          m_edges[i + 1].start_node_idx != m_edges[i].start_node_idx ||
                                          m_edges[i + 1].end_node_idx != m_edges[i].end_node_idx;
                if (last_of_pair) {
                    unique.push_back(std::move(m_edges[i]));
                }
            }
            m_edges = std::move(unique);
        }
        return Graph<NodePropertyT, EdgePropertyT>(std::move(m_nodes), std::move(m_edges));
    }

private:
    std::vector<Node<NodePropertyT>> m_nodes;
    std::vector<Edge<EdgePropertyT>> m_edges;
};

/* Mobility coefficients of one edge: a vector over the 10G compartments with
 * baseline, minimum and dampings (MobilityCoefficientGroup with one matrix). */
class MobilityCoefficientGroup
{
public:
    MobilityCoefficientGroup(size_t num_matrices = 1, size_t n = 0)
        : m_coeffs(n, 1)
    {
        if (num_matrices != 1) {
            throw Error(MGPU_UNSUPPORTED, "one mobility coefficient matrix per edge");
        }
    }
    DampingMatrixExpression& operator[](size_t i)
    {
        if (i != 0) {
            throw std::out_of_range("one mobility coefficient matrix per edge");
        }
        return m_coeffs;
    }
    const DampingMatrixExpression& operator[](size_t i) const
    {
        return const_cast<MobilityCoefficientGroup*>(this)->operator[](i);
    }
    size_t get_num_matrices() const
    {
        return 1;
    }

private:
    DampingMatrixExpression m_coeffs;
};

/* Sets of flat compartment indices whose travelers are summed in the edge's
 * mobility results (MobilityParameters' save indices, :145-170). */
using SaveIndices = std::vector<std::vector<size_t>>;

/* mio::MobilityParameters (:106-290). */
template <typename FP = double>
class MobilityParameters
{
public:
    explicit MobilityParameters(const std::vector<FP>& coeffs, const SaveIndices& save_indices = {})
        : m_coeffs(1, coeffs.size())
        , m_save_indices(save_indices)
    {
        std::copy(coeffs.begin(), coeffs.end(), m_coeffs[0].get_baseline().data());
    }
    explicit MobilityParameters(const MobilityCoefficientGroup& coeffs, const SaveIndices& save_indices = {})
        : m_coeffs(coeffs)
        , m_save_indices(save_indices)
    {
    }
    /* The groups of compartments the edge's mobility results sum up (:241-244). */
    const SaveIndices& get_save_indices() const
    {
        return m_save_indices;
    }
    MobilityCoefficientGroup& get_coefficients()
    {
        return m_coeffs;
    }
    const MobilityCoefficientGroup& get_coefficients() const
    {
        return m_coeffs;
    }
    /* The edge's dynamic NPIs on the source's symptomatic infections (:237-244). */
    DynamicNPIs<FP>& get_dynamic_npis_infected()
    {
        return m_dynamic_npis;
    }
    const DynamicNPIs<FP>& get_dynamic_npis_infected() const
    {
        return m_dynamic_npis;
    }

private:
    MobilityCoefficientGroup m_coeffs;
    DynamicNPIs<FP> m_dynamic_npis;
    SaveIndices m_save_indices;
};

/* mio::MobilityEdge (:300-623): the edge property of a simulation graph. */
template <typename FP = double>
class MobilityEdge
{
public:
    explicit MobilityEdge(const MobilityParameters<FP>& params)
        : m_params(params)
        , m_save_indices(params.get_save_indices())
        , m_results(m_save_indices.size() + 1)
    {
    }
    MobilityEdge(const MobilityParameters<FP>& params, const SaveIndices& save_indices)
        : m_params(params)
        , m_save_indices(save_indices)
        , m_results(m_save_indices.size() + 1)
    {
    }
    explicit MobilityEdge(const std::vector<FP>& coeffs)
        : m_params(coeffs)
        , m_results(1)
    {
    }
    MobilityEdge(const std::vector<FP>& coeffs, const SaveIndices& save_indices)
        : m_params(coeffs)
        , m_save_indices(save_indices)
        , m_results(m_save_indices.size() + 1)
    {
    }
    /* The travelers' sums over the save-index sets and their total, one time
     * point per departure and per return (get_mobility_results, :371-383,
     * add_mobility_result_time_point, :423-447); empty without save indices. */
    TimeSeries<FP>& get_mobility_results()
    {
        return m_results;
    }
    const TimeSeries<FP>& get_mobility_results() const
    {
        return m_results;
    }
    const SaveIndices& get_save_indices() const
    {
        return m_save_indices;
    }
    const MobilityParameters<FP>& get_parameters() const
    {
        return m_params;
    }
    MobilityParameters<FP>& get_parameters()
    {
        return m_params;
    }
    /* The edge's NPI state (m_dynamic_npi). */
    DynamicNPIState& get_dynamic_npi_state()
    {
        return m_npi;
    }
    const DynamicNPIState& get_dynamic_npi_state() const
    {
        return m_npi;
    }

private:
    MobilityParameters<FP> m_params;
    DynamicNPIState m_npi;
    SaveIndices m_save_indices;
    TimeSeries<FP> m_results;
};

/* mio::SimulationNode (:39-101): a node's simulation and its results. */
template <class Sim>
class SimulationNode
{
public:
    template <class... Args>
    SimulationNode(Args&&... args)
        : m_simulation(std::forward<Args>(args)...)
        , m_last_state(m_simulation.get_result().get_last_value())
    {
    }
    Sim& get_simulation()
    {
        return m_simulation;
    }
    const Sim& get_simulation() const
    {
        return m_simulation;
    }
    decltype(auto) get_result()
    {
        return m_simulation.get_result();
    }
    decltype(auto) get_result() const
    {
        return m_simulation.get_result();
    }
    const std::vector<double>& get_last_state() const
    {
        return m_last_state;
    }
    void set_last_state(const double* v)
    {
        m_last_state.assign(v, v + m_last_state.size());
    }

private:
    Sim m_simulation;
    std::vector<double> m_last_state;
};

namespace detail
{

/* Does a node simulation keep flow results (FlowSimulation::get_flows)? */
template <class S, class = void>
struct has_flows : std::false_type {
};
template <class S>
struct has_flows<S, std::void_t<decltype(std::declval<S&>().get_flows())>> : std::true_type {
};

/* The arrays of one graph in the layout of include/miogpu_layout.h. */
struct GraphArrays {
    int N = 0, G = 0, E = 0, M = 0, K = 0, Ke = 0;
    std::vector<double> params, contact_baseline, contact_minimum, damping_times, damping_values, state;
    std::vector<int32_t> src, dst;
    std::vector<double> coeff_baseline, coeff_minimum, edge_damping_times, edge_damping_values;

    mgpu_graph view() const
    {
        mgpu_graph g{};
        g.num_nodes               = N;
        g.num_groups              = G;
        g.num_edges               = E;
        g.num_contact_matrices    = M;
        g.num_damping_points      = K;
        g.num_edge_damping_points = Ke;
        g.params                  = params.data();
        g.contact_baseline        = contact_baseline.data();
        g.contact_minimum         = contact_minimum.data();
        g.damping_times           = K ? damping_times.data() : nullptr;
        g.damping_values          = K ? damping_values.data() : nullptr;
        g.init_state              = state.data();
        g.edge_src                = E ? src.data() : nullptr;
        g.edge_dst                = E ? dst.data() : nullptr;
        g.edge_coeff_baseline     = E ? coeff_baseline.data() : nullptr;
        g.edge_coeff_minimum      = E ? coeff_minimum.data() : nullptr;
        g.edge_damping_times      = Ke ? edge_damping_times.data() : nullptr;
        g.edge_damping_values     = Ke ? edge_damping_values.data() : nullptr;
        return g;
    }
};

/* Packs models (one per node, with its current state) and edge coefficients. */
template <class ModelT, class EdgeT>
GraphArrays pack_graph(const std::vector<const ModelT*>& models, const std::vector<const std::vector<double>*>& states,
                       const std::vector<Edge<EdgeT>>& edges, std::function<const MobilityParameters<double>&(const EdgeT&)> params_of,
                       int extra_damping_points = 0, int extra_edge_damping_points = 0)
{
    GraphArrays a;
    a.N = (int)models.size();
    if (a.N == 0) {
        throw Error(MGPU_INVALID_VALUE, "graph without nodes");
    }
    a.G = (int)models[0]->num_groups();
    std::vector<osecir::NodeRecord> recs;
    int K = 0;
    for (size_t v = 0; v < models.size(); ++v) {
        if ((int)models[v]->num_groups() != a.G) {
            throw Error(MGPU_INVALID_VALUE, "all nodes of a graph need the same number of age groups");
        }
        recs.push_back(models[v]->pack(states[v]));
        K = std::max(K, recs.back().K);
    }
    a.M = recs[0].M;
    if (extra_damping_points > 0) {
        K = std::max(K, 2) + extra_damping_points; // room for dampings added at run time
    }
    a.K = K;
    const size_t GG = (size_t)a.G * a.G;
    for (auto& r : recs) {
        if (r.M != a.M) {
            throw Error(MGPU_INVALID_VALUE, "all nodes of a graph need the same number of contact matrices");
        }
        a.params.insert(a.params.end(), r.params.begin(), r.params.end());
        a.contact_baseline.insert(a.contact_baseline.end(), r.contact_baseline.begin(), r.contact_baseline.end());
        a.contact_minimum.insert(a.contact_minimum.end(), r.contact_minimum.begin(), r.contact_minimum.end());
        a.state.insert(a.state.end(), r.state.begin(), r.state.end());
        if (K > 0) {
            // pad every matrix's cache to K points (DBL_MAX times repeating the last matrix)
            for (int m = 0; m < r.M; ++m) {
                for (int k = 0; k < K; ++k) {
                    if (k < r.K) {
                        a.damping_times.push_back(r.damping_times[(size_t)(m * r.K + k)]);
                        a.damping_values.insert(a.damping_values.end(),
                                                r.damping_values.begin() + (long)(((size_t)m * r.K + k) * GG),
                                                r.damping_values.begin() + (long)(((size_t)m * r.K + k + 1) * GG));
                    }
                    else if (r.K == 0) {
                        // no dampings: a zero cache
                        a.damping_times.push_back(k == 0 ? std::numeric_limits<double>::lowest()
                                                         : std::numeric_limits<double>::max());
                        a.damping_values.insert(a.damping_values.end(), GG, 0.0);
                    }
                    else {
                        a.damping_times.push_back(std::numeric_limits<double>::max());
                        a.damping_values.insert(a.damping_values.end(),
                                                r.damping_values.begin() + (long)(((size_t)m * r.K + r.K - 1) * GG),
                                                r.damping_values.begin() + (long)(((size_t)m * r.K + r.K) * GG));
                    }
                }
            }
        }
    }
    const size_t n = (size_t)a.G * osecir::num_compartments;
    a.E            = (int)edges.size();
    std::vector<const DampingMatrixExpression*> ecs;
    for (auto& e : edges) {
        const auto& c = params_of(e.property).get_coefficients()[0];
        if (c.get_baseline().size() != n) {
            throw Error(MGPU_INVALID_VALUE, "edge coefficients need 10 G entries");
        }
        a.src.push_back((int32_t)e.start_node_idx);
        a.dst.push_back((int32_t)e.end_node_idx);
        a.coeff_baseline.insert(a.coeff_baseline.end(), c.get_baseline().data(), c.get_baseline().data() + n);
        a.coeff_minimum.insert(a.coeff_minimum.end(), c.get_minimum().data(), c.get_minimum().data() + n);
        ecs.push_back(&c);
    }
    a.Ke = edges.empty() ? 0 : flatten_damping_caches(ecs, a.edge_damping_times, a.edge_damping_values);
    if (extra_edge_damping_points > 0 && !edges.empty()) {
        // room for coefficient dampings added at run time: pad every edge's cache
        const int Ke = std::max(a.Ke, 2) + extra_edge_damping_points;
        std::vector<double> t, v;
        for (size_t e = 0; e < edges.size(); ++e) {
            for (int k = 0; k < Ke; ++k) {
                if (a.Ke && k < a.Ke) {
                    t.push_back(a.edge_damping_times[e * (size_t)a.Ke + (size_t)k]);
                    v.insert(v.end(), a.edge_damping_values.begin() + (long)((e * (size_t)a.Ke + (size_t)k) * n),
                             a.edge_damping_values.begin() + (long)((e * (size_t)a.Ke + (size_t)k + 1) * n));
                }
                else if (a.Ke) {
                    t.push_back(std::numeric_limits<double>::max());
                    v.insert(v.end(), a.edge_damping_values.begin() + (long)((e * (size_t)a.Ke + (size_t)a.Ke - 1) * n),
                             a.edge_damping_values.begin() + (long)((e * (size_t)a.Ke + (size_t)a.Ke) * n));
                }
                else {
                    t.push_back(k == 0 ? std::numeric_limits<double>::lowest() : std::numeric_limits<double>::max());
                    v.insert(v.end(), n, 0.0);
                }
            }
        }
        a.Ke                  = Ke;
        a.edge_damping_times  = std::move(t);
        a.edge_damping_values = std::move(v);
    }
    return a;
}

} // namespace detail

/* mio::GraphSimulation over a graph of SimulationNode<Simulation> and
 * MobilityEdge (graph_simulation.h:63-120). */
template <class GraphT>
class GraphSimulation
{
public:
    GraphSimulation(double t0, double dt, GraphT&& graph)
        : m_t(t0)
        , m_dt(dt)
        , m_graph(std::move(graph))
    {
    }
    GraphSimulation(GraphSimulation&&)            = default;
    GraphSimulation& operator=(GraphSimulation&&) = default;
    ~GraphSimulation()
    {
        if (m_batch) {
            mgpu_batch_destroy(m_batch);
        }
    }

    /* MGPU_PRECISION_FP64 (default: the reference's arithmetic on the batched
     * solver) or MGPU_PRECISION_MIXED; set before the first advance. */
    void set_precision(int precision)
    {
        m_precision = precision;
    }
    /* Record node results at every exchange boundary (default) or only at tmax. */
    void set_record_boundaries(bool on)
    {
        m_record = on;
    }

    /* Alternates node solves and mobility exchanges up to tmax
     * (GraphSimulation::advance, graph_simulation.h:101-120). */
    void advance(double tmax)
    {
        ensure_batch();
        mgpu_context* ctx = Device::context();
        if (!m_save_sets.empty()) {
            arm_mobility_results(tmax);
        }
        // NPI checks need every exchange boundary; without them and without
        // recording, one batch advance covers the whole span
        const bool per_interval = m_record || m_any_npis || m_any_edge_npis;
        while (m_t < tmax) {
            double t_next = per_interval ? std::min(m_t + m_dt, tmax) : tmax;
            if (tmax - t_next < 1e-12 * std::max(1.0, std::abs(tmax))) {
                t_next = tmax;
            }
            if (m_any_npis) {
                apply_dynamic_npis(t_next);
            }
            if (m_any_edge_npis) {
                // the edges' NPI checks see the nodes' states between their solves and the exchange
                check(mgpu_batch_step_nodes(m_batch, t_next, nullptr), ctx, "mgpu_batch_step_nodes");
                apply_edge_npis(t_next);
                check(mgpu_batch_step_exchange(m_batch), ctx, "mgpu_batch_step_exchange");
            }
            else {
                check(mgpu_batch_advance(m_batch, t_next, nullptr), ctx, "mgpu_batch_advance");
            }
            m_t = t_next;
            if (m_record || m_t >= tmax) {
                record();
            }
        }
        if (!m_save_sets.empty()) {
            collect_mobility_results();
        }
    }
    double get_t() const
    {
        return m_t;
    }
    GraphT& get_graph() &
    {
        return m_graph;
    }
    const GraphT& get_graph() const&
    {
        return m_graph;
    }
    GraphT&& get_graph() &&
    {
        return std::move(m_graph);
    }
    mgpu_batch* batch()
    {
        ensure_batch();
        return m_batch;
    }

private:
    /* Room for damping-cache points added by dynamic NPIs during a run. */
    static constexpr int kNpiDampingPoints = 64;

    /* The dynamic-NPI check of every node at the start of its next chunk
     * (osecir::Simulation::advance, model.h:299-350, reached through
     * SimulationNode::advance): enacted NPIs change the node's contact
     * dampings, whose new cache goes to the batch. A chunk ends at the active
     * NPI's end (model.h:352-357); that end must lie on the exchange grid. */
    void apply_dynamic_npis(double t_next)
    {
        mgpu_context* ctx = Device::context();
        std::vector<double> sums; // without recorded results: the symptomatic infections per node, summed on the device
        if (!m_record) {
            sums.resize(m_graph.nodes().size());
            check(mgpu_batch_get_compartment_sums(m_batch, MGPU_ISY, sums.data()), ctx,
                  "mgpu_batch_get_compartment_sums");
        }
        auto& nodes = m_graph.nodes();
        for (size_t v = 0; v < nodes.size(); ++v) {
            auto& sim   = nodes[v].property.get_simulation();
            auto& model = sim.get_model();
            using FPT   = double;
            const auto& npis = model.parameters.template get<osecir::DynamicNPIsInfectedSymptoms<FPT>>();
            if (npis.get_thresholds().empty()) {
                continue;
            }
            const double inf_rel =
                m_record ? osecir::get_infections_relative(sim, m_t, nodes[v].property.get_result().get_last_value())
                         : osecir::get_infections_relative_of_sum(sim, sums[v]);
            auto& contacts = model.parameters.template get<osecir::ContactPatterns<FPT>>();
            if (check_dynamic_npis(npis, sim.get_dynamic_npi_state(), contacts, m_t, inf_rel)) {
                upload_dampings((int)v, contacts);
            }
            const double te = sim.get_dynamic_npi_state().t_end;
            if (m_t < te && te < t_next - 1e-12 * std::max(1.0, std::abs(t_next))) {
                throw Error(MGPU_UNSUPPORTED, "a dynamic NPI ends inside an exchange interval: choose its duration, "
                                              "delay and directive end on the exchange grid");
            }
        }
    }

    /* MobilityEdge::apply_mobility's NPI check (metapopulation_mobility_instant.h:
     * 549-566) for every edge with thresholds, on its source's state before the
     * exchange at t; enacted NPIs change the edge's coefficient cache. */
    void apply_edge_npis(double t)
    {
        mgpu_context* ctx = Device::context();
        std::vector<double> sums(m_graph.nodes().size()); // the sources' symptomatic infections after their solves
        check(mgpu_batch_get_compartment_sums(m_batch, MGPU_ISY, sums.data()), ctx, "mgpu_batch_get_compartment_sums");
        const size_t n = (size_t)m_arrays.G * osecir::num_compartments;
        auto& edges    = m_graph.edges();
        for (size_t e = 0; e < edges.size(); ++e) {
            auto& params     = edges[e].property.get_parameters();
            const auto& npis = params.get_dynamic_npis_infected();
            if (npis.get_thresholds().empty()) {
                continue;
            }
            const size_t u      = edges[e].start_node_idx;
            const auto& src_sim = m_graph.nodes()[u].property.get_simulation();
            if (!check_edge_dynamic_npis(npis, edges[e].property.get_dynamic_npi_state(), params.get_coefficients(), t,
                                         osecir::get_infections_relative_of_sum(src_sim, sums[u]))) {
                continue;
            }
            std::vector<double> times;
            std::vector<Matrix> vals;
            params.get_coefficients()[0].get_dampings().cache(times, vals);
            if ((int)times.size() > m_arrays.Ke) {
                throw Error(MGPU_UNSUPPORTED, "edge NPIs exceeded the coefficient-cache capacity of the batch");
            }
            std::vector<double> flat;
            for (auto& m : vals) {
                flat.insert(flat.end(), m.data(), m.data() + n);
            }
            check(mgpu_batch_set_edge_damping_cache(m_batch, 0, (int32_t)e, (int32_t)times.size(), times.data(),
                                                    flat.data()),
                  ctx, "mgpu_batch_set_edge_damping_cache");
        }
    }

    void upload_dampings(int v, const ContactMatrixGroup& contacts)
    {
        const int K     = m_arrays.K;
        const size_t GG = (size_t)m_arrays.G * m_arrays.G;
        for (size_t m = 0; m < contacts.get_num_matrices(); ++m) {
            std::vector<double> times;
            std::vector<Matrix> vals;
            contacts[m].get_dampings().cache(times, vals);
            if ((int)times.size() > K) {
                throw Error(MGPU_UNSUPPORTED, "dynamic NPIs exceeded the damping-cache capacity of the batch");
            }
            std::vector<double> flat;
            for (auto& mat : vals) {
                flat.insert(flat.end(), mat.data(), mat.data() + GG);
            }
            check(mgpu_batch_set_damping_cache(m_batch, 0, v, (int32_t)m, (int32_t)times.size(), times.data(),
                                               flat.data()),
                  Device::context(), "mgpu_batch_set_damping_cache");
        }
    }

    /* Commuter statistics of this advance: recording restarts with room for
     * one time point per exchange up to tmax. */
    void arm_mobility_results(double tmax)
    {
        std::vector<int32_t> offsets(1, 0), indices;
        for (auto& set : m_save_sets) {
            for (size_t j : set) {
                indices.push_back((int32_t)j);
            }
            offsets.push_back((int32_t)indices.size());
        }
        indices.push_back(0); // never empty
        const int32_t capacity = (int32_t)std::ceil((tmax - m_t) / m_dt + 1e-9) + 1;
        check(mgpu_batch_set_commuter_stats(m_batch, 0, (int32_t)m_save_sets.size(), offsets.data(), indices.data(),
                                            std::max(capacity, 1)),
              Device::context(), "mgpu_batch_set_commuter_stats");
        m_stats_capacity = std::max(capacity, 1);
    }
    /* Appends the recorded time points to every edge with save indices. */
    void collect_mobility_results()
    {
        auto& edges     = m_graph.edges();
        const size_t E  = edges.size();
        const size_t S1 = m_save_sets.size() + 1;
        std::vector<int32_t> counts(std::max<size_t>(E, 1));
        std::vector<double> times(std::max<size_t>(E, 1) * (size_t)m_stats_capacity);
        std::vector<double> values(times.size() * S1);
        check(mgpu_batch_get_commuter_stats(m_batch, 0, counts.data(), times.data(), values.data()),
              Device::context(), "mgpu_batch_get_commuter_stats");
        for (size_t e = 0; e < E; ++e) {
            auto& prop = edges[e].property;
            if (prop.get_save_indices().empty()) {
                continue;
            }
            for (int32_t k = 0; k < counts[e]; ++k) {
                const size_t row = e * (size_t)m_stats_capacity + (size_t)k;
                prop.get_mobility_results().add_time_point(times[row], values.data() + row * S1);
            }
        }
    }

    void ensure_batch()
    {
        if (m_batch) {
            return;
        }
        // the edges' save indices: the device records one set list per graph
        m_save_sets.clear();
        for (auto& e : m_graph.edges()) {
            const auto& si = e.property.get_save_indices();
            if (si.empty()) {
                continue;
            }
            if (!m_save_sets.empty() && si != m_save_sets) {
                throw Error(MGPU_UNSUPPORTED, "edges of one graph with different save indices");
            }
            m_save_sets = si;
        }
        std::vector<const typename std::decay_t<decltype(m_graph.nodes()[0].property.get_simulation().get_model())>*>
            models;
        std::vector<std::vector<double>> states;
        for (auto& nd : m_graph.nodes()) {
            models.push_back(&nd.property.get_simulation().get_model());
            states.push_back(nd.property.get_result().get_last_value());
        }
        std::vector<const std::vector<double>*> sp;
        for (auto& s : states) {
            sp.push_back(&s);
        }
        using EdgeT    = typename GraphT::EdgeProperty;
        m_any_edge_npis = false;
        for (auto& e : m_graph.edges()) {
            m_any_edge_npis = m_any_edge_npis || !e.property.get_parameters().get_dynamic_npis_infected()
                                                      .get_thresholds()
                                                      .empty();
        }
        m_any_npis = false;
        for (auto* mdl : models) {
            m_any_npis = m_any_npis || !mdl->parameters.template get<osecir::DynamicNPIsInfectedSymptoms<double>>()
                                            .get_thresholds()
                                            .empty();
        }
        m_arrays       = detail::pack_graph<typename std::decay_t<decltype(*models[0])>, EdgeT>(
            models, sp, m_graph.edges(),
            [](const EdgeT& e) -> const MobilityParameters<double>& {
                return e.get_parameters();
            },
            m_any_npis ? kNpiDampingPoints : 0, m_any_edge_npis ? kNpiDampingPoints : 0);
        mgpu_graph g     = m_arrays.view();
        mgpu_solver_opts o;
        mgpu_default_solver_opts(&o);
        o.precision   = m_precision;
        o.dt_exchange = m_dt;
        if (!m_graph.nodes().empty()) {
            const auto& sim = m_graph.nodes()[0].property.get_simulation();
            o.integrator    = sim.get_integrator_core().opts();
            o.dt0           = sim.get_dt();
        }
        mgpu_context* ctx = Device::context();
        check(mgpu_batch_create(ctx, &g, 1, m_t, &o, &m_batch), ctx, "mgpu_batch_create");
        using SimT = std::decay_t<decltype(m_graph.nodes()[0].property.get_simulation())>;
        if constexpr (detail::has_flows<SimT>::value) {
            // FlowSimulation nodes: the device sums their flows from here on
            check(mgpu_batch_set_flow_recording(m_batch, 1), ctx, "mgpu_batch_set_flow_recording");
            m_flow_offsets.clear();
            for (auto& nd : m_graph.nodes()) {
                m_flow_offsets.push_back(nd.property.get_simulation().get_flows().get_last_value());
            }
        }
    }
    void record()
    {
        mgpu_context* ctx = Device::context();
        const size_t n    = (size_t)m_arrays.G * osecir::num_compartments;
        std::vector<double> st((size_t)m_arrays.N * n);
        check(mgpu_batch_get_state(m_batch, st.data()), ctx, "mgpu_batch_get_state");
        for (size_t v = 0; v < m_graph.nodes().size(); ++v) {
            auto& nd = m_graph.nodes()[v].property;
            nd.get_result().add_time_point(m_t, st.data() + v * n);
            nd.set_last_state(st.data() + v * n);
        }
        using SimT = std::decay_t<decltype(m_graph.nodes()[0].property.get_simulation())>;
        if constexpr (detail::has_flows<SimT>::value) {
            // the flows of the nodes' own models at the same time (mobility moves people without flows)
            const size_t nf = (size_t)m_arrays.G * MGPU_NUM_FLOWS;
            std::vector<double> fl((size_t)m_arrays.N * nf);
            check(mgpu_batch_get_flows(m_batch, fl.data()), ctx, "mgpu_batch_get_flows");
            for (size_t v = 0; v < m_graph.nodes().size(); ++v) {
                std::vector<double> acc(m_flow_offsets[v]);
                for (size_t q = 0; q < nf; ++q) {
                    acc[q] += fl[v * nf + q];
                }
                m_graph.nodes()[v].property.get_simulation().get_flows().add_time_point(m_t, acc);
            }
        }
    }

    double m_t, m_dt;
    GraphT m_graph;
    int m_precision   = MGPU_PRECISION_FP64;
    bool m_record     = true;
    bool m_any_npis   = false;
    bool m_any_edge_npis = false;
    mgpu_batch* m_batch = nullptr;
    detail::GraphArrays m_arrays;
    SaveIndices m_save_sets; // the edges' save indices (all equal)
    std::vector<std::vector<double>> m_flow_offsets; // FlowSimulation nodes: their flows when the batch began
    int32_t m_stats_capacity = 0;
};

template <class Sim>
using MobilitySimGraph = Graph<SimulationNode<Sim>, MobilityEdge<double>>;

/* make_mobility_sim (:656-678). */
template <class Sim>
GraphSimulation<MobilitySimGraph<Sim>> make_mobility_sim(double t0, double dt, MobilitySimGraph<Sim>&& graph)
{
    return GraphSimulation<MobilitySimGraph<Sim>>(t0, dt, std::move(graph));
}
template <class Sim>
GraphSimulation<MobilitySimGraph<Sim>> make_mobility_sim(double t0, double dt, const MobilitySimGraph<Sim>& graph)
{
    MobilitySimGraph<Sim> copy = graph;
    return GraphSimulation<MobilitySimGraph<Sim>>(t0, dt, std::move(copy));
}

/* Result of one run of a ParameterStudy: the sampled graph's node states at tmax. */
struct StudyResult {
    size_t run_idx = 0;
    double t       = 0.0;
    int num_groups = 0;
    std::vector<std::vector<double>> node_states; // [node][10G]
};

/* mio::ParameterStudy (parameter_studies.h:47-374) over graphs of models and
 * mobility parameters: run() samples num_runs graphs on the host and solves
 * them all in one batch on the GPU. */
template <class Sim>
class ParameterStudy
{
public:
    using Model     = typename Sim::Model;
    using GraphType = Graph<Model, MobilityParameters<double>>;

    ParameterStudy(const GraphType& graph, double t0, double tmax, double dt_graph_sim, size_t num_runs)
        : m_graph(graph)
        , m_t0(t0)
        , m_tmax(tmax)
        , m_dt(dt_graph_sim)
        , m_num_runs(num_runs)
    {
    }
    void set_precision(int precision)
    {
        m_precision = precision;
    }
    void set_integrator_core(const IntegratorCore& core)
    {
        m_core = core;
    }

    /* sample_graph(const GraphType&) -> GraphType; result_processing(StudyResult, run_idx) -> R. */
    template <class SampleGraphFn, class HandleResultFn>
    auto run(SampleGraphFn sample_graph, HandleResultFn result_processing)
        -> std::vector<decltype(result_processing(std::declval<StudyResult>(), size_t(0)))>
    {
        std::vector<GraphType> graphs;
        graphs.reserve(m_num_runs);
        for (size_t r = 0; r < m_num_runs; ++r) {
            graphs.push_back(sample_graph(m_graph));
        }
        std::vector<detail::GraphArrays> arrays;
        std::vector<mgpu_graph> views;
        for (auto& g : graphs) {
            std::vector<const Model*> models;
            std::vector<const std::vector<double>*> states;
            for (auto& nd : g.nodes()) {
                models.push_back(&nd.property);
                states.push_back(&nd.property.populations.array());
            }
            arrays.push_back(detail::pack_graph<Model, MobilityParameters<double>>(
                models, states, g.edges(), [](const MobilityParameters<double>& p) -> const MobilityParameters<double>& {
                    return p;
                }));
        }
        for (auto& a : arrays) {
            views.push_back(a.view());
        }
        mgpu_solver_opts o;
        mgpu_default_solver_opts(&o);
        o.precision       = m_precision;
        o.dt_exchange     = m_dt;
        o.integrator      = m_core.opts();
        mgpu_context* ctx = Device::context();
        mgpu_batch* b     = nullptr;
        check(mgpu_batch_create(ctx, views.data(), (int32_t)views.size(), m_t0, &o, &b), ctx, "mgpu_batch_create");
        std::vector<decltype(result_processing(std::declval<StudyResult>(), size_t(0)))> out;
        try {
            check(mgpu_batch_advance(b, m_tmax, nullptr), ctx, "mgpu_batch_advance");
            for (size_t r = 0; r < arrays.size(); ++r) {
                const size_t n = (size_t)arrays[r].G * osecir::num_compartments;
                std::vector<double> st((size_t)arrays[r].N * n);
                check(mgpu_batch_get_graph_state(b, (int32_t)r, st.data()), ctx, "mgpu_batch_get_graph_state");
                StudyResult res;
                res.run_idx    = r;
                res.t          = m_tmax;
                res.num_groups = arrays[r].G;
                for (int v = 0; v < arrays[r].N; ++v) {
                    res.node_states.emplace_back(st.begin() + (long)(v * n), st.begin() + (long)((v + 1) * n));
                }
                out.push_back(result_processing(std::move(res), r));
            }
        }
        catch (...) {
            mgpu_batch_destroy(b);
            throw;
        }
        mgpu_batch_destroy(b);
        return out;
    }

private:
    GraphType m_graph;
    double m_t0, m_tmax, m_dt;
    size_t m_num_runs;
    int m_precision = MGPU_PRECISION_FP64;
    IntegratorCore m_core;
};

} // namespace miogpu

#endif // MIOGPU_FACADE_MOBILITY_H
