// facade_check — drives the C++ facade for the Python tests and prints JSON.
//
//   facade_check dampings   host only: damping caches of several damping lists
//   facade_check pack       host only: the node/edge arrays of a small graph
//   facade_check builder    host only: GraphBuilder against Graph::add_edge
//   facade_check simulate   GPU: Simulation::advance in two pieces and in one
//   facade_check flows      GPU: simulate_flows (FlowSimulation)
//   facade_check graph      GPU: make_mobility_sim(...).advance, every boundary
//   facade_check study      GPU: ParameterStudy over 4 sampled graphs
//   facade_check commuters  GPU: the edges' mobility results (commuter statistics)
//   facade_check flows_graph  GPU: a graph of FlowSimulation nodes next to Simulation nodes
//   facade_check npi_logic  host only: implement_dynamic_npis and the NPI check
//                           of Simulation::advance with the state held fixed
//   facade_check npi_graph  GPU: a graph simulation with dynamic NPIs (FP64 and mixed)
//   facade_check npi_edges  GPU: the same with dynamic NPIs on the mobility edges too
//   facade_check interpolate  host only: interpolate_simulation_result of small series
//
// The Python side rebuilds the same inputs from the printed arrays and checks
// the outputs against the FP64 oracle.
#include "miogpu/mobility.h"

#include <cstdio>
#include <cstring>
#include <random>

using namespace miogpu;
using namespace miogpu::osecir;

namespace
{

void print_vec(const char* key, const std::vector<double>& v, bool comma = true)
{
    std::printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); ++i) {
        std::printf("%s%.17g", i ? ", " : "", v[i] == std::numeric_limits<double>::max() ? 1.7976931348623157e308
                                                                                         : v[i]);
    }
    std::printf("]%s\n", comma ? "," : "");
}

Model<double> make_model(int G, unsigned seed)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    auto U = [&](double a, double b) {
        return a + (b - a) * u(rng);
    };
    Model<double> m(G);
    auto& p = m.parameters;
    p.get<Seasonality<double>>()        = 0.1;
    p.get<StartDay<double>>()           = 40.0;
    p.get<TestAndTraceCapacity<double>>() = 60.0;
    p.get<ICUCapacity<double>>()        = 30.0;
    for (int i = 0; i < G; ++i) {
        const AgeGroup g((size_t)i);
        p.get<TimeExposed<double>>()[g]                       = U(2, 5);
        p.get<TimeInfectedNoSymptoms<double>>()[g]            = U(2, 5);
        p.get<TimeInfectedSymptoms<double>>()[g]              = U(4, 8);
        p.get<TimeInfectedSevere<double>>()[g]                = U(5, 10);
        p.get<TimeInfectedCritical<double>>()[g]              = U(5, 10);
        p.get<TransmissionProbabilityOnContact<double>>()[g]  = U(0.05, 0.15);
        p.get<RelativeTransmissionNoSymptoms<double>>()[g]    = U(0.5, 1.0);
        p.get<RecoveredPerInfectedNoSymptoms<double>>()[g]    = U(0.1, 0.3);
        p.get<RiskOfInfectionFromSymptomatic<double>>()[g]    = U(0.1, 0.3);
        p.get<MaxRiskOfInfectionFromSymptomatic<double>>()[g] = U(0.3, 0.5);
        p.get<SeverePerInfectedSymptoms<double>>()[g]         = U(0.05, 0.2);
        p.get<CriticalPerSevere<double>>()[g]                 = U(0.1, 0.3);
        p.get<DeathsPerCritical<double>>()[g]                 = U(0.1, 0.4);
        m.populations[{g, InfectionState::Exposed}]            = U(10, 100);
        m.populations[{g, InfectionState::InfectedNoSymptoms}] = U(10, 100);
        m.populations[{g, InfectionState::InfectedSymptoms}]   = U(0, 20);
        m.populations.set_difference_from_group_total<AgeGroup>({g, InfectionState::Susceptible}, U(2e4, 6e4));
    }
    auto& c = p.get<ContactPatterns<double>>().get_cont_freq_mat();
    for (int i = 0; i < G; ++i) {
        for (int j = 0; j < G; ++j) {
            c[0].get_baseline()((size_t)i, (size_t)j) = U(1, 6);
            c[0].get_minimum()((size_t)i, (size_t)j)  = U(0, 0.5);
        }
    }
    c[0].add_damping(0.4, SimulationTime<double>(6.0));
    c[0].add_damping(Matrix::Constant((size_t)G, (size_t)G, 0.2), DampingLevel(1), DampingType(0),
                     SimulationTime<double>(9.0));
    return m;
}

std::vector<double> commuters(int G, double f)
{
    std::vector<double> c(10 * (size_t)G, 0.0);
    for (int g = 0; g < G; ++g) {
        for (int k : {0, 1, 2, 4, 8}) {
            c[(size_t)(10 * g + k)] = f * (1.0 + 0.1 * g);
        }
    }
    return c;
}

void print_graph_arrays(const detail::GraphArrays& a)
{
    std::printf("\"N\": %d, \"G\": %d, \"E\": %d, \"M\": %d, \"K\": %d, \"Ke\": %d,\n", a.N, a.G, a.E, a.M, a.K, a.Ke);
    print_vec("params", a.params);
    print_vec("contact_baseline", a.contact_baseline);
    print_vec("contact_minimum", a.contact_minimum);
    print_vec("damping_times", a.damping_times);
    print_vec("damping_values", a.damping_values);
    print_vec("state", a.state);
    std::vector<double> s(a.src.begin(), a.src.end()), d(a.dst.begin(), a.dst.end());
    print_vec("src", s);
    print_vec("dst", d);
    print_vec("coeff_baseline", a.coeff_baseline);
    print_vec("coeff_minimum", a.coeff_minimum);
}

MobilitySimGraph<Simulation<double>> three_nodes(int G)
{
    MobilitySimGraph<Simulation<double>> graph;
    for (int v = 0; v < 3; ++v) {
        graph.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
    }
    // added out of order on purpose: the graph keeps (start, end) order
    graph.add_edge(2, 0, commuters(G, 0.02));
    graph.add_edge(0, 1, commuters(G, 0.03));
    graph.add_edge(1, 0, commuters(G, 0.01));
    graph.add_edge(0, 2, commuters(G, 0.02));
    return graph;
}

detail::GraphArrays arrays_of(MobilitySimGraph<Simulation<double>>& graph)
{
    std::vector<const Model<double>*> models;
    std::vector<std::vector<double>> st;
    for (auto& n : graph.nodes()) {
        models.push_back(&n.property.get_simulation().get_model());
        st.push_back(n.property.get_result().get_last_value());
    }
    std::vector<const std::vector<double>*> sp;
    for (auto& s : st) {
        sp.push_back(&s);
    }
    return detail::pack_graph<Model<double>, MobilityEdge<double>>(
        models, sp, graph.edges(), [](const MobilityEdge<double>& e) -> const MobilityParameters<double>& {
            return e.get_parameters();
        });
}

int mode_dampings()
{
    // (level, type, time, value) lists; the value fills a 2 x 2 matrix
    const std::vector<std::vector<std::tuple<int, int, double, double>>> cases = {
        {},
        {{0, 0, 20.0, 0.3}},
        {{0, 0, 5.0, 0.2}, {0, 1, 5.0, 0.1}, {1, 0, 8.0, 0.5}},
        {{0, 0, 5.0, 0.2}, {0, 0, 9.0, 0.6}, {1, 0, 7.0, 0.4}, {1, 1, 7.0, 0.1}, {0, 0, 12.0, 0.0}},
        {{2, 0, 3.0, 0.25}, {0, 0, 3.0, 0.5}, {0, 0, 3.0, 0.7}}, // equal key replaces
    };
    std::printf("{\"cases\": [\n");
    for (size_t k = 0; k < cases.size(); ++k) {
        Dampings d(2, 2);
        for (auto& c : cases[k]) {
            d.add(std::get<3>(c), DampingLevel(std::get<0>(c)), DampingType(std::get<1>(c)),
                  SimulationTime<double>(std::get<2>(c)));
        }
        std::vector<double> times;
        std::vector<Matrix> values;
        d.cache(times, values);
        std::vector<double> lv, ty, tm, va, flat;
        for (auto& x : d.list()) {
            lv.push_back(x.level.get());
            ty.push_back(x.type.get());
            tm.push_back(x.time.get());
            va.insert(va.end(), x.values.data(), x.values.data() + 4);
        }
        for (auto& m : values) {
            flat.insert(flat.end(), m.data(), m.data() + 4);
        }
        std::printf("{");
        print_vec("levels", lv);
        print_vec("types", ty);
        print_vec("times", tm);
        print_vec("matrices", va);
        print_vec("cache_times", times);
        print_vec("cache_values", flat, false);
        std::printf("}%s\n", k + 1 < cases.size() ? "," : "");
    }
    std::printf("]}\n");
    return 0;
}

int mode_pack()
{
    auto graph = three_nodes(2);
    auto a     = arrays_of(graph);
    std::printf("{");
    print_graph_arrays(a);
    std::printf("\"ok\": 1}\n");
    return 0;
}

// GraphBuilder (graph_builder.h): edges added out of order and twice between
// nodes 0 and 1; build(true) keeps the one added last, like Graph::add_edge.
int mode_builder()
{
    const int G = 2;
    GraphBuilder<SimulationNode<Simulation<double>>, MobilityEdge<double>> builder(3, 5);
    MobilitySimGraph<Simulation<double>> direct;
    for (int v = 0; v < 3; ++v) {
        builder.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
        direct.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
    }
    const std::vector<std::tuple<int, int, double>> adds = {
        {2, 0, 0.02}, {0, 1, 0.05}, {1, 0, 0.01}, {0, 2, 0.02}, {0, 1, 0.03}};
    for (auto& a : adds) {
        builder.add_edge(std::get<0>(a), std::get<1>(a), commuters(G, std::get<2>(a)));
        direct.add_edge(std::get<0>(a), std::get<1>(a), commuters(G, std::get<2>(a)));
    }
    auto built = std::move(builder).build(true);
    auto a     = arrays_of(built);
    auto b     = arrays_of(direct);
    std::printf("{\"same\": %d, \"E\": %d,\n", (int)(a.src == b.src && a.dst == b.dst &&
                                                      a.coeff_baseline == b.coeff_baseline && a.params == b.params),
                a.E);
    std::vector<double> s(a.src.begin(), a.src.end()), d(a.dst.begin(), a.dst.end());
    print_vec("src", s);
    print_vec("dst", d);
    print_vec("coeff_baseline", a.coeff_baseline, false);
    std::printf("}\n");
    return 0;
}

int mode_simulate()
{
    const Model<double> m = make_model(3, 3u);
    Simulation<double> pieces(m, 0.0, 0.1);
    pieces.advance(4.0);
    const double dt_mid = pieces.get_dt();
    pieces.advance(12.0);
    Simulation<double> whole(m, 0.0, 0.1);
    whole.advance(12.0);
    std::vector<double> dydt;
    m.get_derivatives(m.populations.array(), m.populations.array(), 5.0, dydt);
    auto a = m.pack();
    std::printf("{\"G\": 3, \"K\": %d, \"M\": %d,\n", a.K, a.M);
    print_vec("params", a.params);
    print_vec("contact_baseline", a.contact_baseline);
    print_vec("contact_minimum", a.contact_minimum);
    print_vec("damping_times", a.damping_times);
    print_vec("damping_values", a.damping_values);
    print_vec("state", a.state);
    print_vec("dydt_t5", dydt);
    std::printf("\"dt_mid\": %.17g, \"dt_end\": %.17g, \"points_pieces\": %zu, \"points_whole\": %zu,\n", dt_mid,
                pieces.get_dt(), pieces.get_result().get_num_time_points(), whole.get_result().get_num_time_points());
    std::vector<double> tp, tw;
    for (size_t i = 0; i < pieces.get_result().get_num_time_points(); ++i) {
        tp.push_back(pieces.get_result().get_time(i));
    }
    for (size_t i = 0; i < whole.get_result().get_num_time_points(); ++i) {
        tw.push_back(whole.get_result().get_time(i));
    }
    print_vec("times_pieces", tp);
    print_vec("times_whole", tw);
    print_vec("last_pieces", pieces.get_result().get_last_value());
    print_vec("last_whole", whole.get_result().get_last_value(), false);
    std::printf("}\n");
    return 0;
}

int mode_flows()
{
    const Model<double> m = make_model(2, 5u);
    auto res              = simulate_flows(0.0, 10.0, 0.1, m);
    auto a                = m.pack();
    std::printf("{\"G\": 2, \"K\": %d, \"M\": %d,\n", a.K, a.M);
    print_vec("params", a.params);
    print_vec("contact_baseline", a.contact_baseline);
    print_vec("contact_minimum", a.contact_minimum);
    print_vec("damping_times", a.damping_times);
    print_vec("damping_values", a.damping_values);
    print_vec("state", a.state);
    std::vector<double> t;
    for (size_t i = 0; i < res[0].get_num_time_points(); ++i) {
        t.push_back(res[0].get_time(i));
    }
    print_vec("t", t);
    print_vec("last_pop", res[0].get_last_value());
    print_vec("last_flows", res[1].get_last_value(), false);
    std::printf("}\n");
    return 0;
}

int mode_graph()
{
    auto graph = three_nodes(2);
    auto a     = arrays_of(graph);
    auto sim   = make_mobility_sim(0.0, 0.5, std::move(graph));
    sim.advance(6.0);
    std::printf("{");
    print_graph_arrays(a);
    std::vector<double> t, states;
    auto& nodes = sim.get_graph().nodes();
    for (size_t i = 0; i < nodes[0].property.get_result().get_num_time_points(); ++i) {
        t.push_back(nodes[0].property.get_result().get_time(i));
        for (auto& n : nodes) {
            const double* v = n.property.get_result().value_ptr(i);
            states.insert(states.end(), v, v + 20);
        }
    }
    print_vec("t", t);
    print_vec("states", states);
    std::printf("\"t_end\": %.17g}\n", sim.get_t());
    return 0;
}

// Mobility results of every edge (MobilityEdge(coeffs, save_indices),
// get_mobility_results) with the save indices of cpp/examples/ode_secir_graph.cpp
// (INS + INSC and ISy + ISyC of every age group), over two advances.
int mode_commuters()
{
    const int G = 2;
    SaveIndices sets(2);
    for (size_t g = 0; g < (size_t)G; ++g) {
        sets[0].push_back(g * 10 + (size_t)InfectionState::InfectedNoSymptoms);
        sets[0].push_back(g * 10 + (size_t)InfectionState::InfectedNoSymptomsConfirmed);
        sets[1].push_back(g * 10 + (size_t)InfectionState::InfectedSymptoms);
        sets[1].push_back(g * 10 + (size_t)InfectionState::InfectedSymptomsConfirmed);
    }
    MobilitySimGraph<Simulation<double>> graph;
    for (int v = 0; v < 3; ++v) {
        graph.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
    }
    graph.add_edge(2, 0, commuters(G, 0.02), sets);
    graph.add_edge(0, 1, commuters(G, 0.03), sets);
    graph.add_edge(1, 0, commuters(G, 0.01), sets);
    graph.add_edge(0, 2, commuters(G, 0.02), sets);
    auto a   = arrays_of(graph);
    auto sim = make_mobility_sim(0.0, 0.5, std::move(graph));
    sim.set_record_boundaries(false);
    sim.advance(2.5);
    sim.advance(6.0);
    std::printf("{");
    print_graph_arrays(a);
    std::vector<double> t, v, counts;
    for (auto& e : sim.get_graph().edges()) {
        const auto& r = e.property.get_mobility_results();
        counts.push_back((double)r.get_num_time_points());
        for (size_t k = 0; k < r.get_num_time_points(); ++k) {
            t.push_back(r.get_time(k));
            const auto x = r.get_value(k);
            v.insert(v.end(), x.begin(), x.end());
        }
    }
    print_vec("counts", counts);
    print_vec("times", t);
    print_vec("values", v, false);
    std::printf("}\n");
    return 0;
}

// A graph of FlowSimulation nodes (the reference's graph of FlowSimulation
// nodes, cpp/tests/test_graph_simulation.cpp:276-340) next to the same graph of
// Simulation nodes: the states at every boundary and the flows of the nodes.
int mode_flows_graph()
{
    const int G = 2;
    MobilitySimGraph<Simulation<double>> plain;
    Graph<SimulationNode<FlowSimulation<double>>, MobilityEdge<double>> flows;
    for (int v = 0; v < 3; ++v) {
        plain.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
        flows.add_node(100 + v, make_model(G, 7u + (unsigned)v), 0.0, 0.1);
    }
    const std::vector<std::tuple<int, int, double>> edges = {{2, 0, 0.02}, {0, 1, 0.03}, {1, 0, 0.01}, {0, 2, 0.02}};
    for (auto& e : edges) {
        plain.add_edge(std::get<0>(e), std::get<1>(e), commuters(G, std::get<2>(e)));
        flows.add_edge(std::get<0>(e), std::get<1>(e), commuters(G, std::get<2>(e)));
    }
    auto a    = arrays_of(plain);
    auto sim0 = make_mobility_sim(0.0, 0.5, std::move(plain));
    GraphSimulation<decltype(flows)> sim1(0.0, 0.5, std::move(flows));
    sim0.advance(3.0);
    sim1.advance(3.0);
    sim1.advance(6.0);
    sim0.advance(6.0);
    std::printf("{");
    print_graph_arrays(a);
    std::vector<double> s0, s1, f, t;
    for (size_t v = 0; v < 3; ++v) {
        const auto& r0 = sim0.get_graph().nodes()[v].property.get_result();
        const auto& r1 = sim1.get_graph().nodes()[v].property.get_result();
        const auto& fl = sim1.get_graph().nodes()[v].property.get_simulation().get_flows();
        for (size_t k = 0; k < r1.get_num_time_points(); ++k) {
            const auto x0 = r0.get_value(k), x1 = r1.get_value(k), y = fl.get_value(k);
            s0.insert(s0.end(), x0.begin(), x0.end());
            s1.insert(s1.end(), x1.begin(), x1.end());
            f.insert(f.end(), y.begin(), y.end());
            if (v == 0) {
                t.push_back(fl.get_time(k));
            }
        }
    }
    print_vec("t", t);
    print_vec("states_plain", s0);
    print_vec("states_flows", s1);
    print_vec("flows", f, false);
    std::printf("}\n");
    return 0;
}

int mode_study()
{
    using GraphT = ParameterStudy<Simulation<double>>::GraphType;
    GraphT base;
    for (int v = 0; v < 3; ++v) {
        base.add_node(v, make_model(2, 11u + (unsigned)v));
    }
    base.add_edge(0, 1, MobilityParameters<double>(commuters(2, 0.02)));
    base.add_edge(1, 2, MobilityParameters<double>(commuters(2, 0.02)));
    base.add_edge(2, 0, MobilityParameters<double>(commuters(2, 0.02)));
    ParameterStudy<Simulation<double>> study(base, 0.0, 5.0, 0.5, 4);
    std::vector<GraphT> sampled;
    unsigned run = 0;
    auto results = study.run(
        [&](const GraphT& g) {
            GraphT s = g;
            const double f = 0.8 + 0.1 * run++;
            for (auto& n : s.nodes()) {
                for (size_t i = 0; i < 2; ++i) {
                    n.property.parameters.get<TransmissionProbabilityOnContact<double>>()[AgeGroup(i)] *= f;
                }
            }
            sampled.push_back(s);
            return s;
        },
        [](StudyResult r, size_t idx) {
            return std::make_pair(idx, r.node_states);
        });
    std::printf("{\"runs\": [\n");
    for (size_t r = 0; r < results.size(); ++r) {
        std::vector<const Model<double>*> models;
        std::vector<const std::vector<double>*> st;
        for (auto& n : sampled[r].nodes()) {
            models.push_back(&n.property);
            st.push_back(&n.property.populations.array());
        }
        auto a = detail::pack_graph<Model<double>, MobilityParameters<double>>(
            models, st, sampled[r].edges(), [](const MobilityParameters<double>& p) -> const MobilityParameters<double>& {
                return p;
            });
        std::vector<double> fin;
        for (auto& s : results[r].second) {
            fin.insert(fin.end(), s.begin(), s.end());
        }
        std::printf("{");
        print_graph_arrays(a);
        print_vec("final", fin, false);
        std::printf("}%s\n", r + 1 < results.size() ? "," : "");
    }
    std::printf("]}\n");
    return 0;
}

void print_dampings(const char* key, const ContactMatrixGroup& c, bool comma = true)
{
    std::printf("\"%s\": [", key);
    for (size_t m = 0; m < c.get_num_matrices(); ++m) {
        std::printf("%s[", m ? ", " : "");
        const Dampings& d = c[m].get_dampings();
        for (size_t i = 0; i < d.size(); ++i) {
            std::printf("%s[%.17g, %d, %d, %.17g]", i ? ", " : "", d[i].time.get(), d[i].level.get(), d[i].type.get(),
                        d[i].values[0]);
        }
        std::printf("]");
    }
    std::printf("]%s\n", comma ? "," : "");
}

// The chunk loop of osecir::Simulation::advance (model.h:299-365) with the
// integration left out, as the reference's tests do with a mock simulation.
void advance_fixed_state(ContactMatrixGroup& c, const DynamicNPIs<double>& npis, DynamicNPIState& st, double t0,
                         double tmax, double inf_rel)
{
    double t = t0;
    while (t < tmax) {
        check_dynamic_npis(npis, st, c, t, inf_rel);
        double dt = std::min(1.0, tmax - t);
        if (t < st.t_end) {
            dt = std::min(dt, st.t_end - t);
        }
        t += dt;
    }
}

int mode_npi_logic()
{
    auto constant = [](const std::vector<double>& g) {
        return Matrix::Constant(g.size(), g.size(), g[0]);
    };
    std::printf("{");
    {
        // two matrices without dampings, one NPI on both (test_dynamic_npis.cpp implement_empty)
        ContactMatrixGroup c(2, 2);
        std::vector<DampingSampling<double>> npis{
            DampingSampling<double>(0.8, DampingLevel(0), DampingType(0), SimulationTime<double>(0), {0, 1}, {1.0, 1.0})};
        implement_dynamic_npis(c, npis, SimulationTime<double>(0.45), SimulationTime<double>(0.6), constant);
        print_dampings("implement_empty", c);
    }
    {
        // test_dynamic_npis.cpp implement: existing dampings of several types and levels
        ContactMatrixGroup c(2, 3);
        c[0].add_damping(0.15, DampingLevel(0), DampingType(0), SimulationTime<double>(0.3));
        c[0].add_damping(0.2, DampingLevel(0), DampingType(0), SimulationTime<double>(0.4));
        c[0].add_damping(0.25, DampingLevel(0), DampingType(1), SimulationTime<double>(0.5));
        c[0].add_damping(0.35, DampingLevel(0), DampingType(0), SimulationTime<double>(0.7));
        c[1].add_damping(0.25, DampingLevel(1), DampingType(1), SimulationTime<double>(0.5));
        c[1].add_damping(0.45, DampingLevel(0), DampingType(0), SimulationTime<double>(0.9));
        implement_dynamic_npis(c,
                               std::vector<DampingSampling<double>>{DampingSampling<double>(
                                   0.4, DampingLevel(0), DampingType(0), SimulationTime<double>(0), {0, 1}, {1, 1, 1})},
                               SimulationTime<double>(0.45), SimulationTime<double>(0.6), constant);
        print_dampings("implement_first", c);
        implement_dynamic_npis(c,
                               std::vector<DampingSampling<double>>{DampingSampling<double>(
                                   0.3, DampingLevel(0), DampingType(0), SimulationTime<double>(0), {0}, {1, 1, 1})},
                               SimulationTime<double>(0.3), SimulationTime<double>(0.9), constant);
        print_dampings("implement_second", c);
    }
    // one group: 10 symptomatic of 110 against a threshold of 0.05 * base (test_dynamic_npis.cpp secir_*)
    auto npis_of = [](double value, double base, double delay, double duration) {
        DynamicNPIs<double> n;
        n.set_threshold(0.05 * base, {DampingSampling<double>(value, DampingLevel(0), DampingType(0),
                                                              SimulationTime<double>(0), {0}, {1.0})});
        n.set_duration(SimulationTime<double>(duration));
        n.set_base_value(base);
        n.set_implementation_delay(SimulationTime<double>(delay));
        return n;
    };
    {
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(1.0, 23000, 0.0, 5.0), st, 0.0, 3.0, 1.0 / 101.0);
        print_dampings("threshold_safe", c);
    }
    {
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(1.0, 50000, 0.0, 5.0), st, 0.0, 3.0, 10.0 / 110.0);
        print_dampings("threshold_exceeded", c);
    }
    {
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(0.5, 50000, 3.0, 5.0), st, 0.0, 3.0, 10.0 / 110.0);
        print_dampings("delayed_t0", c);
    }
    {
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(0.5, 50000, 2.0, 5.0), st, 1.0, 5.0, 10.0 / 110.0);
        print_dampings("delayed_t1", c);
    }
    {
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(0.5, 50000, 10.0, 5.0), st, 1.0, 4.0, 10.0 / 110.0);
        print_dampings("delayed_long", c);
    }
    {
        // keep-alive: the threshold stays exceeded past the NPI's end
        ContactMatrixGroup c(1, 1);
        DynamicNPIState st;
        advance_fixed_state(c, npis_of(0.5, 50000, 0.0, 2.0), st, 0.0, 7.0, 10.0 / 110.0);
        print_dampings("keep_alive", c, false);
    }
    std::printf("}\n");
    return 0;
}

// Every node of the three-node graph with dynamic NPIs on the symptomatic
// infections: a threshold most nodes cross within the run, an implementation
// delay of one day and three-day NPIs (on the exchange grid).
MobilitySimGraph<Simulation<double>> three_nodes_npi(int G)
{
    auto graph = three_nodes(G);
    DynamicNPIs<double> npis;
    npis.set_threshold(2.0, {DampingSampling<double>(0.5, DampingLevel(0), DampingType(0), SimulationTime<double>(0),
                                                     {0}, std::vector<double>((size_t)G, 1.0))});
    npis.set_threshold(6.0, {DampingSampling<double>(0.8, DampingLevel(2), DampingType(0), SimulationTime<double>(0),
                                                     {0}, std::vector<double>((size_t)G, 1.0))});
    npis.set_duration(SimulationTime<double>(3.0));
    npis.set_implementation_delay(SimulationTime<double>(1.0));
    npis.set_base_value(1e5);
    for (auto& n : graph.nodes()) {
        n.property.get_simulation().get_model().parameters.get<DynamicNPIsInfectedSymptoms<double>>() = npis;
    }
    return graph;
}

int mode_npi_graph()
{
    std::printf("{");
    for (int precision : {MGPU_PRECISION_FP64, MGPU_PRECISION_MIXED}) {
        auto graph = three_nodes_npi(2);
        auto a     = arrays_of(graph);
        auto sim   = make_mobility_sim(0.0, 0.5, std::move(graph));
        sim.set_precision(precision);
        sim.advance(12.0);
        std::vector<double> fin, enacted;
        for (auto& n : sim.get_graph().nodes()) {
            auto v = n.property.get_result().get_last_value();
            fin.insert(fin.end(), v.begin(), v.end());
            enacted.push_back(n.property.get_simulation().get_dynamic_npi_state().enacted);
        }
        if (precision == MGPU_PRECISION_FP64) {
            print_graph_arrays(a);
            print_dampings("initial_dampings", three_nodes(2).nodes()[0].property.get_simulation().get_model()
                                                   .parameters.get<ContactPatterns<double>>());
        }
        const char* tag = precision == MGPU_PRECISION_FP64 ? "fp64" : "mixed";
        char key[64];
        std::snprintf(key, sizeof key, "final_%s", tag);
        print_vec(key, fin);
        std::snprintf(key, sizeof key, "enacted_%s", tag);
        print_vec(key, enacted, precision == MGPU_PRECISION_FP64);
    }
    std::printf("}\n");
    return 0;
}

// Dynamic NPIs on every mobility edge of three_nodes_npi: a lower threshold
// than the nodes' (the edges see their sources' states before every exchange)
// and two-day NPIs that halve, then cut by 80 %, the commuters.
DynamicNPIs<double> edge_npis(int G)
{
    DynamicNPIs<double> npis;
    npis.set_threshold(1.0, {DampingSampling<double>(0.5, DampingLevel(0), DampingType(0), SimulationTime<double>(0),
                                                     {0}, std::vector<double>((size_t)G, 1.0))});
    npis.set_threshold(4.0, {DampingSampling<double>(0.8, DampingLevel(1), DampingType(0), SimulationTime<double>(0),
                                                     {0}, std::vector<double>((size_t)G, 1.0))});
    npis.set_duration(SimulationTime<double>(2.0));
    npis.set_base_value(1e5);
    return npis;
}

int mode_npi_edges()
{
    std::printf("{");
    for (int precision : {MGPU_PRECISION_FP64, MGPU_PRECISION_MIXED}) {
        auto graph = three_nodes_npi(2);
        for (auto& e : graph.edges()) {
            e.property.get_parameters().get_dynamic_npis_infected() = edge_npis(2);
        }
        auto a   = arrays_of(graph);
        auto sim = make_mobility_sim(0.0, 0.5, std::move(graph));
        sim.set_precision(precision);
        sim.advance(12.0);
        std::vector<double> fin, enacted, edge_enacted;
        for (auto& n : sim.get_graph().nodes()) {
            auto v = n.property.get_result().get_last_value();
            fin.insert(fin.end(), v.begin(), v.end());
            enacted.push_back(n.property.get_simulation().get_dynamic_npi_state().enacted);
        }
        for (auto& e : sim.get_graph().edges()) {
            edge_enacted.push_back(e.property.get_dynamic_npi_state().enacted);
        }
        if (precision == MGPU_PRECISION_FP64) {
            print_graph_arrays(a);
            print_dampings("initial_dampings", three_nodes(2).nodes()[0].property.get_simulation().get_model()
                                                   .parameters.get<ContactPatterns<double>>());
        }
        const char* tag = precision == MGPU_PRECISION_FP64 ? "fp64" : "mixed";
        char key[64];
        std::snprintf(key, sizeof key, "final_%s", tag);
        print_vec(key, fin);
        std::snprintf(key, sizeof key, "enacted_%s", tag);
        print_vec(key, enacted);
        std::snprintf(key, sizeof key, "edge_enacted_%s", tag);
        print_vec(key, edge_enacted);
    }
    {
        // the same FP64 run recording only at tmax: the checks read the device's per-node sums
        auto graph = three_nodes_npi(2);
        for (auto& e : graph.edges()) {
            e.property.get_parameters().get_dynamic_npis_infected() = edge_npis(2);
        }
        auto sim = make_mobility_sim(0.0, 0.5, std::move(graph));
        sim.set_record_boundaries(false);
        sim.advance(12.0);
        std::vector<double> fin, enacted;
        for (auto& n : sim.get_graph().nodes()) {
            auto v = n.property.get_result().get_last_value();
            fin.insert(fin.end(), v.begin(), v.end());
            enacted.push_back(n.property.get_simulation().get_dynamic_npi_state().enacted);
        }
        for (auto& e : sim.get_graph().edges()) {
            enacted.push_back(e.property.get_dynamic_npi_state().enacted);
        }
        std::printf("\"num_points_norecord\": %zu,\n",
                    sim.get_graph().nodes()[0].property.get_result().get_num_time_points());
        print_vec("final_norecord", fin);
        print_vec("enacted_norecord", enacted, false);
    }
    std::printf("}\n");
    return 0;
}

void print_series(const char* key, const TimeSeries<double>& ts, bool comma = true)
{
    std::printf("\"%s\": {", key);
    std::vector<double> t, v;
    for (size_t i = 0; i < ts.get_num_time_points(); ++i) {
        t.push_back(ts.get_time(i));
        const double* p = ts.value_ptr(i);
        v.insert(v.end(), p, p + ts.get_num_elements());
    }
    print_vec("t", t);
    print_vec("v", v, false);
    std::printf("}%s\n", comma ? "," : "");
}

TimeSeries<double> series(size_t n, const std::vector<std::pair<double, std::vector<double>>>& pts)
{
    TimeSeries<double> ts(n);
    for (auto& p : pts) {
        ts.add_time_point(p.first, p.second);
    }
    return ts;
}

int mode_interpolate()
{
    // the series of the reference's tests (cpp/tests/test_analyze_result.cpp:68-175)
    std::printf("{");
    print_series("simple", interpolate_simulation_result(series(
                               1, {{0.0, {0.1}}, {0.5, {0.2}}, {1.5, {0.3}}, {2.5, {0.4}}, {3.5, {0.5}}, {4.5, {0.6}},
                                   {5.5, {0.7}}})));
    print_series("complex", interpolate_simulation_result(series(2, {{0.0, {1.0, 2.0}}, {1.5, {3.0, 10.0}},
                                                                     {2.1, {5.0, 3.0}}})));
    print_series("exact_day", interpolate_simulation_result(series(
                                  1, {{0.0, {0.0}}, {0.5, {1.0}}, {1.0, {2.0}}, {2.1, {3.0}}, {3.0, {4.0}}})));
    print_series("default_tol",
                 interpolate_simulation_result(series(1, {{0.0 + 1e-15, {0.0}}, {1.0, {0.0}}, {2.0 - 1e-15, {0.0}}})));
    print_series("given_tol", interpolate_simulation_result(
                                  series(1, {{0.0 + 1e-2, {0.0}}, {1.0, {0.0}}, {2.0 - 1e-3, {0.0}}}), 5e-3));
    print_series("chosen", interpolate_simulation_result(series(1, {{0.1, {0.0}}, {0.9, {1.0}}, {1.4, {2.0}},
                                                                    {2.5, {3.0}}, {3.0, {4.0}}}),
                                                         std::vector<double>{0.2, 0.6, 1.0, 1.3, 2.4}),
                 false);
    std::printf("}\n");
    return 0;
}

} // namespace

int main(int argc, char** argv)
{
    const char* mode = argc > 1 ? argv[1] : "";
    try {
        if (!std::strcmp(mode, "dampings")) {
            return mode_dampings();
        }
        if (!std::strcmp(mode, "pack")) {
            return mode_pack();
        }
        if (!std::strcmp(mode, "builder")) {
            return mode_builder();
        }
        if (!std::strcmp(mode, "simulate")) {
            return mode_simulate();
        }
        if (!std::strcmp(mode, "flows")) {
            return mode_flows();
        }
        if (!std::strcmp(mode, "graph")) {
            return mode_graph();
        }
        if (!std::strcmp(mode, "study")) {
            return mode_study();
        }
        if (!std::strcmp(mode, "commuters")) {
            return mode_commuters();
        }
        if (!std::strcmp(mode, "flows_graph")) {
            return mode_flows_graph();
        }
        if (!std::strcmp(mode, "npi_logic")) {
            return mode_npi_logic();
        }
        if (!std::strcmp(mode, "npi_graph")) {
            return mode_npi_graph();
        }
        if (!std::strcmp(mode, "npi_edges")) {
            return mode_npi_edges();
        }
        if (!std::strcmp(mode, "interpolate")) {
            return mode_interpolate();
        }
    }
    catch (const Error& e) {
        std::fprintf(stderr, "miogpu error: %s\n", e.what());
        return 3;
    }
    std::fprintf(stderr, "usage: facade_check dampings|pack|simulate|graph|study\n");
    return 2;
}
