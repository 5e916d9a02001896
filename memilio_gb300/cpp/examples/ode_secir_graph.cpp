// A two-county SECIR mobility simulation written against the C++ facade, in
// the shape of MEmilio's examples/ode_secir_graph.cpp: build two models, add a
// commuter edge each way, simulate 30 days with an exchange every half day,
// and print every node's compartments at the end.
#include "miogpu/mobility.h"

#include <cstdio>

int main()
{
    using namespace miogpu;
    using namespace miogpu::osecir;
    const double t0 = 0.0, tmax = 30.0, dt = 0.5;
    const int G     = 1;

    Model<double> model(G);
    auto& params = model.parameters;
    params.get<ICUCapacity<double>>() = 250;
    params.get<TestAndTraceCapacity<double>>() = 40;
    params.get<TimeExposed<double>>()[AgeGroup(0)] = 3.5;
    params.get<TimeInfectedNoSymptoms<double>>()[AgeGroup(0)] = 2.5;
    params.get<TimeInfectedSymptoms<double>>()[AgeGroup(0)] = 6.0;
    params.get<TimeInfectedSevere<double>>()[AgeGroup(0)] = 8.0;
    params.get<TimeInfectedCritical<double>>()[AgeGroup(0)] = 6.5;
    params.get<TransmissionProbabilityOnContact<double>>()[AgeGroup(0)] = 0.08;
    params.get<RelativeTransmissionNoSymptoms<double>>()[AgeGroup(0)] = 0.6;
    params.get<RecoveredPerInfectedNoSymptoms<double>>()[AgeGroup(0)] = 0.15;
    params.get<RiskOfInfectionFromSymptomatic<double>>()[AgeGroup(0)] = 0.2;
    params.get<MaxRiskOfInfectionFromSymptomatic<double>>()[AgeGroup(0)] = 0.5;
    params.get<SeverePerInfectedSymptoms<double>>()[AgeGroup(0)] = 0.12;
    params.get<CriticalPerSevere<double>>()[AgeGroup(0)] = 0.3;
    params.get<DeathsPerCritical<double>>()[AgeGroup(0)] = 0.25;
    auto& contacts = params.get<ContactPatterns<double>>().get_cont_freq_mat();
    contacts[0].get_baseline().setConstant(8);
    contacts[0].add_damping(0.5, SimulationTime<double>(15.0));

    model.populations[{AgeGroup(0), InfectionState::Exposed}] = 80;
    model.populations[{AgeGroup(0), InfectionState::InfectedNoSymptoms}] = 40;
    model.populations.set_difference_from_group_total<AgeGroup>({AgeGroup(0), InfectionState::Susceptible}, 20000);
    model.apply_constraints();

    Model<double> model2 = model;
    model2.populations[{AgeGroup(0), InfectionState::Exposed}] = 0;
    model2.populations[{AgeGroup(0), InfectionState::InfectedNoSymptoms}] = 0;
    model2.populations.set_difference_from_group_total<AgeGroup>({AgeGroup(0), InfectionState::Susceptible}, 10000);

    MobilitySimGraph<Simulation<double>> graph;
    graph.add_node(1001, model, t0);
    graph.add_node(1002, model2, t0);
    std::vector<double> commuters(10 * G, 0.0);
    for (int c : {0, 1, 2, 4, 8}) { // S, E, INS, ISy, R commute
        commuters[(size_t)c] = 0.01;
    }
    graph.add_edge(0, 1, commuters);
    graph.add_edge(1, 0, commuters);

    auto sim = make_mobility_sim(t0, dt, std::move(graph));
    sim.advance(tmax);

    for (auto& n : sim.get_graph().nodes()) {
        const auto y = n.property.get_result().get_last_value();
        double total = 0.0;
        std::printf("node %d at t=%.1f:", n.id, n.property.get_result().get_last_time());
        for (double v : y) {
            std::printf(" %.6f", v);
            total += v;
        }
        std::printf("  (total %.6f, %zu time points)\n", total, n.property.get_result().get_num_time_points());
    }
    return 0;
}
