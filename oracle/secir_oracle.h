/*
 * secir_oracle.h — TEST INFRASTRUCTURE, not product code.
 *
 * An FP64 CPU restatement of MEmilio's graph-ODE SECIR path, used only as
 * the checker of the GPU library (tests/, __graft_entry__.smoke()) and as
 * the timed CPU baseline in bench.py. Nothing in memilio_gb300/ links,
 * loads or calls it.
 *
 * It follows, function by function (see secir_oracle.cpp for line cites):
 *   models/ode_secir/model.h          get_flows, get_mobility_factors, test_commuters
 *   memilio/compartments/flow_model.h get_derivatives
 *   memilio/epidemiology/damping.h, contact_matrix.h, math/smoother.h
 *   memilio/math/integrator.h         SystemIntegrator::advance
 *   memilio/math/stepper_wrapper.h    ControlledStepperWrapper<cash_karp54>
 *   memilio/math/adapt_rk.h           RKIntegratorCore (RKF45)
 *   memilio/math/euler.h              EulerIntegratorCore
 *   memilio/mobility/metapopulation_mobility_instant.h, graph_simulation.h
 *   memilio/compartments/parameter_studies.h (run distribution)
 *
 * Parity pins: the reference's golden CSVs (tests/golden/), see tests/test_oracle_golden.py.
 */
#ifndef SECIR_ORACLE_H
#define SECIR_ORACLE_H

#include "../include/miogpu_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_stats {
    int64_t accepted_steps;   /* accepted integrator steps, all nodes */
    int64_t rejected_steps;   /* rejected attempts (error or dt_max), all nodes */
    int64_t rhs_evals;        /* right-hand-side evaluations incl. mobility returns */
    int64_t underflow_fixes;  /* negative compartments fixed on mobility return */
    int64_t failed_steps;     /* steps forced at dt_min */
} orc_stats;

/* Right-hand side of node `node` of graph g: dydt = f(pop, y, t)
 * (FlowModel::get_derivatives(pop, y, t, dydt)). */
int orc_eval_rhs(const mgpu_graph* g, int node, const double* pop, const double* y, double t, double* dydt);

/* Flows of node `node` (Model::get_flows), 15G values. */
int orc_eval_flows(const mgpu_graph* g, int node, const double* pop, const double* y, double t, double* flows);

/* Single-node simulate(t0, tmax, dt, model, core) (compartments/simulation.h:99-110):
 * records every accepted step. out_t [max_points], out_y [max_points][10G].
 * Returns 0, or -1 when max_points is too small. */
int orc_simulate(const mgpu_graph* g, int node, double t0, double tmax, double dt,
                 const mgpu_integrator_opts* opts, int max_points, double* out_t, double* out_y,
                 int* num_points, orc_stats* stats);

/* simulate_flows(t0, tmax, dt, model, core) (compartments/flow_simulation.h:36-121,
 * flow_simulation_base.h:90-103): the integrator's state is the accumulated flows
 * (from zero); every accepted step is recorded with its flows out_f
 * [max_points][15G] and populations out_y [max_points][10G]. Returns 0, or -1
 * when max_points is too small. */
int orc_simulate_flows(const mgpu_graph* g, int node, double t0, double tmax, double dt,
                       const mgpu_integrator_opts* opts, int max_points, double* out_t, double* out_f,
                       double* out_y, int* num_points, orc_stats* stats);

/* make_mobility_sim(t0, dt_exchange, graph).advance(tmax). Writes the node
 * states after every exchange boundary into out_states
 * [num_boundaries][N][10G] when out_states != NULL (num_boundaries =
 * ceil((tmax-t0)/dt_exchange)), and the final states into final_state [N][10G]. */
int orc_graph_run(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                  const mgpu_integrator_opts* opts, double* out_states, double* final_state,
                  orc_stats* stats);

/* orc_graph_run recording MobilityEdge's mobility results
 * (add_mobility_result_time_point, mobility/metapopulation_mobility_instant.h:
 * 423-447) on every edge with the same save indices: num_sets sets of flat
 * compartment indices, set_offsets [num_sets + 1], set_indices. Per edge:
 * counts [E] time points (one per departure, one per return), times
 * [E][capacity], values [E][capacity][num_sets + 1] (the sets' sums of the
 * travelers, then their total). */
int orc_graph_run_commuters(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                            const mgpu_integrator_opts* opts, int num_sets, const int32_t* set_offsets,
                            const int32_t* set_indices, int capacity, double* final_state, int32_t* counts,
                            double* times, double* values, orc_stats* stats);

/* One MobilityEdge::apply_mobility(t, 0, node_from, node_to) of edge `edge` on
 * the graph's initial states (a departure, as the reference's
 * test_mobility.cpp add_mobility_result_time_point does): the mobility result
 * it records, values [num_sets + 1]. */
int orc_departure_commuters(const mgpu_graph* g, int edge, double t, int num_sets, const int32_t* set_offsets,
                            const int32_t* set_indices, double* values);

/* ParameterStudy-style ensemble: graphs[0..num_graphs) each run independently,
 * one graph per thread, num_threads std::threads (0 = all hardware threads).
 * final_states is the concatenation of each graph's [N_b][10G] block.
 * elapsed_s receives the wall time of the runs alone (no setup). */
int orc_ensemble_run(const mgpu_graph* graphs, int num_graphs, double t0, double tmax,
                     double dt_exchange, double dt0, const mgpu_integrator_opts* opts,
                     int num_threads, double* final_states, double* elapsed_s, orc_stats* stats);

/* Cache builder for Dampings (damping.h:570-600). Dampings given sorted as
 * Dampings::add_ keeps them (by time, type, level). Writes K points (times,
 * G x G matrices, rows*cols values each). Returns K, or -1 if cap too small. */
int orc_damping_cache(int rows, int cols, int num_dampings, const double* times, const int32_t* levels,
                      const int32_t* types, const double* matrices, int cap, double* out_times,
                      double* out_matrices);

/* Dynamic NPIs (epidemiology/dynamic_npis.h, damping_sampling.h): one NPI of a
 * threshold, a damping of value * group weights on the listed contact
 * matrices; thresholds in any order with their NPIs samplings[first[k] ..
 * first[k+1]). */
typedef struct orc_npi_sampling {
    double value;
    int32_t level, type, num_matrices, pad;
    const int32_t* matrices;
    const double* group_weights; /* [G] */
} orc_npi_sampling;
typedef struct orc_dynamic_npis {
    int32_t num_thresholds, pad;
    const double* thresholds;
    const int32_t* first; /* [num_thresholds + 1] */
    const orc_npi_sampling* samplings;
    double duration, delay, base_value, directive_begin, directive_end;
} orc_dynamic_npis;
/* One contact damping of a node's initial list (the list every node starts with). */
typedef struct orc_damping {
    double time;
    int32_t level, type, matrix, pad;
    const double* coeffs; /* [G][G] */
} orc_damping;

/* orc_graph_run with the same dynamic NPIs on every node, and optionally the
 * same edge NPIs on every edge (edge_npis, MobilityEdge::apply_mobility,
 * mobility/metapopulation_mobility_instant.h:549-566: checked on the source's
 * state before each exchange, the coefficient dampings starting empty; the
 * graph must have no edge damping cache); edge_npi_count [E] receives the
 * enactments per edge. (The rest as for the nodes:) (osecir::Simulation::
 * advance, models/ode_secir/model.h:289-367, reached through
 * SimulationNode::advance): the nodes' contact dampings start from `dampings`
 * (the graph's damping caches are not used) and change as NPIs are enacted.
 * npi_count [N] receives the number of enactments per node. */
int orc_graph_run_npi(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                      const mgpu_integrator_opts* opts, const orc_dynamic_npis* npis, int num_dampings,
                      const orc_damping* dampings, const orc_dynamic_npis* edge_npis, double* final_state,
                      int32_t* npi_count, int32_t* edge_npi_count, orc_stats* stats);

#ifdef __cplusplus
}
#endif

#endif
