/*
 * miogpu.h — C ABI of libmiogpu, the GB300 (sm_103a) implementation of
 * MEmilio's graph-ODE SECIR hot path.
 *
 * Plain C: opaque handles, flat arrays, int status codes, no exceptions and
 * no CUDA or C++ types in the signatures. The data format of a graph is in
 * miogpu_layout.h. Each entry point names the reference interface it
 * replaces (paths inside the MEmilio source tree).
 *
 * Threading: one context per host thread; calls on one context are not
 * reentrant. Every context owns one CUDA stream; all device memory belongs
 * to the context and its batches, and no device pointer is returned.
 */
#ifndef MIOGPU_H
#define MIOGPU_H

#include "miogpu_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. 0..7 mirror mio::StatusCode (cpp/memilio/io/io.h:49-59). */
enum mgpu_status {
    MGPU_OK                  = 0,
    MGPU_UNKNOWN_ERROR       = 1,
    MGPU_OUT_OF_RANGE        = 2,
    MGPU_INVALID_VALUE       = 3,
    MGPU_INVALID_FILE_FORMAT = 4,
    MGPU_KEY_NOT_FOUND       = 5,
    MGPU_INVALID_TYPE        = 6,
    MGPU_FILE_NOT_FOUND      = 7,
    MGPU_CUDA_ERROR          = 100, /* a CUDA call failed; see mgpu_last_error */
    MGPU_OOM                 = 101, /* device memory budget exceeded */
    MGPU_TIMEOUT             = 102, /* a bounded device wait gave up */
    MGPU_STEP_FAILED         = 103, /* an instance hit the step cap or produced NaN/Inf */
    MGPU_UNSUPPORTED         = 104  /* valid input this library does not implement */
};

/* Arithmetic of the node ODE solves. */
enum mgpu_precision {
    MGPU_PRECISION_FP64_PLAIN = 0, /* one thread per node, FP64, stage vectors in HBM (the plain drop-in) */
    MGPU_PRECISION_FP64       = 1, /* batched lane-per-age-group solver, FP64 throughout */
    MGPU_PRECISION_MIXED      = 2, /* batched: FP32 flows, stage combinations, error norm and step-size
                                      controller on an FP32 interval clock; node states as float-float
                                      pairs (~48-bit significand) updated with exact TwoSum */
    MGPU_PRECISION_MIXED_FP64_CONTROL = 3 /* batched: FP32 flows and stage combinations; FP64 state
                                      accumulation, embedded-error norm, step-size controller and
                                      interval clock (the exchange as in MGPU_PRECISION_MIXED) */
};

typedef struct mgpu_context mgpu_context;
typedef struct mgpu_batch mgpu_batch;

typedef struct mgpu_solver_opts {
    mgpu_integrator_opts integrator; /* tolerances and dt bounds of every node's core */
    double dt0;                      /* initial integrator step, Simulation(model, t0, dt) (default 0.1) */
    double dt_exchange;              /* mobility interval, make_mobility_sim(t0, dt, graph) (0.5) */
    int32_t precision;               /* enum mgpu_precision */
    int32_t instances_per_block;     /* batched solver: node instances per CTA; 0 = autotuned */
    int32_t max_steps_per_interval;  /* per node and exchange interval; 0 = 100000 */
    int32_t use_cuda_graph;          /* capture the fixed exchange schedule as a CUDA graph */
    int32_t profile;                 /* time node solves and exchanges separately with CUDA events
                                        (launches stream by stream; no CUDA graph) */
    int32_t staged_exchange;         /* mixed solvers: graphs whose exchange tables fit in shared
                                        memory return and depart in one CTA per chunk of the graph
                                        from a copy there: 1 (default) when those CTAs fill the GPU
                                        (two per SM), 2 always, 0 never (every graph in the
                                        node-list passes). All give identical results. */
} mgpu_solver_opts;

/* Device times of the last mgpu_batch_advance, from CUDA events on the context's stream. */
typedef struct mgpu_timing {
    double advance_ms;      /* whole advance */
    double ode_ms;          /* node solves (profile mode only) */
    double exchange_ms;     /* exchanges incl. interval bookkeeping (profile mode only) */
    int64_t ode_launches;   /* node-solve kernel launches timed in ode_ms */
    int64_t attempts;       /* integrator attempts (accepted + rejected) during the advance */
    /* parts of exchange_ms, batched solvers in profile mode only: */
    double prep_ms;         /* per-node pass (snapshots, factors, return-time rates) */
    double return_ms;       /* return pass with the no-underflow bound */
    double exact_ms;        /* exact underflow path and commit */
    double depart_ms;       /* departure pass and interval bookkeeping */
} mgpu_timing;

typedef struct mgpu_stats {
    int64_t accepted_steps;   /* accepted integrator steps over all node instances */
    int64_t rejected_steps;   /* rejected attempts */
    int64_t failed_steps;     /* steps forced at dt_min (adaptive step sizing failed) */
    int64_t underflow_fixes;  /* negative compartments fixed on mobility returns */
    int64_t sequential_exchanges; /* graph exchanges that took the exact sequential path */
    int64_t phases;           /* exchange intervals simulated */
    int64_t kernel_launches;  /* kernels launched by this batch */
    int64_t scan_items;       /* (node, age group) items the exact underflow scan of the
                                 batched exchange visited */
} mgpu_stats;

/* Default solver options: Cash-Karp 5(4) with the default core's tolerances
 * (cpp/memilio/math/stepper_wrapper.h:83-91), dt0 0.1, exchange every 0.5 days. */
void mgpu_default_solver_opts(mgpu_solver_opts* opts);

/* Create / destroy a context on CUDA device `device`. */
int mgpu_create(int device, mgpu_context** out);
void mgpu_destroy(mgpu_context* ctx);
/* Message of the last failed call on this context (never NULL). */
const char* mgpu_last_error(const mgpu_context* ctx);
/* Caps the device memory this context may allocate (bytes; 0 = free HBM). */
int mgpu_set_memory_budget(mgpu_context* ctx, int64_t bytes);

/*
 * Right-hand side of node models: for k < count,
 *   dydt[k] = f_{nodes[k]}(pop[k], y[k], t[k])
 * Replaces FlowModel::get_derivatives(pop, y, t, dydt)
 * (cpp/memilio/compartments/flow_model.h:138-144) with osecir::Model::get_flows
 * (cpp/models/ode_secir/model.h:82-214). pop, y, dydt: [count][10G] host arrays.
 */
int mgpu_eval_rhs(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes,
                  const double* pop, const double* y, const double* t, double* dydt);

/*
 * Single-node simulations: for k < count, integrate node nodes[k] of `graph`
 * (edges ignored) from t0 to tmax, initial step dt0, recording every accepted
 * step. Replaces mio::simulate / osecir::simulate (cpp/memilio/compartments/simulation.h:99-110,
 * cpp/models/ode_secir/model.h:385-390) and Simulation::advance with its
 * TimeSeries result. out_t [count][max_points], out_y [count][max_points][10G],
 * num_points [count]. Returns MGPU_OUT_OF_RANGE if a trajectory needs more than
 * max_points (num_points then holds max_points). FP64, one thread per node.
 */
int mgpu_simulate(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                  double tmax, double dt0, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                  double* out_y, int32_t* num_points);

/*
 * Flow simulations: for k < count, simulate_flows (cpp/memilio/compartments/
 * flow_simulation.h:104-121) of node nodes[k] of `graph` (edges ignored): the
 * integrator's state is the accumulated flows (starting at zero) and the
 * population is the initial population plus the flows scattered to their
 * compartments. Every accepted step is recorded: out_t [count][max_points],
 * out_flows [count][max_points][15G] (flat index g*15 + k as the Flows
 * typelist), out_y [count][max_points][10G] (compute_population_results).
 * FP64, one thread per node.
 */
int mgpu_simulate_flows(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                        double tmax, double dt0, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                        double* out_flows, double* out_y, int32_t* num_points);

/*
 * mgpu_simulate with a step size that persists across calls, as
 * Simulation::advance keeps it (cpp/memilio/compartments/simulation_base.h:86-168,
 * cpp/memilio/math/integrator.h:184-249): dt [count] holds each node's initial
 * step on entry and the integrator's next step (Simulation::get_dt) on return.
 */
int mgpu_simulate_dt(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                     double tmax, double* dt, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                     double* out_y, int32_t* num_points);

/*
 * Allocation-free variant of mgpu_simulate for callers that must not allocate
 * device memory inside their loop. No counterpart in the reference: MEmilio
 * integrates on the host, where this question does not arise.
 *
 * Who needs it: every other entry point allocates its device buffers per call
 * (cudaMalloc) and frees them again (cudaFree), and cudaFree waits for the
 * whole device. A caller that keeps other work in flight on other streams (a
 * request loop overlapping solves) would stall on that wait, and a caller whose
 * device memory is held by another allocator (a framework's caching allocator
 * that owns the free HBM) may not get the memory at all. This call uses only
 * memory the caller already owns plus a fixed work space inside the library.
 *
 * What it does: integrates `count` isolated nodes from t0 to tmax with initial
 * step dt0 and the plain FP64 integrator of mgpu_simulate (same kernel
 * arithmetic, so the same final states), and writes only the final states.
 * The nodes share num_groups G, num_contact_matrices M and num_damping_points K.
 * Every array is DEVICE memory owned by the caller:
 *   params          [count][MGPU_PARAM_STRIDE(G)]
 *   contact         [count][M][2][G][G]   baseline, then minimum, per matrix
 *   damping_times   [count][M][K]         (NULL when K == 0; non-decreasing)
 *   damping_values  [count][M][K][G][G]   (NULL when K == 0)
 *   y0              [count][10G]
 *   y_out           [count][10G]          equal to y0 (in place) or not overlapping it
 *   status          [count]               0 = reached tmax, bit 0 = step cap hit,
 *                                         bit 1 = non-finite state
 * The call enqueues one kernel on the context's stream and returns without
 * waiting; the outputs are valid once that stream has been synchronized.
 *
 * Limit: the work space is MGPU_NOALLOC_SCRATCH_BYTES (4 MiB), of which a call
 * needs 640 * G * count bytes (8 stage vectors of 10G doubles per node), so
 * count * G <= 6553 (count <= 1092 nodes at G = 6). Larger calls return
 * MGPU_OUT_OF_RANGE without launching anything.
 *
 * Nothing in the work space has to start at zero: every stage vector is
 * written before it is read, and `status` is written for every node.
 *
 * Set-up: the first call on each device looks up the work space's device
 * address (cudaGetSymbolAddress), which may load the library's device code;
 * make that first call before any stream capture begins on that device.
 * The address is kept for the life of the process: after cudaDeviceReset (a
 * new primary context) the library must not be used again in that process.
 *
 * Overlapping calls race: all calls on one device share the one work space, so
 * a call must not start while another call's kernel may still run (on another
 * stream or from another thread); two calls on the same stream are ordered.
 *
 * Returns MGPU_INVALID_VALUE / MGPU_UNSUPPORTED for bad arguments as
 * mgpu_simulate does, MGPU_CUDA_ERROR if the launch fails. It does not update
 * mgpu_last_error (setting the message could allocate host memory).
 */
#define MGPU_NOALLOC_SCRATCH_BYTES (4 * 1024 * 1024)
int mgpu_simulate_final_noalloc(mgpu_context* ctx, int32_t num_groups, int32_t num_contact_matrices,
                                int32_t num_damping_points, int32_t count, const double* params,
                                const double* contact, const double* damping_times, const double* damping_values,
                                const double* y0, double t0, double tmax, double dt0,
                                const mgpu_integrator_opts* opts, double* y_out, int32_t* status);

/*
 * Upload graphs and create their simulations: for every graph b,
 *   make_mobility_sim(t0, opts->dt_exchange, graph_b)
 * (cpp/memilio/mobility/metapopulation_mobility_instant.h:656-678) with each
 * node's Simulation(model, t0, opts->dt0) (cpp/models/ode_secir/model.h:277-280).
 * A batch of several graphs is ParameterStudy's set of runs
 * (cpp/memilio/compartments/parameter_studies.h:288-345); graphs are independent.
 */
int mgpu_batch_create(mgpu_context* ctx, const mgpu_graph* graphs, int32_t num_graphs, double t0,
                      const mgpu_solver_opts* opts, mgpu_batch** out);

/*
 * GraphSimulation::advance(tmax) (cpp/memilio/mobility/graph_simulation.h:101-120)
 * for every graph: node solves, then MobilityEdge::apply_mobility
 * (metapopulation_mobility_instant.h:544-623) every dt_exchange. tmax_per_graph
 * [num_graphs] gives each graph its own horizon; NULL uses `tmax` for all.
 *
 * Graphs fail one by one: a node instance that hits the step cap
 * (max_steps_per_interval) or ends an interval with a NaN/Inf state marks its
 * own graph failed and the batch carries on; every other graph completes as if
 * it ran alone. The call then returns MGPU_STEP_FAILED (the message names the
 * failed graphs) and mgpu_batch_get_failed lists them. In the reference every
 * ParameterStudy run is an independent simulation and a failed adaptive step
 * logs and continues (cpp/memilio/compartments/parameter_studies.h:288-345,
 * cpp/memilio/math/integrator.h:236-246).
 */
int mgpu_batch_advance(mgpu_batch* batch, double tmax, const double* tmax_per_graph);

/*
 * Commuter statistics of the edges of one graph: MobilityEdge's mobility
 * results (MobilityEdge::add_mobility_result_time_point,
 * cpp/memilio/mobility/metapopulation_mobility_instant.h:423-447, with the save
 * indices of MobilityParameters, :145-170, 241-244). At every departure and at
 * every return (after the underflow fix) of an edge that carries travelers,
 * one time point: the exchange time, the travelers' sum over each of num_sets
 * sets of flat compartment indices (g * 10 + c, summed in the set's order), and
 * their sum over all compartments. The sets apply to every edge of the graph:
 * set_offsets [num_sets + 1] (set_offsets[0] = 0), set_indices
 * [set_offsets[num_sets]]. capacity: time points kept per edge (one advance of
 * D days with 0.5-day exchanges makes 2 D). Recording starts with the next
 * advance and restarts at mgpu_batch_reset; num_sets = 0 switches it off for
 * the graph. Batched precisions only (MGPU_UNSUPPORTED for
 * MGPU_PRECISION_FP64_PLAIN).
 */
int mgpu_batch_set_commuter_stats(mgpu_batch* batch, int32_t graph, int32_t num_sets, const int32_t* set_offsets,
                                  const int32_t* set_indices, int32_t capacity);
/* The recorded time points of every edge of the graph (edges in the graph's
 * (start, end) order): counts [E], times [E][capacity], values
 * [E][capacity][num_sets + 1] (times and values may be NULL; the slots after an
 * edge's counts[e] points are zero). MGPU_OUT_OF_RANGE
 * if an edge recorded more points than the capacity (the first ones are kept;
 * counts holds the true numbers). */
int mgpu_batch_get_commuter_stats(mgpu_batch* batch, int32_t graph, int32_t* counts, double* times, double* values);

/*
 * Flow results of every node: FlowSimulation::get_flows()
 * (cpp/memilio/compartments/flow_simulation.h:36-121, flow_simulation_base.h:
 * 64-82) of each SimulationNode of the batch's graphs. With recording on, the
 * node solves also sum, per node, age group and flow, the persons their own
 * model moved along the flow (the 5th-order flow increments of every applied
 * step); mobility moves persons without flows. So between two times, a node's
 * population changes by its flows scattered to their compartments plus what
 * the exchanges moved. The integrator's state stays the population (its error
 * control is over compartments, where FlowSimulation's is over the flows), so
 * the values agree with a FlowSimulation within the integrator's tolerance.
 * mgpu_batch_set_flow_recording(batch, 1) starts from zero (and costs one sum
 * per flow and step); mgpu_batch_reset sets them to zero again.
 * mgpu_batch_get_flows: [sum_b N_b][15 G_b], flat index g * 15 + k in the
 * order of the Flows typelist (models/ode_secir/model.h:45-59).
 * Batched precisions only.
 */
int mgpu_batch_set_flow_recording(mgpu_batch* batch, int32_t on);
int mgpu_batch_get_flows(mgpu_batch* batch, double* out);

/* Failure flags of the node solves since creation or the last reset, per graph
 * [num_graphs]: 0, or MGPU_FAILED_STEP_CAP | MGPU_FAILED_NONFINITE; and the
 * number of failed graphs (either output may be NULL, not both). During an
 * asynchronous advance it waits for the intervals launched so far and reports
 * their flags. */
#define MGPU_FAILED_STEP_CAP 1
#define MGPU_FAILED_NONFINITE 2
int mgpu_batch_get_failed(mgpu_batch* batch, int32_t* flags, int32_t* num_failed);

/*
 * Regroup running graphs into one new batch on `ctx` (no counterpart in the
 * reference; used by request loops to merge small batches): graph i of the new
 * batch is graph src_graph[i] of batch src[i], described again by graphs[i]
 * (the same arrays it was created from), and continues where it stands: node
 * states, node times and step sizes, the graph's exchange clock and failure
 * flag are copied, so it goes on exactly as in its source batch. Every source
 * graph must be between exchange intervals with no travelers away (after a
 * return, or before the first departure), its batch idle (an asynchronous
 * advance may be open if the intervals it launched have finished); the
 * sources must share the device,
 * the precision and the exchange interval, and record no flows or commuter
 * statistics. The sources are left unchanged (destroy them when done); the new
 * batch's next mgpu_batch_launch / mgpu_batch_advance sets the horizons.
 */
int mgpu_batch_regroup(mgpu_context* ctx, const mgpu_graph* graphs, int32_t num_graphs, mgpu_batch* const* src,
                       const int32_t* src_graph, mgpu_batch** out);

/* Restart every graph at time t0 from the initial states given at creation,
 * with the inputs still resident on the device: the equivalent of building
 * a fresh make_mobility_sim(t0, dt, graph) from the same graph
 * (cpp/memilio/mobility/metapopulation_mobility_instant.h:656-678). Clears the
 * failure flags. */
int mgpu_batch_reset(mgpu_batch* batch, double t0);

/* Node states (result last values) of all graphs, concatenated [sum_b N_b][10 G_b]. */
int mgpu_batch_get_state(mgpu_batch* batch, double* out);
/* Per node, the sum over its age groups of one compartment of its current
 * state, all graphs concatenated [sum_b N_b]: the numerator of the dynamic-NPI
 * check's get_infections_relative (cpp/models/ode_secir/model.h:413-423, with
 * compartment = MGPU_ISY), reduced on the device so that the check reads one
 * value per node instead of the whole state. */
int mgpu_batch_get_compartment_sums(mgpu_batch* batch, int32_t compartment, double* out);
/* Graph times GraphSimulation::get_t() [num_graphs]. */
int mgpu_batch_get_time(mgpu_batch* batch, double* out);
/* Replace the node states (e.g. after a host-side intervention) [sum_b N_b][10 G_b]. */
int mgpu_batch_set_state(mgpu_batch* batch, const double* state);
/*
 * Replace the damping cache of contact matrix `matrix` of one node between two
 * advances: the accumulated damping matrices of Dampings::update_cache
 * (memilio/epidemiology/damping.h:570-600) after dampings were added at run
 * time, e.g. by dynamic NPIs (osecir::Simulation::advance, models/ode_secir/
 * model.h:289-367, implement_dynamic_npis in epidemiology/dynamic_npis.h).
 * times [num_points] (first -DBL_MAX, last DBL_MAX), values [num_points][G][G];
 * num_points may not exceed the graph's num_damping_points (the cache is padded
 * with its last point). The graph's damping arrays must not have been shared
 * with another graph of the batch (same host pointers at creation):
 * MGPU_UNSUPPORTED otherwise.
 */
int mgpu_batch_set_damping_cache(mgpu_batch* batch, int32_t graph, int32_t node, int32_t matrix, int32_t num_points,
                                 const double* times, const double* values);
/*
 * The same for the mobility coefficients of one edge (MobilityEdge's
 * coefficient dampings, e.g. after the edge's dynamic NPIs were enacted,
 * mobility/metapopulation_mobility_instant.h:549-566): times [num_points],
 * values [num_points][10 G], num_points <= the graph's num_edge_damping_points;
 * MGPU_UNSUPPORTED if the graph shares its edge coefficient arrays with another.
 */
int mgpu_batch_set_edge_damping_cache(mgpu_batch* batch, int32_t graph, int32_t edge, int32_t num_points,
                                      const double* times, const double* values);
/*
 * One exchange interval in two halves (GraphSimulation::advance,
 * mobility/graph_simulation.h:101-120: all nodes advance, then all edges
 * apply): step_nodes begins the next interval towards tmax (or tmax_per_graph)
 * and solves the nodes to its end; between the halves the node states are the
 * states before the exchange (SimulationNode::get_last_state) and edge caches
 * may be replaced; step_exchange applies the exchange that ends the interval.
 * Batched precisions only. mgpu_batch_advance refuses while a half is pending.
 */
int mgpu_batch_step_nodes(mgpu_batch* batch, double tmax, const double* tmax_per_graph);
int mgpu_batch_step_exchange(mgpu_batch* batch);
int mgpu_batch_get_stats(mgpu_batch* batch, mgpu_stats* out);
/*
 * Asynchronous advance, for request loops that keep several batches in flight
 * (one context, i.e. one stream, per batch): enqueue at most max_phases exchange
 * intervals towards tmax (or tmax_per_graph) and return without waiting;
 * *remaining = intervals still to launch. The horizon is fixed by the first
 * call after creation or after the previous advance finished. Batched
 * precisions only (MGPU_UNSUPPORTED for MGPU_PRECISION_FP64_PLAIN).
 */
int mgpu_batch_launch(mgpu_batch* batch, double tmax, const double* tmax_per_graph, int32_t max_phases,
                      int32_t* remaining);
/* Non-blocking: *done = 1 once the launched intervals have finished on the
 * device. When no interval remains, this also completes the advance (graph
 * times updated) and reports device-side errors as its status. */
int mgpu_batch_query(mgpu_batch* batch, int32_t* done);
/* Node states of one graph of the batch ([N][10G] doubles), waiting for the stream. */
int mgpu_batch_get_graph_state(mgpu_batch* batch, int32_t graph, double* out);
/*
 * Ensemble statistics of the current node states over the graphs of a batch
 * (all graphs of one node count and age-group count, at most 4096):
 * ensemble_mean and ensemble_percentile (cpp/memilio/data/analyze_result.h:
 * 289-338) on the device. mean [N][10G]; out_percentiles [num_percentiles][N][10G]
 * with the value at sorted index floor(runs * p), p in (0, 1). Call after each
 * advance for a time series.
 */
int mgpu_batch_ensemble_stats(mgpu_batch* batch, const double* percentiles, int32_t num_percentiles, double* mean,
                              double* out_percentiles);

/* Autotuner of the batched solver's schedule: for every age-group count of
 * the batch, times one exchange interval of the node solves for each candidate
 * (32, 64 or 128 threads per block; one slot per lane or a persistent grid of
 * 2, 3, 4 or 6 blocks per SM) on a copy of the current state, restores the state
 * and keeps the fastest. Reports the choice for the largest instance list. */
int mgpu_batch_autotune(mgpu_batch* batch, int32_t* instances_per_block, int32_t* grid_blocks);
/* Upper estimate of the device bytes mgpu_batch_create would allocate for these
 * graphs (admission control); -1 for invalid arguments. */
int64_t mgpu_batch_estimate_bytes(const mgpu_graph* graphs, int32_t num_graphs, const mgpu_solver_opts* opts);

/* Event-measured device times of the last advance (no reference counterpart:
 * replaces the reference's wall-clock timers, cpp/memilio/timer/auto_timer.h). */
int mgpu_batch_get_timing(mgpu_batch* batch, mgpu_timing* out);
/* Device bytes held by the batch. */
int64_t mgpu_batch_device_bytes(const mgpu_batch* batch);
void mgpu_batch_destroy(mgpu_batch* batch);

/*
 * Serving: a device-resident request loop with continuous batching (no
 * counterpart in the reference, which runs one simulation per call).
 *
 * mgpu_server_submit queues a solve of one graph from t0 to tmax; the graph's
 * host arrays must stay valid until the request has been taken.
 * mgpu_server_step runs one scheduling round without waiting for the device:
 * running batches whose launched exchange intervals have finished get their
 * next intervals enqueued (each batch on its own stream, so batches admitted
 * at different times overlap on the device); a request completes as soon as
 * the intervals up to its own horizon have finished; a batch whose requests
 * have all completed releases its device memory; then the queued requests
 * that fit into the memory budget are admitted as a new batch (one batch per
 * start time). mgpu_server_take hands out one completed request: its id, its
 * final node states ([N][10G] doubles, N and G of its graph), the time from
 * submission to completion, and its status as the return value (*request_id = 0
 * when none is ready). With final_state = NULL it only reports the next ready
 * request's id and value count and keeps it ready.
 */
typedef struct mgpu_server mgpu_server;
typedef struct mgpu_server_opts {
    mgpu_solver_opts solver;       /* batched precision; default mixed */
    int64_t memory_budget;         /* bytes the server may hold; 0 = 90% of the free HBM at creation */
    int32_t max_batches;           /* batches (streams) in flight, default 16 */
    int32_t phases_per_launch;     /* exchange intervals enqueued per batch and round, default 2 */
    int32_t max_graphs_per_batch;  /* default 4096 */
    int32_t min_batch_graphs;      /* while batches run, admit once this many requests wait ... */
    double max_wait_ms;            /* ... or the oldest has waited this long (default 1 and 0:
                                      at once); with nothing running, requests are admitted at once */
    int32_t rebatch_max_graphs;    /* re-batching: while the batch limit holds back admission,
                                      running batches of at most this many unfinished requests that
                                      stand between intervals with no travelers away are merged
                                      into one (mgpu_batch_regroup), which frees batch slots and
                                      runs their intervals as one launch sequence; 0 = off
                                      (default: a merge rebuilds the merged graphs' batch on the
                                      host, which on uneven request streams cost more latency
                                      than the launches it saved) */
    int32_t pad;
} mgpu_server_opts;

void mgpu_default_server_opts(mgpu_server_opts* opts);
int mgpu_server_create(int device, const mgpu_server_opts* opts, mgpu_server** out);
void mgpu_server_destroy(mgpu_server* server);
int mgpu_server_submit(mgpu_server* server, const mgpu_graph* graph, double t0, double tmax, int64_t* request_id);
int mgpu_server_step(mgpu_server* server, int32_t* completed, int32_t* running, int32_t* queued);
int mgpu_server_take(mgpu_server* server, int64_t* request_id, double* final_state, int64_t capacity,
                     int64_t* count, double* latency_s);
/* Device bytes held by running batches, and their number. */
int64_t mgpu_server_memory_in_use(const mgpu_server* server);
int32_t mgpu_server_num_batches(const mgpu_server* server);
/* Re-batching merges the server has made (rebatch_max_graphs). */
int64_t mgpu_server_num_merges(const mgpu_server* server);

#ifdef __cplusplus
}
#endif

#endif /* MIOGPU_H */
