/*
 * miogpu_layout.h — the in-memory format of an age-resolved ODE-SECIR
 * metapopulation graph, shared by the GPU library (libmiogpu), the C++
 * facade and the CPU oracle.
 *
 * Everything is plain C: flat arrays, row-major, FP64 unless noted.
 *
 * Compartments (osecir::InfectionState, models/ode_secir/infection_state.h:33-47)
 * are stored per age group, group-major: flat index = g*10 + c, exactly the
 * flat index of Populations<FP, AgeGroup, InfectionState>
 * (memilio/utils/custom_index_array.h:59-95).
 *
 * The 15 flows per group are ordered as the osecir Flows typelist
 * (models/ode_secir/model.h:45-59); flat flow index = g*15 + k
 * (memilio/compartments/flow_model.h:181-192).
 */
#ifndef MIOGPU_LAYOUT_H
#define MIOGPU_LAYOUT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGPU_NUM_COMPARTMENTS 10
#define MGPU_NUM_FLOWS 15

/* osecir::InfectionState */
enum mgpu_compartment {
    MGPU_S = 0,    /* Susceptible */
    MGPU_E,        /* Exposed */
    MGPU_INS,      /* InfectedNoSymptoms */
    MGPU_INSC,     /* InfectedNoSymptomsConfirmed */
    MGPU_ISY,      /* InfectedSymptoms */
    MGPU_ISYC,     /* InfectedSymptomsConfirmed */
    MGPU_ISEV,     /* InfectedSevere */
    MGPU_ICRI,     /* InfectedCritical */
    MGPU_R,        /* Recovered */
    MGPU_D         /* Dead */
};

/* Scalar parameters, at the head of each node's parameter record
 * (models/ode_secir/parameters.h:47-84,358-394,765-767). */
enum mgpu_scalar_param {
    MGPU_P_START_DAY = 0,
    MGPU_P_SEASONALITY,
    MGPU_P_ICU_CAPACITY,
    MGPU_P_TNT_CAPACITY,              /* TestAndTraceCapacity */
    MGPU_P_TNT_MAX_RISK,              /* TestAndTraceCapacityMaxRisk */
    MGPU_P_COMMUTER_NONDETECTION,     /* Parameters::get_commuter_nondetection */
    MGPU_P_START_COMMUTER_DETECTION,
    MGPU_P_END_COMMUTER_DETECTION,
    MGPU_NUM_SCALAR_PARAMS
};

/* Per-age-group parameters (parameters.h:96-324). Stored as G consecutive
 * values per parameter after the scalars. */
enum mgpu_group_param {
    MGPU_G_TIME_EXPOSED = 0,
    MGPU_G_TIME_INS,                  /* TimeInfectedNoSymptoms */
    MGPU_G_TIME_ISY,                  /* TimeInfectedSymptoms */
    MGPU_G_TIME_ISEV,                 /* TimeInfectedSevere */
    MGPU_G_TIME_ICRI,                 /* TimeInfectedCritical */
    MGPU_G_TRANSMISSION_PROB,         /* TransmissionProbabilityOnContact */
    MGPU_G_REL_TRANSMISSION_NS,       /* RelativeTransmissionNoSymptoms */
    MGPU_G_RECOVERED_PER_INS,         /* RecoveredPerInfectedNoSymptoms */
    MGPU_G_RISK_FROM_SYMPTOMATIC,     /* RiskOfInfectionFromSymptomatic */
    MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, /* MaxRiskOfInfectionFromSymptomatic */
    MGPU_G_SEVERE_PER_ISY,            /* SeverePerInfectedSymptoms */
    MGPU_G_CRITICAL_PER_SEVERE,       /* CriticalPerSevere */
    MGPU_G_DEATHS_PER_SEVERE,         /* DeathsPerSevere */
    MGPU_G_DEATHS_PER_CRITICAL,       /* DeathsPerCritical */
    MGPU_NUM_GROUP_PARAMS
};

#define MGPU_PARAM_STRIDE(G) (MGPU_NUM_SCALAR_PARAMS + MGPU_NUM_GROUP_PARAMS * (G))
#define MGPU_GROUP_PARAM(p, g, G) (MGPU_NUM_SCALAR_PARAMS + (p) * (G) + (g))

/* Largest number of age groups the GPU kernels accept. */
#define MGPU_MAX_GROUPS 8
/* Largest number of contact matrices in a ContactMatrixGroup. */
#define MGPU_MAX_CONTACT_MATRICES 4

/*
 * One metapopulation graph: Graph<SimulationNode<Simulation>, MobilityEdge>
 * (memilio/mobility/graph.h:144-303, metapopulation_mobility_instant.h).
 *
 * Contact patterns: ContactMatrixGroup of M matrices (contact_matrix.h:392-399).
 * Matrix m of node v has a baseline and a minimum (G x G) and a damping
 * cache of K points: the accumulated damping matrices D_k that
 * Dampings::update_cache (damping.h:570-600) builds, each valid from time
 * t_k. K == 0 means no dampings (the contact matrix is its baseline).
 * Otherwise the first point must be (-DBL_MAX, 0) and the last (DBL_MAX, ...)
 * as in the reference cache; K is the same for all matrices of all nodes
 * of one graph. Shorter caches are padded with extra points at time
 * DBL_MAX that repeat the last matrix; lookups never select them.
 *
 * Edges are sorted by (src, dst) as Graph::add_edge keeps them
 * (graph.h:231-241). Mobility coefficients follow the same damping-cache
 * convention with Ke points (MobilityCoefficients = DampingMatrixExpression
 * over VectorDampings, metapopulation_mobility_instant.h:103-110).
 */
typedef struct mgpu_graph {
    int32_t num_nodes;              /* N */
    int32_t num_groups;             /* G */
    int32_t num_edges;              /* E */
    int32_t num_contact_matrices;   /* M >= 1 */
    int32_t num_damping_points;     /* K >= 0 */
    int32_t num_edge_damping_points;/* Ke >= 0 */
    const double* params;           /* [N][MGPU_PARAM_STRIDE(G)] */
    const double* contact_baseline; /* [N][M][G][G] */
    const double* contact_minimum;  /* [N][M][G][G] */
    const double* damping_times;    /* [N][M][K] */
    const double* damping_values;   /* [N][M][K][G][G] */
    const double* init_state;       /* [N][10G] */
    const int32_t* edge_src;        /* [E] */
    const int32_t* edge_dst;        /* [E] */
    const double* edge_coeff_baseline; /* [E][10G] */
    const double* edge_coeff_minimum;  /* [E][10G], may be NULL (zeros) */
    const double* edge_damping_times;  /* [E][Ke] */
    const double* edge_damping_values; /* [E][Ke][10G] */
} mgpu_graph;

/* Integrator choice and options. */
enum mgpu_method {
    MGPU_METHOD_CASH_KARP54 = 0, /* ControlledStepperWrapper<runge_kutta_cash_karp54> (default core) */
    MGPU_METHOD_RKF45 = 1        /* RKIntegratorCore (math/adapt_rk.h) */
};

typedef struct mgpu_integrator_opts {
    int32_t method;   /* enum mgpu_method */
    int32_t reserved;
    double abs_tol;   /* default 1e-10 (stepper_wrapper.h:83) */
    double rel_tol;   /* default 1e-5 */
    double dt_min;    /* default DBL_MIN */
    double dt_max;    /* default DBL_MAX */
} mgpu_integrator_opts;

#ifdef __cplusplus
}
#endif

#endif /* MIOGPU_LAYOUT_H */
