// mgpu_internal.cuh — device-side data structures and the FP64 thread-level
// ODE-SECIR model shared by the kernels of libmiogpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/miogpu.h"

namespace mgpu
{

constexpr int kC = MGPU_NUM_COMPARTMENTS;
constexpr int kF = MGPU_NUM_FLOWS;
constexpr double kPi = 3.14159265358979323846;
constexpr double kZeroTol = 1e-12; // Limits<double>::zero_tolerance (memilio/config.h:73-79)

// Device error word bits (per batch).
enum : int32_t {
    ERR_STEP_CAP   = 1, // an instance exceeded max steps in one interval
    ERR_NONFINITE  = 2, // NaN/Inf in a state
    ERR_BAD_GRAPH  = 4, // inconsistent graph descriptor met on the device
    ERR_SEQ_BOUNDS = 8  // sequential exchange met an out-of-range index
};

// Immutable per-graph descriptor (offsets into the batch pools).
struct DevGraph {
    int32_t N, G, E, M, K, Ke;
    int32_t n;      // 10 G
    int32_t method; // integrator
    int64_t node0;  // first global node id
    int64_t edge0;  // first global edge id
    int64_t param_off;   // doubles, [N][stride(G)]
    int64_t contact_off; // doubles, [N][M][2][G][G] (baseline, minimum)
    int64_t dtime_off;   // doubles, [N][M][K]
    int64_t dval_off;    // doubles, [N][M][K][G][G]
    int64_t state_off;   // doubles, [N][n] (state, v0, ypre, ynew pools share it)
    int64_t ecoef_off;   // doubles, [E][2][n] (baseline, minimum)
    int64_t edt_off;     // doubles, [E][Ke]
    int64_t edv_off;     // doubles, [E][Ke][n]
    int64_t ecoef_f_off; // [E][n] floats before the records: the edges' first row * 10 (Ke == 0, mixed)
    int32_t mob_mask;    // compartments c with a nonzero coefficient on some edge and age group
    int32_t staged;      // the FP32 return and departure run one CTA per graph from shared memory
    int64_t ecoef_in_off; // ecoef_in row of the graph's first in-edge (its in-edges in CSC order), or -1
    int64_t trav0;       // traveler-record offset of the graph's first edge ([E][n] doubles)
};

// Mutable per-graph state (GraphSimulation::m_t and the edges' shared return flag).
struct GraphRt {
    double t;          // graph time
    double t_next;     // end of the current interval
    double dt;         // length of the current interval
    double tmax;       // horizon
    double t_dep;      // time of the pending departure
    double t_ret;      // its return time (t_dep + dt at departure)
    int32_t return_mobile; // MobilityEdge::m_return_mobile_population (identical for all edges)
    int32_t active;    // takes part in the current interval
    int32_t fallback;  // current return needs the sequential path
    int32_t has_pending; // travelers are away
    int32_t do_return; // current interval ends with returns
    int32_t do_depart; // current interval ends with departures
    int32_t snap_slot; // snapshot slot of the pending departure (batched exchange)
    int32_t pad1;
};

// Integrator options on the device.
struct DevOpts {
    double abs_tol, rel_tol, dt_min, dt_max;
    int32_t max_steps;
    int32_t method;
};

// Commuter statistics of the edges of one graph (MobilityEdge's mobility
// results, add_mobility_result_time_point): per edge, one time point per
// departure and per return, the travelers' sums over num_sets sets of flat
// compartment indices and their total.
struct EdgeStatsDev {
    int32_t num_sets;        // 0: not recorded
    int32_t capacity;        // time points kept per edge
    const int32_t* set_ptr;  // [num_sets + 1]
    const int32_t* set_idx;  // [set_ptr[num_sets]]
    int32_t* count;          // [E] time points recorded (later ones beyond capacity are counted only)
    double* times;           // [E][capacity]
    double* values;          // [E][capacity][num_sets + 1]
};

// All device pointers of a batch.
struct BatchDev {
    int32_t num_graphs;
    int64_t num_nodes, num_edges;
    const DevGraph* graphs;
    GraphRt* rt;
    const int32_t* node_graph;   // [num_nodes]
    const int32_t* edge_graph;   // [num_edges]
    const double* params;
    const double* contact;
    const double* dtimes;
    const double* dvals;
    double* state;               // result last values (FP64 solvers)
    double* v0;                  // post-departure snapshot (destination state at t_dep)
    double* ypre;                // pre-exchange snapshot
    double* ynew;                // scratch for the parallel return
    // mixed solver: the same three arrays as float-float pairs (value = hi + lo)
    float *st_hi, *st_lo, *v0_hi, *v0_lo, *yn_hi, *yn_lo;
    double* node_t;              // integrator time per node
    double* node_dt;             // integrator step per node
    const int32_t* edge_src;     // global node ids
    const int32_t* edge_dst;
    const double* ecoef;
    const double* edt;
    const double* edv;
    const uint8_t* edge_static_any; // coefficients constant and some > 0 (Ke == 0)
    uint8_t* edge_pending;       // travelers away on this edge
    double* trav;                // [sum_e n_e] stored travelers
    double* mfix;                // [sum_e n_e] travelers after an underflow fix at the destination
    int32_t* edge_fixed;         // [num_edges] number of fixed compartments (0: mfix unused)
    uint8_t* node_flag;          // [num_nodes] return needs the exact per-node scan
    uint8_t* node_dirty;         // [2][num_nodes] an out-edge changed: rescan (double-buffered)
    // batched exchange: exact-scan work lists (0: flagged by the bound, 1/2: rescans)
    // node instances per age-group count (dense (node, group) mappings): glist[G], gcount[G]
    int32_t mob_union;           // OR of the graphs' mob_mask
    const int32_t* glist[MGPU_MAX_GROUPS + 1];
    int64_t gcount[MGPU_MAX_GROUPS + 1];
    // the mixed node kernel's order of the same instances for the current interval
    // (nodes expected to need one step first, the others last) and its two fill
    // counters per age-group count, zeroed at each interval start
    int32_t* gorder[MGPU_MAX_GROUPS + 1];
    int32_t* order_cnt; // [2 * (MAX_GROUPS + 1)]
    int32_t* scan_mark;          // [3][num_nodes * MAX_GROUPS] (node, group) item is in list k
    int32_t* scan_list;          // [3][num_nodes * MAX_GROUPS] items node * MAX_GROUPS + group
    int32_t* scan_count;         // [3]
    uint8_t* fix_cnt;            // [num_edges][MAX_GROUPS] fixed compartments per edge and age group
    int32_t* fix_edges;          // [fix_cap] edges whose fix counts became nonzero in this interval
    int32_t* fix_meta;           // [2]: entries pushed, overflow flag (zeroed at each interval start)
    int64_t fix_cap;
    const int64_t* trav_off;     // [num_edges] offset of each edge's travelers
    const int64_t* out_ptr;      // [num_nodes+1] CSR (edges sorted by (src, dst))
    const int64_t* in_ptr;       // [num_nodes+1] CSC
    const int64_t* in_edges;     // [num_edges] edge ids sorted by (dst, src)
    const int2* in_se;           // [num_edges] (source node, edge id) of in_edges[k]
    const int64_t* in_mid;       // [num_nodes] first k of the node's in-edges with a higher source
    int64_t state_total;         // doubles in a state pool
    double* ysnap;               // [2][state_total] departure snapshots (batched exchange)
    float* gsnap;                // [2][state_total / 10][kRec] FP32 snapshot records (mixed), see rec_vec
    void* risk;                  // [2][num_nodes][MAX_GROUPS] ISy mobility factor at departure (R)
    void* aux;                   // [num_nodes][MAX_GROUPS][12] return-time force of infection and rates (R)
    const float* ecoef_r;        // FP32 coefficient records of edges without dampings (mixed), see rec_vec
    const float* ecoef_u;        // the same as one value per (edge, group) row when every moved
                                 // compartment has the same coefficient everywhere (else null)
    const float* ecoef_in;       // ecoef_u in each graph's in-edge (CSC) order, [in-edge][group], so
                                 // that an in-edge's coefficient is read without its edge id first
    // chunks of the graphs whose FP32 return and departure run with the graph's
    // snapshot records (and return-time rates) copied to shared memory, one CTA
    // per chunk: (graph, chunk << 16 | chunks of the graph); their count and
    // the dynamic shared memory of those launches
    const int2* xs_work;
    // the node instances of the other graphs, per age-group count, for the
    // FP32 passes over node lists
    const int32_t* xlist[MGPU_MAX_GROUPS + 1];
    int64_t xcount[MGPU_MAX_GROUPS + 1];
    int32_t xs_count;
    int32_t xs_smem_ret, xs_smem_dep;
    int32_t xs_aux; // the staged return also copies the return-time rates
    const float* tab_f;          // [num_nodes][MAX_GROUPS][kTabF] FP32 node constants (mixed solver)
    const float* contact_f;      // FP32 copy of the contact pool
    const float* dvals_f;        // FP32 copy of the damping-value pool
    double* scratch;             // plain ODE stage vectors, [8][scratch_nmax][scratch_stride]
    int64_t scratch_stride;      // node slots (distance between consecutive components)
    int32_t scratch_nmax;        // components per scratch vector
    DevOpts opts;
    const EdgeStatsDev* estats;  // [num_graphs] commuter statistics, or null (none recorded)
    double* flows;               // [state_total / 10][15] accumulated flows per (node, group), or null
    int32_t* err;                // device error word (ERR_* bits of the whole batch)
    int32_t* graph_err;          // [num_graphs] ERR_STEP_CAP / ERR_NONFINITE of each graph's own instances
    unsigned long long* counters; // [8]: accepted, rejected, failed, underflow, sequential
};

enum { CNT_ACCEPTED = 0, CNT_REJECTED, CNT_FAILED, CNT_UNDERFLOW, CNT_SEQUENTIAL, CNT_SCANNED, CNT_NUM };

// FP32 per-(node, age group) constants of the mixed solver, computed once from
// the FP64 parameters (rates as the reference forms them: (1-mu)*(1/T) etc.).
enum {
    TF_A_TNT = 0, TF_BETA, TF_XI, TF_RHO, TF_RHO_MAX, TF_R1, TF_R2, TF_R3, TF_R6, TF_R7, TF_R11, TF_R13, TF_R14,
    TF_R10L, TF_R12L, TF_CPS, TF_DPS, TF_INV_TISEV, TF_TNT_CAP, TF_TNT_CAP2, TF_ICU_LO, TF_ICU_CAP, TF_SEASON_K,
    kTabF = 24
};

// FP32 group records of the mixed exchange: the departure snapshot of a
// (node, age group) with its two mobility factors, and the coefficients of an
// (edge, age group), 12 floats each in three float4 vectors. Within a node (an
// edge) the records are vector-major, [vector][group][4], so that the age
// groups of one node read one contiguous block per vector. Vector 0 holds S, E,
// INS, ISy (the usual commuter compartments), vector 1 R, the ISy mobility
// factor, the commuter nondetection factor and INSC, vector 2 ISyC, ISev, ICri,
// D. Coefficient records keep the two factor slots zero. Rows are dense
// (node, group) or (edge, group) ordinals: a node's first row is its state
// offset / 10, an edge's is ecoef_f_off / 10 + (local edge) * G.
constexpr int kRec = 12;
// the usual commuter compartments S, E, INS, ISy, R as a bit mask
constexpr int kMaskSEIYRBits = (1 << MGPU_S) | (1 << MGPU_E) | (1 << MGPU_INS) | (1 << MGPU_ISY) | (1 << MGPU_R);
enum { REC_RISK = 5, REC_ND = 6 };
__host__ __device__ constexpr int rec_pos(int c)
{
    return c == MGPU_S ? 0 : c == MGPU_E ? 1 : c == MGPU_INS ? 2 : c == MGPU_ISY ? 3 : c == MGPU_R ? 4
         : c == MGPU_INSC ? 7 : c == MGPU_ISYC ? 8 : c == MGPU_ISEV ? 9 : c == MGPU_ICRI ? 10 : 11;
}
// float offset of vector v of group gr's record, the node's (edge's) rows starting at row r0
__host__ __device__ inline int64_t rec_vec(int64_t r0, int G, int gr, int v)
{
    return r0 * kRec + (int64_t)v * G * 4 + (int64_t)gr * 4;
}
__host__ __device__ inline int64_t rec_elem(int64_t r0, int G, int gr, int p)
{
    return rec_vec(r0, G, gr, p / 4) + p % 4;
}

// Return-side values per (node, age group) at the pending departure, written
// before each return: lambda, r1, r2, r3, r6, r7, r10, r11, r12, r13, r14 and a
// flag (1: one Euler step of the interval's length may drive a compartment negative).
constexpr int kAux = 12;

// A node instance of graph gi hit the step cap or ended its interval with a
// non-finite state: recorded for that graph (the other graphs of the batch run
// on unaffected) and in the batch's error word.
__device__ __forceinline__ void report_instance_failure(const BatchDev& B, int gi, bool cap_hit, bool nonfinite)
{
    const int32_t bits = (cap_hit ? ERR_STEP_CAP : 0) | (nonfinite ? ERR_NONFINITE : 0);
    if (bits) {
        atomicOr(B.graph_err + gi, bits);
        atomicOr(B.err, bits);
    }
}

// The mixed solvers keep node states as float-float pairs and share the FP32
// exchange; they differ only in the node kernel's step arithmetic.
__host__ __device__ inline bool is_mixed(int precision)
{
    return precision == MGPU_PRECISION_MIXED || precision == MGPU_PRECISION_MIXED_FP64_CONTROL;
}

__host__ __device__ inline int param_stride(int G)
{
    return MGPU_NUM_SCALAR_PARAMS + MGPU_NUM_GROUP_PARAMS * G;
}

// Node state access for code shared by both representations (FP64 array, or
// float-float pairs in the mixed solver).
__device__ __forceinline__ double state_get(const BatchDev& B, int64_t o)
{
    return B.st_hi ? (double)B.st_hi[o] + (double)B.st_lo[o] : B.state[o];
}
__device__ __forceinline__ void pair_set(float* hi, float* lo, int64_t o, double v)
{
    const float h = (float)v;
    hi[o]         = h;
    lo[o]         = (float)(v - (double)h);
}
__device__ __forceinline__ void state_set(const BatchDev& B, int64_t o, double v)
{
    if (B.st_hi) {
        pair_set(B.st_hi, B.st_lo, o, v);
    }
    else {
        B.state[o] = v;
    }
}
__device__ __forceinline__ double v0_get(const BatchDev& B, int64_t o)
{
    return B.v0_hi ? (double)B.v0_hi[o] + (double)B.v0_lo[o] : B.v0[o];
}
__device__ __forceinline__ void ynew_set(const BatchDev& B, int64_t o, double v)
{
    if (B.yn_hi) {
        pair_set(B.yn_hi, B.yn_lo, o, v);
    }
    else {
        B.ynew[o] = v;
    }
}

// Source/target compartment of the 15 flows (osecir Flows typelist, models/ode_secir/model.h:45-59).
__device__ __constant__ const int8_t kFlowSrc[kF] = {MGPU_S,    MGPU_E,    MGPU_INS,  MGPU_INS,  MGPU_INSC,
                                                      MGPU_INSC, MGPU_ISY,  MGPU_ISY,  MGPU_ISYC, MGPU_ISYC,
                                                      MGPU_ISEV, MGPU_ISEV, MGPU_ISEV, MGPU_ICRI, MGPU_ICRI};
__device__ __constant__ const int8_t kFlowDst[kF] = {MGPU_E,    MGPU_INS,  MGPU_ISY,  MGPU_R,    MGPU_ISYC,
                                                      MGPU_R,    MGPU_ISEV, MGPU_R,    MGPU_ISEV, MGPU_R,
                                                      MGPU_ICRI, MGPU_R,    MGPU_D,    MGPU_D,    MGPU_R};

// The same tables as compile-time functions (fold to register indices in unrolled loops).
__host__ __device__ __forceinline__ constexpr int kFlowSrcI(int f)
{
    return f == 0 ? MGPU_S
         : f == 1 ? MGPU_E
         : f <= 3 ? MGPU_INS
         : f <= 5 ? MGPU_INSC
         : f <= 7 ? MGPU_ISY
         : f <= 9 ? MGPU_ISYC
         : f <= 12 ? MGPU_ISEV
                   : MGPU_ICRI;
}
__host__ __device__ __forceinline__ constexpr int kFlowDstI(int f)
{
    return f == 0 ? MGPU_E
         : f == 1 ? MGPU_INS
         : f == 2 ? MGPU_ISY
         : f == 3 ? MGPU_R
         : f == 4 ? MGPU_ISYC
         : f == 5 ? MGPU_R
         : f == 6 ? MGPU_ISEV
         : f == 7 ? MGPU_R
         : f == 8 ? MGPU_ISEV
         : f == 9 ? MGPU_R
         : f == 10 ? MGPU_ICRI
         : f == 11 ? MGPU_R
         : f == 12 ? MGPU_D
         : f == 13 ? MGPU_D
                   : MGPU_R;
}

// smoother_cosine (memilio/math/smoother.h:46-60).
template <class R>
__device__ __forceinline__ R smoother_cosine(R x, R xleft, R xright, R yleft, R yright)
{
    if (x <= xleft) {
        return yleft;
    }
    if (x >= xright) {
        return yright;
    }
    return R(0.5) * (yleft - yright) * cos(R(kPi) / (xright - xleft) * (x - xleft)) + R(0.5) * (yleft + yright);
}

// The branch of a cosine smoother, shared by all coefficients that use the
// same x and interval: 0 = left value, 1 = right value, 2 = ramp with cosine c.
struct Ramp {
    int mode;
    double c;
};

__device__ __forceinline__ Ramp ramp_at(double x, double xleft, double xright)
{
    Ramp r;
    if (x <= xleft) {
        r.mode = 0;
        r.c    = 0.0;
    }
    else if (x >= xright) {
        r.mode = 1;
        r.c    = 0.0;
    }
    else {
        r.mode = 2;
        r.c    = cos(kPi / (xright - xleft) * (x - xleft));
    }
    return r;
}

__device__ __forceinline__ double ramp_apply(const Ramp& r, double yleft, double yright)
{
    return r.mode == 0 ? yleft : (r.mode == 1 ? yright : 0.5 * (yleft - yright) * r.c + 0.5 * (yleft + yright));
}

// Position in a damping cache (Dampings::get_matrix_at, memilio/epidemiology/damping.h:381-396):
// ub = first point with time > t; the matrix is a cosine ramp over [t_ub - 1, t_ub].
__device__ __forceinline__ int damping_upper_bound(const double* times, int K, double t)
{
    int ub = 0;
    while (ub < K && !(t < times[ub])) {
        ++ub;
    }
    return ub < K ? ub : K - 1;
}

// Node model accessor over the batch pools.
struct NodeModel {
    int G, M, K;
    const double* p;      // parameter record
    const double* cm;     // [M][2][G][G]
    const double* dtimes; // [M][K]
    const double* dvals;  // [M][K][G][G]
    __device__ double scalar(int w) const
    {
        return p[w];
    }
    __device__ double gp(int w, int g) const
    {
        return p[MGPU_NUM_SCALAR_PARAMS + w * G + g];
    }
};

__device__ __forceinline__ NodeModel node_model(const BatchDev& B, const DevGraph& g, int64_t local)
{
    NodeModel m;
    m.G            = g.G;
    m.M            = g.M;
    m.K            = g.K;
    const long GG  = (long)g.G * g.G;
    m.p            = B.params + g.param_off + local * param_stride(g.G);
    m.cm           = B.contact + g.contact_off + local * g.M * 2 * GG;
    m.dtimes       = g.K ? B.dtimes + g.dtime_off + local * g.M * g.K : nullptr;
    m.dvals        = g.K ? B.dvals + g.dval_off + local * g.M * g.K * GG : nullptr;
    return m;
}

// Strided vector view (SoA scratch or contiguous rows).
struct SVec {
    double* p;
    int64_t s;
    __device__ __forceinline__ double& operator[](int i) const
    {
        return p[(int64_t)i * s];
    }
};
struct CVec {
    const double* p;
    int64_t s;
    __device__ __forceinline__ double operator[](int i) const
    {
        return p[(int64_t)i * s];
    }
};

// ContactMatrixGroup::get_matrix_at(t) element (i, j) times the seasonality
// factor, for all (i, j) at once (contact_matrix.h:190-194,392-399).
// `C` receives G*G values (row-major).
__device__ inline void contact_matrix_at(const NodeModel& nm, double t, double* C)
{
    const int G   = nm.G;
    const long GG = (long)G * G;
    for (int k = 0; k < GG; ++k) {
        C[k] = 0.0;
    }
    for (int m = 0; m < nm.M; ++m) {
        const double* B = nm.cm + m * 2 * GG;
        const double* L = B + GG;
        if (nm.K) {
            const double* T  = nm.dtimes + m * nm.K;
            const int ub     = damping_upper_bound(T, nm.K, t);
            const Ramp r     = ramp_at(t, T[ub] - 1.0, T[ub]);
            const double* Dl = nm.dvals + ((long)m * nm.K + ub - 1) * GG;
            const double* Dr = Dl + GG;
            for (int k = 0; k < GG; ++k) {
                const double D = ramp_apply(r, Dl[k], Dr[k]);
                C[k]           = C[k] + (B[k] - D * (B[k] - L[k]));
            }
        }
        else {
            for (int k = 0; k < GG; ++k) {
                C[k] = C[k] + (B[k] - 0.0 * (B[k] - L[k]));
            }
        }
    }
}

// osecir::Model::get_flows + FlowModel::get_derivatives (models/ode_secir/model.h:82-214,
// compartments/flow_model.h:112-144) for one node, FP64, one thread. The
// contact matrix, seasonality and risk smoother are evaluated once per call
// (they depend on t and pop only) instead of once per (i, j).
// The 15 flows of every age group, handed to sink(i, f) group by group.
template <class PopV, class YV, class Sink>
__device__ void secir_flows_core(const NodeModel& nm, const PopV& pop, const YV& y, double t, Sink&& sink)
{
    const int G = nm.G;
    double C[MGPU_MAX_GROUPS * MGPU_MAX_GROUPS];
    contact_matrix_at(nm, t, C);
    double icu = 0.0, tnt = 0.0;
    for (int i = 0; i < G; ++i) {
        tnt += (1 - nm.gp(MGPU_G_RECOVERED_PER_INS, i)) / nm.gp(MGPU_G_TIME_INS, i) * pop[i * kC + MGPU_INS];
        icu += pop[i * kC + MGPU_ICRI];
    }
    const double cap    = nm.scalar(MGPU_P_TNT_CAPACITY);
    const Ramp rrisk    = ramp_at(tnt, cap, cap * nm.scalar(MGPU_P_TNT_MAX_RISK));
    const double season = (1 + nm.scalar(MGPU_P_SEASONALITY) *
                                   sin(kPi * ((nm.scalar(MGPU_P_START_DAY) + t) / 182.5 + 0.5)));
    const double icu_cap = nm.scalar(MGPU_P_ICU_CAPACITY);
    const Ramp ricu      = ramp_at(icu, 0.90 * icu_cap, icu_cap);
    // per source group j: 1/N_j and the infectious pressure
    double divN[MGPU_MAX_GROUPS], press[MGPU_MAX_GROUPS];
    for (int j = 0; j < G; ++j) {
        const int o = j * kC;
        const double Nj = pop[o + MGPU_S] + pop[o + MGPU_E] + pop[o + MGPU_INS] + pop[o + MGPU_ISY] +
                          pop[o + MGPU_ISEV] + pop[o + MGPU_ICRI] + pop[o + MGPU_R];
        divN[j]           = (Nj < kZeroTol) ? 0.0 : 1.0 / Nj;
        const double risk = ramp_apply(rrisk, nm.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, j),
                                       nm.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, j));
        press[j] = nm.gp(MGPU_G_REL_TRANSMISSION_NS, j) * pop[o + MGPU_INS] + risk * pop[o + MGPU_ISY];
    }
    for (int i = 0; i < G; ++i) {
        const int o       = i * kC;
        const double beta = nm.gp(MGPU_G_TRANSMISSION_PROB, i);
        double f[kF];
        f[0] = 0.0;
        for (int j = 0; j < G; ++j) {
            const double cont = season * C[i * G + j];
            f[0] += y[o + MGPU_S] * cont * divN[j] * beta * press[j];
        }
        const double cps       = nm.gp(MGPU_G_CRITICAL_PER_SEVERE, i);
        const double crit_adj  = ramp_apply(ricu, cps, 0.0);
        const double death_adj = cps - crit_adj;
        const double mu        = nm.gp(MGPU_G_RECOVERED_PER_INS, i);
        const double tins      = nm.gp(MGPU_G_TIME_INS, i);
        const double sev       = nm.gp(MGPU_G_SEVERE_PER_ISY, i);
        const double tisy      = nm.gp(MGPU_G_TIME_ISY, i);
        const double tisev     = nm.gp(MGPU_G_TIME_ISEV, i);
        const double dps       = nm.gp(MGPU_G_DEATHS_PER_SEVERE, i);
        const double dpc       = nm.gp(MGPU_G_DEATHS_PER_CRITICAL, i);
        const double ticri     = nm.gp(MGPU_G_TIME_ICRI, i);
        f[1]  = (1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i)) * y[o + MGPU_E];
        f[2]  = (1 - mu) * (1 / tins) * y[o + MGPU_INS];
        f[3]  = mu * (1.0 / tins) * y[o + MGPU_INS];
        f[4]  = (1.0 - mu) * (1.0 / tins) * y[o + MGPU_INSC];
        f[5]  = mu * (1.0 / tins) * y[o + MGPU_INSC];
        f[6]  = sev / tisy * y[o + MGPU_ISY];
        f[7]  = (1 - sev) / tisy * y[o + MGPU_ISY];
        f[8]  = sev / tisy * y[o + MGPU_ISYC];
        f[9]  = (1.0 - sev) / tisy * y[o + MGPU_ISYC];
        f[10] = crit_adj / tisev * y[o + MGPU_ISEV];
        f[11] = (1.0 - cps - dps) / tisev * y[o + MGPU_ISEV];
        f[12] = (dps + death_adj) / tisev * y[o + MGPU_ISEV];
        f[13] = dpc / ticri * y[o + MGPU_ICRI];
        f[14] = (1.0 - dpc) / ticri * y[o + MGPU_ICRI];
        sink(i, f);
    }
}

// dydt = f(pop, y, t): the flows scattered to their compartments (FlowModel::get_derivatives).
template <class PopV, class YV, class OutV>
__device__ void secir_rhs(const NodeModel& nm, const PopV& pop, const YV& y, double t, const OutV& dydt)
{
    for (int k = 0; k < nm.G * kC; ++k) {
        dydt[k] = 0.0;
    }
    secir_flows_core(nm, pop, y, t, [&](int i, const double (&f)[kF]) {
        const int o = i * kC;
#pragma unroll
        for (int k = 0; k < kF; ++k) {
            dydt[o + kFlowSrc[k]] -= f[k];
            dydt[o + kFlowDst[k]] += f[k];
        }
    });
}

// The flows themselves, flat index i*15 + k (osecir::Model::get_flows).
template <class PopV, class YV, class OutV>
__device__ void secir_flows(const NodeModel& nm, const PopV& pop, const YV& y, double t, const OutV& flows)
{
    secir_flows_core(nm, pop, y, t, [&](int i, const double (&f)[kF]) {
#pragma unroll
        for (int k = 0; k < kF; ++k) {
            flows[i * kF + k] = f[k];
        }
    });
}

// Mobility risk factor of the ISy compartments (get_mobility_factors,
// models/ode_secir/model.h:687-715) for group g, from state y.
template <class YV>
__device__ inline double mobility_isy_factor(const NodeModel& nm, const YV& y, int g)
{
    double tnt = 0.0;
    for (int i = 0; i < nm.G; ++i) {
        tnt += (1 - nm.gp(MGPU_G_RECOVERED_PER_INS, i)) / nm.gp(MGPU_G_TIME_INS, i) * y[i * kC + MGPU_INS];
    }
    const double cap = nm.scalar(MGPU_P_TNT_CAPACITY);
    return smoother_cosine(tnt, cap, cap * nm.scalar(MGPU_P_TNT_MAX_RISK), nm.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, g),
                           nm.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, g));
}

// Coefficient j of edge e at time t (MobilityCoefficientGroup::get_matrix_at with one matrix).
__device__ inline double edge_coeff_at(const BatchDev& B, const DevGraph& g, int64_t local_e, int j, double t)
{
    const double* base = B.ecoef + g.ecoef_off + local_e * 2 * g.n;
    const double Bv    = base[j];
    const double Lv    = base[g.n + j];
    double D           = 0.0;
    if (g.Ke) {
        const double* T  = B.edt + g.edt_off + local_e * g.Ke;
        const int ub     = damping_upper_bound(T, g.Ke, t);
        const Ramp r     = ramp_at(t, T[ub] - 1.0, T[ub]);
        const double* Dv = B.edv + g.edv_off + local_e * g.Ke * g.n;
        D                = ramp_apply(r, Dv[(ub - 1) * g.n + j], Dv[ub * g.n + j]);
    }
    return 0.0 + (Bv - D * (Bv - Lv));
}

// Launchers (defined in the .cu files).
void launch_ode_plain(const BatchDev& B, int64_t node_begin, int64_t node_end, cudaStream_t s);
void launch_simulate(const BatchDev& B, const int32_t* d_nodes, int count, double t0, double tmax, double dt0,
                     int max_points, double* d_out_t, double* d_out_y, int32_t* d_num_points, cudaStream_t s,
                     double* d_dt_io = nullptr);
void launch_simulate_flows(const BatchDev& B, const int32_t* d_nodes, int count, double t0, double tmax, double dt0,
                           int max_points, double* d_out_t, double* d_out_f, double* d_out_y, int32_t* d_num_points,
                           int nf_max, double* d_flow_rows, cudaStream_t s);
void launch_eval_rhs(const BatchDev& B, const int32_t* d_nodes, int count, const double* d_pop, const double* d_y,
                     const double* d_t, double* d_dydt, cudaStream_t s);
int launch_ode_batched(const BatchDev& B, int G, int precision, const int32_t* d_instances, int64_t count,
                       int instances_per_block, int grid_blocks, cudaStream_t s);
void launch_phase_begin(const BatchDev& B, double dt_exchange, cudaStream_t s);
void launch_exchange(const BatchDev& B, int64_t max_n, cudaStream_t s, int64_t* launches);
int exchange_launches(bool has_edges);
void launch_exchange_batched(const BatchDev& B, int precision, int64_t n_max, bool any_edge_dampings,
                             cudaStream_t s, int64_t* launches,
                             cudaEvent_t* ev = nullptr);
int exchange_batched_launches(const BatchDev& B, int precision, bool any_edge_dampings);
// Fills the per-edge traveler offsets, the in-edges' (source, edge) pairs and
// every node's first in-edge from a higher source, from B.graphs, B.edge_graph,
// B.edge_src, B.in_ptr and B.in_edges (already on the device).
cudaError_t launch_edge_indices(const BatchDev& B, int64_t* trav_off, int2* in_se, int64_t* in_mid,
                                cudaStream_t s);
// Marks the graphs of a mixed batch whose FP32 return and departure run from
// shared memory (static coefficients, edges, enough (node, group) items, tables
// within the device's shared memory per block) and lists their chunks, one CTA
// each, largest graphs first; gives the dynamic shared memory of the return and
// departure launches and whether the return copies the rates. err: the first
// failed CUDA call.
struct XsPlan {
    std::vector<int2> work;
    int32_t smem_ret = 0, smem_dep = 0, aux = 0;
    cudaError_t err = cudaSuccess;
};
// mode 1: only when the chunks give at least two CTAs per SM; 2: always.
XsPlan plan_staged_exchange(std::vector<DevGraph>& dg, int mob_union, int device, int mode);

// Device and stream of a context (for entry points defined outside capi.cu).
int context_device_stream(const mgpu_context* ctx, int* device, cudaStream_t* stream);
void launch_exchange_range(const BatchDev& B, int g0, int ng, int64_t n0, int64_t nn, int64_t e0, int64_t ne,
                           int64_t n_max, cudaStream_t s, int64_t* launches);
void launch_phase_end(const BatchDev& B, cudaStream_t s);

} // namespace mgpu
