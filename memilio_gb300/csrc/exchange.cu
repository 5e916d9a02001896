// exchange.cu — the half-day mobility exchange of MobilityEdge::apply_mobility
// (memilio/mobility/metapopulation_mobility_instant.h:544-623) for every graph
// of a batch, and the interval bookkeeping of GraphSimulation::advance
// (memilio/mobility/graph_simulation.h:101-120).
//
// Node updates are per-(node, compartment) threads that walk the node's
// incident edges in the order the reference's serial edge loop visits them
// (edges sorted by (src, dst), graph.h:231-241): in-edges from smaller
// sources, then the node's own out-edges, then in-edges from larger
// sources. Each compartment therefore receives the same FP64 additions in
// the same order as in the reference, without atomics.
//
// The underflow fix of a return (:576-596) depends on the destination's
// state at the moment the serial loop reaches the edge. A per-node bound
// (state minus all positive incoming returns plus all negative outgoing
// returns) proves that no partial state can go negative; a graph for
// which the bound fails anywhere is redone by an exact sequential pass.
#include "mgpu_internal.cuh"

#include <cstdio>

namespace mgpu
{
namespace
{

__device__ __forceinline__ bool departing(const GraphRt& rt)
{
    return rt.active && rt.do_depart;
}
__device__ __forceinline__ bool returning(const GraphRt& rt)
{
    return rt.active && rt.do_return;
}

// GraphSimulation::advance: length of the next interval (dt clipped at tmax).
__global__ void k_phase_begin(BatchDev B, double dt_exchange)
{
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= B.num_graphs) {
        return;
    }
    if (gi == 0 && B.order_cnt) {
        for (int k = 0; k < 2 * (MGPU_MAX_GROUPS + 1); ++k) {
            B.order_cnt[k] = 0;
        }
    }
    if (gi == 0 && B.fix_meta) {
        B.fix_meta[0] = 0;
        B.fix_meta[1] = 0;
    }
    if (gi == 0 && B.scan_count) {
        B.scan_count[0] = B.scan_count[1] = B.scan_count[2] = 0; // the exact path's work lists
    }
    GraphRt& rt = B.rt[gi];
    rt.fallback = 0;
    if (rt.t < rt.tmax) {
        double dt = dt_exchange;
        if (rt.t + dt > rt.tmax) {
            dt = rt.tmax - rt.t;
        }
        rt.active    = 1;
        rt.dt        = dt;
        rt.t_next    = rt.t + dt;
        rt.do_return = rt.has_pending && (rt.t_ret <= rt.t_next);
        rt.do_depart = !rt.return_mobile;
    }
    else {
        rt.active    = 0;
        rt.do_return = 0;
        rt.do_depart = 0;
    }
}

__global__ void k_phase_end(BatchDev B)
{
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= B.num_graphs) {
        return;
    }
    GraphRt& rt = B.rt[gi];
    if (!rt.active) {
        return;
    }
    rt.t = rt.t_next;
    if (rt.do_return) {
        rt.has_pending = 0;
    }
    if (rt.do_depart) {
        rt.has_pending = 1;
        rt.t_dep       = rt.t_next;
        rt.t_ret       = rt.t_next + rt.dt;
        rt.snap_slot ^= 1;
    }
    rt.return_mobile = !rt.return_mobile;
    rt.active        = 0;
}

// Pre-exchange snapshot (SimulationNode::m_last_state) of departing graphs.
__global__ void k_snapshot(BatchDev B, int n_max, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn * n_max) {
        return;
    }
    const int64_t node = n0 + tid / n_max;
    const int j        = (int)(tid % n_max);
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    if (j >= g.n || !departing(B.rt[gi])) {
        return;
    }
    const int64_t o = g.state_off + (node - g.node0) * g.n + j;
    B.ypre[o]       = B.state[o];
}

// Departure travelers of one edge: m = y_from o c(t) o factors (:605-621,
// get_mobility_factors model.h:687-715, test_commuters model.h:717-742).
__global__ void k_depart_edges(BatchDev B, int64_t e0, int64_t ne)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne) {
        return;
    }
    const int64_t e = e0 + tid;
    const int gi      = B.edge_graph[e];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!departing(rt)) {
        return;
    }
    const int64_t le = e - g.edge0;
    const double t   = rt.t_next;
    bool any         = false;
    if (g.Ke == 0) {
        any = B.edge_static_any[e];
    }
    else {
        for (int j = 0; j < g.n && !any; ++j) {
            any = edge_coeff_at(B, g, le, j, t) > 0.0;
        }
    }
    B.edge_pending[e] = any ? 1 : 0;
    if (!any) {
        return;
    }
    const int64_t u     = B.edge_src[e];
    const int64_t lu    = u - g.node0;
    const NodeModel nm  = node_model(B, g, lu);
    const CVec y{B.ypre + g.state_off + lu * g.n, 1};
    double* m           = B.trav + B.trav_off[e];
    double nondetection = 1.0;
    if (t >= nm.scalar(MGPU_P_START_COMMUTER_DETECTION) && t < nm.scalar(MGPU_P_END_COMMUTER_DETECTION)) {
        nondetection = nm.scalar(MGPU_P_COMMUTER_NONDETECTION);
    }
    for (int gr = 0; gr < g.G; ++gr) {
        const double risk = mobility_isy_factor(nm, y, gr);
        for (int c = 0; c < kC; ++c) {
            const int j   = gr * kC + c;
            double factor = (c == MGPU_ISY) ? risk : 1.0;
            double v      = y[j] * edge_coeff_at(B, g, le, j, t) * factor;
            if (c == MGPU_INS || c == MGPU_ISY) {
                v *= nondetection;
            }
            m[j] = v;
        }
    }
}

// Node side of the departure: y_v += sum(in) - sum(out) in serial edge order; v0 := y_v.
__global__ void k_depart_nodes(BatchDev B, int n_max, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn * n_max) {
        return;
    }
    const int64_t node = n0 + tid / n_max;
    const int j        = (int)(tid % n_max);
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (j >= g.n || !departing(rt)) {
        return;
    }
    const int64_t lv = node - g.node0;
    const int64_t o  = g.state_off + lv * g.n + j;
    double val       = B.state[o];
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_src[e] > node) {
            break;
        }
        if (B.edge_pending[e]) {
            val += B.trav[B.trav_off[e] + j];
        }
    }
    // own out-edges: test_commuters moves detected commuters to the confirmed
    // compartments of the source first, then the travelers leave
    const NodeModel nm = node_model(B, g, lv);
    const double t     = rt.t_next;
    const bool detect =
        t >= nm.scalar(MGPU_P_START_COMMUTER_DETECTION) && t < nm.scalar(MGPU_P_END_COMMUTER_DETECTION);
    const double nd = detect ? nm.scalar(MGPU_P_COMMUTER_NONDETECTION) : 1.0;
    const int c     = j % kC;
    const int gr    = j / kC;
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!B.edge_pending[e]) {
            continue;
        }
        if (detect && (c == MGPU_INS || c == MGPU_INSC || c == MGPU_ISY || c == MGPU_ISYC)) {
            const CVec y{B.ypre + g.state_off + lv * g.n, 1};
            const int64_t le = e - g.edge0;
            const int ji     = gr * kC + MGPU_INS;
            const int jy     = gr * kC + MGPU_ISY;
            const double mi  = y[ji] * edge_coeff_at(B, g, le, ji, t) * 1.0;
            const double my  = y[jy] * edge_coeff_at(B, g, le, jy, t) * mobility_isy_factor(nm, y, gr);
            if (c == MGPU_INS) {
                val -= mi * (1 - nd);
            }
            else if (c == MGPU_INSC) {
                val += mi * (1 - nd);
            }
            else if (c == MGPU_ISY) {
                val -= my * (1 - nd);
            }
            else {
                val += my * (1 - nd);
            }
        }
        val -= B.trav[B.trav_off[e] + j];
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_pending[e]) {
            val += B.trav[B.trav_off[e] + j];
        }
    }
    B.state[o] = val;
    B.v0[o]    = val;
}

// Returning travelers: one explicit Euler step of the destination model at the
// departure time with the destination's post-departure state as population
// (calculate_mobility_returns :460-471, EulerIntegratorCore::step math/euler.h:54-62).
__global__ void k_return_edges(BatchDev B, int64_t e0, int64_t ne)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne) {
        return;
    }
    const int64_t e = e0 + tid;
    const int gi      = B.edge_graph[e];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!returning(rt) || !B.edge_pending[e]) {
        return;
    }
    const int64_t lv   = B.edge_dst[e] - g.node0;
    const NodeModel nm = node_model(B, g, lv);
    double* m          = B.trav + B.trav_off[e];
    double dydt[MGPU_MAX_GROUPS * kC];
    secir_rhs(nm, CVec{B.v0 + g.state_off + lv * g.n, 1}, CVec{m, 1}, rt.t_dep, SVec{dydt, 1});
    for (int j = 0; j < g.n; ++j) {
        m[j] = m[j] + rt.dt * dydt[j];
    }
}

// Node side of the returns into ynew, plus the no-underflow bound.
__global__ void k_return_nodes(BatchDev B, int n_max, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn * n_max) {
        return;
    }
    const int64_t node = n0 + tid / n_max;
    const int j        = (int)(tid % n_max);
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    GraphRt& rt       = B.rt[gi];
    if (j >= g.n || !returning(rt)) {
        return;
    }
    const int64_t o  = g.state_off + (node - g.node0) * g.n + j;
    const double y0  = B.state[o];
    double val       = y0;
    double bound     = y0;
    double mag       = fabs(y0);
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_src[e] > node) {
            break;
        }
        if (B.edge_pending[e]) {
            const double m = B.trav[B.trav_off[e] + j];
            val -= m;
            bound -= fmax(m, 0.0);
            mag += fabs(m);
        }
    }
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (B.edge_pending[e]) {
            const double m = B.trav[B.trav_off[e] + j];
            val += m;
            bound += fmin(m, 0.0);
            mag += fabs(m);
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_pending[e]) {
            const double m = B.trav[B.trav_off[e] + j];
            val -= m;
            bound -= fmax(m, 0.0);
            mag += fabs(m);
        }
    }
    B.ynew[o] = val;
    // the serial loop fixes strictly negative remainders only; the margin covers
    // the different rounding of this bound against the serial partial sums
    if (bound < 1e-12 * mag) {
#ifdef MGPU_DEBUG_BOUND
        printf("bound: graph %d node %lld j %d y %.17g bound %.17g mag %.17g t %g\n", gi,
               (long long)(node - g.node0), j, y0, bound, mag, rt.t_next);
#endif
        B.node_flag[node] = 1;
    }
}

// Exact serial return semantics restricted to one node (one warp, lanes over
// compartments): the node's incident edges in serial order, the underflow
// fix of each in-edge against the node's running state, the node's own
// returning travelers (fixed at their destinations when needed) added at
// their place in the order. An in-edge whose fixed travelers change marks its
// source for a rescan (the source's state includes them). Pass 0 scans the
// flagged nodes, later passes the nodes marked in the previous pass.
__global__ void k_return_scan(BatchDev B, int64_t n0, int64_t nn, int pass)
{
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane  = threadIdx.x & 31;
    if (w >= nn) {
        return;
    }
    const int64_t node = n0 + w;
    const int gi       = B.node_graph[node];
    const DevGraph& g  = B.graphs[gi];
    const GraphRt& rt  = B.rt[gi];
    if (!returning(rt)) {
        return;
    }
    uint8_t* dirty_in  = B.node_dirty + (pass & 1) * B.num_nodes;
    uint8_t* dirty_out = B.node_dirty + ((pass + 1) & 1) * B.num_nodes;
    const bool todo    = pass == 0 ? B.node_flag[node] != 0 : dirty_in[node] != 0;
    if (!todo) {
        return;
    }
    if (pass > 0 && lane == 0) {
        dirty_in[node] = 0;
    }
    __shared__ double sm_m[4][MGPU_MAX_GROUPS * kC];
    __shared__ double sm_r[4][MGPU_MAX_GROUPS * kC];
    double* m   = sm_m[(threadIdx.x >> 5) & 3];
    double* rem = sm_r[(threadIdx.x >> 5) & 3];
    const int n = g.n;
    double y[3];
    const double* ys = B.state + g.state_off + (node - g.node0) * n;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = lane + 32 * q;
        y[q]        = j < n ? ys[j] : 0.0;
    }
    auto in_edge = [&](int64_t e) {
        if (!B.edge_pending[e]) {
            return;
        }
        const double* me = B.trav + B.trav_off[e];
        bool neg         = false;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int j = lane + 32 * q;
            if (j < n) {
                m[j]   = me[j];
                rem[j] = y[q] - m[j];
                neg    = neg || (rem[j] < 0);
            }
        }
        neg = __any_sync(0xffffffffu, neg);
        __syncwarp();
        if (neg) {
            if (lane == 0) {
                int fixes = 0;
                for (int j = 0; j < n; ++j) {
                    if (rem[j] < 0) {
                        const int group = j / kC;
                        int max_index   = 0;
                        for (int c = 1; c < kC; ++c) {
                            if (rem[group * kC + c] > rem[group * kC + max_index]) {
                                max_index = c;
                            }
                        }
                        max_index += group * kC;
                        m[max_index] -= rem[j];
                        m[j] += rem[j];
                        ++fixes;
                    }
                }
                rem[0] = (double)fixes;
            }
            __syncwarp();
            const int fixes = (int)rem[0];
            double* mf      = B.mfix + B.trav_off[e];
            bool changed    = B.edge_fixed[e] == 0;
            for (int q = 0; q < 3; ++q) {
                const int j = lane + 32 * q;
                if (j < n) {
                    changed = changed || (__ldcg(mf + j) != m[j]);
                    __stcg(mf + j, m[j]);
                }
            }
            changed = __any_sync(0xffffffffu, changed);
            __threadfence();
            if (lane == 0) {
                B.edge_fixed[e] = fixes;
                if (changed) {
                    dirty_out[B.edge_src[e]] = 1;
                }
            }
        }
        else if (B.edge_fixed[e] != 0) {
            if (lane == 0) {
                B.edge_fixed[e]          = 0;
                dirty_out[B.edge_src[e]] = 1;
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int j = lane + 32 * q;
            if (j < n) {
                y[q] -= m[j];
            }
        }
        __syncwarp();
    };
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_src[e] > node) {
            break;
        }
        in_edge(e);
    }
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!B.edge_pending[e]) {
            continue;
        }
        // fixed travelers are published by another warp (possibly in this pass):
        // read the flag and the values past L1
        const bool fixed  = ((volatile int32_t*)B.edge_fixed)[e] != 0;
        const double* src = fixed ? B.mfix + B.trav_off[e] : B.trav + B.trav_off[e];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int j = lane + 32 * q;
            if (j < n) {
                y[q] += __ldcg(src + j);
            }
        }
    }
    for (; k < ie; ++k) {
        in_edge(B.in_edges[k]);
    }
    double* yn = B.ynew + g.state_off + (node - g.node0) * n;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = lane + 32 * q;
        if (j < n) {
            yn[j] = y[q];
        }
    }
}

// Graphs with a node still marked after the last scan pass take the exact
// sequential path; flags are cleared.
__global__ void k_return_scan_done(BatchDev B, int64_t n0, int64_t nn, int pass_end)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn) {
        return;
    }
    const int64_t node = n0 + tid;
    const int gi       = B.node_graph[node];
    GraphRt& rt        = B.rt[gi];
    uint8_t* dirty     = B.node_dirty + (pass_end & 1) * B.num_nodes;
    if (returning(rt) && dirty[node]) {
        atomicOr(&rt.fallback, 1);
    }
    dirty[node]                                        = 0;
    B.node_dirty[((pass_end + 1) & 1) * B.num_nodes + node] = 0;
    B.node_flag[node]                                  = 0;
}

// Underflow-fix counts of the parallel path; clears the per-edge fix state.
__global__ void k_return_cleanup(BatchDev B, int64_t e0, int64_t ne)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne) {
        return;
    }
    const int64_t e = e0 + tid;
    const int f     = B.edge_fixed[e];
    if (f == 0) {
        return;
    }
    const GraphRt& rt = B.rt[B.edge_graph[e]];
    if (!rt.fallback) {
        atomicAdd(&B.counters[CNT_UNDERFLOW], (unsigned long long)f);
    }
    B.edge_fixed[e] = 0;
}

__global__ void k_return_commit(BatchDev B, int n_max, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn * n_max) {
        return;
    }
    const int64_t node = n0 + tid / n_max;
    const int j        = (int)(tid % n_max);
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (j >= g.n || !returning(rt) || rt.fallback) {
        return;
    }
    const int64_t o = g.state_off + (node - g.node0) * g.n + j;
    B.state[o]      = B.ynew[o];
}

// Exact serial return loop of one graph (one warp per graph), including the
// underflow fix: negative remainders are taken from the largest compartment
// of the same age group (:576-596).
__global__ void k_return_sequential(BatchDev B, int g0, int ng)
{
    const int gi = g0 + blockIdx.x;
    if (blockIdx.x >= ng) {
        return;
    }
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!returning(rt) || !rt.fallback) {
        return;
    }
    __shared__ double m[MGPU_MAX_GROUPS * kC];
    __shared__ double rem[MGPU_MAX_GROUPS * kC];
    const int lane = threadIdx.x;
    const int n    = g.n;
    int64_t fixes  = 0;
    for (int64_t e = g.edge0; e < g.edge0 + g.E; ++e) {
        if (!B.edge_pending[e]) {
            continue;
        }
        const int64_t u  = B.edge_src[e] - g.node0;
        const int64_t v  = B.edge_dst[e] - g.node0;
        double* ym       = B.trav + B.trav_off[e];
        double* yu       = B.state + g.state_off + u * n;
        double* yv       = B.state + g.state_off + v * n;
        bool neg         = false;
        for (int j = lane; j < n; j += 32) {
            m[j]   = ym[j];
            rem[j] = yv[j] - m[j];
            neg    = neg || (rem[j] < 0);
        }
        neg = __any_sync(0xffffffffu, neg);
        __syncwarp();
        if (neg && lane == 0) {
            for (int j = 0; j < n; ++j) {
                if (rem[j] < 0) {
                    const int group = j / kC;
                    int max_index   = 0;
                    for (int c = 1; c < kC; ++c) {
                        if (rem[group * kC + c] > rem[group * kC + max_index]) {
                            max_index = c;
                        }
                    }
                    max_index += group * kC;
                    m[max_index] -= rem[j];
                    m[j] += rem[j];
                    ++fixes;
                }
            }
        }
        __syncwarp();
        for (int j = lane; j < n; j += 32) {
            ym[j] = m[j];
            yu[j] += m[j];
        }
        __syncwarp();
        for (int j = lane; j < n; j += 32) {
            yv[j] -= m[j];
        }
        __syncwarp();
    }
    if (lane == 0) {
        atomicAdd(&B.counters[CNT_SEQUENTIAL], 1ull);
        if (fixes) {
            atomicAdd(&B.counters[CNT_UNDERFLOW], (unsigned long long)fixes);
        }
    }
}

inline int blocks_for(int64_t n, int threads)
{
    return (int)((n + threads - 1) / threads);
}

// Passes of the per-node exact scan before a graph falls back to the
// sequential pass (each pass resolves one more level of the dependency chain).
constexpr int kScanPasses = 4;

} // namespace

void launch_phase_begin(const BatchDev& B, double dt_exchange, cudaStream_t s)
{
    k_phase_begin<<<blocks_for(B.num_graphs, 128), 128, 0, s>>>(B, dt_exchange);
}

void launch_phase_end(const BatchDev& B, cudaStream_t s)
{
    k_phase_end<<<blocks_for(B.num_graphs, 128), 128, 0, s>>>(B);
}

// Returns first (pending travelers whose return time has come), then departures,
// as in apply_mobility, for graphs [g0, g0+ng) with nodes [n0, n0+nn) and edges
// [e0, e0+ne); launches counted in *launches.
void launch_exchange_range(const BatchDev& B, int g0, int ng, int64_t n0, int64_t nn, int64_t e0, int64_t ne,
                           int64_t n_max, cudaStream_t s, int64_t* launches)
{
    const int T        = 256;
    const int64_t nthr = nn * n_max;
    if (nn == 0) {
        return;
    }
    k_snapshot<<<blocks_for(nthr, T), T, 0, s>>>(B, (int)n_max, n0, nn);
    if (ne > 0) {
        k_return_edges<<<blocks_for(ne, 128), 128, 0, s>>>(B, e0, ne);
        k_return_nodes<<<blocks_for(nthr, T), T, 0, s>>>(B, (int)n_max, n0, nn);
        for (int pass = 0; pass < kScanPasses; ++pass) {
            k_return_scan<<<blocks_for(nn * 32, 128), 128, 0, s>>>(B, n0, nn, pass);
        }
        k_return_scan_done<<<blocks_for(nn, T), T, 0, s>>>(B, n0, nn, kScanPasses);
        k_return_commit<<<blocks_for(nthr, T), T, 0, s>>>(B, (int)n_max, n0, nn);
        k_return_sequential<<<ng, 32, 0, s>>>(B, g0, ng);
        k_return_cleanup<<<blocks_for(ne, T), T, 0, s>>>(B, e0, ne);
        k_depart_edges<<<blocks_for(ne, 128), 128, 0, s>>>(B, e0, ne);
        k_depart_nodes<<<blocks_for(nthr, T), T, 0, s>>>(B, (int)n_max, n0, nn);
        *launches += 9 + kScanPasses;
    }
    else {
        *launches += 1;
    }
}

int exchange_launches(bool has_edges)
{
    return has_edges ? 9 + kScanPasses : 1;
}

void launch_exchange(const BatchDev& B, int64_t n_max, cudaStream_t s, int64_t* launches)
{
    launch_exchange_range(B, 0, B.num_graphs, 0, B.num_nodes, 0, B.num_edges, n_max, s, launches);
}

} // namespace mgpu
