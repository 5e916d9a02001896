// exchange_batched.cu — the mobility exchange of the batched solvers.
//
// Same semantics as exchange.cu (MobilityEdge::apply_mobility,
// memilio/mobility/metapopulation_mobility_instant.h:544-623), laid out for
// GB300 instead of mirroring the reference's per-edge traveler vectors:
//
//  * No traveler vectors in HBM. A departure keeps a per-node snapshot of the
//    pre-exchange state (SimulationNode::m_last_state) and the ISy mobility
//    factor; the travelers of an edge, y_src o c_e o f_src, are recomputed
//    wherever they are needed - at both endpoints of the departure and of the
//    return - from the snapshot and the edge coefficients. Coefficient arrays
//    shared by the graphs of an ensemble are uploaded once, so they stay in L2.
//  * The return's explicit Euler step (calculate_mobility_returns, :460-471)
//    uses the destination's force of infection and flow rates at the departure
//    time, computed once per destination node (not once per edge).
//  * Node updates are (node, age group) threads walking the node's incident
//    edges in serial order, so no atomics and a deterministic result.
//  * Graphs whose snapshot records fit in shared memory run those threads in
//    one CTA per chunk of the graph, reading every edge's source record from a
//    copy in shared memory (k_xs_*); the others gather them from L2 (k_xf_*).
//    Both share the per-item code and give bitwise identical results.
//
// Precision (template R): R = double reproduces the FP64 arithmetic of the
// reference (up to the association of the force-of-infection sum). R = float
// computes travelers and Euler increments in FP32 with correctly rounded
// intrinsics only (no contraction), so both endpoints of an edge obtain the
// bit-identical travelers; the destination forms its in-edges' Euler
// increments from their sum (one rounding instead of one per edge). The node
// states accumulate them in float-float (TwoSum) pairs, which conserves every
// node's and the whole population to float-float rounding (an Euler increment
// moves an amount between two compartments of one node; its FP32 rounding only
// shifts the split between compartments).
//
// Underflow fixes: a conservative per-node bound flags the nodes whose serial
// return order might meet a negative remainder; those run the exact
// (node, age group) scan of exchange.cu semantics (k_xg_scan in FP64, k_xf_scan
// in float-float for the mixed solver, which follows the serial order with
// prefix sums over a warp's lanes and stops only at the edges to fix), then the
// per-graph sequential pass handles what the scan passes leave unresolved.
#include "mgpu_internal.cuh"

#include <algorithm>
#include <type_traits>
#include <utility>

namespace mgpu
{
namespace
{

__device__ __forceinline__ bool xb_departing(const GraphRt& rt)
{
    return rt.active && rt.do_depart;
}
__device__ __forceinline__ bool xb_returning(const GraphRt& rt)
{
    return rt.active && rt.do_return;
}

// did edge e carry travelers at the pending departure?
__device__ __forceinline__ bool edge_departed(const BatchDev& B, const DevGraph& g, int64_t e)
{
    return g.Ke == 0 ? B.edge_static_any[e] != 0 : B.edge_pending[e] != 0;
}

// record that edge e got a fix count in this return (for the cleanup pass)
__device__ __forceinline__ void fix_edge_push(const BatchDev& B, int64_t e)
{
    const int32_t pos = atomicAdd(B.fix_meta, 1);
    if (pos < B.fix_cap) {
        B.fix_edges[pos] = (int32_t)e;
    }
    else {
        B.fix_meta[1] = 1;
    }
}

// append a (node, age group) item, node * MAX_GROUPS + group, to exact-scan
// work list `list` once
__device__ __forceinline__ void list_push(const BatchDev& B, int list, int64_t item)
{
    const int64_t NG = B.num_nodes * MGPU_MAX_GROUPS;
    if (atomicExch(&B.scan_mark[list * NG + item], 1) == 0) {
        const int idx               = atomicAdd(&B.scan_count[list], 1);
        B.scan_list[list * NG + idx] = (int32_t)item;
    }
}

// Append item to list 0 when `want`: every (node, group) thread of a return
// pass appends only its own item, so no mark is needed, and the converged
// threads of a warp reserve their slots with one atomic.
__device__ __forceinline__ void list0_push(const BatchDev& B, int64_t item, bool want)
{
    const unsigned active = __activemask();
    const unsigned m      = __ballot_sync(active, want);
    if (m == 0) {
        return;
    }
    const int lane   = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base         = 0;
    if (lane == leader) {
        base = atomicAdd(&B.scan_count[0], __popc(m));
    }
    base = __shfl_sync(active, base, leader);
    if (want) {
        B.scan_list[base + __popc(m & ((1u << lane) - 1u))] = (int32_t)item;
    }
}

template <class R>
__device__ __forceinline__ R rmul(R a, R b)
{
    if constexpr (std::is_same<R, float>::value) {
        return __fmul_rn(a, b);
    }
    else {
        return __dmul_rn(a, b);
    }
}
template <class R>
__device__ __forceinline__ R radd(R a, R b)
{
    if constexpr (std::is_same<R, float>::value) {
        return __fadd_rn(a, b);
    }
    else {
        return __dadd_rn(a, b);
    }
}
template <class R>
__device__ __forceinline__ R rsub(R a, R b)
{
    if constexpr (std::is_same<R, float>::value) {
        return __fsub_rn(a, b);
    }
    else {
        return __dsub_rn(a, b);
    }
}

// FP64 value or float-float pair
template <class R>
struct Acc;
template <>
struct Acc<double> {
    double v;
    __device__ void init(double x)
    {
        v = x;
    }
    __device__ void add(double t)
    {
        v = v + t;
    }
    __device__ double get() const
    {
        return v;
    }
};
template <>
struct Acc<float> {
    float hi, lo;
    __device__ void init(double x)
    {
        hi = (float)x;
        lo = (float)(x - (double)hi);
    }
    __device__ void add(float t)
    {
        const float s  = __fadd_rn(hi, t);
        const float bb = __fsub_rn(s, hi);
        const float e  = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(t, bb));
        hi             = s;
        lo             = __fadd_rn(lo, e);
    }
    __device__ double get() const
    {
        return (double)hi + (double)lo;
    }
    __device__ void init_pair(float h, float l)
    {
        hi = h;
        lo = l;
    }
    // renormalised pair (|lo| <= ulp(hi)/2)
    __device__ void store(float* h, float* l) const
    {
        const float s = __fadd_rn(hi, lo);
        *l            = __fsub_rn(lo, __fsub_rn(s, hi));
        *h            = s;
    }
};

// Coefficient of edge e (local le) for compartment j at time t, in R.
template <class R>
__device__ __forceinline__ R xb_coeff(const BatchDev& B, const DevGraph& g, int64_t le, int j, double t)
{
    if (g.Ke == 0) {
        if constexpr (std::is_same<R, float>::value) {
            return B.ecoef_r[rec_elem(g.ecoef_f_off / kC + le * g.G, g.G, j / kC, rec_pos(j % kC))];
        }
        else {
            return B.ecoef[g.ecoef_off + le * 2 * g.n + j] -
                   0.0 * (B.ecoef[g.ecoef_off + le * 2 * g.n + j] - B.ecoef[g.ecoef_off + le * 2 * g.n + g.n + j]);
        }
    }
    return (R)edge_coeff_at(B, g, le, j, t);
}


template <class R>
__device__ __forceinline__ R* aux_ptr(const BatchDev& B)
{
    return reinterpret_cast<R*>(B.aux);
}

// Travelers of group `gr` on edge e at departure (before the nondetection scaling
// when `orig`): m = y_src o c_e(t) o factors (get_mobility_factors, model.h:687-715;
// test_commuters, model.h:717-742).
template <class R, bool orig = false>
__device__ __forceinline__ void depart_travelers(const BatchDev& B, const DevGraph& g, int64_t e, int gr, int slot,
                                                 double t, R (&m)[kC])
{
    const int64_t u  = B.edge_src[e];
    const int64_t lu = u - g.node0;
    const int64_t le = e - g.edge0;
    R y[kC], risk, nd;
    if constexpr (std::is_same<R, float>::value) {
        // the source's snapshot record (mixed)
        const float* rec = B.gsnap + (int64_t)slot * (B.state_total / kC) * kRec;
        const int64_t r0 = (g.state_off + lu * g.n) / kC;
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            y[c] = rec[rec_elem(r0, g.G, gr, rec_pos(c))];
        }
        risk = rec[rec_elem(r0, g.G, gr, REC_RISK)];
        nd   = rec[rec_elem(r0, g.G, gr, REC_ND)];
    }
    else {
        const R* ys  = B.ysnap + (int64_t)slot * B.state_total + g.state_off + lu * g.n + gr * kC;
        const R* fac = reinterpret_cast<const R*>(B.risk) + (((int64_t)slot * B.num_nodes + u) * MGPU_MAX_GROUPS + gr) * 2;
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            y[c] = ys[c];
        }
        risk = fac[0];
        nd   = fac[1];
    }
    if (orig) {
        nd = (R)1;
    }
    (void)t;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        const R cf = xb_coeff<R>(B, g, le, gr * kC + c, t);
        R v        = rmul(rmul(y[c], cf), c == MGPU_ISY ? risk : (R)1);
        if (!orig && (c == MGPU_INS || c == MGPU_ISY)) {
            v = rmul(v, nd);
        }
        m[c] = v;
    }
}

// Returning travelers of group `gr` on edge e in flow form: the departed
// travelers m and the Euler flow increments phi_k = dt f_k of the destination's
// model at the departure time (calculate_mobility_returns, :460-471); the
// returning compartment c is m_c plus the increments of the flows into c minus
// those out of c.
template <class R>
__device__ __forceinline__ void return_flows(const BatchDev& B, const DevGraph& g, const GraphRt& rt, int64_t e,
                                             int gr, R (&m)[kC], R (&phi)[kF])
{
    depart_travelers<R>(B, g, e, gr, rt.snap_slot, rt.t_dep, m);
    const R* a = aux_ptr<R>(B) + (B.edge_dst[e] * MGPU_MAX_GROUPS + gr) * kAux;
    const R dt = (R)rt.dt;
    const R s[kF] = {m[MGPU_S], m[MGPU_E], m[MGPU_INS], m[MGPU_INS], m[MGPU_INSC], m[MGPU_INSC], m[MGPU_ISY],
                     m[MGPU_ISY], m[MGPU_ISYC], m[MGPU_ISYC], m[MGPU_ISEV], m[MGPU_ISEV], m[MGPU_ISEV],
                     m[MGPU_ICRI], m[MGPU_ICRI]};
    const int ai[kF] = {0, 1, 2, 3, 2, 3, 4, 5, 4, 5, 6, 7, 8, 9, 10};
#pragma unroll
    for (int k = 0; k < kF; ++k) {
        phi[k] = rmul(dt, rmul(a[ai[k]], s[k]));
    }
}

__device__ __forceinline__ void return_travelers_ref(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                                     int64_t e, int gr, double (&m)[kC]);

// Returning travelers of group `gr` on edge e as FP64 values: one explicit
// Euler step of the destination's model at the departure time. The FP32 path
// sums the departed travelers and the flow increments in FP64, which is exact
// for these magnitudes, so it equals the float-float sums of k_xb_return.
template <class R>
__device__ __forceinline__ void return_travelers(const BatchDev& B, const DevGraph& g, const GraphRt& rt, int64_t e,
                                                 int gr, double (&out)[kC])
{
    if constexpr (std::is_same<R, float>::value) {
        float mf[kC], phi[kF];
        return_flows<float>(B, g, rt, e, gr, mf, phi);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            out[c] = (double)mf[c];
        }
#pragma unroll
        for (int k = 0; k < kF; ++k) {
            out[kFlowSrcI(k)] -= (double)phi[k];
            out[kFlowDstI(k)] += (double)phi[k];
        }
        return;
    }
    else {
        return_travelers_ref(B, g, rt, e, gr, out);
    }
}

// FP64 reference form of the Euler step (m + dt * dydt per compartment).
__device__ __forceinline__ void return_travelers_ref(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                                     int64_t e, int gr, double (&m)[kC])
{
    using R = double;
    depart_travelers<R>(B, g, e, gr, rt.snap_slot, rt.t_dep, m);
    const R* a = aux_ptr<R>(B) + (B.edge_dst[e] * MGPU_MAX_GROUPS + gr) * kAux;
    R f[kF];
    f[0]  = rmul(a[0], m[MGPU_S]);
    f[1]  = rmul(a[1], m[MGPU_E]);
    f[2]  = rmul(a[2], m[MGPU_INS]);
    f[3]  = rmul(a[3], m[MGPU_INS]);
    f[4]  = rmul(a[2], m[MGPU_INSC]);
    f[5]  = rmul(a[3], m[MGPU_INSC]);
    f[6]  = rmul(a[4], m[MGPU_ISY]);
    f[7]  = rmul(a[5], m[MGPU_ISY]);
    f[8]  = rmul(a[4], m[MGPU_ISYC]);
    f[9]  = rmul(a[5], m[MGPU_ISYC]);
    f[10] = rmul(a[6], m[MGPU_ISEV]);
    f[11] = rmul(a[7], m[MGPU_ISEV]);
    f[12] = rmul(a[8], m[MGPU_ISEV]);
    f[13] = rmul(a[9], m[MGPU_ICRI]);
    f[14] = rmul(a[10], m[MGPU_ICRI]);
    R d[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        d[c] = (R)0;
    }
#pragma unroll
    for (int k = 0; k < kF; ++k) {
        d[kFlowSrcI(k)] = rsub(d[kFlowSrcI(k)], f[k]);
        d[kFlowDstI(k)] = radd(d[kFlowDstI(k)], f[k]);
    }
    const R dt = (R)rt.dt;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        m[c] = radd(m[c], rmul(dt, d[c]));
    }
}

// MobilityEdge::add_mobility_result_time_point (metapopulation_mobility_instant.h:423-447):
// the sums of the travelers m [10 G] over each index set, in the set's order, then
// over all compartments, as a time point t of local edge le.
__device__ void record_edge_stats(const EdgeStatsDev& S, int64_t le, int n, double t, const double* m)
{
    const int32_t k = S.count[le];
    S.count[le]     = k + 1;
    if (k >= S.capacity) {
        return;
    }
    const int64_t row           = le * S.capacity + k;
    S.times[row]                = t;
    double* v                   = S.values + row * (S.num_sets + 1);
    for (int i = 0; i < S.num_sets; ++i) {
        double sum = 0.0;
        for (int q = S.set_ptr[i]; q < S.set_ptr[i + 1]; ++q) {
            sum += m[S.set_idx[q]];
        }
        v[i] = sum;
    }
    double total = 0.0;
    for (int j = 0; j < n; ++j) {
        total += m[j];
    }
    v[S.num_sets] = total;
}

// Row i of the contact matrix at time t (contact_matrix_at, one row), padded
// to MAX_GROUPS entries.
__device__ __forceinline__ void contact_row(const NodeModel& nm, int i, double t, double (&Crow)[MGPU_MAX_GROUPS])
{
    const int G = nm.G;
#pragma unroll
    for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
        Crow[q] = 0.0;
    }
    const long GG = (long)G * G;
    for (int m = 0; m < nm.M; ++m) {
        const double* Bm = nm.cm + m * 2 * GG + (long)i * G;
        const double* Lm = Bm + GG;
        if (nm.K) {
            const double* T  = nm.dtimes + m * nm.K;
            const int ub     = damping_upper_bound(T, nm.K, t);
            const Ramp r     = ramp_at(t, T[ub] - 1.0, T[ub]);
            const double* Dl = nm.dvals + ((long)m * nm.K + ub - 1) * GG + (long)i * G;
            const double* Dr = Dl + GG;
#pragma unroll
            for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
                if (q < G) {
                    const double D = ramp_apply(r, Dl[q], Dr[q]);
                    Crow[q]        = Crow[q] + (Bm[q] - D * (Bm[q] - Lm[q]));
                }
            }
        }
        else {
#pragma unroll
            for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
                if (q < G) {
                    Crow[q] = Crow[q] + (Bm[q] - 0.0 * (Bm[q] - Lm[q]));
                }
            }
        }
    }
}

// Per node, one 8-lane segment with a lane per age group: the departure snapshot
// and mobility factors; the force of infection and flow rates at the departure
// time for the return's Euler step. Sums over age groups run in group order
// (shuffles from lanes 0..G-1), as in the serial right-hand side. FP64 batches
// only: the mixed node kernel does this pass itself.
template <class R>
__global__ void k_xb_prep(BatchDev B, int64_t n0, int64_t nn)
{
    static_assert(std::is_same<R, double>::value, "the FP64 node pass");
    constexpr unsigned kFull = 0xffffffffu;
    const int64_t tid        = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t seg        = tid / MGPU_MAX_GROUPS;
    const bool in_range      = seg < nn;
    const int64_t node       = n0 + (in_range ? seg : nn - 1); // every lane takes part in the shuffles
    const int lane           = (int)(threadIdx.x % MGPU_MAX_GROUPS);
    const int gi             = B.node_graph[node];
    const DevGraph& g        = B.graphs[gi];
    const GraphRt& rt        = B.rt[gi];
    const int G              = g.G;
    const bool mine          = in_range && lane < G;
    const int i              = lane < G ? lane : 0; // the lane's age group (clamped for idle lanes)
    const int64_t lv         = node - g.node0;
    const NodeModel nm       = node_model(B, g, lv);
    const int64_t so         = g.state_off + lv * g.n + (int64_t)i * kC;
    const bool ret           = in_range && xb_returning(rt);
    const bool dep           = in_range && xb_departing(rt);
    const double tnt_w       = (1 - nm.gp(MGPU_G_RECOVERED_PER_INS, i)) / nm.gp(MGPU_G_TIME_INS, i);
    const double cap         = nm.scalar(MGPU_P_TNT_CAPACITY);
    if (__any_sync(kFull, ret)) {
        double pop[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            pop[c] = v0_get(B, so + c);
        }
        const double tnt_c = tnt_w * pop[MGPU_INS];
        double tnt = 0.0, icu = 0.0;
#pragma unroll
        for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
            const double a = __shfl_sync(kFull, tnt_c, q, MGPU_MAX_GROUPS);
            const double b = __shfl_sync(kFull, pop[MGPU_ICRI], q, MGPU_MAX_GROUPS);
            if (q < G) {
                tnt += a;
                icu += b;
            }
        }
        const Ramp rrisk    = ramp_at(tnt, cap, cap * nm.scalar(MGPU_P_TNT_MAX_RISK));
        const double season = (1 + nm.scalar(MGPU_P_SEASONALITY) *
                                       sin(kPi * ((nm.scalar(MGPU_P_START_DAY) + rt.t_dep) / 182.5 + 0.5)));
        const double icu_cap = nm.scalar(MGPU_P_ICU_CAPACITY);
        const Ramp ricu      = ramp_at(icu, 0.90 * icu_cap, icu_cap);
        // this lane as source group: 1/N and the infectious pressure
        const double Nj = pop[MGPU_S] + pop[MGPU_E] + pop[MGPU_INS] + pop[MGPU_ISY] + pop[MGPU_ISEV] +
                          pop[MGPU_ICRI] + pop[MGPU_R];
        const double divN  = (Nj < kZeroTol) ? 0.0 : 1.0 / Nj;
        const double risk  = ramp_apply(rrisk, nm.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, i),
                                        nm.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, i));
        const double press = nm.gp(MGPU_G_REL_TRANSMISSION_NS, i) * pop[MGPU_INS] + risk * pop[MGPU_ISY];
        // this lane as target group: its row of the contact matrix at t_dep
        // (contact_matrix_at, one row)
        double Crow[MGPU_MAX_GROUPS];
        contact_row(nm, i, rt.t_dep, Crow);
        const double beta = nm.gp(MGPU_G_TRANSMISSION_PROB, i);
        double lam        = 0.0;
#pragma unroll
        for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
            const double dn = __shfl_sync(kFull, divN, q, MGPU_MAX_GROUPS);
            const double pr = __shfl_sync(kFull, press, q, MGPU_MAX_GROUPS);
            if (q < G) {
                lam += (season * Crow[q]) * dn * beta * pr;
            }
        }
        if (ret && mine) {
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
            R v[kAux];
            v[0]  = (R)lam;
            v[1]  = (R)(1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i));
            v[2]  = (R)((1 - mu) * (1 / tins));
            v[3]  = (R)(mu * (1.0 / tins));
            v[4]  = (R)(sev / tisy);
            v[5]  = (R)((1 - sev) / tisy);
            v[6]  = (R)(crit_adj / tisev);
            v[7]  = (R)((1.0 - cps - dps) / tisev);
            v[8]  = (R)((dps + death_adj) / tisev);
            v[9]  = (R)(dpc / ticri);
            v[10] = (R)((1.0 - dpc) / ticri);
            // can one Euler step of length dt drive a returning compartment negative?
            // (it cannot when dt times every compartment's total outflow rate is <= 1)
            const double out_rate = fmax(fmax(lam, 1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i)),
                                         fmax(fmax((double)v[2] + (double)v[3], (double)v[4] + (double)v[5]),
                                              fmax((double)v[6] + (double)v[7] + (double)v[8],
                                                   (double)v[9] + (double)v[10])));
            v[11] = (R)((rt.dt * out_rate > 1.0) ? 1 : 0);
            R* ai = aux_ptr<R>(B) + (node * MGPU_MAX_GROUPS + i) * kAux;
#pragma unroll
            for (int q = 0; q < kAux; ++q) {
                ai[q] = v[q];
            }
        }
    }
    if (__any_sync(kFull, dep)) {
        const int ws = rt.snap_slot ^ 1;
        double ys[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            ys[c] = B.state[so + c];
            if (dep && mine) {
                B.ysnap[(int64_t)ws * B.state_total + so + c] = ys[c];
            }
        }
        // ISy mobility factor (get_mobility_factors, models/ode_secir/model.h:687-715)
        // and commuter nondetection at this departure
        const double tnt_c = tnt_w * ys[MGPU_INS];
        double tnt         = 0.0;
#pragma unroll
        for (int q = 0; q < MGPU_MAX_GROUPS; ++q) {
            const double a = __shfl_sync(kFull, tnt_c, q, MGPU_MAX_GROUPS);
            if (q < G) {
                tnt += a;
            }
        }
        if (dep && mine) {
            const double t  = rt.t_next;
            const double nd = (t >= nm.scalar(MGPU_P_START_COMMUTER_DETECTION) &&
                               t < nm.scalar(MGPU_P_END_COMMUTER_DETECTION))
                                  ? nm.scalar(MGPU_P_COMMUTER_NONDETECTION)
                                  : 1.0;
            R* fac = reinterpret_cast<R*>(B.risk) + (((int64_t)ws * B.num_nodes + node) * MGPU_MAX_GROUPS + i) * 2;
            fac[0] = (R)smoother_cosine(tnt, cap, cap * nm.scalar(MGPU_P_TNT_MAX_RISK),
                                        nm.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, i),
                                        nm.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, i));
            fac[1] = (R)nd;
        }
    }
}

// Per edge with time-dependent coefficients: does it carry travelers at this departure?
__global__ void k_xb_edge_flags(BatchDev B, int64_t e0, int64_t ne)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= ne) {
        return;
    }
    const int64_t e   = e0 + tid;
    const int gi      = B.edge_graph[e];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!xb_departing(rt) || g.Ke == 0) {
        return;
    }
    bool any = false;
    for (int j = 0; j < g.n && !any; ++j) {
        any = edge_coeff_at(B, g, e - g.edge0, j, rt.t_next) > 0.0;
    }
    B.edge_pending[e] = any ? 1 : 0;
}

// Departure, node side: one thread per (node, age group).
template <class R>
__global__ void k_xb_depart(BatchDev B, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t node = n0 + tid / MGPU_MAX_GROUPS;
    const int gr       = (int)(tid % MGPU_MAX_GROUPS);
    if (tid >= nn * MGPU_MAX_GROUPS) {
        return;
    }
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (gr >= g.G || !xb_departing(rt)) {
        return;
    }
    if (std::is_same<R, float>::value && g.Ke == 0) {
        return; // k_xf_depart
    }
    const int ws     = rt.snap_slot ^ 1;
    const double t   = rt.t_next;
    const int64_t lv = node - g.node0;
    const int64_t so = g.state_off + lv * g.n + gr * kC;
    Acc<R> acc[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].init(state_get(B, so + c));
    }
    R m[kC];
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_src[e] > node) {
            break;
        }
        if (edge_departed(B, g, e)) {
            depart_travelers<R>(B, g, e, gr, ws, t, m);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                acc[c].add(m[c]);
            }
        }
    }
    const double* p = B.params + g.param_off + lv * param_stride(g.G);
    const bool detect = t >= p[MGPU_P_START_COMMUTER_DETECTION] && t < p[MGPU_P_END_COMMUTER_DETECTION];
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!edge_departed(B, g, e)) {
            continue;
        }
        if (detect) {
            // test_commuters: detected commuters move to the confirmed compartments first
            R mo[kC];
            depart_travelers<R, true>(B, g, e, gr, ws, t, mo);
            const R q = (R)(1 - p[MGPU_P_COMMUTER_NONDETECTION]);
            acc[MGPU_INS].add(-rmul(mo[MGPU_INS], q));
            acc[MGPU_INSC].add(rmul(mo[MGPU_INS], q));
            acc[MGPU_ISY].add(-rmul(mo[MGPU_ISY], q));
            acc[MGPU_ISYC].add(rmul(mo[MGPU_ISY], q));
        }
        depart_travelers<R>(B, g, e, gr, ws, t, m);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].add(-m[c]);
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (edge_departed(B, g, e)) {
            depart_travelers<R>(B, g, e, gr, ws, t, m);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                acc[c].add(m[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        const double v = acc[c].get();
        state_set(B, so + c, v);
        if (B.v0_hi) {
            pair_set(B.v0_hi, B.v0_lo, so + c, v);
        }
        else {
            B.v0[so + c] = v;
        }
    }
}

// Return, node side: one thread per (node, age group); writes ynew and flags
// nodes whose serial order might need an underflow fix.
template <class R>
__global__ void k_xb_return(BatchDev B, int64_t n0, int64_t nn)
{
    const int64_t tid  = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t node = n0 + tid / MGPU_MAX_GROUPS;
    const int gr       = (int)(tid % MGPU_MAX_GROUPS);
    if (tid >= nn * MGPU_MAX_GROUPS) {
        return;
    }
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (gr >= g.G || !xb_returning(rt)) {
        return;
    }
    if (std::is_same<R, float>::value && g.Ke == 0) {
        return; // k_xf_return
    }
    const int64_t lv = node - g.node0;
    const int64_t so = g.state_off + lv * g.n + gr * kC;
    Acc<R> acc[kC];
    R bound[kC], mag[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        const double y = state_get(B, so + c);
        acc[c].init(y);
        bound[c] = (R)y;
        mag[c]   = (R)fabs(y);
    }
    // sign -1: travelers leave this node (in-edge), +1: they come home (out-edge)
    auto edge = [&](int64_t e, int sign) {
        if constexpr (std::is_same<R, float>::value) {
            // flow form: m_c and every flow increment enter the float-float sums
            // exactly, so both endpoints of the edge move the same amounts
            float m[kC], phi[kF], tv[kC];
            return_flows<float>(B, g, rt, e, gr, m, phi);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                tv[c] = m[c];
                acc[c].add(sign > 0 ? m[c] : -m[c]);
            }
#pragma unroll
            for (int f = 0; f < kF; ++f) {
                const float p = sign > 0 ? phi[f] : -phi[f];
                acc[kFlowSrcI(f)].add(-p);
                acc[kFlowDstI(f)].add(p);
                tv[kFlowSrcI(f)] -= phi[f];
                tv[kFlowDstI(f)] += phi[f];
            }
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                bound[c] += sign > 0 ? fminf(tv[c], 0.0f) : -fmaxf(tv[c], 0.0f);
                mag[c] += fabsf(tv[c]);
            }
        }
        else {
            double m[kC];
            return_travelers<R>(B, g, rt, e, gr, m);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                acc[c].add(sign > 0 ? m[c] : -m[c]);
                bound[c] += sign > 0 ? fmin(m[c], 0.0) : -fmax(m[c], 0.0);
                mag[c] += fabs(m[c]);
            }
        }
    };
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_src[e] > node) {
            break;
        }
        if (edge_departed(B, g, e)) {
            edge(e, -1);
        }
    }
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (edge_departed(B, g, e)) {
            edge(e, +1);
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (edge_departed(B, g, e)) {
            edge(e, -1);
        }
    }
    // margin: the bound's own rounding (FP64: 1e-12, float: 4e-6 relative to the summed magnitudes)
    const R margin = std::is_same<R, float>::value ? (R)4e-6 : (R)1e-12;
    bool flag      = false;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        ynew_set(B, so + c, acc[c].get());
        flag = flag || (bound[c] < margin * mag[c]);
    }
    list0_push(B, node * MGPU_MAX_GROUPS + gr, flag);
}

// ---- FP32 node passes of the mixed solver ------------------------------------
// Per edge: the float4 vectors of the source's snapshot record and of the edge's
// coefficient record that hold mobile compartments (two each for S, E, INS, ISy,
// R), the traveler products, and exact TwoSum updates; everything about the node
// itself (its snapshot and factors for out-edges, its force of infection and
// rates for in-edges) is loaded once.

struct GroupSnap {
    float y[kC];
    float risk, nd;
};

// Vector loads of the FP32 tables. Every age-group state row of the 10
// compartments starts on an 8-byte boundary (state offsets are multiples of 10
// floats); the 12 auxiliary values of a (node, group) and every vector of the
// snapshot and coefficient records start on a 16-byte boundary. The snapshot,
// coefficient and auxiliary tables are read-only in the kernels that use them
// (read-only data path); the node states use plain loads and stores.
static_assert(kC == 10 && kAux == 12, "vector widths of the FP32 tables");
__device__ __forceinline__ void ld_state(const float* p, float (&v)[kC])
{
    const float2* q = reinterpret_cast<const float2*>(p);
#pragma unroll
    for (int i = 0; i < kC / 2; ++i) {
        const float2 a = q[i];
        v[2 * i]       = a.x;
        v[2 * i + 1]   = a.y;
    }
}
__device__ __forceinline__ void st_state(float* p, const float (&v)[kC])
{
    float2* q = reinterpret_cast<float2*>(p);
#pragma unroll
    for (int i = 0; i < kC / 2; ++i) {
        q[i] = make_float2(v[2 * i], v[2 * i + 1]);
    }
}



// Compartment masks of the FP32 passes: MASK holds the compartments whose
// travelers can be nonzero (a nonzero coefficient on some edge of every graph
// of the batch); the other compartments' travelers and the flows out of them
// are exactly zero, so their arithmetic is compiled out. kMaskAll is the
// general case; kMaskSEIYR the usual commuter pattern (S, E, INS, ISy, R).
constexpr int kMaskAll   = (1 << kC) - 1;
constexpr int kMaskSEIYR = (1 << MGPU_S) | (1 << MGPU_E) | (1 << MGPU_INS) | (1 << MGPU_ISY) | (1 << MGPU_R);
__host__ __device__ constexpr bool in_mask(int mask, int c)
{
    return ((mask >> c) & 1) != 0;
}
// compartments a return can change: the mobile ones and the targets of their flows
__host__ __device__ constexpr int touched_mask(int mask)
{
    int t = mask;
    for (int k = 0; k < kF; ++k) {
        if (in_mask(mask, kFlowSrcI(k))) {
            t |= 1 << kFlowDstI(k);
        }
    }
    return t;
}

// The auxiliary values the flows out of MASK need (the others are never used).
__host__ __device__ constexpr int aux_of_flow(int k)
{
    // the rate index of flow k in the auxiliary values (see flows_f)
    return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 2 : k == 3 ? 3 : k == 4 ? 2 : k == 5 ? 3 : k == 6 ? 4 : k == 7 ? 5
         : k == 8 ? 4 : k == 9 ? 5 : k == 10 ? 6 : k == 11 ? 7 : k == 12 ? 8 : k == 13 ? 9 : 10;
}
template <int MASK>
__device__ __forceinline__ void ld_aux_m(const float* p, float (&v)[kAux])
{
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int i = 0; i < kAux / 4; ++i) {
        bool need = false;
#pragma unroll
        for (int k = 0; k < kF; ++k) {
            const int a = aux_of_flow(k);
            need        = need || (in_mask(MASK, kFlowSrcI(k)) && a >= 4 * i && a < 4 * i + 4);
        }
        if (need) {
            const float4 x = __ldg(q + i);
            v[4 * i]       = x.x;
            v[4 * i + 1]   = x.y;
            v[4 * i + 2]   = x.z;
            v[4 * i + 3]   = x.w;
        }
        else {
            v[4 * i] = v[4 * i + 1] = v[4 * i + 2] = v[4 * i + 3] = 0.0f;
        }
    }
}

// m = ((y o c) o f) with the nondetection factor nd on INS and ISy (same operations as depart_travelers<float>)
template <int MASK = kMaskAll>
__device__ __forceinline__ void travelers_cf(const GroupSnap& s, float nd, const float (&cf)[kC], float (&m)[kC])
{
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        if (!in_mask(MASK, c)) {
            m[c] = 0.0f;
            continue;
        }
        float v = __fmul_rn(__fmul_rn(s.y[c], cf[c]), c == MGPU_ISY ? s.risk : 1.0f);
        if (c == MGPU_INS || c == MGPU_ISY) {
            v = __fmul_rn(v, nd);
        }
        m[c] = v;
    }
}

// does MASK need vector v of a record (with the factor slots when `factors`)?
__host__ __device__ constexpr bool rec_need(int mask, int v, bool factors)
{
    bool need = factors && v == REC_RISK / 4 && (in_mask(mask, MGPU_INS) || in_mask(mask, MGPU_ISY));
    for (int c = 0; c < kC; ++c) {
        need = need || (in_mask(mask, c) && rec_pos(c) / 4 == v);
    }
    return need;
}
// Record loads of the vectors MASK needs (the other compartments read as zero).
template <int MASK, bool FACTORS>
__device__ __forceinline__ void ld_rec_m(const float* base, int64_t r0, int G, int gr, float (&y)[kC], float& risk,
                                         float& nd)
{
    float r[kRec];
#pragma unroll
    for (int v = 0; v < kRec / 4; ++v) {
        if (rec_need(MASK, v, FACTORS)) {
            const float4 x = __ldg(reinterpret_cast<const float4*>(base + rec_vec(r0, G, gr, v)));
            r[4 * v]       = x.x;
            r[4 * v + 1]   = x.y;
            r[4 * v + 2]   = x.z;
            r[4 * v + 3]   = x.w;
        }
        else {
            r[4 * v] = r[4 * v + 1] = r[4 * v + 2] = r[4 * v + 3] = 0.0f;
        }
    }
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        y[c] = in_mask(MASK, c) ? r[rec_pos(c)] : 0.0f;
    }
    risk = r[REC_RISK];
    nd   = r[REC_ND];
}

// Record addressing of one graph for the FP32 passes, computed once per thread:
// the snapshot slot, and the record rows of node 0 and edge 0 (a node's first row
// is srow0 + node * G, an edge's crow0 + edge * G, with global node and edge ids).
struct RecCtx {
    const float* snap;
    int64_t srow0, crow0;
    int G;
    __device__ RecCtx(const BatchDev& B, const DevGraph& g, int slot)
        : snap(B.gsnap + (int64_t)slot * (B.state_total / kC) * kRec)
        , srow0(g.state_off / kC - g.node0 * g.G)
        , crow0(g.ecoef_f_off / kC - g.edge0 * g.G)
        , G(g.G)
    {
    }
};

// the coefficients of edge e for age group gr: its record, or (UNI) the one
// value every moved compartment has
template <int MASK, bool UNI>
__device__ __forceinline__ void ld_coef_m(const BatchDev& B, const RecCtx& x, int64_t e, int gr, float (&cf)[kC])
{
    if constexpr (UNI) {
        const float u = __ldg(B.ecoef_u + x.crow0 + e * x.G + gr);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            cf[c] = in_mask(MASK, c) ? u : 0.0f;
        }
    }
    else {
        float unused0, unused1;
        ld_rec_m<MASK, false>(B.ecoef_r, x.crow0 + e * x.G, x.G, gr, cf, unused0, unused1);
    }
}

template <int MASK, bool UNI>
__device__ __forceinline__ void travelers_f(const BatchDev& B, const RecCtx& x, int64_t e, int gr,
                                            const GroupSnap& s, float (&m)[kC])
{
    float cf[kC];
    ld_coef_m<MASK, UNI>(B, x, e, gr, cf);
    travelers_cf<MASK>(s, s.nd, cf, m);
}

template <int MASK>
__device__ __forceinline__ void load_group_snap_m(const RecCtx& x, int64_t node, int gr, GroupSnap& s)
{
    ld_rec_m<MASK, true>(x.snap, x.srow0 + node * x.G, x.G, gr, s.y, s.risk, s.nd);
}

template <int MASK = kMaskAll>
__device__ __forceinline__ void flows_f(const float (&a)[kAux], float dt, const float (&m)[kC], float (&phi)[kF])
{
    const int ai[kF] = {0, 1, 2, 3, 2, 3, 4, 5, 4, 5, 6, 7, 8, 9, 10};
#pragma unroll
    for (int k = 0; k < kF; ++k) {
        phi[k] = in_mask(MASK, kFlowSrcI(k)) ? __fmul_rn(dt, __fmul_rn(a[ai[k]], m[kFlowSrcI(k)])) : 0.0f;
    }
}

// The incident edges of `node` in the serial return order of the reference
// (edges sorted by (src, dst)): in-edges from lower nodes [k0, km), the
// out-edges [o0, o1), then in-edges from higher nodes [km, k1). Three counted
// loops (instead of one loop over a merged sequence) let the compiler issue the
// gathers of the next edges ahead of the arithmetic of the current one.
struct EdgeRanges {
    int64_t k0, km, k1, o0, o1;
    __device__ EdgeRanges(const BatchDev& B, int64_t v)
        : k0(B.in_ptr[v])
        , km(B.in_mid[v])
        , k1(B.in_ptr[v + 1])
        , o0(B.out_ptr[v])
        , o1(B.out_ptr[v + 1])
    {
    }
};

#ifndef MGPU_XF_UNROLL
#define MGPU_XF_UNROLL 2 // edges per iteration of the return and departure loops
#endif
constexpr int kXfUnroll = MGPU_XF_UNROLL;
// resident 128-thread blocks per SM the register budget must allow, for the
// usual commuter mask and for all compartments mobile (measured)
#ifndef MGPU_XF_RETURN_MIN_BLOCKS
#define MGPU_XF_RETURN_MIN_BLOCKS 5
#endif
#ifndef MGPU_XF_RETURN_MIN_BLOCKS_ALL
#define MGPU_XF_RETURN_MIN_BLOCKS_ALL 3
#endif
#ifndef MGPU_XF_DEPART_MIN_BLOCKS
#define MGPU_XF_DEPART_MIN_BLOCKS 5
#endif
#ifndef MGPU_XF_DEPART_MIN_BLOCKS_ALL
#define MGPU_XF_DEPART_MIN_BLOCKS_ALL 4
#endif
// Where the FP32 passes read the snapshot records and the return-time rates:
// TabG gathers them from the global tables (L2), TabS from the copy of one
// graph's rows in shared memory (rates from shared memory when AUXS). Both
// produce the same values, so the two kinds of pass give identical results.
template <int MASK>
struct TabG {
    RecCtx x;
    const float* aux;
    __device__ __forceinline__ void snap(int64_t node, int gr, GroupSnap& s) const
    {
        load_group_snap_m<MASK>(x, node, gr, s);
    }
    __device__ __forceinline__ void rates(int64_t node, int gr, float (&a)[kAux]) const
    {
        ld_aux_m<MASK>(aux + (node * MGPU_MAX_GROUPS + gr) * kAux, a);
    }
};

// record vectors (float4) of the snapshot records, and of the return-time
// rates, that MASK needs: their count and the slot of vector v among them
__host__ __device__ constexpr int aux_need(int mask, int v)
{
    bool need = false;
    for (int k = 0; k < kF; ++k) {
        const int a = aux_of_flow(k);
        need        = need || (in_mask(mask, kFlowSrcI(k)) && a >= 4 * v && a < 4 * v + 4);
    }
    return need;
}
__host__ __device__ constexpr int snap_nvec(int mask)
{
    return (int)rec_need(mask, 0, true) + (int)rec_need(mask, 1, true) + (int)rec_need(mask, 2, true);
}
__host__ __device__ constexpr int aux_nvec(int mask)
{
    return (int)aux_need(mask, 0) + (int)aux_need(mask, 1) + (int)aux_need(mask, 2);
}
__host__ __device__ constexpr int snap_slot_of(int mask, int v)
{
    return v == 0 ? 0 : (int)rec_need(mask, 0, true) + (v == 2 ? (int)rec_need(mask, 1, true) : 0);
}
__host__ __device__ constexpr int aux_slot_of(int mask, int v)
{
    return v == 0 ? 0 : (int)aux_need(mask, 0) + (v == 2 ? (int)aux_need(mask, 1) : 0);
}

// Shared-memory copy of one graph: snapshot vector slot j of (local node v,
// group gr) at float4 (v * NS + j) * G + gr (the groups of a node side by
// side, as in the global records); rate vector slot j at (v * G + gr) * NA + j.
template <int MASK, bool AUXS>
struct TabS {
    static constexpr int NS = snap_nvec(MASK);
    static constexpr int NA = aux_nvec(MASK);
    RecCtx x;
    const float* aux;
    const float4* ss;
    const float4* sa;
    int64_t node0;
    __device__ __forceinline__ void snap(int64_t node, int gr, GroupSnap& s) const
    {
        const int64_t v = node - node0;
        float r[kRec];
#pragma unroll
        for (int q = 0; q < kRec / 4; ++q) {
            if (rec_need(MASK, q, true)) {
                const float4 a = ss[(v * NS + snap_slot_of(MASK, q)) * x.G + gr];
                r[4 * q]       = a.x;
                r[4 * q + 1]   = a.y;
                r[4 * q + 2]   = a.z;
                r[4 * q + 3]   = a.w;
            }
            else {
                r[4 * q] = r[4 * q + 1] = r[4 * q + 2] = r[4 * q + 3] = 0.0f;
            }
        }
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            s.y[c] = in_mask(MASK, c) ? r[rec_pos(c)] : 0.0f;
        }
        s.risk = r[REC_RISK];
        s.nd   = r[REC_ND];
    }
    __device__ __forceinline__ void rates(int64_t node, int gr, float (&a)[kAux]) const
    {
        if constexpr (AUXS) {
            const int64_t i = ((node - node0) * x.G + gr) * NA;
#pragma unroll
            for (int q = 0; q < kAux / 4; ++q) {
                if (aux_need(MASK, q)) {
                    const float4 w = sa[i + aux_slot_of(MASK, q)];
                    a[4 * q]       = w.x;
                    a[4 * q + 1]   = w.y;
                    a[4 * q + 2]   = w.z;
                    a[4 * q + 3]   = w.w;
                }
                else {
                    a[4 * q] = a[4 * q + 1] = a[4 * q + 2] = a[4 * q + 3] = 0.0f;
                }
            }
        }
        else {
            ld_aux_m<MASK>(aux + (node * MGPU_MAX_GROUPS + gr) * kAux, a);
        }
    }
};

// 16-byte asynchronous copy global -> shared (L2 only), and the wait for all of
// this thread's copies (the hardware wait of cp.async, no spin loop)
__device__ __forceinline__ void cp_async16(float4* smem, const float4* gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Copies graph g's snapshot records of slot `slot` (and, when AUXS, its
// return-time rates) to shared memory: the float4 vectors MASK needs, as
// coalesced asynchronous copies by the whole block, all in flight at once.
template <int MASK, bool AUXS>
__device__ __forceinline__ void stage_graph(const BatchDev& B, const DevGraph& g, int slot, float4* ss, float4* sa)
{
    constexpr int NS = snap_nvec(MASK);
    constexpr int NA = aux_nvec(MASK);
    const int G      = g.G;
    const float4* gs = reinterpret_cast<const float4*>(B.gsnap + (int64_t)slot * (B.state_total / kC) * kRec) +
                       (g.state_off / kC) * (kRec / 4);
    const int ns = g.N * NS * G;
    for (int u = threadIdx.x; u < ns; u += blockDim.x) {
        const int v   = u / (NS * G);
        const int rem = u - v * NS * G;
        const int j   = rem / G;
        const int gr  = rem - j * G;
        // the record vector of slot j
        int vec = 0;
#pragma unroll
        for (int q = 0; q < kRec / 4; ++q) {
            if (rec_need(MASK, q, true) && snap_slot_of(MASK, q) == j) {
                vec = q;
            }
        }
        cp_async16(ss + u, gs + (int64_t)v * G * (kRec / 4) + vec * G + gr);
    }
    if constexpr (AUXS) {
        const float4* ga = reinterpret_cast<const float4*>(B.aux) + g.node0 * MGPU_MAX_GROUPS * (kAux / 4);
        const int na     = g.N * G * NA;
        for (int u = threadIdx.x; u < na; u += blockDim.x) {
            const int item = u / NA;
            const int j    = u - item * NA;
            const int v    = item / G;
            const int gr   = item - v * G;
            int vec        = 0;
#pragma unroll
            for (int q = 0; q < kAux / 4; ++q) {
                if (aux_need(MASK, q) && aux_slot_of(MASK, q) == j) {
                    vec = q;
                }
            }
            cp_async16(sa + u, ga + ((int64_t)v * MGPU_MAX_GROUPS + gr) * (kAux / 4) + vec);
        }
    }
    cp_async_wait_all();
    __syncthreads();
}

// The end of an item's return: the in-edges' Euler flows from their sum, the
// flow increments of both directions, the no-underflow bound, the store and the
// exact path's work list.
template <int MASK>
__device__ __forceinline__ void xf_return_finish(const BatchDev& B, const DevGraph& g, int64_t node, int gr,
                                                 float dt, const float (&y0)[kC], const float (&a_own)[kAux],
                                                 Acc<float> (&acc)[kC], const float (&m_in)[kC],
                                                 const float (&m_low)[kC], const float (&m_out)[kC],
                                                 const float (&phi_out)[kF], float neg_in, float neg_low)
{
    // The in-edges' travelers all take this node's own rates, so their Euler
    // flows are those of their sum. Flow increments: in-edges take their
    // travelers' increments away, out-edges bring theirs home.
    float phi_in[kF], phi_low[kF];
    flows_f<MASK>(a_own, dt, m_in, phi_in);
    flows_f<MASK>(a_own, dt, m_low, phi_low);
#pragma unroll
    for (int f = 0; f < kF; ++f) {
        if (in_mask(MASK, kFlowSrcI(f))) {
            const float net = phi_out[f] - phi_in[f];
            acc[kFlowSrcI(f)].add(-net);
            acc[kFlowDstI(f)].add(net);
        }
    }
    // The no-underflow bound. In the reference's serial order (lower in-edges,
    // out-edges, higher in-edges) an in-edge's returning amount
    // t = m + inflows - outflows is taken away and fails when the running state
    // minus t has a negative compartment. At this node's own rates t is linear in
    // the edge's travelers: t_c = d_c m_c + sum over flows f into c of dt a_f m_src(f),
    // d_c = 1 - dt (total outflow rate of c). Per compartment:
    //  * d_c >= 0: every coefficient is >= 0, so t_c >= 0 up to K_c times the
    //    negative parts of the travelers (states slightly below zero),
    //    K_c = |d_c| + the inflow coefficients; the running state only decreases
    //    within a run of in-edges and is smallest at the run's end, where it is
    //    y0 - T(lower) after the lower run and y0 - T(all in) + T(out) after the
    //    higher one, T the summed returning amounts (from the traveler and flow sums);
    //  * d_c < 0 and no inflow into c: t_c <= 0 up to the same correction, so the
    //    in-edges take nothing from c (the serial loop's max(t, 0));
    //  * d_c < 0 with inflows: signs can differ between edges; the item takes the
    //    exact path.
    // The ends are checked less the correction and with a margin of 1e-5 of y0
    // plus the summed magnitudes (above the FP32 rounding of the sums).
    bool flag = false;
    float t_low[kC], t_in[kC], t_out[kC], mag[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        t_low[c] = m_low[c];
        t_in[c]  = m_in[c];
        t_out[c] = m_out[c];
        mag[c]   = fabsf(y0[c]) + m_in[c] + m_out[c];
    }
#pragma unroll
    for (int f = 0; f < kF; ++f) {
        if (in_mask(MASK, kFlowSrcI(f))) {
            t_low[kFlowSrcI(f)] -= phi_low[f];
            t_low[kFlowDstI(f)] += phi_low[f];
            t_in[kFlowSrcI(f)] -= phi_in[f];
            t_in[kFlowDstI(f)] += phi_in[f];
            t_out[kFlowSrcI(f)] -= phi_out[f];
            t_out[kFlowDstI(f)] += phi_out[f];
            mag[kFlowSrcI(f)] += phi_in[f] + phi_out[f];
            mag[kFlowDstI(f)] += phi_in[f] + phi_out[f];
        }
    }
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        if (in_mask(touched_mask(MASK), c)) {
            float rate = 0.0f, inflow = 0.0f;
            bool has_inflow = false;
#pragma unroll
            for (int f = 0; f < kF; ++f) {
                if (in_mask(MASK, kFlowSrcI(f))) {
                    if (kFlowSrcI(f) == c) {
                        rate += a_own[aux_of_flow(f)];
                    }
                    if (kFlowDstI(f) == c) {
                        inflow += dt * a_own[aux_of_flow(f)];
                        has_inflow = true;
                    }
                }
            }
            const float d = 1.0f - dt * rate;
            if (d < 0.0f) {
                if (has_inflow) {
                    flag = true;
                }
                t_low[c] = 0.0f;
                t_in[c]  = 0.0f;
            }
            const float k      = fabsf(d) + inflow;
            const float margin = 1e-5f * mag[c];
            flag = flag || (y0[c] - t_low[c]) + k * neg_low < margin ||
                   ((y0[c] - t_in[c]) + t_out[c]) + k * neg_in < margin;
        }
    }
    const int64_t so = g.state_off + (node - g.node0) * g.n + gr * kC;
    float h[kC], l[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].store(&h[c], &l[c]);
    }
    st_state(B.st_hi + so, h);
    st_state(B.st_lo + so, l);
    list0_push(B, node * MGPU_MAX_GROUPS + gr, flag);
}

// Packed forms for the commuter compartments S, E, INS, ISy, R with one
// coefficient per (edge, group): S and E, INS and ISy as FP32x2 pairs
// (__fadd2_rn / __fmul2_rn / __ffma2_rn, each lane rounded as the scalar
// intrinsic), so the pairs take one instruction where the scalar form takes two,
// with the same roundings in the same order as the general form.
__device__ __forceinline__ float2 f2sub(float2 a, float2 b)
{
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); // a - b, rounded once
}
struct AccP {
    float2 hi, lo;
    // TwoSum of hi and t, the error into lo (Acc<float>::add, lane by lane)
    __device__ __forceinline__ void add(float2 t)
    {
        const float2 s  = __fadd2_rn(hi, t);
        const float2 bb = f2sub(s, hi);
        const float2 e  = __fadd2_rn(f2sub(hi, f2sub(s, bb)), f2sub(t, bb));
        hi              = s;
        lo              = __fadd2_rn(lo, e);
    }
    // add(-m) with the same roundings
    __device__ __forceinline__ void sub(float2 m)
    {
        const float2 s  = f2sub(hi, m);
        const float2 bb = f2sub(s, hi);
        const float2 e  = f2sub(f2sub(hi, f2sub(s, bb)), __fadd2_rn(m, bb));
        hi              = s;
        lo              = __fadd2_rn(lo, e);
    }
};
// travelers of a group snapshot s with coefficient u and nondetection factor
// nd: (S, E), (INS, ISy) and R as in travelers_cf
struct TravP {
    float2 se, iy;
    float r;
};
__device__ __forceinline__ TravP trav_p(const GroupSnap& s, float u, float nd)
{
    const float2 uu = make_float2(u, u);
    TravP m;
    m.se   = __fmul2_rn(make_float2(s.y[MGPU_S], s.y[MGPU_E]), uu);
    m.iy   = __fmul2_rn(make_float2(s.y[MGPU_INS], s.y[MGPU_ISY]), uu);
    m.iy.y = __fmul_rn(m.iy.y, s.risk);
    m.iy   = __fmul2_rn(m.iy, make_float2(nd, nd));
    m.r    = __fmul_rn(s.y[MGPU_R], u);
    return m;
}
__device__ __forceinline__ float coef_u(const BatchDev& B, const RecCtx& x, int64_t e, int gr)
{
    return __ldg(B.ecoef_u + x.crow0 + e * x.G + gr);
}
// the coefficient of in-edge k (CSC position) of graph g, from the in-edge-ordered copy
__device__ __forceinline__ float coef_in(const BatchDev& B, const DevGraph& g, int64_t k, int gr)
{
    return __ldg(B.ecoef_in + g.ecoef_in_off + (k - g.edge0) * g.G + gr);
}
__device__ __forceinline__ void acc_to_array(const AccP& se, const AccP& iy, const Acc<float>& r,
                                             Acc<float> (&acc)[kC])
{
    acc[MGPU_S].init_pair(se.hi.x, se.lo.x);
    acc[MGPU_E].init_pair(se.hi.y, se.lo.y);
    acc[MGPU_INS].init_pair(iy.hi.x, iy.lo.x);
    acc[MGPU_ISY].init_pair(iy.hi.y, iy.lo.y);
    acc[MGPU_R] = r;
}

// xf_return_item for the commuter compartments with one coefficient per (edge, group)
template <int UNR, class Tab>
__device__ __forceinline__ void xf_return_item_p(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                                 const Tab& tab, int64_t node, int gr)
{
    constexpr int MASK = kMaskSEIYR;
    const float dt     = (float)rt.dt;
    const int64_t s0   = g.state_off + (node - g.node0) * g.n + gr * kC;
    float y0[kC], l0[kC];
    ld_state(B.st_hi + s0, y0);
    ld_state(B.st_lo + s0, l0);
    st_state(B.yn_hi + s0, y0);
    st_state(B.yn_lo + s0, l0);
    AccP a_se{make_float2(y0[MGPU_S], y0[MGPU_E]), make_float2(l0[MGPU_S], l0[MGPU_E])};
    AccP a_iy{make_float2(y0[MGPU_INS], y0[MGPU_ISY]), make_float2(l0[MGPU_INS], l0[MGPU_ISY])};
    Acc<float> a_r;
    a_r.init_pair(y0[MGPU_R], l0[MGPU_R]);
    float a_own[kAux];
    tab.rates(node, gr, a_own);
    const RecCtx& x = tab.x;
    GroupSnap own;
    tab.snap(node, gr, own);
    float2 in_se = make_float2(0.0f, 0.0f), in_iy = in_se, out_se = in_se, out_iy = in_se;
    float2 po01 = in_se, po23 = in_se, po67 = in_se;
    float in_r = 0.0f, out_r = 0.0f, neg_in = 0.0f;
    auto leave = [&](int64_t k) {
        GroupSnap src;
        const int2 se = B.in_se[k];
        tab.snap(se.x, gr, src);
        const TravP m = trav_p(src, coef_in(B, g, k, gr), src.nd);
        a_se.sub(m.se);
        a_iy.sub(m.iy);
        a_r.add(-m.r);
        in_se = __fadd2_rn(in_se, m.se);
        in_iy = __fadd2_rn(in_iy, m.iy);
        in_r += m.r;
        neg_in += fminf(m.se.x, 0.0f);
        neg_in += fminf(m.se.y, 0.0f);
        neg_in += fminf(m.iy.x, 0.0f);
        neg_in += fminf(m.iy.y, 0.0f);
        neg_in += fminf(m.r, 0.0f);
    };
    const EdgeRanges r(B, node);
#pragma unroll UNR
    for (int64_t k = r.k0; k < r.km; ++k) {
        leave(k);
    }
    const float2 low_se = in_se, low_iy = in_iy;
    const float low_r = in_r, neg_low = neg_in;
    const float2 dt2  = make_float2(dt, dt);
#pragma unroll UNR
    for (int64_t e = r.o0; e < r.o1; ++e) {
        float ax[kAux];
        tab.rates(B.edge_dst[e], gr, ax);
        const TravP m = trav_p(own, coef_u(B, x, e, gr), own.nd);
        // Euler flows at the destination's rates: S->E, E->INS; INS->ISy, INS->R; ISy->ISev, ISy->R
        const float2 p01 = __fmul2_rn(dt2, __fmul2_rn(make_float2(ax[0], ax[1]), m.se));
        const float2 p23 = __fmul2_rn(dt2, __fmul2_rn(make_float2(ax[2], ax[3]), make_float2(m.iy.x, m.iy.x)));
        const float2 p67 = __fmul2_rn(dt2, __fmul2_rn(make_float2(ax[4], ax[5]), make_float2(m.iy.y, m.iy.y)));
        a_se.add(m.se);
        a_iy.add(m.iy);
        a_r.add(m.r);
        out_se = __fadd2_rn(out_se, m.se);
        out_iy = __fadd2_rn(out_iy, m.iy);
        out_r += m.r;
        po01 = __fadd2_rn(po01, p01);
        po23 = __fadd2_rn(po23, p23);
        po67 = __fadd2_rn(po67, p67);
    }
#pragma unroll UNR
    for (int64_t k = r.km; k < r.k1; ++k) {
        leave(k);
    }
    Acc<float> acc[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].init_pair(y0[c], l0[c]);
    }
    acc_to_array(a_se, a_iy, a_r, acc);
    float m_in[kC] = {}, m_low[kC] = {}, m_out[kC] = {}, phi_out[kF] = {};
    m_in[MGPU_S]   = in_se.x;
    m_in[MGPU_E]   = in_se.y;
    m_in[MGPU_INS] = in_iy.x;
    m_in[MGPU_ISY] = in_iy.y;
    m_in[MGPU_R]   = in_r;
    m_low[MGPU_S]   = low_se.x;
    m_low[MGPU_E]   = low_se.y;
    m_low[MGPU_INS] = low_iy.x;
    m_low[MGPU_ISY] = low_iy.y;
    m_low[MGPU_R]   = low_r;
    m_out[MGPU_S]   = out_se.x;
    m_out[MGPU_E]   = out_se.y;
    m_out[MGPU_INS] = out_iy.x;
    m_out[MGPU_ISY] = out_iy.y;
    m_out[MGPU_R]   = out_r;
    phi_out[0] = po01.x;
    phi_out[1] = po01.y;
    phi_out[2] = po23.x;
    phi_out[3] = po23.y;
    phi_out[6] = po67.x;
    phi_out[7] = po67.y;
    xf_return_finish<MASK>(B, g, node, gr, dt, y0, a_own, acc, m_in, m_low, m_out, phi_out, neg_in, neg_low);
}

// xf_depart_item for the commuter compartments with one coefficient per (edge, group)
template <int UNR, class Tab>
__device__ __forceinline__ void xf_depart_item_p(const BatchDev& B, const DevGraph& g, const Tab& tab, int64_t node,
                                                 int gr)
{
    const int64_t so = g.state_off + (node - g.node0) * g.n + gr * kC;
    float h[kC], l[kC];
    ld_state(B.st_hi + so, h);
    ld_state(B.st_lo + so, l);
    AccP a_se{make_float2(h[MGPU_S], h[MGPU_E]), make_float2(l[MGPU_S], l[MGPU_E])};
    AccP a_iy{make_float2(h[MGPU_INS], h[MGPU_ISY]), make_float2(l[MGPU_INS], l[MGPU_ISY])};
    Acc<float> a_r, a_insc, a_isyc;
    a_r.init_pair(h[MGPU_R], l[MGPU_R]);
    a_insc.init_pair(h[MGPU_INSC], l[MGPU_INSC]);
    a_isyc.init_pair(h[MGPU_ISYC], l[MGPU_ISYC]);
    const RecCtx& x = tab.x;
    GroupSnap own;
    tab.snap(node, gr, own);
    const bool detect = own.nd != 1.0f;
    const float q     = 1.0f - own.nd;
    auto arrive       = [&](int64_t k) {
        GroupSnap src;
        const int2 se = B.in_se[k];
        tab.snap(se.x, gr, src);
        const TravP m = trav_p(src, coef_in(B, g, k, gr), src.nd);
        a_se.add(m.se);
        a_iy.add(m.iy);
        a_r.add(m.r);
    };
    const EdgeRanges r(B, node);
#pragma unroll UNR
    for (int64_t k = r.k0; k < r.km; ++k) {
        arrive(k);
    }
#pragma unroll UNR
    for (int64_t e = r.o0; e < r.o1; ++e) {
        const float u = coef_u(B, x, e, gr);
        if (detect) {
            // test_commuters: detected commuters move to the confirmed compartments first
            const TravP mo = trav_p(own, u, 1.0f);
            const float2 d = __fmul2_rn(mo.iy, make_float2(q, q));
            a_iy.sub(d);
            a_insc.add(d.x);
            a_isyc.add(d.y);
        }
        const TravP m = trav_p(own, u, own.nd);
        a_se.sub(m.se);
        a_iy.sub(m.iy);
        a_r.add(-m.r);
    }
#pragma unroll UNR
    for (int64_t k = r.km; k < r.k1; ++k) {
        arrive(k);
    }
    Acc<float> acc[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].init_pair(h[c], l[c]);
    }
    acc_to_array(a_se, a_iy, a_r, acc);
    acc[MGPU_INSC] = a_insc;
    acc[MGPU_ISYC] = a_isyc;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].store(&h[c], &l[c]);
    }
    st_state(B.st_hi + so, h);
    st_state(B.st_lo + so, l);
    st_state(B.v0_hi + so, h);
    st_state(B.v0_lo + so, l);
}

// Departure of one (node, age group): the travelers of its out-edges leave, the
// travelers of its in-edges arrive, summed in the serial order of the edges.
template <int MASK, bool UNI, int UNR, class Tab>
__device__ __forceinline__ void xf_depart_item(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                               const Tab& tab, int64_t node, int gr)
{
    if constexpr (MASK == kMaskSEIYR && UNI) {
        xf_depart_item_p<UNR>(B, g, tab, node, gr);
        return;
    }
    const int64_t lv = node - g.node0;
    const int64_t so = g.state_off + lv * g.n + gr * kC;
    Acc<float> acc[kC];
    {
        float h[kC], l[kC];
        ld_state(B.st_hi + so, h);
        ld_state(B.st_lo + so, l);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].init_pair(h[c], l[c]);
        }
    }
    const RecCtx& x = tab.x;
    GroupSnap own;
    tab.snap(node, gr, own);
    const bool detect = own.nd != 1.0f;
    const float q     = 1.0f - own.nd;
    // travelers arriving from the source of in-edge k
    // (an edge without travelers has zero coefficients and adds exact zeros)
    auto arrive = [&](int64_t k) {
        GroupSnap src;
        float m[kC];
        const int2 se = B.in_se[k];
        tab.snap(se.x, gr, src);
        travelers_f<MASK, UNI>(B, x, se.y, gr, src, m);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if (in_mask(MASK, c)) {
                acc[c].add(m[c]);
            }
        }
    };
    const EdgeRanges r(B, node);
#pragma unroll UNR
    for (int64_t k = r.k0; k < r.km; ++k) {
        arrive(k);
    }
#pragma unroll UNR
    for (int64_t e = r.o0; e < r.o1; ++e) {
        float cf[kC], m[kC];
        ld_coef_m<MASK, UNI>(B, x, e, gr, cf);
        if (detect) {
            // test_commuters: detected commuters move to the confirmed compartments first
            float mo[kC];
            travelers_cf<MASK>(own, 1.0f, cf, mo);
            if (in_mask(MASK, MGPU_INS)) {
                acc[MGPU_INS].add(-__fmul_rn(mo[MGPU_INS], q));
                acc[MGPU_INSC].add(__fmul_rn(mo[MGPU_INS], q));
            }
            if (in_mask(MASK, MGPU_ISY)) {
                acc[MGPU_ISY].add(-__fmul_rn(mo[MGPU_ISY], q));
                acc[MGPU_ISYC].add(__fmul_rn(mo[MGPU_ISY], q));
            }
        }
        travelers_cf<MASK>(own, own.nd, cf, m);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if (in_mask(MASK, c)) {
                acc[c].add(-m[c]);
            }
        }
    }
#pragma unroll UNR
    for (int64_t k = r.km; k < r.k1; ++k) {
        arrive(k);
    }
    float h[kC], l[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].store(&h[c], &l[c]);
    }
    st_state(B.st_hi + so, h);
    st_state(B.st_lo + so, l);
    st_state(B.v0_hi + so, h);
    st_state(B.v0_lo + so, l);
}

// Dense (node, group) mapping as k_xf_return.
template <int MASK, bool UNI>
__global__ void __launch_bounds__(128, MASK == kMaskAll ? MGPU_XF_DEPART_MIN_BLOCKS_ALL : MGPU_XF_DEPART_MIN_BLOCKS)
    k_xf_depart(BatchDev B, const int32_t* inst, int64_t count, int G)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= count * G) {
        return;
    }
    const int64_t qi   = tid / G;
    const int64_t node = inst[qi];
    const int gr       = (int)(tid - qi * G);
    const int gi       = B.node_graph[node];
    const DevGraph& g  = B.graphs[gi];
    const GraphRt& rt  = B.rt[gi];
    if (!xb_departing(rt) || g.Ke != 0 || g.staged) {
        return;
    }
    const TabG<MASK> tab{RecCtx(B, g, rt.snap_slot ^ 1), reinterpret_cast<const float*>(B.aux)};
    xf_depart_item<MASK, UNI, kXfUnroll>(B, g, rt, tab, node, gr);
}

#ifndef MGPU_XS_THREADS
#define MGPU_XS_THREADS 512 // threads of the per-graph passes
#endif
#ifndef MGPU_XS_DEPART_MIN_BLOCKS
#define MGPU_XS_DEPART_MIN_BLOCKS 2
#endif
#ifndef MGPU_XS_RETURN_MIN_BLOCKS
#define MGPU_XS_RETURN_MIN_BLOCKS 1
#endif
#ifndef MGPU_XS_UNROLL
#define MGPU_XS_UNROLL 4 // edges per iteration of the per-graph passes' edge loops
#endif
#ifndef MGPU_XS_DEPART_THREADS
#define MGPU_XS_DEPART_THREADS MGPU_XS_THREADS
#endif
constexpr int kXsThreads    = MGPU_XS_THREADS;
constexpr int kXsDepThreads = MGPU_XS_DEPART_THREADS;

// The (node, group) items [i0, i1) of the work item's chunk of its graph: a
// graph of I items split into n chunks has chunks of R items, R = I / n rounded
// up to whole rounds of the block's threads, so that only its last chunk
// leaves threads idle in its last round.
struct XsChunk {
    int gi, i0, i1;
    __device__ XsChunk(const BatchDev& B, const DevGraph* graphs)
    {
        const int2 w = B.xs_work[blockIdx.x];
        gi           = w.x;
        const int k  = w.y >> 16;
        const int n  = w.y & 0xffff;
        const int I  = graphs[gi].N * graphs[gi].G;
        const int T  = (int)blockDim.x;
        const int R  = ((I + n - 1) / n + T - 1) / T * T;
        i0           = min(k * R, I);
        i1           = min(i0 + R, I);
    }
};

// One CTA per chunk of a staged graph (B.xs_work): the departure snapshot of
// the whole graph in shared memory, then the chunk's (node, group) items.
template <int MASK, bool UNI>
__global__ void __launch_bounds__(kXsDepThreads, MGPU_XS_DEPART_MIN_BLOCKS) k_xs_depart(BatchDev B)
{
    extern __shared__ float4 xs_smem[];
    const XsChunk c(B, B.graphs);
    const DevGraph& g = B.graphs[c.gi];
    const GraphRt& rt = B.rt[c.gi];
    if (!xb_departing(rt)) {
        return;
    }
    const int ws = rt.snap_slot ^ 1;
    stage_graph<MASK, false>(B, g, ws, xs_smem, nullptr);
    const TabS<MASK, false> tab{RecCtx(B, g, ws), reinterpret_cast<const float*>(B.aux), xs_smem, nullptr, g.node0};
    const int G = g.G;
    for (int i = c.i0 + threadIdx.x; i < c.i1; i += blockDim.x) {
        const int v = i / G;
        xf_depart_item<MASK, UNI, MGPU_XS_UNROLL>(B, g, rt, tab, g.node0 + v, i - v * G);
    }
}

// Return of one (node, age group): the travelers of its in-edges go home, the
// travelers of its out-edges come home, each with its Euler flows; the state
// is updated in place, the state before it kept for the exact path, and the
// item queued for that path when the no-underflow bound fails.
template <int MASK, bool UNI, int UNR, class Tab>
__device__ __forceinline__ void xf_return_item(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                               const Tab& tab, int64_t node, int gr)
{
    if constexpr (MASK == kMaskSEIYR && UNI) {
        xf_return_item_p<UNR>(B, g, rt, tab, node, gr);
        return;
    }
    const float dt   = (float)rt.dt;
    const int64_t lv = node - g.node0;
    const int64_t s0 = g.state_off + lv * g.n + gr * kC;
    Acc<float> acc[kC];
    float y0[kC];
    {
        // the return is applied in place; the state before it goes to yn for the
        // exact path (rescans and the sequential fallback start from it)
        float h[kC], l[kC];
        ld_state(B.st_hi + s0, h);
        ld_state(B.st_lo + s0, l);
        st_state(B.yn_hi + s0, h);
        st_state(B.yn_lo + s0, l);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].init_pair(h[c], l[c]);
            y0[c] = h[c];
        }
    }
    float a_own[kAux];
    tab.rates(node, gr, a_own);
    const RecCtx& x = tab.x;
    GroupSnap own;
    tab.snap(node, gr, own);
    // Sums of the travelers of the in-edges (all of them, and of the lower run)
    // and of the out-edges, the out-edges' Euler flows at their destinations'
    // rates, and the sum of the in-edge travelers' negative parts (for the bound).
    float m_in[kC], m_out[kC], phi_out[kF];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        m_in[c] = m_out[c] = 0.0f;
    }
#pragma unroll
    for (int f = 0; f < kF; ++f) {
        phi_out[f] = 0.0f;
    }
    float neg_in = 0.0f;
    // in-edge k: its travelers leave this node (an edge without travelers has
    // zero coefficients and adds exact zeros)
    auto leave = [&](int64_t k) {
        GroupSnap src;
        float m[kC];
        const int2 se = B.in_se[k];
        tab.snap(se.x, gr, src);
        travelers_f<MASK, UNI>(B, x, se.y, gr, src, m);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if (in_mask(MASK, c)) {
                acc[c].add(-m[c]);
                m_in[c] += m[c];
                neg_in += fminf(m[c], 0.0f);
            }
        }
    };
    const EdgeRanges r(B, node);
#pragma unroll UNR
    for (int64_t k = r.k0; k < r.km; ++k) {
        leave(k);
    }
    float m_low[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        m_low[c] = m_in[c];
    }
    const float neg_low = neg_in;
    // out-edge e: this node's travelers come home with their Euler flows at the
    // destination's rates
#pragma unroll UNR
    for (int64_t e = r.o0; e < r.o1; ++e) {
        float ax[kAux], m[kC], phi[kF];
        tab.rates(B.edge_dst[e], gr, ax);
        travelers_f<MASK, UNI>(B, x, e, gr, own, m);
        flows_f<MASK>(ax, dt, m, phi);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if (in_mask(MASK, c)) {
                acc[c].add(m[c]);
                m_out[c] += m[c];
            }
        }
#pragma unroll
        for (int f = 0; f < kF; ++f) {
            if (in_mask(MASK, kFlowSrcI(f))) {
                phi_out[f] += phi[f];
            }
        }
    }
#pragma unroll UNR
    for (int64_t k = r.km; k < r.k1; ++k) {
        leave(k);
    }
    xf_return_finish<MASK>(B, g, node, gr, dt, y0, a_own, acc, m_in, m_low, m_out, phi_out, neg_in, neg_low);
}

// One thread per (node, group) of the nodes with G age groups (dense: node
// = inst[tid / G], group = tid % G, so no lane idles on unused groups).
template <int MASK, bool UNI>
__global__ void __launch_bounds__(128, MASK == kMaskAll ? MGPU_XF_RETURN_MIN_BLOCKS_ALL : MGPU_XF_RETURN_MIN_BLOCKS)
    k_xf_return(BatchDev B, const int32_t* inst, int64_t count, int G)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= count * G) {
        return;
    }
    const int64_t q    = tid / G;
    const int64_t node = inst[q];
    const int gr       = (int)(tid - q * G);
    const int gi       = B.node_graph[node];
    const DevGraph& g  = B.graphs[gi];
    const GraphRt& rt  = B.rt[gi];
    if (!xb_returning(rt) || g.Ke != 0 || g.staged) {
        return;
    }
    const TabG<MASK> tab{RecCtx(B, g, rt.snap_slot), reinterpret_cast<const float*>(B.aux)};
    xf_return_item<MASK, UNI, kXfUnroll>(B, g, rt, tab, node, gr);
}

// One CTA per chunk of a staged graph: the whole graph's departure snapshot
// (and, when AUXS, its return-time rates) in shared memory, then the chunk's
// (node, group) items.
template <int MASK, bool UNI, bool AUXS>
__global__ void __launch_bounds__(kXsThreads, MGPU_XS_RETURN_MIN_BLOCKS) k_xs_return(BatchDev B)
{
    extern __shared__ float4 xs_smem[];
    const XsChunk c(B, B.graphs);
    const DevGraph& g = B.graphs[c.gi];
    const GraphRt& rt = B.rt[c.gi];
    if (!xb_returning(rt)) {
        return;
    }
    constexpr int NS = snap_nvec(MASK);
    float4* sa       = xs_smem + g.N * g.G * NS;
    stage_graph<MASK, AUXS>(B, g, rt.snap_slot, xs_smem, sa);
    const TabS<MASK, AUXS> tab{RecCtx(B, g, rt.snap_slot), reinterpret_cast<const float*>(B.aux), xs_smem, sa,
                               g.node0};
    const int G = g.G;
    for (int i = c.i0 + threadIdx.x; i < c.i1; i += blockDim.x) {
        const int v = i / G;
        xf_return_item<MASK, UNI, MGPU_XS_UNROLL>(B, g, rt, tab, g.node0 + v, i - v * G);
    }
}

// ---- exact underflow path ------------------------------------------------------
// The reference fixes a negative remainder of compartment c by moving the deficit
// to the largest compartment of the same age group (:576-596). All of it stays
// inside one age group, so the exact serial order can be replayed by independent
// (node, age group) threads. A (node, group) item enters list 0 when its bound
// fails; a scan of the item fixes its in-edges against its running FP64 state and
// publishes the fixed travelers per (edge, group) in mfix / fix_cnt; a change
// marks the edge's (source, group) for a rescan (the source's state contains
// those travelers). A few passes settle the chains of fixes; a graph with items
// still marked after the last pass takes the sequential pass.

// The three work lists rotate over the scan passes: pass p reads list p % 3 and
// fills list (p + 1) % 3; the interval start empties all three, and pass p >= 1
// empties list (p + 2) % 3, which pass p + 1 fills (its last reader, pass p - 1,
// has finished). The return pass fills list 0.
__device__ __forceinline__ int scan_list_in(int pass)
{
    return pass % 3;
}
__device__ __forceinline__ int scan_list_out(int pass)
{
    return (pass + 1) % 3;
}
__device__ __forceinline__ void scan_list_prepare(const BatchDev& B, int pass)
{
    if (pass >= 1 && blockIdx.x == 0 && threadIdx.x == 0) {
        B.scan_count[(pass + 2) % 3] = 0;
    }
}

// Exact fix of one (edge, age group) against the running state y: with
// rem = y - t, every negative rem[c] is moved, in compartment order, to the
// first largest remainder (:576-596). Returns the number of fixed compartments.
__device__ __forceinline__ int fix_group(const double (&y)[kC], double (&t)[kC])
{
    double rem[kC];
    bool neg = false;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        rem[c] = y[c] - t[c];
        neg    = neg || rem[c] < 0;
    }
    if (!neg) {
        return 0;
    }
    int mx     = 0;
    double rmx = rem[0];
#pragma unroll
    for (int q = 1; q < kC; ++q) {
        if (rem[q] > rmx) {
            rmx = rem[q];
            mx  = q;
        }
    }
    int nfix = 0;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        if (rem[c] < 0) {
#pragma unroll
            for (int q = 0; q < kC; ++q) {
                if (q == mx) {
                    t[q] -= rem[c];
                }
            }
            t[c] += rem[c];
            ++nfix;
        }
    }
    return nfix;
}

template <class R>
__global__ void k_xg_scan(BatchDev B, int pass)
{
    const int lin    = scan_list_in(pass);
    const int lout   = scan_list_out(pass);
    scan_list_prepare(B, pass);
    const int cnt    = B.scan_count[lin];
    const int64_t NG = B.num_nodes * MGPU_MAX_GROUPS;
    if (blockIdx.x == 0 && threadIdx.x == 0 && cnt > 0) {
        atomicAdd(&B.counters[CNT_SCANNED], (unsigned long long)cnt);
    }
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < cnt;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = B.scan_list[lin * NG + idx];
        B.scan_mark[lin * NG + item] = 0; // consumed
        const int64_t node = item / MGPU_MAX_GROUPS;
        const int gr       = (int)(item % MGPU_MAX_GROUPS);
        const int gi       = B.node_graph[node];
        const DevGraph& g  = B.graphs[gi];
        const GraphRt& rt  = B.rt[gi];
        if (gr >= g.G || !xb_returning(rt)) {
            continue;
        }
        const int64_t so = g.state_off + (node - g.node0) * g.n + gr * kC;
        double y[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            y[c] = state_get(B, so + c);
        }
        auto in_edge = [&](int64_t e) {
            double t[kC];
            return_travelers<R>(B, g, rt, e, gr, t);
            const int nfix = fix_group(y, t);
            uint8_t* fc    = B.fix_cnt + e * MGPU_MAX_GROUPS + gr;
            const int prev = *(volatile uint8_t*)fc;
            bool changed   = false;
            double* mf     = B.mfix + B.trav_off[e] + gr * kC;
            if (nfix) {
                changed = prev == 0;
                if (prev == 0) {
                    fix_edge_push(B, e);
                }
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    changed = changed || __ldcg(mf + c) != t[c];
                    __stcg(mf + c, t[c]);
                }
                __threadfence();
                *(volatile uint8_t*)fc = (uint8_t)nfix;
            }
            else if (prev) {
                *(volatile uint8_t*)fc = 0;
                changed                = true;
            }
            if (changed) {
                list_push(B, lout, B.edge_src[e] * MGPU_MAX_GROUPS + gr);
            }
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                y[c] -= t[c];
            }
        };
        const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
        int64_t k        = ib;
        for (; k < ie; ++k) {
            const int64_t e = B.in_edges[k];
            if (B.edge_src[e] > node) {
                break;
            }
            if (edge_departed(B, g, e)) {
                in_edge(e);
            }
        }
        for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
            if (!edge_departed(B, g, e)) {
                continue;
            }
            double t[kC];
            if (((volatile uint8_t*)B.fix_cnt)[e * MGPU_MAX_GROUPS + gr] != 0) {
                const double* mf = B.mfix + B.trav_off[e] + gr * kC;
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    t[c] = __ldcg(mf + c);
                }
            }
            else {
                return_travelers<R>(B, g, rt, e, gr, t);
            }
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                y[c] += t[c];
            }
        }
        for (; k < ie; ++k) {
            const int64_t e = B.in_edges[k];
            if (edge_departed(B, g, e)) {
                in_edge(e);
            }
        }
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            ynew_set(B, so + c, y[c]);
        }
    }
}

// ---- the exact path of the mixed solver in float-float arithmetic -------------
// GB300 runs FP64 at a small fraction of its FP32 rate, so the mixed solver
// replays the serial return order with float-float values (hi + lo, ~48 bits):
// the same decisions as FP64 except where a remainder is within ~1e-14 of zero,
// and node totals conserved to the same order. Fixed travelers are published as
// the exact pair (two floats in the 8-byte record).

struct FF {
    float h, l;
};
__device__ __forceinline__ FF ff_two_sum(float a, float b)
{
    const float s  = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e  = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ FF ff_norm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const FF s = ff_two_sum(a.h, b.h);
    const FF t = ff_two_sum(a.l, b.l);
    FF r       = ff_norm(s.h, __fadd_rn(s.l, t.h));
    return ff_norm(r.h, __fadd_rn(r.l, t.l));
}
__device__ __forceinline__ FF ff_neg(FF a)
{
    return {-a.h, -a.l};
}
__device__ __forceinline__ FF ff_add_f(FF a, float b)
{
    const FF s = ff_two_sum(a.h, b);
    return ff_norm(s.h, __fadd_rn(s.l, a.l));
}
__device__ __forceinline__ bool ff_neg_p(FF a)
{
    return a.h < 0.0f || (a.h == 0.0f && a.l < 0.0f);
}
__device__ __forceinline__ bool ff_gt(FF a, FF b)
{
    return a.h > b.h || (a.h == b.h && a.l > b.l);
}

// Returning travelers of group gr on edge e as float-float values: the FP32
// travelers plus the Euler flow increments (return_travelers in pairs). Only
// the compartments of MASK move (every coefficient of the others is zero, so
// their travelers and the flows out of them are exact zeros and are skipped).
template <int MASK>
__device__ __forceinline__ void return_travelers_ff(const BatchDev& B, const DevGraph& g, const GraphRt& rt,
                                                    int64_t e, int gr, FF (&t)[kC])
{
    float m[kC], phi[kF];
    return_flows<float>(B, g, rt, e, gr, m, phi);
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        t[c] = {in_mask(MASK, c) ? m[c] : 0.0f, 0.0f};
    }
#pragma unroll
    for (int k = 0; k < kF; ++k) {
        if (in_mask(MASK, kFlowSrcI(k))) {
            t[kFlowSrcI(k)] = ff_add_f(t[kFlowSrcI(k)], -phi[k]);
            t[kFlowDstI(k)] = ff_add_f(t[kFlowDstI(k)], phi[k]);
        }
    }
}

// fix_group in pairs
__device__ __forceinline__ int fix_group_ff(const FF (&y)[kC], FF (&t)[kC])
{
    FF rem[kC];
    bool neg = false;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        rem[c] = ff_add(y[c], ff_neg(t[c]));
        neg    = neg || ff_neg_p(rem[c]);
    }
    if (!neg) {
        return 0;
    }
    int mx = 0;
    FF rmx = rem[0];
#pragma unroll
    for (int q = 1; q < kC; ++q) {
        if (ff_gt(rem[q], rmx)) {
            rmx = rem[q];
            mx  = q;
        }
    }
    int nfix = 0;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        if (ff_neg_p(rem[c])) {
#pragma unroll
            for (int q = 0; q < kC; ++q) {
                if (q == mx) {
                    t[q] = ff_add(t[q], ff_neg(rem[c]));
                }
            }
            t[c] = ff_add(t[c], rem[c]);
            ++nfix;
        }
    }
    return nfix;
}

// One warp per item: the lanes compute the returning travelers of 32 incident
// edges at a time in parallel (the gathers), then follow the serial order with
// prefix sums over the lanes, stopping only at the edges that need the fix:
// every lane holds the same running state, and lane j publishes edge j's fix.
template <int MASK>
__global__ void k_xf_scan(BatchDev B, int pass)
{
    constexpr unsigned kFull = 0xffffffffu;
    const int lin    = scan_list_in(pass);
    const int lout   = scan_list_out(pass);
    scan_list_prepare(B, pass);
    const int cnt    = B.scan_count[lin];
    const int64_t NG = B.num_nodes * MGPU_MAX_GROUPS;
    const int lane   = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (blockIdx.x == 0 && threadIdx.x == 0 && cnt > 0) {
        atomicAdd(&B.counters[CNT_SCANNED], (unsigned long long)cnt);
    }
    for (int64_t idx = w0; idx < cnt; idx += nw) {
        const int64_t item = B.scan_list[lin * NG + idx];
        const int64_t node = item / MGPU_MAX_GROUPS;
        const int gr       = (int)(item % MGPU_MAX_GROUPS);
        __syncwarp();
        if (lane == 0) {
            B.scan_mark[lin * NG + item] = 0; // consumed
        }
        const int gi      = B.node_graph[node];
        const DevGraph& g = B.graphs[gi];
        const GraphRt& rt = B.rt[gi];
        if (gr >= g.G || !xb_returning(rt)) {
            continue; // the whole warp
        }
        const int64_t so = g.state_off + (node - g.node0) * g.n + gr * kC;
        // static graphs: the return pass ran in place and left the state before
        // the return in yn; graphs with edge dampings: the state is still in st
        const bool inplace  = g.Ke == 0;
        const float* src_hi = inplace ? B.yn_hi : B.st_hi;
        const float* src_lo = inplace ? B.yn_lo : B.st_lo;
        FF y[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            y[c] = {src_hi[so + c], src_lo[so + c]};
        }
        const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
        const int64_t ob = B.out_ptr[node], oe = B.out_ptr[node + 1];
        // in-edges from lower nodes come first (the sources ascend within the node)
        int nlow = 0;
        for (int64_t base = ib; base < ie; base += 32) {
            const int64_t k = base + lane;
            nlow += __popc(__ballot_sync(kFull, k < ie && B.in_se[k].x < node));
        }
        const int nout = (int)(oe - ob);
        const int deg  = (int)(ie - ib) + nout;
        for (int base = 0; base < deg; base += 32) {
            // this lane's edge of the chunk, in the serial order
            const int i    = base + lane;
            int kind       = 0;
            int64_t e      = 0, u = 0;
            if (i < deg) {
                if (i < nlow) {
                    kind = 1;
                    e    = B.in_se[ib + i].y;
                    u    = B.in_se[ib + i].x;
                }
                else if (i < nlow + nout) {
                    kind = 2;
                    e    = ob + (i - nlow);
                }
                else {
                    kind = 1;
                    e    = B.in_se[ib + i - nout].y;
                    u    = B.in_se[ib + i - nout].x;
                }
                if (!edge_departed(B, g, e)) {
                    kind = 0;
                }
            }
            FF t[kC];
            int prev = 0;
            if (kind != 0) {
                prev = *(volatile uint8_t*)(B.fix_cnt + e * MGPU_MAX_GROUPS + gr);
                if (kind == 2 && prev != 0) {
                    // fixed by the destination's scan: the published pair
                    const float2* mf = reinterpret_cast<const float2*>(B.mfix + B.trav_off[e] + gr * kC);
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        const float2 v = __ldcg(mf + c);
                        t[c]           = {v.x, v.y};
                    }
                }
                else {
                    return_travelers_ff<MASK>(B, g, rt, e, gr, t);
                }
            }
            else {
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    t[c] = {0.0f, 0.0f};
                }
            }
            const int nchunk = deg - base < 32 ? deg - base : 32;
            // publication of this lane's in-edge after the serial step decided
            // it: the fixed travelers and fix count (nfix > 0) or the reset of
            // an earlier fix; a change sends the source's item to a rescan
            auto publish = [&](int nfix, const FF (&tf)[kC]) {
                uint8_t* fc  = B.fix_cnt + e * MGPU_MAX_GROUPS + gr;
                float2* mf   = reinterpret_cast<float2*>(B.mfix + B.trav_off[e] + gr * kC);
                bool changed = false;
                if (nfix) {
                    changed = prev == 0;
                    if (prev == 0) {
                        fix_edge_push(B, e);
                    }
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        const float2 old = __ldcg(mf + c);
                        changed          = changed || old.x != tf[c].h || old.y != tf[c].l;
                        __stcg(mf + c, make_float2(tf[c].h, tf[c].l));
                    }
                    __threadfence();
                    *(volatile uint8_t*)fc = (uint8_t)nfix;
                }
                else if (prev) {
                    *(volatile uint8_t*)fc = 0;
                    changed                = true;
                }
                if (changed) {
                    list_push(B, lout, u * MGPU_MAX_GROUPS + gr);
                }
            };
            // The serial order in parallel: the running state after edge k is
            // y + P_k, P the inclusive prefix sum of the signed travelers (out-edges
            // add theirs, in-edges take theirs away) over the lanes not yet
            // applied; an in-edge needs the underflow fix when y + P_k has a
            // negative compartment. The first such edge j is fixed against the
            // exact running state (y advanced to just before it), as in the serial
            // loop, and the scan restarts after it with the fixed travelers applied.
            // The travelers of unfixed edges are zero outside touched_mask(MASK);
            // a published fix can carry any compartment, so a chunk holding one
            // sums all ten.
            const bool any_fixed = __any_sync(kFull, kind == 2 && prev != 0);
            auto scan_chunk = [&](auto tm) {
                constexpr int TM = decltype(tm)::value;
            int start = 0;
            while (start < nchunk) {
                FF p[kC];
                const bool live = lane >= start && lane < nchunk && kind != 0;
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    p[c] = (!live || !in_mask(TM, c)) ? FF{0.0f, 0.0f} : (kind == 2 ? t[c] : ff_neg(t[c]));
                }
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        if (in_mask(TM, c)) {
                            FF q;
                            q.h = __shfl_up_sync(kFull, p[c].h, d);
                            q.l = __shfl_up_sync(kFull, p[c].l, d);
                            if (lane >= d) {
                                p[c] = ff_add(q, p[c]);
                            }
                        }
                    }
                }
                bool need = false;
                if (live && kind == 1) {
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        need = need || ff_neg_p(in_mask(TM, c) ? ff_add(y[c], p[c]) : y[c]);
                    }
                }
                const unsigned m = __ballot_sync(kFull, need);
                const int j      = m ? __ffs(m) - 1 : nchunk;
                // in-edges before j keep their travelers: only an earlier fix is reset
                if (live && kind == 1 && lane < j && prev != 0) {
                    const FF none[kC] = {};
                    publish(0, none);
                }
                if (j > start) {
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        if (in_mask(TM, c)) {
                            FF q;
                            q.h  = __shfl_sync(kFull, p[c].h, j - 1);
                            q.l  = __shfl_sync(kFull, p[c].l, j - 1);
                            y[c] = ff_add(y[c], q);
                        }
                    }
                }
                if (j >= nchunk) {
                    break;
                }
                FF tj[kC];
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    tj[c].h = __shfl_sync(kFull, t[c].h, j);
                    tj[c].l = __shfl_sync(kFull, t[c].l, j);
                }
                const int nfix = fix_group_ff(y, tj);
                if (lane == j) {
                    publish(nfix, tj);
                }
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    y[c] = ff_add(y[c], ff_neg(tj[c]));
                }
                start = j + 1;
            }
            };
            if (any_fixed) {
                scan_chunk(std::integral_constant<int, kMaskAll>());
            }
            else {
                scan_chunk(std::integral_constant<int, touched_mask(MASK)>());
            }
        }
        if (lane == 0) {
            float* dst_hi = inplace ? B.st_hi : B.yn_hi;
            float* dst_lo = inplace ? B.st_lo : B.yn_lo;
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                const FF v     = ff_norm(y[c].h, y[c].l);
                dst_hi[so + c] = v.h;
                dst_lo[so + c] = v.l;
            }
        }
    }
}

// Nodes still marked after the last pass send their graph to the sequential
// pass; resets the lists for the next return.
__global__ void k_xg_scan_done(BatchDev B, int last_list)
{
    const int cnt    = B.scan_count[last_list];
    const int64_t NG = B.num_nodes * MGPU_MAX_GROUPS;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t item = B.scan_list[last_list * NG + i];
        B.scan_mark[last_list * NG + item] = 0;
        GraphRt& rt = B.rt[B.node_graph[item / MGPU_MAX_GROUPS]];
        if (xb_returning(rt)) {
            atomicOr(&rt.fallback, 1);
        }
    }
}

// Counts the fixes of this return and clears the per-edge fix counts: over the
// edges pushed by the scans (an edge can be listed more than once; the exchange
// of its count word makes only the first visit count), or over all edges when
// the list overflowed.
__global__ void k_xg_cleanup(BatchDev B, int64_t ne)
{
    static_assert(MGPU_MAX_GROUPS == 8, "one 8-byte count word per edge");
    const int64_t pushed = B.fix_meta[0];
    const bool all       = B.fix_meta[1] != 0 || pushed > B.fix_cap;
    const int64_t n      = all ? ne : pushed;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = all ? i : B.fix_edges[i];
        unsigned long long* word = reinterpret_cast<unsigned long long*>(B.fix_cnt) + e;
        if (*word == 0ull) {
            continue;
        }
        const unsigned long long w = atomicExch(word, 0ull);
        unsigned f                 = 0;
        for (int q = 0; q < 8; ++q) {
            f += (unsigned)(w >> (8 * q)) & 0xffu;
        }
        if (f && !B.rt[B.edge_graph[e]].fallback) {
            atomicAdd(&B.counters[CNT_UNDERFLOW], (unsigned long long)f);
        }
    }
}

// Exact serial return loop of one graph (one warp per graph) for the graphs
// the scan passes did not resolve.
template <class R>
__global__ void k_xb_sequential(BatchDev B, int g0, int ng)
{
    const int gi = g0 + blockIdx.x;
    if (blockIdx.x >= ng) {
        return;
    }
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!xb_returning(rt) || !rt.fallback) {
        return;
    }
    __shared__ double m[MGPU_MAX_GROUPS * kC];
    __shared__ double rem[MGPU_MAX_GROUPS * kC];
    const int lane = threadIdx.x;
    const int n    = g.n;
    if (B.st_hi && g.Ke == 0) {
        // the in-place return pass left the state before the return in yn
        for (int64_t j = lane; j < (int64_t)g.N * n; j += 32) {
            B.st_hi[g.state_off + j] = B.yn_hi[g.state_off + j];
            B.st_lo[g.state_off + j] = B.yn_lo[g.state_off + j];
        }
        __syncwarp();
    }
    int64_t fixes  = 0;
    for (int64_t e = g.edge0; e < g.edge0 + g.E; ++e) {
        if (!edge_departed(B, g, e)) {
            continue;
        }
        if (lane < g.G) {
            double mt[kC];
            return_travelers<R>(B, g, rt, e, lane, mt);
            for (int c = 0; c < kC; ++c) {
                m[lane * kC + c] = mt[c];
            }
        }
        __syncwarp();
        const int64_t u  = B.edge_src[e] - g.node0;
        const int64_t v  = B.edge_dst[e] - g.node0;
        const int64_t ou = g.state_off + u * n;
        const int64_t ov = g.state_off + v * n;
        bool neg         = false;
        for (int j = lane; j < n; j += 32) {
            rem[j] = state_get(B, ov + j) - m[j];
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
        if (B.estats && B.estats[gi].num_sets && lane == 0) {
            record_edge_stats(B.estats[gi], e - g.edge0, n, rt.t_next, m);
        }
        for (int j = lane; j < n; j += 32) {
            state_set(B, ou + j, state_get(B, ou + j) + m[j]);
        }
        __syncwarp();
        for (int j = lane; j < n; j += 32) {
            state_set(B, ov + j, state_get(B, ov + j) - m[j]);
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

__global__ void k_xb_commit(BatchDev B, int64_t n0, int64_t nn, int n_max)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn * n_max) {
        return;
    }
    const int64_t node = n0 + tid / n_max;
    const int j        = (int)(tid % n_max);
    const int gi       = B.node_graph[node];
    const DevGraph& g  = B.graphs[gi];
    const GraphRt& rt  = B.rt[gi];
    if (j >= g.n || !xb_returning(rt) || rt.fallback || (B.st_hi && (g.Ke == 0 || g.E == 0))) {
        return; // the mixed return of static graphs runs in place; without edges nothing returns
    }
    const int64_t o = g.state_off + (node - g.node0) * g.n + j;
    if (B.st_hi) {
        B.st_hi[o] = B.yn_hi[o];
        B.st_lo[o] = B.yn_lo[o];
    }
    else {
        B.state[o] = B.ynew[o];
    }
}

// Commuter statistics of one exchange, one thread per edge of the graphs that
// record them. returns = true: after the return passes and the exact path (before
// the cleanup clears the fix counts), the returning travelers after the underflow
// fix (graphs that took the sequential pass record there); false: after the
// departure passes (before the interval ends), the departing travelers.
template <class R>
__global__ void k_edge_stats(BatchDev B, bool returns)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= B.num_edges) {
        return;
    }
    const int gi          = B.edge_graph[e];
    const EdgeStatsDev& S = B.estats[gi];
    if (S.num_sets == 0) {
        return;
    }
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (returns ? (!xb_returning(rt) || rt.fallback) : !xb_departing(rt)) {
        return;
    }
    if (!edge_departed(B, g, e)) {
        return; // no travelers on this edge
    }
    double m[MGPU_MAX_GROUPS * kC];
    for (int gr = 0; gr < g.G; ++gr) {
        double t[kC];
        if (returns) {
            if (B.fix_cnt[e * MGPU_MAX_GROUPS + gr] != 0) {
                // the travelers after the fix, as the exact path published them
                if constexpr (std::is_same<R, float>::value) {
                    const float2* mf = reinterpret_cast<const float2*>(B.mfix + B.trav_off[e] + gr * kC);
                    for (int c = 0; c < kC; ++c) {
                        t[c] = (double)mf[c].x + (double)mf[c].y;
                    }
                }
                else {
                    for (int c = 0; c < kC; ++c) {
                        t[c] = B.mfix[B.trav_off[e] + gr * kC + c];
                    }
                }
            }
            else {
                return_travelers<R>(B, g, rt, e, gr, t);
            }
        }
        else {
            R md[kC];
            depart_travelers<R>(B, g, e, gr, rt.snap_slot ^ 1, rt.t_next, md);
            for (int c = 0; c < kC; ++c) {
                t[c] = (double)md[c];
            }
        }
        for (int c = 0; c < kC; ++c) {
            m[gr * kC + c] = t[c];
        }
    }
    record_edge_stats(S, e - g.edge0, g.n, rt.t_next, m);
}

inline unsigned blocks_of(int64_t n, int t)
{
    return (unsigned)((n + t - 1) / t);
}

constexpr int kXbScanPasses = 4;

// ev (profiling, may be null): recorded after the node pass, after the return
// pass, and after the exact path with the commit.
// The FP32 return (RET) or departure pass of a mixed batch: one launch over the
// staged graphs (one CTA each) and one per age-group count over the nodes of
// the other graphs, each instantiated for the batch's compartment mask and
// coefficient form.
template <int MASK, bool UNI, bool RET>
void launch_xf_pass_m(const BatchDev& B, cudaStream_t s, int64_t* launches)
{
    if (B.xs_count > 0) {
        if constexpr (RET) {
            if (B.xs_aux) {
                k_xs_return<MASK, UNI, true><<<(unsigned)B.xs_count, kXsThreads, B.xs_smem_ret, s>>>(B);
            }
            else {
                k_xs_return<MASK, UNI, false><<<(unsigned)B.xs_count, kXsThreads, B.xs_smem_ret, s>>>(B);
            }
        }
        else {
            k_xs_depart<MASK, UNI><<<(unsigned)B.xs_count, kXsDepThreads, B.xs_smem_dep, s>>>(B);
        }
        *launches += 1;
    }
    const int T = 128;
    for (int G = 1; G <= MGPU_MAX_GROUPS; ++G) {
        if (B.xcount[G] > 0) {
            const unsigned nb = blocks_of(B.xcount[G] * G, T);
            if constexpr (RET) {
                k_xf_return<MASK, UNI><<<nb, T, 0, s>>>(B, B.xlist[G], B.xcount[G], G);
            }
            else {
                k_xf_depart<MASK, UNI><<<nb, T, 0, s>>>(B, B.xlist[G], B.xcount[G], G);
            }
            *launches += 1;
        }
    }
}
template <bool RET>
void launch_xf_pass(const BatchDev& B, cudaStream_t s, int64_t* launches)
{
    if ((B.mob_union & ~kMaskSEIYR) == 0) {
        if (B.ecoef_u) {
            launch_xf_pass_m<kMaskSEIYR, true, RET>(B, s, launches);
        }
        else {
            launch_xf_pass_m<kMaskSEIYR, false, RET>(B, s, launches);
        }
    }
    else {
        if (B.ecoef_u) {
            launch_xf_pass_m<kMaskAll, true, RET>(B, s, launches);
        }
        else {
            launch_xf_pass_m<kMaskAll, false, RET>(B, s, launches);
        }
    }
}

template <class R>
void launch_xb(const BatchDev& B, int64_t n_max, bool any_edge_dampings, cudaStream_t s, int64_t* launches,
               cudaEvent_t* ev)
{
    auto mark = [&](int k) {
        if (ev) {
            cudaEventRecord(ev[k], s);
        }
    };
    const int64_t nn = B.num_nodes, ne = B.num_edges;
    if (nn == 0) {
        return;
    }
    const int T = 128;
    // (the mixed solver's node kernel does the node pass itself)
    if constexpr (!std::is_same<R, float>::value) {
        k_xb_prep<R><<<blocks_of(nn * MGPU_MAX_GROUPS, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    mark(0);
    if (ne == 0) {
        mark(1);
        mark(2);
        return;
    }
    const int64_t ng  = nn * MGPU_MAX_GROUPS;
    const bool mixed  = std::is_same<R, float>::value;
    if (mixed) {
        launch_xf_pass<true>(B, s, launches);
    }
    if (!mixed || any_edge_dampings) {
        k_xb_return<R><<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    mark(1);
    // exact underflow path over the work lists (list 0 was filled by the return pass)
    const unsigned scan_blocks = 152 * 8;
    for (int pass = 0; pass < kXbScanPasses; ++pass) {
        if (std::is_same<R, float>::value) {
            if ((B.mob_union & ~kMaskSEIYR) == 0) {
                k_xf_scan<kMaskSEIYR><<<scan_blocks, 128, 0, s>>>(B, pass);
            }
            else {
                k_xf_scan<kMaskAll><<<scan_blocks, 128, 0, s>>>(B, pass);
            }
        }
        else {
            k_xg_scan<R><<<scan_blocks, 128, 0, s>>>(B, pass);
        }
    }
    k_xg_scan_done<<<scan_blocks, 128, 0, s>>>(B, kXbScanPasses % 3); // the list the last pass filled
    if (!mixed || any_edge_dampings) {
        // (mixed batches without edge dampings return in place)
        k_xb_commit<<<blocks_of(nn * n_max, 256), 256, 0, s>>>(B, 0, nn, (int)n_max);
    }
    k_xb_sequential<R><<<B.num_graphs, 32, 0, s>>>(B, 0, B.num_graphs);
    if (B.estats) {
        k_edge_stats<R><<<blocks_of(ne, 128), 128, 0, s>>>(B, true);
        *launches += 1;
    }
    k_xg_cleanup<<<152 * 4, 256, 0, s>>>(B, ne);
    mark(2);
    if (any_edge_dampings) {
        k_xb_edge_flags<<<blocks_of(ne, 256), 256, 0, s>>>(B, 0, ne);
        *launches += 1;
    }
    if (mixed) {
        launch_xf_pass<false>(B, s, launches);
    }
    if (!mixed || any_edge_dampings) {
        k_xb_depart<R><<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    if (B.estats) {
        k_edge_stats<R><<<blocks_of(ne, 128), 128, 0, s>>>(B, false);
        *launches += 1;
    }
    *launches += 3 + kXbScanPasses + ((!mixed || any_edge_dampings) ? 1 : 0);
}

} // namespace

int exchange_batched_launches(const BatchDev& B, int precision, bool any_edge_dampings)
{
    const bool mixed = is_mixed(precision);
    const int prep   = mixed ? 0 : 1; // the node pass (inside the node kernel when mixed)
    if (B.num_edges == 0) {
        return prep;
    }
    const int extra  = !any_edge_dampings ? 0 : (mixed ? 3 : 1);
    const int commit = (!mixed || any_edge_dampings) ? 1 : 0;
    // return and departure passes (when mixed: one over the staged graphs and
    // one per age-group count of the other nodes); the exact path: scan passes,
    // done, sequential, cleanup
    int passes = 2;
    if (mixed) {
        passes = B.xs_count > 0 ? 2 : 0;
        for (int G = 1; G <= MGPU_MAX_GROUPS; ++G) {
            passes += B.xcount[G] > 0 ? 2 : 0;
        }
    }
    return prep + 3 + passes + kXbScanPasses + commit + extra + (B.estats ? 2 : 0);
}

namespace
{
// Per-edge and per-node indices of a batch (one grid-stride pass each): the
// traveler offset of every edge, the (source, edge) pair of every in-edge in
// CSC order, and for every node the first of its in-edges whose source is not
// lower than the node (sources ascend within a node's in-edges, so a binary
// search finds it): the split of the serial return order.
__global__ void k_edge_indices(BatchDev B, int64_t* trav_off, int2* in_se, int64_t* in_mid)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0     = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t e = t0; e < B.num_edges; e += stride) {
        const DevGraph& g = B.graphs[B.edge_graph[e]];
        trav_off[e]       = g.trav0 + (e - g.edge0) * g.n;
        const int64_t ie  = B.in_edges[e];
        in_se[e]          = make_int2(B.edge_src[ie], (int32_t)ie);
    }
    for (int64_t v = t0; v < B.num_nodes; v += stride) {
        int64_t lo = B.in_ptr[v], hi = B.in_ptr[v + 1];
        while (lo < hi) {
            const int64_t mid = lo + (hi - lo) / 2;
            if (B.edge_src[B.in_edges[mid]] < v) {
                lo = mid + 1;
            }
            else {
                hi = mid;
            }
        }
        in_mid[v] = lo;
    }
}
} // namespace

cudaError_t launch_edge_indices(const BatchDev& B, int64_t* trav_off, int2* in_se, int64_t* in_mid,
                                cudaStream_t s)
{
    const int64_t n = std::max<int64_t>(B.num_edges, B.num_nodes);
    if (n == 0) {
        return cudaSuccess;
    }
    const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
    k_edge_indices<<<blocks, 256, 0, s>>>(B, trav_off, in_se, in_mid);
    return cudaGetLastError();
}

#ifndef MGPU_XS_MIN_ITEMS
#define MGPU_XS_MIN_ITEMS 256 // smaller graphs stay in the node-list passes, which pack them densely
#endif
#ifndef MGPU_XS_AUX
#define MGPU_XS_AUX 1 // the staged return also copies the return-time rates when they fit
#endif
#ifndef MGPU_XS_CHUNK
#define MGPU_XS_CHUNK 2560 // (node, group) items per CTA of the per-graph passes, at most
#endif

namespace
{
template <int MASK, bool UNI>
void set_xs_smem(int bytes, cudaError_t& err)
{
    const cudaError_t e[3] = {
        cudaFuncSetAttribute(k_xs_depart<MASK, UNI>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
        cudaFuncSetAttribute(k_xs_return<MASK, UNI, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
        cudaFuncSetAttribute(k_xs_return<MASK, UNI, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)};
    for (const cudaError_t x : e) {
        err = err == cudaSuccess ? x : err;
    }
}
} // namespace

XsPlan plan_staged_exchange(std::vector<DevGraph>& dg, int mob_union, int device, int mode)
{
    XsPlan p;
    const bool seiyr  = (mob_union & ~kMaskSEIYR) == 0;
    const int64_t ns  = 16 * (seiyr ? snap_nvec(kMaskSEIYR) : snap_nvec(kMaskAll)); // bytes per (node, group)
    const int64_t na  = 16 * (seiyr ? aux_nvec(kMaskSEIYR) : aux_nvec(kMaskAll));
    int limit = 0, per_sm = 0, reserved = 0;
    p.err = cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (p.err == cudaSuccess) {
        p.err = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    }
    if (p.err == cudaSuccess) {
        p.err = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, device);
    }
    if (p.err != cudaSuccess) {
        limit = per_sm = 0; // nothing staged
    }
    // a staged graph's snapshot leaves room for two departure CTAs per SM: one
    // larger graph would raise every CTA's shared memory and halve the
    // departure's residency (measured: a batch with graphs up to the per-block
    // limit lost more on the departure than staging gained)
    const int64_t cap = std::min<int64_t>(limit, per_sm / 2 - reserved);
    std::vector<std::pair<int64_t, int32_t>> by_size;
    for (size_t i = 0; i < dg.size(); ++i) {
        DevGraph& d         = dg[i];
        const int64_t items = (int64_t)d.N * d.G;
        d.staged            = d.E > 0 && d.Ke == 0 && items >= MGPU_XS_MIN_ITEMS && items * ns <= cap;
        if (d.staged) {
            by_size.push_back({items, (int32_t)i});
        }
    }
    // largest graphs first: the CTAs that run longest start first
    std::stable_sort(by_size.begin(), by_size.end(),
                     [](const std::pair<int64_t, int32_t>& a, const std::pair<int64_t, int32_t>& b) {
                         return a.first > b.first;
                     });
    // each graph in near-equal chunks of at most MGPU_XS_CHUNK items, one CTA
    // each, so that a few large graphs do not leave the last wave of CTAs short
    int64_t max_items = 0;
    for (const auto& it : by_size) {
        const int n = (int)std::min<int64_t>((it.first + MGPU_XS_CHUNK - 1) / MGPU_XS_CHUNK, 0xffff);
        for (int k = 0; k < n; ++k) {
            p.work.push_back(make_int2(it.second, (k << 16) | n));
        }
        max_items = std::max(max_items, it.first);
    }
    // automatic mode: per-graph passes only when their CTAs fill the GPU (two
    // per SM); a batch of a few graphs spreads better over the node lists
    int sms = 0;
    if (mode == 1 && (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
                      (int64_t)p.work.size() < 2 * (int64_t)sms)) {
        p.work.clear();
        max_items = 0;
        for (DevGraph& d : dg) {
            d.staged = 0;
        }
        return p;
    }
    p.aux      = MGPU_XS_AUX && max_items * (ns + na) <= limit;
    p.smem_dep = (int32_t)(max_items * ns);
    p.smem_ret = (int32_t)(max_items * (ns + (p.aux ? na : 0)));
    if (!p.work.empty()) {
        // the largest allowed size: the attribute is per kernel, and batches of
        // different sizes share the kernels
        set_xs_smem<kMaskSEIYR, true>(limit, p.err);
        set_xs_smem<kMaskSEIYR, false>(limit, p.err);
        set_xs_smem<kMaskAll, true>(limit, p.err);
        set_xs_smem<kMaskAll, false>(limit, p.err);
    }
    return p;
}

void launch_exchange_batched(const BatchDev& B, int precision, int64_t n_max, bool any_edge_dampings,
                             cudaStream_t s, int64_t* launches, cudaEvent_t* ev)
{
    if (is_mixed(precision)) {
        launch_xb<float>(B, n_max, any_edge_dampings, s, launches, ev);
    }
    else {
        launch_xb<double>(B, n_max, any_edge_dampings, s, launches, ev);
    }
}

} // namespace mgpu
