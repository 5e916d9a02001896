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
//
// Precision (template R): R = double reproduces the FP64 arithmetic of the
// reference (up to the association of the force-of-infection sum). R = float
// computes travelers and Euler increments in FP32 with correctly rounded
// intrinsics only (no contraction), so both endpoints of an edge obtain the
// bit-identical value; the node states accumulate them in float-float
// (TwoSum) pairs and are stored as FP64, which conserves every population.
//
// Underflow fixes: a conservative per-node bound flags the nodes whose serial
// return order might meet a negative remainder; those run the exact
// per-node scan of exchange.cu semantics in FP64 (k_xb_scan), then the
// per-graph sequential pass handles what the scan passes leave unresolved.
#include "mgpu_internal.cuh"

#include <type_traits>

namespace mgpu
{
namespace
{

constexpr int kAux = 12; // per destination and age group: lambda, r1, r2, r3, r6, r7, r10, r11, r12, r13, r14

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
            return B.ecoef_f[g.ecoef_f_off + le * g.n + j];
        }
        else {
            return B.ecoef[g.ecoef_off + le * 2 * g.n + j] -
                   0.0 * (B.ecoef[g.ecoef_off + le * 2 * g.n + j] - B.ecoef[g.ecoef_off + le * 2 * g.n + g.n + j]);
        }
    }
    return (R)edge_coeff_at(B, g, le, j, t);
}

template <class R>
__device__ __forceinline__ const R* snap_ptr(const BatchDev& B, int slot)
{
    if constexpr (std::is_same<R, float>::value) {
        return B.ysnap_f + (int64_t)slot * B.state_total;
    }
    else {
        return B.ysnap + (int64_t)slot * B.state_total;
    }
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
    const R* y       = snap_ptr<R>(B, slot) + g.state_off + lu * g.n + gr * kC;
    const R* fac     = reinterpret_cast<const R*>(B.risk) + (((int64_t)slot * B.num_nodes + u) * MGPU_MAX_GROUPS + gr) * 2;
    const R risk     = fac[0];
    const R nd       = orig ? (R)1 : fac[1];
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

// Per node: departure snapshot and ISy factor; return-time force of infection and rates.
template <class R>
__global__ void k_xb_prep(BatchDev B, int64_t n0, int64_t nn)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn) {
        return;
    }
    const int64_t node = n0 + tid;
    const int gi       = B.node_graph[node];
    const DevGraph& g  = B.graphs[gi];
    const GraphRt& rt  = B.rt[gi];
    if (!rt.active) {
        return;
    }
    const int64_t lv   = node - g.node0;
    const NodeModel nm = node_model(B, g, lv);
    const int64_t so   = g.state_off + lv * g.n;
    if (xb_returning(rt)) {
        double popv[MGPU_MAX_GROUPS * kC];
        for (int j = 0; j < g.n; ++j) {
            popv[j] = v0_get(B, so + j);
        }
        const double* pop = popv;
        const int G       = g.G;
        double C[MGPU_MAX_GROUPS * MGPU_MAX_GROUPS];
        contact_matrix_at(nm, rt.t_dep, C);
        double icu = 0.0, tnt = 0.0;
        for (int i = 0; i < G; ++i) {
            tnt += (1 - nm.gp(MGPU_G_RECOVERED_PER_INS, i)) / nm.gp(MGPU_G_TIME_INS, i) * pop[i * kC + MGPU_INS];
            icu += pop[i * kC + MGPU_ICRI];
        }
        const double cap    = nm.scalar(MGPU_P_TNT_CAPACITY);
        const Ramp rrisk    = ramp_at(tnt, cap, cap * nm.scalar(MGPU_P_TNT_MAX_RISK));
        const double season = (1 + nm.scalar(MGPU_P_SEASONALITY) *
                                       sin(kPi * ((nm.scalar(MGPU_P_START_DAY) + rt.t_dep) / 182.5 + 0.5)));
        const double icu_cap = nm.scalar(MGPU_P_ICU_CAPACITY);
        const Ramp ricu      = ramp_at(icu, 0.90 * icu_cap, icu_cap);
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
        R* a = aux_ptr<R>(B) + node * MGPU_MAX_GROUPS * kAux;
        for (int i = 0; i < G; ++i) {
            const double beta = nm.gp(MGPU_G_TRANSMISSION_PROB, i);
            double lam        = 0.0;
            for (int j = 0; j < G; ++j) {
                lam += (season * C[i * G + j]) * divN[j] * beta * press[j];
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
            R* ai                  = a + i * kAux;
            ai[0]                  = (R)lam;
            ai[1]                  = (R)(1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i));
            ai[2]                  = (R)((1 - mu) * (1 / tins));
            ai[3]                  = (R)(mu * (1.0 / tins));
            ai[4]                  = (R)(sev / tisy);
            ai[5]                  = (R)((1 - sev) / tisy);
            ai[6]                  = (R)(crit_adj / tisev);
            ai[7]                  = (R)((1.0 - cps - dps) / tisev);
            ai[8]                  = (R)((dps + death_adj) / tisev);
            ai[9]                  = (R)(dpc / ticri);
            ai[10]                 = (R)((1.0 - dpc) / ticri);
            // can one Euler step of length dt drive a returning compartment negative?
            // (it cannot when dt times every compartment's total outflow rate is <= 1)
            const double out_rate = fmax(fmax(lam, 1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i)),
                                         fmax(fmax((double)ai[2] + (double)ai[3], (double)ai[4] + (double)ai[5]),
                                              fmax((double)ai[6] + (double)ai[7] + (double)ai[8],
                                                   (double)ai[9] + (double)ai[10])));
            ai[11] = (R)((rt.dt * out_rate > 1.0) ? 1 : 0);
        }
    }
    if (xb_departing(rt)) {
        const int ws = rt.snap_slot ^ 1;
        float* yf    = B.ysnap_f + (int64_t)ws * B.state_total + so;
        double ys[MGPU_MAX_GROUPS * kC];
        if (B.st_hi) {
            for (int j = 0; j < g.n; ++j) {
                yf[j] = B.st_hi[so + j]; // the FP32 rounding of hi + lo
                ys[j] = (double)B.st_hi[so + j] + (double)B.st_lo[so + j];
            }
        }
        else {
            double* yd = B.ysnap + (int64_t)ws * B.state_total + so;
            for (int j = 0; j < g.n; ++j) {
                const double v = B.state[so + j];
                yd[j]          = v;
                yf[j]          = (float)v;
                ys[j]          = v;
            }
        }
        // per age group: ISy mobility factor and commuter nondetection at this departure
        R* fac = reinterpret_cast<R*>(B.risk) + ((int64_t)ws * B.num_nodes + node) * MGPU_MAX_GROUPS * 2;
        const CVec y{ys, 1};
        const double t    = rt.t_next;
        const double nd   = (t >= nm.scalar(MGPU_P_START_COMMUTER_DETECTION) &&
                           t < nm.scalar(MGPU_P_END_COMMUTER_DETECTION))
                                ? nm.scalar(MGPU_P_COMMUTER_NONDETECTION)
                                : 1.0;
        for (int gr = 0; gr < g.G; ++gr) {
            fac[2 * gr]     = (R)mobility_isy_factor(nm, y, gr);
            fac[2 * gr + 1] = (R)nd;
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
    if (flag) {
        B.node_flag[node] = 1;
    }
}

// ---- FP32 node passes of the mixed solver ------------------------------------
// Per edge: 22 loads (source snapshot, source factors, coefficients), the
// traveler products, and 10 exact TwoSum updates; everything about the node
// itself (its snapshot and factors for out-edges, its force of infection and
// rates for in-edges) is loaded once.

struct GroupSnap {
    float y[kC];
    float risk, nd;
};

__device__ __forceinline__ void load_group_snap(const BatchDev& B, const DevGraph& g, int64_t node, int gr, int slot,
                                                GroupSnap& s)
{
    const float* y = B.ysnap_f + (int64_t)slot * B.state_total + g.state_off + (node - g.node0) * g.n + gr * kC;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        s.y[c] = y[c];
    }
    const float* fac = reinterpret_cast<const float*>(B.risk) + (((int64_t)slot * B.num_nodes + node) * MGPU_MAX_GROUPS + gr) * 2;
    s.risk           = fac[0];
    s.nd             = fac[1];
}

// m = ((y o c) o f) with the nondetection factor on INS and ISy (same operations as depart_travelers<float>)
__device__ __forceinline__ void travelers_f(const BatchDev& B, const DevGraph& g, int64_t e, int gr,
                                            const GroupSnap& s, float (&m)[kC])
{
    const float* cf = B.ecoef_f + g.ecoef_f_off + (e - g.edge0) * g.n + gr * kC;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        float v = __fmul_rn(__fmul_rn(s.y[c], cf[c]), c == MGPU_ISY ? s.risk : 1.0f);
        if (c == MGPU_INS || c == MGPU_ISY) {
            v = __fmul_rn(v, s.nd);
        }
        m[c] = v;
    }
}

__device__ __forceinline__ void flows_f(const float* a, float dt, const float (&m)[kC], float (&phi)[kF])
{
    const float s[kF] = {m[MGPU_S],    m[MGPU_E],    m[MGPU_INS],  m[MGPU_INS],  m[MGPU_INSC],
                         m[MGPU_INSC], m[MGPU_ISY],  m[MGPU_ISY],  m[MGPU_ISYC], m[MGPU_ISYC],
                         m[MGPU_ISEV], m[MGPU_ISEV], m[MGPU_ISEV], m[MGPU_ICRI], m[MGPU_ICRI]};
    const int ai[kF] = {0, 1, 2, 3, 2, 3, 4, 5, 4, 5, 6, 7, 8, 9, 10};
#pragma unroll
    for (int k = 0; k < kF; ++k) {
        phi[k] = __fmul_rn(dt, __fmul_rn(a[ai[k]], s[k]));
    }
}

__global__ void k_xf_depart(BatchDev B, int64_t n0, int64_t nn)
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
    if (gr >= g.G || !xb_departing(rt) || g.Ke != 0) {
        return;
    }
    const int ws     = rt.snap_slot ^ 1;
    const int64_t lv = node - g.node0;
    const int64_t so = g.state_off + lv * g.n + gr * kC;
    Acc<float> acc[kC];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].init_pair(B.st_hi[so + c], B.st_lo[so + c]);
    }
    GroupSnap own, src;
    load_group_snap(B, g, node, gr, ws, own);
    float m[kC];
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        const int64_t u = B.edge_src[e];
        if (u > node) {
            break;
        }
        if (B.edge_static_any[e]) {
            load_group_snap(B, g, u, gr, ws, src);
            travelers_f(B, g, e, gr, src, m);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                acc[c].add(m[c]);
            }
        }
    }
    const bool detect = own.nd != 1.0f;
    const float q     = 1.0f - own.nd;
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!B.edge_static_any[e]) {
            continue;
        }
        if (detect) {
            // test_commuters: detected commuters move to the confirmed compartments first
            GroupSnap o = own;
            o.nd        = 1.0f;
            float mo[kC];
            travelers_f(B, g, e, gr, o, mo);
            acc[MGPU_INS].add(-__fmul_rn(mo[MGPU_INS], q));
            acc[MGPU_INSC].add(__fmul_rn(mo[MGPU_INS], q));
            acc[MGPU_ISY].add(-__fmul_rn(mo[MGPU_ISY], q));
            acc[MGPU_ISYC].add(__fmul_rn(mo[MGPU_ISY], q));
        }
        travelers_f(B, g, e, gr, own, m);
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].add(-m[c]);
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_static_any[e]) {
            load_group_snap(B, g, B.edge_src[e], gr, ws, src);
            travelers_f(B, g, e, gr, src, m);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                acc[c].add(m[c]);
            }
        }
    }
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].store(B.st_hi + so + c, B.st_lo + so + c);
        B.v0_hi[so + c] = B.st_hi[so + c];
        B.v0_lo[so + c] = B.st_lo[so + c];
    }
}

__global__ void k_xf_return(BatchDev B, int64_t n0, int64_t nn)
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
    if (gr >= g.G || !xb_returning(rt) || g.Ke != 0) {
        return;
    }
    const int slot   = rt.snap_slot;
    const float dt   = (float)rt.dt;
    const int64_t lv = node - g.node0;
    const int64_t s0 = g.state_off + lv * g.n + gr * kC;
    Acc<float> acc[kC];
    float yf[kC], min_in[kC], phi_in[kF], phi_out[kF];
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].init_pair(B.st_hi[s0 + c], B.st_lo[s0 + c]);
        yf[c]     = acc[c].hi;
        min_in[c] = 0.0f;
    }
#pragma unroll
    for (int f = 0; f < kF; ++f) {
        phi_in[f]  = 0.0f;
        phi_out[f] = 0.0f;
    }
    const float* aux = reinterpret_cast<const float*>(B.aux);
    float a_own[kAux];
#pragma unroll
    for (int q = 0; q < kAux; ++q) {
        a_own[q] = aux[(node * MGPU_MAX_GROUPS + gr) * kAux + q];
    }
    GroupSnap own, src;
    load_group_snap(B, g, node, gr, slot, own);
    float m[kC], phi[kF];
    float lowest = 0.0f; // a negative traveler voids the bound
    bool unsafe  = false; // a destination whose Euler step may drive travelers negative
    auto in_edge = [&](int64_t e, int64_t u) {
        load_group_snap(B, g, u, gr, slot, src);
        travelers_f(B, g, e, gr, src, m);
        flows_f(a_own, dt, m, phi);
        // returning amounts t_c = m_c + inflows - outflows (for the bound only)
        float t[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].add(-m[c]);
            t[c]   = m[c];
            lowest = fminf(lowest, m[c]);
        }
#pragma unroll
        for (int f = 0; f < kF; ++f) {
            phi_in[f] += phi[f];
            t[kFlowSrcI(f)] -= phi[f];
            t[kFlowDstI(f)] += phi[f];
        }
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            min_in[c] += fmaxf(t[c], 0.0f);
        }
    };
    const int64_t ib = B.in_ptr[node], ie = B.in_ptr[node + 1];
    int64_t k        = ib;
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        const int64_t u = B.edge_src[e];
        if (u > node) {
            break;
        }
        if (B.edge_static_any[e]) {
            in_edge(e, u);
        }
    }
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!B.edge_static_any[e]) {
            continue;
        }
        const float* ax = aux + (B.edge_dst[e] * MGPU_MAX_GROUPS + gr) * kAux;
        travelers_f(B, g, e, gr, own, m);
        flows_f(ax, dt, m, phi);
        unsafe = unsafe || ax[11] != 0.0f;
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            acc[c].add(m[c]);
            lowest = fminf(lowest, m[c]);
        }
#pragma unroll
        for (int f = 0; f < kF; ++f) {
            phi_out[f] += phi[f];
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (B.edge_static_any[e]) {
            in_edge(e, B.edge_src[e]);
        }
    }
    // flow increments: in-edges take travelers away (their increments count
    // with the opposite sign), out-edges bring them home
#pragma unroll
    for (int f = 0; f < kF; ++f) {
        acc[kFlowSrcI(f)].add(phi_in[f]);
        acc[kFlowDstI(f)].add(-phi_in[f]);
        acc[kFlowSrcI(f)].add(-phi_out[f]);
        acc[kFlowDstI(f)].add(phi_out[f]);
    }
    // conservative no-underflow bound: with nonnegative travelers whose Euler
    // step stays nonnegative, every partial state of the serial order is at
    // least y minus the positive parts of all returning in-edge amounts
    bool flag = lowest < 0.0f || unsafe;
    const int64_t so = g.state_off + lv * g.n + gr * kC;
#pragma unroll
    for (int c = 0; c < kC; ++c) {
        acc[c].store(B.yn_hi + so + c, B.yn_lo + so + c);
        const float bound = yf[c] - min_in[c];
        const float mag   = fabsf(yf[c]) + min_in[c];
        flag              = flag || (bound < 1e-5f * mag);
    }
    if (flag) {
        B.node_flag[node] = 1;
    }
}

// Exact serial return order for one flagged or marked node (one warp): FP64
// state, the underflow fix of each in-edge, fixed travelers published in mfix
// for the source's rescan. Travelers are the same values as in k_xb_return.
template <class R>
__global__ void k_xb_scan(BatchDev B, int64_t n0, int64_t nn, int pass)
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
    if (!xb_returning(rt)) {
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
    const int64_t s0 = g.state_off + (node - g.node0) * n;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = lane + 32 * q;
        y[q]        = j < n ? state_get(B, s0 + j) : 0.0;
    }
    // lanes 0..G-1 compute one age group's travelers each into shared memory
    auto travelers = [&](int64_t e) {
        if (lane < g.G) {
            double mt[kC];
            return_travelers<R>(B, g, rt, e, lane, mt);
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                m[lane * kC + c] = mt[c];
            }
        }
        __syncwarp();
    };
    auto in_edge = [&](int64_t e) {
        travelers(e);
        bool neg = false;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int j = lane + 32 * q;
            if (j < n) {
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
        if (edge_departed(B, g, e)) {
            in_edge(e);
        }
    }
    for (int64_t e = B.out_ptr[node]; e < B.out_ptr[node + 1]; ++e) {
        if (!edge_departed(B, g, e)) {
            continue;
        }
        const bool fixed = ((volatile int32_t*)B.edge_fixed)[e] != 0;
        if (fixed) {
            const double* src = B.mfix + B.trav_off[e];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const int j = lane + 32 * q;
                if (j < n) {
                    y[q] += __ldcg(src + j);
                }
            }
        }
        else {
            travelers(e);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const int j = lane + 32 * q;
                if (j < n) {
                    y[q] += m[j];
                }
            }
            __syncwarp();
        }
    }
    for (; k < ie; ++k) {
        const int64_t e = B.in_edges[k];
        if (edge_departed(B, g, e)) {
            in_edge(e);
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int j = lane + 32 * q;
        if (j < n) {
            ynew_set(B, s0 + j, y[q]);
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

// bookkeeping kernels shared with exchange.cu semantics
__global__ void k_xb_scan_done(BatchDev B, int64_t n0, int64_t nn, int pass_end)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= nn) {
        return;
    }
    const int64_t node = n0 + tid;
    GraphRt& rt        = B.rt[B.node_graph[node]];
    uint8_t* dirty     = B.node_dirty + (pass_end & 1) * B.num_nodes;
    if (xb_returning(rt) && dirty[node]) {
        atomicOr(&rt.fallback, 1);
    }
    dirty[node]                                             = 0;
    B.node_dirty[((pass_end + 1) & 1) * B.num_nodes + node] = 0;
    B.node_flag[node]                                       = 0;
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
    if (j >= g.n || !xb_returning(rt) || rt.fallback) {
        return;
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

__global__ void k_xb_cleanup(BatchDev B, int64_t e0, int64_t ne)
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
    if (!B.rt[B.edge_graph[e]].fallback) {
        atomicAdd(&B.counters[CNT_UNDERFLOW], (unsigned long long)f);
    }
    B.edge_fixed[e] = 0;
}

inline unsigned blocks_of(int64_t n, int t)
{
    return (unsigned)((n + t - 1) / t);
}

constexpr int kXbScanPasses = 4;

template <class R>
void launch_xb(const BatchDev& B, int64_t n_max, bool any_edge_dampings, cudaStream_t s, int64_t* launches)
{
    const int64_t nn = B.num_nodes, ne = B.num_edges;
    if (nn == 0) {
        return;
    }
    const int T = 128;
    k_xb_prep<R><<<blocks_of(nn, T), T, 0, s>>>(B, 0, nn);
    *launches += 1;
    if (ne == 0) {
        return;
    }
    const int64_t ng  = nn * MGPU_MAX_GROUPS;
    const bool mixed  = std::is_same<R, float>::value;
    if (mixed) {
        k_xf_return<<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    if (!mixed || any_edge_dampings) {
        k_xb_return<R><<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    for (int pass = 0; pass < kXbScanPasses; ++pass) {
        k_xb_scan<R><<<blocks_of(nn * 32, 128), 128, 0, s>>>(B, 0, nn, pass);
    }
    k_xb_scan_done<<<blocks_of(nn, 256), 256, 0, s>>>(B, 0, nn, kXbScanPasses);
    k_xb_commit<<<blocks_of(nn * n_max, 256), 256, 0, s>>>(B, 0, nn, (int)n_max);
    k_xb_sequential<R><<<B.num_graphs, 32, 0, s>>>(B, 0, B.num_graphs);
    k_xb_cleanup<<<blocks_of(ne, 256), 256, 0, s>>>(B, 0, ne);
    if (any_edge_dampings) {
        k_xb_edge_flags<<<blocks_of(ne, 256), 256, 0, s>>>(B, 0, ne);
        *launches += 1;
    }
    if (mixed) {
        k_xf_depart<<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    if (!mixed || any_edge_dampings) {
        k_xb_depart<R><<<blocks_of(ng, T), T, 0, s>>>(B, 0, nn);
        *launches += 1;
    }
    *launches += 5 + kXbScanPasses;
}

} // namespace

int exchange_batched_launches(bool has_edges, bool any_edge_dampings)
{
    return has_edges ? 8 + kXbScanPasses + (any_edge_dampings ? 3 : 0) : 1;
}

void launch_exchange_batched(const BatchDev& B, int precision, int64_t n_max, bool any_edge_dampings,
                             cudaStream_t s, int64_t* launches)
{
    if (precision == MGPU_PRECISION_MIXED) {
        launch_xb<float>(B, n_max, any_edge_dampings, s, launches);
    }
    else {
        launch_xb<double>(B, n_max, any_edge_dampings, s, launches);
    }
}

} // namespace mgpu
