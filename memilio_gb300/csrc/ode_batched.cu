// ode_batched.cu — batched node solver: one exchange interval of many node
// instances (all nodes of all graphs of a batch) per launch.
//
// Work mapping: one lane per age group. A node instance with G groups is a
// segment of G consecutive lanes; a warp carries floor(32/G) instances
// (G = 6: 5 instances on 30 lanes). Every lane keeps its group's 10
// compartments in registers; the force of infection is a G-term contraction
// whose source terms come from the other lanes of the segment by
// __shfl_sync, and the embedded error norm is a max-reduction over the
// segment. Each instance has its own adaptive dt: segments of one warp step
// independently.
//
// Kernels:
//   k_ode_batched<G, FLOWS>  FP64 throughout, the reference's evaluation order
//                            (MGPU_PRECISION_FP64).
//   k_ode_mixed<G, false, FLOWS>  FP32 flows, stage combinations, error norm and
//                            step-size controller on an FP32 interval clock; the
//                            node state as float-float pairs updated in flow
//                            space with exact TwoSum (MGPU_PRECISION_MIXED).
//   k_ode_mixed<G, true, FLOWS>   FP32 flows and stage combinations; the state
//                            update, the error norm, the controller and the
//                            clock in FP64 (MGPU_PRECISION_MIXED_FP64_CONTROL).
// In both mixed kernels every flow increment leaves its source and enters its
// target with the same value, so every node conserves its population.
// FLOWS: the flow increments of every applied step are also summed per (node,
// age group, flow) into B.flows (FlowSimulation's flow result, FP64).
//
// Integrator: ControlledStepperWrapper<cash_karp54> inside
// SystemIntegrator::advance (memilio/math/stepper_wrapper.h:112-163,
// memilio/math/integrator.h:184-249), same controller rules as ode_plain.cu.
#include "mgpu_internal.cuh"

#include <type_traits>

namespace mgpu
{
namespace
{

__device__ __constant__ const double bk_c[6]    = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
__device__ __constant__ const double bk_a[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 5.0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
    {3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0, 0, 0},
    {-11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0, 0},
    {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
__device__ __constant__ const double bk_b5[6] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
__device__ __constant__ const double bk_db[6] = {
    37.0 / 378.0 - 2825.0 / 27648.0, 0.0, 250.0 / 621.0 - 18575.0 / 48384.0, 125.0 / 594.0 - 13525.0 / 55296.0,
    0.0 - 277.0 / 14336.0, 512.0 / 1771.0 - 1.0 / 4.0};

constexpr int S_ = MGPU_S, E_ = MGPU_E, INS_ = MGPU_INS, INSC_ = MGPU_INSC, ISY_ = MGPU_ISY, ISYC_ = MGPU_ISYC,
              ISEV_ = MGPU_ISEV, ICRI_ = MGPU_ICRI, R_ = MGPU_R, D_ = MGPU_D;

// Row i of ContactMatrixGroup::get_matrix_at(t) in FP64 (contact_matrix.h:190-194,392-399).
__device__ inline void contact_row_at(const NodeModel& nm, int i, double t, double* C)
{
    const int G   = nm.G;
    const long GG = (long)G * G;
    for (int j = 0; j < G; ++j) {
        C[j] = 0.0;
    }
    for (int m = 0; m < nm.M; ++m) {
        const double* Bm = nm.cm + m * 2 * GG + (long)i * G;
        const double* Lm = Bm + GG;
        if (nm.K) {
            const double* T  = nm.dtimes + m * nm.K;
            const int ub     = damping_upper_bound(T, nm.K, t);
            const Ramp r     = ramp_at(t, T[ub] - 1.0, T[ub]);
            const double* Dl = nm.dvals + ((long)m * nm.K + ub - 1) * GG + (long)i * G;
            const double* Dr = Dl + GG;
            for (int j = 0; j < G; ++j) {
                const double D = ramp_apply(r, Dl[j], Dr[j]);
                C[j]           = C[j] + (Bm[j] - D * (Bm[j] - Lm[j]));
            }
        }
        else {
            for (int j = 0; j < G; ++j) {
                C[j] = C[j] + (Bm[j] - 0.0 * (Bm[j] - Lm[j]));
            }
        }
    }
}

// Per-lane constants of one node instance for one interval (FP64 solver).
template <int G>
struct Seg {
    int base;
    unsigned mask;
    int gi;
    NodeModel nm;
    // own group
    double a_tnt, beta, xi, rho, rho_max;
    double r1, r2, r3, r6, r7, r11, r13, r14, r10l, r12l, cps, dps, tisev;
    // scalars
    double tnt_cap, tnt_cap2, icu_lo, icu_cap;
    double season_k, start_day;
};

template <int G>
__device__ void seg_load(Seg<G>& X, const BatchDev& B, const DevGraph& g, int64_t local)
{
    X.nm                 = node_model(B, g, local);
    const NodeModel& nm  = X.nm;
    const int i          = X.gi;
    const double mu      = nm.gp(MGPU_G_RECOVERED_PER_INS, i);
    const double tins    = nm.gp(MGPU_G_TIME_INS, i);
    const double sev     = nm.gp(MGPU_G_SEVERE_PER_ISY, i);
    const double tisy    = nm.gp(MGPU_G_TIME_ISY, i);
    const double tisev   = nm.gp(MGPU_G_TIME_ISEV, i);
    const double cps     = nm.gp(MGPU_G_CRITICAL_PER_SEVERE, i);
    const double dps     = nm.gp(MGPU_G_DEATHS_PER_SEVERE, i);
    const double dpc     = nm.gp(MGPU_G_DEATHS_PER_CRITICAL, i);
    const double ticri   = nm.gp(MGPU_G_TIME_ICRI, i);
    X.a_tnt              = (1 - mu) / tins;
    X.beta               = nm.gp(MGPU_G_TRANSMISSION_PROB, i);
    X.xi                 = nm.gp(MGPU_G_REL_TRANSMISSION_NS, i);
    X.rho                = nm.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, i);
    X.rho_max            = nm.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, i);
    X.r1                 = 1.0 / nm.gp(MGPU_G_TIME_EXPOSED, i);
    X.r2                 = (1 - mu) * (1 / tins);
    X.r3                 = mu * (1.0 / tins);
    X.r6                 = sev / tisy;
    X.r7                 = (1 - sev) / tisy;
    X.r11                = (1.0 - cps - dps) / tisev;
    X.r13                = dpc / ticri;
    X.r14                = (1.0 - dpc) / ticri;
    X.r10l               = cps / tisev;
    X.r12l               = (dps + (cps - cps)) / tisev;
    X.cps                = cps;
    X.dps                = dps;
    X.tisev              = tisev;
    const double cap     = nm.scalar(MGPU_P_TNT_CAPACITY);
    X.tnt_cap            = cap;
    X.tnt_cap2           = cap * nm.scalar(MGPU_P_TNT_MAX_RISK);
    const double icu_cap = nm.scalar(MGPU_P_ICU_CAPACITY);
    X.icu_lo             = 0.90 * icu_cap;
    X.icu_cap            = icu_cap;
    X.season_k           = nm.scalar(MGPU_P_SEASONALITY);
    X.start_day          = nm.scalar(MGPU_P_START_DAY);
}

template <int G>
__device__ __forceinline__ double seg_sum(const Seg<G>& X, double v)
{
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < G; ++k) {
        s += __shfl_sync(X.mask, v, X.base + k);
    }
    return s;
}

// Flows of the lane's age group (osecir::Model::get_flows, models/ode_secir/model.h:82-214)
// and the derivative of its 10 compartments (FlowModel::get_derivatives, flow_model.h:112-125).
template <int G>
__device__ __forceinline__ void seg_rhs(Seg<G>& X, const double (&u)[kC], double tau, double (&fl)[kF],
                                        double (&kc)[kC])
{
    const double tnt = seg_sum(X, X.a_tnt * u[INS_]);
    const double icu = seg_sum(X, u[ICRI_]);
    // own group as source j of the contact sum
    const double risk  = smoother_cosine(tnt, X.tnt_cap, X.tnt_cap2, X.rho, X.rho_max);
    const double Nj    = u[S_] + u[E_] + u[INS_] + u[ISY_] + u[ISEV_] + u[ICRI_] + u[R_];
    const double divN  = (Nj < kZeroTol) ? 0.0 : 1.0 / Nj;
    const double press = X.xi * u[INS_] + risk * u[ISY_];
    const double season =
        X.season_k == 0.0 ? 1.0 : (1 + X.season_k * sin(kPi * ((X.start_day + tau) / 182.5 + 0.5)));
    double C[G];
    contact_row_at(X.nm, X.gi, tau, C);
    double f0 = 0.0;
#pragma unroll
    for (int j = 0; j < G; ++j) {
        const double dN   = __shfl_sync(X.mask, divN, X.base + j);
        const double pr   = __shfl_sync(X.mask, press, X.base + j);
        const double cont = season * C[j];
        f0 += u[S_] * cont * dN * X.beta * pr;
    }
    // ICU smoother for CriticalPerSevere
    double r10 = X.r10l, r12 = X.r12l;
    if (!(icu <= X.icu_lo)) {
        const double crit_adj = smoother_cosine(icu, X.icu_lo, X.icu_cap, X.cps, 0.0);
        r10                   = crit_adj / X.tisev;
        r12                   = (X.dps + (X.cps - crit_adj)) / X.tisev;
    }
    fl[0]  = f0;
    fl[1]  = X.r1 * u[E_];
    fl[2]  = X.r2 * u[INS_];
    fl[3]  = X.r3 * u[INS_];
    fl[4]  = X.r2 * u[INSC_];
    fl[5]  = X.r3 * u[INSC_];
    fl[6]  = X.r6 * u[ISY_];
    fl[7]  = X.r7 * u[ISY_];
    fl[8]  = X.r6 * u[ISYC_];
    fl[9]  = X.r7 * u[ISYC_];
    fl[10] = r10 * u[ISEV_];
    fl[11] = X.r11 * u[ISEV_];
    fl[12] = r12 * u[ISEV_];
    fl[13] = X.r13 * u[ICRI_];
    fl[14] = X.r14 * u[ICRI_];
    // derivative scatter in flow order
    kc[S_]    = -fl[0];
    kc[E_]    = fl[0] - fl[1];
    kc[INS_]  = (fl[1] - fl[2]) - fl[3];
    kc[INSC_] = -fl[4] - fl[5];
    kc[ISY_]  = (fl[2] - fl[6]) - fl[7];
    kc[ISYC_] = (fl[4] - fl[8]) - fl[9];
    kc[ISEV_] = (((fl[6] + fl[8]) - fl[10]) - fl[11]) - fl[12];
    kc[ICRI_] = (fl[10] - fl[13]) - fl[14];
    kc[R_]    = ((((fl[3] + fl[5]) + fl[7]) + fl[9]) + fl[11]) + fl[14];
    kc[D_]    = fl[12] + fl[13];
}

template <int G>
__device__ __forceinline__ double seg_max(const Seg<G>& X, double v)
{
    double m = v;
#pragma unroll
    for (int k = 0; k < G; ++k) {
        m = fmax(m, __shfl_sync(X.mask, v, X.base + k));
    }
    return m;
}

template <int G, bool FLOWS>
__global__ void __launch_bounds__(128) k_ode_batched(BatchDev B, const int32_t* inst, int64_t count)
{
    constexpr int IPW = 32 / G;
    const int lane    = threadIdx.x & 31;
    const int seg     = lane / G;
    if (seg >= IPW) {
        return;
    }
    Seg<G> X;
    X.gi   = lane - seg * G;
    X.base = seg * G;
    X.mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << X.base);
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw  = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const DevOpts o   = B.opts;
    unsigned long long n_acc = 0, n_rej = 0, n_fail = 0;

    for (int64_t slot = wid * IPW + seg; slot < count; slot += nw * IPW) {
        const int64_t node = inst[slot];
        const int gidx     = B.node_graph[node];
        const DevGraph& g  = B.graphs[gidx];
        const GraphRt& rt  = B.rt[gidx];
        if (!rt.active) {
            continue;
        }
        const int64_t local = node - g.node0;
        double* yp          = B.state + g.state_off + local * g.n + X.gi * kC;
        double y[kC];
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            y[c] = yp[c];
        }
        double t          = B.node_t[node];
        double dt         = B.node_dt[node];
        const double tmax = rt.t_next;
        seg_load(X, B, g, local);
        bool cap_hit = false;

        // SystemIntegrator::advance
        const double t0   = t;
        double dt_restore = 0.0;
        double dt_min     = o.dt_min;
        int steps         = 0;
        while (fabs((tmax - t) / (tmax - t0)) > kZeroTol) {
            if (steps++ >= o.max_steps) {
                cap_hit = true;
                break;
            }
            if (dt > tmax - t) {
                dt_restore = dt;
                dt         = tmax - t;
                dt_min     = fmin(tmax - t, dt_min);
            }
            // ControlledStepperWrapper::step
            bool success     = false;
            bool is_dt_valid = true;
            double yn[kC]; // 5th-order result
            double phi[FLOWS ? kF : 1]; // (FLOWS) its flow increments
            while (!success && is_dt_valid) {
                if (dt < dt_min) {
                    is_dt_valid = false;
                    dt          = dt_min;
                }
                if (o.dt_max != 0.0 && fabs(dt) > o.dt_max) {
                    dt = o.dt_max;
                    ++n_rej;
                    continue;
                }
                // ---- one Cash-Karp attempt ----
                double k[5][kC];
                double kc[kC], fl[kF], xe[kC];
                seg_rhs(X, y, t, fl, kc);
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    k[0][c] = kc[c];
                    xe[c]   = (bk_db[0] * dt) * kc[c];
                    yn[c]   = y[c] + (bk_b5[0] * dt) * kc[c];
                }
                if constexpr (FLOWS) {
#pragma unroll
                    for (int f = 0; f < kF; ++f) {
                        phi[f] = (bk_b5[0] * dt) * fl[f];
                    }
                }
#pragma unroll
                for (int s = 1; s < 6; ++s) {
                    double u[kC];
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        double v = y[c];
#pragma unroll
                        for (int j = 0; j < s; ++j) {
                            v = v + (bk_a[s][j] * dt) * k[j][c];
                        }
                        u[c] = v;
                    }
                    seg_rhs(X, u, t + bk_c[s] * dt, fl, kc);
#pragma unroll
                    for (int c = 0; c < kC; ++c) {
                        xe[c] = xe[c] + (bk_db[s] * dt) * kc[c];
                        yn[c] = yn[c] + (bk_b5[s] * dt) * kc[c];
                        if (s < 5) {
                            k[s][c] = kc[c];
                        }
                    }
                    if constexpr (FLOWS) {
                        if (bk_b5[s] != 0.0) {
#pragma unroll
                            for (int f = 0; f < kF; ++f) {
                                phi[f] = phi[f] + (bk_b5[s] * dt) * fl[f];
                            }
                        }
                    }
                }
                // Odeint error measure, max over the instance
                double el = 0.0;
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    el = fmax(el, fabs(xe[c]) / (o.abs_tol + o.rel_tol * (fabs(y[c]) + dt * fabs(k[0][c]))));
                }
                const double err = seg_max(X, el);
                // ---- controller ----
                if (err > 1.0) {
                    dt *= fmax(0.9 * pow(err, -1.0 / 3.0), 0.2);
                    if (o.dt_max != 0.0) {
                        dt = fmin(dt, o.dt_max);
                    }
                    ++n_rej;
                }
                else {
                    t += dt;
                    if (err < 0.5) {
                        const double e = fmax(0.00032 /* 5^-5 */, err);
                        dt *= 0.9 * pow(e, -1.0 / 5.0);
                        if (o.dt_max != 0.0) {
                            dt = fmin(dt, o.dt_max);
                        }
                    }
                    success = true;
                }
            }
            dt = fmax(dt, dt_min);
            if (!success) {
                t += dt_min;
                ++n_fail;
            }
            else {
                ++n_acc;
            }
            // apply the (last) attempt
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                y[c] = yn[c];
            }
            if constexpr (FLOWS) {
                double* F = B.flows + ((g.state_off + local * g.n) / kC + X.gi) * kF;
#pragma unroll
                for (int f = 0; f < kF; ++f) {
                    F[f] += phi[f];
                }
            }
        }
        dt = fmax(dt, dt_restore);
        bool nonfinite = false;
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            yp[c]     = y[c];
            nonfinite = nonfinite || !isfinite(y[c]);
        }
        if (X.gi == 0) {
            B.node_t[node]  = t;
            B.node_dt[node] = dt;
        }
        report_instance_failure(B, gidx, cap_hit, nonfinite);
    }
    if (X.gi == 0) {
        if (n_acc) {
            atomicAdd(&B.counters[CNT_ACCEPTED], n_acc);
        }
        if (n_rej) {
            atomicAdd(&B.counters[CNT_REJECTED], n_rej);
        }
        if (n_fail) {
            atomicAdd(&B.counters[CNT_FAILED], n_fail);
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision solver. GB300 executes FP64 at ~1/64 of the FP32 rate, so
// inside an interval everything runs in FP32 except the clock (t, dt) and the
// state accumulator: each lane holds its 10 compartments as float-float pairs
// (hi + lo, ~48-bit significand, error-free TwoSum updates). Every flow
// increment is subtracted from its source and added to its target through
// the same exact TwoSum, so populations are conserved to ~2^-48 per step.
// The state is loaded from and stored to FP64 HBM once per interval.

__device__ __constant__ const float fk_c[6]    = {0.0f, 1.0f / 5.0f, 3.0f / 10.0f, 3.0f / 5.0f, 1.0f, 7.0f / 8.0f};
__device__ __constant__ const float fk_a[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0f / 5.0f, 0, 0, 0, 0},
    {3.0f / 40.0f, 9.0f / 40.0f, 0, 0, 0},
    {3.0f / 10.0f, -9.0f / 10.0f, 6.0f / 5.0f, 0, 0},
    {-11.0f / 54.0f, 5.0f / 2.0f, -70.0f / 27.0f, 35.0f / 27.0f, 0},
    {1631.0f / 55296.0f, 175.0f / 512.0f, 575.0f / 13824.0f, 44275.0f / 110592.0f, 253.0f / 4096.0f}};
__device__ __constant__ const float fk_b5[6] = {(float)(37.0 / 378.0), 0.0f, (float)(250.0 / 621.0),
                                                (float)(125.0 / 594.0), 0.0f, (float)(512.0 / 1771.0)};
__device__ __constant__ const float fk_db[6] = {
    (float)(37.0 / 378.0 - 2825.0 / 27648.0), 0.0f, (float)(250.0 / 621.0 - 18575.0 / 48384.0),
    (float)(125.0 / 594.0 - 13525.0 / 55296.0), (float)(0.0 - 277.0 / 14336.0), (float)(512.0 / 1771.0 - 1.0 / 4.0)};

// Error-free a + b (Knuth's TwoSum): hi takes the rounded sum, lo the rounding error.
__device__ __forceinline__ void df_add(float& hi, float& lo, float b)
{
    const float s  = __fadd_rn(hi, b);
    const float bb = __fsub_rn(s, hi);
    const float e  = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    hi             = s;
    lo             = __fadd_rn(lo, e);
}

__device__ __forceinline__ void df_renorm(float& hi, float& lo)
{
    const float s = __fadd_rn(hi, lo);
    lo            = __fsub_rn(lo, __fsub_rn(s, hi));
    hi            = s;
}

template <int G>
struct SegF {
    int base;
    unsigned mask;
    int gi;
    NodeModel nm;
    // per-(node, group) constants (TF_* of the FP32 table), in registers
    float tabv[kTabF];
    __device__ __forceinline__ float tc(int i) const
    {
        return tabv[i];
    }
    float season_s0;
    bool fast;
    float P[G], Q[G];
    float t_lo, t_hi, xl, scale; // damping segment and ramp, relative to t_base
    double t_base;
    float t_base_f;
    const float* cm_f; // the node's contact matrix (baseline, minimum) in FP32
    const float* dv_f; // the node's damping cache values in FP32
};

template <int G>
__device__ void segf_load_contact(SegF<G>& X, float tau_rel)
{
    const NodeModel& nm = X.nm;
    const long GG       = (long)G * G;
    const float* Bm     = X.cm_f + (long)X.gi * G;
    const float* Lm     = Bm + GG;
    if (nm.K == 0) {
#pragma unroll
        for (int j = 0; j < G; ++j) {
            X.P[j] = Bm[j];
            X.Q[j] = 0.0f;
        }
        X.t_lo  = -INFINITY;
        X.t_hi  = INFINITY;
        X.xl    = INFINITY;
        X.scale = 0.0f;
        return;
    }
    // FP32 on the interval-relative clock: the FP64 pipe of GB300 is a small
    // fraction of the FP32 one, and relative times within an interval need no
    // more than FP32 (the cache times are converted once per lookup)
    const double* T  = nm.dtimes;
    int ub           = 0;
    while (ub < nm.K && !(tau_rel < (float)T[ub] - X.t_base_f)) {
        ++ub;
    }
    ub              = ub < nm.K ? ub : nm.K - 1;
    const float* Dl = X.dv_f + (long)(ub - 1) * GG + (long)X.gi * G;
    const float* Dr = Dl + GG;
#pragma unroll
    for (int j = 0; j < G; ++j) {
        const float BL = Bm[j] - Lm[j];
        X.P[j]         = Bm[j] - (0.5f * (Dl[j] + Dr[j])) * BL;
        X.Q[j]         = -(0.5f * (Dl[j] - Dr[j])) * BL;
    }
    // times relative to the interval start; far sentinels saturate to +-inf
    const float tu = (float)T[ub];
    X.t_lo         = (float)T[ub - 1] - X.t_base_f;
    X.t_hi         = tu - X.t_base_f;
    X.xl           = (tu - 1.0f) - X.t_base_f;
    X.scale        = __frcp_rn(tu - (tu - 1.0f));
}

template <int G>
__device__ void segf_load(SegF<G>& X, const BatchDev& B, const DevGraph& g, int64_t local, double t_base)
{
    X.nm                = node_model(B, g, local);
    const NodeModel& nm = X.nm;
    const long GG       = (long)G * G;
    X.cm_f              = B.contact_f + g.contact_off + local * g.M * 2 * GG;
    X.dv_f              = g.K ? B.dvals_f + g.dval_off + local * g.M * g.K * GG : nullptr;
    // per-(node, group) constants precomputed in FP32 at upload (no FP64 division here)
    const float* T = B.tab_f + ((g.node0 + local) * MGPU_MAX_GROUPS + X.gi) * kTabF;
    X.t_base       = t_base;
    X.t_base_f     = (float)t_base;
#pragma unroll
    for (int q = 0; q < kTabF / 4; ++q) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(T) + q);
        X.tabv[4 * q] = v.x; X.tabv[4 * q + 1] = v.y; X.tabv[4 * q + 2] = v.z; X.tabv[4 * q + 3] = v.w;
    }
    X.season_s0    = (float)((nm.scalar(MGPU_P_START_DAY) + t_base) * (1.0 / 182.5) + 0.5);
    X.fast         = nm.M == 1;
    if (X.fast) {
        segf_load_contact(X, 0.0f);
    }
}

template <int G>
__device__ __forceinline__ float segf_sum(const SegF<G>& X, float v)
{
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < G; ++k) {
        s += __shfl_sync(X.mask, v, X.base + k);
    }
    return s;
}

// Rates of the lane's age group at state u: the force-of-infection factors
// (season and the contact-weighted pressure acc, so lambda = beta * season * acc)
// and the ICU-adjusted ISev -> ICri and ISev -> D rates.
template <int G>
__device__ __forceinline__ void segf_rates(SegF<G>& X, const float (&u)[kC], float tau_rel, float& season,
                                           float& acc, float& r10, float& r12)
{
    const float tnt   = segf_sum(X, X.tc(TF_A_TNT) * u[INS_]);
    const float icu   = segf_sum(X, u[ICRI_]);
    const float risk  = smoother_cosine(tnt, X.tc(TF_TNT_CAP), X.tc(TF_TNT_CAP2), X.tc(TF_RHO), X.tc(TF_RHO_MAX));
    const float Nj    = u[S_] + u[E_] + u[INS_] + u[ISY_] + u[ISEV_] + u[ICRI_] + u[R_];
    // the weighted infectious share of the group: an approximate quotient (a
    // correctly rounded reciprocal costs several times more, for no accuracy
    // the FP32 right-hand side keeps)
    const float w = (Nj < (float)kZeroTol) ? 0.0f : __fdividef(X.tc(TF_XI) * u[INS_] + risk * u[ISY_], Nj);
    season =
        X.tc(TF_SEASON_K) == 0.0f ? 1.0f : 1.0f + X.tc(TF_SEASON_K) * sinpif(X.season_s0 + tau_rel * (float)(1.0 / 182.5));
    acc = 0.0f;
    if (X.fast) {
        if (!(tau_rel >= X.t_lo && tau_rel < X.t_hi)) {
            segf_load_contact(X, tau_rel);
        }
        const float c = (tau_rel <= X.xl) ? 1.0f : cospif((tau_rel - X.xl) * X.scale);
#pragma unroll
        for (int j = 0; j < G; ++j) {
            acc += (X.P[j] + X.Q[j] * c) * __shfl_sync(X.mask, w, X.base + j);
        }
    }
    else {
        double C[G];
        contact_row_at(X.nm, X.gi, X.t_base + (double)tau_rel, C);
#pragma unroll
        for (int j = 0; j < G; ++j) {
            acc += (float)C[j] * __shfl_sync(X.mask, w, X.base + j);
        }
    }
    r10 = X.tc(TF_R10L);
    r12 = X.tc(TF_R12L);
    if (!(icu <= X.tc(TF_ICU_LO))) {
        const float crit_adj = smoother_cosine(icu, X.tc(TF_ICU_LO), X.tc(TF_ICU_CAP), X.tc(TF_CPS), 0.0f);
        r10                  = crit_adj * X.tc(TF_INV_TISEV);
        r12                  = (X.tc(TF_DPS) + (X.tc(TF_CPS) - crit_adj)) * X.tc(TF_INV_TISEV);
    }
}

// Flows and derivative of the lane's age group in FP32 (same model as seg_rhs).
template <int G>
__device__ __forceinline__ void segf_rhs(SegF<G>& X, const float (&u)[kC], float tau_rel, float (&fl)[kF],
                                         float (&kc)[kC])
{
    float season, acc, r10, r12;
    segf_rates(X, u, tau_rel, season, acc, r10, r12);
    fl[0]  = u[S_] * X.tc(TF_BETA) * season * acc;
    fl[1]  = X.tc(TF_R1) * u[E_];
    fl[2]  = X.tc(TF_R2) * u[INS_];
    fl[3]  = X.tc(TF_R3) * u[INS_];
    fl[4]  = X.tc(TF_R2) * u[INSC_];
    fl[5]  = X.tc(TF_R3) * u[INSC_];
    fl[6]  = X.tc(TF_R6) * u[ISY_];
    fl[7]  = X.tc(TF_R7) * u[ISY_];
    fl[8]  = X.tc(TF_R6) * u[ISYC_];
    fl[9]  = X.tc(TF_R7) * u[ISYC_];
    fl[10] = r10 * u[ISEV_];
    fl[11] = X.tc(TF_R11) * u[ISEV_];
    fl[12] = r12 * u[ISEV_];
    fl[13] = X.tc(TF_R13) * u[ICRI_];
    fl[14] = X.tc(TF_R14) * u[ICRI_];
    kc[S_]    = -fl[0];
    kc[E_]    = fl[0] - fl[1];
    kc[INS_]  = (fl[1] - fl[2]) - fl[3];
    kc[INSC_] = -fl[4] - fl[5];
    kc[ISY_]  = (fl[2] - fl[6]) - fl[7];
    kc[ISYC_] = (fl[4] - fl[8]) - fl[9];
    kc[ISEV_] = (((fl[6] + fl[8]) - fl[10]) - fl[11]) - fl[12];
    kc[ICRI_] = (fl[10] - fl[13]) - fl[14];
    kc[R_]    = ((((fl[3] + fl[5]) + fl[7]) + fl[9]) + fl[11]) + fl[14];
    kc[D_]    = fl[12] + fl[13];
}

// shared memory per lane of the mixed solver: 5 stage derivative vectors and the
// flow increments (15, padded to 16 for the float2 pairs)
constexpr int kOdeSmemPerLane = 5 * kC + 16;
static_assert(kC % 2 == 0 && kF == 15, "pair layout of the stage storage");
constexpr int kMixedThreads   = 128; // largest block of the mixed node kernels
// resident blocks per SM the register budget must allow (measured best for the
// FP32 step; the FP64 step holds its state and clock in FP64 registers)
constexpr int kMixedMinBlocks    = 3;
constexpr int kMixedMinBlocks64  = 2;

// Odeint's error measure of one compartment: |x_err| / (abs + rel (|x| + dt |dxdt|))
__device__ __forceinline__ float err_ratio(float xe, float x, float dxdt, float dt, float abs_tol, float rel_tol)
{
    // (an approximate quotient: the controller needs no correctly rounded ratios)
    return __fdividef(fabsf(xe), abs_tol + rel_tol * (fabsf(x) + dt * fabsf(dxdt)));
}
__device__ __forceinline__ double err_ratio(float xe, double x, float dxdt, double dt, double abs_tol,
                                            double rel_tol)
{
    return fabs((double)xe) / (abs_tol + rel_tol * (fabs(x) + dt * fabs((double)dxdt)));
}

// One exchange interval of every active instance of the list, mixed precision.
// CTL64 = false: the state as float-float pairs (hi + lo) updated with exact
// TwoSum; the error norm, the controller and the interval clock in FP32.
// CTL64 = true : the state accumulated in FP64; the error norm (from the FP32
// error estimate), the controller and the interval clock in FP64.
// In both, the right-hand side and the stage combinations run in FP32 from the
// FP32 rounding of the state.
template <int G, bool CTL64, bool FLOWS>
__global__ void __launch_bounds__(kMixedThreads, CTL64 ? kMixedMinBlocks64 : kMixedMinBlocks)
    k_ode_mixed(BatchDev B, const int32_t* inst, int64_t count)
{
    using Clk         = typename std::conditional<CTL64, double, float>::type;
    constexpr int IPW = 32 / G;
    const int lane    = threadIdx.x & 31;
    const int seg     = lane / G;
    if (seg >= IPW) {
        return;
    }
    SegF<G> X;
    X.gi              = lane - seg * G;
    X.base            = seg * G;
    X.mask            = (((1u << G) - 1u) << X.base);
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw  = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const DevOpts o    = B.opts;
    const Clk abs_tol  = (Clk)o.abs_tol, rel_tol = (Clk)o.rel_tol;
    const Clk o_dt_min = (Clk)o.dt_min; // FP32: DBL_MIN becomes 0, no lower bound, as in FP64
    const Clk o_dt_max = (Clk)o.dt_max; // FP32: DBL_MAX becomes +inf
    // stage derivatives k_0..k_4 as compartment pairs: [warp][stage*5 + pair][lane]
    // float2 (conflict-free 64-bit columns), so that the stage combinations run
    // as FP32x2 multiply-adds (__ffma2_rn: each lane the FFMA of the scalar form)
    extern __shared__ float ode_smem[];
    float* skw = ode_smem + (threadIdx.x >> 5) * ((kOdeSmemPerLane + (FLOWS ? kF : 0)) * 32);
#define SK2(s, p) reinterpret_cast<float2*>(skw)[((s) * (kC / 2) + (p)) * 32 + lane]
#define SK(s, c) skw[(((s) * (kC / 2) + (c) / 2) * 32 + lane) * 2 + ((c) & 1)]
    // the 5th-order flow increments of the attempt as flow pairs, after the stage derivatives
#define SP2(p) reinterpret_cast<float2*>(skw + 5 * kC * 32)[(p) * 32 + lane]
#define SP(f) skw[5 * kC * 32 + (((f) / 2) * 32 + lane) * 2 + ((f) & 1)]
    // (FLOWS) the increments of the interval's applied steps, summed per flow
#define SF(f) skw[(kOdeSmemPerLane + (f)) * 32 + lane]
    unsigned long long n_acc = 0, n_rej = 0, n_fail = 0;

    for (int64_t slot = wid * IPW + seg; slot < count; slot += nw * IPW) {
        const int64_t node = inst[slot];
        const int gidx     = B.node_graph[node];
        const DevGraph& g  = B.graphs[gidx];
        const GraphRt& rt  = B.rt[gidx];
        if (!rt.active) {
            continue;
        }
        const int64_t local = node - g.node0;
        const int64_t so    = g.state_off + local * g.n + X.gi * kC;
        float* yhi          = B.st_hi + so;
        float* ylo          = B.st_lo + so;
        // hi: the FP32 state the stages start from; lo (FP32 step) or y64 (FP64 step) the accumulator
        float hi[kC], lo[kC];
        double y64[CTL64 ? kC : 1];
#pragma unroll
        for (int c = 0; c < kC; c += 2) {
            const float2 h2 = *reinterpret_cast<const float2*>(yhi + c);
            const float2 l2 = *reinterpret_cast<const float2*>(ylo + c);
            hi[c] = h2.x; hi[c + 1] = h2.y; lo[c] = l2.x; lo[c + 1] = l2.y;
        }
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if constexpr (CTL64) {
                y64[c] = (double)hi[c] + (double)lo[c];
            }
        }
        const double t_start = B.node_t[node];
        const double tmax    = rt.t_next;
        segf_load(X, B, g, local, t_start);
        if constexpr (FLOWS) {
#pragma unroll
            for (int f = 0; f < kF; ++f) {
                SF(f) = 0.0f;
            }
        }
        // Return-side values of the pending departure (the exchange's node pass,
        // done here): lambda and the transition rates at the state the travelers
        // left, i.e. at t_dep. That state is this interval's start state unless a
        // horizon split the interval; then it is read back from v0.
        if (rt.do_return && g.E > 0) {
            const bool at_dep = t_start == rt.t_dep;
            float pop[kC];
            if (at_dep) {
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    pop[c] = __fadd_rn(hi[c], lo[c]);
                }
            }
            else {
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    pop[c] = __fadd_rn(B.v0_hi[so + c], B.v0_lo[so + c]);
                }
            }
            float season, acc, r10, r12;
            segf_rates(X, pop, at_dep ? 0.0f : (float)(rt.t_dep - t_start), season, acc, r10, r12);
            float v[kAux];
            v[0]  = X.tc(TF_BETA) * season * acc;
            v[1]  = X.tc(TF_R1);
            v[2]  = X.tc(TF_R2);
            v[3]  = X.tc(TF_R3);
            v[4]  = X.tc(TF_R6);
            v[5]  = X.tc(TF_R7);
            v[6]  = r10;
            v[7]  = X.tc(TF_R11);
            v[8]  = r12;
            v[9]  = X.tc(TF_R13);
            v[10] = X.tc(TF_R14);
            // can one Euler step of length dt drive a returning compartment negative?
            // (it cannot when dt times every compartment's total outflow rate is <= 1;
            // the FP32 test keeps a margin for its own rounding)
            const float out_rate =
                fmaxf(fmaxf(v[0], v[1]), fmaxf(fmaxf(v[2] + v[3], v[4] + v[5]), fmaxf(v[6] + v[7] + v[8], v[9] + v[10])));
            v[11]     = ((float)rt.dt * out_rate > 0.99999f) ? 1.0f : 0.0f;
            float4* a = reinterpret_cast<float4*>(reinterpret_cast<float*>(B.aux) + (node * MGPU_MAX_GROUPS + X.gi) * kAux);
            a[0]      = make_float4(v[0], v[1], v[2], v[3]);
            a[1]      = make_float4(v[4], v[5], v[6], v[7]);
            a[2]      = make_float4(v[8], v[9], v[10], v[11]);
        }

        // SystemIntegrator::advance on an interval-relative clock: tr runs from
        // 0 to span (0.5 days is exact in FP32); a step clipped to the remaining
        // span lands exactly on it.
        const Clk span   = (Clk)(tmax - t_start);
        const Clk eps_t  = (Clk)kZeroTol * span;
        Clk tr           = 0;
        Clk dt           = (Clk)B.node_dt[node];
        Clk dt_restore   = 0;
        Clk dt_min       = o_dt_min;
        int steps        = 0;
        bool cap_hit     = false;
        while (span - tr > eps_t) {
            if (steps++ >= o.max_steps) {
                cap_hit = true;
                break;
            }
            bool last = false;
            if (dt >= span - tr) {
                if (dt > span - tr) {
                    dt_restore = dt;
                }
                dt     = span - tr;
                dt_min = fmin(span - tr, dt_min);
                last   = true;
            }
            // ControlledStepperWrapper::step
            bool success      = false;
            bool is_dt_valid  = true;
            const Clk dt_try0 = dt;
            while (!success && is_dt_valid) {
                if (dt < dt_min) {
                    is_dt_valid = false;
                    dt          = dt_min;
                }
                if (o_dt_max != 0 && fabs(dt) > o_dt_max) {
                    dt = o_dt_max;
                    ++n_rej;
                    continue;
                }
                const float dtf  = (float)dt;
                const float trel = (float)tr;
                float kc[kC], fl[kF];
                // the six stages: one copy of the right-hand side in the code,
                // stage derivatives in this lane's shared-memory column
#pragma unroll 1
                for (int s = 0; s < 6; ++s) {
                    float2 u2[kC / 2];
#pragma unroll
                    for (int q = 0; q < kC / 2; ++q) {
                        u2[q] = make_float2(hi[2 * q], hi[2 * q + 1]);
                    }
#pragma unroll 1
                    for (int j = 0; j < s; ++j) {
                        const float a   = fk_a[s][j] * dtf;
                        const float2 a2 = make_float2(a, a);
#pragma unroll
                        for (int q = 0; q < kC / 2; ++q) {
                            u2[q] = __ffma2_rn(a2, SK2(j, q), u2[q]);
                        }
                    }
                    float u[kC];
#pragma unroll
                    for (int q = 0; q < kC / 2; ++q) {
                        u[2 * q]     = u2[q].x;
                        u[2 * q + 1] = u2[q].y;
                    }
                    segf_rhs(X, u, trel + fk_c[s] * dtf, fl, kc);
                    if (s < 5) {
#pragma unroll
                        for (int q = 0; q < kC / 2; ++q) {
                            SK2(s, q) = make_float2(kc[2 * q], kc[2 * q + 1]);
                        }
                    }
                    const float b5   = fk_b5[s] * dtf;
                    const float2 b52 = make_float2(b5, b5);
                    if (s == 0) {
#pragma unroll
                        for (int q = 0; q < kF / 2; ++q) {
                            SP2(q) = __fmul2_rn(b52, make_float2(fl[2 * q], fl[2 * q + 1]));
                        }
                        SP(kF - 1) = b5 * fl[kF - 1];
                    }
                    else if (b5 != 0.0f) {
#pragma unroll
                        for (int q = 0; q < kF / 2; ++q) {
                            SP2(q) = __ffma2_rn(b52, make_float2(fl[2 * q], fl[2 * q + 1]), SP2(q));
                        }
                        SP(kF - 1) = SP(kF - 1) + b5 * fl[kF - 1];
                    }
                }
                // embedded error: the stage derivatives weighted in stage order
                // (k_0..k_4 from shared memory, k_5 still in registers)
                float2 xe2[kC / 2];
                {
                    const float d0 = fk_db[0] * dtf;
#pragma unroll
                    for (int q = 0; q < kC / 2; ++q) {
                        xe2[q] = __fmul2_rn(make_float2(d0, d0), SK2(0, q));
                    }
                }
#pragma unroll 1
                for (int s = 1; s < 5; ++s) {
                    const float db = fk_db[s] * dtf;
#pragma unroll
                    for (int q = 0; q < kC / 2; ++q) {
                        xe2[q] = __ffma2_rn(make_float2(db, db), SK2(s, q), xe2[q]);
                    }
                }
                {
                    const float db = fk_db[5] * dtf;
#pragma unroll
                    for (int q = 0; q < kC / 2; ++q) {
                        xe2[q] = __ffma2_rn(make_float2(db, db), make_float2(kc[2 * q], kc[2 * q + 1]), xe2[q]);
                    }
                }
                float xe[kC];
#pragma unroll
                for (int q = 0; q < kC / 2; ++q) {
                    xe[2 * q]     = xe2[q].x;
                    xe[2 * q + 1] = xe2[q].y;
                }
                // Odeint error measure, max over the instance
                Clk el = 0;
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    if constexpr (CTL64) {
                        el = fmax(el, err_ratio(xe[c], y64[c], SK(0, c), dt, abs_tol, rel_tol));
                    }
                    else {
                        el = fmaxf(el, err_ratio(xe[c], hi[c], SK(0, c), dtf, abs_tol, rel_tol));
                    }
                }
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    el = fmax(el, __shfl_sync(X.mask, el, X.base + q));
                }
                // controller (Odeint rules)
                if (el > 1) {
                    if constexpr (CTL64) {
                        dt *= fmax(0.9 * pow(el, -1.0 / 3.0), 0.2);
                    }
                    else {
                        dt *= fmaxf(0.9f * exp2f(__log2f(el) * (-1.0f / 3.0f)), 0.2f);
                    }
                    if (o_dt_max != 0) {
                        dt = fmin(dt, o_dt_max);
                    }
                    ++n_rej;
                }
                else {
                    // the step taken with the clipped size reaches the boundary exactly
                    tr = (last && dt == dt_try0) ? span : tr + dt;
                    if (el < (Clk)0.5) {
                        if constexpr (CTL64) {
                            dt *= 0.9 * pow(fmax(0.00032 /* 5^-5 */, el), -1.0 / 5.0);
                        }
                        else {
                            dt *= 0.9f * exp2f(__log2f(fmaxf(0.00032f /* 5^-5 */, el)) * -0.2f);
                        }
                        if (o_dt_max != 0) {
                            dt = fmin(dt, o_dt_max);
                        }
                    }
                    success = true;
                }
            }
            dt = fmax(dt, dt_min);
            if (!success) {
                tr += dt_min;
                ++n_fail;
            }
            else {
                ++n_acc;
            }
            // flow-space update of the (last) attempt: each increment leaves its
            // source and enters its target with the same value
            if constexpr (FLOWS) {
#pragma unroll
                for (int f = 0; f < kF; ++f) {
                    SF(f) = SF(f) + SP(f);
                }
            }
            if constexpr (CTL64) {
#pragma unroll
                for (int f = 0; f < kF; ++f) {
                    const double ph = (double)SP(f);
                    y64[kFlowSrcI(f)] -= ph;
                    y64[kFlowDstI(f)] += ph;
                }
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    hi[c] = (float)y64[c];
                }
            }
            else {
#pragma unroll
                for (int f = 0; f < kF; ++f) {
                    const float ph = SP(f);
                    df_add(hi[kFlowSrcI(f)], lo[kFlowSrcI(f)], -ph);
                    df_add(hi[kFlowDstI(f)], lo[kFlowDstI(f)], ph);
                }
#pragma unroll
                for (int c = 0; c < kC; ++c) {
                    df_renorm(hi[c], lo[c]);
                }
            }
        }
        dt             = fmax(dt, dt_restore);
        bool nonfinite = false;
#pragma unroll
        for (int c = 0; c < kC; ++c) {
            if constexpr (CTL64) {
                lo[c] = (float)(y64[c] - (double)hi[c]);
            }
            yhi[c]    = hi[c];
            ylo[c]    = lo[c];
            nonfinite = nonfinite || !isfinite(hi[c]);
        }
        if (X.gi == 0) {
            B.node_t[node]  = (tr >= span) ? tmax : t_start + (double)tr;
            B.node_dt[node] = (double)dt;
        }
        if constexpr (FLOWS) {
            double* F = B.flows + (so / kC) * kF;
#pragma unroll
            for (int f = 0; f < kF; ++f) {
                F[f] += (double)SF(f);
            }
        }
        report_instance_failure(B, gidx, cap_hit, nonfinite);
        // Departure at the interval's end (the exchange's node pass, done here):
        // the snapshot record, i.e. the FP32 rounding of the state, the ISy mobility
        // factor and the commuter nondetection (get_mobility_factors,
        // models/ode_secir/model.h:687-715), into the free snapshot slot.
        if (rt.do_depart && g.E > 0) {
            const int ws    = rt.snap_slot ^ 1;
            const float tnt = segf_sum(X, X.tc(TF_A_TNT) * hi[INS_]);
            const double t  = rt.t_next;
            float r[kRec];
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                r[rec_pos(c)] = hi[c];
            }
            r[REC_RISK] = smoother_cosine(tnt, X.tc(TF_TNT_CAP), X.tc(TF_TNT_CAP2), X.tc(TF_RHO), X.tc(TF_RHO_MAX));
            r[REC_ND]   = (t >= X.nm.scalar(MGPU_P_START_COMMUTER_DETECTION) &&
                         t < X.nm.scalar(MGPU_P_END_COMMUTER_DETECTION))
                              ? (float)X.nm.scalar(MGPU_P_COMMUTER_NONDETECTION)
                              : 1.0f;
            float* base      = B.gsnap + (int64_t)ws * (B.state_total / kC) * kRec;
            const int64_t r0 = (g.state_off + local * g.n) / kC;
#pragma unroll
            for (int v = 0; v < kRec / 4; ++v) {
                *reinterpret_cast<float4*>(base + rec_vec(r0, G, X.gi, v)) =
                    make_float4(r[4 * v], r[4 * v + 1], r[4 * v + 2], r[4 * v + 3]);
            }
        }
    }
#undef SK
#undef SP
#undef SF
    if (X.gi == 0) {
        if (n_acc) {
            atomicAdd(&B.counters[CNT_ACCEPTED], n_acc);
        }
        if (n_rej) {
            atomicAdd(&B.counters[CNT_REJECTED], n_rej);
        }
        if (n_fail) {
            atomicAdd(&B.counters[CNT_FAILED], n_fail);
        }
    }
}

// Order of the instances with G age groups for the mixed node kernel in this
// interval: a node whose proposed step size covers the whole interval is likely
// done in one step and goes to the front, the others to the back. The segments
// of a warp move in lockstep until the last of them finishes its interval, so
// warps of nodes with similar step counts idle less. (Only the order changes:
// every node is solved by the same code wherever it lands.)
__global__ void k_ode_order(BatchDev B, int G)
{
    const int64_t i   = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n   = B.gcount[G];
    const bool valid  = i < n;
    int32_t node      = 0;
    bool front        = false;
    if (valid) {
        node             = B.glist[G][i];
        const GraphRt rt = B.rt[B.node_graph[node]];
        front            = !rt.active || B.node_dt[node] >= rt.t_next - B.node_t[node];
    }
    const unsigned lanes = __ballot_sync(0xffffffffu, valid);
    const unsigned fm    = __ballot_sync(0xffffffffu, valid && front);
    const unsigned bm    = lanes & ~fm;
    const int lane       = threadIdx.x & 31;
    const int leader     = __ffs(lanes) - 1;
    int fb = 0, bb = 0;
    if (lane == leader) {
        fb = fm ? atomicAdd(B.order_cnt + 2 * G, __popc(fm)) : 0;
        bb = bm ? atomicAdd(B.order_cnt + 2 * G + 1, __popc(bm)) : 0;
    }
    fb                 = __shfl_sync(0xffffffffu, fb, leader < 0 ? 0 : leader);
    bb                 = __shfl_sync(0xffffffffu, bb, leader < 0 ? 0 : leader);
    const unsigned below = (1u << lane) - 1u;
    if (valid) {
        const int64_t pos = front ? (int64_t)fb + __popc(fm & below) : n - 1 - ((int64_t)bb + __popc(bm & below));
        B.gorder[G][pos]  = node;
    }
}

template <int G>
int launch_g(const BatchDev& B, int precision, const int32_t* inst, int64_t count, int ipb, int grid, cudaStream_t s)
{
    constexpr int IPW  = 32 / G;
    const int warps    = ipb > 0 ? (ipb + IPW - 1) / IPW : 4;
    const int threads  = 32 * (warps < 1 ? 1 : (warps > 4 ? 4 : warps)); // launch bounds: 128 threads
    const int64_t per  = (int64_t)(threads / 32) * IPW;
    int64_t blocks     = (count + per - 1) / per;
    if (grid > 0 && blocks > grid) {
        blocks = grid;
    }
    if (blocks < 1) {
        blocks = 1;
    }
    const bool flows = B.flows != nullptr;
    if (is_mixed(precision)) {
        const size_t smem = (size_t)(threads / 32) * (kOdeSmemPerLane + (flows ? kF : 0)) * 32 * sizeof(float);
        if (B.gorder[G] && inst == B.glist[G] && count == B.gcount[G]) {
            k_ode_order<<<(unsigned)((count + 127) / 128), 128, 0, s>>>(B, G);
            inst = B.gorder[G];
        }
        const bool ctl64 = precision == MGPU_PRECISION_MIXED_FP64_CONTROL;
        if (ctl64 && flows) {
            k_ode_mixed<G, true, true><<<(unsigned)blocks, threads, smem, s>>>(B, inst, count);
        }
        else if (ctl64) {
            k_ode_mixed<G, true, false><<<(unsigned)blocks, threads, smem, s>>>(B, inst, count);
        }
        else if (flows) {
            k_ode_mixed<G, false, true><<<(unsigned)blocks, threads, smem, s>>>(B, inst, count);
        }
        else {
            k_ode_mixed<G, false, false><<<(unsigned)blocks, threads, smem, s>>>(B, inst, count);
        }
    }
    else if (flows) {
        k_ode_batched<G, true><<<(unsigned)blocks, threads, 0, s>>>(B, inst, count);
    }
    else {
        k_ode_batched<G, false><<<(unsigned)blocks, threads, 0, s>>>(B, inst, count);
    }
    return 0;
}

} // namespace

int launch_ode_batched(const BatchDev& B, int G, int precision, const int32_t* d_instances, int64_t count,
                       int instances_per_block, int grid_blocks, cudaStream_t s)
{
    if (count <= 0) {
        return 0;
    }
    switch (G) {
    case 1: return launch_g<1>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 2: return launch_g<2>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 3: return launch_g<3>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 4: return launch_g<4>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 5: return launch_g<5>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 6: return launch_g<6>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 7: return launch_g<7>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    case 8: return launch_g<8>(B, precision, d_instances, count, instances_per_block, grid_blocks, s);
    default: return -1;
    }
}

} // namespace mgpu
