// secir_oracle.cpp — TEST INFRASTRUCTURE (checker and CPU baseline only).
//
// FP64 CPU restatement of the MEmilio graph-ODE SECIR path. It keeps the
// reference's algorithm and loop structure: the contact matrix, the risk
// smoother and the seasonality are evaluated per (i, j) inside get_flows,
// every integrator step goes through the same controller sequence, and the
// graph simulation runs a serial node loop followed by a serial edge loop.
// Each function cites the reference file:line it restates.
//
// Cash-Karp 5(4) inside Boost.Odeint's controlled_runge_kutta (Boost 1.84.0,
// pinned at cpp/thirdparty/CMakeLists.txt:5, not vendored) is restated from
// the published method (Cash & Karp, ACM TOMS 16:201-222, 1990) and from
// Odeint's documented controller rules:
//   err = max_i |xerr_i| / (eps_abs + eps_rel * (|x_i| + dt * |dxdt_i|))
//   err > 1  : reject, dt *= max(0.9 * err^(-1/(q_err - 1)), 0.2), q_err = 4
//   err < 0.5: accept and grow, dt *= 0.9 * max(err, 5^-q)^(-1/q), q = 5
//   otherwise: accept, keep dt;  |dt| > dt_max: reject with dt = dt_max.
// Its parity is pinned by the reference's Cash-Karp golden files.

#include "secir_oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <tuple>
#include <vector>

namespace
{

constexpr double kPi       = 3.14159265358979323846; // std::numbers::pi_v<double>
constexpr double kZeroTol  = 1e-12;                  // Limits<double>::zero_tolerance, config.h:73-79
constexpr int kC           = MGPU_NUM_COMPARTMENTS;
constexpr int kF           = MGPU_NUM_FLOWS;

// Source and target compartment of the 15 flows, in the order of the
// osecir Flows typelist (models/ode_secir/model.h:45-59).
constexpr int kFlowSrc[kF] = {MGPU_S,    MGPU_E,    MGPU_INS,  MGPU_INS,  MGPU_INSC,
                              MGPU_INSC, MGPU_ISY,  MGPU_ISY,  MGPU_ISYC, MGPU_ISYC,
                              MGPU_ISEV, MGPU_ISEV, MGPU_ISEV, MGPU_ICRI, MGPU_ICRI};
constexpr int kFlowDst[kF] = {MGPU_E,    MGPU_INS,  MGPU_ISY,  MGPU_R,    MGPU_ISYC,
                              MGPU_R,    MGPU_ISEV, MGPU_R,    MGPU_ISEV, MGPU_R,
                              MGPU_ICRI, MGPU_R,    MGPU_D,    MGPU_D,    MGPU_R};

struct NodeView {
    int G, M, K;
    const double* p;
    const double* base;   // [M][G][G]
    const double* mini;   // [M][G][G] (may be null: zeros)
    const double* dtimes; // [M][K]
    const double* dvals;  // [M][K][G][G]
    double scalar(int which) const
    {
        return p[which];
    }
    double gp(int which, int g) const
    {
        return p[MGPU_NUM_SCALAR_PARAMS + which * G + g];
    }
};

NodeView node_view(const mgpu_graph* g, int v)
{
    NodeView nv;
    nv.G               = g->num_groups;
    nv.M               = g->num_contact_matrices;
    nv.K               = g->num_damping_points;
    const long GG      = (long)nv.G * nv.G;
    nv.p               = g->params + (long)v * MGPU_PARAM_STRIDE(nv.G);
    nv.base            = g->contact_baseline + (long)v * nv.M * GG;
    nv.mini            = g->contact_minimum ? g->contact_minimum + (long)v * nv.M * GG : nullptr;
    nv.dtimes          = nv.K ? g->damping_times + (long)v * nv.M * nv.K : nullptr;
    nv.dvals           = nv.K ? g->damping_values + (long)v * nv.M * nv.K * GG : nullptr;
    return nv;
}

// smoother_cosine (memilio/math/smoother.h:46-60).
inline double smoother_cosine(double x, double xleft, double xright, double yleft, double yright)
{
    if (x <= xleft) {
        return yleft;
    }
    if (x >= xright) {
        return yright;
    }
    return 0.5 * (yleft - yright) * std::cos(kPi / (xright - xleft) * (x - xleft)) + 0.5 * (yleft + yright);
}

// One coefficient of Dampings::get_matrix_at(t) (damping.h:381-396): the
// upper bound in the cached time line, then a cosine ramp over the day
// before the next cached time.
inline double damping_coeff_at(const double* times, const double* vals, int K, long stride, long idx, double t)
{
    if (K == 0) {
        return 0.0;
    }
    int ub = (int)(std::upper_bound(times, times + K, t) - times);
    if (ub >= K) {
        ub = K - 1; // t >= DBL_MAX; unreachable for finite t
    }
    return smoother_cosine(t, times[ub] - 1.0, times[ub], vals[(long)(ub - 1) * stride + idx],
                           vals[(long)ub * stride + idx]);
}

// Element (i, j) of ContactMatrixGroup::get_matrix_at(t)
// (contact_matrix.h:392-399 summing DampingMatrixExpression::get_matrix_at,
// contact_matrix.h:190-194: B - D(t) o (B - Min)).
inline double contact_at(const NodeView& nv, double t, int i, int j)
{
    const long GG = (long)nv.G * nv.G;
    double s      = 0.0;
    for (int m = 0; m < nv.M; ++m) {
        const long idx = (long)i * nv.G + j;
        const double B = nv.base[m * GG + idx];
        const double L = nv.mini ? nv.mini[m * GG + idx] : 0.0;
        const double D =
            nv.K ? damping_coeff_at(nv.dtimes + (long)m * nv.K, nv.dvals + (long)m * nv.K * GG, nv.K, GG, idx, t)
                 : 0.0;
        s = s + (B - D * (B - L));
    }
    return s;
}

// osecir::Model::get_flows (models/ode_secir/model.h:82-214). `flows` must be zero on entry
// (FlowModel::get_derivatives zeroes its flow cache first, flow_model.h:141).
void get_flows(const NodeView& nv, const double* pop, const double* y, double t, double* flows)
{
    const int G          = nv.G;
    double icu_occupancy = 0.0;
    double tnt_required  = 0.0;
    for (int i = 0; i < G; ++i) {
        tnt_required += (1 - nv.gp(MGPU_G_RECOVERED_PER_INS, i)) / nv.gp(MGPU_G_TIME_INS, i) * pop[i * kC + MGPU_INS];
        icu_occupancy += pop[i * kC + MGPU_ICRI];
    }
    const double tnt_cap  = nv.scalar(MGPU_P_TNT_CAPACITY);
    const double tnt_risk = nv.scalar(MGPU_P_TNT_MAX_RISK);
    const double icu_cap  = nv.scalar(MGPU_P_ICU_CAPACITY);
    for (int i = 0; i < G; ++i) {
        const int Si = i * kC + MGPU_S;
        for (int j = 0; j < G; ++j) {
            const int o = j * kC;
            const double risk =
                smoother_cosine(tnt_required, tnt_cap, tnt_cap * tnt_risk, nv.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, j),
                                nv.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, j));
            const double season_val =
                (1 + nv.scalar(MGPU_P_SEASONALITY) *
                         std::sin(kPi * ((nv.scalar(MGPU_P_START_DAY) + t) / 182.5 + 0.5)));
            const double cont_freq_eff = season_val * contact_at(nv, t, i, j);
            const double Nj = pop[o + MGPU_S] + pop[o + MGPU_E] + pop[o + MGPU_INS] + pop[o + MGPU_ISY] +
                              pop[o + MGPU_ISEV] + pop[o + MGPU_ICRI] + pop[o + MGPU_R];
            const double divNj   = (Nj < kZeroTol) ? 0.0 : 1.0 / Nj;
            const double dummy_S = y[Si] * cont_freq_eff * divNj * nv.gp(MGPU_G_TRANSMISSION_PROB, i) *
                                   (nv.gp(MGPU_G_REL_TRANSMISSION_NS, j) * pop[o + MGPU_INS] + risk * pop[o + MGPU_ISY]);
            flows[i * kF + 0] += dummy_S;
        }
        const double cps      = nv.gp(MGPU_G_CRITICAL_PER_SEVERE, i);
        const double crit_adj = smoother_cosine(icu_occupancy, 0.90 * icu_cap, icu_cap, cps, 0.0);
        const double deaths_adj = cps - crit_adj;
        const double mu         = nv.gp(MGPU_G_RECOVERED_PER_INS, i);
        const double tins       = nv.gp(MGPU_G_TIME_INS, i);
        const double sev        = nv.gp(MGPU_G_SEVERE_PER_ISY, i);
        const double tisy       = nv.gp(MGPU_G_TIME_ISY, i);
        const double tisev      = nv.gp(MGPU_G_TIME_ISEV, i);
        const double dps        = nv.gp(MGPU_G_DEATHS_PER_SEVERE, i);
        const double dpc        = nv.gp(MGPU_G_DEATHS_PER_CRITICAL, i);
        const double ticri      = nv.gp(MGPU_G_TIME_ICRI, i);
        const double* yi        = y + i * kC;
        double* f               = flows + i * kF;
        f[1]  = (1.0 / nv.gp(MGPU_G_TIME_EXPOSED, i)) * yi[MGPU_E];
        f[2]  = (1 - mu) * (1 / tins) * yi[MGPU_INS];
        f[3]  = mu * (1.0 / tins) * yi[MGPU_INS];
        f[4]  = (1.0 - mu) * (1.0 / tins) * yi[MGPU_INSC];
        f[5]  = mu * (1.0 / tins) * yi[MGPU_INSC];
        f[6]  = sev / tisy * yi[MGPU_ISY];
        f[7]  = (1 - sev) / tisy * yi[MGPU_ISY];
        f[8]  = sev / tisy * yi[MGPU_ISYC];
        f[9]  = (1.0 - sev) / tisy * yi[MGPU_ISYC];
        f[10] = crit_adj / tisev * yi[MGPU_ISEV];
        f[11] = (1.0 - cps - dps) / tisev * yi[MGPU_ISEV];
        f[12] = (dps + deaths_adj) / tisev * yi[MGPU_ISEV];
        f[13] = dpc / ticri * yi[MGPU_ICRI];
        f[14] = (1.0 - dpc) / ticri * yi[MGPU_ICRI];
    }
}

// FlowModel::get_derivatives(pop, y, t, dydt) (flow_model.h:138-144) with
// get_derivatives(flows, dydt) / get_rhs_impl (flow_model.h:112-125,219-235).
struct Rhs {
    NodeView nv;
    mutable std::vector<double> flows;
    mutable int64_t evals = 0;
    explicit Rhs(const NodeView& v)
        : nv(v)
        , flows((size_t)v.G * kF)
    {
    }
    void operator()(const double* pop, const double* y, double t, double* dydt) const
    {
        ++evals;
        const int n = nv.G * kC;
        std::fill(flows.begin(), flows.end(), 0.0);
        get_flows(nv, pop, y, t, flows.data());
        std::fill(dydt, dydt + n, 0.0);
        for (int g = 0; g < nv.G; ++g) {
            for (int k = 0; k < kF; ++k) {
                const double fv = flows[g * kF + k];
                dydt[g * kC + kFlowSrc[k]] -= fv;
                dydt[g * kC + kFlowDst[k]] += fv;
            }
        }
    }
};

// Cash-Karp 5(4) tableau (Cash & Karp 1990, Table 5).
constexpr double ck_c[6]    = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
constexpr double ck_a[6][5] = {{0, 0, 0, 0, 0},
                               {1.0 / 5.0, 0, 0, 0, 0},
                               {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
                               {3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0, 0, 0},
                               {-11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0, 0},
                               {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
constexpr double ck_b5[6]   = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
constexpr double ck_b4[6]   = {2825.0 / 27648.0, 0.0, 18575.0 / 48384.0, 13525.0 / 55296.0, 277.0 / 14336.0, 1.0 / 4.0};

// Runge-Kutta-Fehlberg 4(5) tableau as MEmilio's RKIntegratorCore uses it (math/adapt_rk.h:47-138).
constexpr double rkf_c[6]    = {0.0, 0.25, 3.0 / 8.0, 12.0 / 13.0, 1.0, 0.5};
constexpr double rkf_a[6][5] = {{0, 0, 0, 0, 0},
                                {0.25, 0, 0, 0, 0},
                                {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0},
                                {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0},
                                {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0},
                                {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0}};
constexpr double rkf_low[6]  = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -0.2, 0.0};
constexpr double rkf_high[6] = {16.0 / 135.0, 0.0, 6656.0 / 12825.0, 28561.0 / 56430.0, -9.0 / 50.0, 2.0 / 55.0};

struct Counters {
    int64_t accepted = 0, rejected = 0, failed = 0;
};

// An integrator core with the reference's dt bounds (IntegratorCore, math/integrator.h:46-129).
struct Core {
    int method;
    double abs_tol, rel_tol, dt_min, dt_max;
    int n;
    mutable std::vector<double> k[6], xt, xerr;
    Counters* cnt;

    Core(const mgpu_integrator_opts& o, int n_, Counters* c)
        : method(o.method)
        , abs_tol(o.abs_tol)
        , rel_tol(o.rel_tol)
        , dt_min(o.dt_min)
        , dt_max(o.dt_max)
        , n(n_)
        , xt(n_)
        , xerr(n_)
        , cnt(c)
    {
        for (auto& v : k) {
            v.resize(n_);
        }
    }

    // One Cash-Karp attempt with error estimate (odeint explicit_error_generic_rk::do_step
    // called from controlled_runge_kutta::try_step, stepper_wrapper.h:141-146).
    // Returns the Odeint error measure.
    template <class F>
    double ck_attempt(const F& f, const double* x, double t, double dt, double* out) const
    {
        f(x, x, t, k[0].data()); // try_step(sys, in, t, out, dt) evaluates dxdt(in, t) first
        for (int s = 1; s < 6; ++s) {
            for (int i = 0; i < n; ++i) {
                double v = x[i];
                for (int j = 0; j < s; ++j) {
                    v = v + (ck_a[s][j] * dt) * k[j][i];
                }
                xt[i] = v;
            }
            f(xt.data(), xt.data(), t + ck_c[s] * dt, k[s].data());
        }
        double err = 0.0;
        for (int i = 0; i < n; ++i) {
            double v = x[i];
            double e = 0.0;
            for (int j = 0; j < 6; ++j) {
                v = v + (ck_b5[j] * dt) * k[j][i];
            }
            for (int j = 0; j < 6; ++j) {
                e = e + ((ck_b5[j] - ck_b4[j]) * dt) * k[j][i];
            }
            out[i]  = v;
            double r = std::fabs(e) / (abs_tol + rel_tol * (std::fabs(x[i]) + dt * std::fabs(k[0][i])));
            err      = std::max(err, r);
        }
        return err;
    }

    // ControlledStepperWrapper::step (stepper_wrapper.h:112-163) around Odeint's try_step.
    template <class F>
    bool ck_step(const F& f, const double* yt, double& t, double& dt, double* ytp1) const
    {
        bool success     = false;
        bool is_dt_valid = true;
        while (!success && is_dt_valid) {
            if (dt < dt_min) {
                is_dt_valid = false;
                dt          = dt_min;
            }
            if (dt_max != 0.0 && std::fabs(dt) > dt_max) {
                // step size above limit: reject and set dt = dt_max (after evaluating dxdt, as try_step does)
                f(yt, yt, t, k[0].data());
                dt = dt_max;
                cnt->rejected++;
                continue;
            }
            const double err = ck_attempt(f, yt, t, dt, ytp1);
            if (err > 1.0) {
                dt *= std::max(0.9 * std::pow(err, -1.0 / 3.0), 0.2);
                if (dt_max != 0.0) {
                    dt = std::min(dt, dt_max);
                }
                cnt->rejected++;
            }
            else {
                t += dt;
                if (err < 0.5) {
                    const double e = std::max(std::pow(5.0, -5.0), err);
                    dt *= 0.9 * std::pow(e, -1.0 / 5.0);
                    if (dt_max != 0.0) {
                        dt = std::min(dt, dt_max);
                    }
                }
                success = true;
            }
        }
        dt = std::max(dt, dt_min);
        if (!success) {
            t += dt_min;
            cnt->failed++;
            return false;
        }
        cnt->accepted++;
        return true;
    }

    // RKIntegratorCore::step (math/adapt_rk.h:217-298), Fehlberg 4(5), lower order propagated.
    template <class F>
    bool rkf_step(const F& f, const double* yt, double& t, double& dt, double* ytp1) const
    {
        dt                 = std::min(dt, dt_max);
        bool converged     = false;
        bool dt_is_invalid = false;
        std::vector<double> yt_eval(yt, yt + n);
        while (!converged && !dt_is_invalid) {
            if (dt < dt_min) {
                dt_is_invalid = true;
                dt            = dt_min;
            }
            f(yt_eval.data(), yt_eval.data(), t, k[0].data());
            for (int s = 1; s < 6; ++s) {
                double t_eval = t;
                t_eval += rkf_c[s] * dt;
                for (int i = 0; i < n; ++i) {
                    double v = yt_eval[i];
                    for (int j = 0; j < s; ++j) {
                        v += (dt * rkf_a[s][j]) * k[j][i];
                    }
                    ytp1[i] = v;
                }
                f(ytp1, ytp1, t_eval, k[s].data());
            }
            double minratio = std::numeric_limits<double>::infinity();
            converged       = true;
            for (int i = 0; i < n; ++i) {
                double lo = 0.0, d = 0.0;
                for (int j = 0; j < 6; ++j) {
                    lo += k[j][i] * rkf_low[j];
                    d += k[j][i] * (rkf_high[j] - rkf_low[j]);
                }
                ytp1[i]          = yt_eval[i] + dt * lo;
                const double est = dt * std::fabs(d);
                const double eps = abs_tol + std::fabs(ytp1[i]) * rel_tol;
                converged        = converged && (est <= eps);
                minratio         = std::min(minratio, eps / est);
            }
            if (converged || dt_is_invalid) {
                t += dt;
            }
            else {
                cnt->rejected++;
            }
            double dt_new = dt * std::pow(minratio, 1.0 / 5.0);
            dt_new *= 0.9;
            dt = std::min(dt_new, dt_max);
        }
        dt = std::max(dt, dt_min);
        if (converged) {
            cnt->accepted++;
        }
        else {
            cnt->failed++;
        }
        return converged;
    }

    template <class F>
    bool step(const F& f, const double* yt, double& t, double& dt, double* ytp1) const
    {
        return method == MGPU_METHOD_RKF45 ? rkf_step(f, yt, t, dt, ytp1) : ck_step(f, yt, t, dt, ytp1);
    }
};

// SystemIntegrator::advance (math/integrator.h:184-249). `y` holds the
// value at t on entry and at the end time on exit; `rec` (optional) is
// called with (t, y) after every step (TimeSeries::add_time_point).
template <class F, class Rec>
void system_advance(Core& core, const F& f, double tmax, double& t, double& dt, std::vector<double>& y, Rec rec)
{
    const double t0 = t;
    const double eps = kZeroTol;
    double dt_restore     = 0.0;
    double dt_min_restore = core.dt_min;
    std::vector<double> ynext(y.size());
    while (std::fabs((tmax - t) / (tmax - t0)) > eps) {
        if (dt > tmax - t) {
            dt_restore  = dt;
            dt          = tmax - t;
            core.dt_min = std::min(tmax - t, core.dt_min);
        }
        core.step(f, y.data(), t, dt, ynext.data());
        y.swap(ynext);
        rec(t, y);
    }
    core.dt_min = dt_min_restore;
    dt          = std::max(dt, dt_restore);
}

// ---- graph simulation -----------------------------------------------------

struct NodeState {
    std::vector<double> y;          // result last value (mutated by the edge loop)
    std::vector<double> last_state; // SimulationNode::m_last_state
    double t  = 0.0;
    double dt = 0.1;
    std::vector<double> snap_t;               // exchange-boundary times
    std::vector<std::vector<double>> snap_y;  // post-exchange values at those times
};

struct EdgeState {
    bool return_mobile = false; // MobilityEdge::m_return_mobile_population
    std::vector<double> trav_t, ret_t;
    std::vector<std::vector<double>> trav;
};

// Mobility coefficient vector of edge e at time t (DampingMatrixExpression over VectorDampings).
void edge_coeffs_at(const mgpu_graph* g, int e, double t, double* c)
{
    const int n  = g->num_groups * kC;
    const int Ke = g->num_edge_damping_points;
    const double* B = g->edge_coeff_baseline + (long)e * n;
    const double* L = g->edge_coeff_minimum ? g->edge_coeff_minimum + (long)e * n : nullptr;
    for (int i = 0; i < n; ++i) {
        double D = 0.0;
        if (Ke) {
            D = damping_coeff_at(g->edge_damping_times + (long)e * Ke, g->edge_damping_values + (long)e * Ke * n, Ke,
                                 n, i, t);
        }
        const double Li = L ? L[i] : 0.0;
        c[i]            = 0.0 + (B[i] - D * (B[i] - Li));
    }
}

// floating_point_equal (math/floating_point.h:56-62).
bool fp_equal(double v1, double v2, double abs_tol, double rel_tol)
{
    const double diff = std::fabs(v1 - v2);
    return diff <= abs_tol || diff <= std::max(std::fabs(v1), std::fabs(v2)) * rel_tol;
}

struct GraphRun {
    const mgpu_graph* g;
    int n;
    mgpu_integrator_opts opts;
    std::vector<NodeView> views;
    std::vector<NodeState> nodes;
    std::vector<EdgeState> edges;
    Counters cnt;
    int64_t rhs_evals = 0, underflow_fixes = 0;
    // MobilityEdge::m_saved_compartment_indices (metapopulation_mobility_instant.h:427) and
    // m_mobility_results, the same sets on every edge; empty: nothing is recorded
    std::vector<std::vector<int>> save_sets;
    std::vector<std::vector<double>> result_t, result_v; // per edge: times, [points][sets + 1]

    // MobilityEdge::add_mobility_result_time_point (metapopulation_mobility_instant.h:423-447):
    // the travelers' sums over each set of indices, then over all compartments.
    void add_mobility_result_time_point(int e, double t, const std::vector<double>& m)
    {
        if (save_sets.empty()) {
            return;
        }
        result_t[e].push_back(t);
        for (const auto& set : save_sets) {
            double sum = 0.0;
            for (int index : set) {
                sum += m[index];
            }
            result_v[e].push_back(sum);
        }
        double total = 0.0;
        for (int j = 0; j < n; ++j) {
            total += m[j];
        }
        result_v[e].push_back(total);
    }

    GraphRun(const mgpu_graph* g_, double t0, double dt0, const mgpu_integrator_opts& o)
        : g(g_)
        , n(g_->num_groups * kC)
        , opts(o)
    {
        nodes.resize(g->num_nodes);
        views.resize(g->num_nodes);
        for (int v = 0; v < g->num_nodes; ++v) {
            views[v] = node_view(g, v);
            auto& ns = nodes[v];
            ns.y.assign(g->init_state + (long)v * n, g->init_state + (long)(v + 1) * n);
            ns.last_state = ns.y;
            ns.t          = t0;
            ns.dt         = dt0;
        }
        edges.resize(g->num_edges);
    }

    // SimulationNode::advance (metapopulation_mobility_instant.h:91-95) -> osecir::Simulation::advance
    // -> Simulation::advance (compartments/simulation.h:66-73): pop == y.
    void advance_node(int v, double tmax)
    {
        Rhs rhs(views[v]);
        Core core(opts, n, &cnt);
        auto f = [&](const double* pop, const double* y, double t, double* dydt) {
            rhs(pop, y, t, dydt);
        };
        auto& ns = nodes[v];
        system_advance(core, f, tmax, ns.t, ns.dt, ns.y, [](double, const std::vector<double>&) {});
        ns.last_state = ns.y;
        rhs_evals += rhs.evals;
    }

    const std::vector<double>* find_snapshot(int v, double t_search) const
    {
        const auto& ns = nodes[v];
        for (long i = (long)ns.snap_t.size() - 1; i >= 0; --i) {
            if (fp_equal(ns.snap_t[i], t_search, 1e-10, 1e-10)) {
                return &ns.snap_y[i];
            }
        }
        return nullptr;
    }

    // MobilityEdge::apply_mobility (metapopulation_mobility_instant.h:544-623).
    void apply_mobility(int e, double t, double dt)
    {
        const int u = g->edge_src[e];
        const int v = g->edge_dst[e];
        auto& es    = edges[e];
        auto& from  = nodes[u];
        auto& to    = nodes[v];
        const int G = g->num_groups;
        if (enpis) {
            check_edge_npis(e, t);
        }
        // returns (:568-603)
        for (long i = (long)es.ret_t.size() - 1; i >= 0; --i) {
            if (es.ret_t[i] <= t) {
                const std::vector<double>* v0 = find_snapshot(v, es.trav_t[i]);
                std::vector<double>& m        = es.trav[i];
                // calculate_mobility_returns (:460-471): one explicit Euler step of the
                // destination model, EulerIntegratorCore::step (math/euler.h:54-62).
                Rhs rhs(views[v]);
                std::vector<double> dydt(n);
                rhs(v0 ? v0->data() : to.y.data(), m.data(), es.trav_t[i], dydt.data());
                rhs_evals += rhs.evals;
                for (int j = 0; j < n; ++j) {
                    m[j] = m[j] + dt * dydt[j];
                }
                // underflow fix (:576-596)
                std::vector<double> remaining(n);
                for (int j = 0; j < n; ++j) {
                    remaining[j] = to.y[j] - m[j];
                }
                for (int j = 0; j < n; ++j) {
                    if (remaining[j] < 0) {
                        const int group = j / kC;
                        int max_index   = 0;
                        for (int c = 1; c < kC; ++c) {
                            if (remaining[group * kC + c] > remaining[group * kC + max_index]) {
                                max_index = c;
                            }
                        }
                        max_index += group * kC;
                        m[max_index] -= remaining[j];
                        m[j] += remaining[j];
                        ++underflow_fixes;
                    }
                }
                for (int j = 0; j < n; ++j) {
                    from.y[j] += m[j];
                }
                for (int j = 0; j < n; ++j) {
                    to.y[j] -= m[j];
                }
                add_mobility_result_time_point(e, t, m);
                es.trav.erase(es.trav.begin() + i);
                es.trav_t.erase(es.trav_t.begin() + i);
                es.ret_t.erase(es.ret_t.begin() + i);
            }
        }
        // departure (:605-621)
        if (!es.return_mobile) {
            std::vector<double> c(n);
            if (enpis) {
                edge_coeffs_npi(e, t, c.data());
            }
            else {
                edge_coeffs_at(g, e, t, c.data());
            }
            bool any = false;
            for (int j = 0; j < n; ++j) {
                any = any || (c[j] > 0.0);
            }
            if (any) {
                const NodeView& nv = views[u];
                const double* y    = from.last_state.data();
                // get_mobility_factors (models/ode_secir/model.h:687-715)
                double tnt = 0.0;
                for (int i = 0; i < G; ++i) {
                    tnt += (1 - nv.gp(MGPU_G_RECOVERED_PER_INS, i)) / nv.gp(MGPU_G_TIME_INS, i) * y[i * kC + MGPU_INS];
                }
                const double cap = nv.scalar(MGPU_P_TNT_CAPACITY);
                std::vector<double> m(n);
                for (int j = 0; j < n; ++j) {
                    double factor = 1.0;
                    if (j % kC == MGPU_ISY) {
                        const int gi = j / kC;
                        factor       = smoother_cosine(tnt, cap, cap * nv.scalar(MGPU_P_TNT_MAX_RISK),
                                                       nv.gp(MGPU_G_RISK_FROM_SYMPTOMATIC, gi),
                                                       nv.gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC, gi));
                    }
                    m[j] = y[j] * c[j] * factor;
                }
                // test_commuters (models/ode_secir/model.h:717-742)
                double nondetection = 1.0;
                if (t >= nv.scalar(MGPU_P_START_COMMUTER_DETECTION) && t < nv.scalar(MGPU_P_END_COMMUTER_DETECTION)) {
                    nondetection = nv.scalar(MGPU_P_COMMUTER_NONDETECTION);
                }
                for (int i = 0; i < G; ++i) {
                    const int INSi = i * kC + MGPU_INS, INSCi = i * kC + MGPU_INSC;
                    const int ISyi = i * kC + MGPU_ISY, ISyCi = i * kC + MGPU_ISYC;
                    from.y[INSi] -= m[INSi] * (1 - nondetection);
                    from.y[INSCi] += m[INSi] * (1 - nondetection);
                    from.y[ISyi] -= m[ISyi] * (1 - nondetection);
                    from.y[ISyCi] += m[ISyi] * (1 - nondetection);
                    m[ISyi] *= nondetection;
                    m[INSi] *= nondetection;
                }
                for (int j = 0; j < n; ++j) {
                    to.y[j] += m[j];
                }
                for (int j = 0; j < n; ++j) {
                    from.y[j] -= m[j];
                }
                add_mobility_result_time_point(e, t, m);
                es.trav.push_back(std::move(m));
                es.trav_t.push_back(t);
                es.ret_t.push_back(t + dt);
            }
        }
        es.return_mobile = !es.return_mobile;
    }

    // ---- dynamic NPIs (models/ode_secir/model.h:289-367, epidemiology/dynamic_npis.h) ----
    struct ODamping {
        double time;
        int level, type;
        std::vector<double> m; // G x G
    };
    struct NpiNode {
        std::vector<std::vector<ODamping>> lists; // per contact matrix, sorted by (time, type, level)
        std::vector<double> ctimes, cvals;        // the node's damping caches [M][K], [M][K][G][G]
        double thr   = std::numeric_limits<double>::lowest(); // m_dynamic_npi
        double t_end = 0.0;
        double total = 0.0; // the model's total population (populations.get_total())
        int count    = 0;
    };
    const orc_dynamic_npis* npis = nullptr;
    std::vector<int> thr_order; // thresholds in descending order
    std::vector<NpiNode> npi;

    // floating_point_greater_equal (math/floating_point.h:136-139), rel_tol = DBL_MIN
    static bool fp_ge(double v1, double v2, double abs_tol)
    {
        return !(v1 - v2 < -(abs_tol + std::numeric_limits<double>::min() * std::max(std::fabs(v1), std::fabs(v2))));
    }

    // Dampings::add_ (damping.h:603-614): sorted by (time, type, level), an equal key replaced
    static void add_damping(std::vector<ODamping>& l, const ODamping& d)
    {
        auto key = [](const ODamping& x) {
            return std::make_tuple(x.time, x.type, x.level);
        };
        auto it = std::lower_bound(l.begin(), l.end(), d, [&](const ODamping& a, const ODamping& b) {
            return key(a) < key(b);
        });
        if (it != l.end() && key(*it) == key(d)) {
            *it = d;
        }
        else {
            l.insert(it, d);
        }
    }

    void init_npis(const orc_dynamic_npis* p, int num_dampings, const orc_damping* dampings)
    {
        npis           = p;
        const int G    = g->num_groups;
        const int M    = g->num_contact_matrices;
        thr_order.resize(p->num_thresholds);
        for (int k = 0; k < p->num_thresholds; ++k) {
            thr_order[k] = k;
        }
        std::stable_sort(thr_order.begin(), thr_order.end(), [&](int a, int b) {
            return p->thresholds[a] > p->thresholds[b];
        });
        npi.resize(g->num_nodes);
        for (int v = 0; v < g->num_nodes; ++v) {
            auto& nn = npi[v];
            nn.lists.assign(M, {});
            for (int d = 0; d < num_dampings; ++d) {
                const orc_damping& x = dampings[d];
                add_damping(nn.lists[x.matrix],
                            {x.time, x.level, x.type, std::vector<double>(x.coeffs, x.coeffs + (long)G * G)});
            }
            for (int j = 0; j < n; ++j) {
                nn.total += g->init_state[(long)v * n + j];
            }
            rebuild_cache(v);
        }
    }

    // Dampings::update_cache for every contact matrix of node v, padded to one K
    void rebuild_cache(int v)
    {
        auto& nn      = npi[v];
        const int G   = g->num_groups;
        const int M   = g->num_contact_matrices;
        const long GG = (long)G * G;
        std::vector<std::vector<double>> ts(M), vs(M);
        int K = 0;
        for (int m = 0; m < M; ++m) {
            const auto& l = nn.lists[m];
            const int nd  = (int)l.size();
            std::vector<double> times(nd), mats((size_t)nd * GG);
            std::vector<int32_t> levels(nd), types(nd);
            for (int d = 0; d < nd; ++d) {
                times[d]  = l[d].time;
                levels[d] = l[d].level;
                types[d]  = l[d].type;
                std::copy(l[d].m.begin(), l[d].m.end(), mats.begin() + (long)d * GG);
            }
            ts[m].resize(nd + 2);
            vs[m].resize((size_t)(nd + 2) * GG);
            const int k = orc_damping_cache(G, G, nd, times.data(), levels.data(), types.data(), mats.data(), nd + 2,
                                            ts[m].data(), vs[m].data());
            ts[m].resize(k);
            vs[m].resize((size_t)k * GG);
            K = std::max(K, k);
        }
        nn.ctimes.clear();
        nn.cvals.clear();
        for (int m = 0; m < M; ++m) {
            while ((int)ts[m].size() < K) {
                ts[m].push_back(std::numeric_limits<double>::max());
                vs[m].insert(vs[m].end(), vs[m].end() - GG, vs[m].end());
            }
            nn.ctimes.insert(nn.ctimes.end(), ts[m].begin(), ts[m].end());
            nn.cvals.insert(nn.cvals.end(), vs[m].begin(), vs[m].end());
        }
        views[v].K      = K;
        views[v].dtimes = nn.ctimes.data();
        views[v].dvals  = nn.cvals.data();
    }

    // make_contact_damping_matrix (damping_sampling.h:282-288)
    std::vector<double> contact_damping(const orc_npi_sampling& s) const
    {
        const int G = g->num_groups;
        std::vector<double> m((size_t)G * G);
        for (int i = 0; i < G; ++i) {
            for (int j = 0; j < G; ++j) {
                const double gi = s.value * s.group_weights[i], gj = s.value * s.group_weights[j];
                m[(size_t)i * G + j] = 1.0 - std::sqrt((1.0 - gi) * (1.0 - gj));
            }
        }
        return m;
    }

    // get_active_damping (dynamic_npis.h:246-258)
    static std::vector<double> active_damping(const std::vector<ODamping>& l, int level, int type, double t,
                                              size_t size)
    {
        for (size_t k = l.size(); k-- > 0;) {
            if (l[k].level == level && l[k].type == type && l[k].time <= t) {
                return l[k].m;
            }
        }
        return std::vector<double>(size, 0.0);
    }

    // one NPI on one damping list (implement_dynamic_npis, dynamic_npis.h:338-369)
    void implement_list(std::vector<ODamping>& l, int level, int type, double begin, double end,
                        const std::vector<double>& value) const
    {
        const std::vector<double> act     = active_damping(l, level, type, begin, value.size());
        const std::vector<double> act_end = active_damping(l, level, type, end, value.size());
        bool implemented                  = false;
        bool less                         = false;
        std::vector<double> mx(value.size());
        for (size_t i = 0; i < value.size(); ++i) {
            less  = less || act[i] < value[i];
            mx[i] = std::max(value[i], act[i]);
        }
        if (less) {
            add_damping(l, {begin, level, type, mx});
            implemented = true;
        }
        std::vector<size_t> idx; // get_damping_indices (dynamic_npis.h:232-244)
        for (size_t i = 0; i < l.size(); ++i) {
            if (l[i].level == level && l[i].type == type && l[i].time > begin && l[i].time < end) {
                idx.push_back(i);
            }
        }
        for (size_t i : idx) {
            ODamping d = l[i];
            for (size_t k = 0; k < d.m.size(); ++k) {
                d.m[k] = std::max(d.m[k], value[k]);
            }
            add_damping(l, d);
            implemented = true;
        }
        if (implemented) {
            add_damping(l, {end, level, type, act_end});
        }
    }

    // remove dampings that repeat the previous value of their (level, type) (dynamic_npis.h:372-390)
    static void dedupe(std::vector<ODamping>& l)
    {
        for (int i = 0; i < (int)l.size() - 1; ++i) {
            const size_t cur = l.size() - 1 - (size_t)i;
            for (size_t k = cur; k-- > 0;) {
                if (l[k].level == l[cur].level && l[k].type == l[cur].type) {
                    if (l[k].m == l[cur].m) {
                        l.erase(l.begin() + (long)cur);
                    }
                    break;
                }
            }
        }
    }

    // implement_dynamic_npis (dynamic_npis.h:335-391) on the contact matrices of node v
    void implement(int v, int thr, double begin, double end)
    {
        auto& nn = npi[v];
        for (int s = npis->first[thr]; s < npis->first[thr + 1]; ++s) {
            const orc_npi_sampling& smp = npis->samplings[s];
            for (int q = 0; q < smp.num_matrices; ++q) {
                implement_list(nn.lists[smp.matrices[q]], smp.level, smp.type, begin, end, contact_damping(smp));
            }
        }
        for (auto& l : nn.lists) {
            dedupe(l);
        }
    }

    // The check at the start of a chunk (model.h:299-350).
    void check_npis(int v, double t)
    {
        const orc_dynamic_npis& p = *npis;
        if (p.num_thresholds == 0) {
            return;
        }
        auto& nn           = npi[v];
        const double delay = t > 0 ? p.delay : 0.0;
        if (!(fp_ge(t, p.directive_begin, 1e-10) && t < p.directive_end)) {
            return;
        }
        const auto& y = nodes[v].y;
        double sum    = 0.0;
        for (int gi = 0; gi < g->num_groups; ++gi) {
            sum += y[(long)gi * kC + MGPU_ISY];
        }
        const double inf_rel = sum / nn.total * p.base_value;
        int thr              = -1;
        for (int k : thr_order) { // get_max_exceeded_threshold: the highest threshold below the value
            if (inf_rel > p.thresholds[k]) {
                thr = k;
                break;
            }
        }
        const bool expired = fp_ge(t, nn.t_end, 1e-10);
        if (thr < 0 || !(p.thresholds[thr] > nn.thr || expired)) {
            return;
        }
        const bool renewal = expired && !(p.thresholds[thr] > nn.thr);
        const double eff   = renewal ? 0.0 : delay;
        if (!(t + eff < p.directive_end)) {
            return;
        }
        const double t_start = t + eff;
        const double t_end   = std::min(p.directive_end, t_start + p.duration);
        nn.thr               = p.thresholds[thr];
        nn.t_end             = t_end;
        const double tsd     = (!renewal && t_start > 0) ? t_start + 1.0 : t_start;
        implement(v, thr, tsd, t_end + 1.0);
        nn.count += 1;
        rebuild_cache(v);
    }

    // osecir::Simulation::advance with dynamic NPIs: chunks of at most a day,
    // ending at the active NPI's end, each after the check at its start.
    void advance_node_npi(int v, double tmax)
    {
        double t = nodes[v].t;
        while (t < tmax) {
            check_npis(v, t);
            double dt_eff = std::min(1.0, tmax - t);
            if (t < npi[v].t_end) {
                dt_eff = std::min(dt_eff, npi[v].t_end - t);
            }
            advance_node(v, t + dt_eff);
            t = t + dt_eff;
        }
    }

    // ---- edge NPIs (MobilityEdge::apply_mobility, metapopulation_mobility_instant.h:549-566) ----
    struct EdgeNpi {
        std::vector<ODamping> list; // coefficient dampings, vectors of 10 G
        std::vector<double> ctimes, cvals;
        double thr   = std::numeric_limits<double>::lowest();
        double t_end = 0.0;
        int count    = 0;
    };
    const orc_dynamic_npis* enpis = nullptr;
    std::vector<int> ethr_order;
    std::vector<EdgeNpi> enpi;
    std::vector<double> node_total; // the models' total populations

    void init_edge_npis(const orc_dynamic_npis* p)
    {
        enpis = p;
        ethr_order.resize(p->num_thresholds);
        for (int k = 0; k < p->num_thresholds; ++k) {
            ethr_order[k] = k;
        }
        std::stable_sort(ethr_order.begin(), ethr_order.end(), [&](int a, int b) {
            return p->thresholds[a] > p->thresholds[b];
        });
        enpi.assign(g->num_edges, {});
        for (int e = 0; e < g->num_edges; ++e) {
            rebuild_edge_cache(e);
        }
        node_total.assign(g->num_nodes, 0.0);
        for (int v = 0; v < g->num_nodes; ++v) {
            for (int j = 0; j < n; ++j) {
                node_total[v] += g->init_state[(long)v * n + j];
            }
        }
    }

    void rebuild_edge_cache(int e)
    {
        auto& en     = enpi[e];
        const int nd = (int)en.list.size();
        std::vector<double> times(nd), mats((size_t)nd * n);
        std::vector<int32_t> levels(nd), types(nd);
        for (int d = 0; d < nd; ++d) {
            times[d]  = en.list[d].time;
            levels[d] = en.list[d].level;
            types[d]  = en.list[d].type;
            std::copy(en.list[d].m.begin(), en.list[d].m.end(), mats.begin() + (long)d * n);
        }
        en.ctimes.assign(nd + 2, 0.0);
        en.cvals.assign((size_t)(nd + 2) * n, 0.0);
        const int k = orc_damping_cache(n, 1, nd, times.data(), levels.data(), types.data(), mats.data(), nd + 2,
                                        en.ctimes.data(), en.cvals.data());
        en.ctimes.resize(k);
        en.cvals.resize((size_t)k * n);
    }

    // DampingMatrixExpression::get_matrix_at of the edge's coefficients with its own cache
    void edge_coeffs_npi(int e, double t, double* c) const
    {
        const auto& en  = enpi[e];
        const int K     = (int)en.ctimes.size();
        const double* B = g->edge_coeff_baseline + (long)e * n;
        const double* L = g->edge_coeff_minimum ? g->edge_coeff_minimum + (long)e * n : nullptr;
        for (int i = 0; i < n; ++i) {
            const double D  = damping_coeff_at(en.ctimes.data(), en.cvals.data(), K, n, i, t);
            const double Li = L ? L[i] : 0.0;
            c[i]            = 0.0 + (B[i] - D * (B[i] - Li));
        }
    }

    void check_edge_npis(int e, double t)
    {
        const orc_dynamic_npis& p = *enpis;
        if (p.num_thresholds == 0) {
            return;
        }
        auto& en      = enpi[e];
        const int u   = g->edge_src[e];
        const auto& y = nodes[u].last_state; // SimulationNode::get_last_state
        double sum    = 0.0;
        for (int gi = 0; gi < g->num_groups; ++gi) {
            sum += y[(long)gi * kC + MGPU_ISY];
        }
        const double inf_rel = sum / node_total[u] * p.base_value;
        int thr              = -1;
        for (int k : ethr_order) {
            if (inf_rel > p.thresholds[k]) {
                thr = k;
                break;
            }
        }
        const bool expired = fp_ge(t, en.t_end, 1e-10);
        if (thr < 0 || !(p.thresholds[thr] > en.thr || expired)) {
            return;
        }
        const double t_end = t + p.duration;
        en.thr             = p.thresholds[thr];
        en.t_end           = t_end;
        const int G        = g->num_groups;
        for (int s = p.first[thr]; s < p.first[thr + 1]; ++s) {
            const orc_npi_sampling& smp = p.samplings[s];
            std::vector<double> value(n); // make_mobility_damping_vector (damping_sampling.h:290-306)
            for (int i = 0; i < n; ++i) {
                value[i] = smp.value * smp.group_weights[i / (n / G)];
            }
            implement_list(en.list, smp.level, smp.type, t, t_end, value);
        }
        dedupe(en.list);
        en.count += 1;
        rebuild_edge_cache(e);
    }

    // GraphSimulation::advance (mobility/graph_simulation.h:101-120).
    void run(double t0, double tmax, double dt_exchange, double* out_states)
    {
        double t  = t0;
        double dt = dt_exchange;
        long b    = 0;
        while (t < tmax) {
            if (t + dt > tmax) {
                dt = tmax - t;
            }
            for (int v = 0; v < g->num_nodes; ++v) {
                if (npis) {
                    advance_node_npi(v, t + dt);
                }
                else {
                    advance_node(v, t + dt);
                }
            }
            t += dt;
            for (int e = 0; e < g->num_edges; ++e) {
                apply_mobility(e, t, dt);
            }
            // The value column at time t now holds the post-exchange state; keep it for
            // find_value_reverse (utils/time_series.h:904-914) at the matching return.
            for (int v = 0; v < g->num_nodes; ++v) {
                auto& ns = nodes[v];
                // only the last two boundaries can be asked for by pending returns
                if (ns.snap_t.size() >= 2) {
                    ns.snap_t.erase(ns.snap_t.begin());
                    ns.snap_y.erase(ns.snap_y.begin());
                }
                ns.snap_t.push_back(t);
                ns.snap_y.push_back(ns.y);
            }
            if (out_states) {
                for (int v = 0; v < g->num_nodes; ++v) {
                    std::memcpy(out_states + (b * g->num_nodes + v) * (long)n, nodes[v].y.data(), n * sizeof(double));
                }
            }
            ++b;
        }
    }

    void write_final(double* final_state) const
    {
        for (int v = 0; v < g->num_nodes; ++v) {
            std::memcpy(final_state + (long)v * n, nodes[v].y.data(), n * sizeof(double));
        }
    }

    void add_stats(orc_stats* s) const
    {
        if (!s) {
            return;
        }
        s->accepted_steps += cnt.accepted;
        s->rejected_steps += cnt.rejected;
        s->failed_steps += cnt.failed;
        s->rhs_evals += rhs_evals;
        s->underflow_fixes += underflow_fixes;
    }
};

bool graph_ok(const mgpu_graph* g)
{
    return g && g->num_nodes >= 0 && g->num_groups >= 1 && g->num_edges >= 0 && g->num_contact_matrices >= 1 &&
           g->params && g->contact_baseline && g->init_state;
}

} // namespace

extern "C" {

int orc_eval_flows(const mgpu_graph* g, int node, const double* pop, const double* y, double t, double* flows)
{
    if (!graph_ok(g) || node < 0 || node >= g->num_nodes) {
        return -1;
    }
    NodeView nv = node_view(g, node);
    std::fill(flows, flows + nv.G * kF, 0.0);
    get_flows(nv, pop, y, t, flows);
    return 0;
}

int orc_eval_rhs(const mgpu_graph* g, int node, const double* pop, const double* y, double t, double* dydt)
{
    if (!graph_ok(g) || node < 0 || node >= g->num_nodes) {
        return -1;
    }
    Rhs rhs(node_view(g, node));
    rhs(pop, y, t, dydt);
    return 0;
}

// FlowSimulation::advance (flow_simulation.h:56-79): f(flows) = get_flows(pop, pop, t)
// with pop = y0 + get_derivatives(flows) (groups outer, flows inner, as
// FlowModel::get_derivatives, flow_model.h:112-125); populations of the
// recorded points by compute_population_results (flow_simulation_base.h:90-103).
int orc_simulate_flows(const mgpu_graph* g, int node, double t0, double tmax, double dt,
                       const mgpu_integrator_opts* opts, int max_points, double* out_t, double* out_f,
                       double* out_y, int* num_points, orc_stats* stats)
{
    if (!graph_ok(g) || node < 0 || node >= g->num_nodes || !opts || max_points < 1) {
        return -1;
    }
    const int G  = g->num_groups;
    const int n  = G * kC;
    const int nf = G * kF;
    const NodeView nv = node_view(g, node);
    const double* y0  = g->init_state + (long)node * n;
    auto scatter = [&](const double* flows, double* dydt) {
        std::fill(dydt, dydt + n, 0.0);
        for (int i = 0; i < G; ++i) {
            for (int k = 0; k < kF; ++k) {
                const double fv = flows[i * kF + k];
                dydt[i * kC + kFlowSrc[k]] -= fv;
                dydt[i * kC + kFlowDst[k]] += fv;
            }
        }
    };
    std::vector<double> pop(n);
    long evals = 0;
    auto f = [&](const double*, const double* flows, double t, double* dflows) {
        scatter(flows, pop.data());
        for (int j = 0; j < n; ++j) {
            pop[j] += y0[j];
        }
        std::fill(dflows, dflows + nf, 0.0);
        get_flows(nv, pop.data(), pop.data(), t, dflows);
        ++evals;
    };
    Counters cnt;
    Core core(*opts, nf, &cnt);
    std::vector<double> x(nf, 0.0);
    int np    = 0;
    bool full = false;
    auto rec  = [&](double t, const std::vector<double>& v) {
        if (np >= max_points) {
            full = true;
            return;
        }
        out_t[np] = t;
        std::memcpy(out_f + (long)np * nf, v.data(), nf * sizeof(double));
        double* yrow = out_y + (long)np * n;
        scatter(v.data(), yrow);
        for (int j = 0; j < n; ++j) {
            yrow[j] += y0[j];
        }
        ++np;
    };
    double t = t0;
    rec(t, x);
    system_advance(core, f, tmax, t, dt, x, rec);
    *num_points = np;
    if (stats) {
        stats->accepted_steps += cnt.accepted;
        stats->rejected_steps += cnt.rejected;
        stats->failed_steps += cnt.failed;
        stats->rhs_evals += evals;
    }
    return full ? -1 : 0;
}

int orc_simulate(const mgpu_graph* g, int node, double t0, double tmax, double dt, const mgpu_integrator_opts* opts,
                 int max_points, double* out_t, double* out_y, int* num_points, orc_stats* stats)
{
    if (!graph_ok(g) || node < 0 || node >= g->num_nodes || !opts || max_points < 1) {
        return -1;
    }
    const int n = g->num_groups * kC;
    Counters cnt;
    Core core(*opts, n, &cnt);
    Rhs rhs(node_view(g, node));
    auto f = [&](const double* pop, const double* y, double t, double* dydt) {
        rhs(pop, y, t, dydt);
    };
    std::vector<double> y(g->init_state + (long)node * n, g->init_state + (long)(node + 1) * n);
    int np    = 0;
    bool full = false;
    auto rec  = [&](double t, const std::vector<double>& v) {
        if (np >= max_points) {
            full = true;
            return;
        }
        out_t[np] = t;
        std::memcpy(out_y + (long)np * n, v.data(), n * sizeof(double));
        ++np;
    };
    double t = t0;
    rec(t, y);
    system_advance(core, f, tmax, t, dt, y, rec);
    *num_points = np;
    if (stats) {
        stats->accepted_steps += cnt.accepted;
        stats->rejected_steps += cnt.rejected;
        stats->failed_steps += cnt.failed;
        stats->rhs_evals += rhs.evals;
    }
    return full ? -1 : 0;
}

int orc_graph_run(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                  const mgpu_integrator_opts* opts, double* out_states, double* final_state, orc_stats* stats)
{
    if (!graph_ok(g) || !opts || !(dt_exchange > 0)) {
        return -1;
    }
    GraphRun run(g, t0, dt0, *opts);
    run.run(t0, tmax, dt_exchange, out_states);
    if (final_state) {
        run.write_final(final_state);
    }
    run.add_stats(stats);
    return 0;
}

int orc_graph_run_commuters(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                            const mgpu_integrator_opts* opts, int num_sets, const int32_t* set_offsets,
                            const int32_t* set_indices, int capacity, double* final_state, int32_t* counts,
                            double* times, double* values, orc_stats* stats)
{
    if (!graph_ok(g) || !opts || !(dt_exchange > 0) || num_sets < 1 || !set_offsets || !set_indices ||
        capacity < 0 || !counts) {
        return -1;
    }
    GraphRun run(g, t0, dt0, *opts);
    const int n = g->num_groups * kC;
    for (int i = 0; i < num_sets; ++i) {
        std::vector<int> set;
        for (int q = set_offsets[i]; q < set_offsets[i + 1]; ++q) {
            if (set_indices[q] < 0 || set_indices[q] >= n) {
                return -1;
            }
            set.push_back(set_indices[q]);
        }
        run.save_sets.push_back(set);
    }
    run.result_t.resize(g->num_edges);
    run.result_v.resize(g->num_edges);
    run.run(t0, tmax, dt_exchange, nullptr);
    for (int e = 0; e < g->num_edges; ++e) {
        const int np = (int)run.result_t[e].size();
        counts[e]    = np;
        for (int k = 0; k < np && k < capacity; ++k) {
            times[(long)e * capacity + k] = run.result_t[e][k];
            for (int i = 0; i <= num_sets; ++i) {
                values[((long)e * capacity + k) * (num_sets + 1) + i] = run.result_v[e][(long)k * (num_sets + 1) + i];
            }
        }
    }
    if (final_state) {
        run.write_final(final_state);
    }
    run.add_stats(stats);
    return 0;
}

int orc_departure_commuters(const mgpu_graph* g, int edge, double t, int num_sets, const int32_t* set_offsets,
                            const int32_t* set_indices, double* values)
{
    if (!graph_ok(g) || edge < 0 || edge >= g->num_edges || num_sets < 1 || !set_offsets || !set_indices ||
        !values) {
        return -1;
    }
    mgpu_integrator_opts o{};
    o.abs_tol = 1e-10;
    o.rel_tol = 1e-5;
    o.dt_min  = 0.0;
    o.dt_max  = 0.0;
    GraphRun run(g, t, 0.1, o);
    for (int i = 0; i < num_sets; ++i) {
        run.save_sets.emplace_back(set_indices + set_offsets[i], set_indices + set_offsets[i + 1]);
    }
    run.result_t.resize(g->num_edges);
    run.result_v.resize(g->num_edges);
    run.apply_mobility(edge, t, 0.0);
    if (run.result_v[edge].size() != (size_t)(num_sets + 1)) {
        return -1;
    }
    std::copy(run.result_v[edge].begin(), run.result_v[edge].end(), values);
    return 0;
}

int orc_graph_run_npi(const mgpu_graph* g, double t0, double tmax, double dt_exchange, double dt0,
                      const mgpu_integrator_opts* opts, const orc_dynamic_npis* npis, int num_dampings,
                      const orc_damping* dampings, const orc_dynamic_npis* edge_npis, double* final_state,
                      int32_t* npi_count, int32_t* edge_npi_count, orc_stats* stats)
{
    if (!graph_ok(g) || !opts || !npis || !(dt_exchange > 0) || (num_dampings > 0 && !dampings) ||
        (edge_npis && g->num_edge_damping_points != 0)) {
        return -1;
    }
    for (int d = 0; d < num_dampings; ++d) {
        if (dampings[d].matrix < 0 || dampings[d].matrix >= g->num_contact_matrices || !dampings[d].coeffs) {
            return -1;
        }
    }
    GraphRun run(g, t0, dt0, *opts);
    run.init_npis(npis, num_dampings, dampings);
    if (edge_npis) {
        run.init_edge_npis(edge_npis);
    }
    run.run(t0, tmax, dt_exchange, nullptr);
    if (edge_npi_count && edge_npis) {
        for (int e = 0; e < g->num_edges; ++e) {
            edge_npi_count[e] = run.enpi[e].count;
        }
    }
    if (final_state) {
        run.write_final(final_state);
    }
    if (npi_count) {
        for (int v = 0; v < g->num_nodes; ++v) {
            npi_count[v] = run.npi[v].count;
        }
    }
    run.add_stats(stats);
    return 0;
}

int orc_ensemble_run(const mgpu_graph* graphs, int num_graphs, double t0, double tmax, double dt_exchange,
                     double dt0, const mgpu_integrator_opts* opts, int num_threads, double* final_states,
                     double* elapsed_s, orc_stats* stats)
{
    if (!graphs || num_graphs < 0 || !opts) {
        return -1;
    }
    std::vector<long> offset(num_graphs + 1, 0);
    for (int b = 0; b < num_graphs; ++b) {
        if (!graph_ok(&graphs[b])) {
            return -1;
        }
        offset[b + 1] = offset[b] + (long)graphs[b].num_nodes * graphs[b].num_groups * kC;
    }
    int nt = num_threads > 0 ? num_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    nt     = std::max(1, std::min(nt, std::max(1, num_graphs)));
    std::atomic<int> next{0};
    std::vector<orc_stats> per(nt);
    std::memset(per.data(), 0, sizeof(orc_stats) * nt);
    auto t_start = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    for (int w = 0; w < nt; ++w) {
        pool.emplace_back([&, w] {
            for (int b = next.fetch_add(1); b < num_graphs; b = next.fetch_add(1)) {
                GraphRun run(&graphs[b], t0, dt0, *opts);
                run.run(t0, tmax, dt_exchange, nullptr);
                if (final_states) {
                    run.write_final(final_states + offset[b]);
                }
                run.add_stats(&per[w]);
            }
        });
    }
    for (auto& th : pool) {
        th.join();
    }
    auto t_end = std::chrono::steady_clock::now();
    if (elapsed_s) {
        *elapsed_s = std::chrono::duration<double>(t_end - t_start).count();
    }
    if (stats) {
        for (auto& s : per) {
            stats->accepted_steps += s.accepted_steps;
            stats->rejected_steps += s.rejected_steps;
            stats->failed_steps += s.failed_steps;
            stats->rhs_evals += s.rhs_evals;
            stats->underflow_fixes += s.underflow_fixes;
        }
    }
    return 0;
}

// Dampings::update_cache (damping.h:570-600) with update_active_dampings
// (:616-658) and inclusive_exclusive_sum (:545-562).
int orc_damping_cache(int rows, int cols, int num_dampings, const double* times, const int32_t* levels,
                      const int32_t* types, const double* matrices, int cap, double* out_times,
                      double* out_matrices)
{
    const int sz = rows * cols;
    struct Active {
        std::vector<double> m;
        int level, type;
    };
    struct Sum {
        std::vector<double> m;
        int level;
    };
    std::vector<Active> active_by_type;
    std::vector<Sum> sum_by_level;
    std::vector<double> ct;
    std::vector<std::vector<double>> cm;
    ct.push_back(std::numeric_limits<double>::lowest());
    cm.emplace_back(sz, 0.0);
    for (int d = 0; d < num_dampings; ++d) {
        const double* dm = matrices + (long)d * sz;
        auto it          = std::find_if(active_by_type.begin(), active_by_type.end(), [&](const Active& a) {
            return a.level == levels[d] && a.type == types[d];
        });
        if (it != active_by_type.end()) {
            auto& s = *std::find_if(sum_by_level.begin(), sum_by_level.end(), [&](const Sum& x) {
                return x.level == levels[d];
            });
            for (int i = 0; i < sz; ++i) {
                s.m[i] += dm[i] - it->m[i];
            }
            it->m.assign(dm, dm + sz);
        }
        else {
            active_by_type.push_back({std::vector<double>(dm, dm + sz), levels[d], types[d]});
            auto sit = std::find_if(sum_by_level.begin(), sum_by_level.end(), [&](const Sum& x) {
                return x.level == levels[d];
            });
            if (sit != sum_by_level.end()) {
                for (int i = 0; i < sz; ++i) {
                    sit->m[i] += dm[i];
                }
            }
            else {
                sum_by_level.push_back({std::vector<double>(dm, dm + sz), levels[d]});
            }
        }
        std::vector<double> comb = sum_by_level.front().m;
        for (size_t l = 1; l < sum_by_level.size(); ++l) {
            for (int i = 0; i < sz; ++i) {
                const double prod = comb[i] * sum_by_level[l].m[i];
                comb[i]           = comb[i] + sum_by_level[l].m[i] - prod;
            }
        }
        if (fp_equal(times[d], ct.back(), 1e-15, 1e-15)) {
            cm.back() = comb;
        }
        else {
            ct.push_back(times[d]);
            cm.push_back(comb);
        }
    }
    ct.push_back(std::numeric_limits<double>::max());
    cm.push_back(cm.back());
    if ((int)ct.size() > cap) {
        return -1;
    }
    for (size_t k = 0; k < ct.size(); ++k) {
        out_times[k] = ct[k];
        std::memcpy(out_matrices + k * sz, cm[k].data(), sz * sizeof(double));
    }
    return (int)ct.size();
}

} // extern "C"
