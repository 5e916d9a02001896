/*
 * miogpu/osecir.h — the age-resolved ODE-SECIR model and its simulation, with
 * the API of MEmilio's mio::osecir (cpp/models/ode_secir/infection_state.h,
 * parameters.h, model.h) and mio::Simulation (cpp/memilio/compartments/
 * simulation.h, simulation_base.h), computing on the GPU through libmiogpu:
 *
 *   Model::get_derivatives  -> mgpu_eval_rhs
 *   Simulation::advance     -> mgpu_simulate_dt (every accepted step recorded)
 *
 * A model packs into one node record of include/miogpu_layout.h (pack()).
 */
#ifndef MIOGPU_FACADE_OSECIR_H
#define MIOGPU_FACADE_OSECIR_H

#include "core.h"
#include "dynamic_npis.h"

namespace miogpu
{
namespace osecir
{

/* mio::osecir::InfectionState (infection_state.h:33-47). */
enum class InfectionState
{
    Susceptible = 0,
    Exposed,
    InfectedNoSymptoms,
    InfectedNoSymptomsConfirmed,
    InfectedSymptoms,
    InfectedSymptomsConfirmed,
    InfectedSevere,
    InfectedCritical,
    Recovered,
    Dead,
    Count
};

constexpr size_t num_compartments = (size_t)InfectionState::Count;
static_assert(num_compartments == MGPU_NUM_COMPARTMENTS, "compartment count of the layout");

/* Values per age group of one parameter (CustomIndexArray<UncertainValue, AgeGroup>),
 * a view into the node record. */
class GroupValues
{
public:
    GroupValues(double* p, size_t n)
        : m_p(p)
        , m_n(n)
    {
    }
    double& operator[](AgeGroup g)
    {
        return m_p[g.get()];
    }
    double operator[](AgeGroup g) const
    {
        return m_p[g.get()];
    }
    GroupValues& operator=(double v)
    {
        std::fill(m_p, m_p + m_n, v);
        return *this;
    }
    size_t numel() const
    {
        return m_n;
    }

private:
    double* m_p;
    size_t m_n;
};

/* Parameter tags (parameters.h:47-394). `scalar` / `group` index the record. */
#define MIOGPU_SCALAR_TAG(NAME, IDX)                                                                                 \
    template <typename FP = double>                                                                                  \
    struct NAME {                                                                                                    \
        static constexpr int scalar = IDX;                                                                           \
        static constexpr int group  = -1;                                                                            \
        static const char* name()                                                                                    \
        {                                                                                                            \
            return #NAME;                                                                                            \
        }                                                                                                            \
    };
#define MIOGPU_GROUP_TAG(NAME, IDX)                                                                                  \
    template <typename FP = double>                                                                                  \
    struct NAME {                                                                                                    \
        static constexpr int scalar = -1;                                                                            \
        static constexpr int group  = IDX;                                                                           \
        static const char* name()                                                                                    \
        {                                                                                                            \
            return #NAME;                                                                                            \
        }                                                                                                            \
    };
MIOGPU_SCALAR_TAG(StartDay, MGPU_P_START_DAY)
MIOGPU_SCALAR_TAG(Seasonality, MGPU_P_SEASONALITY)
MIOGPU_SCALAR_TAG(ICUCapacity, MGPU_P_ICU_CAPACITY)
MIOGPU_SCALAR_TAG(TestAndTraceCapacity, MGPU_P_TNT_CAPACITY)
MIOGPU_SCALAR_TAG(TestAndTraceCapacityMaxRisk, MGPU_P_TNT_MAX_RISK)
MIOGPU_GROUP_TAG(TimeExposed, MGPU_G_TIME_EXPOSED)
MIOGPU_GROUP_TAG(TimeInfectedNoSymptoms, MGPU_G_TIME_INS)
MIOGPU_GROUP_TAG(TimeInfectedSymptoms, MGPU_G_TIME_ISY)
MIOGPU_GROUP_TAG(TimeInfectedSevere, MGPU_G_TIME_ISEV)
MIOGPU_GROUP_TAG(TimeInfectedCritical, MGPU_G_TIME_ICRI)
MIOGPU_GROUP_TAG(TransmissionProbabilityOnContact, MGPU_G_TRANSMISSION_PROB)
MIOGPU_GROUP_TAG(RelativeTransmissionNoSymptoms, MGPU_G_REL_TRANSMISSION_NS)
MIOGPU_GROUP_TAG(RecoveredPerInfectedNoSymptoms, MGPU_G_RECOVERED_PER_INS)
MIOGPU_GROUP_TAG(RiskOfInfectionFromSymptomatic, MGPU_G_RISK_FROM_SYMPTOMATIC)
MIOGPU_GROUP_TAG(MaxRiskOfInfectionFromSymptomatic, MGPU_G_MAX_RISK_FROM_SYMPTOMATIC)
MIOGPU_GROUP_TAG(SeverePerInfectedSymptoms, MGPU_G_SEVERE_PER_ISY)
MIOGPU_GROUP_TAG(CriticalPerSevere, MGPU_G_CRITICAL_PER_SEVERE)
MIOGPU_GROUP_TAG(DeathsPerSevere, MGPU_G_DEATHS_PER_SEVERE)
MIOGPU_GROUP_TAG(DeathsPerCritical, MGPU_G_DEATHS_PER_CRITICAL)
#undef MIOGPU_SCALAR_TAG
#undef MIOGPU_GROUP_TAG

template <typename FP = double>
struct ContactPatterns {
    static const char* name()
    {
        return "ContactPatterns";
    }
};

/* Dynamic NPIs on the symptomatic infections (parameters.h DynamicNPIsInfectedSymptoms). */
template <typename FP = double>
struct DynamicNPIsInfectedSymptoms {
    static const char* name()
    {
        return "DynamicNPIsInfectedSymptoms";
    }
};

/* mio::osecir::Parameters: the node record of include/miogpu_layout.h with the
 * reference's defaults (get_default of every tag), plus the contact patterns. */
template <typename FP = double>
class Parameters
{
public:
    explicit Parameters(AgeGroup num_groups)
        : m_G(num_groups.get())
        , m_rec((size_t)MGPU_PARAM_STRIDE((int)num_groups.get()), 0.0)
        , m_contacts(1, num_groups.get())
    {
        m_rec[MGPU_P_ICU_CAPACITY] = std::numeric_limits<double>::max();
        m_rec[MGPU_P_TNT_CAPACITY] = std::numeric_limits<double>::max();
        m_rec[MGPU_P_TNT_MAX_RISK] = 5.0;
        for (int p : {MGPU_G_TIME_EXPOSED, MGPU_G_TIME_INS, MGPU_G_TIME_ISY, MGPU_G_TIME_ISEV, MGPU_G_TIME_ICRI,
                      MGPU_G_TRANSMISSION_PROB, MGPU_G_REL_TRANSMISSION_NS, MGPU_G_RISK_FROM_SYMPTOMATIC,
                      MGPU_G_MAX_RISK_FROM_SYMPTOMATIC}) {
            group(p) = 1.0;
        }
    }

    AgeGroup get_num_groups() const
    {
        return AgeGroup(m_G);
    }

    template <class Tag>
    decltype(auto) get()
    {
        if constexpr (std::is_same<Tag, ContactPatterns<FP>>::value) {
            return static_cast<ContactMatrixGroup&>(m_contacts);
        }
        else if constexpr (std::is_same<Tag, DynamicNPIsInfectedSymptoms<FP>>::value) {
            return static_cast<DynamicNPIs<FP>&>(m_npis);
        }
        else if constexpr (Tag::scalar >= 0) {
            return static_cast<double&>(m_rec[Tag::scalar]);
        }
        else {
            return group(Tag::group);
        }
    }
    template <class Tag>
    decltype(auto) get() const
    {
        return const_cast<Parameters*>(this)->template get<Tag>();
    }
    template <class Tag, class V>
    void set(const V& v)
    {
        get<Tag>() = v;
    }

    double& get_commuter_nondetection()
    {
        return m_rec[MGPU_P_COMMUTER_NONDETECTION];
    }
    double& get_start_commuter_detection()
    {
        return m_rec[MGPU_P_START_COMMUTER_DETECTION];
    }
    double& get_end_commuter_detection()
    {
        return m_rec[MGPU_P_END_COMMUTER_DETECTION];
    }

    /* apply_constraints (parameters.h:465-611): clamps out-of-range values to the
     * reference's corrections; returns true if anything changed. */
    bool apply_constraints()
    {
        const double tol_times = 1e-1;
        bool corrected         = false;
        auto fix               = [&](double& v, bool bad, double to) {
            if (bad) {
                v         = to;
                corrected = true;
            }
        };
        double& season = m_rec[MGPU_P_SEASONALITY];
        fix(season, season < 0.0 || season > 0.5, 0.0);
        fix(m_rec[MGPU_P_ICU_CAPACITY], m_rec[MGPU_P_ICU_CAPACITY] < 0.0, 0.0);
        fix(m_rec[MGPU_P_TNT_CAPACITY], m_rec[MGPU_P_TNT_CAPACITY] < 0.0, 0.0);
        fix(m_rec[MGPU_P_TNT_MAX_RISK], m_rec[MGPU_P_TNT_MAX_RISK] < 0.0, 0.0);
        for (size_t i = 0; i < m_G; ++i) {
            const AgeGroup g(i);
            for (int p : {MGPU_G_TIME_EXPOSED, MGPU_G_TIME_INS, MGPU_G_TIME_ISY, MGPU_G_TIME_ISEV, MGPU_G_TIME_ICRI}) {
                fix(group(p)[g], group(p)[g] < tol_times, tol_times);
            }
            for (int p : {MGPU_G_TRANSMISSION_PROB, MGPU_G_RECOVERED_PER_INS, MGPU_G_RISK_FROM_SYMPTOMATIC,
                          MGPU_G_SEVERE_PER_ISY, MGPU_G_CRITICAL_PER_SEVERE, MGPU_G_DEATHS_PER_SEVERE}) {
                fix(group(p)[g], group(p)[g] < 0.0 || group(p)[g] > 1.0, 0.0);
            }
            fix(group(MGPU_G_REL_TRANSMISSION_NS)[g], group(MGPU_G_REL_TRANSMISSION_NS)[g] < 0.0, 0.0);
            fix(group(MGPU_G_DEATHS_PER_SEVERE)[g],
                group(MGPU_G_CRITICAL_PER_SEVERE)[g] + group(MGPU_G_DEATHS_PER_SEVERE)[g] > 1.0, 0.0);
            fix(group(MGPU_G_DEATHS_PER_CRITICAL)[g],
                group(MGPU_G_DEATHS_PER_CRITICAL)[g] < 0.0 || group(MGPU_G_DEATHS_PER_CRITICAL)[g] > 1.0, 0.0);
        }
        return corrected;
    }

    /* check_constraints (parameters.h:618-742): true if a constraint is violated. */
    bool check_constraints() const
    {
        Parameters copy = *this;
        return copy.apply_constraints();
    }

    const std::vector<double>& record() const
    {
        return m_rec;
    }
    const ContactMatrixGroup& contacts() const
    {
        return m_contacts;
    }

private:
    GroupValues group(int p)
    {
        return GroupValues(m_rec.data() + MGPU_GROUP_PARAM(p, 0, (int)m_G), m_G);
    }

    size_t m_G;
    std::vector<double> m_rec;
    ContactMatrixGroup m_contacts;
    DynamicNPIs<FP> m_npis;
};

/* Compartment populations per age group (Populations<FP, AgeGroup, InfectionState>),
 * flat index g*10 + c. */
class Populations
{
public:
    struct Index {
        AgeGroup group;
        InfectionState state;
    };
    explicit Populations(size_t num_groups)
        : m_G(num_groups)
        , m_v(num_groups * num_compartments, 0.0)
    {
    }
    double& operator[](const Index& i)
    {
        return m_v.at(i.group.get() * num_compartments + (size_t)i.state);
    }
    double operator[](const Index& i) const
    {
        return m_v.at(i.group.get() * num_compartments + (size_t)i.state);
    }
    double get_total() const
    {
        double s = 0.0;
        for (double v : m_v) {
            s += v;
        }
        return s;
    }
    double get_group_total(AgeGroup g) const
    {
        double s = 0.0;
        for (size_t c = 0; c < num_compartments; ++c) {
            s += m_v[g.get() * num_compartments + c];
        }
        return s;
    }
    /* Sets compartment i so that its age group sums to `total`. */
    template <class Category = AgeGroup>
    void set_difference_from_group_total(const Index& i, double total)
    {
        const double others = get_group_total(i.group) - (*this)[i];
        (*this)[i]          = total - others;
    }
    size_t get_num_compartments() const
    {
        return m_v.size();
    }
    const std::vector<double>& array() const
    {
        return m_v;
    }
    std::vector<double>& array()
    {
        return m_v;
    }
    bool check_constraints() const
    {
        for (double v : m_v) {
            if (v < 0.0) {
                return true;
            }
        }
        return false;
    }
    bool apply_constraints()
    {
        bool c = false;
        for (double& v : m_v) {
            if (v < 0.0) {
                v = 0.0;
                c = true;
            }
        }
        return c;
    }

private:
    size_t m_G;
    std::vector<double> m_v;
};

/* One model's arrays in the layout of include/miogpu_layout.h. */
struct NodeRecord {
    int G = 0, M = 0, K = 0;
    std::vector<double> params, contact_baseline, contact_minimum, damping_times, damping_values, state;
};

/* mio::osecir::Model (model.h:76-80, get_flows :82-214). */
template <typename FP = double>
class Model
{
public:
    explicit Model(int num_agegroups)
        : populations((size_t)num_agegroups)
        , parameters(AgeGroup((size_t)num_agegroups))
    {
        if (num_agegroups < 1 || num_agegroups > MGPU_MAX_GROUPS) {
            throw Error(MGPU_UNSUPPORTED, "number of age groups out of [1, MGPU_MAX_GROUPS]");
        }
    }

    Populations populations;
    Parameters<FP> parameters;

    size_t num_groups() const
    {
        return parameters.get_num_groups().get();
    }
    bool check_constraints() const
    {
        return parameters.check_constraints() || populations.check_constraints();
    }
    bool apply_constraints()
    {
        const bool a = parameters.apply_constraints();
        const bool b = populations.apply_constraints();
        return a || b;
    }
    std::vector<FP> get_initial_values() const
    {
        return populations.array();
    }

    /* The node record; `state` is the given value vector (default: the populations). */
    NodeRecord pack(const std::vector<FP>* state = nullptr) const
    {
        NodeRecord r;
        const size_t G = num_groups();
        r.G            = (int)G;
        r.params       = parameters.record();
        const auto& cm = parameters.contacts();
        r.M            = (int)cm.get_num_matrices();
        std::vector<const DampingMatrixExpression*> ms;
        for (size_t m = 0; m < cm.get_num_matrices(); ++m) {
            const auto& c = cm[m];
            r.contact_baseline.insert(r.contact_baseline.end(), c.get_baseline().data(),
                                      c.get_baseline().data() + G * G);
            r.contact_minimum.insert(r.contact_minimum.end(), c.get_minimum().data(), c.get_minimum().data() + G * G);
            ms.push_back(&c);
        }
        r.K     = flatten_damping_caches(ms, r.damping_times, r.damping_values);
        r.state = state ? *state : populations.array();
        return r;
    }

    /* dydt = f(pop, y, t) (FlowModel::get_derivatives, flow_model.h:138-144). */
    void get_derivatives(const std::vector<FP>& pop, const std::vector<FP>& y, FP t, std::vector<FP>& dydt) const
    {
        const NodeRecord r = pack();
        mgpu_graph g       = graph_of(r);
        const int32_t node = 0;
        dydt.assign(y.size(), 0.0);
        mgpu_context* ctx = Device::context();
        check(mgpu_eval_rhs(ctx, &g, 1, &node, pop.data(), y.data(), &t, dydt.data()), ctx, "mgpu_eval_rhs");
    }

    /* A one-node graph over the arrays of r (which must outlive it). */
    static mgpu_graph graph_of(const NodeRecord& r)
    {
        mgpu_graph g{};
        g.num_nodes               = 1;
        g.num_groups              = r.G;
        g.num_edges               = 0;
        g.num_contact_matrices    = r.M;
        g.num_damping_points      = r.K;
        g.num_edge_damping_points = 0;
        g.params                  = r.params.data();
        g.contact_baseline        = r.contact_baseline.data();
        g.contact_minimum         = r.contact_minimum.data();
        g.damping_times           = r.K ? r.damping_times.data() : nullptr;
        g.damping_values          = r.K ? r.damping_values.data() : nullptr;
        g.init_state              = r.state.data();
        return g;
    }
};

/* mio::osecir::Simulation / mio::Simulation (simulation.h:41-74,
 * simulation_base.h:40-183): owns a model copy, the result time series and
 * the step size that persists across advance() calls. */
template <typename FP = double>
class Simulation
{
public:
    using Model = osecir::Model<FP>;

    explicit Simulation(const Model& model, FP t0 = 0., FP dt = 0.1)
        : m_model(model)
        , m_result(model.populations.get_num_compartments())
        , m_dt(dt)
    {
        m_result.add_time_point(t0, model.get_initial_values());
    }

    /* osecir::Simulation::advance (model.h:289-367): without dynamic NPIs one
     * integration to tmax; with them, chunks of at most one day (ending at the
     * active NPI's end when that comes first), each after the NPI check at its
     * start, which may add dampings to the contact patterns. */
    std::vector<FP> advance(FP tmax)
    {
        auto& npis = m_model.parameters.template get<DynamicNPIsInfectedSymptoms<FP>>();
        if (npis.get_thresholds().empty()) {
            return advance_base(tmax);
        }
        FP t = m_result.get_last_time();
        while (t < tmax) {
            check_dynamic_npis(npis, m_npi, m_model.parameters.template get<ContactPatterns<FP>>(), t,
                               get_infections_relative(*this, t, m_result.get_last_value()));
            FP dt_eff = std::min<FP>(1.0, tmax - t);
            if (t < m_npi.t_end) {
                dt_eff = std::min<FP>(dt_eff, m_npi.t_end - t);
            }
            advance_base(t + dt_eff);
            t = t + dt_eff;
        }
        return m_result.get_last_value();
    }

    /* The NPI state: the active threshold and its end (m_dynamic_npi). */
    const DynamicNPIState& get_dynamic_npi_state() const
    {
        return m_npi;
    }
    DynamicNPIState& get_dynamic_npi_state()
    {
        return m_npi;
    }

    /* Integrates to tmax (SystemIntegrator::advance, integrator.h:184-249) and
     * returns the last value; every accepted step is appended to the result. */
    std::vector<FP> advance_base(FP tmax)
    {
        const FP t0 = m_result.get_last_time();
        if (!(tmax > t0)) {
            return m_result.get_last_value();
        }
        const std::vector<FP> y0 = m_result.get_last_value();
        const NodeRecord r       = m_model.pack(&y0);
        mgpu_graph g             = Model::graph_of(r);
        const mgpu_integrator_opts o = m_core.opts();
        mgpu_context* ctx        = Device::context();
        const int32_t node       = 0;
        const size_t n           = y0.size();
        for (int32_t cap = 1024;; cap *= 4) {
            std::vector<double> t(cap), y((size_t)cap * n);
            int32_t np = 0;
            double dt  = m_dt;
            const int rc = mgpu_simulate_dt(ctx, &g, 1, &node, t0, tmax, &dt, &o, cap, t.data(), y.data(), &np);
            if (rc == MGPU_OUT_OF_RANGE && cap < (1 << 24)) {
                continue; // more accepted steps than room: retry with a larger buffer
            }
            check(rc, ctx, "mgpu_simulate_dt");
            for (int32_t k = 1; k < np; ++k) {
                m_result.add_time_point(t[(size_t)k], y.data() + (size_t)k * n);
            }
            m_dt = dt;
            break;
        }
        return m_result.get_last_value();
    }

    TimeSeries<FP>& get_result()
    {
        return m_result;
    }
    const TimeSeries<FP>& get_result() const
    {
        return m_result;
    }
    Model& get_model()
    {
        return m_model;
    }
    const Model& get_model() const
    {
        return m_model;
    }
    FP& get_dt()
    {
        return m_dt;
    }
    FP get_dt() const
    {
        return m_dt;
    }
    void set_integrator_core(const IntegratorCore& core)
    {
        m_core = core;
    }
    template <class Core>
    void set_integrator_core(std::unique_ptr<Core> core)
    {
        m_core = *core;
    }
    const IntegratorCore& get_integrator_core() const
    {
        return m_core;
    }

private:
    Model m_model;
    TimeSeries<FP> m_result;
    FP m_dt;
    IntegratorCore m_core;
    DynamicNPIState m_npi;
};

/* get_infections_relative (model.h:413-423): the symptomatic infections of the
 * value vector y relative to the model's total population. */
template <typename FP, class Sim>
FP get_infections_relative(const Sim& sim, FP /*t*/, const std::vector<FP>& y)
{
    const auto& model = sim.get_model();
    FP sum_inf        = 0;
    for (size_t g = 0; g < model.num_groups(); ++g) {
        sum_inf += y[g * num_compartments + (size_t)InfectionState::InfectedSymptoms];
    }
    return sum_inf / model.populations.get_total();
}
/* The same from the symptomatic infections summed over the age groups. */
template <typename FP, class Sim>
FP get_infections_relative_of_sum(const Sim& sim, FP sum_inf)
{
    return sum_inf / sim.get_model().populations.get_total();
}

/* mio::FlowSimulation (compartments/flow_simulation.h:36-102): the integrator's
 * state is the accumulated flows; get_result() holds the populations and
 * get_flows() the flows (15G per time point, flat index g*15 + k) of every
 * accepted step. A later advance continues from the last time point with the
 * flows accumulated so far (the step size restarts from dt). */
template <typename FP = double>
class FlowSimulation
{
public:
    using Model = osecir::Model<FP>;

    explicit FlowSimulation(const Model& model, FP t0 = 0., FP dt = 0.1)
        : m_model(model)
        , m_result(model.populations.get_num_compartments())
        , m_flows(model.num_groups() * (size_t)MGPU_NUM_FLOWS)
        , m_dt(dt)
    {
        m_result.add_time_point(t0, model.get_initial_values());
        m_flows.add_time_point(t0, std::vector<FP>(m_flows.get_num_elements(), 0.0));
    }

    std::vector<FP> advance(FP tmax)
    {
        const FP t0 = m_result.get_last_time();
        if (!(tmax > t0)) {
            return m_result.get_last_value();
        }
        const std::vector<FP> y0 = m_result.get_last_value();
        const std::vector<FP> f0 = m_flows.get_last_value();
        const NodeRecord r       = m_model.pack(&y0);
        mgpu_graph g             = Model::graph_of(r);
        const mgpu_integrator_opts o = m_core.opts();
        mgpu_context* ctx        = Device::context();
        const int32_t node       = 0;
        const size_t n = y0.size(), nf = f0.size();
        for (int32_t cap = 1024;; cap *= 4) {
            std::vector<double> t(cap), f((size_t)cap * nf), y((size_t)cap * n);
            int32_t np   = 0;
            const int rc = mgpu_simulate_flows(ctx, &g, 1, &node, t0, tmax, m_dt, &o, cap, t.data(), f.data(),
                                               y.data(), &np);
            if (rc == MGPU_OUT_OF_RANGE && cap < (1 << 22)) {
                continue;
            }
            check(rc, ctx, "mgpu_simulate_flows");
            std::vector<FP> acc(nf);
            for (int32_t k = 1; k < np; ++k) {
                for (size_t q = 0; q < nf; ++q) {
                    acc[q] = f0[q] + f[(size_t)k * nf + q];
                }
                m_flows.add_time_point(t[(size_t)k], acc);
                m_result.add_time_point(t[(size_t)k], y.data() + (size_t)k * n);
            }
            break;
        }
        return m_result.get_last_value();
    }

    TimeSeries<FP>& get_result()
    {
        return m_result;
    }
    const TimeSeries<FP>& get_result() const
    {
        return m_result;
    }
    TimeSeries<FP>& get_flows()
    {
        return m_flows;
    }
    const TimeSeries<FP>& get_flows() const
    {
        return m_flows;
    }
    Model& get_model()
    {
        return m_model;
    }
    const Model& get_model() const
    {
        return m_model;
    }
    FP& get_dt()
    {
        return m_dt;
    }
    const FP& get_dt() const
    {
        return m_dt;
    }
    void set_integrator_core(const IntegratorCore& core)
    {
        m_core = core;
    }
    const IntegratorCore& get_integrator_core() const
    {
        return m_core;
    }
    /* The node's dynamic-NPI state when it runs in a graph simulation. */
    DynamicNPIState& get_dynamic_npi_state()
    {
        return m_npi;
    }
    const DynamicNPIState& get_dynamic_npi_state() const
    {
        return m_npi;
    }

private:
    Model m_model;
    TimeSeries<FP> m_result, m_flows;
    FP m_dt;
    IntegratorCore m_core;
    DynamicNPIState m_npi;
};

/* mio::simulate_flows (flow_simulation.h:104-121): {populations, flows}. */
template <typename FP = double>
std::vector<TimeSeries<FP>> simulate_flows(FP t0, FP tmax, FP dt, const Model<FP>& model,
                                           const IntegratorCore& core = ControlledStepperWrapper())
{
    FlowSimulation<FP> sim(model, t0, dt);
    sim.set_integrator_core(core);
    sim.advance(tmax);
    return {sim.get_result(), sim.get_flows()};
}

/* mio::simulate / osecir::simulate (simulation.h:99-110, model.h:385-390). */
template <typename FP = double>
TimeSeries<FP> simulate(FP t0, FP tmax, FP dt, const Model<FP>& model,
                        const IntegratorCore& core = ControlledStepperWrapper())
{
    Simulation<FP> sim(model, t0, dt);
    sim.set_integrator_core(core);
    sim.advance(tmax);
    return sim.get_result();
}

} // namespace osecir
} // namespace miogpu

#endif // MIOGPU_FACADE_OSECIR_H
