// miogpu/dynamic_npis.h — dynamic NPIs of the C++ facade: thresholds on the
// symptomatic infections that enact contact dampings at run time
// (mio::DynamicNPIs, memilio/epidemiology/dynamic_npis.h; mio::DampingSampling,
// memilio/epidemiology/damping_sampling.h). Host code: the enacted dampings
// change a node's damping cache, which the simulations hand to libmiogpu.
#ifndef MIOGPU_FACADE_DYNAMIC_NPIS_H
#define MIOGPU_FACADE_DYNAMIC_NPIS_H

#include "core.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <utility>
#include <vector>

namespace miogpu
{

/* One NPI of a threshold (DampingSampling, damping_sampling.h): a damping of
 * `value` times the group weights on the listed contact matrices. */
template <typename FP = double>
class DampingSampling
{
public:
    DampingSampling(double value, DampingLevel level, DampingType type, SimulationTime<double> time,
                    std::vector<size_t> matrices, std::vector<double> group_weights)
        : m_value(value)
        , m_level(level)
        , m_type(type)
        , m_time(time)
        , m_matrices(std::move(matrices))
        , m_groups(std::move(group_weights))
    {
    }
    double get_value() const
    {
        return m_value;
    }
    DampingLevel get_level() const
    {
        return m_level;
    }
    DampingType get_type() const
    {
        return m_type;
    }
    SimulationTime<double> get_time() const
    {
        return m_time;
    }
    const std::vector<size_t>& get_matrix_indices() const
    {
        return m_matrices;
    }
    const std::vector<double>& get_group_weights() const
    {
        return m_groups;
    }

private:
    double m_value;
    DampingLevel m_level;
    DampingType m_type;
    SimulationTime<double> m_time;
    std::vector<size_t> m_matrices;
    std::vector<double> m_groups;
};

/* make_contact_damping_matrix (damping_sampling.h:282-288): the contact damping
 * of per-group damping values g, 1 - sqrt((1 - g_i) (1 - g_j)). */
inline Matrix make_contact_damping_matrix(const std::vector<double>& g)
{
    const size_t n = g.size();
    Matrix m(n, n);
    for (size_t i = 0; i < n; ++i) {
        for (size_t j = 0; j < n; ++j) {
            m(i, j) = 1.0 - std::sqrt((1.0 - g[i]) * (1.0 - g[j]));
        }
    }
    return m;
}

/* mio::DynamicNPIs (dynamic_npis.h:31-230): thresholds kept in descending order,
 * each with the NPIs to enact; duration, implementation delay, base value and
 * the directive window. */
template <typename FP = double>
class DynamicNPIs
{
public:
    using Threshold = std::pair<double, std::vector<DampingSampling<FP>>>;

    /* set_threshold: inserted in descending order, an equal threshold replaced. */
    void set_threshold(double threshold, const std::vector<DampingSampling<FP>>& dampings)
    {
        auto it = std::lower_bound(m_thresholds.begin(), m_thresholds.end(), threshold,
                                   [](const Threshold& t, double v) {
                                       return t.first > v;
                                   });
        if (it != m_thresholds.end() && it->first == threshold) {
            it->second = dampings;
        }
        else {
            m_thresholds.insert(it, Threshold(threshold, dampings));
        }
    }
    /* get_max_exceeded_threshold: the highest threshold below `value`, or end(). */
    typename std::vector<Threshold>::const_iterator get_max_exceeded_threshold(double value) const
    {
        return std::upper_bound(m_thresholds.begin(), m_thresholds.end(), value, [](double v, const Threshold& t) {
            return v > t.first;
        });
    }
    const std::vector<Threshold>& get_thresholds() const
    {
        return m_thresholds;
    }
    SimulationTime<double> get_duration() const
    {
        return m_duration;
    }
    void set_duration(SimulationTime<double> v)
    {
        m_duration = v;
    }
    SimulationTime<double> get_implementation_delay() const
    {
        return m_delay;
    }
    void set_implementation_delay(SimulationTime<double> v)
    {
        if (v.get() < 0.0) {
            throw std::invalid_argument("implementation delay must be non-negative");
        }
        m_delay = v;
    }
    double get_base_value() const
    {
        return m_base;
    }
    void set_base_value(double v)
    {
        m_base = v;
    }
    SimulationTime<double> get_directive_begin() const
    {
        return m_directive_begin;
    }
    void set_directive_begin(SimulationTime<double> v)
    {
        m_directive_begin = v;
    }
    SimulationTime<double> get_directive_end() const
    {
        return m_directive_end;
    }
    void set_directive_end(SimulationTime<double> v)
    {
        m_directive_end = v;
    }

private:
    std::vector<Threshold> m_thresholds;
    SimulationTime<double> m_duration{14.0};
    SimulationTime<double> m_delay{0.0};
    SimulationTime<double> m_directive_begin{std::numeric_limits<double>::lowest()};
    SimulationTime<double> m_directive_end{std::numeric_limits<double>::max()};
    double m_base = 1.0;
};

/* get_damping_indices (dynamic_npis.h:232-244): dampings of (level, type) with
 * begin < time < end. */
inline std::vector<size_t> get_damping_indices(const DampingMatrixExpression& e, DampingLevel lvl, DampingType type,
                                               SimulationTime<double> begin, SimulationTime<double> end)
{
    std::vector<size_t> idx;
    const Dampings& d = e.get_dampings();
    for (size_t i = 0; i < d.size(); ++i) {
        if (d[i].level == lvl && d[i].type == type && d[i].time.get() > begin.get() && d[i].time.get() < end.get()) {
            idx.push_back(i);
        }
    }
    return idx;
}

/* get_active_damping (dynamic_npis.h:246-258): the matrix of the last damping
 * of (level, type) at or before t, zero if none. */
inline Matrix get_active_damping(const DampingMatrixExpression& e, DampingLevel lvl, DampingType type,
                                 SimulationTime<double> t)
{
    const Dampings& d = e.get_dampings();
    for (size_t k = d.size(); k-- > 0;) {
        if (d[k].level == lvl && d[k].type == type && d[k].time.get() <= t.get()) {
            return d[k].values;
        }
    }
    return Matrix::Zero(d.rows(), d.cols());
}

namespace detail
{
inline Matrix elementwise_max(const Matrix& a, const Matrix& b)
{
    Matrix m = a;
    for (size_t i = 0; i < m.size(); ++i) {
        m[i] = std::max(a[i], b[i]);
    }
    return m;
}
inline bool any_less(const Matrix& a, const Matrix& b)
{
    for (size_t i = 0; i < a.size(); ++i) {
        if (a[i] < b[i]) {
            return true;
        }
    }
    return false;
}
inline bool equal(const Matrix& a, const Matrix& b)
{
    for (size_t i = 0; i < a.size(); ++i) {
        if (a[i] != b[i]) {
            return false;
        }
    }
    return true;
}
} // namespace detail

/* implement_dynamic_npis (dynamic_npis.h:335-391) for contact matrices: every
 * NPI raises the active damping of its (level, type) to at least its value over
 * [begin, end) and restores the previous one at end; afterwards dampings that
 * repeat the previous value of their (level, type) are removed. */
template <typename FP, class Group, class MakeMatrix>
void implement_dynamic_npis(Group& group, const std::vector<DampingSampling<FP>>& npis,
                            SimulationTime<double> begin, SimulationTime<double> end, MakeMatrix&& make_matrix)
{
    for (const auto& npi : npis) {
        for (size_t mat_idx : npi.get_matrix_indices()) {
            const DampingLevel level = npi.get_level();
            const DampingType type   = npi.get_type();
            DampingMatrixExpression& expr = group[mat_idx];
            const Matrix active           = get_active_damping(expr, level, type, begin);
            const Matrix active_end       = get_active_damping(expr, level, type, end);
            std::vector<double> g         = npi.get_group_weights();
            for (double& x : g) {
                x *= npi.get_value();
            }
            const Matrix value = make_matrix(g);
            bool implemented   = false;
            if (detail::any_less(active, value)) {
                expr.add_damping(detail::elementwise_max(value, active), level, type, begin);
                implemented = true;
            }
            for (size_t i : get_damping_indices(expr, level, type, begin, end)) {
                const Damping d = expr.get_dampings()[i];
                expr.add_damping(detail::elementwise_max(d.values, value), level, type, d.time);
                implemented = true;
            }
            if (implemented) {
                expr.add_damping(active_end, level, type, end);
            }
        }
    }
    // (the reference's loop over i with the size re-read after each removal)
    for (size_t m = 0; m < group.get_num_matrices(); ++m) {
        DampingMatrixExpression& expr = group[m];
        for (int i = 0; i < (int)expr.get_dampings().size() - 1; ++i) {
            const Dampings& d = expr.get_dampings();
            const size_t cur  = d.size() - 1 - (size_t)i;
            for (size_t k = cur; k-- > 0;) {
                if (d[k].level == d[cur].level && d[k].type == d[cur].type) {
                    if (detail::equal(d[cur].values, d[k].values)) {
                        expr.remove_damping(cur);
                    }
                    break;
                }
            }
        }
    }
}

template <typename FP>
void implement_dynamic_npis(ContactMatrixGroup& group, const std::vector<DampingSampling<FP>>& npis,
                            SimulationTime<double> begin, SimulationTime<double> end)
{
    implement_dynamic_npis(group, npis, begin, end, [](const std::vector<double>& g) {
        return make_contact_damping_matrix(g);
    });
}

/* make_mobility_damping_vector (damping_sampling.h:290-306): the per-group values
 * spread over each group's entries of a mobility coefficient vector of size n. */
inline Matrix make_mobility_damping_vector(size_t n, const std::vector<double>& g)
{
    Matrix m(n, 1);
    const size_t per = n / g.size();
    for (size_t i = 0; i < n; ++i) {
        m[i] = g[i / per];
    }
    return m;
}

/* floating_point_greater_equal (math/floating_point.h:136-139) with rel_tol = DBL_MIN. */
inline bool fp_greater_equal(double v1, double v2, double abs_tol)
{
    const double diff = v1 - v2;
    return !(diff < -(abs_tol + std::numeric_limits<double>::min() * std::max(std::abs(v1), std::abs(v2))));
}

/* The dynamic-NPI bookkeeping of one osecir::Simulation (model.h:289-367,
 * m_dynamic_npi): the active threshold and its end. */
struct DynamicNPIState {
    double threshold = std::numeric_limits<double>::lowest();
    double t_end     = 0.0;
    int enacted      = 0; // NPIs enacted so far (for inspection)
};

/* The check at the start of a chunk of osecir::Simulation::advance
 * (model.h:299-350): with `inf_rel` the relative symptomatic infections at t,
 * enact the NPIs of the highest exceeded threshold if it is stronger than the
 * active one or the active one expired. Returns true if the contacts changed. */
template <typename FP>
bool check_dynamic_npis(const DynamicNPIs<FP>& npis, DynamicNPIState& st, ContactMatrixGroup& contacts, double t,
                        double inf_rel)
{
    if (npis.get_thresholds().empty()) {
        return false;
    }
    const double delay     = t > 0 ? npis.get_implementation_delay().get() : 0.0;
    const double dir_begin = npis.get_directive_begin().get();
    const double dir_end   = npis.get_directive_end().get();
    if (!(fp_greater_equal(t, dir_begin, 1e-10) && t < dir_end)) {
        return false;
    }
    auto exceeded     = npis.get_max_exceeded_threshold(inf_rel * npis.get_base_value());
    const bool expired = fp_greater_equal(t, st.t_end, 1e-10);
    if (exceeded == npis.get_thresholds().end() || !(exceeded->first > st.threshold || expired)) {
        return false;
    }
    const bool renewal   = expired && !(exceeded->first > st.threshold);
    const double eff     = renewal ? 0.0 : delay;
    if (!(t + eff < dir_end)) {
        return false;
    }
    const double t_start = t + eff;
    const double t_end   = std::min(dir_end, t_start + npis.get_duration().get());
    st.threshold         = exceeded->first;
    st.t_end             = t_end;
    st.enacted += 1;
    const double t_start_damping = (!renewal && t_start > 0) ? t_start + 1.0 : t_start;
    implement_dynamic_npis(contacts, exceeded->second, SimulationTime<double>(t_start_damping),
                           SimulationTime<double>(t_end + 1.0));
    return true;
}

/* The dynamic-NPI check of a mobility edge at the start of its exchange
 * (MobilityEdge::apply_mobility, metapopulation_mobility_instant.h:549-566):
 * with `inf_rel` the relative symptomatic infections of the edge's source
 * before the exchange, enact the NPIs of the highest exceeded threshold on the
 * edge's coefficients over [t, t + duration) if they are stronger than the
 * active ones or those expired. Returns true if the coefficients changed. */
template <typename FP, class CoefficientGroup>
bool check_edge_dynamic_npis(const DynamicNPIs<FP>& npis, DynamicNPIState& st, CoefficientGroup& coeffs, double t,
                             double inf_rel)
{
    if (npis.get_thresholds().empty()) {
        return false;
    }
    auto exceeded      = npis.get_max_exceeded_threshold(inf_rel * npis.get_base_value());
    const bool expired = fp_greater_equal(t, st.t_end, 1e-10);
    if (exceeded == npis.get_thresholds().end() || !(exceeded->first > st.threshold || expired)) {
        return false;
    }
    const double t_end = t + npis.get_duration().get();
    st.threshold       = exceeded->first;
    st.t_end           = t_end;
    st.enacted += 1;
    const size_t n = coeffs[0].rows();
    implement_dynamic_npis(coeffs, exceeded->second, SimulationTime<double>(t), SimulationTime<double>(t_end),
                           [n](const std::vector<double>& g) {
                               return make_mobility_damping_vector(n, g);
                           });
    return true;
}

} // namespace miogpu

#endif
