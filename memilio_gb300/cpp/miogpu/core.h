/*
 * miogpu/core.h — host-side pieces of the C++ facade shared by the model and
 * the graph classes: errors, the per-device context, index and time types,
 * a dense matrix, dampings and their accumulated cache, and the time series.
 *
 * The names and argument meanings follow MEmilio's C++ API
 * (cpp/memilio/epidemiology/damping.h, contact_matrix.h,
 * cpp/memilio/utils/time_series.h) so that code written against MEmilio reads
 * the same; the facade lives in namespace miogpu and calls libmiogpu
 * (include/miogpu.h) for every computation on the hot path.
 */
#ifndef MIOGPU_FACADE_CORE_H
#define MIOGPU_FACADE_CORE_H

#include "miogpu.h"

#include <algorithm>
#include <cassert>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <limits>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace miogpu
{

/* A failed libmiogpu call: the status code (include/miogpu.h) and message. */
class Error : public std::runtime_error
{
public:
    Error(int code, const std::string& what)
        : std::runtime_error(what + " (status " + std::to_string(code) + ")")
        , m_code(code)
    {
    }
    int code() const
    {
        return m_code;
    }

private:
    int m_code;
};

/* The libmiogpu context of this process on one device, created on first use
 * and shared by all facade objects (one CUDA stream; calls are serialised). */
class Device
{
public:
    static mgpu_context* context(int device = 0)
    {
        struct Destroy {
            void operator()(mgpu_context* c) const
            {
                mgpu_destroy(c);
            }
        };
        static std::mutex mtx;
        static std::vector<std::unique_ptr<mgpu_context, Destroy>> ctxs;
        std::lock_guard<std::mutex> lock(mtx);
        if ((int)ctxs.size() <= device) {
            ctxs.resize((size_t)device + 1);
        }
        if (!ctxs[(size_t)device]) {
            mgpu_context* c = nullptr;
            const int rc    = mgpu_create(device, &c);
            if (rc != MGPU_OK) {
                throw Error(rc, "mgpu_create failed for device " + std::to_string(device));
            }
            ctxs[(size_t)device].reset(c);
        }
        return ctxs[(size_t)device].get();
    }
};

inline void check(int rc, mgpu_context* ctx, const char* what)
{
    if (rc != MGPU_OK) {
        throw Error(rc, std::string(what) + ": " + (ctx ? mgpu_last_error(ctx) : ""));
    }
}

/* Index of an age group (mio::AgeGroup). */
struct AgeGroup {
    explicit constexpr AgeGroup(size_t v = 0)
        : value(v)
    {
    }
    constexpr size_t get() const
    {
        return value;
    }
    explicit operator size_t() const
    {
        return value;
    }
    AgeGroup& operator++()
    {
        ++value;
        return *this;
    }
    AgeGroup operator++(int)
    {
        AgeGroup r = *this;
        ++value;
        return r;
    }
    friend bool operator<(AgeGroup a, AgeGroup b)
    {
        return a.value < b.value;
    }
    friend bool operator==(AgeGroup a, AgeGroup b)
    {
        return a.value == b.value;
    }
    friend bool operator!=(AgeGroup a, AgeGroup b)
    {
        return a.value != b.value;
    }
    size_t value;
};

struct DampingLevel {
    explicit constexpr DampingLevel(int v = 0)
        : value(v)
    {
    }
    constexpr int get() const
    {
        return value;
    }
    friend constexpr bool operator==(DampingLevel a, DampingLevel b)
    {
        return a.value == b.value;
    }
    friend constexpr bool operator!=(DampingLevel a, DampingLevel b)
    {
        return a.value != b.value;
    }
    int value;
};

struct DampingType {
    explicit constexpr DampingType(int v = 0)
        : value(v)
    {
    }
    constexpr int get() const
    {
        return value;
    }
    friend constexpr bool operator==(DampingType a, DampingType b)
    {
        return a.value == b.value;
    }
    friend constexpr bool operator!=(DampingType a, DampingType b)
    {
        return a.value != b.value;
    }
    int value;
};

template <typename FP = double>
struct SimulationTime {
    explicit constexpr SimulationTime(FP v = 0)
        : value(v)
    {
    }
    constexpr FP get() const
    {
        return value;
    }
    FP value;
};

/* Dense row-major matrix (the role Eigen::MatrixX plays in MEmilio). A vector
 * is a matrix with one column. */
class Matrix
{
public:
    Matrix() = default;
    Matrix(size_t rows, size_t cols, double v = 0.0)
        : m_rows(rows)
        , m_cols(cols)
        , m_data(rows * cols, v)
    {
    }
    static Matrix Constant(size_t rows, size_t cols, double v)
    {
        return Matrix(rows, cols, v);
    }
    static Matrix Zero(size_t rows, size_t cols)
    {
        return Matrix(rows, cols, 0.0);
    }
    size_t rows() const
    {
        return m_rows;
    }
    size_t cols() const
    {
        return m_cols;
    }
    size_t size() const
    {
        return m_data.size();
    }
    double& operator()(size_t r, size_t c)
    {
        return m_data[r * m_cols + c];
    }
    double operator()(size_t r, size_t c) const
    {
        return m_data[r * m_cols + c];
    }
    double& operator[](size_t i)
    {
        return m_data[i];
    }
    double operator[](size_t i) const
    {
        return m_data[i];
    }
    Matrix& setConstant(double v)
    {
        std::fill(m_data.begin(), m_data.end(), v);
        return *this;
    }
    Matrix& setZero()
    {
        return setConstant(0.0);
    }
    const double* data() const
    {
        return m_data.data();
    }
    double* data()
    {
        return m_data.data();
    }

private:
    size_t m_rows = 0, m_cols = 0;
    std::vector<double> m_data;
};

/* One damping: a matrix of factors active from `time` (mio::Damping). */
struct Damping {
    Matrix values;
    DampingLevel level;
    DampingType type;
    SimulationTime<double> time;
};

/* Dampings of one matrix (mio::Dampings, damping.h): kept sorted by (time,
 * type, level); adding one with an equal key replaces it (add_, :603-614). */
class Dampings
{
public:
    explicit Dampings(size_t rows = 0, size_t cols = 0)
        : m_rows(rows)
        , m_cols(cols)
    {
    }
    void add(const Matrix& m, DampingLevel level, DampingType type, SimulationTime<double> t)
    {
        if (m.rows() != m_rows || m.cols() != m_cols) {
            throw std::invalid_argument("damping shape does not match the matrix");
        }
        Damping d{m, level, type, t};
        auto key = [](const Damping& x) {
            return std::make_tuple(x.time.get(), x.type.get(), x.level.get());
        };
        auto it = std::lower_bound(m_list.begin(), m_list.end(), d, [&](const Damping& a, const Damping& b) {
            return key(a) < key(b);
        });
        if (it != m_list.end() && key(*it) == key(d)) {
            *it = d;
        }
        else {
            m_list.insert(it, d);
        }
    }
    void add(double v, DampingLevel level, DampingType type, SimulationTime<double> t)
    {
        add(Matrix::Constant(m_rows, m_cols, v), level, type, t);
    }
    void add(const Matrix& m, SimulationTime<double> t)
    {
        add(m, DampingLevel(0), DampingType(0), t);
    }
    void add(double v, SimulationTime<double> t)
    {
        add(v, DampingLevel(0), DampingType(0), t);
    }
    const std::vector<Damping>& list() const
    {
        return m_list;
    }
    size_t size() const
    {
        return m_list.size();
    }
    const Damping& operator[](size_t i) const
    {
        return m_list.at(i);
    }
    /* Dampings::remove (damping.h:336-340) */
    void remove(size_t i)
    {
        m_list.erase(m_list.begin() + (std::ptrdiff_t)i);
    }
    size_t rows() const
    {
        return m_rows;
    }
    size_t cols() const
    {
        return m_cols;
    }
    void clear()
    {
        m_list.clear();
    }

    /* The accumulated damping matrices of Dampings::update_cache
     * (damping.h:570-600): in time order, a new damping replaces the active one
     * of its (level, type); matrices of one level add up, levels combine as
     * 1 - prod(1 - d) (update_active_dampings :616-658, inclusive_exclusive_sum
     * :545-562). Points at equal times (within 1e-15) merge. The cache starts
     * with (-DBL_MAX, 0) and ends with (DBL_MAX, last). */
    void cache(std::vector<double>& times, std::vector<Matrix>& values) const
    {
        times.clear();
        values.clear();
        times.push_back(std::numeric_limits<double>::lowest());
        values.push_back(Matrix::Zero(m_rows, m_cols));
        struct Active {
            const Matrix* m;
            int level, type;
        };
        std::vector<Active> by_type;
        std::vector<std::pair<Matrix, int>> by_level;
        for (const Damping& d : m_list) {
            const int lv = d.level.get(), ty = d.type.get();
            auto lit     = std::find_if(by_level.begin(), by_level.end(), [&](const std::pair<Matrix, int>& x) {
                return x.second == lv;
            });
            auto tit     = std::find_if(by_type.begin(), by_type.end(), [&](const Active& a) {
                return a.level == lv && a.type == ty;
            });
            if (tit != by_type.end()) {
                for (size_t i = 0; i < d.values.size(); ++i) {
                    lit->first[i] += d.values[i] - (*tit->m)[i];
                }
                tit->m = &d.values;
            }
            else {
                by_type.push_back({&d.values, lv, ty});
                if (lit != by_level.end()) {
                    for (size_t i = 0; i < d.values.size(); ++i) {
                        lit->first[i] += d.values[i];
                    }
                }
                else {
                    by_level.emplace_back(d.values, lv);
                }
            }
            Matrix comb = by_level.front().first;
            for (size_t l = 1; l < by_level.size(); ++l) {
                for (size_t i = 0; i < comb.size(); ++i) {
                    const double other = by_level[l].first[i];
                    comb[i]            = comb[i] + other - comb[i] * other;
                }
            }
            const double tb   = times.back();
            const double diff = std::abs(d.time.get() - tb);
            if (diff <= 1e-15 || diff <= 1e-15 * std::max(std::abs(d.time.get()), std::abs(tb))) {
                values.back() = comb;
            }
            else {
                times.push_back(d.time.get());
                values.push_back(comb);
            }
        }
        times.push_back(std::numeric_limits<double>::max());
        values.push_back(values.back());
    }

private:
    size_t m_rows, m_cols;
    std::vector<Damping> m_list;
};

/* Baseline, minimum and dampings of one matrix (mio::DampingMatrixExpression):
 * M(t) = B - D(t) o (B - Min). */
class DampingMatrixExpression
{
public:
    DampingMatrixExpression(size_t rows = 0, size_t cols = 0)
        : m_baseline(rows, cols)
        , m_minimum(rows, cols)
        , m_dampings(rows, cols)
    {
    }
    explicit DampingMatrixExpression(const Matrix& baseline)
        : m_baseline(baseline)
        , m_minimum(baseline.rows(), baseline.cols())
        , m_dampings(baseline.rows(), baseline.cols())
    {
    }
    Matrix& get_baseline()
    {
        return m_baseline;
    }
    const Matrix& get_baseline() const
    {
        return m_baseline;
    }
    Matrix& get_minimum()
    {
        return m_minimum;
    }
    const Matrix& get_minimum() const
    {
        return m_minimum;
    }
    template <class... T>
    void add_damping(T&&... t)
    {
        m_dampings.add(std::forward<T>(t)...);
    }
    const Dampings& get_dampings() const
    {
        return m_dampings;
    }
    /* DampingMatrixExpression::remove_damping (contact_matrix.h:106-109) */
    void remove_damping(size_t i)
    {
        m_dampings.remove(i);
    }
    void clear_dampings()
    {
        m_dampings.clear();
    }
    size_t rows() const
    {
        return m_baseline.rows();
    }
    size_t cols() const
    {
        return m_baseline.cols();
    }

private:
    Matrix m_baseline, m_minimum;
    Dampings m_dampings;
};

using ContactMatrix = DampingMatrixExpression;

/* A sum of contact matrices (mio::ContactMatrixGroup, contact_matrix.h:392-399). */
class ContactMatrixGroup
{
public:
    ContactMatrixGroup(size_t num_matrices = 1, size_t num_groups = 1)
        : m_matrices(num_matrices, ContactMatrix(num_groups, num_groups))
    {
    }
    ContactMatrix& operator[](size_t i)
    {
        return m_matrices.at(i);
    }
    const ContactMatrix& operator[](size_t i) const
    {
        return m_matrices.at(i);
    }
    size_t get_num_matrices() const
    {
        return m_matrices.size();
    }
    size_t get_num_groups() const
    {
        return m_matrices.empty() ? 0 : m_matrices[0].rows();
    }
    template <class... T>
    void add_damping(T&&... t)
    {
        for (auto& m : m_matrices) {
            m.add_damping(std::forward<T>(t)...);
        }
    }
    /* ContactPatterns is an UncertainContactMatrix in MEmilio; its frequency matrix is this group. */
    ContactMatrixGroup& get_cont_freq_mat()
    {
        return *this;
    }
    const ContactMatrixGroup& get_cont_freq_mat() const
    {
        return *this;
    }

private:
    std::vector<ContactMatrix> m_matrices;
};

/* Damping caches of several matrices, padded to one point count K (extra
 * points at DBL_MAX repeat the last matrix), flattened [matrix][K] and
 * [matrix][K][rows*cols] as include/miogpu_layout.h expects. K = 0 when no
 * matrix has dampings. */
inline int flatten_damping_caches(const std::vector<const DampingMatrixExpression*>& ms, std::vector<double>& times,
                                  std::vector<double>& values)
{
    bool any = false;
    for (auto* m : ms) {
        any = any || !m->get_dampings().list().empty();
    }
    times.clear();
    values.clear();
    if (!any) {
        return 0;
    }
    std::vector<std::vector<double>> ts(ms.size());
    std::vector<std::vector<Matrix>> vs(ms.size());
    size_t K = 0;
    for (size_t i = 0; i < ms.size(); ++i) {
        ms[i]->get_dampings().cache(ts[i], vs[i]);
        K = std::max(K, ts[i].size());
    }
    for (size_t i = 0; i < ms.size(); ++i) {
        while (ts[i].size() < K) {
            ts[i].push_back(std::numeric_limits<double>::max());
            vs[i].push_back(vs[i].back());
        }
        times.insert(times.end(), ts[i].begin(), ts[i].end());
        for (auto& m : vs[i]) {
            values.insert(values.end(), m.data(), m.data() + m.size());
        }
    }
    return (int)K;
}

/* Time points with a value vector each (mio::TimeSeries, utils/time_series.h). */
template <typename FP = double>
class TimeSeries
{
public:
    explicit TimeSeries(size_t num_elements = 0)
        : m_n(num_elements)
    {
    }
    size_t get_num_elements() const
    {
        return m_n;
    }
    size_t get_num_time_points() const
    {
        return m_t.size();
    }
    void add_time_point(FP t, const FP* v)
    {
        m_t.push_back(t);
        m_v.insert(m_v.end(), v, v + m_n);
    }
    void add_time_point(FP t, const std::vector<FP>& v)
    {
        add_time_point(t, v.data());
    }
    FP get_time(size_t i) const
    {
        return m_t.at(i);
    }
    FP get_last_time() const
    {
        return m_t.back();
    }
    std::vector<FP> get_value(size_t i) const
    {
        return std::vector<FP>(m_v.begin() + (long)(i * m_n), m_v.begin() + (long)((i + 1) * m_n));
    }
    std::vector<FP> get_last_value() const
    {
        return get_value(m_t.size() - 1);
    }
    const FP* value_ptr(size_t i) const
    {
        return m_v.data() + i * m_n;
    }
    /* Index of the time point within 1e-10 of t, searching from the end, or -1
     * (find_value_reverse, time_series.h:904-914). */
    long find_time_reverse(FP t, FP abs_tol = 1e-10) const
    {
        for (size_t i = m_t.size(); i-- > 0;) {
            if (std::abs(m_t[i] - t) <= abs_tol) {
                return (long)i;
            }
        }
        return -1;
    }
    void clear()
    {
        m_t.clear();
        m_v.clear();
    }

private:
    size_t m_n;
    std::vector<FP> m_t;
    std::vector<FP> m_v;
};

/* interpolate_simulation_result (data/analyze_result.h:186-268): the values at
 * the given sorted times, linear between the neighbouring time points
 * (linear_interpolation, math/interpolation.h:44-48); a first (last) time at or
 * before (after) the series takes its first (last) value. */
template <typename FP>
TimeSeries<FP> interpolate_simulation_result(const TimeSeries<FP>& r, const std::vector<FP>& times)
{
    TimeSeries<FP> out(r.get_num_elements());
    if (times.empty() || r.get_num_time_points() == 0) {
        return out;
    }
    const size_t n = r.get_num_elements();
    size_t k       = 0;
    if (r.get_time(0) >= times[0]) {
        out.add_time_point(times[0], r.value_ptr(0));
        ++k;
    }
    std::vector<FP> v(n);
    for (size_t i = 0; i + 1 < r.get_num_time_points() && k < times.size();) {
        if (r.get_time(i) < times[k] && r.get_time(i + 1) >= times[k]) {
            const FP w    = (times[k] - r.get_time(i)) / (r.get_time(i + 1) - r.get_time(i));
            const FP* y1  = r.value_ptr(i);
            const FP* y2  = r.value_ptr(i + 1);
            for (size_t j = 0; j < n; ++j) {
                v[j] = y1[j] + w * (y2[j] - y1[j]);
            }
            out.add_time_point(times[k], v);
            ++k;
        }
        else {
            ++i;
        }
    }
    if (k < times.size() && r.get_last_time() < times[k]) {
        out.add_time_point(times[k], r.get_last_value());
    }
    return out;
}

/* The same at every whole day from ceil(t0 - abs_tol) to floor(tmax + abs_tol). */
template <typename FP>
TimeSeries<FP> interpolate_simulation_result(const TimeSeries<FP>& r, FP abs_tol = FP(100) * FP(1e-12))
{
    const int day0    = (int)std::ceil(r.get_time(0) - abs_tol);
    const int day_max = (int)std::floor(r.get_last_time() + abs_tol);
    std::vector<FP> tps;
    for (int d = day0; d <= day_max; ++d) {
        tps.push_back(FP(d));
    }
    return interpolate_simulation_result(r, tps);
}

/* The integrator core of a simulation (ControlledStepperWrapper with Cash-Karp
 * 5(4), stepper_wrapper.h:56-202, or RKIntegratorCore, adapt_rk.h). */
struct IntegratorCore {
    int method     = MGPU_METHOD_CASH_KARP54;
    double abs_tol = 1e-10, rel_tol = 1e-5, dt_min = DBL_MIN, dt_max = DBL_MAX;
    mgpu_integrator_opts opts() const
    {
        mgpu_integrator_opts o{};
        o.method  = method;
        o.abs_tol = abs_tol;
        o.rel_tol = rel_tol;
        o.dt_min  = dt_min;
        o.dt_max  = dt_max;
        return o;
    }
};

struct ControlledStepperWrapper : IntegratorCore {
    ControlledStepperWrapper(double abs = 1e-10, double rel = 1e-5, double dtmin = DBL_MIN, double dtmax = DBL_MAX)
    {
        method  = MGPU_METHOD_CASH_KARP54;
        abs_tol = abs;
        rel_tol = rel;
        dt_min  = dtmin;
        dt_max  = dtmax;
    }
};

struct RKIntegratorCore : IntegratorCore {
    RKIntegratorCore(double abs = 1e-10, double rel = 1e-5, double dtmin = DBL_MIN, double dtmax = DBL_MAX)
    {
        method  = MGPU_METHOD_RKF45;
        abs_tol = abs;
        rel_tol = rel;
        dt_min  = dtmin;
        dt_max  = dtmax;
    }
};

} // namespace miogpu

#endif // MIOGPU_FACADE_CORE_H
