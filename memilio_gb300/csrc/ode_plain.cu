// ode_plain.cu — the plain FP64 node solver: one thread integrates one node
// instance over one exchange interval with the reference's adaptive
// integrators, stage vectors in a strided scratch buffer in HBM.
//
// It follows, step for step:
//   SystemIntegrator::advance            memilio/math/integrator.h:184-249
//   ControlledStepperWrapper::step       memilio/math/stepper_wrapper.h:112-163 (Cash-Karp 5(4),
//                                        Odeint controller rules: err norm, shrink 0.9 err^-1/3 >= 0.2,
//                                        grow 0.9 max(err,5^-5)^-1/5 below 0.5, dt_max by a failed try)
//   RKIntegratorCore::step               memilio/math/adapt_rk.h:217-298 (RKF45)
#include "mgpu_internal.cuh"

#include <mutex>

namespace mgpu
{
namespace
{

// Cash-Karp 5(4) tableau (Cash & Karp 1990).
__device__ __constant__ const double ck_c[6]    = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
__device__ __constant__ const double ck_a[6][5] = {
    {0, 0, 0, 0, 0},
    {1.0 / 5.0, 0, 0, 0, 0},
    {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0},
    {3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0, 0, 0},
    {-11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0, 0},
    {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
__device__ __constant__ const double ck_b5[6] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
__device__ __constant__ const double ck_db[6] = {
    37.0 / 378.0 - 2825.0 / 27648.0, 0.0, 250.0 / 621.0 - 18575.0 / 48384.0, 125.0 / 594.0 - 13525.0 / 55296.0,
    0.0 - 277.0 / 14336.0, 512.0 / 1771.0 - 1.0 / 4.0};

// RKF45 tableau (memilio/math/adapt_rk.h:47-138).
__device__ __constant__ const double rkf_c[6]    = {0.0, 0.25, 3.0 / 8.0, 12.0 / 13.0, 1.0, 0.5};
__device__ __constant__ const double rkf_a[6][5] = {{0, 0, 0, 0, 0},
                                                    {0.25, 0, 0, 0, 0},
                                                    {3.0 / 32.0, 9.0 / 32.0, 0, 0, 0},
                                                    {1932.0 / 2197.0, -7200.0 / 2197.0, 7296.0 / 2197.0, 0, 0},
                                                    {439.0 / 216.0, -8.0, 3680.0 / 513.0, -845.0 / 4104.0, 0},
                                                    {-8.0 / 27.0, 2.0, -3544.0 / 2565.0, 1859.0 / 4104.0, -11.0 / 40.0}};
__device__ __constant__ const double rkf_low[6]  = {25.0 / 216.0, 0.0, 1408.0 / 2565.0, 2197.0 / 4104.0, -0.2, 0.0};
__device__ __constant__ const double rkf_high[6] = {16.0 / 135.0, 0.0, 6656.0 / 12825.0, 28561.0 / 56430.0,
                                                    -9.0 / 50.0, 2.0 / 55.0};

struct StepCounts {
    int accepted = 0, rejected = 0, failed = 0;
};

// Work vectors of one thread: k0..k5, a stage state and the next state.
struct Work {
    SVec k[6];
    SVec xt;
    SVec y;  // current state (in place)
    SVec yn; // next state
};

struct NodeRhs {
    NodeModel nm;
    __device__ void operator()(const SVec& x, double t, const SVec& out) const
    {
        secir_rhs(nm, x, x, t, out);
    }
};

// FlowSimulation's right-hand side (compartments/flow_simulation.h:56-79): the
// state is the accumulated flows; the population is the initial population
// plus the flows scattered to their compartments (FlowModel::get_derivatives),
// and the derivative is get_flows(pop, pop, t).
struct FlowRhs {
    NodeModel nm;
    const double* pop0; // initial population [10G]
    __device__ void operator()(const SVec& x, double t, const SVec& out) const
    {
        double pop[MGPU_MAX_GROUPS * kC];
        const int G = nm.G;
        for (int j = 0; j < G * kC; ++j) {
            pop[j] = 0.0;
        }
        for (int i = 0; i < G; ++i) {
#pragma unroll
            for (int k = 0; k < kF; ++k) {
                const double f = x[i * kF + k];
                pop[i * kC + kFlowSrc[k]] -= f;
                pop[i * kC + kFlowDst[k]] += f;
            }
        }
        for (int j = 0; j < G * kC; ++j) {
            pop[j] += pop0[j];
        }
        const CVec p{pop, 1};
        secir_flows(nm, p, p, t, out);
    }
};

// One Cash-Karp attempt; returns Odeint's error measure (writes the 5th-order result into w.yn).
// F: the right-hand side, f(x, t, out) (NodeRhs; FlowRhs for flow simulations).
template <class F>
__device__ double ck_attempt(const F& f, Work& w, int n, double t, double dt, const DevOpts& o)
{
    f(w.y, t, w.k[0]);
    for (int s = 1; s < 6; ++s) {
        for (int i = 0; i < n; ++i) {
            double v = w.y[i];
            for (int j = 0; j < s; ++j) {
                v = v + (ck_a[s][j] * dt) * w.k[j][i];
            }
            w.xt[i] = v;
        }
        f(w.xt, t + ck_c[s] * dt, w.k[s]);
    }
    double err = 0.0;
    for (int i = 0; i < n; ++i) {
        double v = w.y[i];
        double e = 0.0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const double kj = w.k[j][i];
            v               = v + (ck_b5[j] * dt) * kj;
            e               = e + (ck_db[j] * dt) * kj;
        }
        w.yn[i]        = v;
        const double r = fabs(e) / (o.abs_tol + o.rel_tol * (fabs(w.y[i]) + dt * fabs(w.k[0][i])));
        err            = fmax(err, r);
    }
    return err;
}

// ControlledStepperWrapper::step. On return w.yn holds y(t').
template <class F>
__device__ bool ck_step(const F& f, Work& w, int n, double& t, double& dt, double dt_min, const DevOpts& o,
                        StepCounts& c)
{
    bool success     = false;
    bool is_dt_valid = true;
    while (!success && is_dt_valid) {
        if (dt < dt_min) {
            is_dt_valid = false;
            dt          = dt_min;
        }
        if (o.dt_max != 0.0 && fabs(dt) > o.dt_max) {
            dt = o.dt_max;
            ++c.rejected;
            continue;
        }
        const double err = ck_attempt(f, w, n, t, dt, o);
        if (err > 1.0) {
            dt *= fmax(0.9 * pow(err, -1.0 / 3.0), 0.2);
            if (o.dt_max != 0.0) {
                dt = fmin(dt, o.dt_max);
            }
            ++c.rejected;
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
        ++c.failed;
        return false;
    }
    ++c.accepted;
    return true;
}

// RKIntegratorCore::step (RKF45, lower order propagated).
template <class F>
__device__ bool rkf_step(const F& f, Work& w, int n, double& t, double& dt, double dt_min, const DevOpts& o,
                         StepCounts& c)
{
    dt                 = fmin(dt, o.dt_max);
    bool converged     = false;
    bool dt_is_invalid = false;
    while (!converged && !dt_is_invalid) {
        if (dt < dt_min) {
            dt_is_invalid = true;
            dt            = dt_min;
        }
        f(w.y, t, w.k[0]);
        for (int s = 1; s < 6; ++s) {
            double t_eval = t;
            t_eval += rkf_c[s] * dt;
            for (int i = 0; i < n; ++i) {
                double v = w.y[i];
                for (int j = 0; j < s; ++j) {
                    v += (dt * rkf_a[s][j]) * w.k[j][i];
                }
                w.xt[i] = v;
            }
            f(w.xt, t_eval, w.k[s]);
        }
        double minratio = INFINITY;
        converged       = true;
        for (int i = 0; i < n; ++i) {
            double lo = 0.0, d = 0.0;
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                const double kj = w.k[j][i];
                lo += kj * rkf_low[j];
                d += kj * (rkf_high[j] - rkf_low[j]);
            }
            const double yn  = w.y[i] + dt * lo;
            w.yn[i]          = yn;
            const double est = dt * fabs(d);
            const double eps = o.abs_tol + fabs(yn) * o.rel_tol;
            converged        = converged && (est <= eps);
            minratio         = fmin(minratio, eps / est);
        }
        if (converged || dt_is_invalid) {
            t += dt;
        }
        else {
            ++c.rejected;
        }
        double dt_new = dt * pow(minratio, 1.0 / 5.0);
        dt_new *= 0.9;
        dt = fmin(dt_new, o.dt_max);
    }
    dt = fmax(dt, dt_min);
    if (converged) {
        ++c.accepted;
    }
    else {
        ++c.failed;
    }
    return converged;
}

// SystemIntegrator::advance for one node; y advanced in place. `rec` is
// called after every step with (t, y). Returns false when the step cap hit.
template <class F, class Rec>
__device__ bool system_advance(const F& f, Work& w, int n, double tmax, double& t, double& dt, const DevOpts& o,
                               StepCounts& c, Rec rec)
{
    const double t0       = t;
    double dt_restore     = 0.0;
    double dt_min         = o.dt_min;
    int steps             = 0;
    while (fabs((tmax - t) / (tmax - t0)) > kZeroTol) {
        if (steps++ >= o.max_steps) {
            return false;
        }
        if (dt > tmax - t) {
            dt_restore = dt;
            dt         = tmax - t;
            dt_min     = fmin(tmax - t, dt_min);
        }
        if (o.method == MGPU_METHOD_RKF45) {
            rkf_step(f, w, n, t, dt, dt_min, o, c);
        }
        else {
            ck_step(f, w, n, t, dt, dt_min, o, c);
        }
        for (int i = 0; i < n; ++i) {
            w.y[i] = w.yn[i];
        }
        rec(t, w.y);
    }
    dt = fmax(dt, dt_restore);
    return true;
}

__device__ Work make_work(const BatchDev& B, int64_t slot, double* y_row, int n_max)
{
    Work w;
    const int64_t S = B.scratch_stride;
    double* base    = B.scratch + slot;
    for (int q = 0; q < 6; ++q) {
        w.k[q] = SVec{base + (int64_t)q * n_max * S, S};
    }
    w.xt = SVec{base + (int64_t)6 * n_max * S, S};
    w.yn = SVec{base + (int64_t)7 * n_max * S, S};
    w.y  = SVec{y_row, 1};
    return w;
}

__device__ void add_counts(const BatchDev& B, const StepCounts& c)
{
    if (c.accepted) {
        atomicAdd(&B.counters[CNT_ACCEPTED], (unsigned long long)c.accepted);
    }
    if (c.rejected) {
        atomicAdd(&B.counters[CNT_REJECTED], (unsigned long long)c.rejected);
    }
    if (c.failed) {
        atomicAdd(&B.counters[CNT_FAILED], (unsigned long long)c.failed);
    }
}

// One exchange interval of every active node in [node_begin, node_end).
__global__ void k_ode_plain(BatchDev B, int64_t node_begin, int64_t node_end, int n_max)
{
    const int64_t node = node_begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= node_end) {
        return;
    }
    const int gi      = B.node_graph[node];
    const DevGraph& g = B.graphs[gi];
    const GraphRt& rt = B.rt[gi];
    if (!rt.active) {
        return;
    }
    const int64_t local = node - g.node0;
    NodeRhs f{node_model(B, g, local)};
    double* y = B.state + g.state_off + local * g.n;
    Work w    = make_work(B, node - node_begin, y, n_max);
    DevOpts o = B.opts;
    o.method  = g.method;
    StepCounts c;
    double t  = B.node_t[node];
    double dt = B.node_dt[node];
    const bool ok =
        system_advance(f, w, g.n, rt.t_next, t, dt, o, c, [](double, const SVec&) {});
    B.node_t[node]  = t;
    B.node_dt[node] = dt;
    bool nonfinite  = false;
    for (int i = 0; i < g.n; ++i) {
        if (!isfinite(y[i])) {
            nonfinite = true;
            break;
        }
    }
    report_instance_failure(B, gi, !ok, nonfinite);
    add_counts(B, c);
}

// Single-node simulate() with every accepted step recorded.
// dt_io (may be null): per-node initial step on entry, the integrator's next
// step on exit (Simulation::get_dt), instead of dt0.
__global__ void k_simulate(BatchDev B, const int32_t* nodes, int count, double t0, double tmax, double dt0,
                           int max_points, double* out_t, double* out_y, int32_t* num_points, int n_max,
                           double* dt_io)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) {
        return;
    }
    const DevGraph& g   = B.graphs[0];
    const int64_t local = nodes[k];
    NodeRhs f{node_model(B, g, local)};
    // the state row lives in the output buffer; start from the initial value
    double* ys          = out_y + (int64_t)k * max_points * g.n;
    const double* init  = B.state + g.state_off + local * g.n;
    double* y           = B.ynew + (int64_t)k * g.n;
    for (int i = 0; i < g.n; ++i) {
        y[i]  = init[i];
        ys[i] = init[i];
    }
    double* ts = out_t + (int64_t)k * max_points;
    ts[0]      = t0;
    int np     = 1;
    bool full  = false;
    Work w     = make_work(B, k, y, n_max);
    DevOpts o  = B.opts;
    o.method   = g.method;
    StepCounts c;
    double t  = t0;
    double dt = dt_io ? dt_io[k] : dt0;
    const int n = g.n;
    auto rec  = [&](double tt, const SVec& v) {
        if (np >= max_points) {
            full = true;
            return;
        }
        ts[np] = tt;
        for (int i = 0; i < n; ++i) {
            ys[(int64_t)np * n + i] = v[i];
        }
        ++np;
    };
    if (tmax > t0) {
        if (!system_advance(f, w, n, tmax, t, dt, o, c, rec)) {
            atomicOr(B.err, ERR_STEP_CAP);
        }
    }
    num_points[k] = full ? -np : np;
    if (dt_io) {
        dt_io[k] = dt;
    }
    add_counts(B, c);
}

// simulate_flows (flow_simulation.h:104-121): FlowSimulation::advance from zero
// flows with every accepted step recorded; the populations of every time point
// are the initial population plus the scattered flows
// (compute_population_results, flow_simulation_base.h:90-103).
__global__ void k_simulate_flows(BatchDev B, const int32_t* nodes, int count, double t0, double tmax, double dt0,
                                 int max_points, double* out_t, double* out_f, double* out_y, int32_t* num_points,
                                 int nf_max, double* flow_rows)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) {
        return;
    }
    const DevGraph& g   = B.graphs[0];
    const int64_t local = nodes[k];
    const int n         = g.n;
    const int nf        = g.G * kF;
    const double* pop0  = B.state + g.state_off + local * n;
    FlowRhs f{node_model(B, g, local), pop0};
    double* x = flow_rows + (int64_t)k * nf;
    for (int i = 0; i < nf; ++i) {
        x[i] = 0.0;
    }
    double* ts = out_t + (int64_t)k * max_points;
    double* fs = out_f + (int64_t)k * max_points * nf;
    double* ys = out_y + (int64_t)k * max_points * n;
    int np     = 0;
    bool full  = false;
    auto rec   = [&](double tt, const SVec& v) {
        if (np >= max_points) {
            full = true;
            return;
        }
        ts[np] = tt;
        double* yrow = ys + (int64_t)np * n;
        for (int j = 0; j < n; ++j) {
            yrow[j] = 0.0;
        }
        for (int i = 0; i < g.G; ++i) {
            for (int q = 0; q < kF; ++q) {
                const double fl = v[i * kF + q];
                fs[(int64_t)np * nf + i * kF + q] = fl;
                yrow[i * kC + kFlowSrc[q]] -= fl;
                yrow[i * kC + kFlowDst[q]] += fl;
            }
        }
        for (int j = 0; j < n; ++j) {
            yrow[j] += pop0[j];
        }
        ++np;
    };
    Work w    = make_work(B, k, x, nf_max);
    DevOpts o = B.opts;
    o.method  = g.method;
    StepCounts c;
    double t  = t0;
    double dt = dt0;
    rec(t, SVec{x, 1});
    if (tmax > t0) {
        if (!system_advance(f, w, nf, tmax, t, dt, o, c, rec)) {
            atomicOr(B.err, ERR_STEP_CAP);
        }
    }
    num_points[k] = full ? -np : np;
    add_counts(B, c);
}

__global__ void k_eval_rhs(BatchDev B, const int32_t* nodes, int count, const double* pop, const double* y,
                           const double* t, double* dydt)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) {
        return;
    }
    const DevGraph& g = B.graphs[0];
    NodeModel nm      = node_model(B, g, nodes[k]);
    const int64_t o   = (int64_t)k * g.n;
    secir_rhs(nm, CVec{pop + o, 1}, CVec{y + o, 1}, t[k], SVec{dydt + o, 1});
}

} // namespace

void launch_ode_plain(const BatchDev& B, int64_t node_begin, int64_t node_end, cudaStream_t s)
{
    const int64_t count = node_end - node_begin;
    if (count <= 0) {
        return;
    }
    const int threads = 128;
    const int blocks  = (int)((count + threads - 1) / threads);
    k_ode_plain<<<blocks, threads, 0, s>>>(B, node_begin, node_end, B.scratch_nmax);
}

void launch_simulate(const BatchDev& B, const int32_t* d_nodes, int count, double t0, double tmax, double dt0,
                     int max_points, double* d_out_t, double* d_out_y, int32_t* d_num_points, cudaStream_t s,
                     double* d_dt_io)
{
    const int threads = 64;
    const int blocks  = (count + threads - 1) / threads;
    k_simulate<<<blocks, threads, 0, s>>>(B, d_nodes, count, t0, tmax, dt0, max_points, d_out_t, d_out_y,
                                          d_num_points, B.scratch_nmax, d_dt_io);
}

void launch_simulate_flows(const BatchDev& B, const int32_t* d_nodes, int count, double t0, double tmax, double dt0,
                           int max_points, double* d_out_t, double* d_out_f, double* d_out_y, int32_t* d_num_points,
                           int nf_max, double* d_flow_rows, cudaStream_t s)
{
    const int threads = 64;
    const int blocks  = (count + threads - 1) / threads;
    k_simulate_flows<<<blocks, threads, 0, s>>>(B, d_nodes, count, t0, tmax, dt0, max_points, d_out_t, d_out_f,
                                                d_out_y, d_num_points, nf_max, d_flow_rows);
}

void launch_eval_rhs(const BatchDev& B, const int32_t* d_nodes, int count, const double* d_pop, const double* d_y,
                     const double* d_t, double* d_dydt, cudaStream_t s)
{
    const int threads = 128;
    const int blocks  = (count + threads - 1) / threads;
    k_eval_rhs<<<blocks, threads, 0, s>>>(B, d_nodes, count, d_pop, d_y, d_t, d_dydt);
}

} // namespace mgpu

// ---- allocation-free single-node simulate (mgpu_simulate_final_noalloc) ------
// The stage vectors live in a fixed array of this file instead of a buffer
// allocated per call; the kernel is k_simulate's integration (same device
// functions, same compile flags) without the step recording.

namespace mgpu
{
namespace
{

constexpr int64_t kNoallocScratchDoubles = MGPU_NOALLOC_SCRATCH_BYTES / (int64_t)sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

__global__ void k_simulate_final(BatchDev B, DevGraph g, int count, double t0, double tmax, double dt0,
                                 double* y_out, int32_t* status)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) {
        return;
    }
    const int n        = g.n;
    NodeRhs f{node_model(B, g, k)};
    const double* init = B.state + (int64_t)k * n;
    double* y          = y_out + (int64_t)k * n;
    if (y != init) {
        for (int i = 0; i < n; ++i) {
            y[i] = init[i];
        }
    }
    Work w    = make_work(B, k, y, n);
    DevOpts o = B.opts;
    o.method  = g.method;
    StepCounts c;
    double t  = t0;
    double dt = dt0;
    int32_t st = 0;
    if (tmax > t0 && !system_advance(f, w, n, tmax, t, dt, o, c, [](double, const SVec&) {})) {
        st |= 1;
    }
    for (int i = 0; i < n; ++i) {
        if (!isfinite(y[i])) {
            st |= 2;
            break;
        }
    }
    status[k] = st;
}

// Device address of the work space, looked up once per device.
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_addr[kNoallocMaxDevices] = {};

cudaError_t noalloc_scratch(int device, double** out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void* p            = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            return e;
        }
        g_noalloc_addr[device] = static_cast<double*>(p);
    }
    *out = g_noalloc_addr[device];
    return cudaSuccess;
}

} // namespace
} // namespace mgpu

extern "C" int mgpu_simulate_final_noalloc(mgpu_context* ctx, int32_t num_groups, int32_t num_contact_matrices,
                                           int32_t num_damping_points, int32_t count, const double* params,
                                           const double* contact, const double* damping_times,
                                           const double* damping_values, const double* y0, double t0, double tmax,
                                           double dt0, const mgpu_integrator_opts* opts, double* y_out,
                                           int32_t* status)
{
    using namespace mgpu;
    if (!ctx || !opts || count < 0 || num_groups < 1 || !(dt0 > 0)) {
        return MGPU_INVALID_VALUE;
    }
    if (num_groups > MGPU_MAX_GROUPS || num_contact_matrices < 1 ||
        num_contact_matrices > MGPU_MAX_CONTACT_MATRICES ||
        (opts->method != MGPU_METHOD_CASH_KARP54 && opts->method != MGPU_METHOD_RKF45)) {
        return MGPU_UNSUPPORTED;
    }
    if (num_damping_points < 0 || num_damping_points == 1) {
        return MGPU_INVALID_VALUE;
    }
    if (count == 0) {
        return MGPU_OK;
    }
    if (!params || !contact || !y0 || !y_out || !status ||
        (num_damping_points > 0 && (!damping_times || !damping_values))) {
        return MGPU_INVALID_VALUE;
    }
    const int n = num_groups * kC;
    // 8 stage vectors of n doubles per node
    if ((int64_t)8 * n * count > kNoallocScratchDoubles) {
        return MGPU_OUT_OF_RANGE;
    }
    int device          = 0;
    cudaStream_t stream = nullptr;
    if (context_device_stream(ctx, &device, &stream) != 0 || device < 0 || device >= kNoallocMaxDevices) {
        return MGPU_INVALID_VALUE;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    double* scratch = nullptr;
    if (noalloc_scratch(device, &scratch) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    DevGraph g{};
    g.N      = count;
    g.G      = num_groups;
    g.M      = num_contact_matrices;
    g.K      = num_damping_points;
    g.n      = n;
    g.method = opts->method;
    BatchDev B{};
    B.params         = params;
    B.contact        = contact;
    B.dtimes         = num_damping_points ? damping_times : nullptr;
    B.dvals          = num_damping_points ? damping_values : nullptr;
    B.state          = const_cast<double*>(y0); // read only
    B.scratch        = scratch;
    B.scratch_stride = count;
    B.scratch_nmax   = n;
    B.opts.abs_tol   = opts->abs_tol;
    B.opts.rel_tol   = opts->rel_tol;
    B.opts.dt_min    = opts->dt_min;
    B.opts.dt_max    = opts->dt_max;
    B.opts.max_steps = 100000;
    B.opts.method    = opts->method;
    const int threads = 64;
    const int blocks  = (count + threads - 1) / threads;
    // cudaLaunchKernel reports this launch's own status; an error that an
    // earlier, unrelated launch of the caller left pending stays the caller's
    void* args[] = {&B, &g, &count, &t0, &tmax, &dt0, &y_out, &status};
    const cudaError_t e =
        cudaLaunchKernel(reinterpret_cast<const void*>(&k_simulate_final), dim3(blocks), dim3(threads), args, 0, stream);
    return e == cudaSuccess ? MGPU_OK : MGPU_CUDA_ERROR;
}
