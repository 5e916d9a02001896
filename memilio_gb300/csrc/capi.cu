// capi.cu — the extern "C" entry points of libmiogpu (include/miogpu.h):
// contexts, device upload of graph batches, and the exchange-interval
// schedule of GraphSimulation::advance.
#include "mgpu_internal.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <functional>
#include <limits>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <new>
#include <string>
#include <thread>
#include <vector>

using namespace mgpu;

struct mgpu_context {
    int device           = 0;
    cudaStream_t stream  = nullptr;
    std::string error    = "";
    int64_t budget       = 0; // 0 = free HBM
    int64_t allocated    = 0;
    // page-locked host staging of batch uploads, kept for the next batch (grown on demand)
    void* pinned         = nullptr;
    size_t pinned_bytes  = 0;
};

namespace
{
// Live batches of every context. mgpu_destroy releases a context's remaining
// batches first; destroying a batch that is no longer registered (destroyed
// already, or released with its context) does nothing.
std::mutex g_batches_mutex;
std::set<mgpu_batch*> g_batches;
} // namespace

int mgpu::context_device_stream(const mgpu_context* ctx, int* device, cudaStream_t* stream)
{
    if (!ctx) {
        return 1;
    }
    *device = ctx->device;
    *stream = ctx->stream;
    return 0;
}

namespace
{

struct Fail {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg)
{
    throw Fail{code, msg};
}

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        const int code = (e == cudaErrorMemoryAllocation) ? MGPU_OOM : MGPU_CUDA_ERROR;
        fail(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Device allocations owned by a batch or a call, stream-ordered on the
// context's stream (cudaMallocAsync / cudaFreeAsync): a release does not wait
// for the work of other streams, so batches created and destroyed while others
// run (the serving loop) do not stall them; freed blocks stay in the device's
// memory pool for the next batch.
struct DevPool {
    mgpu_context* ctx = nullptr;
    std::vector<std::pair<void*, int64_t>> blocks;
    int64_t bytes = 0;

    template <class T>
    T* alloc(int64_t count)
    {
        const int64_t nb = std::max<int64_t>(count, 1) * (int64_t)sizeof(T);
        if (ctx->budget > 0 && ctx->allocated + nb > ctx->budget) {
            fail(MGPU_OOM, "device memory budget exceeded (" + std::to_string(ctx->allocated + nb) + " > " +
                               std::to_string(ctx->budget) + " bytes)");
        }
        void* p = nullptr;
        const cudaError_t e = cudaMallocAsync(&p, nb, ctx->stream);
        if (e != cudaSuccess) {
            cudaGetLastError(); // an allocation failure leaves no error behind for later launch checks
            ck(e, "cudaMallocAsync");
        }
        blocks.emplace_back(p, nb);
        bytes += nb;
        ctx->allocated += nb;
        return static_cast<T*>(p);
    }
    template <class V>
    typename V::value_type* upload(const V& v)
    {
        using T = typename V::value_type;
        T* d    = alloc<T>((int64_t)v.size());
        if (!v.empty()) {
            ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream), "upload");
        }
        return d;
    }
    void release()
    {
        for (auto& b : blocks) {
            cudaFreeAsync(b.first, ctx->stream);
            ctx->allocated -= b.second;
        }
        blocks.clear();
        bytes = 0;
    }
};


// A typed view of part of the staging arena (the container interface that
// DevPool::upload and the packing code use).
template <class T>
struct HostSpan {
    using value_type = T;
    T* p     = nullptr;
    size_t n = 0;
    T* data() const
    {
        return p;
    }
    size_t size() const
    {
        return n;
    }
    bool empty() const
    {
        return n == 0;
    }
    T& operator[](size_t i) const
    {
        return p[i];
    }
};

// Host staging of one batch upload in the context's page-locked buffer: the
// arrays are laid out first (take), then placed in one block (place), so that
// the uploads run at the page-locked copy rate and need no zero fill.
struct StagingArena {
    mgpu_context* ctx;
    size_t bytes = 0;
    std::vector<std::pair<void**, size_t>> items;
    template <class T>
    void take(HostSpan<T>& s, int64_t count)
    {
        s.n = (size_t)std::max<int64_t>(count, 0);
        items.emplace_back(reinterpret_cast<void**>(&s.p), bytes);
        bytes += (s.n * sizeof(T) + 255) & ~(size_t)255;
    }
    void place()
    {
        if (bytes > ctx->pinned_bytes) {
            if (ctx->pinned) {
                ck(cudaFreeHost(ctx->pinned), "cudaFreeHost");
                ctx->pinned       = nullptr;
                ctx->pinned_bytes = 0;
            }
            ck(cudaHostAlloc(&ctx->pinned, bytes, cudaHostAllocDefault), "cudaHostAlloc");
            ctx->pinned_bytes = bytes;
        }
        for (auto& it : items) {
            *it.first = static_cast<char*>(ctx->pinned) + it.second;
        }
    }
};

// f(i) for i in [0, n) on the host's cores (chunks handed out in order); the
// first exception of any worker is rethrown here.
template <class F>
void parallel_for(int64_t n, F&& f)
{
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t T  = std::min<int64_t>(hw, n);
    if (T <= 1) {
        for (int64_t i = 0; i < n; ++i) {
            f(i);
        }
        return;
    }
    const int64_t chunk = std::max<int64_t>(1, n / (T * 8));
    std::atomic<int64_t> next{0};
    std::vector<std::exception_ptr> err(T);
    std::vector<std::thread> th;
    th.reserve(T);
    for (int64_t t = 0; t < T; ++t) {
        th.emplace_back([&, t]() {
            try {
                for (;;) {
                    const int64_t a = next.fetch_add(chunk);
                    if (a >= n) {
                        break;
                    }
                    const int64_t b = std::min(n, a + chunk);
                    for (int64_t i = a; i < b; ++i) {
                        f(i);
                    }
                }
            }
            catch (...) {
                err[t] = std::current_exception();
                next.store(n);
            }
        });
    }
    for (auto& x : th) {
        x.join();
    }
    for (auto& e : err) {
        if (e) {
            std::rethrow_exception(e);
        }
    }
}

// Counts and pointers of a graph (O(1)); the arrays are checked by validate_graph_arrays.
void validate_graph_header(const mgpu_graph& g)
{
    if (g.num_nodes < 0 || g.num_edges < 0) {
        fail(MGPU_INVALID_VALUE, "negative node or edge count");
    }
    if (g.num_groups < 1) {
        fail(MGPU_INVALID_VALUE, "num_groups must be >= 1");
    }
    if (g.num_groups > MGPU_MAX_GROUPS) {
        fail(MGPU_UNSUPPORTED, "num_groups > MGPU_MAX_GROUPS (" + std::to_string(MGPU_MAX_GROUPS) + ")");
    }
    if (g.num_contact_matrices < 1 || g.num_contact_matrices > MGPU_MAX_CONTACT_MATRICES) {
        fail(MGPU_UNSUPPORTED, "num_contact_matrices must be in [1, MGPU_MAX_CONTACT_MATRICES]");
    }
    if (g.num_damping_points < 0 || g.num_damping_points == 1 || g.num_edge_damping_points < 0 ||
        g.num_edge_damping_points == 1) {
        fail(MGPU_INVALID_VALUE, "a damping cache has 0 or >= 2 points");
    }
    if (g.num_nodes > 0 && (!g.params || !g.contact_baseline || !g.init_state)) {
        fail(MGPU_INVALID_VALUE, "params, contact_baseline and init_state are required");
    }
    if (g.num_damping_points > 0 && (!g.damping_times || !g.damping_values)) {
        fail(MGPU_INVALID_VALUE, "damping_times/values required when num_damping_points > 0");
    }
    if (g.num_edges > 0 && (!g.edge_src || !g.edge_dst || !g.edge_coeff_baseline)) {
        fail(MGPU_INVALID_VALUE, "edge_src, edge_dst and edge_coeff_baseline are required");
    }
    if (g.num_edge_damping_points > 0 && (!g.edge_damping_times || !g.edge_damping_values)) {
        fail(MGPU_INVALID_VALUE, "edge damping times/values required when num_edge_damping_points > 0");
    }
}

// Edge indices (range, no self-loops, sorted by (src, dst)) and damping cache times.
void validate_graph_arrays(const mgpu_graph& g, bool edges, bool dampings, bool need_edges_sorted)
{
    for (int e = 0; edges && e < g.num_edges; ++e) {
        const int s = g.edge_src[e], d = g.edge_dst[e];
        if (s < 0 || s >= g.num_nodes || d < 0 || d >= g.num_nodes) {
            fail(MGPU_OUT_OF_RANGE, "edge node index out of range");
        }
        if (s == d) {
            fail(MGPU_INVALID_VALUE, "self-loop edges are not supported");
        }
        if (need_edges_sorted && e > 0) {
            const int ps = g.edge_src[e - 1], pd = g.edge_dst[e - 1];
            if (ps > s || (ps == s && pd >= d)) {
                fail(MGPU_INVALID_VALUE, "edges must be sorted by (src, dst) without duplicates (graph.h:231-241)");
            }
        }
    }
    const int K = g.num_damping_points;
    if (dampings && K > 0) {
        const long GG = (long)g.num_groups * g.num_groups;
        for (long v = 0; v < (long)g.num_nodes * g.num_contact_matrices; ++v) {
            const double* T = g.damping_times + v * K;
            for (int k = 1; k < K; ++k) {
                if (!(T[k] >= T[k - 1])) {
                    fail(MGPU_INVALID_VALUE, "damping cache times must be non-decreasing");
                }
            }
            (void)GG;
        }
    }
}

} // namespace

struct mgpu_batch {
    mgpu_context* ctx = nullptr;
    mgpu_solver_opts opts{};
    DevPool pool;
    BatchDev dev{};
    int32_t num_graphs = 0;
    int64_t n_max      = 0;
    std::vector<int32_t> N, G, n;
    std::vector<int64_t> node0, edge0, state_off;
    std::vector<DevGraph> host_graphs; // the graph records as uploaded
    std::vector<char> damping_shared;  // damping arrays shared with another graph (same host pointers)
    std::vector<char> coeff_shared;    // edge coefficient arrays shared with another graph
    bool half_step     = false;        // an interval begun by mgpu_batch_step_nodes awaits its exchange
    std::vector<double> half_t_next;   // its end per graph
    int64_t state_total = 0;
    double* init_state  = nullptr; // initial states (for reset)
    float* init_hi      = nullptr; // the same as float-float pairs (mixed solver)
    float* init_lo      = nullptr;
    bool pairs          = false;   // node states are float-float pairs on the device
    double dt0          = 0.1;
    std::vector<double> t_host;  // mirror of rt.t
    std::vector<double> tmax_host;
    double* d_tmax = nullptr;
    double* d_out  = nullptr; // FP64 read-back buffer of float-float states (allocated on first read)
    double* d_sums = nullptr; // per-node compartment sums (allocated on first use)
    // batched solver work lists per age-group count
    std::map<int, std::pair<int32_t*, int64_t>> inst_by_G;
    int instances_per_block = 0;
    // autotuned schedule of the node solves per age-group count: {instances per block, grid blocks}
    std::map<int, std::pair<int, int>> tuned;
    bool any_edge_dampings  = false;
    int64_t launches        = 0;
    int64_t phases          = 0;
    int64_t seq_exchanges   = 0;
    // commuter statistics per graph (mgpu_batch_set_commuter_stats): descriptors as
    // uploaded to dev.estats, and the device buffers of all graphs that record
    std::vector<EdgeStatsDev> stats_host;
    DevPool stats_pool;
    // accumulated flows per (node, group) (mgpu_batch_set_flow_recording), kept once allocated
    double* flows_buf = nullptr;
    // CUDA graph of one batched interval
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_failed          = false;
    // asynchronous advance (mgpu_batch_launch / mgpu_batch_query)
    bool async_active   = false;
    int64_t async_left  = 0;
    std::vector<double> async_t_end;
    cudaEvent_t ev_async = nullptr;
    // timing
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    std::vector<cudaEvent_t> ev_phase;
    mgpu_timing timing{};

    ~mgpu_batch()
    {
        if (graph_exec) {
            cudaGraphExecDestroy(graph_exec);
        }
        for (auto e : ev_phase) {
            cudaEventDestroy(e);
        }
        if (ev_start) {
            cudaEventDestroy(ev_start);
        }
        if (ev_stop) {
            cudaEventDestroy(ev_stop);
        }
        if (ev_async) {
            cudaEventDestroy(ev_async);
        }
        stats_pool.release();
        pool.release();
    }

    // the captured interval holds the kernels' parameters: capture again after they change
    void drop_graph()
    {
        if (graph_exec) {
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
    }

    cudaEvent_t phase_event(size_t i)
    {
        while (ev_phase.size() <= i) {
            cudaEvent_t e;
            ck(cudaEventCreate(&e), "cudaEventCreate");
            ev_phase.push_back(e);
        }
        return ev_phase[i];
    }
};

namespace
{

__global__ void k_set_tmax(GraphRt* rt, const double* tmax, int num_graphs)
{
    const int gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi < num_graphs) {
        rt[gi].tmax = tmax[gi];
    }
}

// FP64 value -> float-float pair (hi = nearest float, lo = the rest rounded)
void split_pairs(const double* v, int64_t n, float* hi, float* lo)
{
    for (int64_t i = 0; i < n; ++i) {
        hi[i] = (float)v[i];
        lo[i] = (float)(v[i] - (double)hi[i]);
    }
}

// FP64 value -> float-float pair on the device (the same roundings as split_pairs)
__global__ void k_split_pairs(const double* v, int64_t n, float* hi, float* lo, float* hi2, float* lo2)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    const float h = __double2float_rn(v[i]);
    const float l = __double2float_rn(v[i] - (double)h);
    hi[i] = hi2[i] = h;
    lo[i] = lo2[i] = l;
}

__global__ void k_pairs_to_double(const float* hi, const float* lo, int64_t n, double* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = (double)hi[i] + (double)lo[i];
    }
}

__global__ void k_to_float(const double* v, int64_t n, float* out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = __double2float_rn(v[i]);
    }
}

// FP32 per-(node, age group) constants of the mixed solver from the FP64
// parameters, with the rates formed as the reference forms them.
__global__ void k_build_tab(BatchDev B, float* tab)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= B.num_nodes * MGPU_MAX_GROUPS) {
        return;
    }
    const int64_t node = tid / MGPU_MAX_GROUPS;
    const int gr       = (int)(tid % MGPU_MAX_GROUPS);
    const DevGraph& d  = B.graphs[B.node_graph[node]];
    const int G        = d.G;
    if (gr >= G) {
        return;
    }
    const double* p = B.params + d.param_off + (node - d.node0) * param_stride(G);
    auto gp         = [&](int w) {
        return p[MGPU_NUM_SCALAR_PARAMS + w * G + gr];
    };
    float* T           = tab + tid * kTabF;
    const double mu    = gp(MGPU_G_RECOVERED_PER_INS);
    const double tins  = gp(MGPU_G_TIME_INS);
    const double sev   = gp(MGPU_G_SEVERE_PER_ISY);
    const double tisy  = gp(MGPU_G_TIME_ISY);
    const double tisev = gp(MGPU_G_TIME_ISEV);
    const double cps   = gp(MGPU_G_CRITICAL_PER_SEVERE);
    const double dps   = gp(MGPU_G_DEATHS_PER_SEVERE);
    const double dpc   = gp(MGPU_G_DEATHS_PER_CRITICAL);
    const double ticri = gp(MGPU_G_TIME_ICRI);
    T[TF_A_TNT]        = __double2float_rn(__ddiv_rn(1 - mu, tins));
    T[TF_BETA]         = __double2float_rn(gp(MGPU_G_TRANSMISSION_PROB));
    T[TF_XI]           = __double2float_rn(gp(MGPU_G_REL_TRANSMISSION_NS));
    T[TF_RHO]          = __double2float_rn(gp(MGPU_G_RISK_FROM_SYMPTOMATIC));
    T[TF_RHO_MAX]      = __double2float_rn(gp(MGPU_G_MAX_RISK_FROM_SYMPTOMATIC));
    T[TF_R1]           = __double2float_rn(__ddiv_rn(1.0, gp(MGPU_G_TIME_EXPOSED)));
    T[TF_R2]           = __double2float_rn(__dmul_rn(1 - mu, __ddiv_rn(1.0, tins)));
    T[TF_R3]           = __double2float_rn(__dmul_rn(mu, __ddiv_rn(1.0, tins)));
    T[TF_R6]           = __double2float_rn(__ddiv_rn(sev, tisy));
    T[TF_R7]           = __double2float_rn(__ddiv_rn(1 - sev, tisy));
    T[TF_R11]          = __double2float_rn(__ddiv_rn(1.0 - cps - dps, tisev));
    T[TF_R13]          = __double2float_rn(__ddiv_rn(dpc, ticri));
    T[TF_R14]          = __double2float_rn(__ddiv_rn(1.0 - dpc, ticri));
    T[TF_R10L]         = __double2float_rn(__ddiv_rn(cps, tisev));
    T[TF_R12L]         = __double2float_rn(__ddiv_rn(dps + (cps - cps), tisev));
    T[TF_CPS]          = __double2float_rn(cps);
    T[TF_DPS]          = __double2float_rn(dps);
    T[TF_INV_TISEV]    = __double2float_rn(__ddiv_rn(1.0, tisev));
    const double cap   = p[MGPU_P_TNT_CAPACITY];
    T[TF_TNT_CAP]      = __double2float_rn(cap);
    T[TF_TNT_CAP2]     = __double2float_rn(__dmul_rn(cap, p[MGPU_P_TNT_MAX_RISK]));
    const double icu   = p[MGPU_P_ICU_CAPACITY];
    T[TF_ICU_LO]       = __double2float_rn(__dmul_rn(0.90, icu));
    T[TF_ICU_CAP]      = __double2float_rn(icu);
    T[TF_SEASON_K]     = __double2float_rn(p[MGPU_P_SEASONALITY]);
}

// Restart: graph clocks and flags, node clocks, states, pending travelers.
__global__ void k_reset(BatchDev B, const double* init_state, const float* init_hi, const float* init_lo,
                        int64_t state_total, double t0, double dt0)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < state_total) {
        if (B.st_hi) {
            B.st_hi[tid] = init_hi[tid];
            B.st_lo[tid] = init_lo[tid];
        }
        else {
            B.state[tid] = init_state[tid];
        }
    }
    if (tid < B.num_nodes) {
        B.node_t[tid]  = t0;
        B.node_dt[tid] = dt0;
    }
    if (tid < B.num_edges) {
        B.edge_pending[tid] = 0;
    }
    if (tid < B.num_graphs) {
        GraphRt r;
        memset(&r, 0, sizeof(r));
        r.t              = t0;
        r.tmax           = t0;
        B.rt[tid]        = r;
        B.graph_err[tid] = 0; // a restarted graph has not failed
    }
    if (tid == 0) {
        *B.err = 0;
    }
}

// Phase times of a batch creation on stderr when MIOGPU_TRACE is set.
struct PhaseTrace {
    bool on = std::getenv("MIOGPU_TRACE") != nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now(), last = t0;
    void mark(const char* what)
    {
        if (!on) {
            return;
        }
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "miogpu: %-28s %8.2f ms\n", what,
                     std::chrono::duration<double, std::milli>(now - last).count());
        last = now;
    }
};

// Upload graphs into one set of pools. `with_edges` false: edges ignored.
void build_batch(mgpu_batch* b, const mgpu_graph* graphs, int32_t num_graphs, double t0, double dt0,
                 bool with_edges, int64_t scratch_slots)
{
    mgpu_context* ctx = b->ctx;
    b->pool.ctx       = ctx;
    b->num_graphs     = num_graphs;
    std::vector<DevGraph> dg(num_graphs);
    int64_t nodes = 0, edges = 0, par = 0, con = 0, dtt = 0, dtv = 0, st = 0, ec = 0, edt = 0, edv = 0, tr = 0,
            ecf = 0;
    // Arrays that several graphs pass by the same host pointer (the shared
    // topology, contacts and coefficients of an ensemble) are uploaded once.
    using Key = std::tuple<const void*, const void*, const void*, const void*, int64_t, int64_t, int64_t>;
    std::map<Key, int> contact_first, damping_first, coeff_first;
    std::vector<char> own_contact(num_graphs, 1), own_damping(num_graphs, 1), own_coeff(num_graphs, 1);
    std::vector<int> coeff_src(num_graphs, -1); // graph whose edge coefficients this one shares
    b->N.resize(num_graphs);
    b->G.resize(num_graphs);
    b->n.resize(num_graphs);
    b->node0.resize(num_graphs);
    b->edge0.resize(num_graphs);
    b->state_off.resize(num_graphs);
    b->n_max = 0;
    std::vector<int64_t> trav0(num_graphs);
    // arrays to check: each (edge index arrays, damping times) once, however many graphs share it
    using AKey = std::tuple<const void*, const void*, int64_t, int64_t>;
    std::map<AKey, int> edges_seen, times_seen;
    std::vector<char> check_edges(num_graphs, 0), check_times(num_graphs, 0);
    for (int i = 0; i < num_graphs; ++i) {
        const mgpu_graph& g = graphs[i];
        validate_graph_header(g);
        check_edges[i] = edges_seen.emplace(AKey{g.edge_src, g.edge_dst, g.num_edges, g.num_nodes}, i).second;
        check_times[i] = times_seen
                             .emplace(AKey{g.damping_times, nullptr, (int64_t)g.num_nodes * g.num_contact_matrices,
                                           g.num_damping_points},
                                      i)
                             .second;

        DevGraph& d   = dg[i];
        const int G   = g.num_groups;
        const int n   = G * kC;
        const int E   = with_edges ? g.num_edges : 0;
        const long GG = (long)G * G;
        d.N           = g.num_nodes;
        d.G           = G;
        d.E           = E;
        d.M           = g.num_contact_matrices;
        d.K           = g.num_damping_points;
        d.Ke          = with_edges ? g.num_edge_damping_points : 0;
        d.n           = n;
        d.method      = b->opts.integrator.method;
        d.node0       = nodes;
        d.edge0       = edges;
        d.param_off   = par;
        d.state_off   = st;
        nodes += g.num_nodes;
        edges += E;
        par += (int64_t)g.num_nodes * param_stride(G);
        st += (int64_t)g.num_nodes * n;
        trav0[i] = tr;
        d.trav0  = tr;
        tr += (int64_t)E * n;
        const Key kc{g.contact_baseline, g.contact_minimum, nullptr, nullptr, g.num_nodes, d.M, G};
        auto itc = contact_first.find(kc);
        if (itc != contact_first.end()) {
            d.contact_off  = dg[itc->second].contact_off;
            own_contact[i] = 0;
        }
        else {
            contact_first[kc] = i;
            d.contact_off     = con;
            con += (int64_t)g.num_nodes * d.M * 2 * GG;
        }
        const Key kd{g.damping_times, g.damping_values, nullptr, nullptr, g.num_nodes, d.M * 64 + d.K, G};
        auto itd = damping_first.find(kd);
        if (d.K && itd != damping_first.end()) {
            d.dtime_off    = dg[itd->second].dtime_off;
            d.dval_off     = dg[itd->second].dval_off;
            own_damping[i] = 0;
        }
        else {
            damping_first[kd] = i;
            d.dtime_off       = dtt;
            d.dval_off        = dtv;
            dtt += (int64_t)g.num_nodes * d.M * d.K;
            dtv += (int64_t)g.num_nodes * d.M * d.K * GG;
        }
        const Key ke{g.edge_coeff_baseline, g.edge_coeff_minimum, g.edge_damping_times, g.edge_damping_values, E,
                     d.Ke, n};
        auto ite = coeff_first.find(ke);
        if (E && ite != coeff_first.end()) {
            d.ecoef_off   = dg[ite->second].ecoef_off;
            d.edt_off     = dg[ite->second].edt_off;
            d.edv_off     = dg[ite->second].edv_off;
            d.ecoef_f_off = dg[ite->second].ecoef_f_off;
            own_coeff[i]  = 0;
            coeff_src[i]  = ite->second;
        }
        else {
            coeff_first[ke] = i;
            d.ecoef_off     = ec;
            d.edt_off       = edt;
            d.edv_off       = edv;
            d.ecoef_f_off   = ecf;
            ec += (int64_t)E * 2 * n;
            edt += (int64_t)E * d.Ke;
            edv += (int64_t)E * d.Ke * n;
            ecf += (int64_t)E * n;
        }
        b->N[i]         = g.num_nodes;
        b->G[i]         = G;
        b->n[i]         = n;
        b->node0[i]     = d.node0;
        b->edge0[i]     = d.edge0;
        b->state_off[i] = d.state_off;
        b->n_max        = std::max<int64_t>(b->n_max, n);
    }
    b->state_total = st;
    if (nodes * MGPU_MAX_GROUPS > INT32_MAX) {
        fail(MGPU_INVALID_VALUE, "batch too large: more than 2^28 nodes in one batch");
    }
    if (edges > INT32_MAX) {
        fail(MGPU_INVALID_VALUE, "batch too large: more than 2^31 - 1 edges in one batch");
    }
    // edge index arrays and damping times, each distinct array once, on the host's cores
    PhaseTrace trace;
    trace.mark("layout");
    parallel_for(num_graphs, [&](int64_t i) {
        validate_graph_arrays(graphs[i], with_edges && check_edges[i], check_times[i], true);
    });
    trace.mark("checks");
    // host staging in the context's page-locked buffer (every element is written below)
    HostSpan<double> h_par, h_con, h_dtt, h_dtv, h_state, h_ec, h_edt, h_edv;
    HostSpan<int32_t> h_node_graph, h_edge_graph, h_src, h_dst;
    HostSpan<uint8_t> h_any;
    HostSpan<int64_t> h_in_ptr, h_in_edges;
    StagingArena arena{ctx};
    arena.take(h_par, par);
    arena.take(h_con, con);
    arena.take(h_dtt, dtt);
    arena.take(h_dtv, dtv);
    arena.take(h_state, st);
    arena.take(h_ec, ec);
    arena.take(h_edt, edt);
    arena.take(h_edv, edv);
    arena.take(h_node_graph, nodes);
    arena.take(h_edge_graph, edges);
    arena.take(h_src, edges);
    arena.take(h_dst, edges);
    arena.take(h_any, edges);
    arena.take(h_in_ptr, nodes + 1);
    arena.take(h_in_edges, edges);
    ck(cudaStreamSynchronize(ctx->stream), "staging sync"); // an earlier upload may still read the buffer
    arena.place();
    trace.mark("page-locked staging");
    // FP32 coefficient records (rec_vec layout) of the mixed exchange; the factor slots stay zero
    std::vector<float> h_ecr(is_mixed(b->opts.precision) ? ecf / kC * kRec : 0, 0.0f);
    std::vector<int64_t> h_out_ptr(nodes + 1, 0);
    std::vector<int32_t> mob_mask(num_graphs, 0);
    // Graphs pack into disjoint ranges of the staging buffers, on the host's
    // cores; a graph that shares the coefficient arrays of an earlier one copies
    // that graph's flags afterwards, and a graph that passes the same edge
    // arrays as an earlier one (the samples of an ensemble) copies that graph's
    // edge indices with its own node and edge offsets.
    std::vector<int> edge_owner(num_graphs);
    {
        std::map<Key, int> first;
        for (int i = 0; i < num_graphs; ++i) {
            edge_owner[i] = i;
            if (dg[i].E > 0) {
                const Key k{graphs[i].edge_src, graphs[i].edge_dst, nullptr, nullptr, dg[i].N, dg[i].E, 0};
                auto it = first.find(k);
                if (it != first.end()) {
                    edge_owner[i] = it->second;
                }
                else {
                    first[k] = i;
                }
            }
        }
    }
    parallel_for(num_graphs, [&](int64_t gi) {
        const int i         = (int)gi;
        const mgpu_graph& g = graphs[i];
        const DevGraph& d   = dg[i];
        const int G = d.G, n = d.n;
        const long GG = (long)G * G;
        std::memcpy(h_par.data() + d.param_off, g.params, sizeof(double) * (size_t)g.num_nodes * param_stride(G));
        for (long v = 0; own_contact[i] && v < g.num_nodes; ++v) {
            for (int m = 0; m < d.M; ++m) {
                double* dst      = h_con.data() + d.contact_off + (v * d.M + m) * 2 * GG;
                const double* Bs = g.contact_baseline + (v * d.M + m) * GG;
                std::memcpy(dst, Bs, sizeof(double) * GG);
                if (g.contact_minimum) {
                    std::memcpy(dst + GG, g.contact_minimum + (v * d.M + m) * GG, sizeof(double) * GG);
                }
                else {
                    std::fill(dst + GG, dst + 2 * GG, 0.0);
                }
            }
        }
        if (d.K && own_damping[i]) {
            std::memcpy(h_dtt.data() + d.dtime_off, g.damping_times, sizeof(double) * (size_t)g.num_nodes * d.M * d.K);
            std::memcpy(h_dtv.data() + d.dval_off, g.damping_values,
                        sizeof(double) * (size_t)g.num_nodes * d.M * d.K * GG);
        }
        std::memcpy(h_state.data() + d.state_off, g.init_state, sizeof(double) * (size_t)g.num_nodes * n);
        for (long v = 0; v < g.num_nodes; ++v) {
            h_node_graph[d.node0 + v] = i;
        }
        // edges: CSR by source (already sorted), CSC by destination (sorted by source within)
        const bool own_edges = edge_owner[i] == i;
        std::vector<int64_t> indeg(own_edges ? g.num_nodes + 1 : 0, 0);
        for (int e = 0; e < d.E; ++e) {
            const int64_t ge = d.edge0 + e;
            h_edge_graph[ge] = i;
            if (own_edges) {
                h_src[ge] = (int32_t)(d.node0 + g.edge_src[e]);
                h_dst[ge] = (int32_t)(d.node0 + g.edge_dst[e]);
                h_out_ptr[d.node0 + g.edge_src[e] + 1]++;
                indeg[g.edge_dst[e] + 1]++;
            }
            const double* cb = g.edge_coeff_baseline + (int64_t)e * n;
            if (own_coeff[i]) {
                double* dc = h_ec.data() + d.ecoef_off + (int64_t)e * 2 * n;
                std::memcpy(dc, cb, sizeof(double) * n);
                if (g.edge_coeff_minimum) {
                    std::memcpy(dc + n, g.edge_coeff_minimum + (int64_t)e * n, sizeof(double) * n);
                }
                else {
                    std::fill(dc + n, dc + 2 * n, 0.0);
                }
                // an edge with no positive coefficient carries nobody (apply_mobility,
                // metapopulation_mobility_instant.h:606): its FP32 row is zero, so the
                // FP32 passes, which do not test the edge, add exact zeros for it
                bool any = false;
                for (int j = 0; j < n; ++j) {
                    any = any || (cb[j] > 0.0);
                    if (cb[j] != 0.0 || (g.edge_coeff_minimum && g.edge_coeff_minimum[(int64_t)e * n + j] != 0.0)) {
                        mob_mask[i] |= 1 << (j % kC);
                    }
                }
                if (!h_ecr.empty()) {
                    for (int j = 0; j < n; ++j) {
                        h_ecr[rec_elem(d.ecoef_f_off / kC + (int64_t)e * G, G, j / kC, rec_pos(j % kC))] =
                            any ? (float)cb[j] : 0.0f;
                    }
                }
                h_any[ge] = any ? 1 : 0;
                if (d.Ke) {
                    std::memcpy(h_edt.data() + d.edt_off + (int64_t)e * d.Ke,
                                g.edge_damping_times + (int64_t)e * d.Ke, sizeof(double) * d.Ke);
                    std::memcpy(h_edv.data() + d.edv_off + (int64_t)e * d.Ke * n,
                                g.edge_damping_values + (int64_t)e * d.Ke * n, sizeof(double) * d.Ke * n);
                }
            }
        }
        if (!own_edges) {
            return;
        }
        for (int v = 0; v < g.num_nodes; ++v) {
            indeg[v + 1] += indeg[v];
        }
        std::vector<int64_t> fillp(indeg.begin(), indeg.end() - 1);
        for (int e = 0; e < d.E; ++e) { // edges visited in (src, dst) order -> CSC sorted by src
            const int v                          = g.edge_dst[e];
            h_in_edges[d.edge0 + fillp[v]++]     = d.edge0 + e;
        }
        for (int v = 0; v < g.num_nodes; ++v) {
            h_in_ptr[d.node0 + v] = d.edge0 + indeg[v];
        }
    });
    parallel_for(num_graphs, [&](int64_t gi) {
        const int i = (int)gi;
        const int o = edge_owner[i];
        if (o == i) {
            return;
        }
        const DevGraph& d  = dg[i];
        const DevGraph& s  = dg[o];
        const int32_t dn   = (int32_t)(d.node0 - s.node0);
        const int64_t de   = d.edge0 - s.edge0;
        for (int64_t e = 0; e < d.E; ++e) {
            h_src[d.edge0 + e]      = h_src[s.edge0 + e] + dn;
            h_dst[d.edge0 + e]      = h_dst[s.edge0 + e] + dn;
            h_in_edges[d.edge0 + e] = h_in_edges[s.edge0 + e] + de;
        }
        for (int64_t v = 0; v < d.N; ++v) {
            h_out_ptr[d.node0 + v + 1] = h_out_ptr[s.node0 + v + 1];
            h_in_ptr[d.node0 + v]      = h_in_ptr[s.node0 + v] + de;
        }
    });
    h_in_ptr[nodes] = edges;
    for (int i = 0; i < num_graphs; ++i) {
        if (!own_coeff[i]) {
            // the same coefficient arrays as an earlier graph: its flags
            const DevGraph& d = dg[i];
            if (d.E) {
                std::memcpy(h_any.data() + d.edge0, h_any.data() + dg[coeff_src[i]].edge0, (size_t)d.E);
            }
            mob_mask[i] = mob_mask[coeff_src[i]];
        }
    }
    for (int64_t v = 0; v < nodes; ++v) {
        h_out_ptr[v + 1] += h_out_ptr[v];
    }
    // the prefix over all nodes of all graphs is global because graphs are concatenated in order
    BatchDev& B      = b->dev;
    B.num_graphs     = num_graphs;
    B.num_nodes      = nodes;
    B.num_edges      = edges;
    B.mob_union = 0;
    for (int i = 0; i < num_graphs; ++i) {
        dg[i].mob_mask = mob_mask[i];
        dg[i].staged   = 0;
        B.mob_union |= mob_mask[i];
    }
    // graphs whose FP32 exchange passes run one CTA per graph from shared memory
    XsPlan xs;
    if (is_mixed(b->opts.precision) && b->opts.staged_exchange) {
        xs = plan_staged_exchange(dg, B.mob_union, ctx->device, b->opts.staged_exchange);
        ck(xs.err, "staged exchange setup");
    }
    // One commuter fraction per (edge, age group): when every compartment the
    // exchange moves has the same coefficient on every edge of every graph with
    // static coefficients, the FP32 passes read that one float per (edge, group)
    // instead of the two coefficient vectors (the products are the same).
    std::vector<float> h_ecu;
    if (is_mixed(b->opts.precision) && ecf > 0) {
        const int mask = (B.mob_union & ~kMaskSEIYRBits) == 0 ? kMaskSEIYRBits : (1 << kC) - 1;
        std::vector<char> uniform(num_graphs, 1);
        parallel_for(num_graphs, [&](int64_t gi) {
            const DevGraph& d = dg[gi];
            if (!own_coeff[gi] || d.Ke != 0 || d.E == 0) {
                return;
            }
            const int G = d.G;
            for (int e = 0; e < d.E && uniform[gi]; ++e) {
                for (int gr = 0; gr < G && uniform[gi]; ++gr) {
                    const int64_t r0 = d.ecoef_f_off / kC + (int64_t)e * G;
                    float u          = 0.0f;
                    bool first       = true;
                    for (int c = 0; c < kC; ++c) {
                        if (!((mask >> c) & 1)) {
                            continue;
                        }
                        const float v = h_ecr[rec_elem(r0, G, gr, rec_pos(c))];
                        if (first) {
                            u     = v;
                            first = false;
                        }
                        else if (v != u) {
                            uniform[gi] = 0;
                        }
                    }
                }
            }
        });
        bool all = true;
        for (int i = 0; i < num_graphs; ++i) {
            all = all && uniform[i];
        }
        if (all) {
            int first_c = 0; // the first moved compartment (all carry the same value)
            while (!((mask >> first_c) & 1)) {
                ++first_c;
            }
            h_ecu.resize((size_t)(ecf / kC));
            for (int i = 0; i < num_graphs; ++i) {
                const DevGraph& d = dg[i];
                if (!own_coeff[i] || d.Ke != 0) {
                    continue;
                }
                for (int64_t r = 0; r < (int64_t)d.E * d.G; ++r) {
                    const int64_t row = d.ecoef_f_off / kC + r;
                    const int64_t r0  = d.ecoef_f_off / kC + (r / d.G) * d.G;
                    h_ecu[(size_t)row] = h_ecr[rec_elem(r0, d.G, (int)(r % d.G), rec_pos(first_c))];
                }
            }
        }
    }
    // the one-value coefficients also in each graph's in-edge order (graphs with
    // the same coefficient and edge arrays share one copy, as they share ecoef_u)
    std::vector<float> h_ecu_in;
    for (int i = 0; i < num_graphs; ++i) {
        dg[i].ecoef_in_off = -1;
    }
    if (!h_ecu.empty()) {
        std::map<Key, int> ein_first;
        std::vector<int> ein_own;
        int64_t pos = 0;
        for (int i = 0; i < num_graphs; ++i) {
            DevGraph& d = dg[i];
            if (d.E == 0 || d.Ke != 0) {
                continue;
            }
            const Key k{graphs[i].edge_coeff_baseline, graphs[i].edge_src, graphs[i].edge_dst, nullptr, d.E, d.G, 0};
            auto it = ein_first.find(k);
            if (it != ein_first.end()) {
                d.ecoef_in_off = dg[it->second].ecoef_in_off;
            }
            else {
                ein_first[k]   = i;
                d.ecoef_in_off = pos;
                pos += (int64_t)d.E * d.G;
                ein_own.push_back(i);
            }
        }
        h_ecu_in.resize((size_t)pos);
        parallel_for((int64_t)ein_own.size(), [&](int64_t q) {
            const DevGraph& d = dg[ein_own[(size_t)q]];
            for (int64_t k = 0; k < d.E; ++k) {
                const int64_t el = h_in_edges[d.edge0 + k] - d.edge0;
                for (int gr = 0; gr < d.G; ++gr) {
                    h_ecu_in[(size_t)(d.ecoef_in_off + k * d.G + gr)] =
                        h_ecu[(size_t)(d.ecoef_f_off / kC + el * d.G + gr)];
                }
            }
        });
    }
    trace.mark("packing");
    b->host_graphs = dg;
    b->damping_shared.assign(num_graphs, 0);
    {
        std::map<int64_t, int> users;
        for (int i = 0; i < num_graphs; ++i) {
            if (dg[i].K) {
                ++users[dg[i].dtime_off];
            }
        }
        for (int i = 0; i < num_graphs; ++i) {
            b->damping_shared[i] = dg[i].K && users[dg[i].dtime_off] > 1;
        }
        std::map<int64_t, int> cusers;
        for (int i = 0; i < num_graphs; ++i) {
            if (dg[i].E) {
                ++cusers[dg[i].ecoef_off];
            }
        }
        b->coeff_shared.assign(num_graphs, 0);
        for (int i = 0; i < num_graphs; ++i) {
            b->coeff_shared[i] = dg[i].E && cusers[dg[i].ecoef_off] > 1;
        }
    }
    B.graphs         = b->pool.upload(dg);
    std::vector<GraphRt> h_rt(num_graphs);
    for (auto& r : h_rt) {
        std::memset(&r, 0, sizeof(r));
        r.t    = t0;
        r.tmax = t0;
    }
    B.rt         = b->pool.upload(h_rt);
    B.node_graph = b->pool.upload(h_node_graph);
    B.edge_graph = b->pool.upload(h_edge_graph);
    B.params     = b->pool.upload(h_par);
    B.contact    = b->pool.upload(h_con);
    B.dtimes     = b->pool.upload(h_dtt);
    B.dvals      = b->pool.upload(h_dtv);
    b->dt0     = dt0;
    b->pairs   = is_mixed(b->opts.precision);
    B.st_hi    = B.st_lo = B.v0_hi = B.v0_lo = B.yn_hi = B.yn_lo = nullptr;
    B.state    = nullptr;
    B.v0       = nullptr;
    B.ynew     = nullptr;
    DevPool staging; // released at the end of the upload
    staging.ctx = ctx;
    if (b->pairs) {
        // the mixed solver keeps node states as float-float pairs on the device;
        // the FP64 states are uploaded once and split there
        double* d_state = staging.upload(h_state);
        B.st_hi         = b->pool.alloc<float>(st);
        B.st_lo         = b->pool.alloc<float>(st);
        b->init_hi      = b->pool.alloc<float>(st);
        b->init_lo      = b->pool.alloc<float>(st);
        k_split_pairs<<<(unsigned)std::max<int64_t>((st + 255) / 256, 1), 256, 0, ctx->stream>>>(
            d_state, st, B.st_hi, B.st_lo, b->init_hi, b->init_lo);
        ck(cudaGetLastError(), "k_split_pairs");
        B.v0_hi       = b->pool.alloc<float>(st);
        B.v0_lo       = b->pool.alloc<float>(st);
        B.yn_hi       = b->pool.alloc<float>(st);
        B.yn_lo       = b->pool.alloc<float>(st);
    }
    else {
        B.state       = b->pool.upload(h_state);
        b->init_state = b->pool.upload(h_state);
        B.v0          = b->pool.alloc<double>(st);
        B.ynew        = b->pool.alloc<double>(std::max<int64_t>(st, scratch_slots * b->n_max));
    }
    B.ypre = b->opts.precision == MGPU_PRECISION_FP64_PLAIN ? b->pool.alloc<double>(st) : nullptr;
    std::vector<double> h_t(nodes, t0), h_dt(nodes, dt0);
    trace.mark("uploads: node and state pools");
    B.node_t          = b->pool.upload(h_t);
    B.node_dt         = b->pool.upload(h_dt);
    B.edge_src        = b->pool.upload(h_src);
    B.edge_dst        = b->pool.upload(h_dst);
    B.ecoef           = b->pool.upload(h_ec);
    B.edt             = b->pool.upload(h_edt);
    B.edv             = b->pool.upload(h_edv);
    B.edge_static_any = b->pool.upload(h_any);
    B.edge_pending    = b->pool.alloc<uint8_t>(edges);
    ck(cudaMemsetAsync(B.edge_pending, 0, std::max<int64_t>(edges, 1), ctx->stream), "memset");
    const bool plain = b->opts.precision == MGPU_PRECISION_FP64_PLAIN;
    B.trav       = plain ? b->pool.alloc<double>(tr) : nullptr; // the batched exchange recomputes travelers
    B.mfix       = b->pool.alloc<double>(tr);
    B.state_total = st;
    B.ysnap      = (plain || b->pairs) ? nullptr : b->pool.alloc<double>(2 * st);
    B.gsnap      = b->pairs ? b->pool.alloc<float>(2 * (st / kC) * kRec) : nullptr;
    B.risk       = (plain || b->pairs) ? nullptr : (void*)b->pool.alloc<double>(2 * nodes * MGPU_MAX_GROUPS * 2);
    B.aux        = plain ? nullptr : (void*)b->pool.alloc<double>(nodes * MGPU_MAX_GROUPS * 12);
    trace.mark("uploads: edge arrays, snapshots");
    B.ecoef_r    = b->pairs ? b->pool.upload(h_ecr) : nullptr;
    B.ecoef_u    = h_ecu.empty() ? nullptr : b->pool.upload(h_ecu);
    B.ecoef_in   = h_ecu_in.empty() ? nullptr : b->pool.upload(h_ecu_in);
    B.tab_f      = nullptr;
    B.contact_f  = nullptr;
    B.dvals_f    = nullptr;
    if (is_mixed(b->opts.precision)) {
        // FP32 node constants, contact and damping pools of the mixed solver
        // derived on the device from the uploaded FP64 pools (no second host copy, no second upload)
        float* tab = b->pool.alloc<float>(nodes * MGPU_MAX_GROUPS * kTabF);
        float* cf  = b->pool.alloc<float>(con);
        float* df  = b->pool.alloc<float>(dtv);
        ck(cudaMemsetAsync(tab, 0, sizeof(float) * std::max<int64_t>(nodes * MGPU_MAX_GROUPS * kTabF, 1), ctx->stream),
           "memset");
        k_build_tab<<<(unsigned)std::max<int64_t>((nodes * MGPU_MAX_GROUPS + 255) / 256, 1), 256, 0, ctx->stream>>>(
            B, tab);
        k_to_float<<<(unsigned)std::max<int64_t>((con + 255) / 256, 1), 256, 0, ctx->stream>>>(B.contact, con, cf);
        k_to_float<<<(unsigned)std::max<int64_t>((dtv + 255) / 256, 1), 256, 0, ctx->stream>>>(B.dvals, dtv, df);
        B.tab_f     = tab;
        B.contact_f = cf;
        B.dvals_f   = df;
        ck(cudaGetLastError(), "table kernels");
    }
    b->any_edge_dampings = false;
    for (int i = 0; i < num_graphs; ++i) {
        b->any_edge_dampings = b->any_edge_dampings || (dg[i].Ke > 0 && dg[i].E > 0);
    }
    trace.mark("FP32 coefficients and tables");
    B.edge_fixed = b->pool.alloc<int32_t>(edges);
    B.scan_mark  = b->pool.alloc<int32_t>(3 * nodes * MGPU_MAX_GROUPS);
    B.scan_list  = b->pool.alloc<int32_t>(3 * nodes * MGPU_MAX_GROUPS);
    B.scan_count = b->pool.alloc<int32_t>(3);
    B.fix_cnt    = b->pool.alloc<uint8_t>(edges * MGPU_MAX_GROUPS);
    B.fix_cap    = std::min<int64_t>(std::max<int64_t>(edges, 1), 1 << 22);
    B.fix_edges  = b->pool.alloc<int32_t>(B.fix_cap);
    B.fix_meta   = b->pool.alloc<int32_t>(2);
    ck(cudaMemsetAsync(B.fix_meta, 0, sizeof(int32_t) * 2, ctx->stream), "memset");
    ck(cudaMemsetAsync(B.scan_mark, 0, sizeof(int32_t) * std::max<int64_t>(3 * nodes * MGPU_MAX_GROUPS, 1), ctx->stream),
       "memset");
    ck(cudaMemsetAsync(B.scan_count, 0, sizeof(int32_t) * 3, ctx->stream), "memset");
    ck(cudaMemsetAsync(B.fix_cnt, 0, std::max<int64_t>(edges * MGPU_MAX_GROUPS, 1), ctx->stream), "memset");
    B.node_flag  = b->pool.alloc<uint8_t>(nodes);
    B.node_dirty = b->pool.alloc<uint8_t>(2 * nodes);
    ck(cudaMemsetAsync(B.edge_fixed, 0, sizeof(int32_t) * std::max<int64_t>(edges, 1), ctx->stream), "memset");
    ck(cudaMemsetAsync(B.node_flag, 0, std::max<int64_t>(nodes, 1), ctx->stream), "memset");
    ck(cudaMemsetAsync(B.node_dirty, 0, std::max<int64_t>(2 * nodes, 1), ctx->stream), "memset");
    trace.mark("exchange work space");
    B.out_ptr  = b->pool.upload(h_out_ptr);
    B.in_ptr   = b->pool.upload(h_in_ptr);
    B.in_edges = b->pool.upload(h_in_edges);
    {
        // derived on the device from the uploaded edge arrays: the (source, edge)
        // pairs of the in-edges, each node's first in-edge from a higher source,
        // and the offsets of the edges' traveler records
        int64_t* trav_off = b->pool.alloc<int64_t>(edges);
        int2* in_se       = b->pool.alloc<int2>(edges);
        int64_t* in_mid   = b->pool.alloc<int64_t>(nodes);
        B.trav_off        = trav_off;
        B.in_se           = in_se;
        B.in_mid          = in_mid;
        ck(launch_edge_indices(B, trav_off, in_se, in_mid, ctx->stream), "edge index kernel");
        trace.mark("edge indices");
    }
    B.scratch_stride = std::max<int64_t>(scratch_slots, 1);
    B.scratch_nmax   = (int32_t)b->n_max;
    B.scratch        = scratch_slots > 0 ? b->pool.alloc<double>(8 * b->n_max * B.scratch_stride) : nullptr;
    B.opts.abs_tol   = b->opts.integrator.abs_tol;
    B.opts.rel_tol   = b->opts.integrator.rel_tol;
    B.opts.dt_min    = b->opts.integrator.dt_min;
    B.opts.dt_max    = b->opts.integrator.dt_max;
    B.opts.max_steps = b->opts.max_steps_per_interval > 0 ? b->opts.max_steps_per_interval : 100000;
    B.opts.method    = b->opts.integrator.method;
    B.err            = b->pool.alloc<int32_t>(1);
    B.graph_err      = b->pool.alloc<int32_t>(num_graphs);
    B.counters       = b->pool.alloc<unsigned long long>(CNT_NUM);
    ck(cudaMemsetAsync(B.err, 0, sizeof(int32_t), ctx->stream), "memset");
    ck(cudaMemsetAsync(B.graph_err, 0, sizeof(int32_t) * std::max(num_graphs, 1), ctx->stream), "memset");
    ck(cudaMemsetAsync(B.counters, 0, sizeof(unsigned long long) * CNT_NUM, ctx->stream), "memset");
    b->d_tmax = b->pool.alloc<double>(num_graphs);
    b->t_host.assign(num_graphs, t0);
    b->tmax_host.assign(num_graphs, t0);
    // instance lists per G for the batched solver
    std::map<int, std::vector<int32_t>> lists;
    for (int i = 0; i < num_graphs; ++i) {
        auto& l = lists[b->G[i]];
        for (int v = 0; v < b->N[i]; ++v) {
            l.push_back((int32_t)(b->node0[i] + v));
        }
    }
    for (auto& kv : lists) {
        b->inst_by_G[kv.first] = {b->pool.upload(kv.second), (int64_t)kv.second.size()};
    }
    for (int G = 0; G <= MGPU_MAX_GROUPS; ++G) {
        auto it     = b->inst_by_G.find(G);
        B.glist[G]  = it != b->inst_by_G.end() ? it->second.first : nullptr;
        B.gcount[G] = it != b->inst_by_G.end() ? it->second.second : 0;
        B.gorder[G] = (is_mixed(b->opts.precision) && B.gcount[G] > 0)
                          ? b->pool.alloc<int32_t>(B.gcount[G])
                          : nullptr;
    }
    // the exchange passes: the staged graphs, and per G the nodes of the others
    B.xs_count    = (int32_t)xs.work.size();
    B.xs_work     = xs.work.empty() ? nullptr : b->pool.upload(xs.work);
    B.xs_smem_ret = xs.smem_ret;
    B.xs_smem_dep = xs.smem_dep;
    B.xs_aux      = xs.aux;
    // (graphs without edges or with edge dampings take no part in the FP32 node-list passes)
    for (int G = 0; G <= MGPU_MAX_GROUPS; ++G) {
        B.xlist[G]  = nullptr;
        B.xcount[G] = 0;
    }
    if (is_mixed(b->opts.precision)) {
        std::map<int, std::vector<int32_t>> xl;
        for (int i = 0; i < num_graphs; ++i) {
            if (!dg[i].staged && dg[i].E > 0 && dg[i].Ke == 0) {
                auto& l = xl[b->G[i]];
                for (int v = 0; v < b->N[i]; ++v) {
                    l.push_back((int32_t)(b->node0[i] + v));
                }
            }
        }
        for (int G = 0; G <= MGPU_MAX_GROUPS; ++G) {
            auto it = xl.find(G);
            if (it == xl.end()) {
                continue;
            }
            auto ig = b->inst_by_G.find(G);
            // the same list as the node solves' when it holds every node with G groups
            const bool all = ig != b->inst_by_G.end() && ig->second.second == (int64_t)it->second.size();
            B.xlist[G]     = all ? ig->second.first : b->pool.upload(it->second);
            B.xcount[G]    = (int64_t)it->second.size();
        }
    }
    B.order_cnt = b->pool.alloc<int32_t>(2 * (MGPU_MAX_GROUPS + 1));
    ck(cudaMemsetAsync(B.order_cnt, 0, sizeof(int32_t) * 2 * (MGPU_MAX_GROUPS + 1), ctx->stream), "memset");
    ck(cudaStreamSynchronize(ctx->stream), "upload sync");
    trace.mark("tables, lists, sync");
    staging.release();
}

// The per-graph failure words of the batch ([num_graphs], ERR_STEP_CAP / ERR_NONFINITE).
std::vector<int32_t> read_graph_errors(mgpu_batch* b)
{
    std::vector<int32_t> f((size_t)b->num_graphs, 0);
    if (b->num_graphs > 0) {
        ck(cudaMemcpyAsync(f.data(), b->dev.graph_err, sizeof(int32_t) * f.size(), cudaMemcpyDeviceToHost,
                           b->ctx->stream),
           "read graph error words");
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
    }
    return f;
}

// MGPU_STEP_FAILED when instances of some graphs hit the step cap or produced
// non-finite states; those graphs are named (mgpu_batch_get_failed lists all),
// and every other graph of the batch has completed normally.
int check_device_error(mgpu_batch* b)
{
    int32_t err = 0;
    ck(cudaMemcpyAsync(&err, b->dev.err, sizeof(err), cudaMemcpyDeviceToHost, b->ctx->stream), "read error word");
    ck(cudaStreamSynchronize(b->ctx->stream), "sync");
    if (err & ~(ERR_STEP_CAP | ERR_NONFINITE)) {
        fail(MGPU_UNKNOWN_ERROR, "device error word " + std::to_string(err));
    }
    if (err) {
        const std::vector<int32_t> f = read_graph_errors(b);
        std::string which;
        int failed = 0;
        for (int i = 0; i < b->num_graphs; ++i) {
            if (f[(size_t)i]) {
                if (++failed <= 8) {
                    which += " " + std::to_string(i) + ((f[(size_t)i] & ERR_STEP_CAP) ? " (step cap)" : "") +
                             ((f[(size_t)i] & ERR_NONFINITE) ? " (non-finite state)" : "");
                }
            }
        }
        fail(MGPU_STEP_FAILED, "node solves failed in " + std::to_string(failed) + " of " +
                                   std::to_string(b->num_graphs) + " graphs:" + which + (failed > 8 ? " ..." : "") +
                                   "; the other graphs completed (mgpu_batch_get_failed)");
    }
    return MGPU_OK;
}

// node-solve launches per interval: one per age-group count (mixed: with its ordering pass)
int64_t node_kernel_launches(const mgpu_batch* b)
{
    return (int64_t)b->inst_by_G.size() * (is_mixed(b->opts.precision) ? 2 : 1);
}

// One batched interval: interval bookkeeping, node solves per G, exchange.
// With events (profile mode): ev[0] before the node solves, ev[1] after them,
// ev[2] after the exchange.
void enqueue_batched_phase(mgpu_batch* b, cudaStream_t s, cudaEvent_t* ev = nullptr)
{
    const BatchDev& B = b->dev;
    launch_phase_begin(B, b->opts.dt_exchange, s);
    if (ev) {
        ck(cudaEventRecord(ev[0], s), "cudaEventRecord");
    }
    for (auto& kv : b->inst_by_G) {
        auto it       = b->tuned.find(kv.first);
        const int ipb = it != b->tuned.end() ? it->second.first : b->instances_per_block;
        const int grd = it != b->tuned.end() ? it->second.second : 0;
        launch_ode_batched(B, kv.first, b->opts.precision, kv.second.first, kv.second.second, ipb, grd, s);
    }
    if (ev) {
        ck(cudaEventRecord(ev[1], s), "cudaEventRecord");
    }
    int64_t l = 0;
    launch_exchange_batched(B, b->opts.precision, b->n_max, b->any_edge_dampings, s, &l, ev ? ev + 2 : nullptr);
    launch_phase_end(B, s);
    if (ev) {
        ck(cudaEventRecord(ev[5], s), "cudaEventRecord");
    }
}

int64_t phases_needed(const mgpu_batch* b, std::vector<double>& t)
{
    // mirrors k_phase_begin/k_phase_end arithmetic
    int64_t P = 0;
    for (int i = 0; i < b->num_graphs; ++i) {
        int64_t p = 0;
        double tt = t[i];
        while (tt < b->tmax_host[i]) {
            double dt = b->opts.dt_exchange;
            if (tt + dt > b->tmax_host[i]) {
                dt = b->tmax_host[i] - tt;
            }
            tt += dt;
            ++p;
        }
        t[i] = tt;
        P    = std::max(P, p);
    }
    return P;
}

template <class F>
int guarded(mgpu_context* ctx, F&& f)
{
    if (!ctx) {
        return MGPU_INVALID_VALUE;
    }
    try {
        const int rc = f();
        if (rc == MGPU_OK) {
            ctx->error.clear();
        }
        return rc;
    }
    catch (const Fail& e) {
        ctx->error = e.msg;
        return e.code;
    }
    catch (const std::bad_alloc&) {
        ctx->error = "host allocation failed";
        return MGPU_OOM;
    }
    catch (const std::exception& e) {
        ctx->error = e.what();
        return MGPU_UNKNOWN_ERROR;
    }
}

} // namespace

extern "C" {

void mgpu_default_solver_opts(mgpu_solver_opts* o)
{
    if (!o) {
        return;
    }
    std::memset(o, 0, sizeof(*o));
    o->integrator.method  = MGPU_METHOD_CASH_KARP54;
    o->integrator.abs_tol = 1e-10;
    o->integrator.rel_tol = 1e-5;
    o->integrator.dt_min  = DBL_MIN;
    o->integrator.dt_max  = DBL_MAX;
    o->dt0                = 0.1;
    o->dt_exchange        = 0.5;
    o->precision          = MGPU_PRECISION_MIXED;
    o->use_cuda_graph     = 1;
    o->staged_exchange    = 1;
}

int mgpu_create(int device, mgpu_context** out)
{
    if (!out) {
        return MGPU_INVALID_VALUE;
    }
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        return MGPU_CUDA_ERROR;
    }
    if (device < 0 || device >= count) {
        return MGPU_OUT_OF_RANGE;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    auto* ctx   = new (std::nothrow) mgpu_context();
    if (!ctx) {
        return MGPU_OOM;
    }
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return MGPU_CUDA_ERROR;
    }
    // batch allocations come from the device's default memory pool; keep freed
    // blocks there (for the process's next batch) instead of returning them at
    // every synchronisation
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    *out = ctx;
    return MGPU_OK;
}

void mgpu_destroy(mgpu_context* ctx)
{
    if (!ctx) {
        return;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // the context's remaining batches free their device memory on its stream, before it goes
    std::vector<mgpu_batch*> mine;
    {
        std::lock_guard<std::mutex> lock(g_batches_mutex);
        for (auto it = g_batches.begin(); it != g_batches.end();) {
            if ((*it)->ctx == ctx) {
                mine.push_back(*it);
                it = g_batches.erase(it);
            }
            else {
                ++it;
            }
        }
    }
    for (mgpu_batch* b : mine) {
        delete b;
    }
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    if (ctx->pinned) {
        cudaFreeHost(ctx->pinned);
    }
    // return the pool's unused blocks to the device
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        cudaMemPoolTrimTo(pool, 0);
    }
    delete ctx;
}

const char* mgpu_last_error(const mgpu_context* ctx)
{
    return ctx ? ctx->error.c_str() : "no context";
}

int mgpu_set_memory_budget(mgpu_context* ctx, int64_t bytes)
{
    return guarded(ctx, [&]() -> int {
        if (bytes < 0) {
            fail(MGPU_INVALID_VALUE, "negative budget");
        }
        ctx->budget = bytes;
        return MGPU_OK;
    });
}

int mgpu_eval_rhs(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes,
                  const double* pop, const double* y, const double* t, double* dydt)
{
    return guarded(ctx, [&]() -> int {
        if (!graph || count < 0 || (count > 0 && (!nodes || !pop || !y || !t || !dydt))) {
            fail(MGPU_INVALID_VALUE, "null argument");
        }
        if (count == 0) {
            return MGPU_OK;
        }
        ck(cudaSetDevice(ctx->device), "cudaSetDevice");
        mgpu_graph g = *graph;
        g.num_edges  = 0;
        for (int k = 0; k < count; ++k) {
            if (nodes[k] < 0 || nodes[k] >= g.num_nodes) {
                fail(MGPU_OUT_OF_RANGE, "node index out of range");
            }
        }
        mgpu_batch b;
        b.ctx = ctx;
        mgpu_default_solver_opts(&b.opts);
        b.opts.precision = MGPU_PRECISION_FP64_PLAIN; // FP64 states, one thread per node
        build_batch(&b, &g, 1, 0.0, 0.1, false, 0);
        const int n = g.num_groups * kC;
        DevPool io;
        io.ctx = ctx;
        try {
            int32_t* d_nodes = io.alloc<int32_t>(count);
            double* d_pop    = io.alloc<double>((int64_t)count * n);
            double* d_y      = io.alloc<double>((int64_t)count * n);
            double* d_t      = io.alloc<double>(count);
            double* d_out    = io.alloc<double>((int64_t)count * n);
            cudaStream_t s   = ctx->stream;
            ck(cudaMemcpyAsync(d_nodes, nodes, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s), "h2d");
            ck(cudaMemcpyAsync(d_pop, pop, sizeof(double) * count * n, cudaMemcpyHostToDevice, s), "h2d");
            ck(cudaMemcpyAsync(d_y, y, sizeof(double) * count * n, cudaMemcpyHostToDevice, s), "h2d");
            ck(cudaMemcpyAsync(d_t, t, sizeof(double) * count, cudaMemcpyHostToDevice, s), "h2d");
            launch_eval_rhs(b.dev, d_nodes, count, d_pop, d_y, d_t, d_out, s);
            ck(cudaGetLastError(), "k_eval_rhs");
            ck(cudaMemcpyAsync(dydt, d_out, sizeof(double) * count * n, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaStreamSynchronize(s), "sync");
        }
        catch (...) {
            io.release();
            throw;
        }
        io.release();
        return MGPU_OK;
    });
}

namespace
{
// mgpu_simulate and mgpu_simulate_dt; dt_io (host, may be null) holds the
// per-node step size in and out
int simulate_impl(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                  double tmax, double dt0, double* dt_io, const mgpu_integrator_opts* opts, int32_t max_points,
                  double* out_t, double* out_y, int32_t* num_points)
{
    return guarded(ctx, [&]() -> int {
        if (!graph || !opts || count < 0 || max_points < 1 ||
            (count > 0 && (!nodes || !out_t || !out_y || !num_points))) {
            fail(MGPU_INVALID_VALUE, "null argument");
        }
        if (!(dt0 > 0)) {
            fail(MGPU_INVALID_VALUE, "dt0 must be > 0");
        }
        for (int k = 0; dt_io && k < count; ++k) {
            if (!(dt_io[k] > 0)) {
                fail(MGPU_INVALID_VALUE, "dt must be > 0");
            }
        }
        if (count == 0) {
            return MGPU_OK;
        }
        ck(cudaSetDevice(ctx->device), "cudaSetDevice");
        mgpu_graph g = *graph;
        g.num_edges  = 0;
        for (int k = 0; k < count; ++k) {
            if (nodes[k] < 0 || nodes[k] >= g.num_nodes) {
                fail(MGPU_OUT_OF_RANGE, "node index out of range");
            }
        }
        mgpu_batch b;
        b.ctx = ctx;
        mgpu_default_solver_opts(&b.opts);
        b.opts.precision = MGPU_PRECISION_FP64_PLAIN; // FP64 states, one thread per node
        b.opts.integrator = *opts;
        build_batch(&b, &g, 1, t0, dt0, false, count);
        const int n = g.num_groups * kC;
        DevPool io;
        io.ctx = ctx;
        int rc = MGPU_OK;
        try {
            int32_t* d_nodes = io.alloc<int32_t>(count);
            double* d_t      = io.alloc<double>((int64_t)count * max_points);
            double* d_y      = io.alloc<double>((int64_t)count * max_points * n);
            int32_t* d_np    = io.alloc<int32_t>(count);
            double* d_dt     = dt_io ? io.alloc<double>(count) : nullptr;
            cudaStream_t s   = ctx->stream;
            ck(cudaMemcpyAsync(d_nodes, nodes, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s), "h2d");
            if (d_dt) {
                ck(cudaMemcpyAsync(d_dt, dt_io, sizeof(double) * count, cudaMemcpyHostToDevice, s), "h2d");
            }
            launch_simulate(b.dev, d_nodes, count, t0, tmax, dt0, max_points, d_t, d_y, d_np, s, d_dt);
            ck(cudaGetLastError(), "k_simulate");
            if (d_dt) {
                ck(cudaMemcpyAsync(dt_io, d_dt, sizeof(double) * count, cudaMemcpyDeviceToHost, s), "d2h");
            }
            ck(cudaMemcpyAsync(num_points, d_np, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(out_t, d_t, sizeof(double) * count * max_points, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(out_y, d_y, sizeof(double) * count * max_points * n, cudaMemcpyDeviceToHost, s),
               "d2h");
            ck(cudaStreamSynchronize(s), "sync");
            for (int k = 0; k < count; ++k) {
                if (num_points[k] < 0) {
                    num_points[k] = max_points;
                    rc            = MGPU_OUT_OF_RANGE;
                }
            }
            check_device_error(&b);
        }
        catch (...) {
            io.release();
            throw;
        }
        io.release();
        if (rc != MGPU_OK) {
            ctx->error = "trajectory longer than max_points";
        }
        return rc;
    });
}
} // namespace

int mgpu_simulate(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                  double tmax, double dt0, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                  double* out_y, int32_t* num_points)
{
    return simulate_impl(ctx, graph, count, nodes, t0, tmax, dt0, nullptr, opts, max_points, out_t, out_y,
                         num_points);
}

int mgpu_simulate_flows(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                        double tmax, double dt0, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                        double* out_flows, double* out_y, int32_t* num_points)
{
    return guarded(ctx, [&]() -> int {
        if (!graph || !opts || count < 0 || max_points < 1 ||
            (count > 0 && (!nodes || !out_t || !out_flows || !out_y || !num_points))) {
            fail(MGPU_INVALID_VALUE, "null argument");
        }
        if (!(dt0 > 0)) {
            fail(MGPU_INVALID_VALUE, "dt0 must be > 0");
        }
        if (count == 0) {
            return MGPU_OK;
        }
        ck(cudaSetDevice(ctx->device), "cudaSetDevice");
        mgpu_graph g = *graph;
        g.num_edges  = 0;
        for (int k = 0; k < count; ++k) {
            if (nodes[k] < 0 || nodes[k] >= g.num_nodes) {
                fail(MGPU_OUT_OF_RANGE, "node index out of range");
            }
        }
        mgpu_batch b;
        b.ctx = ctx;
        mgpu_default_solver_opts(&b.opts);
        b.opts.precision  = MGPU_PRECISION_FP64_PLAIN;
        b.opts.integrator = *opts;
        build_batch(&b, &g, 1, t0, dt0, false, 0);
        const int n  = g.num_groups * kC;
        const int nf = g.num_groups * kF;
        DevPool io;
        io.ctx = ctx;
        int rc = MGPU_OK;
        try {
            int32_t* d_nodes = io.alloc<int32_t>(count);
            double* d_t      = io.alloc<double>((int64_t)count * max_points);
            double* d_f      = io.alloc<double>((int64_t)count * max_points * nf);
            double* d_y      = io.alloc<double>((int64_t)count * max_points * n);
            int32_t* d_np    = io.alloc<int32_t>(count);
            double* d_rows   = io.alloc<double>((int64_t)count * nf);
            BatchDev B       = b.dev;
            B.scratch        = io.alloc<double>((int64_t)8 * nf * count);
            B.scratch_stride = count;
            B.scratch_nmax   = nf;
            cudaStream_t s   = ctx->stream;
            ck(cudaMemcpyAsync(d_nodes, nodes, sizeof(int32_t) * count, cudaMemcpyHostToDevice, s), "h2d");
            launch_simulate_flows(B, d_nodes, count, t0, tmax, dt0, max_points, d_t, d_f, d_y, d_np, nf, d_rows, s);
            ck(cudaGetLastError(), "k_simulate_flows");
            ck(cudaMemcpyAsync(num_points, d_np, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(out_t, d_t, sizeof(double) * count * max_points, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaMemcpyAsync(out_flows, d_f, sizeof(double) * count * max_points * nf, cudaMemcpyDeviceToHost, s),
               "d2h");
            ck(cudaMemcpyAsync(out_y, d_y, sizeof(double) * count * max_points * n, cudaMemcpyDeviceToHost, s),
               "d2h");
            ck(cudaStreamSynchronize(s), "sync");
            for (int k = 0; k < count; ++k) {
                if (num_points[k] < 0) {
                    num_points[k] = max_points;
                    rc            = MGPU_OUT_OF_RANGE;
                }
            }
            check_device_error(&b);
        }
        catch (...) {
            io.release();
            throw;
        }
        io.release();
        if (rc != MGPU_OK) {
            ctx->error = "trajectory longer than max_points";
        }
        return rc;
    });
}

int mgpu_simulate_dt(mgpu_context* ctx, const mgpu_graph* graph, int32_t count, const int32_t* nodes, double t0,
                     double tmax, double* dt, const mgpu_integrator_opts* opts, int32_t max_points, double* out_t,
                     double* out_y, int32_t* num_points)
{
    if (count > 0 && !dt) {
        return MGPU_INVALID_VALUE;
    }
    return simulate_impl(ctx, graph, count, nodes, t0, tmax, count > 0 ? dt[0] : 1.0, dt, opts, max_points, out_t,
                         out_y, num_points);
}

int mgpu_batch_create(mgpu_context* ctx, const mgpu_graph* graphs, int32_t num_graphs, double t0,
                      const mgpu_solver_opts* opts, mgpu_batch** out)
{
    return guarded(ctx, [&]() -> int {
        if (!graphs || num_graphs < 1 || !out) {
            fail(MGPU_INVALID_VALUE, "null argument or no graphs");
        }
        *out = nullptr;
        mgpu_solver_opts o;
        if (opts) {
            o = *opts;
        }
        else {
            mgpu_default_solver_opts(&o);
        }
        if (!(o.dt_exchange > 0) || !(o.dt0 > 0)) {
            fail(MGPU_INVALID_VALUE, "dt0 and dt_exchange must be > 0");
        }
        if (o.precision < MGPU_PRECISION_FP64_PLAIN || o.precision > MGPU_PRECISION_MIXED_FP64_CONTROL) {
            fail(MGPU_INVALID_VALUE, "unknown precision");
        }
        if (o.precision != MGPU_PRECISION_FP64_PLAIN && o.integrator.method != MGPU_METHOD_CASH_KARP54) {
            fail(MGPU_UNSUPPORTED, "the batched solvers implement Cash-Karp 5(4) only; use MGPU_PRECISION_FP64_PLAIN");
        }
        ck(cudaSetDevice(ctx->device), "cudaSetDevice");
        auto* b = new mgpu_batch();
        b->ctx  = ctx;
        b->opts = o;
        try {
            int64_t max_nodes = 0;
            for (int i = 0; i < num_graphs; ++i) {
                max_nodes = std::max<int64_t>(max_nodes, graphs[i].num_nodes);
            }
            const int64_t slots = (o.precision == MGPU_PRECISION_FP64_PLAIN) ? max_nodes : 0;
            build_batch(b, graphs, num_graphs, t0, o.dt0, true, slots);
            b->instances_per_block = o.instances_per_block;
        }
        catch (...) {
            delete b;
            throw;
        }
        {
            std::lock_guard<std::mutex> lock(g_batches_mutex);
            g_batches.insert(b);
        }
        *out = b;
        return MGPU_OK;
    });
}

int mgpu_batch_regroup(mgpu_context* ctx, const mgpu_graph* graphs, int32_t num_graphs, mgpu_batch* const* src,
                       const int32_t* src_graph, mgpu_batch** out)
{
    return guarded(ctx, [&]() -> int {
        if (!graphs || num_graphs < 1 || !src || !src_graph || !out) {
            fail(MGPU_INVALID_VALUE, "null argument or no graphs");
        }
        *out = nullptr;
        {
            std::lock_guard<std::mutex> lock(g_batches_mutex);
            for (int i = 0; i < num_graphs; ++i) {
                if (!src[i] || !g_batches.count(src[i])) {
                    fail(MGPU_INVALID_VALUE, "source " + std::to_string(i) + " is not a live batch");
                }
            }
        }
        const mgpu_solver_opts o = src[0]->opts;
        if (o.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "regrouping needs a batched precision");
        }
        std::vector<GraphRt> rts((size_t)num_graphs);
        for (int i = 0; i < num_graphs; ++i) {
            mgpu_batch* sb = src[i];
            const int j    = src_graph[i];
            if (j < 0 || j >= sb->num_graphs) {
                fail(MGPU_OUT_OF_RANGE, "source graph index out of range");
            }
            if (sb->ctx->device != ctx->device || sb->opts.precision != o.precision ||
                sb->opts.dt_exchange != o.dt_exchange || sb->dev.flows || !sb->stats_host.empty()) {
                fail(MGPU_UNSUPPORTED, "sources differ in device, precision or exchange interval, or record "
                                       "flows or commuter statistics");
            }
            if (sb->half_step) {
                fail(MGPU_INVALID_VALUE, "a source batch awaits mgpu_batch_step_exchange");
            }
            if (sb->async_active && cudaEventQuery(sb->ev_async) != cudaSuccess) {
                cudaGetLastError(); // (not-ready is no error of this call)
                fail(MGPU_INVALID_VALUE, "a source batch's launched intervals are still running");
            }
            const DevGraph& d = sb->host_graphs[(size_t)j];
            if (graphs[i].num_nodes != d.N || graphs[i].num_groups != d.G || graphs[i].num_edges != d.E) {
                fail(MGPU_INVALID_VALUE, "graph " + std::to_string(i) + " is not the source graph's shape");
            }
            ck(cudaSetDevice(sb->ctx->device), "cudaSetDevice");
            ck(cudaMemcpyAsync(&rts[(size_t)i], sb->dev.rt + j, sizeof(GraphRt), cudaMemcpyDeviceToHost,
                               sb->ctx->stream),
               "d2h graph record");
            ck(cudaStreamSynchronize(sb->ctx->stream), "sync");
            if (rts[(size_t)i].has_pending) {
                fail(MGPU_INVALID_VALUE, "graph " + std::to_string(i) + " has travelers away");
            }
        }
        mgpu_batch* b = nullptr;
        const int rc  = mgpu_batch_create(ctx, graphs, num_graphs, 0.0, &o, &b);
        if (rc != MGPU_OK) {
            return rc;
        }
        try {
            cudaStream_t s = ctx->stream;
            for (int i = 0; i < num_graphs; ++i) {
                const mgpu_batch* sb = src[i];
                const int j          = src_graph[i];
                const int64_t cnt    = (int64_t)b->N[(size_t)i] * b->n[(size_t)i];
                const int64_t so     = sb->state_off[(size_t)j], dn = b->state_off[(size_t)i];
                if (b->pairs) {
                    ck(cudaMemcpyAsync(b->dev.st_hi + dn, sb->dev.st_hi + so, sizeof(float) * cnt,
                                       cudaMemcpyDeviceToDevice, s),
                       "d2d state");
                    ck(cudaMemcpyAsync(b->dev.st_lo + dn, sb->dev.st_lo + so, sizeof(float) * cnt,
                                       cudaMemcpyDeviceToDevice, s),
                       "d2d state");
                }
                else {
                    ck(cudaMemcpyAsync(b->dev.state + dn, sb->dev.state + so, sizeof(double) * cnt,
                                       cudaMemcpyDeviceToDevice, s),
                       "d2d state");
                }
                const int64_t N = b->N[(size_t)i];
                ck(cudaMemcpyAsync(b->dev.node_t + b->node0[(size_t)i], sb->dev.node_t + sb->node0[(size_t)j],
                                   sizeof(double) * N, cudaMemcpyDeviceToDevice, s),
                   "d2d node times");
                ck(cudaMemcpyAsync(b->dev.node_dt + b->node0[(size_t)i], sb->dev.node_dt + sb->node0[(size_t)j],
                                   sizeof(double) * N, cudaMemcpyDeviceToDevice, s),
                   "d2d node steps");
                ck(cudaMemcpyAsync(b->dev.rt + i, &rts[(size_t)i], sizeof(GraphRt), cudaMemcpyHostToDevice, s),
                   "h2d graph record");
                ck(cudaMemcpyAsync(b->dev.graph_err + i, sb->dev.graph_err + j, sizeof(int32_t),
                                   cudaMemcpyDeviceToDevice, s),
                   "d2d failure word");
                // (the source's host mirror of the time lags during an asynchronous advance)
                b->t_host[(size_t)i]    = rts[(size_t)i].t;
                b->tmax_host[(size_t)i] = rts[(size_t)i].tmax;
            }
            // a graph that failed before keeps failing the advances of the new batch
            const std::vector<int32_t> f = read_graph_errors(b);
            int32_t any = 0;
            for (int32_t x : f) {
                any |= x;
            }
            if (any) {
                ck(cudaMemcpyAsync(b->dev.err, &any, sizeof(int32_t), cudaMemcpyHostToDevice, s), "h2d error word");
            }
            ck(cudaStreamSynchronize(s), "sync");
        }
        catch (...) {
            mgpu_batch_destroy(b);
            throw;
        }
        *out = b;
        return MGPU_OK;
    });
}

int mgpu_batch_advance(mgpu_batch* b, double tmax, const double* tmax_per_graph)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        if (b->half_step) {
            fail(MGPU_INVALID_VALUE, "the interval begun by mgpu_batch_step_nodes awaits mgpu_batch_step_exchange");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        for (int i = 0; i < b->num_graphs; ++i) {
            b->tmax_host[i] = tmax_per_graph ? tmax_per_graph[i] : tmax;
        }
        ck(cudaMemcpyAsync(b->d_tmax, b->tmax_host.data(), sizeof(double) * b->num_graphs, cudaMemcpyHostToDevice,
                           s),
           "h2d tmax");
        if (!b->ev_start) {
            ck(cudaEventCreate(&b->ev_start), "cudaEventCreate");
            ck(cudaEventCreate(&b->ev_stop), "cudaEventCreate");
        }
        unsigned long long c0[CNT_NUM];
        ck(cudaMemcpyAsync(c0, b->dev.counters, sizeof(c0), cudaMemcpyDeviceToHost, s), "d2h counters");
        ck(cudaStreamSynchronize(s), "sync");
        const int64_t attempts0 = (int64_t)(c0[CNT_ACCEPTED] + c0[CNT_REJECTED]);
        std::vector<size_t> ev_base;
        size_t nev           = 0;
        bool six_events      = false; // batched phases: start, ODE, prep, return, exact path, end
        int64_t ode_launches = 0;
        ck(cudaEventRecord(b->ev_start, s), "cudaEventRecord");
        k_set_tmax<<<(b->num_graphs + 127) / 128, 128, 0, s>>>(b->dev.rt, b->d_tmax, b->num_graphs);
        ++b->launches;
        std::vector<double> t_end = b->t_host;
        const int64_t P           = phases_needed(b, t_end);
        const BatchDev& B         = b->dev;
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            // the plain drop-in: graphs one after another, as ParameterStudy runs them
            for (int i = 0; i < b->num_graphs; ++i) {
                BatchDev Bi   = B;
                std::vector<double> ti(1, b->t_host[i]);
                int64_t Pi    = 0;
                {
                    double tt = b->t_host[i];
                    while (tt < b->tmax_host[i]) {
                        double dt = b->opts.dt_exchange;
                        if (tt + dt > b->tmax_host[i]) {
                            dt = b->tmax_host[i] - tt;
                        }
                        tt += dt;
                        ++Pi;
                    }
                }
                // restrict every kernel to graph i
                Bi.graphs     = B.graphs + i;
                Bi.rt         = B.rt + i;
                Bi.num_graphs = 1;
                for (int64_t p = 0; p < Pi; ++p) {
                    cudaEvent_t* ev = nullptr;
                    if (b->opts.profile) {
                        ev_base.push_back(nev);
                        b->phase_event(nev + 2);
                        ev = &b->ev_phase[nev];
                        nev += 3;
                    }
                    launch_phase_begin(Bi, b->opts.dt_exchange, s);
                    if (ev) {
                        ck(cudaEventRecord(ev[0], s), "cudaEventRecord");
                    }
                    launch_ode_plain(B, b->node0[i], b->node0[i] + b->N[i], s);
                    if (ev) {
                        ck(cudaEventRecord(ev[1], s), "cudaEventRecord");
                    }
                    int64_t l = 0;
                    launch_exchange_range(B, i, 1, b->node0[i], b->N[i], b->edge0[i],
                                          (i + 1 < b->num_graphs ? b->edge0[i + 1] : B.num_edges) - b->edge0[i],
                                          b->n[i], s, &l);
                    launch_phase_end(Bi, s);
                    if (ev) {
                        ck(cudaEventRecord(ev[2], s), "cudaEventRecord");
                    }
                    b->launches += 3 + l;
                    ++ode_launches;
                }
                b->phases += Pi;
            }
        }
        else if (b->opts.profile) {
            for (int64_t p = 0; p < P; ++p) {
                b->phase_event(nev + 5);
                ev_base.push_back(nev);
                enqueue_batched_phase(b, s, &b->ev_phase[nev]);
                nev += 6;
                six_events = true;
                ode_launches += (int64_t)b->inst_by_G.size(); // node-solve kernels (their ordering passes excluded)
            }
            b->launches +=
                P * (2 + node_kernel_launches(b) + exchange_batched_launches(b->dev, b->opts.precision, b->any_edge_dampings));
            b->phases += P;
        }
        else {
            const bool use_graph = b->opts.use_cuda_graph && !b->graph_failed;
            if (use_graph && !b->graph_exec && P > 0) {
                cudaGraph_t graph = nullptr;
                ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
                enqueue_batched_phase(b, s);
                cudaError_t e = cudaStreamEndCapture(s, &graph);
                if (e == cudaSuccess) {
                    e = cudaGraphInstantiate(&b->graph_exec, graph, 0);
                    cudaGraphDestroy(graph);
                }
                if (e != cudaSuccess) {
                    cudaGetLastError();
                    b->graph_failed = true;
                    b->graph_exec   = nullptr;
                }
            }
            const int64_t per_phase = 2 + node_kernel_launches(b) +
                                      exchange_batched_launches(b->dev, b->opts.precision, b->any_edge_dampings);
            for (int64_t p = 0; p < P; ++p) {
                if (b->graph_exec) {
                    ck(cudaGraphLaunch(b->graph_exec, s), "cudaGraphLaunch");
                }
                else {
                    enqueue_batched_phase(b, s);
                }
            }
            b->launches += P * per_phase;
            b->phases += P;
        }
        ck(cudaGetLastError(), "advance launch");
        ck(cudaEventRecord(b->ev_stop, s), "cudaEventRecord");
        b->t_host = t_end;
        const int rc = check_device_error(b);
        float ms = 0.0f;
        ck(cudaEventElapsedTime(&ms, b->ev_start, b->ev_stop), "cudaEventElapsedTime");
        b->timing.advance_ms = ms;
        double ode = 0.0, exch = 0.0, part[4] = {0.0, 0.0, 0.0, 0.0};
        const int last = six_events ? 5 : 2;
        for (size_t k : ev_base) {
            float a = 0.0f, c = 0.0f;
            ck(cudaEventElapsedTime(&a, b->ev_phase[k], b->ev_phase[k + 1]), "cudaEventElapsedTime");
            ck(cudaEventElapsedTime(&c, b->ev_phase[k + 1], b->ev_phase[k + last]), "cudaEventElapsedTime");
            ode += a;
            exch += c;
            if (six_events) {
                for (int q = 0; q < 4; ++q) {
                    float x = 0.0f;
                    ck(cudaEventElapsedTime(&x, b->ev_phase[k + 1 + q], b->ev_phase[k + 2 + q]),
                       "cudaEventElapsedTime");
                    part[q] += x;
                }
            }
        }
        b->timing.ode_ms       = ode;
        b->timing.exchange_ms  = exch;
        b->timing.prep_ms      = part[0];
        b->timing.return_ms    = part[1];
        b->timing.exact_ms     = part[2];
        b->timing.depart_ms    = part[3];
        b->timing.ode_launches = ode_launches;
        unsigned long long c1[CNT_NUM];
        ck(cudaMemcpy(c1, b->dev.counters, sizeof(c1), cudaMemcpyDeviceToHost), "d2h counters");
        b->timing.attempts = (int64_t)(c1[CNT_ACCEPTED] + c1[CNT_REJECTED]) - attempts0;
        return rc;
    });
}

int mgpu_batch_launch(mgpu_batch* b, double tmax, const double* tmax_per_graph, int32_t max_phases,
                      int32_t* remaining)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (max_phases < 1 || !remaining) {
            fail(MGPU_INVALID_VALUE, "max_phases must be >= 1 and remaining non-null");
        }
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "asynchronous advance needs a batched precision");
        }
        if (b->half_step) {
            fail(MGPU_INVALID_VALUE, "the interval begun by mgpu_batch_step_nodes awaits mgpu_batch_step_exchange");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        if (!b->async_active) {
            for (int i = 0; i < b->num_graphs; ++i) {
                b->tmax_host[i] = tmax_per_graph ? tmax_per_graph[i] : tmax;
            }
            ck(cudaMemcpyAsync(b->d_tmax, b->tmax_host.data(), sizeof(double) * b->num_graphs,
                               cudaMemcpyHostToDevice, s),
               "h2d tmax");
            k_set_tmax<<<(b->num_graphs + 127) / 128, 128, 0, s>>>(b->dev.rt, b->d_tmax, b->num_graphs);
            ++b->launches;
            b->async_t_end  = b->t_host;
            b->async_left   = phases_needed(b, b->async_t_end);
            b->async_active = true;
            if (!b->ev_async) {
                ck(cudaEventCreateWithFlags(&b->ev_async, cudaEventDisableTiming), "cudaEventCreate");
            }
        }
        const int64_t n = std::min<int64_t>(max_phases, b->async_left);
        const bool use_graph = b->opts.use_cuda_graph && !b->graph_failed;
        if (use_graph && !b->graph_exec && n > 0) {
            cudaGraph_t graph = nullptr;
            ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
            enqueue_batched_phase(b, s);
            cudaError_t e = cudaStreamEndCapture(s, &graph);
            if (e == cudaSuccess) {
                e = cudaGraphInstantiate(&b->graph_exec, graph, 0);
                cudaGraphDestroy(graph);
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                b->graph_failed = true;
                b->graph_exec   = nullptr;
            }
        }
        for (int64_t p = 0; p < n; ++p) {
            if (b->graph_exec) {
                ck(cudaGraphLaunch(b->graph_exec, s), "cudaGraphLaunch");
            }
            else {
                enqueue_batched_phase(b, s);
            }
        }
        ck(cudaGetLastError(), "launch");
        b->launches += n * (2 + node_kernel_launches(b) +
                            exchange_batched_launches(b->dev, b->opts.precision, b->any_edge_dampings));
        b->phases += n;
        b->async_left -= n;
        ck(cudaEventRecord(b->ev_async, s), "cudaEventRecord");
        *remaining = (int32_t)b->async_left;
        return MGPU_OK;
    });
}

int mgpu_batch_query(mgpu_batch* b, int32_t* done)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!done) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        *done = 1;
        if (!b->async_active) {
            return MGPU_OK;
        }
        const cudaError_t e = cudaEventQuery(b->ev_async);
        if (e == cudaErrorNotReady) {
            *done = 0;
            return MGPU_OK;
        }
        ck(e, "cudaEventQuery");
        if (b->async_left > 0) {
            return MGPU_OK; // the launched intervals are done; more remain
        }
        b->async_active = false;
        b->t_host       = b->async_t_end;
        return check_device_error(b);
    });
}

// Float-float node states [off, off + cnt) as FP64 into host memory: combined on
// the device (hi + lo in FP64 is exact), copied into the context's page-locked
// staging, then into `out` on the host's cores.
void read_pairs(mgpu_batch* b, int64_t off, int64_t cnt, double* out)
{
    cudaStream_t s = b->ctx->stream;
    if (!b->d_out) {
        b->d_out = b->pool.alloc<double>(b->state_total);
    }
    k_pairs_to_double<<<(unsigned)std::max<int64_t>((cnt + 255) / 256, 1), 256, 0, s>>>(
        b->dev.st_hi + off, b->dev.st_lo + off, cnt, b->d_out + off);
    ck(cudaGetLastError(), "k_pairs_to_double");
    ck(cudaStreamSynchronize(s), "sync");
    HostSpan<double> stage;
    StagingArena arena{b->ctx};
    arena.take(stage, cnt);
    arena.place();
    ck(cudaMemcpyAsync(stage.data(), b->d_out + off, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s), "d2h state");
    ck(cudaStreamSynchronize(s), "sync");
    const int64_t chunk = 1 << 20;
    parallel_for((cnt + chunk - 1) / chunk, [&](int64_t k) {
        const int64_t a = k * chunk;
        std::memcpy(out + a, stage.data() + a, sizeof(double) * (size_t)std::min(chunk, cnt - a));
    });
}

int mgpu_batch_get_graph_state(mgpu_batch* b, int32_t graph, double* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out || graph < 0 || graph >= b->num_graphs) {
            fail(MGPU_INVALID_VALUE, "null output or graph index out of range");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const int64_t off = b->state_off[graph];
        const int64_t cnt = (int64_t)b->N[graph] * b->n[graph];
        if (cnt == 0) {
            return MGPU_OK;
        }
        cudaStream_t s = b->ctx->stream;
        if (b->pairs) {
            read_pairs(b, off, cnt, out);
        }
        else {
            ck(cudaMemcpyAsync(out, b->dev.state + off, sizeof(double) * cnt, cudaMemcpyDeviceToHost, s), "d2h");
            ck(cudaStreamSynchronize(s), "sync");
        }
        return MGPU_OK;
    });
}

int64_t mgpu_batch_estimate_bytes(const mgpu_graph* graphs, int32_t num_graphs, const mgpu_solver_opts* opts)
{
    if (!graphs || num_graphs < 1) {
        return -1;
    }
    mgpu_solver_opts o;
    if (opts) {
        o = *opts;
    }
    else {
        mgpu_default_solver_opts(&o);
    }
    const bool plain = o.precision == MGPU_PRECISION_FP64_PLAIN;
    const bool mixed = is_mixed(o.precision);
    int64_t nodes = 0, edges = 0, st = 0, tr = 0, par = 0, con = 0, dtv = 0, dtt = 0, ec = 0, edv = 0, edt = 0,
            nmax = 0;
    for (int i = 0; i < num_graphs; ++i) {
        const mgpu_graph& g = graphs[i];
        const int64_t G = g.num_groups, n = 10 * G, N = g.num_nodes, E = g.num_edges, M = g.num_contact_matrices,
                      K = g.num_damping_points, Ke = g.num_edge_damping_points;
        nodes += N;
        edges += E;
        st += N * n;
        tr += E * n;
        par += N * MGPU_PARAM_STRIDE(G);
        con += N * M * 2 * G * G;
        dtt += N * M * K;
        dtv += N * M * K * G * G;
        ec += E * 2 * n;
        edt += E * Ke;
        edv += E * Ke * n;
        nmax = std::max<int64_t>(nmax, N);
    }
    int64_t b = 8 * (par + con + dtt + dtv + ec + edt + edv) + (mixed ? 4 * (tr / kC) * kRec : 0); // inputs, FP32 coefficients
    b += mixed ? 4 * st * 8 + 8 * st + 4 * nodes * MGPU_MAX_GROUPS * kTabF + 4 * (con + dtv) : 8 * st * 4;
    // snapshots (mixed: two slots of records), factors, auxiliary values
    b += plain ? 8 * st + 8 * tr + 8 * 8 * nmax * 60
               : (mixed ? 4 * 2 * (st / kC) * kRec : 8 * st * 2 + 8 * nodes * MGPU_MAX_GROUPS * 4) +
                     8 * nodes * MGPU_MAX_GROUPS * 12;
    b += 8 * tr;                                             // fixed travelers
    b += 24 * nodes + 4 * 2 * 3 * nodes * MGPU_MAX_GROUPS + 4 * nodes + 3 * nodes + 16 * (nodes + 1);
    b += edges * (4 + 4 + 8 + 1 + 1 + 4 + 8 + 8 + 4 + MGPU_MAX_GROUPS);
    b += num_graphs * (int64_t)(sizeof(DevGraph) + sizeof(GraphRt) + 8) + 64 * 1024;
    return b + b / 10;
}

int mgpu_batch_autotune(mgpu_batch* b, int32_t* instances_per_block, int32_t* grid_blocks)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "the autotuner schedules the batched solvers");
        }
        if (b->half_step) {
            fail(MGPU_INVALID_VALUE, "the interval begun by mgpu_batch_step_nodes awaits mgpu_batch_step_exchange");
        }
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s   = b->ctx->stream;
        const BatchDev& B = b->dev;
        // snapshot of everything one interval of node solves changes
        struct Saved {
            void* dst;
            void* copy;
            size_t bytes;
        };
        std::vector<Saved> saved;
        DevPool tmp;
        tmp.ctx  = b->ctx;
        auto keep = [&](void* p, size_t bytes) {
            if (p && bytes) {
                void* c = tmp.alloc<char>((int64_t)bytes);
                ck(cudaMemcpyAsync(c, p, bytes, cudaMemcpyDeviceToDevice, s), "d2d");
                saved.push_back({p, c, bytes});
            }
        };
        int best_ipb = 0, best_grid = 0;
        std::function<void()> restore_all;
        try {
            const size_t st = (size_t)b->state_total;
            if (b->pairs) {
                keep(B.st_hi, st * sizeof(float));
                keep(B.st_lo, st * sizeof(float));
            }
            else {
                keep(B.state, st * sizeof(double));
            }
            keep(B.node_t, sizeof(double) * (size_t)B.num_nodes);
            keep(B.node_dt, sizeof(double) * (size_t)B.num_nodes);
            keep(B.rt, sizeof(GraphRt) * (size_t)b->num_graphs);
            keep(B.counters, sizeof(unsigned long long) * CNT_NUM);
            keep(B.err, sizeof(int32_t));
            keep(B.graph_err, sizeof(int32_t) * (size_t)b->num_graphs);
            if (B.flows) {
                keep(B.flows, sizeof(double) * (size_t)(b->state_total / kC) * kF);
            }
            for (int i = 0; i < b->num_graphs && !b->stats_host.empty(); ++i) {
                if (b->stats_host[(size_t)i].num_sets) {
                    keep(b->stats_host[(size_t)i].count, sizeof(int32_t) * (size_t)b->host_graphs[(size_t)i].E);
                }
            }
            keep(b->d_tmax, sizeof(double) * (size_t)b->num_graphs);
            restore_all = [&]() {
                for (auto& x : saved) {
                    ck(cudaMemcpyAsync(x.dst, x.copy, x.bytes, cudaMemcpyDeviceToDevice, s), "d2d");
                }
            };
            auto& restore = restore_all;
            // one interval for every graph: horizon t + dt_exchange
            std::vector<double> h(b->num_graphs);
            for (int i = 0; i < b->num_graphs; ++i) {
                h[i] = b->t_host[i] + b->opts.dt_exchange;
            }
            ck(cudaMemcpyAsync(b->d_tmax, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s), "h2d");
            cudaEvent_t e0, e1;
            ck(cudaEventCreate(&e0), "cudaEventCreate");
            ck(cudaEventCreate(&e1), "cudaEventCreate");
            // the node-solve kernels take at most 128 threads per block (their launch bounds)
            const int warps_c[3] = {1, 2, 4};
            const int grid_c[5]  = {0, 152 * 2, 152 * 3, 152 * 4, 152 * 6};
            size_t most = 0;
            for (auto& kv : b->inst_by_G) {
                const int G   = kv.first;
                const int ipw = 32 / G;
                float best    = 1e30f;
                std::pair<int, int> pick{4 * ipw, 0};
                for (int w : warps_c) {
                    for (int gr : grid_c) {
                        k_set_tmax<<<(b->num_graphs + 127) / 128, 128, 0, s>>>(B.rt, b->d_tmax, b->num_graphs);
                        launch_phase_begin(B, b->opts.dt_exchange, s);
                        ck(cudaEventRecord(e0, s), "cudaEventRecord");
                        launch_ode_batched(B, G, b->opts.precision, kv.second.first, kv.second.second, w * ipw, gr, s);
                        ck(cudaEventRecord(e1, s), "cudaEventRecord");
                        ck(cudaGetLastError(), "autotune launch");
                        restore();
                        ck(cudaStreamSynchronize(s), "sync");
                        float ms = 0.0f;
                        ck(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
                        if (ms < best) {
                            best = ms;
                            pick = {w * ipw, gr};
                        }
                    }
                }
                b->tuned[G] = pick;
                if ((size_t)kv.second.second > most) {
                    most      = (size_t)kv.second.second;
                    best_ipb  = pick.first;
                    best_grid = pick.second;
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (b->graph_exec) {
                cudaGraphExecDestroy(b->graph_exec); // recaptured with the tuned schedule
                b->graph_exec = nullptr;
            }
        }
        catch (...) {
            // put the batch back as it was before the failed candidate
            cudaGetLastError();
            if (restore_all) {
                try {
                    restore_all();
                    cudaStreamSynchronize(s);
                }
                catch (...) {
                }
            }
            b->tuned.clear();
            tmp.release();
            throw;
        }
        tmp.release();
        if (instances_per_block) {
            *instances_per_block = best_ipb;
        }
        if (grid_blocks) {
            *grid_blocks = best_grid;
        }
        return MGPU_OK;
    });
}

namespace
{
// ensemble_mean / ensemble_percentile (cpp/memilio/data/analyze_result.h:289-338) of
// one (node, compartment) column over the graphs of a batch: one block per
// column, the values sorted in shared memory (bitonic, padded with +inf to a
// power of two); mean = sum over runs of x / runs, in run order.
__global__ void k_ensemble_stats(BatchDev B, const int64_t* state_off, int runs, int pow2, int64_t n_col,
                                 const double* p, int num_p, double* mean, double* pct)
{
    extern __shared__ double vals[];
    const int64_t col = blockIdx.x;
    if (col >= n_col) {
        return;
    }
    for (int r = threadIdx.x; r < pow2; r += blockDim.x) {
        vals[r] = r < runs ? state_get(B, state_off[r] + col) : INFINITY;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int r = 0; r < runs; ++r) {
            m += vals[r] / runs;
        }
        mean[col] = m;
    }
    __syncthreads();
    for (int k = 2; k <= pow2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const double a = vals[i], b = vals[l];
                    if ((a > b) == up) {
                        vals[i] = b;
                        vals[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int q = threadIdx.x; q < num_p; q += blockDim.x) {
        pct[(int64_t)q * n_col + col] = vals[(int)((double)runs * p[q])];
    }
}
} // namespace

int mgpu_batch_ensemble_stats(mgpu_batch* b, const double* percentiles, int32_t num_percentiles, double* mean,
                              double* out_percentiles)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!mean || num_percentiles < 0 || (num_percentiles > 0 && (!percentiles || !out_percentiles))) {
            fail(MGPU_INVALID_VALUE, "null argument");
        }
        for (int q = 0; q < num_percentiles; ++q) {
            if (!(percentiles[q] > 0.0 && percentiles[q] < 1.0)) {
                fail(MGPU_INVALID_VALUE, "percentiles must lie in (0, 1)");
            }
        }
        const int runs = b->num_graphs;
        for (int i = 1; i < runs; ++i) {
            if (b->N[i] != b->N[0] || b->G[i] != b->G[0]) {
                fail(MGPU_INVALID_VALUE, "ensemble statistics need graphs of one shape");
            }
        }
        if (runs > 4096) {
            fail(MGPU_UNSUPPORTED, "ensemble statistics over at most 4096 graphs per batch");
        }
        int pow2 = 1;
        while (pow2 < runs) {
            pow2 <<= 1;
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const int64_t n_col = (int64_t)b->N[0] * b->n[0];
        cudaStream_t s      = b->ctx->stream;
        DevPool io;
        io.ctx = b->ctx;
        try {
            int64_t* d_off = io.upload(b->state_off);
            double* d_p    = io.alloc<double>(std::max(num_percentiles, 1));
            double* d_mean = io.alloc<double>(n_col);
            double* d_pct  = io.alloc<double>(std::max<int64_t>(n_col * num_percentiles, 1));
            if (num_percentiles > 0) {
                ck(cudaMemcpyAsync(d_p, percentiles, sizeof(double) * num_percentiles, cudaMemcpyHostToDevice, s),
                   "h2d");
            }
            k_ensemble_stats<<<(unsigned)n_col, 256, sizeof(double) * pow2, s>>>(b->dev, d_off, runs, pow2, n_col, d_p,
                                                                                num_percentiles, d_mean, d_pct);
            ck(cudaGetLastError(), "k_ensemble_stats");
            ck(cudaMemcpyAsync(mean, d_mean, sizeof(double) * n_col, cudaMemcpyDeviceToHost, s), "d2h");
            if (num_percentiles > 0) {
                ck(cudaMemcpyAsync(out_percentiles, d_pct, sizeof(double) * n_col * num_percentiles,
                                   cudaMemcpyDeviceToHost, s),
                   "d2h");
            }
            ck(cudaStreamSynchronize(s), "sync");
        }
        catch (...) {
            io.release();
            throw;
        }
        io.release();
        return MGPU_OK;
    });
}

int mgpu_batch_get_timing(mgpu_batch* b, mgpu_timing* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        *out = b->timing;
        return MGPU_OK;
    });
}

int mgpu_batch_reset(mgpu_batch* b, double t0)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const int64_t n = std::max<int64_t>(
            std::max<int64_t>(b->state_total, b->dev.num_nodes),
            std::max<int64_t>(b->dev.num_edges, (int64_t)b->num_graphs));
        k_reset<<<(unsigned)((n + 255) / 256), 256, 0, b->ctx->stream>>>(b->dev, b->init_state, b->init_hi,
                                                                          b->init_lo, b->state_total, t0,
                                                                          b->dt0);
        ++b->launches;
        ck(cudaGetLastError(), "k_reset");
        if (b->dev.flows) {
            ck(cudaMemsetAsync(b->dev.flows, 0, sizeof(double) * (size_t)(b->state_total / kC) * kF, b->ctx->stream),
               "memset");
        }
        for (int i = 0; i < b->num_graphs && !b->stats_host.empty(); ++i) {
            const EdgeStatsDev& S = b->stats_host[(size_t)i];
            if (S.num_sets) {
                ck(cudaMemsetAsync(S.count, 0, sizeof(int32_t) * std::max(b->host_graphs[(size_t)i].E, 1),
                                   b->ctx->stream),
                   "memset");
            }
        }
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
        b->half_step = false;
        b->t_host.assign(b->num_graphs, t0);
        b->tmax_host.assign(b->num_graphs, t0);
        return MGPU_OK;
    });
}

int mgpu_batch_get_state(mgpu_batch* b, double* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        if (b->pairs) {
            if (b->state_total > 0) {
                read_pairs(b, 0, b->state_total, out);
            }
            return MGPU_OK;
        }
        ck(cudaMemcpyAsync(out, b->dev.state, sizeof(double) * b->state_total, cudaMemcpyDeviceToHost,
                           b->ctx->stream),
           "d2h state");
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
        return MGPU_OK;
    });
}

int mgpu_batch_set_damping_cache(mgpu_batch* b, int32_t graph, int32_t node, int32_t matrix, int32_t num_points,
                                 const double* times, const double* values)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active) {
            // a cache written now would take effect at an interval boundary that
            // depends on how the advance was split into launches
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        if (!times || !values || graph < 0 || graph >= b->num_graphs) {
            fail(MGPU_INVALID_VALUE, "null array or graph index out of range");
        }
        const DevGraph& d = b->host_graphs[graph];
        if (node < 0 || node >= d.N || matrix < 0 || matrix >= d.M) {
            fail(MGPU_OUT_OF_RANGE, "node or contact matrix index out of range");
        }
        if (d.K == 0 || num_points < 2 || num_points > d.K) {
            fail(MGPU_INVALID_VALUE, "num_points must lie in [2, num_damping_points of the graph]");
        }
        if (b->damping_shared[graph]) {
            fail(MGPU_UNSUPPORTED, "the graph's damping arrays are shared with another graph of the batch");
        }
        for (int k = 1; k < num_points; ++k) {
            if (!(times[k] >= times[k - 1])) {
                fail(MGPU_INVALID_VALUE, "damping cache times must be non-decreasing");
            }
        }
        const long GG = (long)d.G * d.G;
        std::vector<double> t((size_t)d.K), v((size_t)d.K * GG);
        for (int k = 0; k < d.K; ++k) {
            const int src = std::min(k, num_points - 1);
            t[(size_t)k]  = k < num_points ? times[k] : std::numeric_limits<double>::max();
            std::memcpy(v.data() + (size_t)k * GG, values + (size_t)src * GG, sizeof(double) * GG);
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s    = b->ctx->stream;
        const int64_t row = (int64_t)node * d.M + matrix;
        double* dt        = const_cast<double*>(b->dev.dtimes) + d.dtime_off + row * d.K;
        double* dv        = const_cast<double*>(b->dev.dvals) + d.dval_off + row * d.K * GG;
        ck(cudaMemcpyAsync(dt, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, s), "h2d damping times");
        ck(cudaMemcpyAsync(dv, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, s), "h2d damping values");
        if (b->dev.dvals_f) {
            // the mixed solver's FP32 copy (rounded to nearest, as at creation)
            std::vector<float> vf(v.size());
            for (size_t i = 0; i < v.size(); ++i) {
                vf[i] = (float)v[i];
            }
            float* dvf = const_cast<float*>(b->dev.dvals_f) + d.dval_off + row * d.K * GG;
            ck(cudaMemcpyAsync(dvf, vf.data(), sizeof(float) * vf.size(), cudaMemcpyHostToDevice, s), "h2d damping values");
        }
        ck(cudaStreamSynchronize(s), "sync");
        return MGPU_OK;
    });
}

int mgpu_batch_set_edge_damping_cache(mgpu_batch* b, int32_t graph, int32_t edge, int32_t num_points,
                                      const double* times, const double* values)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        if (!times || !values || graph < 0 || graph >= b->num_graphs) {
            fail(MGPU_INVALID_VALUE, "null array or graph index out of range");
        }
        const DevGraph& d = b->host_graphs[graph];
        if (edge < 0 || edge >= d.E) {
            fail(MGPU_OUT_OF_RANGE, "edge index out of range");
        }
        if (d.Ke == 0 || num_points < 2 || num_points > d.Ke) {
            fail(MGPU_INVALID_VALUE, "num_points must lie in [2, num_edge_damping_points of the graph]");
        }
        if (b->coeff_shared[graph]) {
            fail(MGPU_UNSUPPORTED, "the graph's edge coefficient arrays are shared with another graph of the batch");
        }
        for (int k = 1; k < num_points; ++k) {
            if (!(times[k] >= times[k - 1])) {
                fail(MGPU_INVALID_VALUE, "damping cache times must be non-decreasing");
            }
        }
        const int n = d.n;
        std::vector<double> t((size_t)d.Ke), v((size_t)d.Ke * n);
        for (int k = 0; k < d.Ke; ++k) {
            const int src = std::min(k, num_points - 1);
            t[(size_t)k]  = k < num_points ? times[k] : std::numeric_limits<double>::max();
            std::memcpy(v.data() + (size_t)k * n, values + (size_t)src * n, sizeof(double) * n);
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        double* dt     = const_cast<double*>(b->dev.edt) + d.edt_off + (int64_t)edge * d.Ke;
        double* dv     = const_cast<double*>(b->dev.edv) + d.edv_off + (int64_t)edge * d.Ke * n;
        ck(cudaMemcpyAsync(dt, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, s), "h2d damping times");
        ck(cudaMemcpyAsync(dv, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice, s), "h2d damping values");
        ck(cudaStreamSynchronize(s), "sync");
        return MGPU_OK;
    });
}

int mgpu_batch_step_nodes(mgpu_batch* b, double tmax, const double* tmax_per_graph)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "interval steps need a batched precision");
        }
        if (b->half_step) {
            fail(MGPU_INVALID_VALUE, "the begun interval awaits mgpu_batch_step_exchange");
        }
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        for (int i = 0; i < b->num_graphs; ++i) {
            b->tmax_host[i] = tmax_per_graph ? tmax_per_graph[i] : tmax;
        }
        ck(cudaMemcpyAsync(b->d_tmax, b->tmax_host.data(), sizeof(double) * b->num_graphs, cudaMemcpyHostToDevice,
                           s),
           "h2d tmax");
        // the interval's end per graph (k_phase_begin)
        b->half_t_next = b->t_host;
        for (int i = 0; i < b->num_graphs; ++i) {
            const double t = b->t_host[i];
            if (t < b->tmax_host[i]) {
                b->half_t_next[i] = t + std::min(b->opts.dt_exchange, b->tmax_host[i] - t);
            }
        }
        const BatchDev& B = b->dev;
        k_set_tmax<<<(b->num_graphs + 127) / 128, 128, 0, s>>>(B.rt, b->d_tmax, b->num_graphs);
        launch_phase_begin(B, b->opts.dt_exchange, s);
        for (auto& kv : b->inst_by_G) {
            auto it       = b->tuned.find(kv.first);
            const int ipb = it != b->tuned.end() ? it->second.first : b->instances_per_block;
            const int grd = it != b->tuned.end() ? it->second.second : 0;
            launch_ode_batched(B, kv.first, b->opts.precision, kv.second.first, kv.second.second, ipb, grd, s);
        }
        ck(cudaGetLastError(), "step launch");
        b->launches += 2 + node_kernel_launches(b);
        b->half_step = true;
        return check_device_error(b);
    });
}

int mgpu_batch_step_exchange(mgpu_batch* b)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!b->half_step) {
            fail(MGPU_INVALID_VALUE, "no interval begun by mgpu_batch_step_nodes");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s    = b->ctx->stream;
        const BatchDev& B = b->dev;
        int64_t l         = 0;
        launch_exchange_batched(B, b->opts.precision, b->n_max, b->any_edge_dampings, s, &l, nullptr);
        launch_phase_end(B, s);
        ck(cudaGetLastError(), "step launch");
        b->launches += l + 1;
        b->phases += 1;
        b->half_step = false;
        b->t_host    = b->half_t_next;
        return check_device_error(b);
    });
}

int mgpu_batch_set_state(mgpu_batch* b, const double* state)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!state) {
            fail(MGPU_INVALID_VALUE, "null input");
        }
        if (b->half_step || b->async_active) {
            // the departure snapshots of a begun interval come from the states its solves left
            fail(MGPU_INVALID_VALUE, "states can be replaced only between whole intervals");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        if (b->pairs) {
            std::vector<float> hi(b->state_total), lo(b->state_total);
            split_pairs(state, b->state_total, hi.data(), lo.data());
            ck(cudaMemcpyAsync(b->dev.st_hi, hi.data(), sizeof(float) * b->state_total, cudaMemcpyHostToDevice,
                               b->ctx->stream),
               "h2d state");
            ck(cudaMemcpyAsync(b->dev.st_lo, lo.data(), sizeof(float) * b->state_total, cudaMemcpyHostToDevice,
                               b->ctx->stream),
               "h2d state");
            ck(cudaStreamSynchronize(b->ctx->stream), "sync");
            return MGPU_OK;
        }
        ck(cudaMemcpyAsync(b->dev.state, state, sizeof(double) * b->state_total, cudaMemcpyHostToDevice,
                           b->ctx->stream),
           "h2d state");
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
        return MGPU_OK;
    });
}

__global__ void k_compartment_sums(BatchDev B, int c, double* out)
{
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= B.num_nodes) {
        return;
    }
    const DevGraph& g  = B.graphs[B.node_graph[v]];
    const int64_t base = g.state_off + (v - g.node0) * (int64_t)g.G * kC + c;
    double s           = 0.0;
    for (int gr = 0; gr < g.G; ++gr) {
        s += state_get(B, base + (int64_t)gr * kC);
    }
    out[v] = s;
}

int mgpu_batch_get_compartment_sums(mgpu_batch* b, int32_t compartment, double* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out || compartment < 0 || compartment >= kC) {
            fail(MGPU_INVALID_VALUE, "null output or compartment out of range");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s   = b->ctx->stream;
        const int64_t nn = b->dev.num_nodes;
        if (nn == 0) {
            return MGPU_OK;
        }
        if (!b->d_sums) {
            b->d_sums = b->pool.alloc<double>(nn);
        }
        k_compartment_sums<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(b->dev, compartment, b->d_sums);
        ck(cudaGetLastError(), "k_compartment_sums");
        ck(cudaMemcpyAsync(out, b->d_sums, sizeof(double) * nn, cudaMemcpyDeviceToHost, s), "d2h sums");
        ck(cudaStreamSynchronize(s), "sync");
        ++b->launches;
        return MGPU_OK;
    });
}

int mgpu_batch_get_time(mgpu_batch* b, double* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        std::copy(b->t_host.begin(), b->t_host.end(), out);
        return MGPU_OK;
    });
}

int mgpu_batch_get_stats(mgpu_batch* b, mgpu_stats* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        unsigned long long c[CNT_NUM];
        ck(cudaMemcpyAsync(c, b->dev.counters, sizeof(c), cudaMemcpyDeviceToHost, b->ctx->stream), "d2h");
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
        out->accepted_steps       = (int64_t)c[CNT_ACCEPTED];
        out->rejected_steps       = (int64_t)c[CNT_REJECTED];
        out->failed_steps         = (int64_t)c[CNT_FAILED];
        out->underflow_fixes      = (int64_t)c[CNT_UNDERFLOW];
        out->sequential_exchanges = (int64_t)c[CNT_SEQUENTIAL];
        out->scan_items           = (int64_t)c[CNT_SCANNED];
        out->phases               = b->phases;
        out->kernel_launches      = b->launches;
        return MGPU_OK;
    });
}

int mgpu_batch_set_commuter_stats(mgpu_batch* b, int32_t graph, int32_t num_sets, const int32_t* set_offsets,
                                  const int32_t* set_indices, int32_t capacity)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active || b->half_step) {
            fail(MGPU_INVALID_VALUE, "an advance is in progress");
        }
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "commuter statistics need a batched precision");
        }
        if (graph < 0 || graph >= b->num_graphs) {
            fail(MGPU_OUT_OF_RANGE, "graph index out of range");
        }
        if (num_sets < 0 || (num_sets > 0 && (!set_offsets || !set_indices || capacity < 1))) {
            fail(MGPU_INVALID_VALUE, "index sets (offsets, indices) and capacity >= 1 needed");
        }
        const DevGraph& d = b->host_graphs[(size_t)graph];
        if (num_sets > 0) {
            if (set_offsets[0] != 0) {
                fail(MGPU_INVALID_VALUE, "set_offsets[0] must be 0");
            }
            for (int i = 0; i < num_sets; ++i) {
                if (set_offsets[i + 1] < set_offsets[i]) {
                    fail(MGPU_INVALID_VALUE, "set_offsets must be non-decreasing");
                }
            }
            for (int q = 0; q < set_offsets[num_sets]; ++q) {
                if (set_indices[q] < 0 || set_indices[q] >= d.n) {
                    fail(MGPU_OUT_OF_RANGE, "compartment index outside [0, 10 G)");
                }
            }
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        if (b->stats_host.empty()) {
            b->stats_host.assign((size_t)b->num_graphs, EdgeStatsDev{});
        }
        // the buffers of every graph that keeps recording are laid out again (the
        // pool frees all at once); recorded points of the other graphs are kept
        std::vector<EdgeStatsDev> old = b->stats_host;
        DevPool fresh;
        fresh.ctx = b->ctx;
        std::vector<EdgeStatsDev> next((size_t)b->num_graphs, EdgeStatsDev{});
        for (int i = 0; i < b->num_graphs; ++i) {
            const bool is_new = i == graph;
            const int32_t S   = is_new ? num_sets : old[(size_t)i].num_sets;
            if (S == 0) {
                continue;
            }
            const int64_t E   = std::max(b->host_graphs[(size_t)i].E, 1);
            const int32_t cap = is_new ? capacity : old[(size_t)i].capacity;
            EdgeStatsDev& x   = next[(size_t)i];
            x.num_sets        = S;
            x.capacity        = cap;
            int32_t* sp       = fresh.alloc<int32_t>(S + 1);
            const int64_t ni  = is_new ? set_offsets[S] : 0;
            int32_t* si       = fresh.alloc<int32_t>(is_new ? ni : 1);
            x.count           = fresh.alloc<int32_t>(E);
            x.times           = fresh.alloc<double>(E * cap);
            x.values          = fresh.alloc<double>(E * cap * (S + 1));
            if (is_new) {
                ck(cudaMemcpyAsync(sp, set_offsets, sizeof(int32_t) * (S + 1), cudaMemcpyHostToDevice, s), "h2d");
                if (ni > 0) {
                    ck(cudaMemcpyAsync(si, set_indices, sizeof(int32_t) * ni, cudaMemcpyHostToDevice, s), "h2d");
                }
                ck(cudaMemsetAsync(x.count, 0, sizeof(int32_t) * E, s), "memset");
                x.set_ptr = sp;
                x.set_idx = si;
            }
            else {
                // carry the other graphs' sets and recorded points over
                const EdgeStatsDev& o = old[(size_t)i];
                int32_t np = 0;
                ck(cudaMemcpyAsync(&np, o.set_ptr + S, sizeof(int32_t), cudaMemcpyDeviceToHost, s), "d2h");
                ck(cudaStreamSynchronize(s), "sync");
                int32_t* si2 = fresh.alloc<int32_t>(std::max(np, 1));
                ck(cudaMemcpyAsync(sp, o.set_ptr, sizeof(int32_t) * (S + 1), cudaMemcpyDeviceToDevice, s), "d2d");
                ck(cudaMemcpyAsync(si2, o.set_idx, sizeof(int32_t) * np, cudaMemcpyDeviceToDevice, s), "d2d");
                ck(cudaMemcpyAsync(x.count, o.count, sizeof(int32_t) * E, cudaMemcpyDeviceToDevice, s), "d2d");
                ck(cudaMemcpyAsync(x.times, o.times, sizeof(double) * E * cap, cudaMemcpyDeviceToDevice, s), "d2d");
                ck(cudaMemcpyAsync(x.values, o.values, sizeof(double) * E * cap * (S + 1), cudaMemcpyDeviceToDevice,
                                   s),
                   "d2d");
                x.set_ptr = sp;
                x.set_idx = si2;
            }
        }
        bool any = false;
        for (const auto& x : next) {
            any = any || x.num_sets > 0;
        }
        EdgeStatsDev* table = any ? fresh.upload(next) : nullptr;
        ck(cudaStreamSynchronize(s), "sync");
        b->stats_pool.release();
        b->stats_pool = fresh;
        b->stats_host = next;
        b->dev.estats = table;
        b->drop_graph();
        return MGPU_OK;
    });
}

int mgpu_batch_get_commuter_stats(mgpu_batch* b, int32_t graph, int32_t* counts, double* times, double* values)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        if (graph < 0 || graph >= b->num_graphs) {
            fail(MGPU_OUT_OF_RANGE, "graph index out of range");
        }
        if (b->stats_host.empty() || b->stats_host[(size_t)graph].num_sets == 0) {
            fail(MGPU_INVALID_VALUE, "the graph records no commuter statistics");
        }
        if (!counts) {
            fail(MGPU_INVALID_VALUE, "null counts");
        }
        const EdgeStatsDev& x = b->stats_host[(size_t)graph];
        const int64_t E       = b->host_graphs[(size_t)graph].E;
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        cudaStream_t s = b->ctx->stream;
        if (E > 0) {
            ck(cudaMemcpyAsync(counts, x.count, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s), "d2h");
            if (times) {
                ck(cudaMemcpyAsync(times, x.times, sizeof(double) * E * x.capacity, cudaMemcpyDeviceToHost, s), "d2h");
            }
            if (values) {
                ck(cudaMemcpyAsync(values, x.values, sizeof(double) * E * x.capacity * (x.num_sets + 1),
                                   cudaMemcpyDeviceToHost, s),
                   "d2h");
            }
        }
        ck(cudaStreamSynchronize(s), "sync");
        // the slots after an edge's recorded points read as zero
        const int64_t w = x.num_sets + 1;
        for (int64_t e = 0; e < E; ++e) {
            const int64_t k = std::min<int64_t>(std::max(counts[e], 0), x.capacity);
            if (times) {
                std::fill(times + e * x.capacity + k, times + (e + 1) * x.capacity, 0.0);
            }
            if (values) {
                std::fill(values + (e * x.capacity + k) * w, values + (e + 1) * x.capacity * w, 0.0);
            }
        }
        for (int64_t e = 0; e < E; ++e) {
            if (counts[e] > x.capacity) {
                fail(MGPU_OUT_OF_RANGE, "an edge recorded more time points than the capacity (" +
                                            std::to_string(counts[e]) + " > " + std::to_string(x.capacity) +
                                            "); the first capacity points were kept");
            }
        }
        return MGPU_OK;
    });
}

int mgpu_batch_set_flow_recording(mgpu_batch* b, int32_t on)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (b->async_active || b->half_step) {
            fail(MGPU_INVALID_VALUE, "an advance is in progress");
        }
        if (b->opts.precision == MGPU_PRECISION_FP64_PLAIN) {
            fail(MGPU_UNSUPPORTED, "flow recording needs a batched precision");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const size_t count = (size_t)(b->state_total / kC) * kF;
        if (on && !b->dev.flows) {
            if (!b->flows_buf) {
                b->flows_buf = b->pool.alloc<double>((int64_t)count);
            }
            ck(cudaMemsetAsync(b->flows_buf, 0, sizeof(double) * std::max<size_t>(count, 1), b->ctx->stream),
               "memset");
            ck(cudaStreamSynchronize(b->ctx->stream), "sync");
            b->dev.flows = b->flows_buf;
            b->drop_graph();
        }
        else if (!on && b->dev.flows) {
            b->dev.flows = nullptr;
            b->drop_graph();
        }
        return MGPU_OK;
    });
}

int mgpu_batch_get_flows(mgpu_batch* b, double* out)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!out) {
            fail(MGPU_INVALID_VALUE, "null output");
        }
        if (b->async_active) {
            fail(MGPU_INVALID_VALUE, "an asynchronous advance is in progress");
        }
        if (!b->dev.flows) {
            fail(MGPU_INVALID_VALUE, "flow recording is off (mgpu_batch_set_flow_recording)");
        }
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const size_t count = (size_t)(b->state_total / kC) * kF;
        if (count > 0) {
            ck(cudaMemcpyAsync(out, b->dev.flows, sizeof(double) * count, cudaMemcpyDeviceToHost, b->ctx->stream),
               "d2h flows");
        }
        ck(cudaStreamSynchronize(b->ctx->stream), "sync");
        return MGPU_OK;
    });
}

int mgpu_batch_get_failed(mgpu_batch* b, int32_t* flags, int32_t* num_failed)
{
    if (!b) {
        return MGPU_INVALID_VALUE;
    }
    return guarded(b->ctx, [&]() -> int {
        if (!flags && !num_failed) {
            fail(MGPU_INVALID_VALUE, "null outputs");
        }
        // (read-only: during an asynchronous advance, after the launched intervals)
        ck(cudaSetDevice(b->ctx->device), "cudaSetDevice");
        const std::vector<int32_t> f = read_graph_errors(b);
        int32_t n = 0;
        for (int i = 0; i < b->num_graphs; ++i) {
            const int32_t bits = (f[(size_t)i] & ERR_STEP_CAP ? MGPU_FAILED_STEP_CAP : 0) |
                                 (f[(size_t)i] & ERR_NONFINITE ? MGPU_FAILED_NONFINITE : 0);
            if (flags) {
                flags[i] = bits;
            }
            n += bits ? 1 : 0;
        }
        if (num_failed) {
            *num_failed = n;
        }
        return MGPU_OK;
    });
}

int64_t mgpu_batch_device_bytes(const mgpu_batch* b)
{
    return b ? b->pool.bytes : 0;
}

void mgpu_batch_destroy(mgpu_batch* b)
{
    {
        std::lock_guard<std::mutex> lock(g_batches_mutex);
        if (!b || g_batches.erase(b) == 0) {
            return; // not a live batch: destroyed already or released with its context
        }
    }
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    delete b;
}

} // extern "C"
