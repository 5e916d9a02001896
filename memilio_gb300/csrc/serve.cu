// serve.cu — a device-resident request loop over the batched solver
// (mgpu_server_*, include/miogpu.h).
//
// Requests (one graph, a start and a horizon each) queue on the host. Every
// scheduling round admits the queued requests whose device memory fits the
// budget as a new batch on its own stream (a context per batch), so batches
// admitted at different times run concurrently on the device; every running
// batch gets its next exchange intervals enqueued without waiting; a request
// completes as soon as the intervals up to its own horizon have finished,
// and a batch releases its memory when its last request has completed. Node
// states stay on the device between intervals.
//
// Built on the public C ABI only; the host loop never blocks on the device
// except for the copy of a completed request's states.
#include "../../include/miogpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <memory>
#include <new>
#include <string>
#include <vector>

namespace
{

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int64_t id       = 0;
    mgpu_graph graph = {};
    double t0 = 0.0, tmax = 0.0;
    int64_t bytes    = 0; // estimate when queued alone
    int64_t phases   = 0; // exchange intervals to its horizon
    double t_submit  = 0.0;
};

struct Done {
    int64_t id = 0;
    std::vector<double> state;
    int status      = MGPU_OK;
    double latency_s = 0.0;
};

struct Running {
    mgpu_context* ctx = nullptr;
    mgpu_batch* batch = nullptr;
    std::vector<Request> reqs;
    std::vector<char> delivered;
    std::vector<int64_t> base; // intervals each request had completed before it joined this batch
    int64_t bytes     = 0;
    int64_t launched  = 0; // intervals enqueued so far
    int64_t finished  = 0; // intervals known to have finished
    int32_t remaining = 0;
    bool in_flight    = false;
    bool started      = false; // the batch's advance has been launched (its horizons are set)
};

} // namespace

struct mgpu_server {
    int device = 0;
    mgpu_server_opts opts{};
    int64_t budget = 0, in_use = 0;
    int64_t next_id = 1;
    std::deque<Request> queue;
    std::vector<Running> running;
    std::deque<Done> done;
    std::vector<mgpu_context*> idle_ctx;
    int64_t completed_total = 0;
    int64_t merges          = 0; // re-batching merges so far
};

namespace
{

int64_t phases_to(double t0, double tmax, double dt)
{
    int64_t p = 0;
    double t  = t0;
    while (t < tmax) {
        double d = dt;
        if (t + d > tmax) {
            d = tmax - t;
        }
        t += d;
        ++p;
    }
    return p;
}

mgpu_context* take_ctx(mgpu_server* s)
{
    if (!s->idle_ctx.empty()) {
        mgpu_context* c = s->idle_ctx.back();
        s->idle_ctx.pop_back();
        return c;
    }
    mgpu_context* c = nullptr;
    return mgpu_create(s->device, &c) == MGPU_OK ? c : nullptr;
}

// Completes the requests of r whose horizon lies within the finished intervals.
// Each request gets its own status: a request whose node solves failed (step cap,
// non-finite state) is reported as MGPU_STEP_FAILED, and the other requests of
// its batch complete normally; any other batch status fails every request.
int deliver(mgpu_server* s, Running& r, bool all_done, int32_t batch_status)
{
    int n = 0;
    std::vector<int32_t> failed;
    for (size_t i = 0; i < r.reqs.size(); ++i) {
        if (r.delivered[i] || (!all_done && r.reqs[i].phases > r.base[i] + r.finished)) {
            continue;
        }
        Done d;
        d.id        = r.reqs[i].id;
        d.status    = batch_status == MGPU_STEP_FAILED ? MGPU_OK : batch_status;
        const int64_t cnt = (int64_t)r.reqs[i].graph.num_nodes * 10 * r.reqs[i].graph.num_groups;
        d.state.resize((size_t)cnt);
        if (d.status == MGPU_OK && failed.empty()) {
            failed.assign(r.reqs.size(), 0);
            d.status = mgpu_batch_get_failed(r.batch, failed.data(), nullptr);
        }
        if (d.status == MGPU_OK && failed[i]) {
            d.status = MGPU_STEP_FAILED;
        }
        if (d.status == MGPU_OK) {
            d.status = mgpu_batch_get_graph_state(r.batch, (int32_t)i, d.state.data());
        }
        d.latency_s    = now_s() - r.reqs[i].t_submit;
        r.delivered[i] = 1;
        s->done.push_back(std::move(d));
        ++n;
    }
    return n;
}

// Merges the running batches that are between intervals (not in flight, not
// finished) and hold at most rebatch_max_graphs unfinished requests into one
// new batch (mgpu_batch_regroup). Batches whose graphs have travelers away, or
// a merge that would not fit the memory budget, are left as they are.
void rebatch(mgpu_server* s)
{
    // only when the batch limit holds back admission: a merge rebuilds the
    // merged graphs' batch on the host, which costs more than the launches it
    // saves while there is room for more batches
    if ((int32_t)s->running.size() < s->opts.max_batches || s->queue.empty()) {
        return;
    }
    std::vector<size_t> cand;
    int64_t graphs = 0;
    for (size_t k = 0; k < s->running.size(); ++k) {
        const Running& r = s->running[k];
        int64_t open     = 0;
        for (char d : r.delivered) {
            open += d ? 0 : 1;
        }
        if (!r.in_flight && r.started && open > 0 && open <= s->opts.rebatch_max_graphs &&
            graphs + open <= s->opts.max_graphs_per_batch) {
            cand.push_back(k);
            graphs += open;
        }
    }
    if (cand.size() < 2) {
        return;
    }
    Running m;
    std::vector<mgpu_graph> gs;
    std::vector<mgpu_batch*> src;
    std::vector<int32_t> src_graph;
    for (size_t k : cand) {
        const Running& r = s->running[k];
        for (size_t i = 0; i < r.reqs.size(); ++i) {
            if (r.delivered[i]) {
                continue;
            }
            m.reqs.push_back(r.reqs[i]);
            m.base.push_back(r.base[i] + r.finished);
            gs.push_back(r.reqs[i].graph);
            src.push_back(r.batch);
            src_graph.push_back((int32_t)i);
        }
    }
    const int64_t est = mgpu_batch_estimate_bytes(gs.data(), (int32_t)gs.size(), &s->opts.solver);
    if (est < 0 || s->in_use + est > s->budget) {
        return;
    }
    m.ctx = take_ctx(s);
    if (!m.ctx) {
        return;
    }
    if (mgpu_batch_regroup(m.ctx, gs.data(), (int32_t)gs.size(), src.data(), src_graph.data(), &m.batch) != MGPU_OK) {
        s->idle_ctx.push_back(m.ctx); // e.g. travelers away: try again at a later step
        return;
    }
    m.delivered.assign(m.reqs.size(), 0);
    m.bytes = std::max<int64_t>(est, mgpu_batch_device_bytes(m.batch));
    for (auto it = cand.rbegin(); it != cand.rend(); ++it) {
        Running& r = s->running[*it];
        mgpu_batch_destroy(r.batch);
        s->idle_ctx.push_back(r.ctx);
        s->in_use -= r.bytes;
        s->running.erase(s->running.begin() + (long)*it);
    }
    s->in_use += m.bytes;
    ++s->merges;
    s->running.push_back(std::move(m));
}

} // namespace

extern "C" {

void mgpu_default_server_opts(mgpu_server_opts* o)
{
    if (!o) {
        return;
    }
    mgpu_default_solver_opts(&o->solver);
    o->solver.precision    = MGPU_PRECISION_MIXED;
    o->memory_budget       = 0;
    o->max_batches         = 16;
    o->phases_per_launch   = 2;
    o->max_graphs_per_batch = 4096;
    o->min_batch_graphs     = 1; // admit at once (measured: waiting to batch did not raise throughput)
    o->max_wait_ms          = 0.0;
    o->rebatch_max_graphs   = 0; // off: measured slower on the uneven request stream (a merge rebuilds on the host)
    o->pad                  = 0;
}

int mgpu_server_create(int device, const mgpu_server_opts* opts, mgpu_server** out)
{
    if (!out) {
        return MGPU_INVALID_VALUE;
    }
    *out = nullptr;
    mgpu_server_opts o;
    if (opts) {
        o = *opts;
    }
    else {
        mgpu_default_server_opts(&o);
    }
    if (o.solver.precision == MGPU_PRECISION_FP64_PLAIN) {
        return MGPU_UNSUPPORTED;
    }
    if (o.max_batches < 1 || o.phases_per_launch < 1 || o.max_graphs_per_batch < 1 || o.memory_budget < 0 ||
        o.min_batch_graphs < 1 || !(o.max_wait_ms >= 0.0) || o.rebatch_max_graphs < 0) {
        return MGPU_INVALID_VALUE;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    auto* s   = new (std::nothrow) mgpu_server();
    if (!s) {
        return MGPU_OOM;
    }
    s->device = device;
    s->opts   = o;
    s->budget = o.memory_budget > 0 ? std::min<int64_t>(o.memory_budget, (int64_t)free_b)
                                    : (int64_t)(0.9 * (double)free_b);
    *out      = s;
    return MGPU_OK;
}

void mgpu_server_destroy(mgpu_server* s)
{
    if (!s) {
        return;
    }
    for (auto& r : s->running) {
        mgpu_batch_destroy(r.batch); // waits for its stream
        mgpu_destroy(r.ctx);
    }
    for (auto* c : s->idle_ctx) {
        mgpu_destroy(c);
    }
    delete s;
}

int mgpu_server_submit(mgpu_server* s, const mgpu_graph* graph, double t0, double tmax, int64_t* request_id)
{
    if (!s || !graph || !request_id || !(tmax >= t0)) {
        return MGPU_INVALID_VALUE;
    }
    Request r;
    r.graph  = *graph;
    r.t0     = t0;
    r.tmax   = tmax;
    r.bytes  = mgpu_batch_estimate_bytes(graph, 1, &s->opts.solver);
    if (r.bytes < 0) {
        return MGPU_INVALID_VALUE;
    }
    if (r.bytes > s->budget) {
        return MGPU_OOM;
    }
    r.phases   = phases_to(t0, tmax, s->opts.solver.dt_exchange);
    r.id       = s->next_id++;
    r.t_submit = now_s();
    s->queue.push_back(r);
    *request_id = r.id;
    return MGPU_OK;
}

int mgpu_server_step(mgpu_server* s, int32_t* completed, int32_t* running, int32_t* queued)
{
    if (!s) {
        return MGPU_INVALID_VALUE;
    }
    if (cudaSetDevice(s->device) != cudaSuccess) {
        return MGPU_CUDA_ERROR;
    }
    int n_completed = 0;
    // 1. progress of the running batches: deliver what their finished intervals completed
    for (size_t k = 0; k < s->running.size();) {
        Running& r = s->running[k];
        if (r.in_flight) {
            int32_t done   = 0;
            const int32_t st = mgpu_batch_query(r.batch, &done);
            if (st == MGPU_OK && !done) {
                ++k;
                continue;
            }
            r.in_flight             = false;
            r.finished              = r.launched;
            const bool finished_all = st != MGPU_OK || r.remaining == 0;
            n_completed += deliver(s, r, finished_all, st);
            if (finished_all) {
                mgpu_batch_destroy(r.batch);
                s->idle_ctx.push_back(r.ctx);
                s->in_use -= r.bytes;
                s->running.erase(s->running.begin() + (long)k);
                continue;
            }
        }
        ++k;
    }
    // 1b. re-batching: small batches that stand between intervals with no
    // travelers away merge into one, so that their next intervals run as one
    // launch sequence (every graph goes on exactly as before)
    if (s->opts.rebatch_max_graphs > 0) {
        rebatch(s);
    }
    // 1c. the next intervals of every running batch that is not in flight
    for (size_t k = 0; k < s->running.size();) {
        Running& r = s->running[k];
        if (r.in_flight) {
            ++k;
            continue;
        }
        int32_t rem = 0;
        int32_t st  = MGPU_OK;
        if (!r.started) {
            // a merged batch: its requests' horizons, from where each stands
            std::vector<double> tmax(r.reqs.size());
            int64_t total = 0;
            for (size_t i = 0; i < r.reqs.size(); ++i) {
                tmax[i] = r.reqs[i].tmax;
                total   = std::max<int64_t>(total, r.reqs[i].phases - r.base[i]);
            }
            st = mgpu_batch_launch(r.batch, 0.0, tmax.data(), s->opts.phases_per_launch, &rem);
            if (st == MGPU_OK) {
                r.started   = true;
                r.launched  = total - rem;
                r.remaining = rem;
            }
        }
        else {
            st = mgpu_batch_launch(r.batch, 0.0, nullptr, s->opts.phases_per_launch, &rem);
            if (st == MGPU_OK) {
                r.launched += r.remaining - rem;
                r.remaining = rem;
            }
        }
        if (st == MGPU_OK) {
            r.in_flight = true;
            ++k;
            continue;
        }
        n_completed += deliver(s, r, true, st);
        mgpu_batch_destroy(r.batch);
        s->idle_ctx.push_back(r.ctx);
        s->in_use -= r.bytes;
        s->running.erase(s->running.begin() + (long)k);
    }
    // 2. admission: the queued requests that fit, as one new batch per start time.
    // While batches run, requests wait until enough of them queue up or the
    // oldest has waited max_wait_ms, so that batches are large enough to fill
    // the device (one small batch per arrival would leave it launch-bound).
    const bool busy  = !s->running.empty();
    const bool ready = !s->queue.empty() &&
                       (!busy || (int32_t)s->queue.size() >= s->opts.min_batch_graphs ||
                        (now_s() - s->queue.front().t_submit) * 1e3 >= s->opts.max_wait_ms);
    while (ready && !s->queue.empty() && (int32_t)s->running.size() < s->opts.max_batches) {
        const double t0 = s->queue.front().t0;
        std::vector<Request> take;
        std::vector<mgpu_graph> graphs;
        int64_t est = 0;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int32_t)take.size() < s->opts.max_graphs_per_batch;) {
            if (it->t0 != t0) {
                ++it;
                continue;
            }
            graphs.push_back(it->graph);
            const int64_t e = mgpu_batch_estimate_bytes(graphs.data(), (int32_t)graphs.size(), &s->opts.solver);
            if (s->in_use + e > s->budget) {
                graphs.pop_back();
                break;
            }
            est = e;
            take.push_back(*it);
            it = s->queue.erase(it);
        }
        if (take.empty()) {
            break; // the next request waits for memory to free up
        }
        Running r;
        r.ctx = take_ctx(s);
        int st = r.ctx ? mgpu_batch_create(r.ctx, graphs.data(), (int32_t)graphs.size(), t0, &s->opts.solver, &r.batch)
                       : MGPU_CUDA_ERROR;
        if (st == MGPU_OOM) {
            // the estimate was short: put the requests back and wait
            if (r.ctx) {
                s->idle_ctx.push_back(r.ctx);
            }
            for (auto it = take.rbegin(); it != take.rend(); ++it) {
                s->queue.push_front(*it);
            }
            break;
        }
        if (st != MGPU_OK) {
            for (auto& q : take) {
                Done d;
                d.id        = q.id;
                d.status    = st;
                d.latency_s = now_s() - q.t_submit;
                s->done.push_back(std::move(d));
                ++n_completed;
            }
            if (r.ctx) {
                s->idle_ctx.push_back(r.ctx);
            }
            continue;
        }
        r.bytes = std::max<int64_t>(est, mgpu_batch_device_bytes(r.batch));
        std::vector<double> tmax(take.size());
        for (size_t i = 0; i < take.size(); ++i) {
            tmax[i] = take[i].tmax;
        }
        int32_t rem = 0;
        int32_t total = 0;
        for (auto& q : take) {
            total = (int32_t)std::max<int64_t>(total, q.phases);
        }
        st = mgpu_batch_launch(r.batch, 0.0, tmax.data(), s->opts.phases_per_launch, &rem);
        r.reqs      = std::move(take);
        r.delivered.assign(r.reqs.size(), 0);
        r.base.assign(r.reqs.size(), 0);
        r.remaining = rem;
        r.launched  = total - rem;
        r.in_flight = st == MGPU_OK;
        r.started   = true;
        s->in_use += r.bytes;
        if (st != MGPU_OK) {
            n_completed += deliver(s, r, true, st);
            mgpu_batch_destroy(r.batch);
            s->idle_ctx.push_back(r.ctx);
            s->in_use -= r.bytes;
            continue;
        }
        s->running.push_back(std::move(r));
    }
    s->completed_total += n_completed;
    if (completed) {
        *completed = n_completed;
    }
    if (running) {
        int32_t nr = 0;
        for (auto& r : s->running) {
            for (char d : r.delivered) {
                nr += d ? 0 : 1;
            }
        }
        *running = nr;
    }
    if (queued) {
        *queued = (int32_t)s->queue.size();
    }
    return MGPU_OK;
}

int mgpu_server_take(mgpu_server* s, int64_t* request_id, double* final_state, int64_t capacity, int64_t* count,
                     double* latency_s)
{
    if (!s || !request_id || !count) {
        return MGPU_INVALID_VALUE;
    }
    if (s->done.empty()) {
        *request_id = 0;
        *count      = 0;
        return MGPU_OK;
    }
    Done& d     = s->done.front();
    *count      = (int64_t)d.state.size();
    *request_id = d.id;
    if (latency_s) {
        *latency_s = d.latency_s;
    }
    if (!final_state) {
        return MGPU_OK; // peek: the request stays ready
    }
    if (capacity < (int64_t)d.state.size()) {
        return MGPU_OUT_OF_RANGE;
    }
    std::copy(d.state.begin(), d.state.end(), final_state);
    const int st = d.status;
    s->done.pop_front();
    return st;
}

int64_t mgpu_server_memory_in_use(const mgpu_server* s)
{
    return s ? s->in_use : -1;
}

int32_t mgpu_server_num_batches(const mgpu_server* s)
{
    return s ? (int32_t)s->running.size() : -1;
}

int64_t mgpu_server_num_merges(const mgpu_server* s)
{
    return s ? s->merges : -1;
}

} // extern "C"
