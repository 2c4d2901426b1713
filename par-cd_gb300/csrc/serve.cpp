// Serving loop over the batched path (pcd_serve_* in pcd.h).
//
// Requests (a graph plus the driver schedule of src/main.cpp:187-266) wait in
// one FIFO queue.  Each worker thread owns a context (its own stream) and,
// whenever it is free, forms the next batch from the queue: the oldest
// request's schedule decides which requests can share the batch (one rule and
// schedule per pcd_batch_run), then requests of that schedule are taken in
// arrival order up to the graph and edge caps and while the HBM budget -- the
// device memory every batch in flight may hold together, counted with
// pcd_estimate_device_bytes -- has room.  A batch smaller than the cap starts
// once its oldest request has waited max_wait_ms.  Batches of different
// workers run concurrently on their own streams, so a batch that finishes
// early makes room for the next one while others still run (continuous
// batching at batch granularity).  A graph gets exactly the result it gets
// alone (the batched path is exact per graph), whatever it was batched with.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "pcd.h"
#include "pcd_internal.h"

namespace pcd {
pcd_status keep_pool_memory(int32_t device, int64_t bytes);  // api.cu
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0, Clock::time_point t1) {
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

struct Request {
    uint64_t id = 0;
    int32_t n = 0, m = 0, max_deg = 0;
    int64_t hubs = 0;
    std::vector<int32_t> indices, adj;
    pcd_schedule sched{};
    Clock::time_point t_submit, t_start, t_done;
    bool done = false;
    pcd_status status = PCD_OK;
    std::vector<int32_t> labels;
    double score = 0.0;
    int32_t iterations = 0;
    int64_t batch_graphs = 0;
    int32_t cls = 0;  // size class: 0 small, 1 medium, 2 large (runs alone)
    pcd_rand seeds{};  // the reference driver's rand() stream after the singleton partition's n draws
};

// A graph's place in a continuously running batch: its own iteration count,
// previous score and seed stream, and its labels across batch rebuilds.
struct Slot {
    std::shared_ptr<Request> r;
    int32_t it = 0;
    double prev = 0.0;
    bool fresh = true;   // still at its singleton start
    bool gone = false;   // returned; still in the device batch until the next rebuild
    std::vector<int32_t> labels;
};

bool same_schedule(const pcd_schedule &a, const pcd_schedule &b) {
    return a.rule.kind == b.rule.kind && a.rule.lambda == b.rule.lambda && a.strategy == b.strategy &&
           a.frac == b.frac && a.rounds == b.rounds && a.n_iter == b.n_iter && a.threshold == b.threshold;
}

}  // namespace

struct pcd_server {
    pcd_serve_config cfg{};
    int32_t num_sms = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> tickets;
    std::vector<std::thread> workers;
    bool stopping = false;
    uint64_t next_id = 1;
    int64_t in_flight = 0;
    int32_t big_in_flight = 0;  // batches of medium or large graphs running
    pcd_serve_stats stats{};
    pcd_status start_status = PCD_OK;
    int32_t started = 0;

    int64_t estimate(const std::vector<std::shared_ptr<Request>> &rs) const {
        int64_t n = 0, nnz = 0, hubs = 0;
        int32_t md = 0;
        for (const auto &r : rs) {
            n += r->n;
            nnz += 2ll * r->m;
            hubs += r->hubs;
            md = std::max(md, r->max_deg);
        }
        const pcd_schedule &s = rs.front()->sched;
        int64_t b = 0;
        if (n > INT32_MAX) return INT64_MAX;
        pcd_estimate_device_bytes((int32_t)n, nnz, md, hubs, (int32_t)rs.size(),
                                  s.n_iter >= 0 ? std::max(s.n_iter, 1) : 1000, s.strategy != 0, num_sms, &b);
        return b;
    }

    void worker_main();
    bool take_batch(std::vector<std::shared_ptr<Request>> &batch, int64_t &bytes);
    void run_batch(pcd_ctx *ctx, std::vector<std::shared_ptr<Request>> &batch, int64_t bytes);
    void run_continuous(pcd_ctx *ctx, std::vector<std::shared_ptr<Request>> &batch, int64_t bytes);
    // requests of `like`'s schedule and size class that fit beside `held`
    // (caps, HBM budget, with `others` bytes held by the other batches);
    // removed from the queue.  Caller holds `mu`.
    std::vector<std::shared_ptr<Request>> admit(const std::vector<std::shared_ptr<Request>> &held,
                                                const Request &like, int64_t others);
    void finish(Request &r, pcd_status st, Clock::time_point t_done, int64_t batch_graphs);
};

std::vector<std::shared_ptr<Request>> pcd_server::admit(const std::vector<std::shared_ptr<Request>> &held,
                                                        const Request &like, int64_t others) {
    std::vector<std::shared_ptr<Request>> out;
    const int32_t cap = like.cls == 2 ? 1 : cfg.max_batch_graphs;
    if ((int32_t)held.size() >= cap || queue.empty()) return out;
    int64_t edges = 0;
    for (const auto &r : held) edges += 2ll * r->m;
    std::vector<std::shared_ptr<Request>> trial = held;
    for (const auto &r : queue) {
        if ((int32_t)trial.size() >= cap) break;
        if (r->cls != like.cls || !same_schedule(r->sched, like.sched)) continue;
        if (edges + 2ll * r->m > cfg.max_batch_edges) break;
        trial.push_back(r);
        if (estimate(trial) > cfg.hbm_budget_bytes - others) {
            trial.pop_back();
            break;
        }
        edges += 2ll * r->m;
        out.push_back(r);
    }
    if (!out.empty()) {
        std::deque<std::shared_ptr<Request>> rest;
        size_t j = 0;
        for (const auto &r : queue) {
            if (j < out.size() && r == out[j])
                ++j;
            else
                rest.push_back(r);
        }
        queue.swap(rest);
        stats.queue_len = (int64_t)queue.size();
    }
    return out;
}

void pcd_server::finish(Request &r, pcd_status st, Clock::time_point t_done, int64_t batch_graphs) {
    r.status = st;
    r.t_done = t_done;
    r.batch_graphs = batch_graphs;
    if (st == PCD_OK)
        ++stats.completed;
    else
        ++stats.failed;
    std::vector<int32_t>().swap(r.indices);
    std::vector<int32_t>().swap(r.adj);
    r.done = true;
}

// Continuous batching: the batch runs the driver loop (src/main.cpp:226-266)
// iteration by iteration on the host, every graph with its own iteration
// count, previous score and seed stream: compress and score the batch, stop
// test per graph, then one propagation or merge step of the whole batch with
// each graph's next seed.  A graph whose schedule ends is returned at once;
// at an iteration boundary the batch is rebuilt without the returned graphs
// and with queued requests of the same schedule and size class (new graphs
// start from singletons at their own iteration 0; under -s 2 they join only
// when the batch's next step is a propagation, so that every graph of a
// batch takes the same kind of step).  Each graph's labels, scores and
// iteration count are exactly those of running it alone.
void pcd_server::run_continuous(pcd_ctx *ctx, std::vector<std::shared_ptr<Request>> &batch, int64_t bytes) {
    const pcd_schedule sched = batch.front()->sched;
    const int32_t cap_it = sched.n_iter >= 0 ? sched.n_iter : 1000;  // threshold mode stops at 1000 iterations
    std::vector<Slot> slots;
    const auto t_start = Clock::now();
    for (auto &r : batch) {
        Slot sl;
        sl.r = r;
        r->t_start = t_start;
        slots.push_back(std::move(sl));
    }
    // held_bytes: this batch's share of in_flight.  It grows when requests
    // join (reserved at admission) and shrinks only once the old device copy
    // is freed.  batch_bytes: the estimate of the copy on the device now;
    // next_bytes: the estimate of the copy the next rebuild loads.
    int64_t held_bytes = bytes, batch_bytes = bytes, next_bytes = bytes;
    pcd_graph *b = nullptr;
    bool rebuild = true;
    pcd_status st = PCD_OK;
    std::vector<int32_t> voff, all_labels;
    std::vector<double> scores;
    auto free_batch = [&]() {
        if (!b) return;
        int64_t held = 0;
        pcd_graph_device_bytes(b, &held);
        pcd_graph_free(b);
        b = nullptr;
        std::lock_guard<std::mutex> lock(mu);
        stats.bytes_measured_peak = std::max(stats.bytes_measured_peak, held);
        if (held > batch_bytes) ++stats.estimate_exceeded;
    };
    while (st == PCD_OK) {
        if (rebuild) {  // pack the graphs still running (returned ones leave here)
            free_batch();
            if (next_bytes < held_bytes) {  // the old copy is gone: release the difference
                std::lock_guard<std::mutex> lock(mu);
                in_flight -= held_bytes - next_bytes;
                held_bytes = next_bytes;
                stats.bytes_in_flight = in_flight;
                cv_work.notify_all();
            }
            batch_bytes = next_bytes;
            slots.erase(std::remove_if(slots.begin(), slots.end(), [](const Slot &x) { return x.gone; }),
                        slots.end());
            if (slots.empty()) break;
            const int32_t G = (int32_t)slots.size();
            voff.assign((size_t)G + 1, 0);
            int64_t nnz = 0;
            for (int32_t i = 0; i < G; ++i) {
                voff[(size_t)i + 1] = voff[(size_t)i] + slots[(size_t)i].r->n;
                nnz += 2ll * slots[(size_t)i].r->m;
            }
            const int32_t N = voff[(size_t)G];
            std::vector<int32_t> ind((size_t)N + 1), adj((size_t)std::max<int64_t>(nnz, 1)), lab((size_t)N);
            int64_t e0 = 0;
            for (int32_t i = 0; i < G; ++i) {
                const Slot &sl = slots[(size_t)i];
                const Request &r = *sl.r;
                for (int32_t v = 0; v < r.n; ++v) {
                    ind[(size_t)voff[(size_t)i] + v] = (int32_t)(e0 + r.indices[(size_t)v]);
                    lab[(size_t)voff[(size_t)i] + v] = sl.fresh ? v : sl.labels[(size_t)v];
                }
                if (r.m) std::memcpy(adj.data() + e0, r.adj.data(), sizeof(int32_t) * 2 * (size_t)r.m);
                e0 += 2ll * r.m;
            }
            ind[(size_t)N] = (int32_t)e0;
            st = pcd_batch_load(ctx, G, voff.data(), ind.data(), adj.data(), &b);
            if (st == PCD_OK) st = pcd_batch_labels_set(b, lab.data());
            if (st != PCD_OK) break;
            rebuild = false;
        }
        const int32_t G = (int32_t)slots.size();
        scores.assign((size_t)G, 0.0);
        st = pcd_batch_score(b, &sched.rule, scores.data());
        if (st != PCD_OK) break;
        // the reference's stop test (src/main.cpp:241-242), per graph
        std::vector<int32_t> fin;
        int32_t live = 0, step_it = 0;
        for (int32_t i = 0; i < G; ++i) {
            const Slot &sl = slots[(size_t)i];
            if (sl.gone) continue;
            const double sc = scores[(size_t)i];
            const bool done = sched.n_iter != -1 ? sl.it >= sched.n_iter
                                                 : ((sl.prev > 0 && sc > 0 && sc / sl.prev - 1 <= sched.threshold) ||
                                                    sl.it >= cap_it - 1);
            if (done) {
                fin.push_back(i);
            } else {
                ++live;
                step_it = sl.it;  // every live graph of the batch has the same parity
            }
        }
        bool have_labels = false;
        if (!fin.empty()) {  // return finished graphs now
            all_labels.assign((size_t)voff[(size_t)G], 0);
            st = pcd_batch_labels_get(b, all_labels.data());
            if (st != PCD_OK) break;
            have_labels = true;
            const auto t_done = Clock::now();
            std::lock_guard<std::mutex> lock(mu);
            for (int32_t i : fin) {
                Slot &sl = slots[(size_t)i];
                Request &r = *sl.r;
                r.labels.assign(all_labels.begin() + voff[(size_t)i], all_labels.begin() + voff[(size_t)i + 1]);
                r.score = scores[(size_t)i];
                r.iterations = sl.it;
                if (live > 0) ++stats.released_early;
                finish(r, PCD_OK, t_done, G);
                sl.gone = true;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
        // queued requests of this schedule and size class join between
        // iterations (under -s 2 only before a propagation step)
        std::vector<std::shared_ptr<Request>> joined;
        const bool prop_next = sched.strategy == 0 || (sched.strategy == 2 && step_it % 2 == 0);
        int32_t gone = 0;
        for (const Slot &sl : slots) gone += sl.gone ? 1 : 0;
        if (live > 0) {
            std::lock_guard<std::mutex> lock(mu);
            std::vector<std::shared_ptr<Request>> held;
            for (const Slot &sl : slots)
                if (!sl.gone) held.push_back(sl.r);
            // the other batches hold in_flight - held_bytes; the copy of this
            // one stays on the device until the rebuild below frees it, so a
            // joining request is charged on top of held_bytes when the new
            // estimate exceeds it
            if (sched.strategy != 2 || prop_next) joined = admit(held, *held.front(), in_flight - held_bytes);
            if (!joined.empty() || 4 * gone >= G) {  // the batch is rebuilt below
                std::vector<std::shared_ptr<Request>> now = held;
                now.insert(now.end(), joined.begin(), joined.end());
                next_bytes = estimate(now);
                if (next_bytes > held_bytes) {
                    in_flight += next_bytes - held_bytes;
                    held_bytes = next_bytes;
                    stats.bytes_in_flight = in_flight;
                    stats.bytes_peak = std::max(stats.bytes_peak, in_flight);
                }
            }
            stats.admitted_running += (int64_t)joined.size();
            stats.batched_graphs += (int64_t)joined.size();
        }
        if (live == 0) break;
        if (!joined.empty() || 4 * gone >= G) {
            // rebuild: running graphs keep their labels, newcomers start from
            // singletons; the next pass scores and stop-tests everyone (the
            // same outcome again for the running graphs)
            if (!have_labels) {
                all_labels.assign((size_t)voff[(size_t)G], 0);
                st = pcd_batch_labels_get(b, all_labels.data());
                if (st != PCD_OK) break;
            }
            for (int32_t i = 0; i < G; ++i) {
                Slot &sl = slots[(size_t)i];
                if (sl.gone) continue;
                sl.labels.assign(all_labels.begin() + voff[(size_t)i], all_labels.begin() + voff[(size_t)i + 1]);
                sl.fresh = false;
            }
            const auto t_join = Clock::now();
            for (auto &r : joined) {
                Slot sl;
                sl.r = r;
                r->t_start = t_join;
                slots.push_back(std::move(sl));
            }
            rebuild = true;
            continue;
        }
        // one step of the batch, every live graph with its own next seed
        // (returned graphs still in the batch step too; their results are unused)
        std::vector<uint32_t> seeds((size_t)G, 0u);
        for (int32_t i = 0; i < G; ++i)
            if (!slots[(size_t)i].gone) seeds[(size_t)i] = (uint32_t)pcd_rand_next(&slots[(size_t)i].r->seeds);
        const bool merge = sched.strategy == 1 || (sched.strategy == 2 && step_it % 2 == 1);
        st = merge ? pcd_batch_merge(b, &sched.rule, sched.rounds, seeds.data())
                   : pcd_batch_refine(b, &sched.rule, sched.frac, seeds.data());
        if (st != PCD_OK) break;
        for (int32_t i = 0; i < G; ++i) {
            Slot &sl = slots[(size_t)i];
            if (sl.gone) continue;
            sl.prev = scores[(size_t)i];
            ++sl.it;
        }
    }
    free_batch();
    std::lock_guard<std::mutex> lock(mu);
    for (Slot &sl : slots)
        if (!sl.gone) finish(*sl.r, st == PCD_OK ? PCD_ERR_CUDA : st, Clock::now(), (int64_t)slots.size());
    if (batch.front()->cls > 0) --big_in_flight;
    in_flight -= held_bytes;
    stats.bytes_in_flight = in_flight;
    ++stats.batches;
    stats.batched_graphs += (int64_t)batch.size();
    cv_done.notify_all();
    cv_work.notify_all();
}


// Forms the next batch, or returns false when stopping with an empty queue.
// Requests too large for the whole budget fail here.  A batch holds one size
// class only, and while workers - 1 batches of medium or large graphs run, a
// free worker serves the oldest small request instead, so small graphs never
// wait behind long runs of big ones.
bool pcd_server::take_batch(std::vector<std::shared_ptr<Request>> &batch, int64_t &bytes) {
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
        cv_work.wait(lock, [&] { return stopping || !queue.empty(); });
        if (queue.empty()) return false;  // stopping
        std::shared_ptr<Request> head = queue.front();
        if (head->cls > 0 && cfg.workers > 1 && big_in_flight >= cfg.workers - 1) {
            head = nullptr;
            for (const auto &r : queue)
                if (r->cls == 0) {
                    head = r;
                    break;
                }
            if (!head) {  // only big requests wait: hold this worker back
                cv_work.wait(lock);
                continue;
            }
        }
        if (estimate({head}) > cfg.hbm_budget_bytes) {
            queue.erase(std::find(queue.begin(), queue.end(), head));
            head->status = PCD_ERR_OUT_OF_MEMORY;
            head->done = true;
            head->t_start = head->t_done = Clock::now();
            ++stats.failed;
            stats.queue_len = (int64_t)queue.size();
            cv_done.notify_all();
            continue;
        }
        // requests of the head's schedule, in arrival order, within the caps
        std::vector<std::shared_ptr<Request>> pick;
        int64_t edges = 0;
        const int32_t cap = head->cls == 2 ? 1 : cfg.max_batch_graphs;
        for (const auto &r : queue) {
            if ((int32_t)pick.size() >= cap) break;
            if (r->cls != head->cls || !same_schedule(r->sched, head->sched)) continue;
            if (!pick.empty() && edges + 2ll * r->m > cfg.max_batch_edges) break;
            pick.push_back(r);
            if (estimate(pick) > cfg.hbm_budget_bytes - in_flight) {
                pick.pop_back();
                break;
            }
            edges += 2ll * r->m;
        }
        if (pick.empty()) {  // the head waits for memory held by batches in flight
            cv_work.wait(lock);
            continue;
        }
        // a partial batch waits for company until its oldest request is max_wait_ms old
        if ((int32_t)pick.size() < cap && !stopping && cfg.max_wait_ms > 0) {
            const auto deadline = head->t_submit + std::chrono::microseconds((int64_t)(cfg.max_wait_ms * 1000.0));
            if (Clock::now() < deadline) {
                cv_work.wait_until(lock, deadline);
                continue;  // the queue may have changed: form the batch again
            }
        }
        bytes = estimate(pick);
        if (head->cls > 0) ++big_in_flight;
        in_flight += bytes;
        stats.bytes_in_flight = in_flight;
        stats.bytes_peak = std::max(stats.bytes_peak, in_flight);
        std::deque<std::shared_ptr<Request>> rest;
        size_t j = 0;
        for (const auto &r : queue) {
            if (j < pick.size() && r == pick[j])
                ++j;
            else
                rest.push_back(r);
        }
        queue.swap(rest);
        stats.queue_len = (int64_t)queue.size();
        batch.swap(pick);
        if (!queue.empty()) cv_work.notify_one();  // another worker may batch the rest
        return true;
    }
}

void pcd_server::run_batch(pcd_ctx *ctx, std::vector<std::shared_ptr<Request>> &batch, int64_t bytes) {
    const auto t_start = Clock::now();
    const int32_t G = (int32_t)batch.size();
    std::vector<int32_t> voff((size_t)G + 1, 0);
    int64_t nnz = 0;
    for (int32_t i = 0; i < G; ++i) {
        voff[(size_t)i + 1] = voff[(size_t)i] + batch[(size_t)i]->n;
        nnz += 2ll * batch[(size_t)i]->m;
    }
    const int32_t N = voff[(size_t)G];
    std::vector<int32_t> ind((size_t)N + 1), adj((size_t)std::max<int64_t>(nnz, 1));
    int64_t e0 = 0;
    for (int32_t i = 0; i < G; ++i) {
        const Request &r = *batch[(size_t)i];
        for (int32_t v = 0; v < r.n; ++v) ind[(size_t)voff[(size_t)i] + v] = (int32_t)(e0 + r.indices[(size_t)v]);
        if (r.m) std::memcpy(adj.data() + e0, r.adj.data(), sizeof(int32_t) * 2 * (size_t)r.m);
        e0 += 2ll * r.m;
    }
    ind[(size_t)N] = (int32_t)e0;
    std::vector<double> scores((size_t)G, 0.0);
    std::vector<int32_t> iters((size_t)G, 0), labels((size_t)std::max(N, 1));
    const pcd_schedule &s = batch.front()->sched;
    pcd_graph *b = nullptr;
    pcd_status st = pcd_batch_load(ctx, G, voff.data(), ind.data(), adj.data(), &b);
    if (st == PCD_OK)
        st = pcd_batch_run(b, &s.rule, s.strategy, s.frac, s.rounds, s.n_iter, s.threshold, cfg.use_cuda_graph,
                           scores.data(), iters.data());
    if (st == PCD_OK) st = pcd_batch_labels_get(b, labels.data());
    int64_t held = 0;
    if (b) {
        pcd_graph_device_bytes(b, &held);
        pcd_graph_free(b);
    }
    const auto t_done = Clock::now();
    std::lock_guard<std::mutex> lock(mu);
    if (batch.front()->cls > 0) --big_in_flight;
    in_flight -= bytes;
    stats.bytes_in_flight = in_flight;
    stats.bytes_measured_peak = std::max(stats.bytes_measured_peak, held);
    if (held > bytes) ++stats.estimate_exceeded;
    ++stats.batches;
    stats.batched_graphs += G;
    for (int32_t i = 0; i < G; ++i) {
        Request &r = *batch[(size_t)i];
        r.status = st;
        r.t_start = t_start;
        r.t_done = t_done;
        r.batch_graphs = G;
        if (st == PCD_OK) {
            r.labels.assign(labels.begin() + voff[(size_t)i], labels.begin() + voff[(size_t)i + 1]);
            r.score = scores[(size_t)i];
            r.iterations = iters[(size_t)i];
            ++stats.completed;
        } else {
            ++stats.failed;
        }
        std::vector<int32_t>().swap(r.indices);
        std::vector<int32_t>().swap(r.adj);
        r.done = true;
    }
    cv_done.notify_all();
    cv_work.notify_all();
}

void pcd_server::worker_main() {
    pcd_ctx *ctx = nullptr;
    const pcd_status st = pcd_init(&ctx, cfg.device);
    {
        std::lock_guard<std::mutex> lock(mu);
        if (st != PCD_OK) start_status = st;
        ++started;
    }
    cv_done.notify_all();
    if (st != PCD_OK) {
        if (ctx) pcd_destroy(ctx);
        return;
    }
    // small batches run on a high-priority stream: whenever blocks of a long
    // run's kernels retire, the scheduler starts the small batch's blocks first
    int lo_prio = 0, hi_prio = 0;
    cudaStream_t s_hi = nullptr, s_lo = nullptr;
    if (cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s_hi, cudaStreamNonBlocking, hi_prio) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s_lo, cudaStreamNonBlocking, lo_prio) != cudaSuccess) {
        cudaGetLastError();  // no priorities: every batch stays on the context's own stream
        if (s_hi) cudaStreamDestroy(s_hi);
        s_hi = s_lo = nullptr;
    }
    cudaStream_t cur = nullptr;
    for (;;) {
        std::vector<std::shared_ptr<Request>> batch;
        int64_t bytes = 0;
        if (!take_batch(batch, bytes)) break;
        cudaStream_t want = s_hi ? (batch.front()->cls == 0 ? s_hi : s_lo) : nullptr;
        if (want != cur && pcd_set_stream(ctx, want) == PCD_OK) cur = want;
        ctx->grid_scale = batch.front()->cls == 0 ? 1 : 8;  // long runs release SMs block by block
        if (cfg.continuous)
            run_continuous(ctx, batch, bytes);
        else
            run_batch(ctx, batch, bytes);
    }
    pcd_set_stream(ctx, nullptr);
    if (s_hi) cudaStreamDestroy(s_hi);
    if (s_lo) cudaStreamDestroy(s_lo);
    pcd_destroy(ctx);
}

extern "C" {

pcd_status pcd_serve_start(const pcd_serve_config *cfg, pcd_server **out) {
    if (!cfg || !out || cfg->workers < 1 || cfg->max_batch_graphs < 1 || cfg->max_batch_edges < 1 ||
        cfg->hbm_budget_bytes < 1 || cfg->max_wait_ms < 0 || cfg->small_graph_edges < 0 ||
        cfg->large_graph_edges < cfg->small_graph_edges)
        return PCD_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pcd_server *s = new (std::nothrow) pcd_server;
    if (!s) return PCD_ERR_OUT_OF_MEMORY;
    s->cfg = *cfg;
    pcd_ctx *probe = nullptr;
    pcd_status st = pcd_init(&probe, cfg->device);
    if (st == PCD_OK) {
        int32_t sms = 0;
        st = pcd_device_sm_count(probe, &sms);
        s->num_sms = std::max(sms, 1);
    }
    if (probe) pcd_destroy(probe);
    if (st == PCD_OK) st = pcd::keep_pool_memory(cfg->device, cfg->hbm_budget_bytes);
    if (st != PCD_OK) {
        delete s;
        return st;
    }
    for (int32_t i = 0; i < cfg->workers; ++i) s->workers.emplace_back([s] { s->worker_main(); });
    {
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv_done.wait(lock, [&] { return s->started == cfg->workers; });
        st = s->start_status;
    }
    if (st != PCD_OK) {
        pcd_serve_stop(s);
        return st;
    }
    *out = s;
    return PCD_OK;
}

pcd_status pcd_serve_submit(pcd_server *s, int32_t n, int32_t m, const int32_t *indices, const int32_t *adj,
                            const pcd_schedule *sched, uint64_t *ticket) {
    if (!s || !sched || !ticket || n < 1 || m < 0 || !indices || (m > 0 && !adj)) return PCD_ERR_INVALID_ARGUMENT;
    if (sched->rule.kind == PCD_RULE_WCC) return PCD_ERR_UNSUPPORTED;  // batched runs start from singletons
    if (!(sched->frac > 0.0 && sched->frac <= 1.0) || sched->rounds < 1 || sched->strategy < 0 ||
        sched->strategy > 2)
        return PCD_ERR_INVALID_ARGUMENT;
    // the CSR is checked here so that one bad graph cannot fail a batch
    if (indices[0] != 0 || (int64_t)indices[n] != 2ll * m) return PCD_ERR_FORMAT;
    auto r = std::make_shared<Request>();
    r->n = n;
    r->m = m;
    r->sched = *sched;
    for (int32_t v = 0; v < n; ++v) {
        const int32_t b = indices[v], e = indices[v + 1];
        if (e < b) return PCD_ERR_FORMAT;
        for (int32_t j = b; j < e; ++j) {
            const int32_t u = adj[j];
            if (u < 0 || u >= n || u == v || (j > b && adj[j - 1] >= u)) return PCD_ERR_FORMAT;
        }
        r->max_deg = std::max(r->max_deg, e - b);
        if (e - b > 8192) ++r->hubs;
    }
    r->cls = 2ll * m <= s->cfg.small_graph_edges ? 0 : (2ll * m <= s->cfg.large_graph_edges ? 1 : 2);
    r->indices.assign(indices, indices + n + 1);
    r->adj.assign(adj, adj + 2 * (size_t)m);
    // the driver's rand() stream: create_singleton_partition draws n values
    // first, then every refinement draws its seed (src/framework.cpp:14-24)
    pcd_rand_seed(&r->seeds, 1);
    pcd_rand_skip(&r->seeds, n);
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stopping) return PCD_ERR_INVALID_ARGUMENT;
        r->id = s->next_id++;
        r->t_submit = Clock::now();
        s->tickets[r->id] = r;
        s->queue.push_back(r);
        ++s->stats.submitted;
        s->stats.queue_len = (int64_t)s->queue.size();
        *ticket = r->id;
    }
    s->cv_work.notify_one();
    return PCD_OK;
}

pcd_status pcd_serve_poll(pcd_server *s, uint64_t ticket, int32_t *done) {
    if (!s || !done) return PCD_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return PCD_ERR_INVALID_ARGUMENT;
    *done = it->second->done ? 1 : 0;
    return PCD_OK;
}

pcd_status pcd_serve_wait(pcd_server *s, uint64_t ticket, int32_t *labels, double *score, int32_t *iterations,
                          pcd_serve_timing *timing) {
    if (!s) return PCD_ERR_INVALID_ARGUMENT;
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return PCD_ERR_INVALID_ARGUMENT;
        r = it->second;
        s->cv_done.wait(lock, [&] { return r->done; });
        s->tickets.erase(ticket);
    }
    if (timing) {
        timing->queue_ms = ms_since(r->t_submit, r->t_start);
        timing->latency_ms = ms_since(r->t_submit, r->t_done);
        timing->batch_graphs = r->batch_graphs;
    }
    if (r->status != PCD_OK) return r->status;
    if (labels) std::memcpy(labels, r->labels.data(), sizeof(int32_t) * r->labels.size());
    if (score) *score = r->score;
    if (iterations) *iterations = r->iterations;
    return PCD_OK;
}

pcd_status pcd_serve_stats_get(pcd_server *s, pcd_serve_stats *out) {
    if (!s || !out) return PCD_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->stats;
    return PCD_OK;
}

pcd_status pcd_serve_stop(pcd_server *s) {
    if (!s) return PCD_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers)
        if (t.joinable()) t.join();
    delete s;
    return PCD_OK;
}

}  // extern "C"
