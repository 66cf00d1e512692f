// serve.cu -- the serving loop: several resident indexes, admission by a
// memory estimate and free batch slots, continuous batching on per-slot
// streams, and latency accounting.
//
// Reference counterparts: knn_MT packs tables into a launch while free device
// memory exceeds an estimate (matching/knn.cu:206-278); the odgenie server
// takes one JSON request off a queue and runs it as one synchronous batch
// (dist_genie/online.cu:37-180, scheduler.cc:20-64).  Here one scheduler
// thread keeps up to slots_per_index batches of every index on the device,
// each a genie_batch (fixed buffers, CUDA graph, own stream); requests that
// arrive while those run are admitted into the next free slot.
#include "capi_internal.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>

using namespace gg;

namespace {

int64_t mono_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Request {
    uint64_t ticket = 0;
    int32_t index = 0;
    uint32_t k = 0;
    uint8_t weighted = 0;
    std::vector<int32_t> dim, low, up;
    std::vector<float> weight;
    int64_t arrival_ns = 0, done_ns = 0, bytes = 0;
    std::vector<uint32_t> ids, counts;
    std::vector<float> scores;
    int status = GENIE_OK;
    std::string error;
    bool done = false;
    bool held = false;                 // its launch waited for in-flight memory to free up
};

// Device-side state a request holds while in flight: its items and plan rows,
// its k result slots, and the per-part keys of its top-k merge.
int64_t request_bytes(int64_t items, uint32_t k) {
    return items * 48 + (int64_t)k * (kMaxDenseParts * 8 + 12) + 256;
}

struct Slot {
    genie_batch *b = nullptr;
    bool busy = false;
    std::vector<Request *> reqs;
    int64_t bytes = 0;
};

struct Served {
    genie_index *ix = nullptr;
    std::vector<Slot> slots;
    std::deque<Request *> pending;     // ordered by arrival
};

}  // namespace

struct genie_server {
    genie_server_config cfg{};
    int device = 0;
    std::vector<Served> idx;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::unordered_map<uint64_t, Request *> reqs;
    uint64_t next_ticket = 1;
    std::thread worker;
    bool running = false, stop = false;
    int64_t in_flight_bytes = 0;
    // statistics since the last reset
    int64_t held = 0, peak_in_flight_bytes = 0;
    std::vector<int64_t> lat_ns;
    int64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched = 0;
    int64_t first_arrival = INT64_MAX, last_done = 0;
    int64_t outstanding = 0;           // submitted and not yet answered
    ~genie_server();
    void loop();
};

genie_server::~genie_server() {
    {
        std::lock_guard<std::mutex> lk(m);
        stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    cudaSetDevice(device);
    for (Served &sv : idx)
        for (Slot &sl : sv.slots)
            if (sl.b) genie_batch_destroy(sl.b);
    for (auto &kv : reqs) delete kv.second;
}

// Scheduler: completions first, then launches, then sleep until the next
// arrival or a short poll interval while batches run.  On destruction the
// batches on the device finish; requests not yet launched are dropped.
void genie_server::loop() {
    cudaSetDevice(device);
    std::vector<int64_t> item_off;
    std::vector<int32_t> dim, low, up;
    std::vector<float> weight;
    std::vector<uint8_t> weighted;
    std::vector<uint32_t> kk, ids, counts;
    std::vector<float> scores;
    std::unique_lock<std::mutex> lk(m);
    for (;;) {
        const int64_t now = mono_ns();
        bool progressed = false, any_busy = false;
        // ---- completions
        for (Served &sv : idx) {
            for (Slot &sl : sv.slots) {
                if (!sl.busy) continue;
                const int r = batch_ready(sl.b);
                if (r == 0) {
                    any_busy = true;
                    continue;
                }
                int64_t total_k = 0;
                for (Request *q : sl.reqs) total_k += q->k;
                ids.resize(total_k);
                counts.resize(total_k);
                scores.resize(total_k);
                int rc = r < 0 ? -r : batch_collect(sl.b, ids.data(), counts.data(), scores.data());
                const std::string err = rc ? genie_last_error() : std::string();
                const int64_t t = mono_ns();
                int64_t off = 0;
                for (Request *q : sl.reqs) {
                    if (!rc) {
                        q->ids.assign(ids.begin() + off, ids.begin() + off + q->k);
                        q->counts.assign(counts.begin() + off, counts.begin() + off + q->k);
                        q->scores.assign(scores.begin() + off, scores.begin() + off + q->k);
                    }
                    off += q->k;
                    q->status = rc;
                    q->error = err;
                    q->done = true;
                    q->done_ns = t;
                    lat_ns.push_back(t - q->arrival_ns);
                    first_arrival = std::min(first_arrival, q->arrival_ns);
                    last_done = std::max(last_done, t);
                    ++completed;
                    --outstanding;
                }
                in_flight_bytes -= sl.bytes;
                sl.bytes = 0;
                sl.reqs.clear();
                sl.busy = false;
                progressed = true;
            }
        }
        if (progressed) cv_done.notify_all();
        // ---- launches: every free slot takes the requests that have arrived
        int64_t next_arrival = INT64_MAX;
        if (stop) {                  // finish what runs; requests not yet launched are dropped
            if (!any_busy) break;
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(2));
            lk.lock();
            continue;
        }
        for (Served &sv : idx) {
            int busy_slots = 0;
            for (Slot &sl : sv.slots) busy_slots += sl.busy ? 1 : 0;
            for (Slot &sl : sv.slots) {
                if (sl.busy || sv.pending.empty()) continue;
                if (sv.pending.front()->arrival_ns > now) {
                    next_arrival = std::min(next_arrival, sv.pending.front()->arrival_ns);
                    break;
                }
                // while another batch of this index runs, let a short window fill the batch
                size_t ready = 0;
                int64_t items = 0, bytes = 0;
                for (Request *q : sv.pending) {
                    if (q->arrival_ns > now || (int64_t)ready >= cfg.max_queries) break;
                    if (items + (int64_t)q->dim.size() > cfg.max_items) break;
                    if (cfg.memory_budget > 0 && in_flight_bytes + bytes + q->bytes > cfg.memory_budget) {
                        if (!q->held) {          // admission holds it back until memory frees up
                            q->held = true;
                            ++held;
                        }
                        break;
                    }
                    ++ready;
                    items += (int64_t)q->dim.size();
                    bytes += q->bytes;
                }
                if (ready == 0) break;      // memory budget: wait for a completion
                const bool full = (int64_t)ready >= cfg.max_queries ||
                                  (ready < sv.pending.size() && sv.pending[ready]->arrival_ns <= now);
                const int64_t waited = now - sv.pending.front()->arrival_ns;
                if (!full && busy_slots > 0 && waited < (int64_t)cfg.window_us * 1000) {
                    next_arrival = std::min(next_arrival, sv.pending.front()->arrival_ns + (int64_t)cfg.window_us * 1000);
                    break;
                }
                // assemble the batch
                item_off.assign(1, 0);
                dim.clear();
                low.clear();
                up.clear();
                weight.clear();
                weighted.clear();
                kk.clear();
                bool any_weighted = false;
                for (size_t i = 0; i < ready; ++i) {
                    Request *q = sv.pending.front();
                    sv.pending.pop_front();
                    sl.reqs.push_back(q);
                    dim.insert(dim.end(), q->dim.begin(), q->dim.end());
                    low.insert(low.end(), q->low.begin(), q->low.end());
                    up.insert(up.end(), q->up.begin(), q->up.end());
                    if (q->weighted) weight.insert(weight.end(), q->weight.begin(), q->weight.end());
                    else weight.insert(weight.end(), q->dim.size(), 1.0f);
                    weighted.push_back(q->weighted);
                    any_weighted = any_weighted || q->weighted;
                    kk.push_back(q->k);
                    item_off.push_back((int64_t)dim.size());
                }
                genie_queries gq{};
                gq.n_queries = (int64_t)ready;
                gq.item_off = item_off.data();
                gq.dim = dim.data();
                gq.low = low.data();
                gq.up = up.data();
                gq.weight = any_weighted ? weight.data() : nullptr;
                gq.weighted = any_weighted ? weighted.data() : nullptr;
                gq.k = kk.data();
                const int rc = batch_submit_async(sl.b, &gq, true);
                sl.bytes = bytes;
                in_flight_bytes += bytes;
                peak_in_flight_bytes = std::max(peak_in_flight_bytes, in_flight_bytes);
                sl.busy = true;
                ++batches;
                batched += (int64_t)ready;
                ++busy_slots;
                progressed = true;
                any_busy = true;
                if (rc) {           // answered at once with the launch error
                    const std::string err = genie_last_error();
                    const int64_t t = mono_ns();
                    for (Request *q : sl.reqs) {
                        q->status = rc;
                        q->error = err;
                        q->done = true;
                        q->done_ns = t;
                        ++completed;
                        --outstanding;
                    }
                    in_flight_bytes -= sl.bytes;
                    sl.bytes = 0;
                    sl.reqs.clear();
                    sl.busy = false;
                    cv_done.notify_all();
                }
            }
            if (!sv.pending.empty() && sv.pending.front()->arrival_ns > now)
                next_arrival = std::min(next_arrival, sv.pending.front()->arrival_ns);
        }
        if (progressed) continue;
        // ---- sleep: poll running batches every few microseconds, else until
        // the next arrival or a submission
        if (any_busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(2));
            lk.lock();
        } else if (next_arrival != INT64_MAX) {
            const int64_t dt = next_arrival - mono_ns();
            if (dt > 0) cv_work.wait_for(lk, std::chrono::nanoseconds(dt));
        } else {
            cv_work.wait(lk);
        }
    }
}

extern "C" {

int64_t genie_server_now_ns(void) { return mono_ns(); }

int genie_server_create(const genie_server_config *cfg, genie_server **out) {
    if (!cfg || !out) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->slots_per_index < 1 || cfg->max_queries < 1 || cfg->max_items < 1 || cfg->max_k < 1 ||
        cfg->max_k > (uint32_t)kMaxK || cfg->window_us < 0 || cfg->memory_budget < 0)
        return fail(GENIE_ERR_INVALID_ARG, "server configuration out of range");
    genie_server *s = new (std::nothrow) genie_server;
    if (!s) return fail(GENIE_ERR_CPU_ALLOC, "server");
    s->cfg = *cfg;
    cudaGetDevice(&s->device);
    *out = s;
    return GENIE_OK;
}

int genie_server_add_index(genie_server *s, genie_index *ix, int32_t *index_id) {
    if (!s || !ix) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->m);
    if (s->running) return fail(GENIE_ERR_INVALID_ARG, "indexes are added before genie_server_start");
    Served sv;
    sv.ix = ix;
    genie_batch_config bc{};
    bc.max_queries = s->cfg.max_queries;
    bc.max_items = s->cfg.max_items;
    bc.max_k = s->cfg.max_k;
    bc.use_graph = 1;
    sv.slots.resize((size_t)s->cfg.slots_per_index);
    for (Slot &sl : sv.slots) {
        const int rc = genie_batch_create(ix, &bc, &sl.b);
        if (rc) {
            for (Slot &t : sv.slots)
                if (t.b) genie_batch_destroy(t.b);
            return rc;
        }
    }
    s->device = ix->device;
    s->idx.push_back(std::move(sv));
    if (index_id) *index_id = (int32_t)s->idx.size() - 1;
    return GENIE_OK;
}

int genie_server_start(genie_server *s) {
    if (!s) return fail(GENIE_ERR_INVALID_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(s->m);
    if (s->running) return GENIE_OK;
    if (s->idx.empty()) return fail(GENIE_ERR_INVALID_ARG, "no index added");
    s->running = true;
    s->worker = std::thread([s] { s->loop(); });
    return GENIE_OK;
}

int genie_server_submit(genie_server *s, int32_t index_id, const genie_queries *q, const int64_t *arrival_ns,
                        uint64_t *first_ticket) {
    if (!s || !q) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    if (!s->running) return fail(GENIE_ERR_INVALID_ARG, "server not started");
    if (index_id < 0 || index_id >= (int32_t)s->idx.size()) return fail(GENIE_ERR_INVALID_ARG, "unknown index %d", index_id);
    std::vector<int64_t> out_off;
    int64_t n_items = 0;
    int rc = validate_queries(q, out_off, n_items);
    if (rc) return rc;
    const int64_t Q = q->n_queries;
    std::vector<Request *> made;
    made.reserve((size_t)Q);
    const int64_t t_now = mono_ns();
    for (int64_t i = 0; i < Q; ++i) {
        const int64_t a = q->item_off[i], b = q->item_off[i + 1];
        const uint32_t k = q->k ? q->k[i] : q->uniform_k;
        const int64_t bytes = request_bytes(b - a, k);
        if (k > s->cfg.max_k || b - a > s->cfg.max_items ||
            (s->cfg.memory_budget > 0 && bytes > s->cfg.memory_budget)) {
            for (Request *r : made) delete r;
            std::lock_guard<std::mutex> lk(s->m);
            s->rejected += Q;
            return fail(GENIE_ERR_ADMISSION,
                        "request %lld (k=%u, %lld items, ~%lld bytes) exceeds the server's limits",
                        (long long)i, k, (long long)(b - a), (long long)bytes);
        }
        Request *r = new Request;
        r->index = index_id;
        r->k = k;
        r->weighted = (q->weighted && q->weight) ? q->weighted[i] : 0;
        r->dim.assign(q->dim + a, q->dim + b);
        r->low.assign(q->low + a, q->low + b);
        r->up.assign(q->up + a, q->up + b);
        if (r->weighted) r->weight.assign(q->weight + a, q->weight + b);
        r->arrival_ns = arrival_ns ? arrival_ns[i] : t_now;
        r->bytes = bytes;
        made.push_back(r);
    }
    {
        std::lock_guard<std::mutex> lk(s->m);
        std::deque<Request *> &pend = s->idx[(size_t)index_id].pending;
        if (first_ticket) *first_ticket = s->next_ticket;
        for (Request *r : made) {
            r->ticket = s->next_ticket++;
            s->reqs[r->ticket] = r;
            if (pend.empty() || pend.back()->arrival_ns <= r->arrival_ns) {
                pend.push_back(r);
            } else {
                auto it = std::upper_bound(pend.begin(), pend.end(), r->arrival_ns,
                                           [](int64_t t, const Request *x) { return t < x->arrival_ns; });
                pend.insert(it, r);
            }
        }
        s->submitted += Q;
        s->outstanding += Q;
    }
    s->cv_work.notify_all();
    return GENIE_OK;
}

int genie_server_wait(genie_server *s, uint64_t ticket, uint32_t *out_ids, uint32_t *out_counts,
                      float *out_scores, int64_t *latency_ns) {
    if (!s) return fail(GENIE_ERR_INVALID_ARG, "server is NULL");
    std::unique_lock<std::mutex> lk(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(GENIE_ERR_INVALID_ARG, "unknown ticket %llu", (unsigned long long)ticket);
    Request *r = it->second;
    s->cv_done.wait(lk, [r] { return r->done; });
    s->reqs.erase(it);
    lk.unlock();
    const int rc = r->status;
    if (!rc) {
        if (out_ids) memcpy(out_ids, r->ids.data(), r->k * 4);
        if (out_counts) memcpy(out_counts, r->counts.data(), r->k * 4);
        if (out_scores) memcpy(out_scores, r->scores.data(), r->k * 4);
    }
    if (latency_ns) *latency_ns = r->done_ns - r->arrival_ns;
    const std::string err = r->error;
    delete r;
    return rc ? fail(rc, "%s", err.c_str()) : GENIE_OK;
}

int genie_server_drain(genie_server *s) {
    if (!s) return fail(GENIE_ERR_INVALID_ARG, "server is NULL");
    std::unique_lock<std::mutex> lk(s->m);
    s->cv_done.wait(lk, [s] { return s->outstanding == 0; });
    return GENIE_OK;
}

int genie_server_stats(genie_server *s, genie_server_report *out) {
    if (!s || !out) return fail(GENIE_ERR_INVALID_ARG, "NULL argument");
    std::vector<int64_t> lat;
    {
        std::lock_guard<std::mutex> lk(s->m);
        lat = s->lat_ns;
        out->submitted = s->submitted;
        out->completed = s->completed;
        out->rejected = s->rejected;
        out->batches = s->batches;
        out->mean_batch = s->batches ? (double)s->batched / (double)s->batches : 0.0;
        out->held = s->held;
        out->peak_in_flight_bytes = s->peak_in_flight_bytes;
        const int64_t span = s->last_done - s->first_arrival;
        out->throughput_qps = (s->completed && span > 0) ? (double)s->completed * 1e9 / (double)span : 0.0;
    }
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)std::min<double>((double)lat.size() - 1, p * (double)(lat.size() - 1) + 0.5);
        return (double)lat[i] / 1e3;
    };
    out->p50_us = pct(0.50);
    out->p99_us = pct(0.99);
    out->max_us = lat.empty() ? 0.0 : (double)lat.back() / 1e3;
    return GENIE_OK;
}

int genie_server_reset_stats(genie_server *s) {
    if (!s) return fail(GENIE_ERR_INVALID_ARG, "server is NULL");
    std::lock_guard<std::mutex> lk(s->m);
    s->lat_ns.clear();
    s->submitted = s->completed = s->rejected = s->batches = s->batched = 0;
    s->held = 0;
    s->peak_in_flight_bytes = s->in_flight_bytes;
    s->first_arrival = INT64_MAX;
    s->last_done = 0;
    return GENIE_OK;
}

int genie_server_destroy(genie_server *s) {
    if (!s) return GENIE_OK;
    delete s;
    return GENIE_OK;
}

}  // extern "C"
