// serve.cu — the served form: continuous batching of requests onto batch slots.
//
// A server keeps the index resident and owns `slots` batchers (the batched form: each
// batch one launch of a captured CUDA graph), each with its own streams and device
// work areas for batches of up to batch_reads reads / batch_bases bases.  The slots are
// created against a device-memory budget (by default half the memory free when the
// server is created): each slot's work areas are measured as it is created, and no
// slot is added once the budget would be exceeded (at least one is).  A host thread
// per slot takes, whenever its slot is free, every request waiting at the head of the
// queue that still fits the slot (reads and bases), maps them as one batch, and copies
// each request's NAMs, offsets, fractions and rescue flags straight from the batch's
// device outputs into that request's buffers.  Requests that arrive while batches are
// on the GPU are taken by the next slot to come free, so small requests share launches
// and requests overlap on the device; each request's results equal gbsa_map_reads'
// for its reads alone (a read's NAMs depend only on the read).  No reference
// counterpart: the reference maps one file per process (step2/main.cu:4100-4760).
#include <atomic>
#include <chrono>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "mapper.h"

namespace {

struct Request {
    gbsa::ServeRequest r;
    uint64_t bases;
    uint64_t tag;
    std::chrono::steady_clock::time_point t_submit;
};

struct Done {
    uint64_t tag;
    int status;
    uint64_t nam_total;
};

}  // namespace

struct gbsa_server {
    const gbsa_index* idx = nullptr;
    int device = 0;
    gbsa_server_config cfg{};
    std::vector<gbsa_batcher*> slots;
    uint64_t slot_bytes = 0;      // device bytes one slot's work areas took at creation
    uint64_t budget = 0;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_req, cv_done;
    std::deque<Request> queue;
    std::deque<Done> done;
    bool stop = false;
    uint64_t in_flight = 0;
    uint64_t batches = 0, requests_batched = 0, max_requests_per_batch = 0;

    void work(gbsa_batcher* b) {
        cudaSetDevice(device);
        std::vector<Request> take;
        std::vector<gbsa::ServeRequest> rq;
        std::vector<int> st;
        std::vector<uint64_t> tot;
        for (;;) {
            take.clear();
            {
                std::unique_lock<std::mutex> g(mu);
                cv_req.wait(g, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;   // stopping
                // continuous batching: every request at the head of the queue that fits
                uint64_t reads = 0, bases = 0;
                while (!queue.empty()) {
                    const Request& q = queue.front();
                    if (!take.empty() && (reads + q.r.n_reads > cfg.batch_reads || bases + q.bases > cfg.batch_bases))
                        break;
                    reads += q.r.n_reads;
                    bases += q.bases;
                    take.push_back(q);
                    queue.pop_front();
                }
                ++batches;
                requests_batched += take.size();
                max_requests_per_batch = std::max<uint64_t>(max_requests_per_batch, take.size());
            }
            if (!queue.empty()) cv_req.notify_one();
            rq.clear();
            for (const Request& q : take) rq.push_back(q.r);
            st.assign(take.size(), GBSA_OK);
            tot.assign(take.size(), 0);
            try {
                gbsa::batcher_run_requests(*b, rq.data(), (uint32_t)rq.size(), st.data(), tot.data());
            } catch (const gbsa::Error& e) {
                gbsa::set_last_error(e.what());
                st.assign(take.size(), e.code);
                tot.assign(take.size(), 0);
            } catch (const std::exception& e) {
                gbsa::set_last_error(e.what());
                st.assign(take.size(), GBSA_ERR_CUDA);
                tot.assign(take.size(), 0);
            }
            {
                std::lock_guard<std::mutex> g(mu);
                for (size_t j = 0; j < take.size(); ++j) {
                    // a failed batch may not have written the offsets: report no NAMs
                    done.push_back(Done{take[j].tag, st[j], st[j] == GBSA_ERR_CAPACITY || st[j] == GBSA_OK ? tot[j] : 0});
                    --in_flight;
                }
            }
            cv_done.notify_all();
        }
    }
};

using namespace gbsa;

extern "C" {

int gbsa_server_create_ex(const gbsa_index* idx, const gbsa_map_options* opt, const gbsa_server_config* cfg,
                          gbsa_server** out) {
    try {
        *out = nullptr;
        if (!idx || !opt || !cfg) throw Error(GBSA_ERR_PARAM, "null index, options or configuration");
        if (cfg->slots == 0 || cfg->slots > 64) throw Error(GBSA_ERR_PARAM, "slots must be in [1, 64]");
        if (cfg->batch_reads == 0) throw Error(GBSA_ERR_PARAM, "batch_reads must be positive");
        std::unique_ptr<gbsa_server> s(new gbsa_server());
        s->idx = idx;
        s->device = idx->device;
        s->cfg = *cfg;
        if (s->cfg.batch_bases == 0) s->cfg.batch_bases = 500ull * cfg->batch_reads;
        GBSA_CUDA(cudaSetDevice(s->device));
        size_t free0 = 0, total = 0;
        GBSA_CUDA(cudaMemGetInfo(&free0, &total));
        s->budget = cfg->memory_budget ? cfg->memory_budget : free0 / 2;
        gbsa_batch_config bc{};
        int from_file = 0;
        if (gbsa_batch_config_default(&bc, &from_file) != GBSA_OK) throw Error(GBSA_ERR_PARAM, gbsa_last_error());
        bc.chunk_reads = std::max<uint32_t>(bc.chunk_reads, s->cfg.batch_reads);
        uint64_t used = 0;
        for (uint32_t i = 0; i < s->cfg.slots; ++i) {
            size_t f_before = 0, f_after = 0;
            GBSA_CUDA(cudaMemGetInfo(&f_before, &total));
            if (i > 0 && used + s->slot_bytes > s->budget) break;   // admission: the next slot would not fit
            gbsa_batcher* b = nullptr;
            const int rc = gbsa_batcher_create(idx, opt, &bc, s->cfg.batch_reads, s->cfg.batch_bases, &b);
            if (rc != GBSA_OK) {
                for (gbsa_batcher* x : s->slots) gbsa_batcher_free(x);
                throw Error(rc, std::string("server slot: ") + gbsa_last_error());
            }
            try {
                // every buffer of a full batch, and the slot's graph, before any request
                batcher_warm_up(*b, s->cfg.batch_reads, 40.0);
            } catch (...) {
                gbsa_batcher_free(b);
                for (gbsa_batcher* x : s->slots) gbsa_batcher_free(x);
                throw;
            }
            GBSA_CUDA(cudaMemGetInfo(&f_after, &total));
            const uint64_t took = f_before > f_after ? f_before - f_after : 0;
            s->slot_bytes = std::max<uint64_t>(s->slot_bytes, took);
            used += took;
            s->slots.push_back(b);
        }
        gbsa_server* raw = s.get();
        for (gbsa_batcher* b : s->slots) s->threads.emplace_back([raw, b] { raw->work(b); });
        *out = s.release();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

int gbsa_server_create(const gbsa_index* idx, const gbsa_map_options* opt, uint32_t workers,
                       uint32_t max_reads_per_request, uint64_t max_bases_per_request, gbsa_server** out) {
    gbsa_server_config c{};
    c.slots = workers;
    c.batch_reads = max_reads_per_request;
    c.batch_bases = max_bases_per_request;
    c.memory_budget = 0;
    if (workers == 0 || workers > 64) {
        set_last_error("workers must be in [1, 64]");
        return GBSA_ERR_PARAM;
    }
    return gbsa_server_create_ex(idx, opt, &c, out);
}

int gbsa_server_info(const gbsa_server* s, uint32_t* slots, uint64_t* slot_bytes, uint64_t* budget,
                     uint64_t* batches, uint64_t* requests) {
    gbsa_server* x = const_cast<gbsa_server*>(s);
    std::lock_guard<std::mutex> g(x->mu);
    if (slots) *slots = (uint32_t)s->slots.size();
    if (slot_bytes) *slot_bytes = s->slot_bytes;
    if (budget) *budget = s->budget;
    if (batches) *batches = s->batches;
    if (requests) *requests = s->requests_batched;
    return GBSA_OK;
}

int gbsa_server_stats(const gbsa_server* s, uint64_t* graph_launches, uint64_t* captures, uint64_t* eager_runs) {
    uint64_t g = 0, c = 0, e = 0;
    for (gbsa_batcher* b : s->slots) {
        uint64_t x = 0, y = 0, z = 0;
        gbsa_batcher_stats(b, &x, &y, &z);
        g += x;
        c += y;
        e += z;
    }
    if (graph_launches) *graph_launches = g;
    if (captures) *captures = c;
    if (eager_runs) *eager_runs = e;
    return GBSA_OK;
}

int gbsa_server_submit(gbsa_server* s, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                       uint32_t n_reads, gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets, float* frac,
                       uint8_t* rescued, uint64_t tag) {
    uint64_t bases = 0;
    for (uint32_t i = 0; i < n_reads; ++i) bases += lengths[i];
    if (n_reads > s->cfg.batch_reads || bases > s->cfg.batch_bases) {
        set_last_error("request larger than a batch slot (batch_reads / batch_bases)");
        return GBSA_ERR_CAPACITY;
    }
    {
        std::lock_guard<std::mutex> g(s->mu);
        Request q;
        q.r = ServeRequest{seqs, offsets, lengths, n_reads, nams, nam_capacity, nam_offsets, frac, rescued};
        q.bases = bases;
        q.tag = tag;
        q.t_submit = std::chrono::steady_clock::now();
        s->queue.push_back(q);
        ++s->in_flight;
    }
    s->cv_req.notify_one();
    return GBSA_OK;
}

uint32_t gbsa_server_poll(gbsa_server* s, uint64_t* tags, int* status, uint64_t* nam_totals, uint32_t cap,
                          int wait_ms) {
    std::unique_lock<std::mutex> g(s->mu);
    if (s->done.empty() && wait_ms != 0) {
        auto ready = [&] { return !s->done.empty() || s->in_flight == 0; };
        if (wait_ms < 0) s->cv_done.wait(g, ready);
        else s->cv_done.wait_for(g, std::chrono::milliseconds(wait_ms), ready);
    }
    uint32_t k = 0;
    while (k < cap && !s->done.empty()) {
        const Done d = s->done.front();
        s->done.pop_front();
        tags[k] = d.tag;
        if (status) status[k] = d.status;
        if (nam_totals) nam_totals[k] = d.nam_total;
        ++k;
    }
    return k;
}

int gbsa_server_replay(gbsa_server* s, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                       const gbsa_replay_request* reqs, uint32_t n_req, uint32_t n_bufs, gbsa_nam* const* nams,
                       uint64_t nam_cap, uint64_t* const* nam_offsets, float* const* frac, uint8_t* const* rescued,
                       uint32_t max_reads, const gbsa_nam* exp_nams, const uint64_t* exp_nam_offsets,
                       const float* exp_frac, const uint8_t* exp_rescued, double* submit_us, double* done_us,
                       int* status, uint8_t* mismatch) {
    try {
        if (n_bufs == 0) throw Error(GBSA_ERR_PARAM, "no output buffers");
        for (uint32_t i = 0; i < n_req; ++i)
            if (reqs[i].n_reads > max_reads) throw Error(GBSA_ERR_CAPACITY, "request larger than the buffers");
        using clk = std::chrono::steady_clock;
        std::mutex mu;
        std::condition_variable cv_free, cv_check;
        std::deque<uint32_t> free_bufs, to_check;   // buffer sets; requests whose results wait for a check
        for (uint32_t b = 0; b < n_bufs; ++b) free_bufs.push_back(b);
        std::vector<uint32_t> buf_of(n_req, 0);
        bool done_all = false;
        const clk::time_point t0 = clk::now() + std::chrono::milliseconds(20);
        auto us_since = [&](clk::time_point t) { return std::chrono::duration<double, std::micro>(t - t0).count(); };
        std::vector<uint64_t> totals(n_req, 0);
        // checkers: compare a finished request with the expected results, then free its buffers
        auto checker = [&] {
            for (;;) {
                uint32_t i;
                {
                    std::unique_lock<std::mutex> g(mu);
                    cv_check.wait(g, [&] { return done_all || !to_check.empty(); });
                    if (to_check.empty()) return;
                    i = to_check.front();
                    to_check.pop_front();
                }
                const uint32_t b = buf_of[i];
                bool bad = status[i] != GBSA_OK;
                if (!bad && exp_nams) {
                    const gbsa_replay_request& r = reqs[i];
                    const uint64_t a = exp_nam_offsets[r.start], e = exp_nam_offsets[r.start + r.n_reads];
                    bad = totals[i] != e - a ||
                          std::memcmp(nams[b], exp_nams + a, sizeof(gbsa_nam) * (e - a)) != 0 ||
                          std::memcmp(frac[b], exp_frac + r.start, 4ull * r.n_reads) != 0 ||
                          std::memcmp(rescued[b], exp_rescued + r.start, r.n_reads) != 0;
                    for (uint32_t j = 0; !bad && j <= r.n_reads; ++j)
                        bad = nam_offsets[b][j] != exp_nam_offsets[r.start + j] - a;
                }
                mismatch[i] = bad ? 1 : 0;
                {
                    std::lock_guard<std::mutex> g(mu);
                    free_bufs.push_back(b);
                }
                cv_free.notify_one();
            }
        };
        // completions, as they arrive (poll returns at once while nothing is in flight:
        // then the poller naps instead of spinning on the server's lock)
        std::atomic<uint32_t> arrived{0};
        std::thread poller([&] {
            std::vector<uint64_t> tags(256), tot(256);
            std::vector<int> st(256);
            while (arrived.load() < n_req) {
                const uint32_t k = gbsa_server_poll(s, tags.data(), st.data(), tot.data(), 256, 50);
                const clk::time_point now = clk::now();
                if (k == 0) {
                    std::this_thread::sleep_for(std::chrono::microseconds(50));
                    continue;
                }
                std::lock_guard<std::mutex> g(mu);
                for (uint32_t j = 0; j < k; ++j) {
                    const uint32_t i = (uint32_t)tags[j];
                    done_us[i] = us_since(now);
                    status[i] = st[j];
                    totals[i] = tot[j];
                    to_check.push_back(i);
                    arrived.fetch_add(1);
                }
                cv_check.notify_all();
            }
        });
        const unsigned n_check = std::max(2u, std::min(8u, std::thread::hardware_concurrency() / 4));
        std::vector<std::thread> checkers;
        for (unsigned c = 0; c < n_check; ++c) checkers.emplace_back(checker);
        // submissions at their times
        int rc = GBSA_OK;
        for (uint32_t i = 0; i < n_req; ++i) {
            std::this_thread::sleep_until(t0 + std::chrono::duration_cast<clk::duration>(
                                                   std::chrono::duration<double, std::micro>(reqs[i].at_us)));
            uint32_t b;
            {
                std::unique_lock<std::mutex> g(mu);
                cv_free.wait(g, [&] { return !free_bufs.empty(); });
                b = free_bufs.front();
                free_bufs.pop_front();
            }
            buf_of[i] = b;
            const gbsa_replay_request& r = reqs[i];
            submit_us[i] = us_since(clk::now());
            const int x = gbsa_server_submit(s, seqs, offsets + r.start, lengths + r.start, r.n_reads, nams[b], nam_cap,
                                             nam_offsets[b], frac[b], rescued[b], i);
            if (x != GBSA_OK) {   // not queued: record it as done at once
                std::lock_guard<std::mutex> g(mu);
                rc = x;
                done_us[i] = submit_us[i];
                status[i] = x;
                to_check.push_back(i);
                arrived.fetch_add(1);
                cv_check.notify_all();
            }
        }
        poller.join();
        {
            std::lock_guard<std::mutex> g(mu);
            done_all = true;
        }
        cv_check.notify_all();
        for (auto& t : checkers) t.join();
        if (rc != GBSA_OK) set_last_error("a request was not accepted");
        return rc;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

void gbsa_server_free(gbsa_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_req.notify_all();
    for (auto& t : s->threads) t.join();
    for (gbsa_batcher* b : s->slots) gbsa_batcher_free(b);
    delete s;
}

}  // extern "C"
