// serve.cu — the served form: a request queue in front of a pool of mappers.
//
// A server keeps the index resident and owns `workers` mappers, each with its own
// streams and device work areas sized for the largest request; those areas are the
// admission budget (a request waits in the queue until a mapper is free).  Each
// worker thread takes the next request and maps it with gbsa_map_reads on its own
// mapper, so requests overlap on the GPU and every request's NAMs equal the plain
// form's.  Callers submit host buffers (kept alive until the request completes) and
// poll for completions.  No reference counterpart: the reference maps one file per
// process (step2/main.cu:4100-4760).
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "index.h"
#include "runtime.h"

namespace {

struct Request {
    const char* seqs;
    const uint64_t* offsets;
    const uint32_t* lengths;
    uint32_t n_reads;
    gbsa_nam* nams;
    uint64_t nam_capacity;
    uint64_t* nam_offsets;
    float* frac;
    uint8_t* rescued;
    uint64_t tag;
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
    uint32_t max_reads = 0;
    std::vector<gbsa_mapper*> mappers;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_req, cv_done;
    std::deque<Request> queue;
    std::deque<Done> done;
    bool stop = false;
    uint64_t in_flight = 0;

    void work(gbsa_mapper* m) {
        cudaSetDevice(device);
        for (;;) {
            Request r;
            {
                std::unique_lock<std::mutex> g(mu);
                cv_req.wait(g, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;   // stopping
                r = queue.front();
                queue.pop_front();
            }
            const int rc = gbsa_map_reads(m, r.seqs, r.offsets, r.lengths, r.n_reads, r.nams, r.nam_capacity,
                                          r.nam_offsets, r.frac, r.rescued);
            {
                std::lock_guard<std::mutex> g(mu);
                // a failed call may not have written the offsets: report no NAMs
                done.push_back(Done{r.tag, rc, rc == GBSA_OK ? r.nam_offsets[r.n_reads] : 0});
                --in_flight;
            }
            cv_done.notify_all();
        }
    }
};

using namespace gbsa;

extern "C" {

int gbsa_server_create(const gbsa_index* idx, const gbsa_map_options* opt, uint32_t workers,
                       uint32_t max_reads_per_request, uint64_t max_bases_per_request, gbsa_server** out) {
    try {
        *out = nullptr;
        if (workers == 0 || workers > 64) throw Error(GBSA_ERR_PARAM, "workers must be in [1, 64]");
        if (max_reads_per_request == 0) throw Error(GBSA_ERR_PARAM, "max_reads_per_request must be positive");
        std::unique_ptr<gbsa_server> s(new gbsa_server());
        s->idx = idx;
        s->device = idx->device;
        s->max_reads = max_reads_per_request;
        GBSA_CUDA(cudaSetDevice(s->device));
        for (uint32_t i = 0; i < workers; ++i) {
            gbsa_mapper* m = nullptr;
            const int rc = gbsa_mapper_create(idx, opt, max_reads_per_request, max_bases_per_request, &m);
            if (rc != GBSA_OK) {
                for (gbsa_mapper* x : s->mappers) gbsa_mapper_free(x);
                throw Error(rc, std::string("mapper for the server: ") + gbsa_last_error());
            }
            s->mappers.push_back(m);
        }
        gbsa_server* raw = s.get();
        for (gbsa_mapper* m : s->mappers) s->threads.emplace_back([raw, m] { raw->work(m); });
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

int gbsa_server_submit(gbsa_server* s, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                       uint32_t n_reads, gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets, float* frac,
                       uint8_t* rescued, uint64_t tag) {
    if (n_reads > s->max_reads) {
        set_last_error("request larger than max_reads_per_request");
        return GBSA_ERR_CAPACITY;
    }
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->queue.push_back(Request{seqs, offsets, lengths, n_reads, nams, nam_capacity, nam_offsets, frac, rescued, tag});
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

void gbsa_server_free(gbsa_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_req.notify_all();
    for (auto& t : s->threads) t.join();
    for (gbsa_mapper* m : s->mappers) gbsa_mapper_free(m);
    delete s;
}

}  // extern "C"
