// batch.cu — the batched form of the read → NAM path.
//
// The plain form (gbsa_map_reads) launches a batch's kernels one by one from the host
// and sizes every launch by the batch.  The batched form replaces that launch chain
// (the reference's per-stage launches with fixed batches, step2/main.cu:4458-4597) by
// a CUDA graph captured once per set of work areas:
//
//   * the batch — its reads, their count, its work items and its output buffers —
//     lives in a device-resident descriptor (BatchDesc) that the kernels read, so one
//     graph serves every batch that fits the work areas it was captured with;
//   * seeding and lookup run as one persistent kernel (a grid of SMs x resident
//     blocks) whose warps pull work items — a single-end read, or both mates of a
//     pair — from a device queue, so reads of uneven lengths balance over the grid;
//   * the NAM phase (lane and warp merges on one stream, rescue and its sorts on a
//     second) pulls its reads from the device lists the front end fills, as in the
//     plain form, inside the same graph.
//
// The first batch on a set of work areas runs eagerly (it sizes the scan workspace
// and sets the kernels' attributes), then the sequence is captured; a batch that
// overflows a work area grows it, runs again eagerly and is captured anew.
//
// The kernel shapes (seeding + lookup variant, the lane / warp split of the NAM merge,
// the block size of the rescued reads' sort) and the host entry point's chunk size come
// from a gbsa_batch_config, by default the one the autotuner committed
// (gpu_index_test_gb300/tuned.json, read next to the library).
//
// The host entry point cuts a call into chunks (aligned to work items) that rotate over
// three sets of work areas, so that one chunk's copies overlap the others' graphs.
#include <dlfcn.h>

#include <algorithm>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "mapper.h"

namespace gbsa {
namespace {

// Sets of work areas of the host entry point: chunk k runs on set k % kLanes, so that
// kLanes chunks are in flight (one's copies overlapping the others' graphs).
constexpr uint32_t kLanes = 3;

// One set of work areas with its captured graph.
struct Lane {
    gbsa_mapper* m = nullptr;
    DeviceBuffer desc;             // BatchDesc read by the graph's kernels
    PinnedBuffer h_desc;
    cudaGraphExec_t exec = nullptr;
    uint32_t cap = 0;              // read slots of the work areas the graph runs over
    std::vector<const void*> key;  // work-area addresses baked into the graph
    // the host entry point's device inputs (items) and outputs
    DeviceBuffer items, out_nams, out_off, out_offg, out_frac, out_resc;
    PinnedBuffer h_items;
    uint64_t out_cap = 0;
    cudaEvent_t done = nullptr, in_ready = nullptr, out_free = nullptr;
    cudaEvent_t wait_ev = nullptr;   // blocking-sync event: the host thread sleeps while it waits
    double nams_per_read = 16.0;
    bool async = false;            // the last batch was launched as a graph and not yet checked
};

// Addresses a captured graph holds: any change (a work area grew) needs a new capture.
std::vector<const void*> graph_key(const gbsa_mapper& m) {
    return {m.rec.as<void>(),   m.q.as<void>(),     m.qaux.as<void>(),  m.qpos.as<void>(),      m.hits.as<void>(),
            m.nams.as<void>(),  m.slots.as<void>(), m.ovf.as<void>(),   m.lists.as<void>(),     m.ctr.as<void>(),
            m.cnt.as<void>(),   m.out_off.as<void>(), m.jobs.as<void>(), m.side_slots.as<void>(), m.lane_lists.as<void>(),
            m.long_scratch.as<void>(), m.h_status.as<void>(), (const void*)m.q_cap, (const void*)m.hit_cap,
            (const void*)m.nam_cap, (const void*)m.ovf_cap, (const void*)m.slot_bytes};
}

// Reads "key": value pairs of integers from a flat JSON object (the tuned config).
bool parse_flat_json(const std::string& text, const char* key, long long* out) {
    const std::string k = std::string("\"") + key + "\"";
    const size_t p = text.find(k);
    if (p == std::string::npos) return false;
    size_t c = text.find(':', p + k.size());
    if (c == std::string::npos) return false;
    ++c;
    while (c < text.size() && (text[c] == ' ' || text[c] == '\t' || text[c] == '\n')) ++c;
    char* end = nullptr;
    const long long v = std::strtoll(text.c_str() + c, &end, 10);
    if (end == text.c_str() + c) return false;
    *out = v;
    return true;
}

std::string library_dir() {
    Dl_info info{};
    if (dladdr(reinterpret_cast<void*>(&library_dir), &info) && info.dli_fname) {
        std::string f = info.dli_fname;
        const size_t s = f.rfind('/');
        return s == std::string::npos ? std::string(".") : f.substr(0, s);
    }
    return ".";
}

gbsa_batch_config builtin_config() {
    gbsa_batch_config c{};
    c.seed_variant = 0;
    c.lane_max_hits = kLaneMaxHitsCap;
    c.sort_variant = 0;
    c.chunk_reads = 1u << 19;
    c.rescue_block_hits = kRescueBlockHitsDefault;
    return c;
}

void check_config(const gbsa_batch_config& c) {
    if (c.seed_variant < 0 || c.seed_variant >= kSeedVariants)
        throw Error(GBSA_ERR_PARAM, "seed_variant out of range");
    if (c.lane_max_hits < 1 || c.lane_max_hits > kLaneMaxHitsCap)
        throw Error(GBSA_ERR_PARAM, "lane_max_hits must be in [1, 160]");
    if (c.sort_variant < 0 || c.sort_variant > 1) throw Error(GBSA_ERR_PARAM, "sort_variant must be 0 or 1");
    if (c.chunk_reads < 1024) throw Error(GBSA_ERR_PARAM, "chunk_reads must be at least 1024");
    if (c.lane_variant < 0 || c.lane_variant > 6) throw Error(GBSA_ERR_PARAM, "lane_variant must be 0 to 6");
    if (c.warp_variant < 0 || c.warp_variant > 4) throw Error(GBSA_ERR_PARAM, "warp_variant must be 0 to 4");
}

// The committed autotuner result next to the library (gpu_index_test_gb300/tuned.json),
// else the built-in shape (the plain form's).
gbsa_batch_config tuned_config(int* from_file) {
    gbsa_batch_config c = builtin_config();
    *from_file = 0;
    std::ifstream f(library_dir() + "/tuned.json");
    if (!f) return c;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string t = ss.str();
    long long v = 0;
    gbsa_batch_config x = c;
    bool ok = true;
    ok &= parse_flat_json(t, "seed_variant", &v);
    x.seed_variant = (int32_t)v;
    ok &= parse_flat_json(t, "lane_max_hits", &v);
    x.lane_max_hits = (uint32_t)v;
    ok &= parse_flat_json(t, "sort_variant", &v);
    x.sort_variant = (int32_t)v;
    ok &= parse_flat_json(t, "chunk_reads", &v);
    x.chunk_reads = (uint32_t)v;
    // the merge kernels' register budgets (a file written before they were tuned lacks them)
    x.lane_variant = parse_flat_json(t, "lane_variant", &v) ? (int32_t)v : 0;
    x.warp_variant = parse_flat_json(t, "warp_variant", &v) ? (int32_t)v : 0;
    x.rescue_block_hits = parse_flat_json(t, "rescue_block_hits", &v) ? (uint32_t)v : kRescueBlockHitsDefault;
    if (!ok) return c;
    try {
        check_config(x);
    } catch (const Error&) {
        return c;
    }
    *from_file = 1;
    return x;
}

}  // namespace
}  // namespace gbsa

struct gbsa_batcher {
    const gbsa_index* idx = nullptr;
    gbsa_map_options opt{};
    gbsa_batch_config cfg{};
    uint32_t max_reads = 0;
    uint64_t max_bases = 0;
    gbsa::Lane lanes[gbsa::kLanes];
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t caller_ev = nullptr;
    uint64_t graph_launches = 0, captures = 0, eager_runs = 0;
    bool profile = false;
};

namespace gbsa {
namespace {

void lane_init(gbsa_batcher& b, Lane& L) {
    if (L.m) return;
    gbsa_mapper* m = nullptr;
    const int rc = gbsa_mapper_create(b.idx, &b.opt, b.max_reads, b.max_bases, &m);
    if (rc != GBSA_OK) throw Error(rc, std::string("batcher work areas: ") + gbsa_last_error());
    L.m = m;
    L.m->cfg.lane_max_hits = b.cfg.lane_max_hits;
    L.m->cfg.sort_variant = b.cfg.sort_variant;
    L.m->cfg.lane_variant = b.cfg.lane_variant;
    L.m->cfg.warp_variant = b.cfg.warp_variant;
    L.m->cfg.rescue_block_hits = b.cfg.rescue_block_hits;
    if (b.profile && gbsa_mapper_set_profile(L.m, 1) != GBSA_OK) throw Error(GBSA_ERR_CUDA, gbsa_last_error());
    L.desc.resize(sizeof(BatchDesc));
    L.h_desc.resize(sizeof(BatchDesc));
    for (cudaEvent_t* e : {&L.done, &L.in_ready, &L.out_free})
        GBSA_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    GBSA_CUDA(cudaEventCreateWithFlags(&L.wait_ev, cudaEventDisableTiming | cudaEventBlockingSync));
}

// Waits for the work queued on st so far without spinning: a server runs a host thread per
// slot, and threads spinning in cudaStreamSynchronize took the cores that submit requests.
void wait_blocking(Lane& L, cudaStream_t st) {
    GBSA_CUDA(cudaEventRecord(L.wait_ev, st));
    GBSA_CUDA(cudaEventSynchronize(L.wait_ev));
}

void drop_graph(Lane& L) {
    if (L.exec) cudaGraphExecDestroy(L.exec);
    L.exec = nullptr;
    L.key.clear();
}

// Work areas for n reads; a growth invalidates the graph.
void lane_reserve(gbsa_batcher& b, Lane& L, uint32_t n) {
    if (n <= L.cap && L.cap) return;
    const uint32_t cap = std::max<uint32_t>(n, L.cap ? L.cap : 1024);
    mapper_reserve(*L.m, cap, std::max<uint64_t>(b.max_bases, 64ull * cap));
    L.cap = cap;
    drop_graph(L);
}

void put_desc(Lane& L, const BatchDesc& d) {
    std::memcpy(L.h_desc.as<void>(), &d, sizeof d);
    GBSA_CUDA(cudaMemcpyAsync(L.desc.as<void>(), L.h_desc.as<void>(), sizeof d, cudaMemcpyHostToDevice, L.m->st));
}

// The batch sequence on the lane's stream, eagerly (sync) until its work areas fit,
// then captured as a graph for the batches that follow.  Returns the NAM total.
uint64_t run_eager(gbsa_batcher& b, Lane& L, const BatchDesc& d) {
    gbsa_mapper& m = *L.m;
    const BatchMode bm{L.desc.as<BatchDesc>(), b.cfg.seed_variant, L.cap};
    for (int attempt = 0; attempt < 8; ++attempt) {
        put_desc(L, d);
        enqueue_batch(m, nullptr, nullptr, nullptr, L.cap, false, m.st, nullptr, nullptr, &bm);
        GBSA_CUDA(cudaStreamSynchronize(m.st));
        ++b.eager_runs;
        if (!check_batch(m, false)) {
            drop_graph(L);
            continue;
        }
        const uint64_t total = batch_total(m);
        // capture the same sequence for the next batches (the eager run sized the scan
        // workspace and set the kernels' attributes, so nothing allocates while capturing)
        drop_graph(L);
        cudaGraph_t g = nullptr;
        GBSA_CUDA(cudaStreamBeginCapture(m.st, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_batch(m, nullptr, nullptr, nullptr, L.cap, false, m.st, nullptr, nullptr, &bm);
        } catch (...) {
            cudaStreamEndCapture(m.st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        GBSA_CUDA(cudaStreamEndCapture(m.st, &g));
        const cudaError_t e = cudaGraphInstantiate(&L.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            L.exec = nullptr;
            throw Error(GBSA_ERR_CUDA, std::string("cudaGraphInstantiate failed: ") + cudaGetErrorString(e));
        }
        L.key = graph_key(m);
        ++b.captures;
        return total;
    }
    throw Error(GBSA_ERR_DEVICE_STATUS, "work areas kept overflowing");
}

// Launches the lane's graph for batch d without waiting (the graph must be current).
void launch_graph(gbsa_batcher& b, Lane& L, const BatchDesc& d) {
    put_desc(L, d);
    GBSA_CUDA(cudaGraphLaunch(L.exec, L.m->st));
    ++b.graph_launches;
    L.async = true;
}

bool graph_ready(const Lane& L) { return L.exec && L.key == graph_key(*L.m); }

// Runs batch d on the lane and waits for it: the graph when one is current, else (or
// when the graph's batch overflowed a work area) the eager path.  Returns the total.
uint64_t run_sync(gbsa_batcher& b, Lane& L, const BatchDesc& d) {
    if (graph_ready(L)) {
        launch_graph(b, L, d);
        wait_blocking(L, L.m->st);
        L.async = false;
        if (check_batch(*L.m, false)) return batch_total(*L.m);
        drop_graph(L);
    }
    return run_eager(b, L, d);
}

}  // namespace

void batcher_warm_up(gbsa_batcher& b, uint32_t max_reads, double nams_per_read) {
    Lane& L = b.lanes[0];
    lane_init(b, L);
    lane_reserve(b, L, max_reads);
    // every buffer a batch of max_reads reads needs, so that serving allocates nothing
    // (cudaFree and cudaFreeHost wait for the whole device, other slots' work included)
    L.h_items.resize(12ull * (max_reads + 1));
    L.h_desc.resize(sizeof(BatchDesc) + 8ull * (max_reads + 1));
    L.out_off.resize(8ull * (max_reads + 1));
    L.out_frac.resize(4ull * (max_reads + 1));
    L.out_resc.resize(max_reads + 1);
    L.nams_per_read = std::max(L.nams_per_read, nams_per_read);
    const uint64_t want = (uint64_t)(L.nams_per_read * 1.25 * max_reads) + 1024;
    if (L.out_cap < want) {
        L.out_nams.release();
        L.out_nams.resize(sizeof(gbsa_nam) * want);
        L.out_cap = want;
    }
    // rescue scratch for the heavy rescued reads of a full batch (repeat-rich genomes use
    // about 1 KB per read of the batch; a batch that outgrows it grows it, which frees
    // device memory and so waits for every other slot's work)
    const uint64_t ovf_want = std::max<uint64_t>(64ull << 20, 4096ull * max_reads);
    if (L.m->ovf_cap < ovf_want) {
        L.m->ovf.release();
        L.m->ovf.resize(ovf_want);
        L.m->ovf_cap = ovf_want;
    }
    // one batch of pseudo-random 150 bp reads runs eagerly and captures the graph
    const uint32_t n = std::min<uint32_t>(1024, max_reads), len = 150;
    std::vector<char> seq((size_t)n * len);
    uint64_t x = 0x9E3779B97F4A7C15ULL;
    for (char& c : seq) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        c = "ACGT"[x & 3];
    }
    std::vector<uint64_t> offs(n), noff(n + 1);
    std::vector<uint32_t> lens(n, len);
    for (uint32_t i = 0; i < n; ++i) offs[i] = (uint64_t)i * len;
    std::vector<gbsa_nam> nams(64ull * n);
    ServeRequest r{seq.data(), offs.data(), lens.data(), n, nams.data(), nams.size(), noff.data(), nullptr, nullptr};
    int st = 0;
    uint64_t tot = 0;
    batcher_run_requests(b, &r, 1, &st, &tot);
}

// Copies the reads of k requests to the mapper's device inputs, one region per request
// in request order: a request whose reads lie in one span of its buffer (gaps of at most
// an eighth: the usual case, a request's reads back to back) is copied from there in one
// transfer;
// the others are gathered into pinned staging first.  Offsets are rebased to the device
// layout.  (One span over all requests would be a host gather whenever the requests'
// buffers lie apart: at saturation that gather took 5 ms per batch.)
void stage_requests(gbsa_mapper& m, const ServeRequest* rq, uint32_t k, const uint32_t* first, uint32_t n,
                    cudaStream_t st) {
    struct Part {
        uint64_t lo = 0, span = 0, total = 0, dst = 0, gather_at = 0;
        bool direct = true;
    };
    // (on the slot's own thread: the host pool runs one job at a time, and slots would
    // queue behind one another for work this small)
    std::vector<Part> parts(k);
    for (uint32_t j = 0; j < k; ++j) {
        const ServeRequest& r = rq[j];
        uint64_t lo = UINT64_MAX, hi = 0, tot = 0;
        for (uint32_t i = 0; i < r.n_reads; ++i) {
            lo = std::min<uint64_t>(lo, r.offsets[i]);
            hi = std::max<uint64_t>(hi, r.offsets[i] + r.lengths[i]);
            tot += r.lengths[i];
        }
        Part& P = parts[j];
        P.lo = r.n_reads ? lo : 0;
        P.span = r.n_reads ? hi - lo : 0;
        P.total = tot;
        P.direct = P.span <= tot + (tot >> 3) + 4096;   // gaps small enough to copy along
    }
    uint64_t dst = 0, gathered = 0;
    for (Part& P : parts) {
        P.dst = dst;
        dst = (dst + (P.direct ? P.span : P.total) + 15) & ~15ull;
        if (!P.direct) {
            P.gather_at = gathered;
            gathered += P.total;
        }
    }
    mapper_reserve(m, n, dst);
    m.seqs.resize(dst + 64);
    m.offs.resize(8ull * (n + 1));
    m.lens.resize(4ull * (n + 1));
    m.h_meta.resize(12ull * (n + 1));
    if (gathered) m.h_seqs.resize(gathered + 1);
    uint64_t* ho = m.h_meta.as<uint64_t>();
    uint32_t* hl = reinterpret_cast<uint32_t*>(ho + n + 1);
    char* hs = gathered ? m.h_seqs.as<char>() : nullptr;
    for (uint32_t j = 0; j < k; ++j) {
        const ServeRequest& r = rq[j];
        const Part& P = parts[j];
        uint64_t acc = 0;
        for (uint32_t i = 0; i < r.n_reads; ++i) {
            const uint32_t x = first[j] + i;
            hl[x] = r.lengths[i];
            if (P.direct) {
                ho[x] = P.dst + r.offsets[i] - P.lo;
            } else {
                std::memcpy(hs + P.gather_at + acc, r.seqs + r.offsets[i], r.lengths[i]);
                ho[x] = P.dst + acc;
                acc += r.lengths[i];
            }
        }
    }
    uint8_t* d = m.seqs.as<uint8_t>();
    for (uint32_t j = 0; j < k; ++j) {
        const Part& P = parts[j];
        if (P.direct && P.span)
            GBSA_CUDA(cudaMemcpyAsync(d + P.dst, rq[j].seqs + P.lo, P.span, cudaMemcpyHostToDevice, st));
        else if (!P.direct && P.total)
            GBSA_CUDA(cudaMemcpyAsync(d + P.dst, hs + P.gather_at, P.total, cudaMemcpyHostToDevice, st));
    }
    GBSA_CUDA(cudaMemcpyAsync(m.offs.as<void>(), ho, 8ull * n, cudaMemcpyHostToDevice, st));
    GBSA_CUDA(cudaMemcpyAsync(m.lens.as<void>(), hl, 4ull * n, cudaMemcpyHostToDevice, st));
}

void batcher_run_requests(gbsa_batcher& b, const ServeRequest* rq, uint32_t k, int* status, uint64_t* totals) {
    Lane& L = b.lanes[0];
    lane_init(b, L);
    uint32_t n = 0;
    for (uint32_t j = 0; j < k; ++j) n += rq[j].n_reads;
    if (n == 0) {
        for (uint32_t j = 0; j < k; ++j) {
            rq[j].nam_offsets[0] = 0;
            status[j] = GBSA_OK;
            totals[j] = 0;
        }
        return;
    }
    GBSA_CUDA(cudaEventSynchronize(L.done));
    lane_reserve(b, L, n);
    std::vector<uint32_t> first(k + 1, 0);
    for (uint32_t j = 0; j < k; ++j) first[j + 1] = first[j] + rq[j].n_reads;
    stage_requests(*L.m, rq, k, first.data(), n, b.copy_in);
    GBSA_CUDA(cudaEventRecord(L.in_ready, b.copy_in));
    GBSA_CUDA(cudaStreamWaitEvent(L.m->st, L.in_ready, 0));
    const uint64_t want = (uint64_t)(L.nams_per_read * 1.25 * n) + 1024;
    if (L.out_cap < want) {
        L.out_nams.release();
        L.out_nams.resize(sizeof(gbsa_nam) * want);
        L.out_cap = want;
    }
    L.out_off.resize(8ull * (n + 1));
    L.out_frac.resize(4ull * (n + 1));
    L.out_resc.resize(n + 1);
    BatchDesc d{};
    d.seqs = L.m->seqs.as<uint8_t>();
    d.offs = L.m->offs.as<uint64_t>();
    d.lens = L.m->lens.as<uint32_t>();
    d.items = nullptr;
    d.n_reads = n;
    d.n_items = n;
    d.out = L.out_nams.as<gbsa_nam>();
    d.out_cap = L.out_cap;
    d.out_off = L.out_off.as<uint64_t>();
    d.frac = L.out_frac.as<float>();
    d.rescued = L.out_resc.as<uint8_t>();
    uint64_t total = run_sync(b, L, d);
    if (total > L.out_cap) {   // more NAMs than the estimate: again with room for them
        L.out_nams.release();
        L.out_nams.resize(sizeof(gbsa_nam) * (total + 1024));
        L.out_cap = total + 1024;
        d.out = L.out_nams.as<gbsa_nam>();
        d.out_cap = L.out_cap;
        total = run_sync(b, L, d);
    }
    L.nams_per_read = std::max(L.nams_per_read, (double)total / n);
    cudaStream_t st = L.m->st;
    L.h_desc.resize(sizeof(BatchDesc) + 8ull * (n + 1));
    uint64_t* h_off = reinterpret_cast<uint64_t*>(L.h_desc.as<uint8_t>() + sizeof(BatchDesc));
    GBSA_CUDA(cudaMemcpyAsync(h_off, L.out_off.as<void>(), 8ull * (n + 1), cudaMemcpyDeviceToHost, st));
    wait_blocking(L, st);
    for (uint32_t j = 0; j < k; ++j) {
        const ServeRequest& r = rq[j];
        const uint64_t a = h_off[first[j]], e = h_off[first[j + 1]];
        for (uint32_t i = 0; i <= r.n_reads; ++i) r.nam_offsets[i] = h_off[first[j] + i] - a;
        totals[j] = e - a;
        status[j] = e - a <= r.nam_capacity ? GBSA_OK : GBSA_ERR_CAPACITY;
        if (status[j] == GBSA_OK && e > a)
            GBSA_CUDA(cudaMemcpyAsync(r.nams, L.out_nams.as<gbsa_nam>() + a, sizeof(gbsa_nam) * (e - a),
                                      cudaMemcpyDeviceToHost, st));
        if (r.frac && r.n_reads)
            GBSA_CUDA(cudaMemcpyAsync(r.frac, L.out_frac.as<float>() + first[j], 4ull * r.n_reads,
                                      cudaMemcpyDeviceToHost, st));
        if (r.rescued && r.n_reads)
            GBSA_CUDA(cudaMemcpyAsync(r.rescued, L.out_resc.as<uint8_t>() + first[j], r.n_reads,
                                      cudaMemcpyDeviceToHost, st));
    }
    wait_blocking(L, st);
    GBSA_CUDA(cudaEventRecord(L.done, st));
}

}  // namespace gbsa

using namespace gbsa;

extern "C" {

int gbsa_batch_config_default(gbsa_batch_config* out, int* from_file) {
    try {
        int f = 0;
        *out = tuned_config(&f);
        if (from_file) *from_file = f;
        return GBSA_OK;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_PARAM;
    }
}

int gbsa_batcher_create(const gbsa_index* idx, const gbsa_map_options* opt, const gbsa_batch_config* cfg,
                        uint32_t max_reads, uint64_t max_bases, gbsa_batcher** out) {
    try {
        *out = nullptr;
        if (!idx || !opt) throw Error(GBSA_ERR_PARAM, "null index or options");
        std::unique_ptr<gbsa_batcher> b(new gbsa_batcher());
        b->idx = idx;
        b->opt = *opt;
        int from_file = 0;
        b->cfg = cfg ? *cfg : tuned_config(&from_file);
        check_config(b->cfg);
        b->max_reads = std::max<uint32_t>(max_reads, 1024);
        b->max_bases = std::max<uint64_t>(max_bases, 64ull * b->max_reads);
        GBSA_CUDA(cudaSetDevice(idx->device));
        GBSA_CUDA(cudaStreamCreateWithFlags(&b->copy_in, cudaStreamNonBlocking));
        GBSA_CUDA(cudaStreamCreateWithFlags(&b->copy_out, cudaStreamNonBlocking));
        GBSA_CUDA(cudaEventCreateWithFlags(&b->caller_ev, cudaEventDisableTiming));
        lane_init(*b, b->lanes[0]);
        lane_reserve(*b, b->lanes[0], b->max_reads);
        *out = b.release();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

void gbsa_batcher_free(gbsa_batcher* b) {
    if (!b) return;
    for (Lane& L : b->lanes) {
        if (L.m) {
            cudaStreamSynchronize(L.m->st);
            cudaStreamSynchronize(L.m->side);
        }
        drop_graph(L);
        for (cudaEvent_t e : {L.done, L.in_ready, L.out_free, L.wait_ev})
            if (e) cudaEventDestroy(e);
        gbsa_mapper_free(L.m);
        L.m = nullptr;
    }
    for (cudaStream_t s : {b->copy_in, b->copy_out})
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    if (b->caller_ev) cudaEventDestroy(b->caller_ev);
    delete b;
}

int gbsa_batcher_get_config(const gbsa_batcher* b, gbsa_batch_config* out) {
    *out = b->cfg;
    return GBSA_OK;
}

int gbsa_batcher_stats(const gbsa_batcher* b, uint64_t* graph_launches, uint64_t* captures, uint64_t* eager_runs) {
    if (graph_launches) *graph_launches = b->graph_launches;
    if (captures) *captures = b->captures;
    if (eager_runs) *eager_runs = b->eager_runs;
    return GBSA_OK;
}

int gbsa_batcher_set_profile(gbsa_batcher* b, int on) {
    try {
        b->profile = on != 0;
        for (Lane& L : b->lanes) {
            if (!L.m) continue;
            GBSA_CUDA(cudaStreamSynchronize(L.m->st));
            GBSA_CUDA(cudaStreamSynchronize(L.m->side));
            if (gbsa_mapper_set_profile(L.m, on) != GBSA_OK) throw Error(GBSA_ERR_CUDA, gbsa_last_error());
            drop_graph(L);   // the graph is captured anew, with (or without) the stage events
        }
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

int gbsa_batcher_stage_ms(const gbsa_batcher* b, float* ms, int n) {
    if (b->lanes[0].m) return gbsa_mapper_stage_ms(b->lanes[0].m, ms, n);
    for (int i = 0; i < n; ++i) ms[i] = 0.0f;
    return GBSA_OK;
}

int gbsa_batcher_map_device(gbsa_batcher* b, const char* d_seqs, const uint64_t* d_offsets, const uint32_t* d_lengths,
                            uint32_t n_reads, const uint32_t* d_items, uint32_t n_items, gbsa_nam* d_nams,
                            uint64_t nam_capacity, uint64_t* d_nam_offsets, float* d_frac, uint8_t* d_rescued,
                            uint64_t* nam_total, void* stream) {
    try {
        if (d_items && n_items == 0 && n_reads) throw Error(GBSA_ERR_PARAM, "items given but n_items is 0");
        GBSA_CUDA(cudaSetDevice(b->idx->device));
        Lane& L = b->lanes[0];
        lane_init(*b, L);
        lane_reserve(*b, L, n_reads);
        cudaStream_t st = (cudaStream_t)stream;
        // the batch runs on the lane's streams, after the caller's stream's work so far
        GBSA_CUDA(cudaEventRecord(b->caller_ev, st));
        GBSA_CUDA(cudaStreamWaitEvent(L.m->st, b->caller_ev, 0));
        BatchDesc d{};
        d.seqs = reinterpret_cast<const uint8_t*>(d_seqs);
        d.offs = d_offsets;
        d.lens = d_lengths;
        d.items = d_items;
        d.n_reads = n_reads;
        d.n_items = d_items ? n_items : n_reads;
        d.out = d_nams;
        d.out_cap = nam_capacity;
        d.out_off = d_nam_offsets;
        d.frac = d_frac;
        d.rescued = d_rescued;
        const uint64_t total = run_sync(*b, L, d);
        GBSA_CUDA(cudaEventRecord(L.done, L.m->st));
        GBSA_CUDA(cudaStreamWaitEvent(st, L.done, 0));
        if (nam_total) *nam_total = total;
        if (total > nam_capacity) throw Error(GBSA_ERR_CAPACITY, "NAM capacity too small");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

int gbsa_batcher_map(gbsa_batcher* b, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                     uint32_t n_reads, const uint32_t* items, uint32_t n_items, gbsa_nam* nams, uint64_t nam_capacity,
                     uint64_t* nam_offsets, float* frac, uint8_t* rescued) {
    try {
        GBSA_CUDA(cudaSetDevice(b->idx->device));
        if (items && (n_items == 0 || items[0] != 0 || items[n_items] != n_reads))
            throw Error(GBSA_ERR_PARAM, "items must start at 0 and end at n_reads");
        if (items)
            for (uint32_t i = 0; i < n_items; ++i)
                if (items[i + 1] < items[i]) throw Error(GBSA_ERR_PARAM, "items must not decrease");
        const uint32_t ni = items ? n_items : n_reads;
        auto item_start = [&](uint32_t i) { return items ? items[i] : i; };
        // chunks of about chunk_reads reads, cut at item boundaries
        std::vector<uint32_t> cuts{0};   // item indices
        for (uint32_t i = 0; i < ni;) {
            const uint32_t r0 = item_start(i);
            uint32_t j = i + 1;
            while (j < ni && item_start(j) - r0 < b->cfg.chunk_reads) ++j;
            cuts.push_back(j);
            i = j;
        }
        const uint32_t n_chunks = (uint32_t)cuts.size() - 1;
        for (uint32_t i = 1; i < std::min<uint32_t>(n_chunks, kLanes); ++i) lane_init(*b, b->lanes[i]);
        uint64_t done_nams = 0;
        // queues chunk k on lane k % kLanes: its reads (and items) in, its batch (the graph
        // when one is current)
        auto enqueue = [&](uint32_t k) {
            Lane& L = b->lanes[k % kLanes];
            const uint32_t i0 = cuts[k], i1 = cuts[k + 1];
            const uint32_t r0 = item_start(i0), r1 = i1 < ni ? item_start(i1) : n_reads;
            const uint32_t n = r1 - r0;
            GBSA_CUDA(cudaEventSynchronize(L.done));
            lane_reserve(*b, L, std::max(n, std::min(b->cfg.chunk_reads + 64, b->max_reads)));
            stage_reads(*L.m, seqs, offsets + r0, lengths + r0, n, b->copy_in);
            if (items) {
                L.h_items.resize(4ull * (i1 - i0 + 1));
                uint32_t* hi = L.h_items.as<uint32_t>();
                for (uint32_t i = i0; i < i1; ++i) hi[i - i0] = items[i] - r0;
                hi[i1 - i0] = n;
                L.items.resize(4ull * (i1 - i0 + 1));
                GBSA_CUDA(cudaMemcpyAsync(L.items.as<void>(), hi, 4ull * (i1 - i0 + 1), cudaMemcpyHostToDevice,
                                          b->copy_in));
            }
            GBSA_CUDA(cudaEventRecord(L.in_ready, b->copy_in));
            GBSA_CUDA(cudaStreamWaitEvent(L.m->st, L.in_ready, 0));
            // the lane's outputs are rewritten once the copies of its previous chunk's
            // results have ended (a wait on the device; the host goes on staging)
            GBSA_CUDA(cudaStreamWaitEvent(L.m->st, L.out_free, 0));
            const uint64_t want = (uint64_t)(L.nams_per_read * 1.25 * n) + 1024;
            if (L.out_cap < want) {
                GBSA_CUDA(cudaEventSynchronize(L.out_free));   // the old buffer is still being read
                L.out_nams.release();
                L.out_nams.resize(sizeof(gbsa_nam) * want);
                L.out_cap = want;
            }
            L.out_off.resize(8ull * (n + 1));
            L.out_offg.resize(8ull * (n + 1));
            L.out_frac.resize(4ull * (n + 1));
            L.out_resc.resize(n + 1);
            BatchDesc d{};
            d.seqs = L.m->seqs.as<uint8_t>();
            d.offs = L.m->offs.as<uint64_t>();
            d.lens = L.m->lens.as<uint32_t>();
            d.items = items ? L.items.as<uint32_t>() : nullptr;
            d.n_reads = n;
            d.n_items = i1 - i0;
            d.out = L.out_nams.as<gbsa_nam>();
            d.out_cap = L.out_cap;
            d.out_off = L.out_off.as<uint64_t>();
            d.frac = L.out_frac.as<float>();
            d.rescued = L.out_resc.as<uint8_t>();
            if (graph_ready(L)) launch_graph(*b, L, d);
            else {
                run_eager(*b, L, d);
                L.async = false;
            }
            GBSA_CUDA(cudaEventRecord(L.done, L.m->st));
            return d;
        };
        std::vector<BatchDesc> descs(n_chunks);
        // waits for chunk k and copies its results out
        auto finish = [&](uint32_t k) {
            Lane& L = b->lanes[k % kLanes];
            const uint32_t i0 = cuts[k], i1 = cuts[k + 1];
            const uint32_t r0 = item_start(i0), r1 = i1 < ni ? item_start(i1) : n_reads;
            const uint32_t n = r1 - r0;
            GBSA_CUDA(cudaEventSynchronize(L.done));
            uint64_t total = 0;
            if (L.async) {
                L.async = false;
                if (check_batch(*L.m, false)) {
                    total = batch_total(*L.m);
                } else {   // a work area grew: again, eagerly
                    drop_graph(L);
                    total = run_eager(*b, L, descs[k]);
                }
            } else {
                total = batch_total(*L.m);
            }
            if (total > L.out_cap) {   // more NAMs than the estimate: again with room for them
                L.out_nams.release();
                L.out_nams.resize(sizeof(gbsa_nam) * (total + 1024));
                L.out_cap = total + 1024;
                descs[k].out = L.out_nams.as<gbsa_nam>();
                descs[k].out_cap = L.out_cap;
                total = run_sync(*b, L, descs[k]);
            }
            GBSA_CUDA(cudaEventRecord(L.done, L.m->st));
            L.nams_per_read = std::max(L.nams_per_read, (double)total / std::max<uint32_t>(n, 1));
            GBSA_CUDA(cudaStreamWaitEvent(b->copy_out, L.done, 0));
            launch_offsets_add(L.out_off.as<uint64_t>(), L.out_offg.as<uint64_t>(), n, done_nams, b->copy_out);
            GBSA_CUDA(cudaMemcpyAsync(nam_offsets + r0, L.out_offg.as<void>(), 8ull * n, cudaMemcpyDeviceToHost,
                                      b->copy_out));
            if (frac)
                GBSA_CUDA(cudaMemcpyAsync(frac + r0, L.out_frac.as<void>(), 4ull * n, cudaMemcpyDeviceToHost,
                                          b->copy_out));
            if (rescued)
                GBSA_CUDA(cudaMemcpyAsync(rescued + r0, L.out_resc.as<void>(), n, cudaMemcpyDeviceToHost, b->copy_out));
            if (done_nams + total <= nam_capacity && total)
                GBSA_CUDA(cudaMemcpyAsync(nams + done_nams, L.out_nams.as<void>(), sizeof(gbsa_nam) * total,
                                          cudaMemcpyDeviceToHost, b->copy_out));
            GBSA_CUDA(cudaEventRecord(L.out_free, b->copy_out));
            done_nams += total;
        };
        struct Drain {
            gbsa_batcher* b;
            bool armed = true;
            ~Drain() {
                if (!armed) return;
                for (Lane& L : b->lanes)
                    if (L.m) {
                        cudaStreamSynchronize(L.m->st);
                        cudaStreamSynchronize(L.m->side);
                        L.async = false;
                    }
                cudaStreamSynchronize(b->copy_in);
                cudaStreamSynchronize(b->copy_out);
            }
        } drain{b};
        uint32_t queued = 0;
        for (uint32_t k = 0; k < n_chunks; ++k) {
            while (queued < n_chunks && queued < k + kLanes) {
                descs[queued] = enqueue(queued);
                ++queued;
            }
            finish(k);
        }
        GBSA_CUDA(cudaStreamSynchronize(b->copy_out));
        drain.armed = false;
        nam_offsets[n_reads] = done_nams;
        if (n_reads == 0) nam_offsets[0] = 0;
        if (done_nams > nam_capacity) throw Error(GBSA_ERR_CAPACITY, "NAM capacity too small");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

}  // extern "C"
