// capi.cu — the C-ABI (include/gbsa.h): parameters, index handle, mapper and the
// host <-> device plumbing around the kernels.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "mapper.h"
#include "prims.cuh"

namespace gbsa {

std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_last_error;

void set_last_error(const std::string& msg) { t_last_error = msg; }

namespace {

// Process-wide pool for host_parallel_for: workers sleep on a condition variable;
// a job is a function and a range handed out in chunks through an atomic counter.
class HostPool {
public:
    static HostPool& get() {
        static HostPool pool;
        return pool;
    }
    void run(size_t n, const std::function<void(size_t, size_t)>& fn, size_t min_chunk = kMinChunk) {
        std::lock_guard<std::mutex> one_job(job_mu_);   // one job at a time
        const size_t chunk = std::max<size_t>(min_chunk, n / (4 * (workers_.size() + 1)) + 1);
        {
            std::lock_guard<std::mutex> g(mu_);
            fn_ = &fn;
            n_ = n;
            chunk_ = chunk;
            next_.store(0);
            active_ = workers_.size();
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> g(mu_);
        done_cv_.wait(g, [&] { return active_ == 0; });
        fn_ = nullptr;
    }
    static constexpr size_t kMinChunk = 1 << 16;

private:
    HostPool() {
        const unsigned hw = std::thread::hardware_concurrency();
        const unsigned nw = std::min(15u, hw > 1 ? hw - 1 : 0u);
        for (unsigned i = 0; i < nw; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }
    void work() {
        for (;;) {
            const size_t b = next_.fetch_add(chunk_);
            if (b >= n_) return;
            (*fn_)(b, std::min(n_, b + chunk_));
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            work();
            std::lock_guard<std::mutex> g(mu_);
            if (--active_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex mu_, job_mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t, size_t)>* fn_ = nullptr;
    size_t n_ = 0, chunk_ = 1, active_ = 0;
    std::atomic<size_t> next_{0};
    uint64_t gen_ = 0;
    bool stop_ = false;
};

}  // namespace

void host_parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn) {
    if (n <= HostPool::kMinChunk) {
        if (n) fn(0, n);
        return;
    }
    HostPool::get().run(n, fn);
}

void host_parallel_tasks(size_t n, const std::function<void(size_t)>& fn) {
    if (n <= 1) {
        if (n) fn(0);
        return;
    }
    HostPool::get().run(n, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) fn(i);
    }, 1);
}

int device_sm_count() {
    static std::mutex mu;
    static std::vector<int> cache;
    int dev = 0;
    GBSA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (!cache[dev]) GBSA_CUDA(cudaDeviceGetAttribute(&cache[dev], cudaDevAttrMultiProcessorCount, dev));
    return cache[dev];
}

template <class F>
static int guarded(F&& f) {
    try {
        f();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return GBSA_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

static void require_device() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error(GBSA_ERR_NO_DEVICE, "no CUDA device visible");
    }
}

// ---- IndexParameters (step2/indexparameters.{hpp,cpp}) -------------------------------
bool params_valid(const gbsa_params& p) {
    if (p.k <= 7 || p.k > 32) return false;                 // indexparameters.hpp:25-27
    if (p.s > p.k || p.s < 1) return false;                 // :28-30
    if ((p.k - p.s) % 2 != 0) return false;                 // :31-33
    if (p.max_dist > 255 || p.max_dist < 0) return false;   // :62-64 (negative: no seed fits)
    if (p.w_min > p.w_max) return false;                    // :65-67
    return true;
}

static void make_params(uint64_t r, int k, int s, int l, int u, int q, int max_dist, gbsa_params* out) {
    gbsa_params p{};
    p.canonical_read_length = (int32_t)r;
    p.k = k;
    p.s = s;
    p.t_syncmer = (k - s) / 2 + 1;
    p.l = l;
    p.u = u;
    p.q = (uint64_t)(int64_t)q;
    p.max_dist = max_dist;
    if (k - s + 1 <= 0) throw Error(GBSA_ERR_PARAM, "s is larger than k");
    p.w_min = (uint32_t)std::max(0, k / (k - s + 1) + l);   // indexparameters.hpp:83
    p.w_max = (uint32_t)(k / (k - s + 1) + u);
    if (!params_valid(p)) throw Error(GBSA_ERR_PARAM, "invalid index parameters (k in [8,32], s <= k, k-s even, "
                                                      "max_dist <= 255, w_min <= w_max)");
    *out = p;
}

int pick_bits_host(const gbsa_params& p, uint64_t size) {   // step2/index.cu:137-141
    const uint64_t est = size / (uint64_t)(p.k - p.s + 1);
    if (est == 0) return 8;
    return std::clamp((int)std::log2((double)est) - 1, 8, 31);
}

void build_index(gbsa_index& ix, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
                 uint32_t n_contigs, float f);

// ---- .sti format version 2 (step2/index.cu:73-134, step2/io.hpp:11-26) --------------
static void write_sti(const gbsa_index& ix, const std::vector<gbsa_ref_randstrobe>& rs,
                      const std::vector<uint64_t>& starts, const char* path) {
    std::ofstream os(path, std::ios::binary);
    if (!os) throw Error(GBSA_ERR_INDEX_FILE, std::string(path) + ": cannot open for writing");
    auto w32 = [&](int32_t v) { os.write(reinterpret_cast<const char*>(&v), 4); };
    auto w64 = [&](uint64_t v) { os.write(reinterpret_cast<const char*>(&v), 8); };
    os.write("STI\1", 4);
    w32(2);
    w64(8);
    const char reserved[8] = {0};
    os.write(reserved, 8);
    w32((int32_t)ix.filter_cutoff);
    w32(ix.bits);
    const gbsa_params& p = ix.params;
    for (int32_t v : {p.canonical_read_length, p.k, p.s, p.l, p.u, (int32_t)p.q, p.max_dist}) w32(v);
    w64(rs.size());
    os.write(reinterpret_cast<const char*>(rs.data()), (std::streamsize)(rs.size() * sizeof(gbsa_ref_randstrobe)));
    w64(starts.size());
    os.write(reinterpret_cast<const char*>(starts.data()), (std::streamsize)(starts.size() * 8));
    if (!os) throw Error(GBSA_ERR_INDEX_FILE, std::string(path) + ": write failed");
}

// ---- mapper --------------------------------------------------------------------------

}  // namespace gbsa

// struct gbsa_mapper: mapper.h

namespace gbsa {

void mapper_reserve(gbsa_mapper& m, uint32_t n, uint64_t bases) {
    m.seqs.resize(bases + 64);
    m.offs.resize(8ull * (n + 1));
    m.lens.resize(4ull * (n + 1));
    m.rec.resize(sizeof(ReadRec) * (n + 1));
    m.lists.resize(16ull * (n + 1));
    m.lane_lists.resize(4ull * kLaneBuckets * (n + 1));
    m.jobs.resize(sizeof(SortJob) * (n + 1));
    m.ctr.resize(sizeof(Counters));
    m.cnt.resize(8ull * (n + 1));
    m.out_off.resize(8ull * (n + 1));
    m.out_frac.resize(4ull * (n + 1));
    m.out_resc.resize(n + 1);
    if (m.profile) {
        m.resc_cycles.resize(64ull * (n + 1));
        m.nam_notes.resize(32ull * (n + 1));
    }
    // query randstrobes: ~2 per 5 bases plus slack
    const uint64_t q_need = std::max<uint64_t>(4096, bases / 2 + 64ull * n / 8);
    if (m.q_cap < q_need) {
        m.q_cap = q_need;
        m.q.resize(sizeof(Query) * m.q_cap);
        m.qaux.resize(4 * m.q_cap);
        m.qpos.resize(8 * m.q_cap);
    }
    if (m.hit_cap < 2 * q_need) {
        m.hit_cap = 2 * q_need;
        m.hits.resize(sizeof(HitPacked) * m.hit_cap);
    }
    if (m.nam_cap < q_need) {
        m.nam_cap = q_need;
        m.nams.resize(sizeof(NamState) * m.nam_cap);
    }
    const uint32_t warps = nam_kernel_warps(std::max<uint32_t>(n, 1));
    if (m.slot_bytes == 0) m.slot_bytes = 32 * 1024;
    m.slots.resize((uint64_t)warps * m.slot_bytes);
    m.side_slots.resize((uint64_t)warps * m.slot_bytes);
    if (m.ovf_cap == 0) {
        m.ovf_cap = 64ull << 20;
        m.ovf.resize(m.ovf_cap);
    }
    if (m.long_warps == 0) {
        m.long_warps = (uint32_t)std::max(8, device_sm_count()) * 2;
        m.long_scratch.resize((uint64_t)m.long_warps * kLongSlotBytes);
    }
}

static Arenas arenas_of(gbsa_mapper& m) {
    Arenas A;
    A.q = m.q.as<Query>();
    A.q_cap = m.q_cap;
    A.q_aux = m.qaux.as<uint32_t>();
    A.q_pos = m.qpos.as<uint64_t>();
    A.hits = m.hits.as<HitPacked>();
    A.hit_cap = m.hit_cap;
    A.nams = m.nams.as<NamState>();
    A.nam_cap = m.nam_cap;
    A.slots = m.slots.as<uint8_t>();
    A.slot_bytes = m.slot_bytes;
    A.ovf = m.ovf.as<uint8_t>();
    A.ovf_cap = m.ovf_cap;
    const size_t per = m.lists.size() / 16;   // u32 entries per list
    A.rescue_list = m.lists.as<uint32_t>();
    A.rescue_cap = (uint32_t)per;
    A.long_list = m.lists.as<uint32_t>() + per;
    A.big_list = m.lists.as<uint32_t>() + 2 * per;
    A.lane_lists = m.lane_lists.as<uint32_t>();
    A.lane_cap = (uint32_t)(m.lane_lists.size() / (4ull * kLaneBuckets));
    A.sort_jobs = m.jobs.as<SortJob>();
    A.jobs_cap = (uint32_t)(m.jobs.size() / sizeof(SortJob));
    A.rescue_cycles = m.profile ? m.resc_cycles.as<uint64_t>() : nullptr;
    A.nam_cycles = m.profile ? m.nam_notes.as<uint64_t>() : nullptr;
    return A;
}

static void grow(DeviceBuffer& b, uint64_t& cap, uint64_t used, size_t elem) {
    const uint64_t want = std::max<uint64_t>(cap * 2, used + used / 4 + 1024);
    cap = want;
    b.release();
    b.resize(elem * cap);
}

// Enqueues one attempt at n reads whose bases/offsets/lengths are on the device:
// seeding (unless the queries are already in place) → lookup → NAMs (main stream) and
// rescue → sorts (side stream), then the per-read NAM offsets into m.out_off[0..n]; the
// device counters and the NAM total are copied to m.h_status (pinned).  Nothing waits
// on the host.

// Records a stage-timing event; inside a stream capture as an external event node, so
// that the graph's launches record it.
void record_stage(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GBSA_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive) GBSA_CUDA(cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal));
    else GBSA_CUDA(cudaEventRecord(ev, st));
}

// Batched form (bm != nullptr): n is bm->cap, the read capacity of the work areas; the
// batch itself (reads, count, work items, outputs) is read from bm->desc in device
// memory by the kernels, so that the sequence can be captured once as a CUDA graph and
// replayed for every batch that fits.  Seeding and lookup then run as one persistent
// kernel pulling work items from a device queue, the records of the batch's reads are
// cleared on the device, and the gather writes the desc's outputs.
void enqueue_batch(gbsa_mapper& m, const uint8_t* d_seqs, const uint64_t* d_offs, const uint32_t* d_lens, uint32_t n,
                   bool seeded, cudaStream_t st, cudaStream_t early, const GatherTarget* gt, const BatchMode* bm) {
    const BatchDesc* desc = bm ? bm->desc : nullptr;
    cudaStream_t main_st = st;
    if (early) {
        GBSA_CUDA(cudaEventRecord(m.early_ev, st));
        GBSA_CUDA(cudaStreamWaitEvent(early, m.early_ev, 0));
        st = early;
    }
    const IndexView I = view_of(*m.idx);
    // the mapper's own scan workspace: a per-call allocation would free device memory,
    // and cudaFree waits for the whole device (other mappers' work included)
    Workspace& ws = m.ws;
    ws.reset();
    m.h_status.resize(sizeof(Counters) + 8);
    Counters* ctr = m.ctr.as<Counters>();
    GBSA_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), st));
    if (desc) {
        launch_clear_recs(n, m.rec.as<ReadRec>(), desc, st);
    } else if (!seeded) {
        GBSA_CUDA(cudaMemsetAsync(m.rec.as<void>(), 0, sizeof(ReadRec) * n, st));
    } else {
        // keep q_off / nq / nq2 written by the caller; clear the rest
        launch_reset_recs(n, m.rec.as<ReadRec>(), st);
    }
    Arenas A = arenas_of(m);
    if (A.rescue_cycles) GBSA_CUDA(cudaMemsetAsync(A.rescue_cycles, 0, m.resc_cycles.size(), st));
    MapConfig C = m.cfg;
    C.count_bytes = m.count_bytes;
    auto mark = [&](int i) {
        if (m.profile) record_stage(m.ev[i], st);
    };
    // Seeding and lookup run as one kernel (a warp seeds a read, then looks it up:
    // hashing overlaps the gathers) unless the index's entries exceed fuse_index_bytes:
    // gathers from an entry array beyond the GPU's TLB reach (3.1 Gbp: 9.9 GB) run
    // faster in a lookup kernel of their own (measured: 56.1 ms fused against 22.7 +
    // 27.8 ms for 10M reads).
    // (the batched form runs its persistent work-queue kernel, with the lookup fused
    // under the same limit)
    const bool fused = !seeded && I.n * sizeof(gbsa_ref_randstrobe) <= m.fuse_index_bytes;
    m.fused = fused;
    mark(0);
    if (desc) launch_seed_lookup_queue(m.idx->dp, I, C, desc, m.rec.as<ReadRec>(), A, ctr, bm->variant, fused, st);
    else if (fused) launch_seed_lookup(m.idx->dp, I, C, d_seqs, d_offs, d_lens, n, m.rec.as<ReadRec>(), A, ctr, st);
    else if (!seeded) launch_seed(m.idx->dp, d_seqs, d_offs, d_lens, n, m.rec.as<ReadRec>(), A, ctr, st);
    mark(1);
    if (!seeded)
        launch_seed_long(m.idx->dp, d_seqs, d_offs, d_lens, m.rec.as<ReadRec>(), A, ctr, m.long_scratch.as<uint8_t>(),
                         m.long_warps, st, desc);
    mark(2);
    if (fused) launch_lookup_long(I, C, n, m.rec.as<ReadRec>(), A, ctr, st);
    else launch_lookup(I, C, n, m.rec.as<ReadRec>(), A, ctr, st, desc);
    launch_bucket_reads(n, C.lane_max_hits, m.rec.as<ReadRec>(), A, ctr, st, desc);
    if (early) {
        GBSA_CUDA(cudaEventRecord(m.early_ev, early));
        GBSA_CUDA(cudaStreamWaitEvent(main_st, m.early_ev, 0));
        st = main_st;
    }
    mark(3);
    // The rescue chain works on the rescued reads only and the NAM kernels on the
    // others: the rescue chain runs on the side stream (with its own scratch slots) so
    // that its tail of reads with thousands of hits overlaps them.
    // (at the main stream's priority: a caller's stream has the lowest)
    cudaStream_t side = m.side;
    if (st != m.st) {
        int prio = 0, lo = 0, hi = 0;
        GBSA_CUDA(cudaStreamGetPriority(st, &prio));
        GBSA_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        if (prio != hi) side = m.side_lo;
    }
    GBSA_CUDA(cudaEventRecord(m.fork_ev, st));
    // the lane merge is submitted ahead of the rescue kernel: the first of two kernels that
    // become ready together takes the SMs first, and the rescue kernel ahead of the lane
    // merge slowed the lane stage by a third
    launch_nams(I, C, n, m.rec.as<ReadRec>(), A, ctr, st);
    mark(4);
    GBSA_CUDA(cudaStreamWaitEvent(side, m.fork_ev, 0));
    Arenas As = A;
    As.slots = m.side_slots.as<uint8_t>();
    launch_rescue(I, C, n, m.rec.as<ReadRec>(), As, ctr, side);
    GBSA_CUDA(cudaEventRecord(m.rescue_ev, side));
    if (m.profile) record_stage(m.ev[6], side);
    if (n) launch_sort_jobs(C, m.rec.as<ReadRec>(), As, ctr, side);
    if (m.profile) record_stage(m.ev[7], side);
    GBSA_CUDA(cudaEventRecord(m.join_ev, side));
    launch_nams_warp(C, n, m.rec.as<ReadRec>(), A, ctr, st);
    mark(5);
    // Every read's NAM count is known once the rescue kernel has ended (the sorts after
    // it only order NAMs): per-read counts → offsets, and the records of the reads that
    // were not rescued, while the side stream may still sort; the rescued reads' records
    // after the join.  (Meaningless when an arena overflowed; the batch then runs again.)
    GBSA_CUDA(cudaStreamWaitEvent(st, m.rescue_ev, 0));
    uint64_t* cnt = m.cnt.as<uint64_t>();
    uint64_t* off = m.out_off.as<uint64_t>();
    launch_read_counts(n, m.rec.as<ReadRec>(), 0, cnt, st, desc);
    scan_exclusive_u64(cnt, off, n, off + n, ws, st);
    if (gt || desc)
        launch_gather_nams(n, m.rec.as<ReadRec>(), m.nams.as<NamState>(), off, gt ? gt->nams : nullptr,
                           gt ? gt->frac : nullptr, gt ? gt->resc : nullptr, st, gt ? gt->cap : 0, 1, nullptr,
                           nullptr, desc);
    GBSA_CUDA(cudaStreamWaitEvent(st, m.join_ev, 0));
    if (gt || desc)
        launch_gather_nams(n, m.rec.as<ReadRec>(), m.nams.as<NamState>(), off, gt ? gt->nams : nullptr, nullptr,
                           nullptr, st, gt ? gt->cap : 0, 2, &A, ctr, desc);
    GBSA_CUDA(cudaMemcpyAsync(m.h_status.as<void>(), ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    GBSA_CUDA(cudaMemcpyAsync(m.h_status.as<uint8_t>() + sizeof(Counters), off + n, 8, cudaMemcpyDeviceToHost, st));
}

// Reads the status of a batch that enqueue_batch ran and that has completed.  Throws for
// a fatal status; grows the work areas that overflowed and returns false (the batch must
// run again); otherwise records the counters and returns true.
bool check_batch(gbsa_mapper& m, bool seeded) {
    const Counters h = *m.h_status.as<Counters>();
    if (m.profile) {
        // seed, long seed, lookup, lane NAMs, warp NAMs (main stream); rescue, its
        // block sorts (side stream, from the fork after the lookup)
        static const int from[7] = {0, 1, 2, 3, 4, 3, 6}, to[7] = {1, 2, 3, 4, 5, 6, 7};
        for (int i = 0; i < 7; ++i) GBSA_CUDA(cudaEventElapsedTime(&m.stage_ms[i], m.ev[from[i]], m.ev[to[i]]));
    }
    if (h.status & kStatusReadTooLong)
        throw Error(GBSA_ERR_READ_TOO_LONG, "a read is longer than GBSA_MAX_READ_LEN bases");
    if (h.status & kStatusSyncmerOverflow) throw Error(GBSA_ERR_DEVICE_STATUS, "syncmer buffer overflow");
    bool retry = false;
    if (h.status & kStatusQueryOverflow) {
        if (seeded) throw Error(GBSA_ERR_DEVICE_STATUS, "query arena overflow");
        grow(m.q, m.q_cap, h.q_used, sizeof(Query));
        m.qaux.release();
        m.qaux.resize(4 * m.q_cap);
        m.qpos.release();
        m.qpos.resize(8 * m.q_cap);
        retry = true;
    }
    if (h.status & kStatusHitOverflow) {
        grow(m.hits, m.hit_cap, h.hit_used, sizeof(HitPacked));
        retry = true;
    }
    if (h.status & kStatusNamOverflow) {
        grow(m.nams, m.nam_cap, h.nam_used, sizeof(NamState));
        retry = true;
    }
    if (h.status & kStatusScratchOverflow) {
        grow(m.ovf, m.ovf_cap, h.scratch_used, 1);
        retry = true;
    }
    if (retry) {
        ++m.retries;
        return false;
    }
    m.alg_bytes = h.alg_bytes;
    m.alg_sectors = h.alg_sectors;
    m.last = h;
    return true;
}

uint64_t batch_total(gbsa_mapper& m) {
    uint64_t t;
    std::memcpy(&t, m.h_status.as<uint8_t>() + sizeof(Counters), 8);
    return t;
}

// enqueue_batch + check_batch until the work areas are large enough: leaves per-read NAM
// offsets in m.out_off[0..n] and returns the NAM total.
static uint64_t run_pipeline(gbsa_mapper& m, const uint8_t* d_seqs, const uint64_t* d_offs, const uint32_t* d_lens,
                             uint32_t n, bool seeded, cudaStream_t st, const GatherTarget* gt = nullptr) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        enqueue_batch(m, d_seqs, d_offs, d_lens, n, seeded, st, nullptr, gt);
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (check_batch(m, seeded)) return batch_total(m);
    }
    throw Error(GBSA_ERR_DEVICE_STATUS, "work areas kept overflowing");
}

// L2 access-policy window over the index's bucket table (the 32-bit copy when there
// is one: 32 MB for 2^23 buckets), read by every probe of the lookup: held persisting
// in L2 so that the entry gathers do not evict it.  Used when the table fits the
// device's largest window; the hit ratio is the part of the table the persisting L2
// set-aside can hold.  The set-aside (cudaLimitPersistingL2CacheSize) is a limit of
// this process's context: it is raised to the largest window of the live mappers and
// returned to zero, with the persisting lines reset, when the last of them is freed.
static std::mutex g_l2_mu;
static std::vector<int> g_l2_users;   // per device: mappers holding a window

void l2_window_attach(gbsa_mapper& m, bool on) {
    const bool had = m.cfg.l2_bytes != 0;
    if (on == had) return;
    int dev = 0;
    GBSA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(g_l2_mu);
    if ((int)g_l2_users.size() <= dev) g_l2_users.resize(dev + 1, 0);
    if (!on) {
        m.cfg.l2_base = nullptr;
        m.cfg.l2_bytes = 0;
        if (--g_l2_users[dev] == 0) {
            GBSA_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0));
            GBSA_CUDA(cudaCtxResetPersistingL2Cache());
        }
        return;
    }
    const gbsa_index& ix = *m.idx;
    const void* base = ix.starts32.size() ? ix.starts32.as<void>() : ix.starts.as<void>();
    const uint64_t bytes = ((1ull << ix.bits) + 1) * (ix.starts32.size() ? 4 : 8);
    int max_window = 0, persist_max = 0;
    GBSA_CUDA(cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, dev));
    GBSA_CUDA(cudaDeviceGetAttribute(&persist_max, cudaDevAttrMaxPersistingL2CacheSize, dev));
    if (!m.use_l2_window || persist_max <= 0 || bytes > (uint64_t)max_window) return;
    size_t cur = 0;
    GBSA_CUDA(cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize));
    const size_t want = std::min<size_t>((size_t)persist_max, bytes);
    if (cur < want) GBSA_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want));
    m.cfg.l2_base = base;
    m.cfg.l2_bytes = bytes;
    m.cfg.l2_hit_ratio = (float)std::min(1.0, (double)want / (double)bytes);
    ++g_l2_users[dev];
}

// Chunks of a pipelined host call: `chunks` full chunks of at least 2^17 reads, with
// the first one cut in half (the GPU waits for its reads alone, and the half chunk ends
// early, so that the following chunks run staggered: one in its NAM phase beside the
// next one's seeding) and the last full chunk cut into two quarters (the results of
// the last chunk are copied out after all work ends).  Returns the chunk starts with
// n_reads at the end.
static std::vector<uint32_t> plan_chunks(uint32_t n_reads, uint32_t chunks, uint32_t max_reads) {
    constexpr uint32_t kMinChunk = 1u << 17;
    const uint32_t c = std::max<uint32_t>(1, std::min<uint32_t>(chunks, n_reads / kMinChunk));
    const uint32_t full = std::min((n_reads + c - 1) / c, max_reads);
    std::vector<uint32_t> sizes;
    if (c >= 2 && full >= 2 * kMinChunk) {
        const uint32_t head = full / 2, quarter = full / 4;
        uint32_t mid = n_reads - head - 2 * quarter;
        sizes.push_back(head);
        while (mid) {
            const uint32_t x = std::min(full, mid);
            sizes.push_back(x);
            mid -= x;
        }
        sizes.push_back(quarter);
        sizes.push_back(quarter);
    } else {
        for (uint32_t b = 0; b < n_reads; b += full) sizes.push_back(std::min(full, n_reads - b));
    }
    std::vector<uint32_t> starts{0};
    for (uint32_t x : sizes)
        if (x) starts.push_back(starts.back() + x);
    return starts;
}

// Copies n reads (host) to the mapper's device inputs.  Reads usually lie back to back:
// the span from the first read's start to the last read's end is copied in one
// transfer and the offsets are rebased to it (in parallel, checking that every read
// lies inside the span); otherwise the reads are gathered into pinned staging first.
uint64_t stage_reads(gbsa_mapper& m, const char* seqs, const uint64_t* offsets, const uint32_t* lengths, uint32_t n,
                     cudaStream_t st) {
    const uint64_t lo = n ? offsets[0] : 0;
    const uint64_t hi = n ? offsets[n - 1] + lengths[n - 1] : 0;
    const bool span_ok = hi >= lo;
    const uint64_t span = span_ok ? hi - lo : 0;
    std::atomic<bool> inside{span_ok};
    std::atomic<uint64_t> total{0};
    m.h_meta.resize(12ull * (n + 1));
    uint64_t* ho = m.h_meta.as<uint64_t>();
    uint32_t* hl = reinterpret_cast<uint32_t*>(ho + n + 1);
    host_parallel_for(n, [&](size_t b, size_t e) {
        bool ok = true;
        uint64_t t = 0;
        for (size_t i = b; i < e; ++i) {
            ok &= offsets[i] >= lo && offsets[i] + lengths[i] <= hi;
            ho[i] = offsets[i] - lo;
            hl[i] = lengths[i];
            t += lengths[i];
        }
        if (!ok) inside.store(false);
        total.fetch_add(t);
    });
    const bool direct = inside.load() && span <= 2 * total.load() + (1u << 20);   // no large gaps
    const uint64_t bases = direct ? span : total.load();
    mapper_reserve(m, n, bases);
    m.seqs.resize(bases + 64);
    m.offs.resize(8ull * (n + 1));
    m.lens.resize(4ull * (n + 1));
    if (direct) {
        if (span) GBSA_CUDA(cudaMemcpyAsync(m.seqs.as<void>(), seqs + lo, span, cudaMemcpyHostToDevice, st));
    } else {
        // exclusive offsets of the gathered layout, then a parallel gather
        uint64_t acc = 0;
        for (uint32_t i = 0; i < n; ++i) {
            ho[i] = acc;
            acc += lengths[i];
        }
        m.h_seqs.resize(acc + 1);
        char* hs = m.h_seqs.as<char>();
        host_parallel_for(n, [&](size_t b, size_t e) {
            for (size_t i = b; i < e; ++i) std::memcpy(hs + ho[i], seqs + offsets[i], lengths[i]);
        });
        if (acc) GBSA_CUDA(cudaMemcpyAsync(m.seqs.as<void>(), hs, acc, cudaMemcpyHostToDevice, st));
    }
    GBSA_CUDA(cudaMemcpyAsync(m.offs.as<void>(), ho, 8ull * n, cudaMemcpyHostToDevice, st));
    GBSA_CUDA(cudaMemcpyAsync(m.lens.as<void>(), hl, 4ull * n, cudaMemcpyHostToDevice, st));
    return total.load();
}

}  // namespace gbsa

using namespace gbsa;

extern "C" {

const char* gbsa_last_error(void) { return t_last_error.c_str(); }
int gbsa_version(void) { return 1; }
uint64_t gbsa_launch_count(void) { return g_launches.load(); }

int gbsa_params_from_read_length(int read_length, int k, int s, int l, int u, int c, int max_seed_len,
                                 gbsa_params* out) {
    return guarded([&] {
        // profiles of step2/indexparameters.cpp:136-144
        struct Profile { int r, thr, k, s_off, l, u; };
        static const Profile profiles[] = {
            {50, 90, 20, -4, -3, 2},  {100, 110, 20, -4, -2, 2}, {125, 135, 20, -4, -1, 4},
            {150, 175, 20, -4, 1, 7}, {250, 275, 20, -4, 4, 13}, {300, 375, 22, -4, 2, 12},
            {400, INT_MAX, 23, -6, 2, 12},
        };
        uint64_t canonical = 50;
        for (const auto& p : profiles) {
            if (read_length <= p.thr) {
                if (k == GBSA_DEFAULT) k = p.k;
                if (s == GBSA_DEFAULT) s = k + p.s_off;
                if (l == GBSA_DEFAULT) l = p.l;
                if (u == GBSA_DEFAULT) u = p.u;
                canonical = (uint64_t)p.r;
                break;
            }
        }
        int max_dist;
        if (max_seed_len == GBSA_DEFAULT) {
            max_dist = std::min(255, std::max((int)canonical - 70, k));
        } else {
            max_dist = max_seed_len - k;
        }
        const int q = (int)(std::pow(2, c == GBSA_DEFAULT ? 8 : c) - 1);
        make_params(canonical, k, s, l, u, q, max_dist, out);
    });
}

int gbsa_params_make(uint64_t canonical_read_length, int k, int s, int l, int u, int q, int max_dist,
                     gbsa_params* out) {
    return guarded([&] { make_params(canonical_read_length, k, s, l, u, q, max_dist, out); });
}

int gbsa_pick_bits(const gbsa_params* p, uint64_t total_length) { return pick_bits_host(*p, total_length); }

int gbsa_index_build(const gbsa_params* p, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
                     uint32_t n_contigs, int bits, float f, gbsa_index** out) {
    return guarded([&] {
        *out = nullptr;
        if (!params_valid(*p)) throw Error(GBSA_ERR_PARAM, "invalid index parameters");
        require_device();
        uint64_t total = 0;
        for (uint32_t c = 0; c < n_contigs; ++c) total += lengths[c];
        const int b = bits == -1 ? pick_bits_host(*p, total) : bits;
        if (b < 8 || b > 31) throw Error(GBSA_ERR_PARAM, "Bits must be between 8 and 31");   // index.hpp:45-47
        std::unique_ptr<gbsa_index> ix(new gbsa_index());
        ix->params = *p;
        ix->dp = make_dev_params(*p);
        ix->bits = b;
        GBSA_CUDA(cudaGetDevice(&ix->device));
        build_index(*ix, seqs, offsets, lengths, n_contigs, f);
        *out = ix.release();
    });
}

int gbsa_index_load(const gbsa_params* p, const gbsa_ref_randstrobe* randstrobes, uint64_t n,
                    const uint64_t* start_indices, int bits, uint32_t filter_cutoff, gbsa_index** out) {
    return guarded([&] {
        *out = nullptr;
        if (!params_valid(*p)) throw Error(GBSA_ERR_PARAM, "invalid index parameters");
        if (bits < 8 || bits > 31) throw Error(GBSA_ERR_PARAM, "Bits must be between 8 and 31");
        require_device();
        std::unique_ptr<gbsa_index> ix(new gbsa_index());
        ix->params = *p;
        ix->dp = make_dev_params(*p);
        ix->bits = bits;
        ix->filter_cutoff = filter_cutoff;
        ix->n = n;
        GBSA_CUDA(cudaGetDevice(&ix->device));
        ix->rs.resize(16 * (n + 1));
        const uint64_t nb = (1ULL << bits) + 1;
        ix->starts.resize(8 * nb);
        if (n) GBSA_CUDA(cudaMemcpy(ix->rs.as<void>(), randstrobes, 16 * n, cudaMemcpyHostToDevice));
        GBSA_CUDA(cudaMemcpy(ix->starts.as<void>(), start_indices, 8 * nb, cudaMemcpyHostToDevice));
        make_compact_starts(*ix, 0);
        ix->info.size = n;
        ix->info.bits = bits;
        ix->info.filter_cutoff = filter_cutoff;
        ix->info.tot_strobemer_count = n;
        *out = ix.release();
    });
}

int gbsa_index_read_sti(const char* path, const gbsa_params* p, gbsa_index** out) {
    return guarded([&] {
        *out = nullptr;
        std::ifstream is(path, std::ios::binary);
        if (!is) throw Error(GBSA_ERR_INDEX_FILE, std::string(path) + ": cannot open");
        char magic[4];
        is.read(magic, 4);
        if (!is || std::memcmp(magic, "STI\1", 4) != 0)
            throw Error(GBSA_ERR_INDEX_FILE, "Index file has incorrect format (magic number mismatch)");
        auto r32 = [&]() {
            int32_t v = 0;
            is.read(reinterpret_cast<char*>(&v), 4);
            return v;
        };
        auto r64 = [&]() {
            uint64_t v = 0;
            is.read(reinterpret_cast<char*>(&v), 8);
            return v;
        };
        const int32_t ver = r32();
        if (ver != 2)
            throw Error(GBSA_ERR_INDEX_FILE, "Can only read index file format version 2, but found version " +
                                                 std::to_string(ver));
        const uint64_t reserved = r64();
        is.seekg((std::streamoff)reserved, std::ios_base::cur);
        const uint32_t fc = (uint32_t)r32();
        const int32_t bits = r32();
        int32_t v[7];
        for (auto& x : v) x = r32();
        gbsa_params fp{};
        make_params((uint64_t)v[0], v[1], v[2], v[3], v[4], v[5], v[6], &fp);
        if (fp.canonical_read_length != p->canonical_read_length || fp.k != p->k || fp.s != p->s || fp.l != p->l ||
            fp.u != p->u || fp.q != p->q || fp.max_dist != p->max_dist)
            throw Error(GBSA_ERR_INDEX_FILE, "Index parameters in .sti file and those specified on command line differ");
        const uint64_t n = r64();
        std::vector<gbsa_ref_randstrobe> rs(n);
        is.read(reinterpret_cast<char*>(rs.data()), (std::streamsize)(16 * n));
        const uint64_t ns = r64();
        if (bits < 8 || bits > 31 || ns != (1ULL << bits) + 1)
            throw Error(GBSA_ERR_INDEX_FILE, "randstrobe_start_indices vector is of the wrong size");
        std::vector<uint64_t> starts(ns);
        is.read(reinterpret_cast<char*>(starts.data()), (std::streamsize)(8 * ns));
        if (!is) throw Error(GBSA_ERR_INDEX_FILE, std::string(path) + ": truncated");
        const int rc = gbsa_index_load(p, rs.data(), n, starts.data(), bits, fc, out);
        if (rc != GBSA_OK) throw Error(rc, t_last_error);
    });
}

int gbsa_index_write_sti(const gbsa_index* idx, const char* path) {
    return guarded([&] {
        std::vector<gbsa_ref_randstrobe> rs(idx->n);
        std::vector<uint64_t> starts((1ULL << idx->bits) + 1);
        if (idx->n) GBSA_CUDA(cudaMemcpy(rs.data(), idx->rs.as<void>(), 16 * idx->n, cudaMemcpyDeviceToHost));
        GBSA_CUDA(cudaMemcpy(starts.data(), idx->starts.as<void>(), 8 * starts.size(), cudaMemcpyDeviceToHost));
        write_sti(*idx, rs, starts, path);
    });
}

int gbsa_index_get_info(const gbsa_index* idx, gbsa_index_info* out) {
    *out = idx->info;
    return GBSA_OK;
}

int gbsa_index_get_params(const gbsa_index* idx, gbsa_params* out) {
    *out = idx->params;
    return GBSA_OK;
}

int gbsa_index_export(const gbsa_index* idx, gbsa_ref_randstrobe* randstrobes, uint64_t* start_indices) {
    return guarded([&] {
        if (idx->n && randstrobes)
            GBSA_CUDA(cudaMemcpy(randstrobes, idx->rs.as<void>(), 16 * idx->n, cudaMemcpyDeviceToHost));
        if (start_indices)
            GBSA_CUDA(cudaMemcpy(start_indices, idx->starts.as<void>(), 8 * ((1ULL << idx->bits) + 1),
                                 cudaMemcpyDeviceToHost));
    });
}

void gbsa_index_free(gbsa_index* idx) { delete idx; }

int gbsa_find(const gbsa_index* idx, const uint64_t* hashes, uint64_t n, uint64_t* positions) {
    return guarded([&] {
        if (!n) return;
        DeviceBuffer dh(8 * n), dp(8 * n);
        GBSA_CUDA(cudaMemcpy(dh.as<void>(), hashes, 8 * n, cudaMemcpyHostToDevice));
        launch_find(view_of(*idx), dh.as<uint64_t>(), n, dp.as<uint64_t>(), 0);
        GBSA_CUDA(cudaMemcpy(positions, dp.as<void>(), 8 * n, cudaMemcpyDeviceToHost));
    });
}

int gbsa_get_count(const gbsa_index* idx, const uint64_t* positions, uint64_t n, uint32_t* counts) {
    return guarded([&] {
        if (!n) return;
        DeviceBuffer dp(8 * n), dc(4 * n);
        GBSA_CUDA(cudaMemcpy(dp.as<void>(), positions, 8 * n, cudaMemcpyHostToDevice));
        launch_get_count(view_of(*idx), dp.as<uint64_t>(), n, dc.as<uint32_t>(), 0);
        GBSA_CUDA(cudaMemcpy(counts, dc.as<void>(), 4 * n, cudaMemcpyDeviceToHost));
    });
}

int gbsa_randstrobes_query(const gbsa_params* p, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                           uint32_t n_reads, gbsa_query_randstrobe* out, uint64_t out_capacity, uint64_t* out_offsets,
                           uint64_t* out_total) {
    return guarded([&] {
        if (!params_valid(*p)) throw Error(GBSA_ERR_PARAM, "invalid index parameters");
        require_device();
        gbsa_index dummy;
        dummy.params = *p;
        dummy.dp = make_dev_params(*p);
        gbsa_mapper m;
        m.idx = &dummy;
        GBSA_CUDA(cudaStreamCreateWithFlags(&m.st, cudaStreamNonBlocking));
        struct G {
            cudaStream_t s;
            ~G() { cudaStreamDestroy(s); }
        } g{m.st};
        Workspace ws;
        const uint32_t n = n_reads;
        stage_reads(m, seqs, offsets, lengths, n, m.st);
        for (int attempt = 0; attempt < 8; ++attempt) {
            Counters* ctr = m.ctr.as<Counters>();
            GBSA_CUDA(cudaMemsetAsync(ctr, 0, sizeof(Counters), m.st));
            GBSA_CUDA(cudaMemsetAsync(m.rec.as<void>(), 0, sizeof(ReadRec) * (n + 1), m.st));
            Arenas A = arenas_of(m);
            launch_seed(dummy.dp, m.seqs.as<uint8_t>(), m.offs.as<uint64_t>(), m.lens.as<uint32_t>(), n,
                        m.rec.as<ReadRec>(), A, ctr, m.st);
            launch_seed_long(dummy.dp, m.seqs.as<uint8_t>(), m.offs.as<uint64_t>(), m.lens.as<uint32_t>(),
                             m.rec.as<ReadRec>(), A, ctr, m.long_scratch.as<uint8_t>(), m.long_warps, m.st);
            Counters h{};
            GBSA_CUDA(cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, m.st));
            GBSA_CUDA(cudaStreamSynchronize(m.st));
            if (h.status & kStatusReadTooLong)
                throw Error(GBSA_ERR_READ_TOO_LONG, "a read is longer than GBSA_MAX_READ_LEN bases");
            if (h.status & kStatusSyncmerOverflow) throw Error(GBSA_ERR_DEVICE_STATUS, "syncmer buffer overflow");
            if (h.status & kStatusQueryOverflow) {
                grow(m.q, m.q_cap, h.q_used, sizeof(Query));
                m.qaux.release();
                m.qaux.resize(4 * m.q_cap);
                m.qpos.release();
                m.qpos.resize(8 * m.q_cap);
                continue;
            }
            uint64_t* cnt = m.cnt.as<uint64_t>();
            uint64_t* off = m.out_off.as<uint64_t>();
            launch_read_counts(n, m.rec.as<ReadRec>(), 1, cnt, m.st);
            scan_exclusive_u64(cnt, off, n, off + n, ws, m.st);
            GBSA_CUDA(cudaMemcpyAsync(out_offsets, off, 8ull * (n + 1), cudaMemcpyDeviceToHost, m.st));
            GBSA_CUDA(cudaStreamSynchronize(m.st));
            const uint64_t total = out_offsets[n];
            if (out_total) *out_total = total;
            if (total > out_capacity) throw Error(GBSA_ERR_CAPACITY, "output capacity too small");
            if (total) {
                DeviceBuffer dout(sizeof(gbsa_query_randstrobe) * total);
                launch_gather_queries(n, m.rec.as<ReadRec>(), m.q.as<Query>(), off,
                                      dout.as<gbsa_query_randstrobe>(), m.st);
                GBSA_CUDA(cudaMemcpyAsync(out, dout.as<void>(), sizeof(gbsa_query_randstrobe) * total,
                                          cudaMemcpyDeviceToHost, m.st));
                GBSA_CUDA(cudaStreamSynchronize(m.st));
            }
            return;
        }
        throw Error(GBSA_ERR_DEVICE_STATUS, "query arena kept overflowing");
    });
}

int gbsa_mapper_create(const gbsa_index* idx, const gbsa_map_options* opt, uint32_t max_reads, uint64_t max_bases,
                       gbsa_mapper** out) {
    return guarded([&] {
        *out = nullptr;
        require_device();
        std::unique_ptr<gbsa_mapper> m(new gbsa_mapper());
        m->idx = idx;
        m->opt = *opt;
        m->cfg.rescue_level = opt->rescue_level;
        m->cfg.rescue_cutoff = opt->rescue_level < 100 ? (uint32_t)(opt->rescue_level * (int)idx->filter_cutoff)
                                                       : 100u;   // step2/main.cu:4204
        m->cfg.count_cap = opt->rescue_count_cap;
        m->cfg.sort_mode = opt->sort_mode;
        {
            // the NAM phase's shape from the committed autotuner result (the same kernels
            // as the batched form's; results do not depend on it)
            gbsa_batch_config bc{};
            int from_file = 0;
            if (gbsa_batch_config_default(&bc, &from_file) == GBSA_OK) {
                m->cfg.lane_max_hits = bc.lane_max_hits;
                m->cfg.sort_variant = bc.sort_variant;
                m->cfg.lane_variant = bc.lane_variant;
                m->cfg.warp_variant = bc.warp_variant;
                // heavy rescued reads of small batches merged a block each (10k-100k-read
                // batches of 150 bp pairs: about 0.3 of the batch time less)
                m->cfg.rescue_block_hits = bc.rescue_block_hits;
            }
        }
        l2_window_attach(*m, true);
        m->max_reads = std::max<uint32_t>(max_reads, 1);
        m->max_bases = std::max<uint64_t>(max_bases, 1);
        // the mapper's own streams run the NAM phase at the highest priority, the seeding
        // and lookup of pipelined chunks (early) at the lowest: the block scheduler then
        // finishes the older chunk first and fills its tails with the next one's seeding
        int lo = 0, hi = 0;
        GBSA_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        GBSA_CUDA(cudaStreamCreateWithPriority(&m->st, cudaStreamNonBlocking, hi));
        GBSA_CUDA(cudaStreamCreateWithPriority(&m->side, cudaStreamNonBlocking, hi));
        GBSA_CUDA(cudaStreamCreateWithPriority(&m->side_lo, cudaStreamNonBlocking, lo));
        GBSA_CUDA(cudaStreamCreateWithPriority(&m->early, cudaStreamNonBlocking, lo));
        GBSA_CUDA(cudaEventCreateWithFlags(&m->early_ev, cudaEventDisableTiming));
        GBSA_CUDA(cudaEventCreateWithFlags(&m->fork_ev, cudaEventDisableTiming));
        GBSA_CUDA(cudaEventCreateWithFlags(&m->join_ev, cudaEventDisableTiming));
        GBSA_CUDA(cudaEventCreateWithFlags(&m->rescue_ev, cudaEventDisableTiming));
        mapper_reserve(*m, m->max_reads, m->max_bases);
        *out = m.release();
    });
}

void gbsa_mapper_free(gbsa_mapper* m) {
    if (!m) return;
    gbsa_mapper_free(m->twin);
    if (m->side) cudaStreamSynchronize(m->side);
    if (m->st) cudaStreamSynchronize(m->st);
    try {
        l2_window_attach(*m, false);
    } catch (const Error&) {
    }
    for (auto& e : m->ev)
        if (e) cudaEventDestroy(e);
    if (m->copy_in) cudaStreamSynchronize(m->copy_in);
    if (m->copy_out) cudaStreamSynchronize(m->copy_out);
    for (cudaEvent_t e : {m->in_ready, m->done_ev, m->outs[0].free, m->outs[1].free})
        if (e) cudaEventDestroy(e);
    if (m->copy_in) cudaStreamDestroy(m->copy_in);
    if (m->copy_out) cudaStreamDestroy(m->copy_out);
    if (m->fork_ev) cudaEventDestroy(m->fork_ev);
    if (m->join_ev) cudaEventDestroy(m->join_ev);
    if (m->rescue_ev) cudaEventDestroy(m->rescue_ev);
    for (cudaStream_t x : {m->early, m->side_lo})
        if (x) {
            cudaStreamSynchronize(x);
            cudaStreamDestroy(x);
        }
    if (m->early_ev) cudaEventDestroy(m->early_ev);
    if (m->side) cudaStreamDestroy(m->side);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
}

int gbsa_map_reads(gbsa_mapper* m, const char* seqs, const uint64_t* offsets, const uint32_t* lengths, uint32_t n_reads,
                   gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets, float* frac, uint8_t* rescued) {
    return guarded([&] {
        // A large call is cut into chunks that alternate between the mapper and its twin
        // (a second set of work areas and streams), so that chunk k+1 is mapped while
        // chunk k finishes: the tail of one chunk (the rescue chain of a few reads in
        // repeats) runs beside the start of the next, and no host synchronisation stands
        // between them.  A chunk's reads are copied in on the copy_in stream; its results
        // are copied out on copy_out once the host has read its status, by which time
        // the next chunk is already running.
        nam_offsets[0] = 0;
        if (n_reads == 0) return;
        if (!m->copy_in) {
            GBSA_CUDA(cudaStreamCreateWithFlags(&m->copy_in, cudaStreamNonBlocking));
            GBSA_CUDA(cudaStreamCreateWithFlags(&m->copy_out, cudaStreamNonBlocking));
        }
        const std::vector<uint32_t> starts = plan_chunks(n_reads, m->pipe_chunks, m->max_reads);
        const uint32_t n_chunks = (uint32_t)starts.size() - 1;
        if (n_chunks > 1 && !m->twin) {
            gbsa_mapper* t = nullptr;
            const int rc = gbsa_mapper_create(m->idx, &m->opt, m->max_reads, m->max_bases, &t);
            if (rc != GBSA_OK) throw Error(rc, t_last_error);
            m->twin = t;
            if (!m->use_l2_window) {
                l2_window_attach(*t, false);
                t->use_l2_window = false;
            }
        }
        if (m->twin) {
            // the twin keeps its own L2 window registration (same window as m's)
            const MapConfig own = m->twin->cfg;
            m->twin->cfg = m->cfg;
            m->twin->cfg.l2_base = own.l2_base;
            m->twin->cfg.l2_bytes = own.l2_bytes;
            m->twin->cfg.l2_hit_ratio = own.l2_hit_ratio;
            m->twin->opt = m->opt;
            m->twin->fuse_index_bytes = m->fuse_index_bytes;
        }
        gbsa_mapper* part[2] = {m, n_chunks > 1 ? m->twin : m};
        for (gbsa_mapper* b : part)
            for (cudaEvent_t* e : {&b->done_ev, &b->in_ready, &b->outs[0].free, &b->outs[1].free})
                if (!*e) GBSA_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        // chunk k runs on part k & 1 and leaves its results in that part's slot (k >> 1) & 1
        auto rows = [&](uint32_t k) { return starts[k + 1] - starts[k]; };
        auto slot_of = [&](uint32_t k) -> gbsa_mapper::OutSlot& { return part[k & 1]->outs[(k >> 1) & 1]; };
        auto gather = [&](uint32_t k) {
            gbsa_mapper& b = *part[k & 1];
            gbsa_mapper::OutSlot& o = slot_of(k);
            launch_gather_nams(rows(k), b.rec.as<ReadRec>(), b.nams.as<NamState>(), b.out_off.as<uint64_t>(),
                               o.nams.as<gbsa_nam>(), o.frac.as<float>(), o.resc.as<uint8_t>(), b.st, o.cap);
        };
        // copies chunk k's reads in and queues its mapping and the gather of its results
        // into its slot on its part's streams
        auto enqueue = [&](uint32_t k) {
            gbsa_mapper& b = *part[k & 1];
            gbsa_mapper::OutSlot& o = slot_of(k);
            const uint32_t b0 = starts[k], n = rows(k);
            // the part's previous chunk is done (the host read its status) and the slot's
            // previous results have been copied out
            GBSA_CUDA(cudaEventSynchronize(b.done_ev));
            GBSA_CUDA(cudaEventSynchronize(o.free));
            stage_reads(b, seqs, offsets + b0, lengths + b0, n, m->copy_in);
            GBSA_CUDA(cudaEventRecord(b.in_ready, m->copy_in));
            const uint64_t want = (uint64_t)(b.nams_per_read * 1.25 * n) + 1024;
            if (o.cap < want) {
                o.nams.release();
                o.nams.resize(sizeof(gbsa_nam) * want);
                o.cap = want;
            }
            o.frac.resize(4ull * (n + 1));
            o.resc.resize(n + 1);
            o.off.resize(8ull * (n + 1));
            o.off_g.resize(8ull * (n + 1));
            GBSA_CUDA(cudaStreamWaitEvent(b.st, b.in_ready, 0));
            const GatherTarget gt{o.nams.as<gbsa_nam>(), o.cap, o.frac.as<float>(), o.resc.as<uint8_t>()};
            enqueue_batch(b, b.seqs.as<uint8_t>(), b.offs.as<uint64_t>(), b.lens.as<uint32_t>(), n, false, b.st,
                          b.early, &gt);
            launch_offsets_add(b.out_off.as<uint64_t>(), o.off.as<uint64_t>(), n, 0, b.st);
            GBSA_CUDA(cudaEventRecord(b.done_ev, b.st));
        };
        uint64_t done_nams = 0;
        // waits for chunk k, reads its status and copies its results out; false when a work
        // area overflowed (it has been grown and the chunk must run again)
        auto finish = [&](uint32_t k) {
            gbsa_mapper& b = *part[k & 1];
            gbsa_mapper::OutSlot& o = slot_of(k);
            const uint32_t b0 = starts[k], n = rows(k);
            GBSA_CUDA(cudaEventSynchronize(b.done_ev));
            if (!check_batch(b, false)) return false;
            const uint64_t total = batch_total(b);
            b.nams_per_read = std::max(b.nams_per_read, (double)total / std::max<uint32_t>(n, 1));
            if (total > o.cap) {
                // more NAMs than the estimate: gather again into a larger slot (the part's
                // work areas are intact, its next chunk is not queued yet)
                o.nams.release();
                o.nams.resize(sizeof(gbsa_nam) * (total + 1));
                o.cap = total + 1;
                gather(k);
                GBSA_CUDA(cudaEventRecord(b.done_ev, b.st));
            }
            GBSA_CUDA(cudaStreamWaitEvent(m->copy_out, b.done_ev, 0));
            launch_offsets_add(o.off.as<uint64_t>(), o.off_g.as<uint64_t>(), n, done_nams, m->copy_out);
            GBSA_CUDA(cudaMemcpyAsync(nam_offsets + b0, o.off_g.as<void>(), 8ull * n, cudaMemcpyDeviceToHost,
                                      m->copy_out));
            if (frac)
                GBSA_CUDA(cudaMemcpyAsync(frac + b0, o.frac.as<void>(), 4ull * n, cudaMemcpyDeviceToHost, m->copy_out));
            if (rescued)
                GBSA_CUDA(cudaMemcpyAsync(rescued + b0, o.resc.as<void>(), n, cudaMemcpyDeviceToHost, m->copy_out));
            if (done_nams + total <= nam_capacity && total)
                GBSA_CUDA(cudaMemcpyAsync(nams + done_nams, o.nams.as<void>(), sizeof(gbsa_nam) * total,
                                          cudaMemcpyDeviceToHost, m->copy_out));
            GBSA_CUDA(cudaEventRecord(o.free, m->copy_out));
            done_nams += total;
            return true;
        };
        // on an error, the work and copies in flight end before the call returns (they
        // write into the caller's buffers)
        struct Drain {
            gbsa_mapper* const* part;
            gbsa_mapper* m;
            bool armed = true;
            ~Drain() {
                if (!armed) return;
                for (int i = 0; i < 2; ++i)
                    for (cudaStream_t x : {part[i]->early, part[i]->side, part[i]->st}) cudaStreamSynchronize(x);
                cudaStreamSynchronize(m->copy_in);
                cudaStreamSynchronize(m->copy_out);
            }
        } drain{part, m};
        // two chunks in flight: chunk k+1 is queued before the host waits for chunk k
        uint32_t queued = 0, finished = 0, retries = 0;
        while (finished < n_chunks) {
            while (queued < n_chunks && queued < finished + 2) enqueue(queued++);
            if (finish(finished)) {
                ++finished;
                continue;
            }
            // a work area overflowed: let everything in flight end, then run the chunk again
            if (++retries > 8) throw Error(GBSA_ERR_DEVICE_STATUS, "work areas kept overflowing");
            for (gbsa_mapper* b : part)
                for (cudaStream_t x : {b->early, b->side, b->st}) GBSA_CUDA(cudaStreamSynchronize(x));
            GBSA_CUDA(cudaStreamSynchronize(m->copy_in));
            queued = finished;
        }
        GBSA_CUDA(cudaStreamSynchronize(m->copy_out));
        drain.armed = false;
        nam_offsets[n_reads] = done_nams;
        if (done_nams > nam_capacity) throw Error(GBSA_ERR_CAPACITY, "NAM capacity too small");
    });
}

int gbsa_mapper_set_pipeline(gbsa_mapper* m, uint32_t chunks) {
    return guarded([&] {
        if (chunks == 0) throw Error(GBSA_ERR_PARAM, "chunks must be at least 1");
        m->pipe_chunks = chunks;
    });
}

int gbsa_map_reads_device(gbsa_mapper* m, const char* d_seqs, const uint64_t* d_offsets, const uint32_t* d_lengths,
                          uint32_t n_reads, gbsa_nam* d_nams, uint64_t nam_capacity, uint64_t* d_nam_offsets,
                          float* d_frac, uint8_t* d_rescued, uint64_t* nam_total, void* stream) {
    return guarded([&] {
        cudaStream_t st = stream ? (cudaStream_t)stream : m->st;
        mapper_reserve(*m, n_reads, m->max_bases);
        // the batch gathers its records into the caller's buffers itself (at most
        // nam_capacity of them)
        const GatherTarget gt{d_nams, nam_capacity, d_frac, d_rescued};
        const uint64_t total = run_pipeline(*m, reinterpret_cast<const uint8_t*>(d_seqs), d_offsets, d_lengths,
                                            n_reads, false, st, &gt);
        if (nam_total) *nam_total = total;
        GBSA_CUDA(cudaMemcpyAsync(d_nam_offsets, m->out_off.as<void>(), 8ull * (n_reads + 1),
                                  cudaMemcpyDeviceToDevice, st));
        if (total > nam_capacity) {
            GBSA_CUDA(cudaStreamSynchronize(st));
            throw Error(GBSA_ERR_CAPACITY, "NAM capacity too small");
        }
    });
}

int gbsa_find_nams(gbsa_mapper* m, const gbsa_query_randstrobe* queries, const uint64_t* q_offsets, uint32_t n_reads,
                   int rescue, uint32_t rescue_cutoff, gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets,
                   float* frac) {
    return guarded([&] {
        cudaStream_t st = m->st;
        const uint32_t n = n_reads;
        const uint64_t nqt = q_offsets[n] - q_offsets[0];
        mapper_reserve(*m, n, std::max<uint64_t>(64, nqt));
        if (m->q_cap < nqt + 1) {
            m->q_cap = nqt + 1;
            m->q.release();
            m->q.resize(sizeof(Query) * m->q_cap);
            m->qaux.release();
            m->qaux.resize(4 * m->q_cap);
            m->qpos.release();
            m->qpos.resize(8 * m->q_cap);
        }
        // Lay the queries of each read out forward-first, each orientation ordered by
        // start (stable), which is the order randstrobes_query produces and in which the
        // reference's (query_start, ref_start) hit sort leaves them.
        std::vector<Query> hq(nqt + 1);
        std::vector<ReadRec> hr(n);
        std::vector<uint32_t> ord;
        uint64_t o = 0;
        for (uint32_t r = 0; r < n; ++r) {
            const uint64_t a = q_offsets[r], b = q_offsets[r + 1];
            ord.resize(b - a);
            std::iota(ord.begin(), ord.end(), 0u);
            std::stable_sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) {
                const auto& qx = queries[a + x];
                const auto& qy = queries[a + y];
                if ((qx.is_reverse != 0) != (qy.is_reverse != 0)) return qx.is_reverse == 0;
                return qx.start < qy.start;
            });
            uint32_t nf = 0;
            for (uint32_t j = 0; j < ord.size(); ++j) {
                const auto& q = queries[a + ord[j]];
                hq[o + j] = Query{q.hash, q.start, q.end};
                nf += q.is_reverse ? 0 : 1;
            }
            ReadRec R{};
            R.q_off = o;
            R.nq = nf;
            R.nq2 = (uint32_t)(b - a);
            hr[r] = R;
            o += b - a;
        }
        if (nqt) GBSA_CUDA(cudaMemcpyAsync(m->q.as<void>(), hq.data(), sizeof(Query) * nqt, cudaMemcpyHostToDevice, st));
        GBSA_CUDA(cudaMemcpyAsync(m->rec.as<void>(), hr.data(), sizeof(ReadRec) * n, cudaMemcpyHostToDevice, st));
        const MapConfig saved = m->cfg;
        m->cfg.rescue_level = 0;          // find_nams alone, or
        m->cfg.force_rescue = rescue ? 1 : 0;   // find_nams_rescue for every read
        m->cfg.rescue_cutoff = rescue_cutoff;
        uint64_t total = 0;
        try {
            total = run_pipeline(*m, nullptr, nullptr, nullptr, n, true, st);
        } catch (...) {
            m->cfg = saved;
            throw;
        }
        m->cfg = saved;
        GBSA_CUDA(cudaMemcpyAsync(nam_offsets, m->out_off.as<void>(), 8ull * (n + 1), cudaMemcpyDeviceToHost, st));
        m->out_nams.resize(sizeof(gbsa_nam) * (total + 1));
        launch_gather_nams(n, m->rec.as<ReadRec>(), m->nams.as<NamState>(), m->out_off.as<uint64_t>(),
                           m->out_nams.as<gbsa_nam>(), m->out_frac.as<float>(), nullptr, st);
        if (frac) GBSA_CUDA(cudaMemcpyAsync(frac, m->out_frac.as<void>(), 4ull * n, cudaMemcpyDeviceToHost, st));
        if (total <= nam_capacity && total)
            GBSA_CUDA(cudaMemcpyAsync(nams, m->out_nams.as<void>(), sizeof(gbsa_nam) * total, cudaMemcpyDeviceToHost,
                                      st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (total > nam_capacity) throw Error(GBSA_ERR_CAPACITY, "NAM capacity too small");
    });
}

// Instrumentation used by the benchmark: enable the algorithmic-byte counter and read
// the value of the last batch.
void gbsa_mapper_set_count_bytes(gbsa_mapper* m, int on) { m->count_bytes = on; }
uint64_t gbsa_mapper_last_alg_bytes(const gbsa_mapper* m) { return m->alg_bytes; }
uint64_t gbsa_mapper_last_alg_sectors(const gbsa_mapper* m) { return m->alg_sectors; }

int gbsa_mapper_set_profile(gbsa_mapper* m, int on) {
    return guarded([&] {
        if (on && !m->ev[0])
            for (auto& e : m->ev) GBSA_CUDA(cudaEventCreate(&e));
        m->profile = on;
    });
}

int gbsa_mapper_last_counts(const gbsa_mapper* m, uint64_t* out) {
    out[0] = m->last.q_used;
    out[1] = m->last.hit_used;
    out[2] = m->last.nam_used;
    out[3] = m->last.n_rescue + m->last.n_rescue_heavy;
    out[4] = m->last.n_long;
    out[5] = m->last.scratch_used;
    out[6] = m->last.n_big;
    return GBSA_OK;
}

uint64_t gbsa_mapper_retries(const gbsa_mapper* m) { return m->retries + (m->twin ? m->twin->retries : 0); }

int gbsa_mapper_fused_lookup(const gbsa_mapper* m) { return m->fused ? 1 : 0; }

int gbsa_mapper_set_l2_window(gbsa_mapper* m, int on, uint64_t* window_bytes) {
    return guarded([&] {
        for (gbsa_mapper* x : {m, m->twin}) {
            if (!x) continue;
            GBSA_CUDA(cudaStreamSynchronize(x->st));
            GBSA_CUDA(cudaStreamSynchronize(x->side));
            l2_window_attach(*x, false);
            x->use_l2_window = on != 0;
            l2_window_attach(*x, true);
        }
        if (window_bytes) *window_bytes = m->cfg.l2_bytes;
    });
}

int gbsa_mapper_set_rescue_block(gbsa_mapper* m, uint32_t hits) {
    m->cfg.rescue_block_hits = hits;
    return GBSA_OK;
}

int gbsa_mapper_set_fuse_limit(gbsa_mapper* m, uint64_t index_bytes) {
    m->fuse_index_bytes = index_bytes;
    if (m->twin) m->twin->fuse_index_bytes = index_bytes;
    return GBSA_OK;
}

int gbsa_mapper_rescue_cycles(const gbsa_mapper* m, uint64_t* out, uint32_t cap, uint32_t* n_out) {
    return guarded([&] {
        const uint32_t total = m->last.n_rescue + m->last.n_rescue_heavy;
        const uint32_t n = std::min<uint32_t>(cap / 8, total);
        n_out[0] = total;
        n_out[1] = m->last.n_heavy + m->last.n_huge;
        if (m->profile && n && m->resc_cycles.size() >= 64ull * n)
            GBSA_CUDA(cudaMemcpy(out, m->resc_cycles.as<void>(), 64ull * n, cudaMemcpyDeviceToHost));
    });
}

int gbsa_mapper_nam_cycles(const gbsa_mapper* m, uint64_t* out, uint32_t cap, uint32_t* n_out) {
    return guarded([&] {
        const uint32_t n = std::min<uint32_t>(cap / 4, m->last.n_big);
        n_out[0] = m->last.n_big;
        if (m->profile && n && m->nam_notes.size() >= 32ull * n)
            GBSA_CUDA(cudaMemcpy(out, m->nam_notes.as<void>(), 32ull * n, cudaMemcpyDeviceToHost));
    });
}

int gbsa_mapper_stage_ms(const gbsa_mapper* m, float* ms, int n) {
    for (int i = 0; i < n && i < 7; ++i) ms[i] = m->stage_ms[i];
    return GBSA_OK;
}

}  // extern "C"
