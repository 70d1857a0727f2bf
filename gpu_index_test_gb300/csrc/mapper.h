// mapper.h — the mapper behind the opaque gbsa_mapper handle (work areas, streams,
// pipelining state) and the batch steps shared by the plain and batched forms.
#pragma once

#include "index.h"
#include "map.cuh"
#include "runtime.h"

struct gbsa_batcher;

struct gbsa_mapper {
    const gbsa_index* idx = nullptr;
    gbsa_map_options opt{};
    gbsa::MapConfig cfg{};
    cudaStream_t st = nullptr;
    cudaStream_t side = nullptr;                           // rescue chain, beside the NAM kernels
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr, rescue_ev = nullptr;
    cudaStream_t side_lo = nullptr;                        // rescue chain of a batch on a caller's stream
    cudaStream_t early = nullptr;                          // seeding + lookup of pipelined chunks
    cudaEvent_t early_ev = nullptr;
    uint32_t max_reads = 0;
    uint64_t max_bases = 0;
    gbsa::DeviceBuffer seqs, offs, lens, rec, q, qaux, qpos, hits, nams, slots, ovf, lists, ctr, long_scratch, cnt,
        out_off, out_nams, out_frac, out_resc, resc_cycles, nam_notes, jobs, side_slots, lane_lists;
    uint64_t q_cap = 0, hit_cap = 0, nam_cap = 0, ovf_cap = 0, slot_bytes = 0;
    uint32_t long_warps = 0;
    gbsa::PinnedBuffer h_seqs, h_meta, h_out;
    gbsa::PinnedBuffer h_status;   // counters + NAM total of the last enqueued batch
    // pipelined host entry point: copy streams, the twin that maps every other chunk,
    // events (reads copied in, batch done), two output slots that a batch's results wait
    // in to be copied out, and NAMs per read seen so far (sizes the slots)
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    gbsa_mapper* twin = nullptr;
    cudaEvent_t in_ready = nullptr, done_ev = nullptr;
    struct OutSlot {
        gbsa::DeviceBuffer nams, frac, resc, off, off_g;   // off: batch offsets, off_g: call offsets
        uint64_t cap = 0;                                 // NAM records nams holds
        cudaEvent_t free = nullptr;                       // copies out of the slot ended
    } outs[2];
    double nams_per_read = 16.0;
    uint64_t retries = 0;   // batches run again after a work area grew
    bool fused = false;     // the last batch ran seeding and lookup as one kernel
    uint64_t fuse_index_bytes = 2ull << 30;   // largest index (entry bytes) seeded and looked up in one kernel
    uint32_t pipe_chunks = 2;   // full chunks a large gbsa_map_reads call is cut into
    gbsa::Workspace ws;       // temporary device buffers of the prefix scans
    uint64_t alg_bytes = 0;   // algorithmic bytes of the last batch (when counting)
    uint64_t alg_sectors = 0; // 32 B sectors of the lookup's gathers in the last batch (when counting)
    int count_bytes = 0;
    bool use_l2_window = true;   // hold the bucket table in L2 when it fits a window
    int profile = 0;          // record per-stage CUDA events
    cudaEvent_t ev[8] = {};
    float stage_ms[8] = {};
    gbsa::Counters last{};    // device counters of the last batch
};


namespace gbsa {

// Where a batch's NAM records, fractions and rescue flags go, when the batch gathers
// them itself.
struct GatherTarget {
    gbsa_nam* nams;
    uint64_t cap;   // records nams holds (the gather writes no further)
    float* frac;
    uint8_t* resc;
};

// A batch of the batched form: its descriptor in device memory, the seeding + lookup
// kernel variant and the read capacity of the work areas the batch runs over.
struct BatchMode {
    const BatchDesc* desc;
    int variant;
    uint32_t cap;
};

void mapper_reserve(gbsa_mapper& m, uint32_t n, uint64_t bases);
// Enqueues one attempt at a batch (see capi.cu); bm selects the batched form.
void enqueue_batch(gbsa_mapper& m, const uint8_t* d_seqs, const uint64_t* d_offs, const uint32_t* d_lens, uint32_t n,
                   bool seeded, cudaStream_t st, cudaStream_t early = nullptr, const GatherTarget* gt = nullptr,
                   const BatchMode* bm = nullptr);
// Reads the status of a completed batch: false when a work area grew and the batch must
// run again; throws on a fatal status.
bool check_batch(gbsa_mapper& m, bool seeded);
uint64_t batch_total(gbsa_mapper& m);
void l2_window_attach(gbsa_mapper& m, bool on);
// Copies n host reads into the mapper's device read buffers on stream st (one transfer
// of their span when they lie back to back); grows the work areas for them.  Returns
// their bases.
uint64_t stage_reads(gbsa_mapper& m, const char* seqs, const uint64_t* offsets, const uint32_t* lengths, uint32_t n,
                     cudaStream_t st);

// One request of the served form: host reads in, host results out (as gbsa_map_reads).
struct ServeRequest {
    const char* seqs;
    const uint64_t* offsets;
    const uint32_t* lengths;
    uint32_t n_reads;
    gbsa_nam* nams;
    uint64_t nam_capacity;
    uint64_t* nam_offsets;
    float* frac;
    uint8_t* rescued;
};

// Maps k requests as one batch of the batcher's first set of work areas (one graph
// launch): their reads are staged back to back, and each request's NAMs, offsets,
// fractions and flags are copied straight from the batch's device outputs into its
// own buffers.  status[j] is GBSA_OK, or GBSA_ERR_CAPACITY when request j's NAMs do
// not fit its nam_capacity (its offsets are still written); totals[j] its NAM count.
void batcher_run_requests(gbsa_batcher& b, const ServeRequest* rq, uint32_t k, int* status, uint64_t* totals);
// Sizes every buffer of the batcher's first set of work areas for batches of up to
// max_reads reads (NAM outputs for nams_per_read NAMs per read) and captures its graph
// with one batch of pseudo-random reads, so that later batches allocate nothing.
void batcher_warm_up(gbsa_batcher& b, uint32_t max_reads, double nams_per_read);

}  // namespace gbsa
