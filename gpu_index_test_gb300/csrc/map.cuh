// map.cuh — the mapper: device work areas and the kernels of the read → NAM path.
#pragma once

#include "index.h"
#include "nam.cuh"
#include "seed.cuh"

namespace gbsa {

// Per-read bookkeeping of one batch.
struct ReadRec {
    uint64_t q_off;      // first query randstrobe in the query arena
    uint32_t nq;         // forward query randstrobes (they come first, by start)
    uint32_t nq2;        // all query randstrobes (the reverse ones follow, by start)
    uint32_t flags;      // kRead* bits
    uint32_t pad0;
    uint64_t hit_off;    // first hit in the hit arena
    uint32_t n_hits;
    float frac;          // nonrepetitive_fraction
    uint64_t nam_off;    // first NAM in the NAM arena
    uint32_t n_nams;
    uint32_t n_found;    // query randstrobes found in the index
};

constexpr uint32_t kReadRescue = 1u << 0;   // NAMs come from the rescue path
constexpr uint32_t kReadLong = 1u << 1;     // seeded by the scratch-memory kernel
constexpr uint32_t kReadFailed = 1u << 2;   // a capacity limit was hit

// Device counters of one batch (bump allocators, work lists, status).
struct Counters {
    unsigned long long q_used;
    unsigned long long hit_used;
    unsigned long long nam_used;
    unsigned long long scratch_used;
    unsigned long long alg_bytes;   // roofline numerator (see k_lookup)
    unsigned long long alg_sectors; // distinct 32 B sectors of the lookup's gathers (see k_lookup)
    unsigned int n_rescue;        // rescued reads on the light end of the rescue list
    unsigned int n_long;
    unsigned int status;
    unsigned int n_big;    // reads merged by the warp-cooperative NAM kernel
    unsigned int n_heavy;  // rescued reads whose NAMs the block-per-read sort kernel orders (small tile)
    unsigned int n_rescue_heavy;  // rescued reads on the heavy end of the rescue list
    unsigned int n_huge;   // rescued reads whose NAMs the large-tile block sort orders
    unsigned int rescue_next;  // next rescue-list entry to take (k_rescue's work counter)
    unsigned int lane_cnt[16]; // reads per hit-count bucket of the lane NAM kernel
    unsigned int queue_head;   // next read (work item) of the seeding (+ lookup) kernel
    unsigned int queue_head2;  // next read of the lookup kernel, when it runs on its own
    unsigned int rescue_block_next;  // next heavy rescued read to take a block (k_rescue)
};

// A batch of the batched form, in device memory: the kernels of a captured batch graph
// read the batch's reads, sizes and output buffers from here, so one graph serves
// every batch that fits the work areas it was captured with.  Work item i is reads
// [items[i], items[i + 1]) (a single-end read, or both mates of a pair); with items ==
// nullptr every read is an item.
struct BatchDesc {
    const uint8_t* seqs;
    const uint64_t* offs;
    const uint32_t* lens;
    const uint32_t* items;
    uint32_t n_reads;
    uint32_t n_items;
    gbsa_nam* out;          // NAM records (at most out_cap are written)
    uint64_t out_cap;
    uint64_t* out_off;      // n_reads + 1 NAM offsets
    float* frac;            // may be null
    uint8_t* rescued;       // may be null
};

constexpr uint32_t kLaneBuckets = 13;   // hit-count buckets of the lane NAM kernel (<= 16)

// A read whose NAMs are sorted by the block-per-read sort kernel.
struct SortJob {
    NamState* closed;   // its NAMs (unsorted)
    NamKey* keys;       // room for next_pow2(n) sort keys
    uint32_t n;
    uint32_t read;
    uint32_t note;      // its index on the rescue list
    uint32_t pad;
};

struct Arenas {
    Query* q;
    uint64_t q_cap;
    uint32_t* q_aux;         // per query: hits emitted (lookup) / exclusive offset
    uint64_t* q_pos;         // per query: index position of its hash (or kNotFound)
    HitPacked* hits;
    uint64_t hit_cap;
    NamState* nams;          // per read, sorted (converted to Nam records on output)
    uint64_t nam_cap;
    uint8_t* slots;          // per-warp scratch slots of the NAM / rescue kernels
    uint64_t slot_bytes;
    uint8_t* ovf;            // shared overflow scratch (bump-allocated)
    uint64_t ovf_cap;
    uint32_t* rescue_list;   // light reads from the front, heavy ones from the back
    uint32_t rescue_cap;
    uint32_t* long_list;
    uint32_t* big_list;
    uint32_t* lane_lists;    // kLaneBuckets lists of lane_cap reads each
    uint32_t lane_cap;
    SortJob* sort_jobs;      // small-tile jobs from the front, large-tile ones from the back
    uint32_t jobs_cap;
    uint64_t* rescue_cycles;   // optional: 8 notes per rescued read (cycles per phase, sizes)
    uint64_t* nam_cycles;      // optional: SM cycles, hits and NAMs of each read of the warp NAM kernel
};

struct MapConfig {
    int rescue_level;
    uint32_t rescue_cutoff;
    uint32_t count_cap;
    int sort_mode;
    int count_bytes;    // accumulate algorithmic bytes
    int force_rescue;   // every read takes the rescue path (find_nams_rescue entry point)
    // L2 access-policy window of the kernels that probe the index (the bucket table,
    // marked persisting), or l2_bytes == 0 for none; host side only
    const void* l2_base;
    uint64_t l2_bytes;
    float l2_hit_ratio;
    // NAM phase shape: reads with at most lane_max_hits hits (<= kLaneMaxHitsCap) are
    // merged by one lane each, heavier ones by a warp each; sort_variant picks the block
    // size of the sort of rescued reads with many NAMs (0: 256 threads, 1: 512)
    uint32_t lane_max_hits;
    int sort_variant;
    // register budgets of the NAM merge kernels (resident blocks they must fit):
    // lane_variant 0 none, 1 six blocks, 2 eight (3-6: the open NAMs in registers,
    // k_nams_lane_r: 10 slots at 168 / 128 registers, 6 slots at 96 / 124); warp_variant
    // 0 five, 1 six, 2 eight
    // (3, 4: 96 / 80 registers launched four blocks per SM)
    int lane_variant;
    int warp_variant;
    // rescued reads whose estimated merge hits (their seeds' runs up to the count cap)
    // reach rescue_block_hits are merged by a whole block each, ahead of the others
    // (0: every rescued read by one warp, those above kRescueHeavyHits first)
    uint32_t rescue_block_hits;
};
constexpr uint32_t kLaneMaxHitsCap = 160;
constexpr uint32_t kRescueBlockHitsDefault = 4000;   // a new mapper's rescue_block_hits

// Reads shorter than this (and with at most kSmemSyncmers syncmers) are seeded
// with shared-memory buffers; the rest by the scratch-memory kernel.
constexpr uint32_t kSmemMaxLen = 1024;
constexpr uint32_t kSmemSyncmers = 256;
// Global scratch per warp of the long-read seeding kernel.
constexpr uint32_t kLongWords = GBSA_MAX_READ_LEN / 32 + 4;
constexpr size_t kLongSlotBytes = (size_t)kLongWords * 8 + (size_t)kLongWords * 4 + 64 * 8 +
                                  (size_t)GBSA_MAX_READ_LEN * 8 + (size_t)GBSA_MAX_READ_LEN * 4;

// Warps launched by the NAM and rescue kernels (one scratch slot each).
uint32_t nam_kernel_warps(uint32_t n_reads);

void launch_seed(const DevParams& P, const uint8_t* seqs, const uint64_t* offs, const uint32_t* lens, uint32_t n,
                 ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st);
void launch_seed_long(const DevParams& P, const uint8_t* seqs, const uint64_t* offs, const uint32_t* lens,
                      ReadRec* rec, Arenas A, Counters* ctr, uint8_t* long_scratch, uint32_t long_warps,
                      cudaStream_t st, const BatchDesc* desc = nullptr);
// Batched form: seeding and lookup in one persistent kernel whose warps pull work items
// (a read, or both mates of a pair) from a device queue (ctr->queue_head) until the
// batch's items run out; desc gives the reads and their count.  variant selects the
// kernel's shape (warps per block, resident blocks per SM, shared-memory read window);
// see batch_variant().
struct SeedVariant {
    int warps;            // warps per block
    int blocks_per_sm;    // resident blocks per SM (launch bound and grid)
    uint32_t max_len;     // longest read seeded in shared memory
    uint32_t syncmers;    // syncmer buffer per warp
};
constexpr int kSeedVariants = 6;
SeedVariant seed_variant(int v);
// lookup false: seeding alone (the lookup then runs as launch_lookup with desc).
void launch_seed_lookup_queue(const DevParams& P, const IndexView& I, const MapConfig& C, const BatchDesc* desc,
                              ReadRec* rec, Arenas A, Counters* ctr, int variant, bool lookup, cudaStream_t st);
// Main path: seeding and lookup fused (a warp per read); reads too long for the
// shared-memory buffers are seeded by launch_seed_long and looked up by launch_lookup_long.
void launch_seed_lookup(const DevParams& P, const IndexView& I, const MapConfig& C, const uint8_t* seqs,
                        const uint64_t* offs, const uint32_t* lens, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                        cudaStream_t st);
void launch_lookup_long(const IndexView& I, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                        cudaStream_t st);
void launch_lookup(const IndexView& I, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                   cudaStream_t st, const BatchDesc* desc = nullptr);
void launch_nams(const IndexView& I, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                 cudaStream_t st);
void launch_bucket_reads(uint32_t n, uint32_t lane_max_hits, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st,
                         const BatchDesc* desc = nullptr);
void launch_nams_warp(const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st);
void launch_rescue(const IndexView& I, const MapConfig& C, uint32_t n_reads, ReadRec* rec, Arenas A, Counters* ctr,
                   cudaStream_t st);
void launch_sort_jobs(const MapConfig& C, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st);
// mode 0: every read; 1: the reads that were not rescued; 2: the rescued reads (A and
// ctr give the rescue list; needed for mode 2 only).
// With desc (batched form): n is the work areas' read capacity, the batch's read count,
// output buffers and capacity come from desc, and mode 1 also copies the NAM offsets of
// reads [0, desc->n_reads] (out_off[n] holding the total) to desc->out_off.
void launch_gather_nams(uint32_t n, const ReadRec* rec, const NamState* arena, const uint64_t* out_off,
                        gbsa_nam* out, float* frac, uint8_t* rescued, cudaStream_t st, uint64_t out_cap = ~0ull,
                        int mode = 0, const Arenas* A = nullptr, const Counters* ctr = nullptr,
                        const BatchDesc* desc = nullptr);
void launch_gather_queries(uint32_t n, const ReadRec* rec, const Query* arena, const uint64_t* out_off,
                           gbsa_query_randstrobe* out, cudaStream_t st);
void launch_find(const IndexView& I, const uint64_t* hashes, uint64_t n, uint64_t* pos, cudaStream_t st);
void launch_get_count(const IndexView& I, const uint64_t* pos, uint64_t n, uint32_t* counts, cudaStream_t st);
// With desc: out[r] for r < n, 0 for the slots at or past desc->n_reads.
void launch_read_counts(uint32_t n, const ReadRec* rec, int what, uint64_t* out, cudaStream_t st,
                        const BatchDesc* desc = nullptr);
void launch_offsets_add(const uint64_t* in, uint64_t* out, uint64_t n, uint64_t base, cudaStream_t st);
void launch_reset_recs(uint32_t n, ReadRec* rec, cudaStream_t st);
// Zeroes the records of reads [0, desc->n_reads) (every field).
void launch_clear_recs(uint32_t cap, ReadRec* rec, const BatchDesc* desc, cudaStream_t st);

}  // namespace gbsa
