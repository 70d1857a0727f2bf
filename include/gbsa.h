/*
 * gbsa.h — C-ABI of the GB300-native strobealign seeding → index lookup → NAM path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (GBSA_OK == 0) and never throws across the boundary.  The text of
 * the last error on the calling thread is returned by gbsa_last_error().
 *
 * Record layouts are byte-identical to the reference structs so that buffers can
 * be handed over without conversion:
 *   gbsa_ref_randstrobe   == RefRandstrobe   (step2/randstrobes.hpp:65-94, 16 B)
 *   gbsa_query_randstrobe == QueryRandstrobe (step2/randstrobes.hpp:96-101, 24 B)
 *   gbsa_nam              == Nam             (step2/my_struct.hpp:48-93, 44 B)
 *   gbsa_params           mirrors IndexParameters (step2/indexparameters.hpp:72-95)
 *
 * Entry points that take HOST buffers copy them to the device and the results
 * back inside the call (one CUDA stream per call).  Entry points whose name ends
 * in `_device` take DEVICE pointers and a cudaStream_t (passed as void*) and do
 * no host<->device copies of the payload.
 */
#ifndef GBSA_H
#define GBSA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define GBSA_OK                 0
#define GBSA_ERR_PARAM          1  /* BadParameter (step2/exceptions.hpp:7-10) */
#define GBSA_ERR_CUDA           2  /* a CUDA runtime call failed */
#define GBSA_ERR_NOMEM          3  /* device or pinned allocation failed */
#define GBSA_ERR_INDEX_FILE     4  /* InvalidIndexFile (step2/exceptions.hpp:17-20) */
#define GBSA_ERR_CAPACITY       5  /* a caller-sized output buffer is too small */
#define GBSA_ERR_READ_TOO_LONG  6  /* a read exceeds GBSA_MAX_READ_LEN */
#define GBSA_ERR_NO_DEVICE      7  /* no CUDA device visible */
#define GBSA_ERR_DEVICE_STATUS  8  /* a kernel reported an internal limit */
#define GBSA_ERR_FORMAT         9  /* malformed FASTQ input */

/* Longest read (bases) accepted by the seeding kernels. */
#define GBSA_MAX_READ_LEN 4096

/* "use the profile default" marker of IndexParameters::from_read_length
 * (step2/indexparameters.hpp:78, numeric_limits<int>::min()). */
#define GBSA_DEFAULT (-2147483647 - 1)

/* ---- records -------------------------------------------------------------- */

/* IndexParameters (step2/indexparameters.hpp:72-95) flattened. */
typedef struct gbsa_params {
    int32_t  canonical_read_length;
    int32_t  k;
    int32_t  s;
    int32_t  t_syncmer;       /* (k - s) / 2 + 1 */
    int32_t  l;
    int32_t  u;
    uint64_t q;               /* 2^c - 1 */
    int32_t  max_dist;
    uint32_t w_min;           /* max(0, k/(k-s+1) + l) */
    uint32_t w_max;           /* k/(k-s+1) + u */
    int32_t  _pad;
} gbsa_params;

/* RefRandstrobe (step2/randstrobes.hpp:65-94). packed = ref_index << 8 | strobe2 offset. */
typedef struct gbsa_ref_randstrobe {
    uint64_t hash;
    uint32_t position;
    uint32_t packed;
} gbsa_ref_randstrobe;

/* QueryRandstrobe (step2/randstrobes.hpp:96-101). */
typedef struct gbsa_query_randstrobe {
    uint64_t hash;
    uint32_t start;
    uint32_t end;
    uint8_t  is_reverse;
    uint8_t  _pad[7];
} gbsa_query_randstrobe;

/* Nam (step2/my_struct.hpp:48-62). */
typedef struct gbsa_nam {
    int32_t nam_id;
    int32_t query_start;
    int32_t query_end;
    int32_t query_prev_hit_startpos;
    int32_t ref_start;
    int32_t ref_end;
    int32_t ref_prev_hit_startpos;
    int32_t n_hits;
    int32_t ref_id;
    float   score;
    uint8_t is_rc;
    uint8_t _pad[3];
} gbsa_nam;

/* IndexCreationStatistics (step2/index.hpp:22-35), counters only. */
typedef struct gbsa_index_info {
    uint64_t size;                 /* number of RefRandstrobe entries */
    int32_t  bits;
    uint32_t filter_cutoff;
    uint64_t tot_strobemer_count;
    uint64_t tot_occur_once;
    uint64_t tot_high_ab;
    uint64_t tot_mid_ab;
    uint64_t index_cutoff;
    uint64_t distinct_strobemers;
} gbsa_index_info;

/* NAM output order. */
#define GBSA_SORT_SCORE       0  /* score desc, is_rc, ref_id, qs, qe, rs, re, n_hits desc */
#define GBSA_SORT_REF_MATE2   1  /* Nam::operator< (step2/my_struct.hpp:78-92) made total */
#define GBSA_SORT_REF_MATE1   2  /* sort_nams_single2 (step2/main.cu:2271-2289) made total */

/* Mate layouts of the NAM lists given to gbsa_classify_pairs_device: pair i is read
 * ends (2i, 2i+1), or (i, i + n_pairs) as in the reference's global_nams. */
#define GBSA_PAIRS_INTERLEAVED 0
#define GBSA_PAIRS_HALVES 1

typedef struct gbsa_map_options {
    int32_t  rescue_level;      /* R (step2/cmdline.hpp:56); rescue runs when R > 1 */
    uint32_t rescue_count_cap;  /* 1000 = CPU find_nams_rescue (step2/nam.cu:964); 100 = step2/main.cu:39 */
    int32_t  sort_mode;         /* GBSA_SORT_* */
    int32_t  _pad;
} gbsa_map_options;

typedef struct gbsa_index  gbsa_index;
typedef struct gbsa_mapper gbsa_mapper;

/* ---- errors / device ------------------------------------------------------- */
const char* gbsa_last_error(void);
int gbsa_version(void);
/* Number of kernel launches this library has issued in this process (all threads). */
uint64_t gbsa_launch_count(void);

/* ---- parameters ------------------------------------------------------------ */
/* IndexParameters::from_read_length (step2/indexparameters.cpp:150-182). */
int gbsa_params_from_read_length(int read_length, int k, int s, int l, int u, int c,
                                 int max_seed_len, gbsa_params* out);
/* IndexParameters(r, k, s, l, u, q, max_dist) (step2/indexparameters.hpp:80-85). */
int gbsa_params_make(uint64_t canonical_read_length, int k, int s, int l, int u, int q,
                     int max_dist, gbsa_params* out);

/* ---- index ------------------------------------------------------------------ */
/* StrobemerIndex::pick_bits (step2/index.cu:137-141). */
int gbsa_pick_bits(const gbsa_params* p, uint64_t total_length);

/* StrobemerIndex(references, parameters, bits) + populate(f, n_threads)
 * (step2/index.hpp:39-54; body restated from step2/index.cu:143-311).
 * Contig i is seqs[offsets[i] .. offsets[i] + lengths[i]).  bits == -1 picks bits. */
int gbsa_index_build(const gbsa_params* p, const char* seqs, const uint64_t* offsets,
                     const uint64_t* lengths, uint32_t n_contigs, int bits, float f,
                     gbsa_index** out);
/* Upload an index held in host memory (e.g. read from a .sti file). */
int gbsa_index_load(const gbsa_params* p, const gbsa_ref_randstrobe* randstrobes, uint64_t n,
                    const uint64_t* start_indices, int bits, uint32_t filter_cutoff,
                    gbsa_index** out);
/* StrobemerIndex::read / write, .sti format version 2 (step2/index.cu:73-134). */
int gbsa_index_read_sti(const char* path, const gbsa_params* p, gbsa_index** out);
int gbsa_index_write_sti(const gbsa_index* idx, const char* path);
int gbsa_index_get_info(const gbsa_index* idx, gbsa_index_info* out);
int gbsa_index_get_params(const gbsa_index* idx, gbsa_params* out);
/* Copy the device tables to host: randstrobes[size], start_indices[2^bits + 1]. */
int gbsa_index_export(const gbsa_index* idx, gbsa_ref_randstrobe* randstrobes,
                      uint64_t* start_indices);
void gbsa_index_free(gbsa_index* idx);

/* StrobemerIndex::find (step2/index.hpp:57-81) for a batch; not found = UINT64_MAX. */
int gbsa_find(const gbsa_index* idx, const uint64_t* hashes, uint64_t n, uint64_t* positions);
/* StrobemerIndex::get_count (step2/index.hpp:115-147) for found positions. */
int gbsa_get_count(const gbsa_index* idx, const uint64_t* positions, uint64_t n, uint32_t* counts);

/* ---- seeding ------------------------------------------------------------------ */
/* randstrobes_query (step2/randstrobes.cu:195-241) for a batch of reads.  Read i is
 * seqs[offsets[i] .. offsets[i] + lengths[i]).  Randstrobes of read i are written to
 * out[out_offsets[i] .. out_offsets[i+1]) (forward ones first, then reverse-complement
 * ones, as the reference orders them).  *out_total receives the total; if it exceeds
 * out_capacity, GBSA_ERR_CAPACITY is returned and nothing but out_offsets is written. */
int gbsa_randstrobes_query(const gbsa_params* p, const char* seqs, const uint64_t* offsets,
                           const uint32_t* lengths, uint32_t n_reads,
                           gbsa_query_randstrobe* out, uint64_t out_capacity,
                           uint64_t* out_offsets, uint64_t* out_total);

/* randstrobes_query for callers that cannot allocate device memory: callers whose
 * device memory is owned by a host framework's pool, and serving loops that must
 * not call cudaMalloc / cudaFree (cudaFree waits for the whole device).  No
 * counterpart in the reference.  Reads and outputs are in device memory and work is
 * queued on `stream`; the call allocates nothing.  Its only scratch is a file-scope
 * device array of about 3.3 MB (64 warp slots for reads of up to GBSA_MAX_READ_LEN
 * bases), held by every GPU that loads the library until the process exits.  The
 * first call on a device looks up that array's address; calls that overlap on the
 * GPU race on the array.  Each call waits for
 * its stream before it returns (it reads the total back).  d_out_offsets has
 * n_reads + 1 entries and is always filled; *out_total receives the total; reads
 * longer than GBSA_MAX_READ_LEN give GBSA_ERR_READ_TOO_LONG and a total above
 * out_capacity gives GBSA_ERR_CAPACITY (nothing written to d_out). */
int gbsa_randstrobes_query_noalloc(const gbsa_params* p, const char* d_seqs,
                                   const uint64_t* d_offsets, const uint32_t* d_lengths,
                                   uint32_t n_reads, gbsa_query_randstrobe* d_out,
                                   uint64_t out_capacity, uint64_t* d_out_offsets,
                                   uint64_t* out_total, void* stream);

/* ---- NAM path ---------------------------------------------------------------- */
/* A mapper owns the device work areas for batches of up to max_reads reads with up
 * to max_bases bases in total; both grow on demand.  The NAM phase's kernel shape (the
 * split between one lane and one warp per read, the block size of the rescued reads'
 * sort) is the one gbsa_batch_config_default gives. */
int gbsa_mapper_create(const gbsa_index* idx, const gbsa_map_options* opt,
                       uint32_t max_reads, uint64_t max_bases, gbsa_mapper** out);
void gbsa_mapper_free(gbsa_mapper* m);

/* Reads → NAMs: randstrobes_query + find_nams (+ find_nams_rescue when
 * nonrepetitive_fraction < 0.7 or no NAM was found and rescue_level > 1) + NAM sort,
 * for every read (step2/main.cu:4461-4597 chain; CPU find_nams step2/nam.cu:748-905).
 * NAMs of read i go to nams[nam_offsets[i] .. nam_offsets[i+1]).  frac[i] receives
 * nonrepetitive_fraction, rescued[i] is 1 when the rescue path produced the NAMs.
 * frac and rescued may be NULL.  If the NAM total exceeds nam_capacity the call
 * returns GBSA_ERR_CAPACITY with nam_offsets filled so that the caller can resize. */
int gbsa_map_reads(gbsa_mapper* m, const char* seqs, const uint64_t* offsets,
                   const uint32_t* lengths, uint32_t n_reads,
                   gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets,
                   float* frac, uint8_t* rescued);

/* Same, with every buffer in device memory and work queued on `stream`.  The call
 * returns after the stream work is queued and the NAM total is known (it syncs
 * the stream once to read the total). */
int gbsa_map_reads_device(gbsa_mapper* m, const char* d_seqs, const uint64_t* d_offsets,
                          const uint32_t* d_lengths, uint32_t n_reads,
                          gbsa_nam* d_nams, uint64_t nam_capacity, uint64_t* d_nam_offsets,
                          float* d_frac, uint8_t* d_rescued, uint64_t* nam_total,
                          void* stream);

/* find_nams (step2/nam.hpp:11-14) / find_nams_rescue (step2/nam.hpp:16-20) for a batch
 * of already-seeded reads: queries of read i are queries[q_offsets[i] .. q_offsets[i+1]).
 * rescue == 0 runs find_nams (frac receives nonrepetitive_fraction), rescue == 1 runs
 * find_nams_rescue with rescue_cutoff.  NAMs are returned in the mapper's sort order. */
int gbsa_find_nams(gbsa_mapper* m, const gbsa_query_randstrobe* queries,
                   const uint64_t* q_offsets, uint32_t n_reads, int rescue,
                   uint32_t rescue_cutoff, gbsa_nam* nams, uint64_t nam_capacity,
                   uint64_t* nam_offsets, float* frac);

/* gbsa_map_reads cuts a call of at least 2 x 131072 reads into up to `chunks` full
 * chunks (default 2; when a full chunk has 262144 reads or more, the first is cut in
 * half and the last into two quarters) that alternate between the mapper's work areas
 * and a second set, and overlaps the transfers of one chunk with the mapping of the
 * next; 1 maps the call as one batch.  No reference counterpart. */
int gbsa_mapper_set_pipeline(gbsa_mapper* m, uint32_t chunks);

/* ---- batched form ------------------------------------------------------------ */
/* Shape of the batched form's kernels, picked by the autotuner
 * (gpu_index_test_gb300/autotune.py) and committed as gpu_index_test_gb300/tuned.json,
 * which the library reads from its own directory.  The results do not depend on it. */
typedef struct gbsa_batch_config {
    int32_t  seed_variant;   /* persistent seeding + lookup kernel: 0 8 warps x 6 blocks/SM, reads up to
                                512 bases in shared memory; 1 8 x 5; 2 4 x 12; 3 8 x 7, 256 bases;
                                4 16 x 3; 5 8 x 6, 256 bases (longer reads take the long-read path) */
    uint32_t lane_max_hits;  /* reads with at most this many hits (1-160) are merged by one lane,
                                heavier ones by a warp */
    int32_t  sort_variant;   /* block size of the sort of rescued reads with many NAMs: 0 256, 1 512 */
    uint32_t chunk_reads;    /* reads per batch of the host entry point (three batches in flight) */
    int32_t  lane_variant;   /* the lane-per-read NAM merge: open NAMs in shared memory with a register
                                budget of 0 no bound (96 registers), 1 six blocks (80), 2 eight (64); or
                                3 open NAMs in registers (168 registers, three blocks per SM), 4 the same
                                at 128 registers and two blocks per SM (room for the rescue kernel);
                                5, 6 six open NAMs per lane in registers (reads needing more go to the warp
                                merge) at 96 registers and three blocks per SM, or 124 and two */
    int32_t  warp_variant;   /* register budget of the warp-per-read NAM merge: 0 five blocks (96 registers),
                                1 six (80), 2 eight (64), launched 5 blocks per SM; 3 (96) and 4 (80)
                                launched 4 blocks per SM; fewer registers leave room for the rescued
                                reads' sorts beside it */
    uint32_t rescue_block_hits;  /* as gbsa_mapper_set_rescue_block (0: every rescued read by one warp) */
    uint32_t _reserved;          /* 0 */
} gbsa_batch_config;

typedef struct gbsa_batcher gbsa_batcher;

/* The committed tuned configuration (*from_file = 1), or the built-in one (0) when the
 * file is absent or malformed.  No reference counterpart. */
int gbsa_batch_config_default(gbsa_batch_config* out, int* from_file);

/* The batched form of gbsa_map_reads (the reference's per-stage launch chain with a
 * fixed batch, step2/main.cu:4458-4597, replaced): each batch is one launch of a CUDA
 * graph captured over the batcher's work areas, whose kernels read the batch (reads,
 * count, work items, outputs) from a device-resident descriptor.  Seeding and lookup
 * are one persistent kernel whose warps pull work items from a device queue; a work
 * item is reads [items[i], items[i+1]) (a single-end read, or the mates of a pair),
 * or every read is an item when items is NULL.  The first batch on a set of work areas
 * (and one that outgrows them) runs without the graph and captures it.  cfg NULL takes
 * gbsa_batch_config_default.  max_reads / max_bases size the work areas (they grow). */
int gbsa_batcher_create(const gbsa_index* idx, const gbsa_map_options* opt, const gbsa_batch_config* cfg,
                        uint32_t max_reads, uint64_t max_bases, gbsa_batcher** out);
void gbsa_batcher_free(gbsa_batcher* b);
int gbsa_batcher_get_config(const gbsa_batcher* b, gbsa_batch_config* out);
/* Graph launches, graph captures and batches run without a graph, since creation. */
int gbsa_batcher_stats(const gbsa_batcher* b, uint64_t* graph_launches, uint64_t* captures, uint64_t* eager_runs);
/* Stage timing of the batches (events inside the graph, captured anew when this changes)
 * and the stage times of the last batch of the device entry point, as
 * gbsa_mapper_set_profile / gbsa_mapper_stage_ms.  No reference counterpart. */
int gbsa_batcher_set_profile(gbsa_batcher* b, int on);
int gbsa_batcher_stage_ms(const gbsa_batcher* b, float* ms, int n);
/* Device buffers, as gbsa_map_reads_device; d_items (device, n_items + 1 entries, from 0
 * to n_reads, non-decreasing) may be NULL.  The batch runs after the work queued on
 * stream so far and the call returns once it has ended (the NAM total is read back);
 * stream then waits for it.  Results equal gbsa_map_reads'. */
int gbsa_batcher_map_device(gbsa_batcher* b, const char* d_seqs, const uint64_t* d_offsets, const uint32_t* d_lengths,
                            uint32_t n_reads, const uint32_t* d_items, uint32_t n_items, gbsa_nam* d_nams,
                            uint64_t nam_capacity, uint64_t* d_nam_offsets, float* d_frac, uint8_t* d_rescued,
                            uint64_t* nam_total, void* stream);
/* Host buffers, as gbsa_map_reads; items (host) may be NULL.  The call is cut into
 * batches of about chunk_reads reads at item boundaries that alternate between two
 * sets of work areas, copies overlapping the other set's graph. */
int gbsa_batcher_map(gbsa_batcher* b, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                     uint32_t n_reads, const uint32_t* items, uint32_t n_items, gbsa_nam* nams, uint64_t nam_capacity,
                     uint64_t* nam_offsets, float* frac, uint8_t* rescued);

/* ---- input staging ----------------------------------------------------------- */
/* Parses the complete 4-line FASTQ records of a chunk of a file (host threads) into
 * the reads layout of gbsa_map_reads: sequence bytes back to back in seqs, offsets
 * (n + 1 entries) and lengths (step2/main.cu:63-81, 4212-4240, 4404-4430 stage the
 * same layout).  CR before LF and blank lines between records are accepted.  When
 * `final` is 0, a record cut by the end of the chunk is left out and *consumed is
 * where it starts (the caller passes the rest again with the next chunk); when 1,
 * the chunk is the end of the file.  seq_capacity >= len and read_capacity >=
 * len / 8 + 1 always suffice; otherwise GBSA_ERR_CAPACITY reports the needed counts
 * in *n_reads / *n_bases.  Malformed input gives GBSA_ERR_FORMAT. */
int gbsa_fastq_parse(const char* buf, uint64_t len, int final, char* seqs, uint64_t seq_capacity,
                     uint64_t* offsets, uint32_t* lengths, uint32_t read_capacity,
                     uint32_t* n_reads, uint64_t* n_bases, uint64_t* consumed);
/* The same for chunks of two mate files: pairs interleaved (mate 1, mate 2), as many
 * pairs as both chunks hold complete; files of different record counts give
 * GBSA_ERR_FORMAT at the end. */
int gbsa_fastq_parse_pairs(const char* buf1, uint64_t len1, const char* buf2, uint64_t len2,
                           int final, char* seqs, uint64_t seq_capacity, uint64_t* offsets,
                           uint32_t* lengths, uint32_t read_capacity, uint32_t* n_reads,
                           uint64_t* n_bases, uint64_t* consumed1, uint64_t* consumed2);

/* ---- served form ------------------------------------------------------------- */
/* A server keeps the index resident and maps requests with continuous batching: it
 * owns up to `slots` batch slots (batchers of the batched form, each with its own
 * streams and device work areas for batches of up to batch_reads reads and
 * batch_bases bases), created against a device-memory budget (memory_budget bytes, 0:
 * half the memory free at creation; a slot is not added once its measured footprint
 * would exceed the budget, and at least one is).  Whenever a slot is free, its host
 * thread takes every request waiting at the head of the queue that still fits the
 * slot and maps them as one batch (one graph launch), so requests that arrive while
 * others are on the GPU share launches and overlap on the device; each request's
 * results are copied from the batch's device outputs into its own buffers and equal
 * gbsa_map_reads' for its reads.  Submit returns at once (GBSA_ERR_CAPACITY for a
 * request larger than a slot); the caller keeps a request's buffers alive until poll
 * reports its tag.  Poll returns up to cap completed requests (tag, status, NAM
 * total; a request whose NAMs exceed its nam_capacity completes with
 * GBSA_ERR_CAPACITY, its offsets written), waiting up to wait_ms for one (-1: until
 * one completes or none is in flight).  No reference counterpart. */
typedef struct gbsa_server gbsa_server;
typedef struct gbsa_server_config {
    uint32_t slots;          /* batch slots at most (1-64) */
    uint32_t batch_reads;    /* reads a batch holds (also the largest request) */
    uint64_t batch_bases;    /* bases a batch holds (0: 500 per read) */
    uint64_t memory_budget;  /* device bytes the slots may take (0: half the free memory) */
} gbsa_server_config;
int gbsa_server_create_ex(const gbsa_index* idx, const gbsa_map_options* opt, const gbsa_server_config* cfg,
                          gbsa_server** out);
/* gbsa_server_create_ex with slots = workers, batch_reads / batch_bases = the request
 * maxima and the default budget. */
int gbsa_server_create(const gbsa_index* idx, const gbsa_map_options* opt, uint32_t workers,
                       uint32_t max_reads_per_request, uint64_t max_bases_per_request,
                       gbsa_server** out);
/* Slots created, device bytes of one slot, the budget, and batches / requests mapped. */
int gbsa_server_info(const gbsa_server* s, uint32_t* slots, uint64_t* slot_bytes, uint64_t* budget,
                     uint64_t* batches, uint64_t* requests);
/* Graph launches, graph captures and batches run without a graph (the first batch of a
 * slot, and one that outgrew its work areas, which frees and allocates device memory)
 * over all slots since creation.  No reference counterpart. */
int gbsa_server_stats(const gbsa_server* s, uint64_t* graph_launches, uint64_t* captures, uint64_t* eager_runs);
int gbsa_server_submit(gbsa_server* s, const char* seqs, const uint64_t* offsets,
                       const uint32_t* lengths, uint32_t n_reads, gbsa_nam* nams,
                       uint64_t nam_capacity, uint64_t* nam_offsets, float* frac,
                       uint8_t* rescued, uint64_t tag);
uint32_t gbsa_server_poll(gbsa_server* s, uint64_t* tags, int* status, uint64_t* nam_totals,
                          uint32_t cap, int wait_ms);
void gbsa_server_free(gbsa_server* s);

/* A request of gbsa_server_replay: reads [start, start + n_reads) of the read pool,
 * submitted at_us microseconds after the replay starts. */
typedef struct gbsa_replay_request {
    double   at_us;
    uint64_t start;
    uint32_t n_reads;
    uint32_t _pad;
} gbsa_replay_request;

/* Load replay for measuring the served form: submits the requests at their times from a
 * native thread (in order; a request waits for one of n_bufs output buffer sets to be
 * free), collects completions on another, and, when exp_nams is not NULL, compares each
 * request's NAMs, offsets, fractions and flags byte for byte with the expected results of
 * the whole pool (exp_nam_offsets has n_pool + 1 entries; a request's offsets are relative
 * to its first read) on checker threads before its buffers are reused.  Buffer set b is
 * nams[b] (room for nam_cap NAMs), nam_offsets[b] (max_reads + 1), frac[b], rescued[b]
 * (max_reads).  Per request: submit_us / done_us (microseconds after the start, of the
 * submit call and of the completion's arrival), status (a GBSA_* code) and mismatch (1 when
 * the results differ from the expected ones).  No reference counterpart. */
int gbsa_server_replay(gbsa_server* s, const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                       const gbsa_replay_request* reqs, uint32_t n_req, uint32_t n_bufs, gbsa_nam* const* nams,
                       uint64_t nam_cap, uint64_t* const* nam_offsets, float* const* frac, uint8_t* const* rescued,
                       uint32_t max_reads, const gbsa_nam* exp_nams, const uint64_t* exp_nam_offsets,
                       const float* exp_frac, const uint8_t* exp_rescued, double* submit_us, double* done_us,
                       int* status, uint8_t* mismatch);

/* Read-pair classification after the NAM sort (gpu_pre_cal_type,
 * step2/main.cu:3552-3580): for each pair, 0 = no NAMs on either end, 1 = NAMs on
 * mate 1 only, 2 = mate 2 only, 3 = both ends' top_dropoff (main.cu:889-898) below
 * dropoff_threshold and their first NAMs a proper pair (is_proper_nam_pair,
 * main.cu:870-887, with insert-size mean mu and deviation sigma; the reference passes
 * a fresh estimate, mu = 300, sigma = 100), 4 = otherwise.  d_nams / d_nam_offsets
 * are the sorted NAM lists of 2 * n_pairs read ends as gbsa_map_reads_device writes
 * them; d_types receives n_pairs bytes.  All pointers are device memory; the kernel
 * runs on `stream` (0: the default stream). */
int gbsa_classify_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs,
                               int layout, float dropoff_threshold, float mu, float sigma,
                               uint8_t* d_types, void* stream);

/* NamPair (step2/main.cu:959-966) with the two NAMs as indices into the mates' NAM
 * lists (-1: no NAM on that end). */
typedef struct gbsa_nam_pair {
    int32_t score;   /* joint n_hits of a pair, or the one NAM's n_hits */
    int32_t i1;      /* index into mate 1's NAM list, or -1 */
    int32_t i2;      /* index into mate 2's NAM list, or -1 */
} gbsa_nam_pair;

#define GBSA_NAM_PAIRS_TOP_K 40   /* TOP_K of the reference's pair heap (main.cu:1428) */

/* NAM-pair scoring of the reads pairs whose two ends both have NAMs
 * (get_best_scoring_nam_pairs_sort3, step2/main.cu:1475-1716, as align_PE_part4 calls
 * it, main.cu:2026-2061): per reference id below 3000, mate-1 NAMs on the forward
 * strand paired with mate-2 NAMs on the reverse strand whose diagonals
 * max(0, ref_start - query_start) lie within [d1, d1 + mu + 10 sigma), then the
 * opposite strands within (d1 - (mu + 10 sigma), d1], mu and sigma truncated to
 * integers; pairs kept in a top-40 heap by joint n_hits with the reference's pruning
 * (half the best joint count); mate-1 NAMs in no pair (at most max_tries per reference
 * id and strand, n_hits at least half the best) and mate-2 NAMs in no pair (through
 * the heap) as single-end entries; the list sorted by the reference's comparator and
 * cut to max_tries.  Mate 1's NAMs must be in GBSA_SORT_REF_MATE1 order and mate 2's
 * in GBSA_SORT_REF_MATE2 order (gpu_sort_nams, main.cu:3449-3466).  For an absent end
 * the comparator reads a default Nam (all zero by Nam's member initialisers) with
 * ref_start -1, as here.  d_pairs receives max_tries records per pair (pair p
 * from p * max_tries on), d_counts the number written (0 when an end has no NAMs).
 * Device pointers; the kernel runs on `stream` (0: the default stream). */
int gbsa_nam_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs, int layout,
                          float mu, float sigma, uint32_t max_tries, gbsa_nam_pair* d_pairs, uint32_t* d_counts,
                          void* stream);

/* One step of a read pair's alignment, in the order align_PE_part1..4 run them
 * (step2/main.cu:1876-2165): kind GBSA_STEP_EXTEND is extend_seed_part of NAM `nam` of
 * read end `nam_read` (after reverse_nam_if_needed) on that read; GBSA_STEP_RESCUE is
 * rescue_mate_part of that NAM (after reverse_nam_if_needed on its own read) for the mate
 * `read`.  is_read1 is the reference's is_read1 tag of the record the step writes. */
#define GBSA_STEP_EXTEND 0
#define GBSA_STEP_RESCUE 1
typedef struct gbsa_align_step {
    uint32_t pair;
    uint32_t read;       /* the read extended (== nam_read), or the mate rescued */
    uint32_t nam_read;   /* the read end whose NAM list holds the NAM */
    uint32_t nam;        /* index of the NAM in that list */
    uint8_t  kind;
    uint8_t  is_read1;
    uint8_t  _pad[2];
} gbsa_align_step;

/* A pair's plan: its type (as gbsa_classify_pairs_device), get_mapq of both ends for
 * type 3 (step2/main.cu:900-910; 0 otherwise), the number of joint NAM pairs the type-4
 * loop visited (type4_loop_size), and its steps [first_step, first_step + n_steps). */
typedef struct gbsa_pair_plan {
    uint8_t  type;
    uint8_t  mapq1;
    uint8_t  mapq2;
    uint8_t  _pad;
    int32_t  type4_loop_size;
    uint32_t first_step;
    uint32_t n_steps;
} gbsa_pair_plan;

/* The alignment orchestration of align_PE_part0..4 (step2/main.cu:1857-2165) as step
 * lists: type 0 nothing; type 1 (2) rescue_read_part: mate 1's (2's) NAMs in order while
 * fewer than max_tries were tried and n_hits / the first NAM's n_hits >= dropoff, each
 * extended, then its mate rescued from it; type 3 both first NAMs extended and their
 * mapq; type 4 the best-scoring NAM of each end extended (the first of equal maxima),
 * then the joint NAM pairs d_pairs / d_pair_counts of gbsa_nam_pairs_device (max_tries
 * records per pair) in order while fewer than max_tries were visited and score / the
 * first pair's score >= dropoff: a present NAM not yet extended is extended, an absent one
 * makes a rescue of that read from the other end's NAM.  d_types from
 * gbsa_classify_pairs_device.  d_plans receives n_pairs records, d_steps the steps (pair
 * after pair); *n_steps the step count (GBSA_ERR_CAPACITY when above step_capacity, with
 * nothing but the count valid).  Device pointers; the call synchronizes stream.  mu and
 * sigma stay fixed: the reference updates its insert-size estimate after a type-3 pair
 * (main.cu:2002-2022), but every pair starts from a fresh estimate (gpu_align_PE3,
 * main.cu:3777), so the update changes no result. */
int gbsa_plan_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs, int layout,
                           const uint8_t* d_types, const gbsa_nam_pair* d_pairs, const uint32_t* d_pair_counts,
                           uint32_t max_tries, float dropoff, gbsa_pair_plan* d_plans, gbsa_align_step* d_steps,
                           uint64_t step_capacity, uint64_t* n_steps, void* stream);

/* AlignmentParameters (step2/aligner.hpp:11-18): match is a score, the others are
 * penalties (all nonnegative). */
typedef struct gbsa_align_params {
    int32_t match;
    int32_t mismatch;
    int32_t gap_open;
    int32_t gap_extend;
    int32_t end_bonus;
} gbsa_align_params;

/* One NAM's seed extension: GPUAlignment (step2/main.cu:418-444) plus the NAM's
 * orientation and query interval after reverse_nam_if_needed and the done_align tag. */
typedef struct gbsa_seed_alignment {
    int32_t ref_id;         /* the NAM's contig */
    int32_t ref_start;      /* alignment start on the reference */
    int32_t edit_distance;  /* mismatches inside the aligned segment */
    int32_t global_ed;      /* edit_distance + soft-clipped bases */
    int32_t score;
    int32_t length;         /* reference span of the aligned segment */
    int32_t query_start;    /* the NAM after reverse_nam_if_needed */
    int32_t query_end;
    uint8_t is_rc;          /* the NAM's (and the alignment's) orientation after reverse_nam_if_needed */
    uint8_t done;           /* done_align: 1 when the ungapped path aligned the NAM; 0 when a gapped
                               aligner must (ref_start, edit_distance, global_ed, score and length
                               are then zero) */
    uint8_t consistent;     /* reverse_nam_if_needed's answer */
    uint8_t _pad;
} gbsa_seed_alignment;

/* Seed extension of NAMs (the first alignment step of align_PE_part1..4): for NAM i,
 * of read nam_reads[i], reverse_nam_if_needed (step2/main.cu:759-793: the k-mers at
 * both NAM ends must match the reference, else the NAM is tried in the other
 * orientation) and extend_seed_part (main.cu:582-643: when the NAM projected over the
 * whole read fits the contig and is consistent, a Hamming distance below 5% of the
 * read length admits my_hamming_align, main.cu:506-580, the best-scoring ungapped
 * segment with end bonuses; otherwise the NAM is left to a gapped aligner).  The
 * reference also builds a CIGAR for the ungapped segment and then drops it; none is
 * returned.  Device pointers: contigs ref_seqs[ref_offsets[j] ..][ref_lengths[j]]
 * (bytes as loaded), reads read_seqs[read_offsets[r] ..][read_lengths[r]] (bytes as
 * given), NAMs as returned by the mapping entry points.  A NAM whose read or
 * contig index is out of range, or whose coordinates leave its read or contig,
 * fails the call (GBSA_ERR_PARAM) after the launch; the call synchronizes stream.
 * No reference C entry point: the reference runs these steps inside its alignment
 * kernels gpu_align_PE0..4 (main.cu:3583-3899). */
int gbsa_extend_seeds_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                             const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                             const uint64_t* d_read_offsets, const uint32_t* d_read_lengths, uint32_t n_reads,
                             const gbsa_nam* d_nams, const uint32_t* d_nam_reads, uint64_t n_nams, int k,
                             const gbsa_align_params* params, gbsa_seed_alignment* d_out, void* stream);

/* One mate-rescue decision: the reference window searched for the mate, and the
 * alignment record rescue_mate_part writes. */
typedef struct gbsa_mate_rescue {
    int32_t ref_id;         /* the NAM's contig */
    int32_t window_start;   /* the window [window_start, window_end) of the contig */
    int32_t window_end;
    int32_t edit_distance;  /* the mate's length when it is unaligned, else 0 */
    uint8_t is_rc;          /* the NAM's orientation */
    uint8_t done;           /* done_align: 1 when the mate is unaligned (window shorter than k, or
                               no substring shared with the window); 0 when a gapped aligner must
                               align the mate in the window */
    uint8_t is_unaligned;
    uint8_t _pad;
} gbsa_mate_rescue;

/* Mate rescue (rescue_mate_part, step2/main.cu:695-757, with has_shared_substring,
 * main.cu:657-693): for NAM i of one read end and the other end's read mate_reads[i],
 * the window where the mate lies for an insert of at most mu + 5 sigma (fr orientation,
 * at most half a read of overlap), and whether the mate (in the orientation opposite to
 * the NAM) shares a 2k/3-base substring, sampled every k/3 bases, with that window.
 * Device pointers as gbsa_extend_seeds_device; k in [3, 32].  A NAM whose contig or mate index is out
 * of range, or whose mate has more than 64 sampled substrings (the reference keeps 50 in
 * a fixed shared array), fails the call (GBSA_ERR_PARAM); the call synchronizes stream. */
int gbsa_rescue_mates_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                             const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                             const uint64_t* d_read_offsets, const uint32_t* d_read_lengths, uint32_t n_reads,
                             const gbsa_nam* d_nams, const uint32_t* d_mate_reads, uint64_t n_nams, int k,
                             float mu, float sigma, gbsa_mate_rescue* d_out, void* stream);

/* Runs the steps of gbsa_plan_pairs_device: d_ext[s] is the seed extension
 * (gbsa_extend_seeds_device) of step s's NAM on its own read for an extension step; for
 * a rescue step it holds only reverse_nam_if_needed's answer (ref_id, is_rc, query
 * interval, consistent; the alignment fields zero and done 0), and d_resc[s] the mate
 * rescue (gbsa_rescue_mates_device) of that NAM, in the orientation the check left it,
 * for the mate step.read (all zero for an extension step).  d_nams / d_nam_offsets are the
 * NAM lists the plan indexes; the other arguments as gbsa_extend_seeds_device and
 * gbsa_rescue_mates_device.  Device pointers; the call synchronizes stream. */
int gbsa_run_align_steps_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                                const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                                const uint64_t* d_read_offsets, const uint32_t* d_read_lengths, uint32_t n_reads,
                                const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, const gbsa_align_step* d_steps,
                                uint64_t n_steps, int k, const gbsa_align_params* params, float mu, float sigma,
                                gbsa_seed_alignment* d_ext, gbsa_mate_rescue* d_resc, void* stream);

/* ---- instrumentation ---------------------------------------------------------- */
/* Count the algorithmic bytes of the lookup stage (roofline numerator) in later
 * calls; gbsa_mapper_last_alg_bytes returns the count of the last batch.  No
 * reference counterpart (the reference prints wall-clock stage times only,
 * step2/main.cu:4743-4746). */
void gbsa_mapper_set_count_bytes(gbsa_mapper* m, int on);
uint64_t gbsa_mapper_last_alg_bytes(const gbsa_mapper* m);
/* Distinct 32-byte sectors the reference's lookup would gather in the last batch
 * (bucket bound pair, entries examined, filter probe, run walk), counted with the
 * bytes.  No reference counterpart. */
uint64_t gbsa_mapper_last_alg_sectors(const gbsa_mapper* m);
/* Achievable random-gather bandwidth of the current GPU: random 32-byte sector reads
 * over a device buffer of buffer_bytes (allocated and freed by the call); reports
 * sectors per second and the corresponding GB/s.  Measurement utility for the
 * lookup's roofline; no reference counterpart. */
int gbsa_bench_gather(uint64_t buffer_bytes, double* sectors_per_s, double* gb_per_s);
/* The same measurement on the lookup's own footprint and access pattern: for uniform
 * random keys, the bucket bound pair from idx's bucket table, then the bucket's first
 * entry (a dependent load), 8 probes in flight per thread; reports probes per second,
 * 32-byte sectors per second (the pair's sector plus the entry's, for a non-empty
 * bucket) and the corresponding GB/s.  The random-gather ceiling of the lookup; no
 * reference counterpart. */
int gbsa_bench_gather_index(const gbsa_index* idx, double* probes_per_s, double* sectors_per_s, double* gb_per_s);
/* Record CUDA events between the stages of later batches; gbsa_mapper_stage_ms
 * returns the last batch's milliseconds for: seeding + lookup (one kernel, a warp
 * per read; seeding alone when gbsa_mapper_fused_lookup is 0), long-read seeding,
 * long-read lookup + read bucketing (the whole lookup + bucketing when not fused),
 * NAM merge + sort (lane per read), NAM merge + sort (warp per read), rescue,
 * sorting of the rescued reads with many NAMs.  The last two run on a second stream
 * beside the two NAM stages and are timed from the end of the lookup.  No reference
 * counterpart. */
int gbsa_mapper_set_profile(gbsa_mapper* m, int on);
int gbsa_mapper_stage_ms(const gbsa_mapper* m, float* ms, int n);
/* Work counts of the last batch: out[0] query randstrobes, [1] hits of the normal
 * path, [2] NAM-state arena slots taken by the merges (the room they reserve: two per hit
 * of a lane-merged read; not the NAMs output, which the call returns), [3] rescued reads,
 * [4] reads seeded by the long-read kernel,
 * [5] overflow scratch bytes, [6] reads merged by the warp-cooperative NAM kernel.
 * out must hold 7 values.  No reference counterpart. */
int gbsa_mapper_last_counts(const gbsa_mapper* m, uint64_t* out);
/* Batches this mapper ran again because a work area (queries, hits, NAMs, overflow
 * scratch) was too small and has grown, since it was created.  No reference
 * counterpart. */
uint64_t gbsa_mapper_retries(const gbsa_mapper* m);
/* 1 when the last batch ran seeding and lookup as one kernel (indexes of up to 2 GiB
 * of entries), 0 when it ran them as two kernels (larger indexes); selects the
 * meaning of the first and third gbsa_mapper_stage_ms values.  No reference
 * counterpart. */
int gbsa_mapper_fused_lookup(const gbsa_mapper* m);
/* Largest index (bytes of entries, 16 per entry) whose batches run seeding and lookup
 * as one kernel; default 2 GiB.  0 runs them as two kernels for every index.  The
 * results are the same either way.  No reference counterpart. */
int gbsa_mapper_set_fuse_limit(gbsa_mapper* m, uint64_t index_bytes);
/* Hold the index's bucket table in L2 during the probing kernels (on = 1, the
 * default) through an access-policy window marked persisting, when the table fits
 * the device's largest window (the 32-bit table of up to 2^25 buckets); the
 * process's persisting L2 set-aside is raised for it while such mappers live.
 * *window_bytes (may be NULL) receives the window's size, 0 when none is used.  The
 * results are the same either way.  No reference counterpart. */
int gbsa_mapper_set_l2_window(gbsa_mapper* m, int on, uint64_t* window_bytes);
/* Rescued reads whose estimated merge hits (the runs of their found seeds, up to the
 * count cap) reach `hits` are taken first by the rescue kernel; in a batch with no more
 * rescued reads than the kernel has warps (small batches), each of them is merged by a
 * whole thread block, the others by a warp each.  0: every rescued read by one warp,
 * those above 2000 estimated hits first.  Default 4000.  Takes effect from the next
 * batch; the results are the same either way.  No reference counterpart. */
int gbsa_mapper_set_rescue_block(gbsa_mapper* m, uint32_t hits);
/* With profiling on: 8 values per rescued read of the last batch, in rescue-list
 * order: SM clock cycles in total (without a block sort), of the planning, of the
 * merge and of the sort (the block sort, for reads with many NAMs), then the hit
 * bound, the NAM count, the SM cycles of the run walks within the merge and the
 * longest hit run.  n_out[0] receives
 * the rescued read count, n_out[1] the count of block-sorted reads; out holds up
 * to cap values.  No reference counterpart. */
int gbsa_mapper_rescue_cycles(const gbsa_mapper* m, uint64_t* out, uint32_t cap, uint32_t* n_out);

/* With profiling on: per read of the last batch's warp-per-read find_nams kernel,
 * four values (SM cycles in total, hits, NAMs, SM cycles of the merge); n_out[0]
 * receives the read count; out holds up to cap values.  No reference counterpart. */
int gbsa_mapper_nam_cycles(const gbsa_mapper* m, uint64_t* out, uint32_t cap, uint32_t* n_out);

#ifdef __cplusplus
}
#endif

#endif /* GBSA_H */
