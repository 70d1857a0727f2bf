/*
 * oracle.h — CPU restatement of strobealign's seeding → lookup → NAM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the GPU path is compared
 * with (tests, __graft_entry__.smoke, and bench.py's cpu_baseline / reference arm).
 * Nothing in the product links, loads or calls it.
 *
 * Each function restates the reference algorithm it cites (paths are inside the
 * reference project, step2/ unless noted).  Parity of this restatement is pinned
 * against the reference's own compiled CPU code (oracle/ref_driver.cpp, built only
 * where the reference sources are present) through the fixtures in tests/golden/.
 */
#ifndef GBSA_ORACLE_H
#define GBSA_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/gbsa.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_index oracle_index;

uint64_t oracle_xxh64(uint64_t x);
int oracle_params_from_read_length(int read_length, int k, int s, int l, int u, int c,
                                   int max_seed_len, gbsa_params* out);
int oracle_pick_bits(const gbsa_params* p, uint64_t total_length);

/* Canonical syncmers of one sequence: writes up to cap (hash, pos) pairs, returns count. */
int64_t oracle_syncmers(const gbsa_params* p, const char* seq, uint64_t len,
                        uint64_t* hashes, uint64_t* positions, uint64_t cap);
/* randstrobes_query of one read; returns count (or -count-1 if cap too small). */
int64_t oracle_randstrobes_query(const gbsa_params* p, const char* seq, uint64_t len,
                                 gbsa_query_randstrobe* out, uint64_t cap);

oracle_index* oracle_index_build(const gbsa_params* p, const char* seqs, const uint64_t* offsets,
                                 const uint64_t* lengths, uint32_t n_contigs, int bits, float f);
oracle_index* oracle_index_load(const gbsa_params* p, const gbsa_ref_randstrobe* rs, uint64_t n,
                                const uint64_t* starts, int bits, uint32_t filter_cutoff);
/* Checks an index built elsewhere against the restatement without building one
 * (generated entries as a multiset, order, bucket table, filter cutoff); 0 = equal. */
int oracle_index_verify(const gbsa_params* p, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
                        uint32_t n_contigs, float f, const gbsa_ref_randstrobe* rs, uint64_t n,
                        const uint64_t* starts, int bits, uint32_t filter_cutoff, int n_threads, uint64_t* report);
void oracle_index_free(oracle_index* idx);
void oracle_index_info(const oracle_index* idx, gbsa_index_info* out);
const gbsa_ref_randstrobe* oracle_index_randstrobes(const oracle_index* idx);
const uint64_t* oracle_index_starts(const oracle_index* idx);
int oracle_index_write_sti(const oracle_index* idx, const char* path);

uint64_t oracle_find(const oracle_index* idx, uint64_t hash);
uint32_t oracle_get_count(const oracle_index* idx, uint64_t position);
int oracle_is_filtered(const oracle_index* idx, uint64_t position);

/* find_nams on already-seeded queries: returns NAM count (or -count-1 if cap too small),
 * NAMs in emission order of the restated merge (not sorted). */
int64_t oracle_find_nams(const oracle_index* idx, const gbsa_query_randstrobe* q, uint64_t nq,
                         gbsa_nam* out, uint64_t cap, float* frac);
int64_t oracle_find_nams_rescue(const oracle_index* idx, const gbsa_query_randstrobe* q,
                                uint64_t nq, uint32_t rescue_cutoff, uint32_t count_cap,
                                gbsa_nam* out, uint64_t cap);
/* Sort NAMs in place in one of the GBSA_SORT_* orders. */
void oracle_sort_nams(gbsa_nam* nams, uint64_t n, int sort_mode);
int oracle_classify_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout,
                          float dropoff_threshold, float mu, float sigma, uint8_t* types);

/* get_best_scoring_nam_pairs_sort3 (step2/main.cu:1475-1716) per pair, cut to max_tries
 * (main.cu:2061-2064); out holds max_tries records per pair, counts the number kept. */
int oracle_nam_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout, float mu,
                     float sigma, uint32_t max_tries, gbsa_nam_pair* out, uint32_t* counts);

/* reverse_nam_if_needed + extend_seed_part (step2/main.cu:759-793, 582-643, 506-580)
 * for each NAM; host pointers, same contract as gbsa_extend_seeds_device.  Returns
 * GBSA_OK or GBSA_ERR_PARAM. */
int oracle_extend_seeds(const char* ref_seqs, const uint64_t* ref_offsets, const uint64_t* ref_lengths,
                        uint32_t n_refs, const char* read_seqs, const uint64_t* read_offsets,
                        const uint32_t* read_lengths, uint32_t n_reads, const gbsa_nam* nams,
                        const uint32_t* nam_reads, uint64_t n_nams, int k, const gbsa_align_params* ap,
                        gbsa_seed_alignment* out);

/* rescue_mate_part with has_shared_substring (step2/main.cu:695-757, 657-693) for each
 * NAM; host pointers, same contract as gbsa_rescue_mates_device. */
int oracle_rescue_mates(const char* ref_seqs, const uint64_t* ref_offsets, const uint64_t* ref_lengths,
                        uint32_t n_refs, const char* read_seqs, const uint64_t* read_offsets,
                        const uint32_t* read_lengths, uint32_t n_reads, const gbsa_nam* nams,
                        const uint32_t* mate_reads, uint64_t n_nams, int k, float mu, float sigma,
                        gbsa_mate_rescue* out);

/* Whole path for a batch of reads with n_threads host threads (0 = all cores).
 * Same contract as gbsa_map_reads.  Returns GBSA_OK or GBSA_ERR_CAPACITY. */
int64_t oracle_plan_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout,
                          const uint8_t* types, const gbsa_nam_pair* jp, const uint32_t* jcounts, uint32_t max_tries,
                          float dropoff, gbsa_pair_plan* plans, gbsa_align_step* steps, uint64_t step_cap);
int oracle_map_reads(const oracle_index* idx, const gbsa_map_options* opt, const char* seqs,
                     const uint64_t* offsets, const uint32_t* lengths, uint32_t n_reads,
                     gbsa_nam* nams, uint64_t nam_capacity, uint64_t* nam_offsets,
                     float* frac, uint8_t* rescued, int n_threads);

/* Algorithmic byte count of the lookup + NAM path for a batch (the roofline
 * numerator): 2-bit read input, bucket bound pair, entries examined, filter probe,
 * hit-run walk, and NAM records written. */
int oracle_algorithmic_bytes(const oracle_index* idx, const gbsa_map_options* opt,
                             const char* seqs, const uint64_t* offsets, const uint32_t* lengths,
                             uint32_t n_reads, uint64_t* bytes_out, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
