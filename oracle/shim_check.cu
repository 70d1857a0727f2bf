/*
 * shim_check.cu — checks include/gbsa_shim.hpp, the binding a maintainer adds to the
 * reference, against the REFERENCE's own CPU code.  TEST INFRASTRUCTURE ONLY: built by
 * oracle/build_ref.sh next to ref_driver (from the reference's sources where they lie,
 * or from the staged copy) and linked with libgbsa.so; run by tests/test_shim_gpu.py.
 *
 *   1. References from the case's contigs; IndexParameters::from_read_length(150);
 *      StrobemerIndex(refs, params) (step2/index.hpp:39-48) populated on the GPU by
 *      gbsa_shim::gpu_populate, which also fills the index's host vectors.
 *   2. For every read: the query randstrobes (the reference's SyncmerIterator and
 *      RandstrobeIterator, with the randstrobes_query glue of step2/randstrobes.cu:
 *      195-241), then
 *        - the reference's find_nams (step2/nam.cu) on those host vectors, against
 *          gbsa_shim::find_nams on the GPU index;
 *        - the reference's find_nams_rescue, against gbsa_shim::find_nams_rescue;
 *      every other read with a NAM buffer of one record, so that the shim's retry on
 *      GBSA_ERR_CAPACITY runs.
 *   3. NAM lists are compared as sets (the reference returns them in hash-map order):
 *      both sorted by (is_rc, ref_id, query start/end, ref start/end, n_hits, score).
 *
 * Input (argv[1]): uint32 n_contigs, uint64 lengths[n_contigs], bases; uint32 n_reads,
 * uint32 lengths[n_reads], bases.  Prints one JSON line; exit 0 when all agree.
 */
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <new>
#include <string>
#include <string_view>
#include <tuple>
#include <vector>
#include <cuda_runtime.h>
#include "robin_hood.h"

#define private public
#include "nam.hpp"
#undef private

#include "gbsa_shim.hpp"

static QueryRandstrobeVector query_randstrobes(const std::string_view seq, const IndexParameters& params) {
    QueryRandstrobeVector qv;
    if (seq.length() < params.randstrobe.w_max) return qv;
    std::deque<uint64_t> queue;
    alignas(SyncmerIterator) unsigned char storage[sizeof(SyncmerIterator)];
    SyncmerIterator* it = new (storage) SyncmerIterator(&seq, params.syncmer);
    it->qs = &queue;
    std::vector<Syncmer> syncmers;
    for (Syncmer s; !(s = it->next()).is_end();) syncmers.push_back(s);
    if (syncmers.empty()) return qv;
    RandstrobeIterator fwd(&syncmers, params.randstrobe);
    while (fwd.has_next()) {
        const Randstrobe x = fwd.next();
        qv.push_back(QueryRandstrobe{x.hash, x.strobe1_pos, x.strobe2_pos + (unsigned)params.syncmer.k, false});
    }
    std::reverse(syncmers.begin(), syncmers.end());
    for (auto& s : syncmers) s.position = seq.length() - s.position - params.syncmer.k;
    RandstrobeIterator rc(&syncmers, params.randstrobe);
    while (rc.has_next()) {
        const Randstrobe x = rc.next();
        qv.push_back(QueryRandstrobe{x.hash, x.strobe1_pos, x.strobe2_pos + (unsigned)params.syncmer.k, true});
    }
    return qv;
}

using Key = std::tuple<int, int, int, int, int, int, int, float>;

static std::vector<Key> keys_of(const std::vector<Nam>& v) {
    std::vector<Key> k;
    for (const Nam& n : v)
        k.emplace_back(n.is_rc ? 1 : 0, n.ref_id, n.query_start, n.query_end, n.ref_start, n.ref_end, n.n_hits,
                       n.score);
    std::sort(k.begin(), k.end());
    return k;
}

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: shim_check case.bin\n");
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    uint32_t nc = 0;
    in.read(reinterpret_cast<char*>(&nc), 4);
    std::vector<uint64_t> clen(nc);
    in.read(reinterpret_cast<char*>(clen.data()), (std::streamsize)(8 * (size_t)nc));
    std::vector<std::string> seqs(nc), names(nc);
    for (uint32_t i = 0; i < nc; ++i) {
        seqs[i].resize(clen[i]);
        in.read(&seqs[i][0], (std::streamsize)clen[i]);
        names[i] = "contig" + std::to_string(i);
    }
    uint32_t nr = 0;
    in.read(reinterpret_cast<char*>(&nr), 4);
    std::vector<uint32_t> rlen(nr);
    in.read(reinterpret_cast<char*>(rlen.data()), (std::streamsize)(4 * (size_t)nr));
    std::vector<std::string> reads(nr);
    for (uint32_t i = 0; i < nr; ++i) {
        reads[i].resize(rlen[i]);
        in.read(&reads[i][0], rlen[i]);
    }
    if (!in) {
        std::fprintf(stderr, "truncated case file\n");
        return 2;
    }

    const References refs(seqs, names);
    const IndexParameters params = IndexParameters::from_read_length(150);
    StrobemerIndex index(refs, params);
    gbsa_index* g = gbsa_shim::gpu_populate(index, refs, 0.0002f);
    gbsa_map_options opt{2, 1000, GBSA_SORT_SCORE, 0};
    gbsa_mapper* m = nullptr;
    if (gbsa_mapper_create(g, &opt, 1024, 1 << 20, &m) != GBSA_OK) {
        std::fprintf(stderr, "mapper: %s\n", gbsa_last_error());
        return 1;
    }
    const unsigned rescue_cutoff = 2 * index.filter_cutoff;   // R = 2 (step2/main.cu:4204)
    uint64_t plain_bad = 0, rescue_bad = 0, frac_bad = 0, nams = 0, retried = 0;
    for (uint32_t r = 0; r < nr; ++r) {
        const QueryRandstrobeVector qv = query_randstrobes(reads[r], params);
        const size_t guess = (r & 1) ? 1 : 0;   // odd reads: a one-record buffer first
        auto [f_ref, n_ref] = find_nams(qv, index);
        auto [f_gpu, n_gpu] = gbsa_shim::find_nams(qv, m, guess);
        if (keys_of(n_ref) != keys_of(n_gpu)) ++plain_bad;
        if (f_ref != f_gpu) ++frac_bad;
        const std::vector<Nam> r_ref = find_nams_rescue(qv, index, rescue_cutoff);
        const std::vector<Nam> r_gpu = gbsa_shim::find_nams_rescue(qv, m, rescue_cutoff, guess);
        if (keys_of(r_ref) != keys_of(r_gpu)) ++rescue_bad;
        nams += n_gpu.size() + r_gpu.size();
        retried += guess && (n_gpu.size() > 1 || r_gpu.size() > 1);
    }
    gbsa_mapper_free(m);
    gbsa_index_free(g);
    std::printf("{\"reads\": %u, \"index_entries\": %zu, \"filter_cutoff\": %u, \"nams\": %llu, "
                "\"find_nams_mismatches\": %llu, \"fraction_mismatches\": %llu, \"rescue_mismatches\": %llu, "
                "\"capacity_retries\": %llu}\n",
                nr, index.randstrobes.size(), index.filter_cutoff, (unsigned long long)nams,
                (unsigned long long)plain_bad, (unsigned long long)frac_bad, (unsigned long long)rescue_bad,
                (unsigned long long)retried);
    return plain_bad || rescue_bad || frac_bad ? 1 : 0;
}
