/*
 * ref_driver.cu — runs the REFERENCE's own CPU code on a test case, to pin the oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/build_ref.sh from the reference sources
 * where they lie (never copied), into oracle/_ref/ (git-ignored).  It exists only
 * where the reference tree is present; the committed fixtures in tests/golden/ carry
 * its outputs to machines without it.
 *
 * Reference code exercised (paths inside the reference project):
 *   IndexParameters::from_read_length      step2/indexparameters.cpp:150-182
 *   StrobemerIndex::read (.sti v2)         step2/index.cu:91-134
 *   StrobemerIndex::find / is_filtered /   step2/index.hpp:57-147
 *     get_count
 *   SyncmerIterator::next                  step2/randstrobes.cu:18-79
 *   RandstrobeIterator::next / get         step2/randstrobes.cu:136-159
 *   find_nams                              step2/nam.cu:553-747
 *   find_nams_rescue                       step2/nam.cu:927-985
 * The read-level glue (randstrobes_query, step2/randstrobes.cu:195-241, and the
 * rescue trigger, step2/main.cu:3209-3216 and :4204) is commented out or GPU-only in
 * the reference, so this driver states it around the reference calls.
 *
 * The reference's host SyncmerIterator keeps its s-mer queue behind a private
 * pointer that no constructor sets (step2/randstrobes.hpp:242-243, 336); the driver
 * opens the class's private members to hand it a queue.
 *
 * `ref_driver xxh64` reads decimal u64 values on stdin and prints the reference
 * xxh64 of each (known-answer vectors).
 *
 * Input (argv[1], binary): int32 read_length, int32 rescue_level, uint32 n_reads,
 *   uint32 lengths[n_reads], then the bases back to back.
 * argv[2]: the .sti index.  argv[3]: output file.  Output per read:
 *   uint32 n_queries, n_queries x {u64 hash, u32 start, u32 end, u8 is_reverse},
 *   float nonrepetitive_fraction, u8 rescued, uint32 n_nams,
 *   n_nams x {i32 query_start, query_end, ref_start, ref_end, n_hits, ref_id,
 *             float score, u8 is_rc}.
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <iostream>
#include <limits>
#include <map>
#include <new>
#include <numeric>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <string_view>
#include <tuple>
#include <thread>
#include <vector>
#include <cuda_runtime.h>
#include "robin_hood.h"

#define private public
#include "nam.hpp"
#undef private

static void put(std::ofstream& o, const void* p, size_t n) { o.write(reinterpret_cast<const char*>(p), (std::streamsize)n); }

/* randstrobes_query glue (step2/randstrobes.cu:195-241, commented out in the reference)
 * around the reference's SyncmerIterator and RandstrobeIterator. */
static QueryRandstrobeVector query_randstrobes(const std::string_view seq, const IndexParameters& params) {
    QueryRandstrobeVector qv;
    if (seq.length() < params.randstrobe.w_max) return qv;
    std::deque<uint64_t> queue;
    /* The class's destructor is __device__-only, so the host object lives in a buffer
     * and is never destroyed (it owns no resources). */
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

/* `ref_driver time case.bin index.sti threads reps`: the reference's CPU path (query
 * randstrobes, find_nams, find_nams_rescue for rescued reads) over every read of the
 * case on `threads` host threads that take reads 256 at a time (the dynamic schedule of
 * the reference's OpenMP loops, cpu_test.cpp:282); prints the best of `reps` wall-clock
 * times as one JSON line.  Reading the case and the index is not timed. */
static int time_mode(int argc, char** argv) {
    if (argc != 6 && argc != 7) {
        std::fprintf(stderr, "usage: ref_driver time case.bin index.sti threads reps [max_reads]\n");
        return 2;
    }
    std::ifstream in(argv[2], std::ios::binary);
    int32_t read_length = 0, rescue_level = 0;
    uint32_t n_reads = 0;
    in.read(reinterpret_cast<char*>(&read_length), 4);
    in.read(reinterpret_cast<char*>(&rescue_level), 4);
    in.read(reinterpret_cast<char*>(&n_reads), 4);
    std::vector<uint32_t> lens(n_reads);
    in.read(reinterpret_cast<char*>(lens.data()), (std::streamsize)(4 * (size_t)n_reads));
    const uint32_t n_all = n_reads;
    if (argc == 7) n_reads = std::min<uint32_t>(n_reads, (uint32_t)std::strtoul(argv[6], nullptr, 10));
    std::vector<uint64_t> offs(n_reads + 1, 0);
    for (uint32_t i = 0; i < n_reads; ++i) offs[i + 1] = offs[i] + lens[i];
    std::string bases(offs[n_reads], '\0');
    in.read(&bases[0], (std::streamsize)bases.size());   // the first n_reads reads' bases
    (void)n_all;
    const IndexParameters params = IndexParameters::from_read_length(read_length);
    References refs(std::vector<std::string>{std::string(64, 'A')}, std::vector<std::string>{"x"});
    StrobemerIndex index(refs, params, 8);
    index.read(argv[3]);
    const unsigned rescue_cutoff = rescue_level < 100 ? (unsigned)(rescue_level * (int)index.filter_cutoff) : 100u;
    const int threads = std::max(1, std::atoi(argv[4]));
    const int reps = std::max(1, std::atoi(argv[5]));
    double best = 1e30;
    std::string rep_list;
    uint64_t total_nams = 0, total_rescued = 0;
    for (int rep = 0; rep < reps; ++rep) {
        std::atomic<uint32_t> next{0};
        std::atomic<uint64_t> nams_sum{0}, resc_sum{0};
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::thread> th;
        for (int t = 0; t < threads; ++t) {
            th.emplace_back([&]() {
                uint64_t my_nams = 0, my_resc = 0;
                for (;;) {
                    const uint32_t a = next.fetch_add(256);
                    if (a >= n_reads) break;
                    const uint32_t b = std::min(n_reads, a + 256);
                    for (uint32_t r = a; r < b; ++r) {
                        const std::string_view seq(bases.data() + offs[r], lens[r]);
                        const QueryRandstrobeVector qv = query_randstrobes(seq, params);
                        auto [frac, nams] = find_nams(qv, index);
                        if (rescue_level > 1 && (nams.empty() || frac < 0.7)) {
                            nams = find_nams_rescue(qv, index, rescue_cutoff);
                            ++my_resc;
                        }
                        my_nams += nams.size();
                    }
                }
                nams_sum += my_nams;
                resc_sum += my_resc;
            });
        }
        for (auto& x : th) x.join();
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        best = std::min(best, dt);
        rep_list += (rep ? ", " : "") + std::to_string(dt);
        total_nams = nams_sum.load();
        total_rescued = resc_sum.load();
    }
    std::printf("{\"reads\": %u, \"seconds\": %.6f, \"rep_seconds\": [%s], \"threads\": %d, \"reps\": %d, "
                "\"nams\": %llu, \"rescued\": %llu}\n",
                n_reads, best, rep_list.c_str(), threads, reps, (unsigned long long)total_nams,
                (unsigned long long)total_rescued);
    return 0;
}

int main(int argc, char** argv) {
    if (argc == 2 && std::string(argv[1]) == "xxh64") {
        /* known-answer mode: decimal u64 values on stdin → xxh64 (step2/hash.hpp:106-119) */
        unsigned long long v;
        while (std::scanf("%llu", &v) == 1) std::printf("%llu\n", (unsigned long long)xxh64((uint64_t)v));
        return 0;
    }
    if (argc >= 2 && std::string(argv[1]) == "time") return time_mode(argc, argv);
    if (argc != 4) {
        std::fprintf(stderr, "usage: ref_driver case.bin index.sti out.bin\n");
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    int32_t read_length = 0, rescue_level = 0;
    uint32_t n_reads = 0;
    in.read(reinterpret_cast<char*>(&read_length), 4);
    in.read(reinterpret_cast<char*>(&rescue_level), 4);
    in.read(reinterpret_cast<char*>(&n_reads), 4);
    std::vector<uint32_t> lens(n_reads);
    in.read(reinterpret_cast<char*>(lens.data()), (std::streamsize)(4 * (size_t)n_reads));
    std::vector<std::string> reads(n_reads);
    for (uint32_t i = 0; i < n_reads; ++i) {
        reads[i].resize(lens[i]);
        in.read(&reads[i][0], lens[i]);
    }

    const IndexParameters params = IndexParameters::from_read_length(read_length);
    References refs(std::vector<std::string>{std::string(64, 'A')}, std::vector<std::string>{"x"});
    StrobemerIndex index(refs, params, 8);
    index.read(argv[2]);
    const unsigned rescue_cutoff =
        rescue_level < 100 ? (unsigned)(rescue_level * (int)index.filter_cutoff) : 100u;

    std::ofstream out(argv[3], std::ios::binary);
    for (uint32_t r = 0; r < n_reads; ++r) {
        const std::string_view seq(reads[r]);
        const QueryRandstrobeVector qv = query_randstrobes(seq, params);
        auto [frac, nams] = find_nams(qv, index);
        uint8_t rescued = 0;
        if (rescue_level > 1 && (nams.empty() || frac < 0.7)) {
            nams = find_nams_rescue(qv, index, rescue_cutoff);
            rescued = 1;
        }
        const uint32_t nq = (uint32_t)qv.size();
        put(out, &nq, 4);
        for (const auto& q : qv) {
            put(out, &q.hash, 8);
            put(out, &q.start, 4);
            put(out, &q.end, 4);
            const uint8_t rv = q.is_reverse ? 1 : 0;
            put(out, &rv, 1);
        }
        put(out, &frac, 4);
        put(out, &rescued, 1);
        const uint32_t nn = (uint32_t)nams.size();
        put(out, &nn, 4);
        for (const auto& n : nams) {
            const int32_t f[6] = {n.query_start, n.query_end, n.ref_start, n.ref_end, n.n_hits, n.ref_id};
            put(out, f, sizeof f);
            put(out, &n.score, 4);
            const uint8_t rc = n.is_rc ? 1 : 0;
            put(out, &rc, 1);
        }
    }
    return 0;
}
