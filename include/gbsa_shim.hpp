/*
 * gbsa_shim.hpp — the reference-side binding of libgbsa.so: drop-in replacements for
 * StrobemerIndex::populate and find_nams / find_nams_rescue that a maintainer of the
 * reference (strobealign 1.0.3 fork, step2/) adds to it.  Compile with the
 * reference's step2/ headers on the include path and link with libgbsa.so.  Checked
 * against the reference's own CPU find_nams / find_nams_rescue by oracle/shim_check.cu.
 *
 *   gbsa_shim::gpu_populate   StrobemerIndex::populate (step2/index.hpp:54; body
 *                             step2/index.cu:143-244): the index built on the GPU, the
 *                             host vectors filled so that the reference's own find(),
 *                             is_filtered() and get_count() keep working on the host
 *   gbsa_shim::find_nams      find_nams (step2/nam.hpp:11-14), one read
 *   gbsa_shim::find_nams_rescue  find_nams_rescue (step2/nam.hpp:16-20), one read
 *
 * NAMs come back in the mapper's sort order (GBSA_SORT_*), not in the reference's
 * hash-map order.  A batched caller maps many reads per call with gbsa_find_nams or
 * gbsa_map_reads instead.
 */
#pragma once

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbsa.h"
#include "index.hpp"
#include "nam.hpp"

namespace gbsa_shim {

static_assert(sizeof(RefRandstrobe) == sizeof(gbsa_ref_randstrobe), "RefRandstrobe layout");
static_assert(sizeof(QueryRandstrobe) == sizeof(gbsa_query_randstrobe), "QueryRandstrobe layout");
static_assert(sizeof(Nam) == sizeof(gbsa_nam), "Nam layout");

inline gbsa_params to_gbsa(const IndexParameters& p) {
    gbsa_params g;
    if (gbsa_params_make(p.canonical_read_length, p.syncmer.k, p.syncmer.s, p.randstrobe.l, p.randstrobe.u,
                         (int)p.randstrobe.q, p.randstrobe.max_dist, &g) != GBSA_OK)
        throw BadParameter(gbsa_last_error());
    return g;
}

// StrobemerIndex::populate(f, n_threads) on the GPU; returns the device index (keep it
// for the batched calls and the mappers; free it with gbsa_index_free).
inline gbsa_index* gpu_populate(StrobemerIndex& idx, const References& refs, float f) {
    std::vector<uint64_t> off(refs.size()), len(refs.size());
    std::string all;
    for (size_t i = 0; i < refs.size(); ++i) {
        off[i] = all.size();
        len[i] = refs.lengths[i];
        all += refs.sequences[i];
    }
    const gbsa_params gp = to_gbsa(idx.parameters);
    gbsa_index* g = nullptr;
    if (gbsa_index_build(&gp, all.data(), off.data(), len.data(), (uint32_t)refs.size(), idx.bits, f, &g) != GBSA_OK)
        throw BadParameter(gbsa_last_error());
    gbsa_index_info info;
    gbsa_index_get_info(g, &info);
    idx.filter_cutoff = info.filter_cutoff;
    idx.randstrobes.resize(info.size);
    idx.randstrobe_start_indices.resize((1ull << info.bits) + 1);
    if (gbsa_index_export(g, reinterpret_cast<gbsa_ref_randstrobe*>(idx.randstrobes.data()),
                          idx.randstrobe_start_indices.data()) != GBSA_OK) {
        gbsa_index_free(g);
        throw std::runtime_error(gbsa_last_error());
    }
    return g;
}

// One read through gbsa_find_nams; the NAM buffer starts at `guess` records and, when
// the read has more NAMs (NAMs are bounded by hits, not by query randstrobes), grows to
// the count the call reports and the call runs again.
inline std::vector<Nam> nams_of(const QueryRandstrobeVector& q, gbsa_mapper* m, int rescue, unsigned rescue_cutoff,
                                float* frac, size_t guess) {
    uint64_t qoff[2] = {0, q.size()};
    std::vector<Nam> nams(guess > 0 ? guess : 1);
    uint64_t noff[2] = {0, 0};
    for (int attempt = 0; attempt < 2; ++attempt) {
        const int rc = gbsa_find_nams(m, reinterpret_cast<const gbsa_query_randstrobe*>(q.data()), qoff, 1, rescue,
                                      rescue_cutoff, reinterpret_cast<gbsa_nam*>(nams.data()), nams.size(), noff,
                                      frac);
        if (rc == GBSA_ERR_CAPACITY) {
            nams.resize(noff[1]);
            continue;
        }
        if (rc != GBSA_OK) throw std::runtime_error(gbsa_last_error());
        nams.resize(noff[1]);
        return nams;
    }
    throw std::runtime_error("NAM buffer still too small");
}

// find_nams (step2/nam.hpp:11-14) for one read on a mapper of the GPU index.
inline std::pair<float, std::vector<Nam>> find_nams(const QueryRandstrobeVector& q, gbsa_mapper* m,
                                                    size_t guess = 0) {
    float frac = 1.0f;
    std::vector<Nam> nams = nams_of(q, m, 0, 0, &frac, guess ? guess : 4 * q.size() + 16);
    return {frac, std::move(nams)};
}

// find_nams_rescue (step2/nam.hpp:16-20) for one read on a mapper of the GPU index.
inline std::vector<Nam> find_nams_rescue(const QueryRandstrobeVector& q, gbsa_mapper* m, unsigned rescue_cutoff,
                                         size_t guess = 0) {
    return nams_of(q, m, 1, rescue_cutoff, nullptr, guess ? guess : 4 * q.size() + 16);
}

}  // namespace gbsa_shim
