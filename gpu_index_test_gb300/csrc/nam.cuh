// nam.cuh — hit → NAM merging and NAM ordering, as warp-level device functions.
//
// Hits of one read are grouped by (orientation, reference id) — the reference keeps
// them in robin_hood maps keyed by ref id, one per orientation (step2/nam.cu:45-62)
// — and each group is merged by one lane:
//   merge_group_hit_major  merge_hits_into_nams, step2/nam.cu:347-513 (find_nams)
//   merge_group_nam_major  merge_hits_into_nams_fast, step2/nam.cu:94-343
//                          (find_nams_rescue)
// Both keep the reference's open-NAM order (creation order; flushing a NAM whose
// query_end is behind the current query_start removes one that could no longer
// take any later hit, so skipping such NAMs is the same as removing them).
#pragma once

#include "lookup.cuh"

namespace gbsa {

// Working state of one NAM (step2/my_struct.hpp:48-62 fields used by the merge).
struct NamState {
    int32_t qs, qe, qprev, rs, re, rprev, n_hits, ref_rc;
};

__device__ __forceinline__ NamState nam_from_hit(const HitRec& h) {
    NamState n;
    n.qs = h.qs;
    n.qe = h.qe;
    n.qprev = h.qs;
    n.rs = h.rs;
    n.re = h.re;
    n.rprev = h.rs;
    n.n_hits = 1;
    n.ref_rc = (int32_t)h.ref_rc;
    return n;
}

// Hits hits[order[b..e)] (sorted by query_start, then ref_start) → NAMs out[0..),
// hit-major: each hit joins the first open NAM that accepts it.  Returns the count.
__device__ __forceinline__ uint32_t merge_group_hit_major(const HitRec* hits, const uint32_t* order, uint32_t b,
                                                          uint32_t e, NamState* out) {
    uint32_t nn = 0;
    uint32_t first_open = 0;   // NAMs before this index are all closed
    for (uint32_t i = b; i < e; ++i) {
        const HitRec h = hits[order[i]];
        bool added = false;
        while (first_open < nn && out[first_open].qe < h.qs) ++first_open;
        for (uint32_t o = first_open; o < nn; ++o) {
            NamState& n = out[o];
            if (n.qe < h.qs) continue;   // closed
            if (n.qprev < h.qs && h.qs <= n.qe && n.rprev < h.rs && h.rs <= n.re) {
                if (h.qe > n.qe && h.re > n.re) {
                    n.qe = h.qe;
                    n.re = h.re;
                    n.qprev = h.qs;
                    n.rprev = h.rs;
                    ++n.n_hits;
                    added = true;
                    break;
                } else if (h.qe <= n.qe && h.re <= n.re) {
                    n.qprev = h.qs;
                    n.rprev = h.rs;
                    ++n.n_hits;
                    added = true;
                    break;
                }
            }
        }
        if (!added) out[nn++] = nam_from_hit(h);
    }
    return nn;
}

// NAM-major variant: hits are taken one query_start group at a time; each open NAM
// (in creation order) takes the first not-yet-taken hit of the group with
// ref_start in (rprev, re] that extends it or lies inside it.  `taken` is per-hit
// scratch of the group's size.  Returns the NAM count.
__device__ __forceinline__ uint32_t merge_group_nam_major(const HitRec* hits, const uint32_t* order, uint32_t b,
                                                          uint32_t e, NamState* out, uint8_t* taken) {
    uint32_t nn = 0;
    for (uint32_t g0 = b; g0 < e;) {
        const int qs = hits[order[g0]].qs;
        uint32_t g1 = g0 + 1;
        while (g1 < e && hits[order[g1]].qs == qs) ++g1;
        const uint32_t gn = g1 - g0;
        for (uint32_t j = 0; j < gn; ++j) taken[j] = 0;
        uint32_t done = 0;
        const uint32_t nn_before = nn;
        for (uint32_t o = 0; o < nn_before && done < gn; ++o) {
            NamState& n = out[o];
            if (n.qe < qs) continue;   // closed (cannot take this or later groups)
            // first hit with rs >= rprev + 1 (hits of the group are sorted by rs)
            uint32_t lo = g0, hi = g1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) / 2;
                if (hits[order[mid]].rs < n.rprev + 1) lo = mid + 1;
                else hi = mid;
            }
            for (uint32_t j = lo; j < g1; ++j) {
                const HitRec h = hits[order[j]];
                if (h.rs > n.re) break;   // upper bound rs <= re
                if (taken[j - g0]) continue;
                if (h.qe > n.qe && h.re > n.re) {
                    n.qe = h.qe;
                    n.re = h.re;
                    n.qprev = h.qs;
                    n.rprev = h.rs;
                    ++n.n_hits;
                    taken[j - g0] = 1;
                    ++done;
                    break;
                } else if (h.qe <= n.qe && h.re <= n.re) {
                    n.qprev = h.qs;
                    n.rprev = h.rs;
                    ++n.n_hits;
                    taken[j - g0] = 1;
                    ++done;
                    break;
                }
            }
        }
        for (uint32_t j = 0; j < gn; ++j)
            if (!taken[j]) out[nn++] = nam_from_hit(hits[order[g0 + j]]);
        g0 = g1;
    }
    return nn;
}

// Score (step2/nam.cu:454-463): n_hits * (2*min_span - max_span) if positive, else 1.
__device__ __forceinline__ float nam_score(const NamState& n) {
    const int qspan = n.qe - n.qs, rspan = n.re - n.rs;
    const int mx = qspan > rspan ? qspan : rspan;
    const int mn = qspan < rspan ? qspan : rspan;
    const int v = 2 * mn - mx;
    return v > 0 ? (float)(n.n_hits * v) : 1.0f;
}

__device__ __forceinline__ void to_gbsa_nam(const NamState& n, int id, gbsa_nam& o) {
    o.nam_id = id;
    o.query_start = n.qs;
    o.query_end = n.qe;
    o.query_prev_hit_startpos = n.qprev;
    o.ref_start = n.rs;
    o.ref_end = n.re;
    o.ref_prev_hit_startpos = n.rprev;
    o.n_hits = n.n_hits;
    o.ref_id = (int32_t)((uint32_t)n.ref_rc & 0x7FFFFFFFu);
    o.score = nam_score(n);
    o.is_rc = ((uint32_t)n.ref_rc >> 31) ? 1 : 0;
    o._pad[0] = o._pad[1] = o._pad[2] = 0;
}

// NAM orders (GBSA_SORT_*): true when a goes before b.  The score order is
// (score desc, is_rc, ref_id, qs, qe, rs, re, n_hits desc); the two reference
// orders follow Nam::operator< (step2/my_struct.hpp:78-92, mate 2) and
// sort_nams_single2 (step2/main.cu:2271-2289, mate 1) with the remaining compared
// field appended so that the order is total.
__device__ __forceinline__ bool nam_before(const NamState& a, const NamState& b, int mode) {
    const uint32_t arc = (uint32_t)a.ref_rc >> 31, brc = (uint32_t)b.ref_rc >> 31;
    const int32_t aref = a.ref_rc & 0x7FFFFFFF, bref = b.ref_rc & 0x7FFFFFFF;
    if (mode == GBSA_SORT_SCORE) {
        const float sa = nam_score(a), sb = nam_score(b);
        if (sa != sb) return sa > sb;
        if (arc != brc) return arc < brc;
        if (aref != bref) return aref < bref;
        if (a.qs != b.qs) return a.qs < b.qs;
        if (a.qe != b.qe) return a.qe < b.qe;
        if (a.rs != b.rs) return a.rs < b.rs;
        if (a.re != b.re) return a.re < b.re;
        return a.n_hits > b.n_hits;
    }
    if (arc != brc) return arc < brc;
    if (aref != bref) return aref < bref;
    if (mode == GBSA_SORT_REF_MATE2) {
        const int da = a.rs - a.qs > 0 ? a.rs - a.qs : 0;
        const int db = b.rs - b.qs > 0 ? b.rs - b.qs : 0;
        if (da != db) return da < db;
    }
    if (a.n_hits != b.n_hits) return a.n_hits > b.n_hits;
    if (a.qe != b.qe) return a.qe < b.qe;
    if (a.qs != b.qs) return a.qs < b.qs;
    if (a.re != b.re) return a.re < b.re;
    if (a.rs != b.rs) return a.rs < b.rs;
    return nam_score(a) > nam_score(b);
}

__device__ __forceinline__ uint32_t next_pow2(uint32_t n) {
    return n <= 1 ? 1 : 1u << (32 - __clz(n - 1));
}

// Warp bitonic sort of u64 keys; keys must have room for next_pow2(n) entries.
__device__ inline void warp_sort_u64(uint64_t* keys, uint32_t n) {
    const uint32_t lane = lane_id();
    const uint32_t P = next_pow2(n);
    for (uint32_t i = n + lane; i < P; i += 32) keys[i] = ~0ULL;
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = keys[i], b = keys[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Warp bitonic sort of indices into nams[] by nam_before; idx must have room for
// next_pow2(n) entries.
__device__ inline void warp_sort_nams(const NamState* nams, uint32_t* idx, uint32_t n, int mode) {
    const uint32_t lane = lane_id();
    const uint32_t P = next_pow2(n);
    for (uint32_t i = lane; i < P; i += 32) idx[i] = i < n ? i : 0xFFFFFFFFu;
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const uint32_t a = idx[i], b = idx[ixj];
                    // padding (0xFFFFFFFF) sorts last
                    bool a_after_b;
                    if (a == 0xFFFFFFFFu) a_after_b = b != 0xFFFFFFFFu;
                    else if (b == 0xFFFFFFFFu) a_after_b = false;
                    else a_after_b = nam_before(nams[b], nams[a], mode);
                    const bool up = (i & k) == 0;
                    if (a_after_b == up) {
                        idx[i] = b;
                        idx[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

}  // namespace gbsa
