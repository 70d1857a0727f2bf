// lookup.cuh — index probes: StrobemerIndex::find / is_filtered / get_count and the
// hit-run walk of add_to_hits_per_ref, as device functions.
#pragma once

#include "index.h"

namespace gbsa {

// Hit record of the NAM stage (step2/my_struct.hpp:95-110 plus its map key):
// ref_rc = is_rc << 31 | ref_id.
struct HitRec {
    uint32_t ref_rc;
    int32_t qs, qe, rs, re;
};

// A hit as stored in the hit arena: 16 bytes, one vector load.  Query coordinates are
// below GBSA_MAX_READ_LEN, so query start and end share a word.
struct __align__(16) HitPacked {
    uint32_t ref_rc;
    uint32_t qse;    // query start | query end << 16
    int32_t rs, re;
};
static_assert(GBSA_MAX_READ_LEN < 65536, "query coordinates fit 16 bits");

__device__ __forceinline__ HitPacked pack_hit(uint32_t ref_rc, int qs, int qe, int rs, int re) {
    HitPacked p;
    p.ref_rc = ref_rc;
    p.qse = (uint32_t)qs | ((uint32_t)qe << 16);
    p.rs = rs;
    p.re = re;
    return p;
}

__device__ __forceinline__ uint64_t get_hash(const IndexView& I, uint64_t pos) {   // index.hpp:83-89
    return pos < I.n ? __ldg(&I.rs[pos].hash) : ~0ULL;
}

// Entry i of the bucket table (the 32-bit copy when the index has one).
__device__ __forceinline__ uint64_t bucket_start(const IndexView& I, uint64_t i) {
    return I.starts32 ? (uint64_t)__ldg(&I.starts32[i]) : __ldg(&I.starts[i]);
}

// StrobemerIndex::find (step2/index.hpp:57-81): first entry of the key's bucket
// whose hash equals the key, or kNotFound.  The in-bucket search examines entries
// in order until one is >= key (buckets hold ~2 entries on average) and switches to
// a binary search for long buckets; both give the reference's answer.  ex receives
// the number of entries examined by the linear rule (for the byte count).
__device__ __forceinline__ uint64_t index_find(const IndexView& I, uint64_t key, uint32_t* ex = nullptr,
                                               uint64_t* bucket_end = nullptr) {
    const uint64_t top = key >> (64 - I.bits);
    const uint64_t a = bucket_start(I, top);
    const uint64_t b = bucket_start(I, top + 1);
    if (bucket_end) *bucket_end = b;
    if (a >= b) {
        if (ex) *ex = 0;
        return kNotFound;
    }
    if (b - a <= 16) {
        for (uint64_t x = a; x < b; ++x) {
            const uint64_t h = __ldg(&I.rs[x].hash);
            if (h >= key) {
                if (ex) *ex = (uint32_t)(x - a + 1);
                return h == key ? x : kNotFound;
            }
        }
        if (ex) *ex = (uint32_t)(b - a);
        return kNotFound;
    }
    uint64_t lo = a, hi = b;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (__ldg(&I.rs[mid].hash) < key) lo = mid + 1;
        else hi = mid;
    }
    if (ex) *ex = (uint32_t)(lo - a + 1 < b - a ? lo - a + 1 : b - a);
    return (lo < b && __ldg(&I.rs[lo].hash) == key) ? lo : kNotFound;
}

__device__ __forceinline__ bool index_is_filtered(const IndexView& I, uint64_t pos) {   // index.hpp:91-93
    return get_hash(I, pos) == get_hash(I, pos + I.filter_cutoff);
}

// index_is_filtered for a position returned by index_find(key) whose bucket ends at
// bucket_end: an entry at or past the bucket's end has other top bits, so it cannot
// equal key, and the second load is needed only when pos + filter_cutoff is still
// inside the bucket (past the table's end get_hash reads all ones).
__device__ __forceinline__ bool index_is_filtered_in(const IndexView& I, uint64_t pos, uint64_t key,
                                                     uint64_t bucket_end) {
    const uint64_t p2 = pos + I.filter_cutoff;
    if (p2 >= bucket_end) return p2 >= I.n && key == ~0ULL;
    return __ldg(&I.rs[p2].hash) == key;
}

// StrobemerIndex::get_count (step2/index.hpp:115-147): length of the equal-hash run
// starting at pos, within the bucket.
__device__ __forceinline__ uint32_t index_get_count(const IndexView& I, uint64_t pos) {
    const uint64_t key = __ldg(&I.rs[pos].hash);
    const uint64_t end = bucket_start(I, (key >> (64 - I.bits)) + 1);
    if (end - pos < 8) {
        uint32_t c = 1;
        for (uint64_t x = pos + 1; x < end && __ldg(&I.rs[x].hash) == key; ++x) ++c;
        return c;
    }
    // upper bound of key in [pos, end)
    uint64_t lo = pos, hi = end;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (__ldg(&I.rs[mid].hash) <= key) lo = mid + 1;
        else hi = mid;
    }
    return (uint32_t)(lo - pos);
}

// add_to_hits_per_ref (step2/nam.cu:45-62): walks the run of entries equal to the
// hash at pos and calls emit(ref_id, rs, re) for each entry whose length difference
// to the query is <= the running minimum.  Stops at the end of the table.
template <class Emit>
__device__ __forceinline__ uint32_t walk_hit_run(const IndexView& I, int qs, int qe, uint64_t pos, Emit&& emit,
                                                 uint32_t* run_len = nullptr) {
    int min_diff = 0x7FFFFFFF;
    const uint64_t key = get_hash(I, pos);
    const uint64_t p0 = pos;
    uint32_t n = 0;
    for (; pos < I.n; ++pos) {
        const gbsa_ref_randstrobe e = I.rs[pos];
        if (e.hash != key) break;
        const int rs = (int)e.position;
        const int re = rs + (int)(e.packed & 0xFF) + I.k;
        const int d = (qe - qs) - (re - rs);
        const int diff = d < 0 ? -d : d;
        if (diff <= min_diff) {
            emit(e.packed >> 8, rs, re);
            min_diff = diff;
            ++n;
        }
    }
    if (run_len) *run_len = (uint32_t)(pos - p0);
    return n;
}

}  // namespace gbsa
