// nam.cuh — hit → NAM merging and NAM ordering, warp-cooperative.
//
// The reference keeps one hit list per (orientation, reference id) in robin_hood
// maps (step2/nam.cu:45-62) and merges each list on its own:
//   merge_hits_into_nams      (hit-major, step2/nam.cu:347-513; find_nams)
//   merge_hits_into_nams_fast (NAM-major, step2/nam.cu:94-343; find_nams_rescue)
// over hits sorted by (query_start, ref_start).  Lists never interact, so the warp
// processes all of them at once, one query randstrobe at a time: the hits of one
// query randstrobe share query_start, arrive sorted by ref_start (a hash run is
// sorted by position) and only meet NAMs of their own (orientation, reference id).
//
// Open NAMs are kept in creation order (the reference's open list order).  A NAM
// whose query_end is behind the current query_start can take no later hit; it is
// moved to the closed list before each query (the reference removes such NAMs at its
// flush points; which NAMs are removed when only changes iteration, not results).
//
//   hit-major: for each hit (ref_start order), the first open NAM in creation order
//     that accepts it takes it — found with a warp ballot over 32 NAMs at a time.
//   NAM-major: for each open NAM (creation order), the first untaken hit of the
//     query with ref_start in (ref_prev, ref_end] that extends it or lies inside it.
//     32 NAMs pick candidates in parallel; if two pick the same hit, the NAMs before
//     the first such clash are final and the rest pick again (each round settles at
//     least one more NAM, and a NAM is final exactly when no earlier NAM in the
//     round took a hit it would have considered).
#pragma once

#include "lookup.cuh"

namespace gbsa {

// Working state of one NAM (step2/my_struct.hpp:48-62 fields used by the merge).
struct NamState {
    int32_t qs, qe, qprev, rs, re, rprev, n_hits;
    uint32_t ref_rc;
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
    n.ref_rc = h.ref_rc;
    return n;
}

__device__ __forceinline__ void nam_add(NamState& n, const HitRec& h) {
    if (h.qe > n.qe && h.re > n.re) {
        n.qe = h.qe;
        n.re = h.re;
    }
    n.qprev = h.qs;
    n.rprev = h.rs;
    ++n.n_hits;
}

// Open and closed NAM lists of one read (any address space).
struct NamLists {
    NamState* open;
    NamState* closed;
    uint32_t n_open, n_closed;
    uint32_t cap;   // capacity of each list
};

// Moves open NAMs with query_end < qs (or all, when qs == INT_MAX) to the closed
// list, keeping the order of both lists.
__device__ __forceinline__ void nam_close_passed(NamLists& L, int qs) {
    const uint32_t lane = lane_id();
    uint32_t keep = 0, done = 0;
    for (uint32_t base = 0; base < L.n_open; base += 32) {
        const uint32_t o = base + lane;
        NamState n;
        bool valid = o < L.n_open, stay = false;
        if (valid) {
            n = L.open[o];
            stay = n.qe >= qs;
        }
        const uint32_t ms = __ballot_sync(0xFFFFFFFFu, valid && stay);
        const uint32_t mc = __ballot_sync(0xFFFFFFFFu, valid && !stay);
        __syncwarp();
        if (valid && stay) L.open[keep + __popc(ms & lanemask_lt())] = n;
        if (valid && !stay) L.closed[L.n_closed + done + __popc(mc & lanemask_lt())] = n;
        keep += __popc(ms);
        done += __popc(mc);
        __syncwarp();
    }
    L.n_open = keep;
    L.n_closed += done;
}

// Hits of one query randstrobe in compact form: they share query_start, query_end
// and orientation, so each hit is its ref_start and (ref id << 8 | ref span - k's
// offset), i.e. the RefRandstrobe position and packed word.
struct QueryHits {
    const uint32_t* rs;
    const uint32_t* packed;
    uint32_t n;
    int qs, qe;
    uint32_t dir;
    int k;
    __device__ HitRec get(uint32_t j) const {
        HitRec h;
        h.ref_rc = (dir << 31) | (packed[j] >> 8);
        h.qs = qs;
        h.qe = qe;
        h.rs = (int)rs[j];
        h.re = (int)rs[j] + (int)(packed[j] & 0xFF) + k;
        return h;
    }
};

// First untaken hit of the query at index from or later (hits sorted by rs) that NAM n
// would take, or -1.
__device__ __forceinline__ int nam_candidate_from(const NamState& n, const QueryHits& Q, const uint8_t* taken,
                                                  uint32_t from) {
    const uint32_t want = n.ref_rc & 0x7FFFFFFFu;
    for (uint32_t j = from; j < Q.n; ++j) {
        const int rs = (int)Q.rs[j];
        if (rs > n.re) break;
        if ((Q.packed[j] >> 8) != want || taken[j]) continue;
        const int re = rs + (int)(Q.packed[j] & 0xFF) + Q.k;
        if ((Q.qe > n.qe && re > n.re) || (Q.qe <= n.qe && re <= n.re)) return (int)j;
    }
    return -1;
}

// First untaken hit of the query (sorted by rs) that NAM n would take, or -1.
__device__ __forceinline__ int nam_candidate_q(const NamState& n, const QueryHits& Q, const uint8_t* taken) {
    uint32_t lo = 0, hi = Q.n;
    const int from = n.rprev + 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((int)Q.rs[mid] < from) lo = mid + 1;
        else hi = mid;
    }
    return nam_candidate_from(n, Q, taken, lo);
}

// One query of the NAM-major merge (hits in compact form), in one pass over the open
// list: NAMs the query has passed (query_end < query_start) go to the closed list in
// open-list order, as nam_close_passed; the others are compacted and, 32 at a time,
// each takes the first untaken hit it accepts (clash-resolved as described at the
// top of this file); untaken hits then open new NAMs in ref_start order.  taken: Q.n
// bytes of scratch.  The next 32 open NAMs are loaded while the current ones
// resolve (writes go only to positions already read).
__device__ __forceinline__ void nam_close_merge_q(NamLists& L, const QueryHits& Q, uint8_t* taken) {
    const uint32_t lane = lane_id();
    const uint32_t nh = Q.n;
    for (uint32_t j = lane; j < nh; j += 32) taken[j] = 0;
    __syncwarp();
    const uint32_t nn = L.n_open;
    const uint32_t dirbit = Q.dir << 31;
    uint32_t keep = 0, done = 0;
    NamState nxt;
    if (lane < nn) nxt = L.open[lane];
    for (uint32_t base = 0; base < nn; base += 32) {
        const uint32_t o = base + lane;
        const bool valid = o < nn;
        NamState mine = nxt;
        if (o + 32 < nn) nxt = L.open[o + 32];
        const bool close = valid && mine.qe < Q.qs;
        const bool stay = valid && !close;
        const uint32_t mc = __ballot_sync(0xFFFFFFFFu, close);
        const uint32_t ms = __ballot_sync(0xFFFFFFFFu, stay);
        bool resolved = !stay || (mine.ref_rc & 0x80000000u) != dirbit;
        bool dirty = false;
        for (;;) {
            int cand = -1;
            if (!resolved) cand = nam_candidate_q(mine, Q, taken);
            const uint32_t key = cand < 0 ? 0xFFFFFFFFu : (uint32_t)cand;
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
            const bool clash = cand >= 0 && (peers & lanemask_lt()) != 0;
            const uint32_t cm = __ballot_sync(0xFFFFFFFFu, clash);
            const uint32_t lim = cm ? (uint32_t)(__ffs(cm) - 1) : 32u;
            if (!resolved && lane < lim) {
                if (cand >= 0) {
                    taken[cand] = 1;
                    nam_add(mine, Q.get((uint32_t)cand));
                    dirty = true;
                }
                resolved = true;
            }
            __syncwarp();
            if (!cm) break;
        }
        if (close) L.closed[L.n_closed + done + __popc(mc & lanemask_lt())] = mine;
        if (stay) {
            const uint32_t to = keep + __popc(ms & lanemask_lt());
            if (dirty || to != o) L.open[to] = mine;
        }
        keep += __popc(ms);
        done += __popc(mc);
    }
    L.n_open = keep;
    L.n_closed += done;
    __syncwarp();
    // untaken hits open new NAMs, in ref_start order
    uint32_t added = 0;
    for (uint32_t b = 0; b < nh; b += 32) {
        const uint32_t j = b + lane;
        const bool mk = j < nh && !taken[j];
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, mk);
        if (mk) L.open[L.n_open + added + __popc(m & lanemask_lt())] = nam_from_hit(Q.get(j));
        added += __popc(m);
    }
    L.n_open += added;
    __syncwarp();
}

// Block-cooperative form of nam_close_merge_q, for reads with thousands of open NAMs
// (reads inside repeat families).  Same result; the open list is taken kBlockSeg NAMs
// at a time in three phases:
//   1. every warp, for its share of the segment's NAMs, finds the first hit each NAM
//      accepts with no hit taken yet (the query's taken flags are clear) and notes
//      which NAMs the query has passed;
//   2. warp 0 walks the segment in open-list order, 32 NAMs at a time, and settles the
//      clashes as nam_close_merge_q does: a NAM whose first choice an earlier NAM took
//      scans on from the next hit (hits before its first choice it rejects whatever is
//      taken);
//   3. every warp applies its NAMs' hits and writes them, by the segment's running
//      counts, to the other open list (NAMs staying, in order) or the closed list.
// The untaken hits then open new NAMs in ref_start order.  Every thread of the block
// calls it with the same arguments; L and spare are updated alike in every thread
// (spare becomes the open list).  cand: kBlockSeg words, bcnt: kBlockSeg / 32 words,
// tot: 3 words of shared memory; taken: Q.n bytes.
constexpr uint32_t kBlockSeg = 8192;
constexpr uint32_t kCandClose = 0xFFFFFFFEu;   // the query has passed the NAM
constexpr uint32_t kCandNone = 0xFFFFFFFFu;    // the NAM takes no hit of the query

__device__ inline void block_close_merge_q(NamLists& L, NamState*& spare, const QueryHits& Q, uint8_t* taken, uint32_t* cand,
                                    uint32_t* bcnt, uint32_t* tot) {
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t nh = Q.n;
    for (uint32_t j = threadIdx.x; j < nh; j += blockDim.x) taken[j] = 0;
    __syncthreads();
    const uint32_t nn = L.n_open;
    const uint32_t dirbit = Q.dir << 31;
    uint32_t keep = 0, done = 0;
    for (uint32_t seg = 0; seg < nn; seg += kBlockSeg) {
        const uint32_t sn = nn - seg < kBlockSeg ? nn - seg : kBlockSeg;
        const uint32_t nb = (sn + 31) >> 5;
        // 1. first choices
        for (uint32_t b = w; b < nb; b += nw) {
            const uint32_t i = (b << 5) + lane;
            const bool valid = i < sn;
            bool close = false;
            if (valid) {
                const NamState m = L.open[seg + i];
                uint32_t c = kCandNone;
                close = m.qe < Q.qs;
                if (close) {
                    c = kCandClose;
                } else if ((m.ref_rc & 0x80000000u) == dirbit) {
                    const int x = nam_candidate_q(m, Q, taken);
                    if (x >= 0) c = (uint32_t)x;
                }
                cand[i] = c;
            }
            const uint32_t ms = __ballot_sync(0xFFFFFFFFu, valid && !close);
            const uint32_t mc = __ballot_sync(0xFFFFFFFFu, close);
            if (lane == 0) bcnt[b] = (uint32_t)__popc(ms) | ((uint32_t)__popc(mc) << 16);
        }
        __syncthreads();
        // 2. clashes, in open-list order; bcnt becomes the exclusive running counts
        if (w == 0) {
            uint32_t run_s = 0, run_c = 0;
            uint32_t nxt = lane < sn ? cand[lane] : kCandNone;
            for (uint32_t b = 0; b < nb; ++b) {
                const uint32_t i = (b << 5) + lane;
                uint32_t c = nxt;
                nxt = i + 32 < sn ? cand[i + 32] : kCandNone;
                bool pending = c < kCandClose;
                for (;;) {
                    if (pending && taken[c]) {
                        const int x = nam_candidate_from(L.open[seg + i], Q, taken, c + 1);
                        if (x < 0) {
                            pending = false;
                            c = kCandNone;
                        } else {
                            c = (uint32_t)x;
                        }
                    }
                    const uint32_t key = pending ? c : 0xFFFFFFFFu;
                    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
                    const bool clash = pending && (peers & lanemask_lt()) != 0;
                    const uint32_t cm = __ballot_sync(0xFFFFFFFFu, clash);
                    const uint32_t lim = cm ? (uint32_t)(__ffs(cm) - 1) : 32u;
                    if (pending && lane < lim) {
                        taken[c] = 1;
                        pending = false;
                    }
                    __syncwarp();
                    if (!cm) break;
                }
                if (i < sn) cand[i] = c;
                const uint32_t v = bcnt[b];
                __syncwarp();
                if (lane == 0) bcnt[b] = run_s | (run_c << 16);
                run_s += v & 0xFFFFu;
                run_c += v >> 16;
            }
            if (lane == 0) {
                tot[0] = run_s;
                tot[1] = run_c;
            }
        }
        __syncthreads();
        // 3. apply and write
        for (uint32_t b = w; b < nb; b += nw) {
            const uint32_t i = (b << 5) + lane;
            const bool valid = i < sn;
            const uint32_t c = valid ? cand[i] : kCandNone;
            const bool close = c == kCandClose;
            const bool stay = valid && !close;
            const uint32_t ms = __ballot_sync(0xFFFFFFFFu, stay);
            const uint32_t mc = __ballot_sync(0xFFFFFFFFu, close);
            const uint32_t pre = bcnt[b];
            if (valid) {
                NamState m = L.open[seg + i];
                if (c < kCandClose) nam_add(m, Q.get(c));
                if (stay) spare[keep + (pre & 0xFFFFu) + __popc(ms & lanemask_lt())] = m;
                else L.closed[L.n_closed + done + (pre >> 16) + __popc(mc & lanemask_lt())] = m;
            }
        }
        keep += tot[0];
        done += tot[1];
        __syncthreads();
    }
    // untaken hits open new NAMs, in ref_start order
    if (w == 0) {
        uint32_t added = 0;
        for (uint32_t b = 0; b < nh; b += 32) {
            const uint32_t j = b + lane;
            const bool mk = j < nh && !taken[j];
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, mk);
            if (mk) spare[keep + added + __popc(m & lanemask_lt())] = nam_from_hit(Q.get(j));
            added += __popc(m);
        }
        if (lane == 0) tot[2] = added;
    }
    __syncthreads();
    NamState* old = L.open;
    L.open = spare;
    spare = old;
    L.n_open = keep + tot[2];
    L.n_closed += done;
    __syncthreads();
}

// Moves every open NAM to the closed list, in order (block-cooperative; every thread
// updates its copy of L alike).
__device__ inline void block_close_all(NamLists& L) {
    for (uint32_t o = threadIdx.x; o < L.n_open; o += blockDim.x) L.closed[L.n_closed + o] = L.open[o];
    L.n_closed += L.n_open;
    L.n_open = 0;
    __syncthreads();
}

// Warp-cooperative add_to_hits_per_ref (step2/nam.cu:45-62) for one query whose
// equal-hash run [pos, pos + cnt) is known: an entry is kept when its length
// difference is <= every earlier difference of the run (the reference's running
// minimum), found with a warp prefix minimum.  Writes the kept hits in compact form
// (rs[] = position, pk[] = packed, in run order) and returns their count (at most
// cap are written).  The entries are loaded 128 at a time, four per lane, so a run
// of up to 128 costs one memory round trip.
__device__ __forceinline__ uint32_t warp_walk_run_n(const IndexView& I, int qs, int qe, uint64_t pos, uint32_t cnt,
                                                    uint32_t* rs_out, uint32_t* pk_out, uint32_t cap) {
    const uint32_t lane = lane_id();
    int carry = 0x7FFFFFFF;
    uint32_t n = 0;
    const uint2* ent = reinterpret_cast<const uint2*>(I.rs + pos);   // (position, packed) at offset 8
    for (uint32_t base = 0; base < cnt; base += 128) {
        uint2 e[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t j = base + 32 * u + lane;
            e[u] = j < cnt ? __ldg(&ent[2 * (size_t)j + 1]) : make_uint2(0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t j = base + 32 * u + lane;
            const bool mine = j < cnt;
            int diff = 0x7FFFFFFF;
            if (mine) {
                const int d = (qe - qs) - ((int)(e[u].y & 0xFF) + I.k);
                diff = d < 0 ? -d : d;
            }
            int pm = diff;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xFFFFFFFFu, pm, o);
                if (lane >= (uint32_t)o) pm = v < pm ? v : pm;
            }
            int excl = __shfl_up_sync(0xFFFFFFFFu, pm, 1);
            if (lane == 0) excl = 0x7FFFFFFF;
            excl = excl < carry ? excl : carry;
            const bool keep = mine && diff <= excl;
            const uint32_t km = __ballot_sync(0xFFFFFFFFu, keep);
            if (keep) {
                const uint32_t k = n + __popc(km & lanemask_lt());
                if (k < cap) {
                    rs_out[k] = e[u].x;
                    pk_out[k] = e[u].y;
                }
            }
            n += __popc(km);
            const int tot = __shfl_sync(0xFFFFFFFFu, pm, 31);
            carry = tot < carry ? tot : carry;
        }
    }
    __syncwarp();
    return n;
}

// Score (step2/nam.cu:454-463): n_hits * (2*min_span - max_span) if positive, else 1.
__device__ __forceinline__ int nam_score_int(const NamState& n) {
    const int qspan = n.qe - n.qs, rspan = n.re - n.rs;
    const int mx = qspan > rspan ? qspan : rspan;
    const int mn = qspan < rspan ? qspan : rspan;
    const int v = 2 * mn - mx;
    return v > 0 ? n.n_hits * v : 1;
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
    o.ref_id = (int32_t)(n.ref_rc & 0x7FFFFFFFu);
    o.score = (float)nam_score_int(n);
    o.is_rc = (n.ref_rc >> 31) ? 1 : 0;
    o._pad[0] = o._pad[1] = o._pad[2] = 0;
}

// Sort key of a NAM: three u64 compared in order, then the index (stable).
//   GBSA_SORT_SCORE:     score desc, is_rc, ref_id, qs | qe, rs, re | n_hits desc
//   GBSA_SORT_REF_MATE2: is_rc, ref_id, max(0, rs-qs) | n_hits desc, qe, qs | re, rs
//                        (Nam::operator<, step2/my_struct.hpp:78-92)
//   GBSA_SORT_REF_MATE1: is_rc, ref_id | n_hits desc, qe, qs | re, rs
//                        (sort_nams_single2, step2/main.cu:2271-2289)
// All compared fields enter a key, so the order is total over the compared fields
// (the score is a function of n_hits and the coordinates).  Field widths: ref_id <
// 2^24 (RefRandstrobe packs it in 24 bits), query coordinates <= GBSA_MAX_READ_LEN,
// score < 2^24, NAM ref spans < 2^19.
struct NamKey {
    uint64_t k1, k2, k3;
    uint32_t idx;
    uint32_t pad;
};

__device__ __forceinline__ NamKey nam_key(const NamState& n, uint32_t idx, int mode) {
    const uint64_t rc = n.ref_rc >> 31, ref = n.ref_rc & 0xFFFFFFu;
    NamKey k;
    k.idx = idx;
    k.pad = 0;
    if (mode == GBSA_SORT_SCORE) {
        const uint64_t sc = (uint64_t)nam_score_int(n);
        k.k1 = ((0xFFFFFFull - sc) << 40) | (rc << 39) | (ref << 15) | ((uint64_t)n.qs & 0x7FFF);
        k.k2 = ((uint64_t)n.qe << 51) | ((uint64_t)(uint32_t)n.rs << 19) | ((uint64_t)(n.re - n.rs) & 0x7FFFF);
        k.k3 = 0xFFFFFFFFull - (uint32_t)n.n_hits;
    } else {
        const int d = n.rs - n.qs;
        const uint64_t diag = mode == GBSA_SORT_REF_MATE2 ? (uint64_t)(uint32_t)(d > 0 ? d : 0) : 0;
        k.k1 = (rc << 56) | (ref << 32) | diag;
        k.k2 = ((0xFFFFull - (uint32_t)n.n_hits) << 48) | ((uint64_t)n.qe << 24) | (uint64_t)n.qs;
        k.k3 = ((uint64_t)(uint32_t)n.re << 32) | (uint32_t)n.rs;
    }
    return k;
}

__device__ __forceinline__ bool key_less(const NamKey& a, const NamKey& b) {
    if (a.k1 != b.k1) return a.k1 < b.k1;
    if (a.k2 != b.k2) return a.k2 < b.k2;
    if (a.k3 != b.k3) return a.k3 < b.k3;
    return a.idx < b.idx;
}

__device__ __forceinline__ uint32_t next_pow2(uint32_t n) {
    return n <= 1 ? 1 : 1u << (32 - __clz(n - 1));
}

// Warp bitonic sort of n keys; keys must have room for next_pow2(n) entries.
__device__ inline void warp_sort_keys(NamKey* keys, uint32_t n) {
    const uint32_t lane = lane_id();
    const uint32_t P = next_pow2(n);
    for (uint32_t i = n + lane; i < P; i += 32) {
        NamKey k;
        k.k1 = k.k2 = k.k3 = ~0ULL;
        k.idx = 0xFFFFFFFFu;
        k.pad = 0;
        keys[i] = k;
    }
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < P; i += 32) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const NamKey a = keys[i], b = keys[ixj];
                    const bool up = (i & k) == 0;
                    if (key_less(b, a) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
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

}  // namespace gbsa
