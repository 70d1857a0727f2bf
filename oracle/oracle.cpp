/*
 * oracle.cpp — CPU restatement of strobealign's seeding → index lookup → NAM path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker that the CUDA path is compared with.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library.
 *
 * Every function cites the reference code it restates (paths inside the reference
 * project; step2/ unless noted).  The restatement keeps the reference's arithmetic
 * and control flow where they decide results (queue-minimum tie rules, strict vs
 * non-strict comparisons, the bucket-table build including its first-bucket quirk,
 * float products and ratios), and differs only where the reference leaves a result
 * unspecified or undefined:
 *   - NAMs are returned in emission order of the restated merge; callers compare
 *     them after oracle_sort_nams (the reference orders by robin_hood map iteration,
 *     step2/nam.cu:368, which is not a specified order).
 *   - The index is sorted by (hash, position, packed); the reference's pdqsort by
 *     (hash, position) leaves cross-contig ties unordered (step2/randstrobes.hpp:77-80).
 *   - k == 32 uses an all-ones k-mer mask; the reference shifts by 64 (UB).
 *   - find() treats a lower_bound that lands at the end of the table as "not found";
 *     the reference dereferences end() there (step2/index.hpp:79).
 *   - Hit-run walks stop at the end of the table; the reference walks past it
 *     forever when a hash equals UINT64_MAX (step2/nam.cu:52).
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <thread>
#include <unordered_map>
#include <string>
#include <vector>

namespace {

/* ---- hash.hpp:97-119 : single-u64 reduced xxh64 ---------------------------- */
constexpr uint64_t kPrime1 = 0x9E3779B185EBCA87ULL;
constexpr uint64_t kPrime2 = 0xC2B2AE3D27D4EB4FULL;
constexpr uint64_t kPrime3 = 0x165667B19E3779F9ULL;
constexpr uint64_t kPrime4 = 0x85EBCA77C2B2AE63ULL;
constexpr uint64_t kPrime5 = 0x27D4EB2F165667C5ULL;

inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

inline uint64_t xxh64(uint64_t v) {
    uint64_t acc = kPrime5 + 8;
    acc ^= rotl64(v * kPrime2, 31) * kPrime1;
    acc = rotl64(acc, 27) * kPrime1 + kPrime4;
    acc = (acc ^ (acc >> 33)) * kPrime2;
    acc = (acc ^ (acc >> 29)) * kPrime3;
    return acc ^ (acc >> 32);
}

/* ---- randstrobes.hpp:26-43 : base → 2-bit code, 4 = not ACGTU -------------- */
struct Nt4Table {
    unsigned char v[256];
    Nt4Table() {
        for (int i = 0; i < 256; ++i) v[i] = 4;
        for (int i = 0; i < 4; ++i) v[i] = (unsigned char)i;   /* raw codes 0..3 */
        const char* up = "ACGT";
        const char* lo = "acgt";
        for (int i = 0; i < 4; ++i) {
            v[(unsigned char)up[i]] = (unsigned char)i;
            v[(unsigned char)lo[i]] = (unsigned char)i;
        }
        v[(unsigned char)'U'] = 3;
        v[(unsigned char)'u'] = 3;
    }
};
const Nt4Table kNt4;

struct Syncmer {
    uint64_t hash;
    uint64_t pos;
};

/* ---- indexparameters.{hpp,cpp} ------------------------------------------------ */
bool verify_params(const gbsa_params& p) {
    if (p.k <= 7 || p.k > 32) return false;               /* indexparameters.hpp:25 */
    if (p.s > p.k) return false;                          /* :28 */
    if ((p.k - p.s) % 2 != 0) return false;               /* :31 */
    if (p.max_dist > 255) return false;                   /* :62 */
    if (p.w_min > p.w_max) return false;                  /* :65 */
    return true;
}

bool make_params(uint64_t r, int k, int s, int l, int u, int q, int max_dist, gbsa_params* out) {
    gbsa_params p{};
    p.canonical_read_length = (int32_t)r;
    p.k = k;
    p.s = s;
    p.t_syncmer = (k - s) / 2 + 1;                         /* indexparameters.hpp:19 */
    p.l = l;
    p.u = u;
    p.q = (uint64_t)(int64_t)q;
    p.max_dist = max_dist;
    if (k - s + 1 <= 0) return false;
    p.w_min = (unsigned)std::max(0, k / (k - s + 1) + l);  /* indexparameters.hpp:83 */
    p.w_max = (unsigned)(k / (k - s + 1) + u);
    if (!verify_params(p)) return false;
    *out = p;
    return true;
}

/* ---- randstrobes.cu:18-79 : canonical open syncmers ---------------------------- */
void canonical_syncmers(const gbsa_params& p, const char* seq, size_t len, std::vector<Syncmer>& out) {
    out.clear();
    const size_t k = (size_t)p.k, s = (size_t)p.s, t = (size_t)p.t_syncmer;
    const size_t W = k - s + 1;
    const uint64_t kmask = (k >= 32) ? ~0ULL : ((1ULL << (2 * k)) - 1);
    const uint64_t smask = (s >= 32) ? ~0ULL : ((1ULL << (2 * s)) - 1);
    const unsigned kshift = (unsigned)((k - 1) * 2);
    const unsigned sshift = (unsigned)((s - 1) * 2);

    std::vector<uint64_t> ring(W + 1);   /* queue of the last W s-mer hashes */
    size_t qhead = 0, qsize = 0;
    auto qat = [&](size_t j) -> uint64_t { return ring[(qhead + j) % (W + 1)]; };

    uint64_t min_val = UINT64_MAX;
    size_t min_pos = (size_t)-1;
    size_t l = 0;
    uint64_t xk0 = 0, xk1 = 0, xs0 = 0, xs1 = 0;
    for (size_t i = 0; i < len; ++i) {
        const int c = kNt4.v[(unsigned char)seq[i]];
        if (c >= 4) {                                   /* "N": restart (:70-76) */
            min_val = UINT64_MAX;
            min_pos = (size_t)-1;
            l = 0;
            xk0 = xk1 = xs0 = xs1 = 0;
            qhead = qsize = 0;
            continue;
        }
        xk0 = ((xk0 << 2) | (uint64_t)c) & kmask;
        xk1 = (xk1 >> 2) | ((uint64_t)(3 - c) << kshift);
        xs0 = ((xs0 << 2) | (uint64_t)c) & smask;
        xs1 = (xs1 >> 2) | ((uint64_t)(3 - c) << sshift);
        if (++l < s) continue;
        const uint64_t hs = xxh64(std::min(xs0, xs1));
        ring[(qhead + qsize) % (W + 1)] = hs;
        ++qsize;
        if (qsize < W) continue;
        if (qsize == W) {
            /* first full window: leftmost minimum (forward scan, strict <) (:38-45) */
            for (size_t j = 0; j < qsize; ++j) {
                if (qat(j) < min_val) {
                    min_val = qat(j);
                    min_pos = i - k + j + 1;
                }
            }
        } else {
            qhead = (qhead + 1) % (W + 1);               /* pop_front (:48) */
            --qsize;
            if (min_pos == i - k) {
                /* popped the minimum: rightmost minimum by reverse scan (:50-58) */
                min_val = UINT64_MAX;
                min_pos = i - s + 1;
                for (size_t jj = qsize; jj-- > 0;) {
                    if (qat(jj) < min_val) {
                        min_val = qat(jj);
                        min_pos = i - k + jj + 1;
                    }
                }
            } else if (hs < min_val) {                  /* newest is a new strict minimum (:59-62) */
                min_val = hs;
                min_pos = i - s + 1;
            }
        }
        if (min_pos == i - k + t) {                     /* minimum at the t-th s-mer (:64-69) */
            out.push_back(Syncmer{xxh64(std::min(xk0, xk1)), i - k + 1});
        }
    }
}

/* ---- randstrobes.cu:136-159 : RandstrobeIterator::get ------------------------ */
struct Strobe {
    uint64_t hash;
    uint32_t s1;
    uint32_t s2;
};

Strobe randstrobe_at(const gbsa_params& p, const std::vector<Syncmer>& v, unsigned j) {
    const unsigned w_end = (unsigned)std::min((size_t)(j + p.w_max), v.size() - 1);
    const Syncmer s1 = v[j];
    const uint64_t max_position = s1.pos + (unsigned)p.max_dist;
    Syncmer s2 = s1;
    uint64_t best = UINT64_MAX;
    for (unsigned i = j + p.w_min; i <= w_end && v[i].pos <= max_position; ++i) {
        const uint64_t score = (uint64_t)__builtin_popcountll((s1.hash ^ v[i].hash) & p.q);
        if (score < best) {                           /* first minimum wins */
            best = score;
            s2 = v[i];
        }
    }
    return Strobe{s1.hash + s2.hash, (uint32_t)s1.pos, (uint32_t)s2.pos};   /* randstrobes.hpp:61-63 */
}

/* ---- randstrobes.cu:195-241 : randstrobes_query --------------------------------- */
void randstrobes_query(const gbsa_params& p, const char* seq, size_t len,
                       std::vector<gbsa_query_randstrobe>& out) {
    out.clear();
    if (len < p.w_max) return;
    std::vector<Syncmer> sm;
    canonical_syncmers(p, seq, len, sm);
    if (sm.empty()) return;
    auto emit = [&](bool rev) {
        for (unsigned j = 0; j + p.w_min < sm.size(); ++j) {
            const Strobe r = randstrobe_at(p, sm, j);
            gbsa_query_randstrobe q{};
            q.hash = r.hash;
            q.start = r.s1;
            q.end = r.s2 + (uint32_t)p.k;
            q.is_reverse = rev ? 1 : 0;
            out.push_back(q);
        }
    };
    emit(false);
    std::reverse(sm.begin(), sm.end());
    for (auto& x : sm) x.pos = len - x.pos - (size_t)p.k;
    emit(true);
}

/* ---- index.hpp / index.cu ------------------------------------------------------- */
int pick_bits(const gbsa_params& p, uint64_t size) {           /* index.cu:137-141 */
    const uint64_t est = size / (uint64_t)(p.k - p.s + 1);
    if (est == 0) return 8;   /* log2(0) = -inf; the reference's int cast is UB there */
    const int b = (int)std::log2((double)est) - 1;
    return std::clamp(b, 8, 31);
}

struct IndexCpu {
    gbsa_params p{};
    int bits = 0;
    uint32_t filter_cutoff = 0;
    std::vector<gbsa_ref_randstrobe> rs;
    std::vector<uint64_t> starts;
    gbsa_index_info info{};

    uint64_t get_hash(uint64_t pos) const {                   /* index.hpp:83-89 */
        return pos < rs.size() ? rs[pos].hash : UINT64_MAX;
    }
    bool is_filtered(uint64_t pos) const {                    /* index.hpp:91-93 */
        return get_hash(pos) == get_hash(pos + filter_cutoff);
    }
    uint64_t find(uint64_t key) const {                       /* index.hpp:57-81 */
        const unsigned top = (unsigned)(key >> (64 - bits));
        uint64_t a = starts[top];
        const uint64_t b = starts[top + 1];
        if (a == b) return UINT64_MAX;
        if (b - a < 4) {
            for (; a < b; ++a) {
                if (rs[a].hash == key) return a;
                if (rs[a].hash > key) return UINT64_MAX;
            }
            return UINT64_MAX;
        }
        auto it = std::lower_bound(rs.begin() + (long)a, rs.begin() + (long)b, key,
                                   [](const gbsa_ref_randstrobe& e, uint64_t k) { return e.hash < k; });
        if (it != rs.end() && it->hash == key) return (uint64_t)(it - rs.begin());
        return UINT64_MAX;
    }
    uint32_t get_count(uint64_t pos) const {                  /* index.hpp:115-147 */
        const uint64_t key = rs[pos].hash;
        const unsigned top = (unsigned)(key >> (64 - bits));
        const uint64_t end = starts[top + 1];
        if (end - pos < 8) {
            uint64_t count = 1;
            for (uint64_t q = pos + 1; q < end; ++q) {
                if (rs[q].hash == key) ++count;
                else break;
            }
            return (uint32_t)count;
        }
        auto it = std::upper_bound(rs.begin() + (long)pos, rs.begin() + (long)end, key,
                                   [](uint64_t k, const gbsa_ref_randstrobe& e) { return k < e.hash; });
        return (uint32_t)((it - rs.begin()) - (long)pos);
    }
};

/* Bucket table and repetition statistics of a sorted entry array (index.cu:176-243):
 * starts (2^bits + 1 entries), filter_cutoff and the counters of info. */
void finish_index(const gbsa_ref_randstrobe* rs, uint64_t n, int bits, float f, std::vector<uint64_t>& st,
                  uint32_t& filter_cutoff, gbsa_index_info& info) {
    const uint64_t nb = (1ULL << bits) + 1;
    st.clear();
    st.reserve(nb);
    std::vector<uint64_t> rep_counts;
    uint64_t once = 0, high = 0, mid = 0;
    uint64_t unique = n == 0 ? 0 : 1;
    uint64_t prev = n == 0 ? 0 : rs[0].hash;
    unsigned run = 0;
    auto close_run = [&](unsigned cnt) {
        if (cnt == 1) {
            ++once;
        } else {
            if (cnt > 100) ++high;
            else ++mid;
            rep_counts.push_back(cnt);
        }
    };
    for (uint64_t pos = 0; pos < n; ++pos) {
        const uint64_t cur = rs[pos].hash;
        if (cur == prev) {
            ++run;
            continue;
        }
        ++unique;
        close_run(run);
        run = 1;
        const unsigned top = (unsigned)(cur >> (64 - bits));
        /* Buckets up to `top` start here; bucket top(hash[0]) and the empty ones
         * before it therefore start at the second distinct hash (index.cu:207-210). */
        while (st.size() <= top) st.push_back(pos);
        prev = cur;
    }
    close_run(run);
    while (st.size() < nb) st.push_back(n);

    std::sort(rep_counts.begin(), rep_counts.end(), [](uint64_t a, uint64_t b) { return a > b; });
    const uint64_t index_cutoff = (uint64_t)((float)unique * f);   /* float product, index.cu:232 */
    unsigned fc;
    if (!rep_counts.empty()) {
        fc = (unsigned)(index_cutoff < rep_counts.size() ? rep_counts[index_cutoff] : rep_counts.back());
        fc = std::max(30U, fc);
        fc = std::min(100U, fc);
    } else {
        fc = 30;
    }
    filter_cutoff = fc;
    info.tot_occur_once = once;
    info.tot_high_ab = high;
    info.tot_mid_ab = mid;
    info.index_cutoff = index_cutoff;
    info.distinct_strobemers = unique;
}

/* Entries of contig c (index.cu:280-311, assign_randstrobes with the RandstrobeGenerator
 * of randstrobes.cu:161-190): fn(entry) for each, in generation order. */
template <class Fn>
void contig_entries(const gbsa_params& p, const char* seq, uint64_t len, uint32_t c, std::vector<Syncmer>& v,
                    Fn&& fn) {
    v.clear();
    canonical_syncmers(p, seq, len, v);
    if (len < p.w_max) return;                                  /* index.cu:282-284 */
    for (unsigned j = 0; j + p.w_min < v.size(); ++j) {
        const Strobe r = randstrobe_at(p, v, j);
        uint32_t packed = (uint32_t)((uint64_t)c << 8);
        packed = packed + (r.s2 - r.s1);
        fn(gbsa_ref_randstrobe{r.hash, r.s1, packed});
    }
}

/* index.cu:28-41 (count_randstrobes), 280-311 (assign_randstrobes with the
 * RandstrobeGenerator of randstrobes.cu:161-190), 143-244 (populate). */
void populate(IndexCpu& idx, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
              uint32_t n_contigs, float f) {
    const gbsa_params& p = idx.p;
    std::vector<Syncmer> sm;
    uint64_t total = 0;
    for (uint32_t c = 0; c < n_contigs; ++c) {
        sm.clear();
        canonical_syncmers(p, seqs + offsets[c], lengths[c], sm);
        const uint64_t n = sm.size();
        total += n < p.w_min ? 0 : n - p.w_min;
    }
    idx.info.tot_strobemer_count = total;
    idx.rs.clear();
    idx.rs.reserve(total);
    for (uint32_t c = 0; c < n_contigs; ++c)
        contig_entries(p, seqs + offsets[c], lengths[c], c, sm, [&](const gbsa_ref_randstrobe& e) { idx.rs.push_back(e); });
    /* contigs shorter than w_max count but assign nothing: their slots stay zero */
    idx.rs.resize(total, gbsa_ref_randstrobe{0, 0, 0});
    std::sort(idx.rs.begin(), idx.rs.end(), [](const gbsa_ref_randstrobe& a, const gbsa_ref_randstrobe& b) {
        if (a.hash != b.hash) return a.hash < b.hash;
        if (a.position != b.position) return a.position < b.position;
        return a.packed < b.packed;
    });
    finish_index(idx.rs.data(), idx.rs.size(), idx.bits, f, idx.starts, idx.filter_cutoff, idx.info);
}

/* ---- nam.cu ------------------------------------------------------------------ */
struct Hit {
    int qs, qe, rs, re;
};
inline bool hit_less(const Hit& a, const Hit& b) {            /* my_struct.hpp:100-103 */
    if (a.qs == b.qs) return a.rs < b.rs;
    return a.qs < b.qs;
}
using HitsPerRef = std::unordered_map<unsigned, std::vector<Hit>>;

/* nam.cu:45-62 : add_to_hits_per_ref, the running-minimum length-difference filter */
template <class Fn>
void walk_run(const IndexCpu& idx, int qs, int qe, uint64_t pos, Fn&& emit) {
    int min_diff = INT_MAX;
    const uint64_t key = idx.get_hash(pos);
    for (; pos < idx.rs.size() && idx.rs[pos].hash == key; ++pos) {
        const int rs = (int)idx.rs[pos].position;
        const int re = rs + (int)(idx.rs[pos].packed & 0xFF) + idx.p.k;
        const int diff = std::abs((qe - qs) - (re - rs));
        if (diff <= min_diff) {
            emit((unsigned)(idx.rs[pos].packed >> 8), Hit{qs, qe, rs, re});
            min_diff = diff;
        }
    }
}

void add_to_hits_per_ref(HitsPerRef& hpr, int qs, int qe, const IndexCpu& idx, uint64_t pos) {
    walk_run(idx, qs, qe, pos, [&](unsigned ref, const Hit& h) { hpr[ref].push_back(h); });
}

inline float nam_score(const gbsa_nam& n) {                   /* nam.cu:454-463 */
    const int qspan = n.query_end - n.query_start;
    const int rspan = n.ref_end - n.ref_start;
    const int mx = std::max(qspan, rspan), mn = std::min(qspan, rspan);
    return (2 * mn - mx) > 0 ? (float)(n.n_hits * (2 * mn - mx)) : 1.0f;
}

gbsa_nam new_nam(const Hit& h, unsigned ref, bool rc) {
    gbsa_nam n{};
    n.query_start = h.qs;
    n.query_end = h.qe;
    n.ref_start = h.rs;
    n.ref_end = h.re;
    n.ref_id = (int)ref;
    n.query_prev_hit_startpos = h.qs;
    n.ref_prev_hit_startpos = h.rs;
    n.n_hits = 1;
    n.is_rc = rc ? 1 : 0;
    return n;
}

void flush_passed(std::vector<gbsa_nam>& open, int qs, std::vector<gbsa_nam>& nams) {
    for (auto& n : open) {
        if (n.query_end < qs) {
            n.score = nam_score(n);
            n.nam_id = (int)nams.size();
            nams.push_back(n);
        }
    }
    open.erase(std::remove_if(open.begin(), open.end(), [qs](const gbsa_nam& n) { return n.query_end < qs; }),
               open.end());
}

void flush_all(std::vector<gbsa_nam>& open, std::vector<gbsa_nam>& nams) {
    for (auto& n : open) {
        n.score = nam_score(n);
        n.nam_id = (int)nams.size();
        nams.push_back(n);
    }
}

/* nam.cu:347-513 : merge_hits_into_nams (hit-major) */
void merge_hit_major(std::vector<Hit>& hits, unsigned ref, int k, bool sort, bool rc, std::vector<gbsa_nam>& nams) {
    if (sort) std::sort(hits.begin(), hits.end(), hit_less);
    std::vector<gbsa_nam> open;
    unsigned prev_q_start = 0;
    for (const Hit& h : hits) {
        bool added = false;
        for (auto& o : open) {
            if (o.query_prev_hit_startpos < h.qs && h.qs <= o.query_end &&
                o.ref_prev_hit_startpos < h.rs && h.rs <= o.ref_end) {
                if (h.qe > o.query_end && h.re > o.ref_end) {
                    o.query_end = h.qe;
                    o.ref_end = h.re;
                    o.query_prev_hit_startpos = h.qs;
                    o.ref_prev_hit_startpos = h.rs;
                    ++o.n_hits;
                    added = true;
                    break;
                } else if (h.qe <= o.query_end && h.re <= o.ref_end) {
                    o.query_prev_hit_startpos = h.qs;
                    o.ref_prev_hit_startpos = h.rs;
                    ++o.n_hits;
                    added = true;
                    break;
                }
            }
        }
        if (!added) open.push_back(new_nam(h, ref, rc));
        if ((unsigned)h.qs > prev_q_start + (unsigned)k) {
            flush_passed(open, h.qs, nams);
            prev_q_start = (unsigned)h.qs;
        }
    }
    flush_all(open, nams);
}

/* nam.cu:94-343 : merge_hits_into_nams_fast (NAM-major, one query_start group at a time) */
void merge_nam_major(std::vector<Hit>& hits, unsigned ref, int k, bool sort, bool rc, std::vector<gbsa_nam>& nams) {
    if (sort) std::sort(hits.begin(), hits.end(), hit_less);
    std::vector<gbsa_nam> open;
    unsigned prev_q_start = 0;
    std::vector<char> added;
    for (size_t i = 0; i < hits.size();) {
        const size_t g0 = i;
        size_t g1 = i + 1;
        while (g1 < hits.size() && hits[g1].qs == hits[i].qs) ++g1;
        i = g1;
        const size_t gn = g1 - g0;
        added.assign(gn, 0);
        const int qs = hits[g0].qs;
        size_t done = 0;
        std::sort(hits.begin() + (long)g0, hits.begin() + (long)g1, hit_less);
        for (auto& o : open) {
            auto lb = [&](int value) {
                return (size_t)(std::lower_bound(hits.begin() + (long)g0, hits.begin() + (long)g1, value,
                                                 [](const Hit& h, int v) { return h.rs < v; }) -
                                hits.begin());
            };
            const size_t lo = lb(o.ref_prev_hit_startpos + 1);
            const size_t hi = lb(o.ref_end + 1);
            for (size_t j = lo; j < hi; ++j) {
                if (added[j - g0]) continue;
                if (qs <= o.query_end) {
                    const Hit& h = hits[j];
                    if (o.ref_prev_hit_startpos < h.rs && h.rs <= o.ref_end) {
                        if (h.qe > o.query_end && h.re > o.ref_end) {
                            o.query_end = h.qe;
                            o.ref_end = h.re;
                            o.query_prev_hit_startpos = h.qs;
                            o.ref_prev_hit_startpos = h.rs;
                            ++o.n_hits;
                            added[j - g0] = 1;
                            ++done;
                            break;
                        } else if (h.qe <= o.query_end && h.re <= o.ref_end) {
                            o.query_prev_hit_startpos = h.qs;
                            o.ref_prev_hit_startpos = h.rs;
                            ++o.n_hits;
                            added[j - g0] = 1;
                            ++done;
                            break;
                        }
                    }
                }
            }
            if (done == gn) break;
        }
        for (size_t j = 0; j < gn; ++j) {
            if (!added[j]) open.push_back(new_nam(hits[g0 + j], ref, rc));
        }
        if ((unsigned)qs > prev_q_start + (unsigned)k) {
            flush_passed(open, qs, nams);
            prev_q_start = (unsigned)qs;
        }
    }
    flush_all(open, nams);
}

/* nam.cu:748-905 : find_nams (untimed variant; same arithmetic as :553-747) */
std::vector<gbsa_nam> find_nams(const IndexCpu& idx, const gbsa_query_randstrobe* q, size_t nq, float* frac) {
    HitsPerRef hpr[2];
    int nr_good = 0, total = 0;
    for (size_t i = 0; i < nq; ++i) {
        const uint64_t pos = idx.find(q[i].hash);
        if (pos == UINT64_MAX) continue;
        ++total;
        if (idx.is_filtered(pos)) continue;
        ++nr_good;
        add_to_hits_per_ref(hpr[q[i].is_reverse ? 1 : 0], (int)q[i].start, (int)q[i].end, idx, pos);
    }
    *frac = total > 0 ? ((float)nr_good) / ((float)total) : 1.0f;
    std::vector<gbsa_nam> nams;
    for (int rc = 0; rc < 2; ++rc) {
        for (auto& kv : hpr[rc]) merge_hit_major(kv.second, kv.first, idx.p.k, true, rc == 1, nams);
    }
    return nams;
}

/* nam.cu:927-985 : find_nams_rescue (pre_sort variant) */
struct RescueHit {
    uint64_t position;
    unsigned count, qs, qe;
};
std::vector<gbsa_nam> find_nams_rescue(const IndexCpu& idx, const gbsa_query_randstrobe* q, size_t nq,
                                       unsigned rescue_cutoff, unsigned count_cap) {
    std::vector<RescueHit> by_dir[2];
    for (size_t i = 0; i < nq; ++i) {
        const uint64_t pos = idx.find(q[i].hash);
        if (pos == UINT64_MAX) continue;
        by_dir[q[i].is_reverse ? 1 : 0].push_back(RescueHit{pos, idx.get_count(pos), q[i].start, q[i].end});
    }
    HitsPerRef hpr[2];
    for (int d = 0; d < 2; ++d) {
        auto& v = by_dir[d];
        std::sort(v.begin(), v.end(), [](const RescueHit& a, const RescueHit& b) {   /* cmp1, nam.cu:909-912 */
            if (a.count != b.count) return a.count < b.count;
            if (a.qs != b.qs) return a.qs < b.qs;
            return a.qe < b.qe;
        });
        std::vector<RescueHit> taken;
        int cnt = 0;
        for (const auto& rh : v) {
            if ((rh.count > rescue_cutoff && cnt >= 5) || rh.count > count_cap) break;
            taken.push_back(rh);
            ++cnt;
        }
        std::sort(taken.begin(), taken.end(), [](const RescueHit& a, const RescueHit& b) { return a.qs < b.qs; });
        for (const auto& rh : taken) add_to_hits_per_ref(hpr[d], (int)rh.qs, (int)rh.qe, idx, rh.position);
    }
    std::vector<gbsa_nam> nams;
    for (int rc = 0; rc < 2; ++rc) {
        for (auto& kv : hpr[rc]) merge_nam_major(kv.second, kv.first, idx.p.k, false, rc == 1, nams);
    }
    return nams;
}

/* ---- NAM orders ------------------------------------------------------------- */
inline int score_key(const gbsa_nam& n) { return (int)n.score; }   /* integer valued, < 2^24 */

bool less_score(const gbsa_nam& a, const gbsa_nam& b) {
    if (a.score != b.score) return a.score > b.score;
    if (a.is_rc != b.is_rc) return a.is_rc < b.is_rc;
    if (a.ref_id != b.ref_id) return a.ref_id < b.ref_id;
    if (a.query_start != b.query_start) return a.query_start < b.query_start;
    if (a.query_end != b.query_end) return a.query_end < b.query_end;
    if (a.ref_start != b.ref_start) return a.ref_start < b.ref_start;
    if (a.ref_end != b.ref_end) return a.ref_end < b.ref_end;
    return a.n_hits > b.n_hits;
}

/* my_struct.hpp:78-92 (mate 2) and main.cu:2271-2289 (mate 1), ties broken by the
 * remaining compared fields so that the order is total. */
bool less_ref(const gbsa_nam& a, const gbsa_nam& b, bool with_diag) {
    if (a.is_rc != b.is_rc) return a.is_rc < b.is_rc;
    if (a.ref_id != b.ref_id) return a.ref_id < b.ref_id;
    if (with_diag) {
        const int d1 = std::max(0, a.ref_start - a.query_start);
        const int d2 = std::max(0, b.ref_start - b.query_start);
        if (d1 != d2) return d1 < d2;
    }
    if (a.n_hits != b.n_hits) return a.n_hits > b.n_hits;
    if (a.query_end != b.query_end) return a.query_end < b.query_end;
    if (a.query_start != b.query_start) return a.query_start < b.query_start;
    if (a.ref_end != b.ref_end) return a.ref_end < b.ref_end;
    if (a.ref_start != b.ref_start) return a.ref_start < b.ref_start;
    return score_key(a) > score_key(b);
}

void sort_nams(gbsa_nam* v, size_t n, int mode) {
    if (mode == GBSA_SORT_REF_MATE2) {
        std::sort(v, v + n, [](const gbsa_nam& a, const gbsa_nam& b) { return less_ref(a, b, true); });
    } else if (mode == GBSA_SORT_REF_MATE1) {
        std::sort(v, v + n, [](const gbsa_nam& a, const gbsa_nam& b) { return less_ref(a, b, false); });
    } else {
        std::sort(v, v + n, less_score);
    }
}

/* Rescue trigger and cutoff: step2/main.cu:3211 (nonrepetitive_fraction < 0.7, a
 * double comparison, or no hits) and step2/main.cu:4204 (R * filter_cutoff). */
unsigned rescue_cutoff_for(const IndexCpu& idx, int rescue_level) {
    return rescue_level < 100 ? (unsigned)(rescue_level * (int)idx.filter_cutoff) : 100u;
}

struct ReadResult {
    std::vector<gbsa_nam> nams;
    float frac = 1.0f;
    bool rescued = false;
};

void map_one(const IndexCpu& idx, const gbsa_map_options& opt, const char* seq, size_t len,
             std::vector<gbsa_query_randstrobe>& qbuf, ReadResult& r) {
    randstrobes_query(idx.p, seq, len, qbuf);
    r.nams = find_nams(idx, qbuf.data(), qbuf.size(), &r.frac);
    r.rescued = false;
    if (opt.rescue_level > 1 && (r.nams.empty() || (double)r.frac < 0.7)) {
        r.nams = find_nams_rescue(idx, qbuf.data(), qbuf.size(), rescue_cutoff_for(idx, opt.rescue_level),
                                  opt.rescue_count_cap);
        r.rescued = true;
    }
    sort_nams(r.nams.data(), r.nams.size(), opt.sort_mode);
}

template <class Fn>
void parallel_for(uint32_t n, int n_threads, Fn&& fn) {
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (n_threads == 1 || n < 64) {
        for (uint32_t i = 0; i < n; ++i) fn(i, 0);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t) {
        th.emplace_back([&, t]() {
            for (;;) {
                const uint32_t a = next.fetch_add(256);
                if (a >= n) break;
                const uint32_t b = std::min(n, a + 256);
                for (uint32_t i = a; i < b; ++i) fn(i, t);
            }
        });
    }
    for (auto& x : th) x.join();
}

}  // namespace

struct oracle_index {
    IndexCpu idx;
};

extern "C" {

uint64_t oracle_xxh64(uint64_t x) { return xxh64(x); }

/* indexparameters.cpp:137-182 */
int oracle_params_from_read_length(int read_length, int k, int s, int l, int u, int c, int max_seed_len,
                                   gbsa_params* out) {
    struct Profile { int r, thr, k, s_off, l, u; };
    static const Profile profiles[] = {
        {50, 90, 20, -4, -3, 2},   {100, 110, 20, -4, -2, 2}, {125, 135, 20, -4, -1, 4},
        {150, 175, 20, -4, 1, 7},  {250, 275, 20, -4, 4, 13}, {300, 375, 22, -4, 2, 12},
        {400, INT_MAX, 23, -6, 2, 12},
    };
    uint64_t canonical = 50;
    for (const auto& pr : profiles) {
        if (read_length <= pr.thr) {
            if (k == GBSA_DEFAULT) k = pr.k;
            if (s == GBSA_DEFAULT) s = k + pr.s_off;
            if (l == GBSA_DEFAULT) l = pr.l;
            if (u == GBSA_DEFAULT) u = pr.u;
            canonical = (uint64_t)pr.r;
            break;
        }
    }
    int max_dist;
    if (max_seed_len == GBSA_DEFAULT) {
        max_dist = std::max((int)canonical - 70, k);
        max_dist = std::min(255, max_dist);
    } else {
        max_dist = max_seed_len - k;
    }
    const int q = (int)(std::pow(2, c == GBSA_DEFAULT ? 8 : c) - 1);
    return make_params(canonical, k, s, l, u, q, max_dist, out) ? GBSA_OK : GBSA_ERR_PARAM;
}

int oracle_pick_bits(const gbsa_params* p, uint64_t total_length) { return pick_bits(*p, total_length); }

int64_t oracle_syncmers(const gbsa_params* p, const char* seq, uint64_t len, uint64_t* hashes,
                        uint64_t* positions, uint64_t cap) {
    std::vector<Syncmer> v;
    canonical_syncmers(*p, seq, len, v);
    const uint64_t n = std::min<uint64_t>(cap, v.size());
    for (uint64_t i = 0; i < n; ++i) {
        hashes[i] = v[i].hash;
        positions[i] = v[i].pos;
    }
    return (int64_t)v.size();
}

int64_t oracle_randstrobes_query(const gbsa_params* p, const char* seq, uint64_t len,
                                 gbsa_query_randstrobe* out, uint64_t cap) {
    std::vector<gbsa_query_randstrobe> v;
    randstrobes_query(*p, seq, len, v);
    if (v.size() > cap) return -(int64_t)v.size() - 1;
    if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(gbsa_query_randstrobe));
    return (int64_t)v.size();
}

oracle_index* oracle_index_build(const gbsa_params* p, const char* seqs, const uint64_t* offsets,
                                 const uint64_t* lengths, uint32_t n_contigs, int bits, float f) {
    auto* h = new oracle_index();
    h->idx.p = *p;
    uint64_t total_len = 0;
    for (uint32_t c = 0; c < n_contigs; ++c) total_len += lengths[c];
    h->idx.bits = bits == -1 ? pick_bits(*p, total_len) : bits;
    if (h->idx.bits < 8 || h->idx.bits > 31) {
        delete h;
        return nullptr;
    }
    populate(h->idx, seqs, offsets, lengths, n_contigs, f);
    h->idx.info.size = h->idx.rs.size();
    h->idx.info.bits = h->idx.bits;
    h->idx.info.filter_cutoff = h->idx.filter_cutoff;
    return h;
}

oracle_index* oracle_index_load(const gbsa_params* p, const gbsa_ref_randstrobe* rs, uint64_t n,
                                const uint64_t* starts, int bits, uint32_t filter_cutoff) {
    auto* h = new oracle_index();
    h->idx.p = *p;
    h->idx.bits = bits;
    h->idx.filter_cutoff = filter_cutoff;
    h->idx.rs.assign(rs, rs + n);
    h->idx.starts.assign(starts, starts + (1ULL << bits) + 1);
    h->idx.info.size = n;
    h->idx.info.bits = bits;
    h->idx.info.filter_cutoff = filter_cutoff;
    return h;
}

/* Checks an index built elsewhere (the GPU's, exported to host memory) against this
 * restatement without building one: the entries the contigs generate (index.cu:280-311,
 * generated per contig on n_threads threads) must be the given entries as a multiset
 * (same count, and two order-independent 64-bit sums of a mix of every entry), the
 * given entries must be sorted by (hash, position, packed), which orders a multiset
 * uniquely, and the bucket table and filter cutoff recomputed from them must be the
 * given ones.  Returns 0 when all hold, else the first failed check: 1 count, 2 order,
 * 3 multiset digest, 4 bucket table, 5 filter cutoff.  report (5 values): expected
 * count, given count, index of the first out-of-order entry (or UINT64_MAX), expected
 * filter cutoff, first differing bucket (or UINT64_MAX). */
int oracle_index_verify(const gbsa_params* p, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
                        uint32_t n_contigs, float f, const gbsa_ref_randstrobe* rs, uint64_t n,
                        const uint64_t* starts, int bits, uint32_t filter_cutoff, int n_threads, uint64_t* report) {
    auto mix = [](uint64_t x) {
        x += 0x9E3779B97F4A7C15ULL;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
        return x ^ (x >> 31);
    };
    auto digest = [&](const gbsa_ref_randstrobe& e, uint64_t& s1, uint64_t& s2) {
        const uint64_t a = mix(e.hash);
        const uint64_t b = mix(a ^ (((uint64_t)e.position << 32) | e.packed));
        s1 += b;
        s2 += mix(b ^ 0xD6E8FEB86659FD93ULL);
    };
    for (int i = 0; i < 5; ++i) report[i] = 0;
    report[1] = n;
    report[2] = UINT64_MAX;
    report[4] = UINT64_MAX;
    /* expected entries, per contig in parallel */
    const int nt = n_threads <= 0 ? (int)std::max(1u, std::thread::hardware_concurrency()) : n_threads;
    std::atomic<uint32_t> next{0};
    std::vector<uint64_t> cnt(nt, 0), d1(nt, 0), d2(nt, 0);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&, t]() {
            std::vector<Syncmer> sm;
            for (;;) {
                const uint32_t c = next.fetch_add(1);
                if (c >= n_contigs) break;
                uint64_t emitted = 0;
                contig_entries(*p, seqs + offsets[c], lengths[c], c, sm, [&](const gbsa_ref_randstrobe& e) {
                    digest(e, d1[t], d2[t]);
                    ++emitted;
                });
                const uint64_t ns = sm.size();
                const uint64_t slots = ns < p->w_min ? 0 : ns - p->w_min;
                /* slots the reference counts but does not assign stay zero entries */
                for (uint64_t z = emitted; z < slots; ++z) digest(gbsa_ref_randstrobe{0, 0, 0}, d1[t], d2[t]);
                cnt[t] += slots;
            }
        });
    }
    for (auto& x : th) x.join();
    uint64_t want = 0, w1 = 0, w2 = 0;
    for (int t = 0; t < nt; ++t) {
        want += cnt[t];
        w1 += d1[t];
        w2 += d2[t];
    }
    report[0] = want;
    if (want != n) return 1;
    /* order and digest of the given entries */
    uint64_t g1 = 0, g2 = 0;
    for (uint64_t i = 0; i < n; ++i) {
        if (i > 0) {
            const gbsa_ref_randstrobe& a = rs[i - 1];
            const gbsa_ref_randstrobe& b = rs[i];
            const bool le = a.hash != b.hash ? a.hash < b.hash
                                             : (a.position != b.position ? a.position < b.position : a.packed <= b.packed);
            if (!le) {
                report[2] = i;
                return 2;
            }
        }
        digest(rs[i], g1, g2);
    }
    if (g1 != w1 || g2 != w2) return 3;
    std::vector<uint64_t> st;
    uint32_t fc = 0;
    gbsa_index_info info{};
    finish_index(rs, n, bits, f, st, fc, info);
    report[3] = fc;
    for (uint64_t i = 0; i < st.size(); ++i)
        if (st[i] != starts[i]) {
            report[4] = i;
            return 4;
        }
    if (fc != filter_cutoff) return 5;
    return 0;
}

void oracle_index_free(oracle_index* idx) { delete idx; }
void oracle_index_info(const oracle_index* idx, gbsa_index_info* out) { *out = idx->idx.info; }
const gbsa_ref_randstrobe* oracle_index_randstrobes(const oracle_index* idx) { return idx->idx.rs.data(); }
const uint64_t* oracle_index_starts(const oracle_index* idx) { return idx->idx.starts.data(); }

/* index.cu:73-89 (write) with io.hpp:11-26 and indexparameters.cpp:184-192 */
int oracle_index_write_sti(const oracle_index* h, const char* path) {
    std::ofstream os(path, std::ios::binary);
    if (!os) return GBSA_ERR_INDEX_FILE;
    auto w32 = [&](int32_t v) { os.write(reinterpret_cast<const char*>(&v), 4); };
    auto w64 = [&](uint64_t v) { os.write(reinterpret_cast<const char*>(&v), 8); };
    const IndexCpu& x = h->idx;
    os.write("STI\1", 4);
    w32(2);
    w64(8);
    const char zeros[8] = {0};
    os.write(zeros, 8);
    w32((int32_t)x.filter_cutoff);
    w32(x.bits);
    w32(x.p.canonical_read_length);
    w32(x.p.k);
    w32(x.p.s);
    w32(x.p.l);
    w32(x.p.u);
    w32((int32_t)x.p.q);
    w32(x.p.max_dist);
    w64(x.rs.size());
    os.write(reinterpret_cast<const char*>(x.rs.data()), (std::streamsize)(x.rs.size() * sizeof(gbsa_ref_randstrobe)));
    w64(x.starts.size());
    os.write(reinterpret_cast<const char*>(x.starts.data()), (std::streamsize)(x.starts.size() * 8));
    return os ? GBSA_OK : GBSA_ERR_INDEX_FILE;
}

uint64_t oracle_find(const oracle_index* idx, uint64_t hash) { return idx->idx.find(hash); }
uint32_t oracle_get_count(const oracle_index* idx, uint64_t position) { return idx->idx.get_count(position); }
int oracle_is_filtered(const oracle_index* idx, uint64_t position) { return idx->idx.is_filtered(position) ? 1 : 0; }

int64_t oracle_find_nams(const oracle_index* idx, const gbsa_query_randstrobe* q, uint64_t nq, gbsa_nam* out,
                         uint64_t cap, float* frac) {
    float fr = 1.0f;
    auto v = find_nams(idx->idx, q, nq, &fr);
    if (frac) *frac = fr;
    if (v.size() > cap) return -(int64_t)v.size() - 1;
    if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(gbsa_nam));
    return (int64_t)v.size();
}

int64_t oracle_find_nams_rescue(const oracle_index* idx, const gbsa_query_randstrobe* q, uint64_t nq,
                                uint32_t rescue_cutoff, uint32_t count_cap, gbsa_nam* out, uint64_t cap) {
    auto v = find_nams_rescue(idx->idx, q, nq, rescue_cutoff, count_cap);
    if (v.size() > cap) return -(int64_t)v.size() - 1;
    if (!v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(gbsa_nam));
    return (int64_t)v.size();
}

void oracle_sort_nams(gbsa_nam* nams, uint64_t n, int sort_mode) { sort_nams(nams, n, sort_mode); }

// top_dropoff (step2/main.cu:889-898): second NAM's hits over the first's, 1 when the
// first has at most 2 hits, 0 for a single NAM; the ratio is a float division.
static float top_dropoff(const gbsa_nam* nams, uint64_t n) {
    const gbsa_nam& n_max = nams[0];
    if (n_max.n_hits <= 2) return 1.0f;
    if (n > 1) return (float)nams[1].n_hits / n_max.n_hits;
    return 0.0f;
}

// is_proper_nam_pair (step2/main.cu:870-887): same reference, opposite orientations,
// and the diagonal starts ordered with the reverse mate downstream, closer than
// mu + 10 sigma (an int difference compared with a float; the bound as one fused
// multiply-add, as nvcc compiles the reference's expression by default).
static bool is_proper_nam_pair(const gbsa_nam& a1, const gbsa_nam& a2, float mu, float sigma) {
    if (a1.ref_id != a2.ref_id || a1.is_rc == a2.is_rc) return false;
    const int a = std::max(0, a1.ref_start - a1.query_start);
    const int b = std::max(0, a2.ref_start - a2.query_start);
    const float limit = std::fma(10.0f, sigma, mu);   // nvcc contracts mu + 10 * sigma
    const bool r1_r2 = a2.is_rc && (a <= b) && ((float)(b - a) < limit);
    const bool r2_r1 = a1.is_rc && (b <= a) && ((float)(a - b) < limit);
    return r1_r2 || r2_r1;
}

// gpu_pre_cal_type (step2/main.cu:3552-3580) over the NAM lists of 2 * n_pairs ends.
int oracle_classify_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout,
                          float dropoff_threshold, float mu, float sigma, uint8_t* types) {
    for (uint32_t i = 0; i < n_pairs; ++i) {
        const uint64_t r1 = layout == GBSA_PAIRS_HALVES ? i : 2ull * i;
        const uint64_t r2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)i + n_pairs : 2ull * i + 1;
        const gbsa_nam* n1 = nams + offsets[r1];
        const gbsa_nam* n2 = nams + offsets[r2];
        const uint64_t c1 = offsets[r1 + 1] - offsets[r1], c2 = offsets[r2 + 1] - offsets[r2];
        uint8_t t;
        if (c1 == 0 && c2 == 0) t = 0;
        else if (c2 == 0) t = 1;
        else if (c1 == 0) t = 2;
        else if (top_dropoff(n1, c1) < dropoff_threshold && top_dropoff(n2, c2) < dropoff_threshold &&
                 is_proper_nam_pair(n1[0], n2[0], mu, sigma))
            t = 3;
        else t = 4;
        types[i] = t;
    }
    return 0;
}

}  // extern "C"

// ---- NAM-pair scoring (step2/main.cu:1428-1716) -------------------------------
//
// The heap keeps the TOP_K pairs of highest score: a binary min-heap on score whose
// sift-up stops at a parent of score <= the child's and whose sift-down moves to the
// smaller child (the left one on a tie) while it is strictly smaller (main.cu:1430-1473).
struct PairHeap {
    gbsa_nam_pair h[GBSA_NAM_PAIRS_TOP_K];
    int size = 0;
    void add(const gbsa_nam_pair& p) {
        if (size < GBSA_NAM_PAIRS_TOP_K) {
            int i = size++;
            h[i] = p;
            while (i > 0) {
                const int up = (i - 1) / 2;
                if (h[up].score <= h[i].score) break;
                std::swap(h[up], h[i]);
                i = up;
            }
        } else if (p.score > h[0].score) {
            h[0] = p;
            int i = 0;
            while (2 * i + 1 < size) {
                int s = i;
                const int l = 2 * i + 1, r = l + 1;
                if (l < size && h[l].score < h[s].score) s = l;
                if (r < size && h[r].score < h[s].score) s = r;
                if (s == i) break;
                std::swap(h[i], h[s]);
                i = s;
            }
        }
    }
};

static inline int nam_diag(const gbsa_nam& n) { return std::max(0, n.ref_start - n.query_start); }

// The comparator of the final sort (main.cu:1674-1713): joint score desc, then mate 1's
// NAM (score desc, forward first, query end, query start, ref end, ref start) and mate
// 2's likewise; an absent end compares as an all-zero NAM with ref_start -1.
static bool nam_pair_before(const gbsa_nam_pair& a, const gbsa_nam_pair& b, const gbsa_nam* n1, const gbsa_nam* n2) {
    gbsa_nam none{};
    none.ref_start = -1;
    const gbsa_nam& a1 = a.i1 < 0 ? none : n1[a.i1];
    const gbsa_nam& a2 = a.i2 < 0 ? none : n2[a.i2];
    const gbsa_nam& b1 = b.i1 < 0 ? none : n1[b.i1];
    const gbsa_nam& b2 = b.i2 < 0 ? none : n2[b.i2];
    if (a.score != b.score) return a.score > b.score;
    if (a1.score != b1.score) return a1.score > b1.score;
    if (a1.is_rc != b1.is_rc) return !a1.is_rc;
    if (a1.query_end != b1.query_end) return a1.query_end < b1.query_end;
    if (a1.query_start != b1.query_start) return a1.query_start < b1.query_start;
    if (a1.ref_end != b1.ref_end) return a1.ref_end < b1.ref_end;
    if (a1.ref_start != b1.ref_start) return a1.ref_start < b1.ref_start;
    if (a2.score != b2.score) return a2.score > b2.score;
    if (a2.is_rc != b2.is_rc) return !a2.is_rc;
    if (a2.query_end != b2.query_end) return a2.query_end < b2.query_end;
    if (a2.query_start != b2.query_start) return a2.query_start < b2.query_start;
    if (a2.ref_end != b2.ref_end) return a2.ref_end < b2.ref_end;
    return a2.ref_start < b2.ref_start;
}

// quick_sort_iterative (main.cu:317-358): Lomuto partition around the last element,
// ranges on an explicit stack (left part pushed before the right one).  Not stable;
// the same steps give the same order of elements that compare equal.
template <class Less>
static void quicksort_stack(gbsa_nam_pair* d, int lo, int hi, Less less) {
    if (lo > hi) return;
    std::vector<int> st;
    st.push_back(lo);
    st.push_back(hi);
    while (!st.empty()) {
        hi = st.back();
        st.pop_back();
        lo = st.back();
        st.pop_back();
        const gbsa_nam_pair pivot = d[hi];
        int i = lo - 1;
        for (int j = lo; j < hi; ++j)
            if (less(d[j], pivot)) std::swap(d[++i], d[j]);
        std::swap(d[i + 1], d[hi]);
        const int p = i + 1;
        if (p - 1 > lo) {
            st.push_back(lo);
            st.push_back(p - 1);
        }
        if (p + 1 < hi) {
            st.push_back(p + 1);
            st.push_back(hi);
        }
    }
}

// Pairs of mate-1 NAMs [b1, e1) with mate-2 NAMs [b2, e2) of opposite strands, one
// reference id at a time (ids below 3000, main.cu:1520-1570 and 1573-1623).  fwd1: mate 1
// on the forward strand (mate 2's diagonal in [d1, d1 + span)), else on the reverse
// strand (mate 2's diagonal in (d1 - span, d1]).
static void pair_pass(const gbsa_nam* n1, int b1, int e1, const gbsa_nam* n2, int b2, int e2, bool fwd1, int span,
                      PairHeap& heap, std::vector<uint8_t>& add1, std::vector<uint8_t>& add2, int& best) {
    int p1 = b1, p2 = b2;
    for (int ref = 0; ref < 3000; ++ref) {
        while (p1 < e1 && n1[p1].ref_id < ref) ++p1;
        while (p2 < e2 && n2[p2].ref_id < ref) ++p2;
        int q1 = p1, q2 = p2;
        while (q1 < e1 && n1[q1].ref_id == ref) ++q1;
        while (q2 < e2 && n2[q2].ref_id == ref) ++q2;
        if (p1 == e1 || p2 == e2) break;
        int best2 = -1;
        for (int j = p2; j < q2; ++j) best2 = std::max(best2, n2[j].n_hits);
        for (int i = p1; i < q1; ++i) {
            const int round_best = n1[i].n_hits + best2;
            if (round_best < best / 2) break;
            if (heap.size == GBSA_NAM_PAIRS_TOP_K && round_best < heap.h[0].score) break;
            const int d1 = nam_diag(n1[i]);
            // first mate-2 NAM of this reference whose diagonal enters the window
            int lo = p2, hi = q2 - 1, at = q2;
            while (lo <= hi) {
                const int mid = (lo + hi) / 2;
                const bool in = fwd1 ? nam_diag(n2[mid]) >= d1 : nam_diag(n2[mid]) > d1 - span;
                if (in) {
                    at = mid;
                    hi = mid - 1;
                } else {
                    lo = mid + 1;
                }
            }
            for (int j = at; j < q2; ++j) {
                const int d2 = nam_diag(n2[j]);
                if (fwd1 ? d2 >= d1 + span : d2 > d1) break;
                const int joint = n1[i].n_hits + n2[j].n_hits;
                if (joint < best / 2) continue;
                heap.add(gbsa_nam_pair{joint, i, j});
                add1[i] = add2[j] = 1;
                best = std::max(best, joint);
            }
        }
    }
}

extern "C" {

int oracle_nam_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout, float mu,
                     float sigma, uint32_t max_tries, gbsa_nam_pair* out, uint32_t* counts) {
    const int imu = (int)mu, isigma = (int)sigma;
    const int span = imu + 10 * isigma;
    for (uint32_t p = 0; p < n_pairs; ++p) {
        const uint64_t r1 = layout == GBSA_PAIRS_HALVES ? p : 2ull * p;
        const uint64_t r2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)p + n_pairs : 2ull * p + 1;
        const int c1 = (int)(offsets[r1 + 1] - offsets[r1]), c2 = (int)(offsets[r2 + 1] - offsets[r2]);
        counts[p] = 0;
        if (c1 == 0 || c2 == 0) continue;
        const gbsa_nam* n1 = nams + offsets[r1];
        const gbsa_nam* n2 = nams + offsets[r2];
        std::vector<uint8_t> add1((size_t)c1, 0), add2((size_t)c2, 0);
        int mid1 = c1, mid2 = c2;   // first reverse-strand NAM of each end
        for (int i = 0; i < c1; ++i)
            if (n1[i].is_rc == 1) {
                mid1 = i;
                break;
            }
        for (int i = 0; i < c2; ++i)
            if (n2[i].is_rc == 1) {
                mid2 = i;
                break;
            }
        PairHeap heap;
        int best = 0;
        pair_pass(n1, 0, mid1, n2, mid2, c2, true, span, heap, add1, add2, best);
        pair_pass(n1, mid1, c1, n2, 0, mid2, false, span, heap, add1, add2, best);
        std::vector<gbsa_nam_pair> list;
        // mate-1 NAMs in no pair: at most max_tries per (reference id, strand)
        int best1 = best;
        if (best1 == 0)
            for (int i = 0; i < c1; ++i) best1 = std::max(best1, n1[i].n_hits);
        int run = 0, prev = n1[0].ref_id + 3000 * n1[0].is_rc;
        for (int i = 0; i < c1; ++i) {
            const int key = n1[i].ref_id + 3000 * n1[i].is_rc;
            if (key == prev) ++run;
            else {
                run = 1;
                prev = key;
            }
            if (run > (int)max_tries) continue;
            if (n1[i].n_hits < best1 / 2 || add1[i]) continue;
            list.push_back(gbsa_nam_pair{n1[i].n_hits, i, -1});
        }
        // mate-2 NAMs in no pair, through the heap
        int best2 = best;
        if (best2 == 0)
            for (int i = 0; i < c2; ++i) best2 = std::max(best2, n2[i].n_hits);
        for (int i = 0; i < c2; ++i) {
            if (n2[i].n_hits < best2 / 2 || add2[i]) continue;
            heap.add(gbsa_nam_pair{n2[i].n_hits, -1, i});
        }
        for (int i = 0; i < heap.size; ++i) list.push_back(heap.h[i]);
        quicksort_stack(list.data(), 0, (int)list.size() - 1,
                        [&](const gbsa_nam_pair& a, const gbsa_nam_pair& b) { return nam_pair_before(a, b, n1, n2); });
        const uint32_t k = std::min<uint32_t>((uint32_t)list.size(), max_tries);
        for (uint32_t i = 0; i < k; ++i) out[(size_t)p * max_tries + i] = list[i];
        counts[p] = k;
    }
    return 0;
}

/* get_mapq (main.cu:900-910) in the reference's float arithmetic: min_matches a float
 * rounded from n_hits / 10.0 (a double) capped at 1, the log a float log of the float
 * score, the products float in the reference's order, truncated to int, capped at 60,
 * returned as uint8 (negative values wrap). */
static uint8_t pair_mapq(const gbsa_nam* nams, uint64_t n) {
    if (n <= 1) return 60;
    const float s1 = nams[0].score, s2 = nams[1].score;
    const double mm = nams[0].n_hits / 10.0;
    const float min_matches = (float)(mm < 1.0 ? mm : 1.0);
    volatile float f = 40.0f * (1.0f - s2 / s1);   /* volatile: no contraction or reassociation */
    f = f * min_matches;
    f = f * std::log(s1);
    const int uncapped = (int)f;
    return (uint8_t)(uncapped < 60 ? uncapped : 60);
}

/* The alignment orchestration of align_PE_part0..4 (main.cu:1857-2165) as step lists
 * (gbsa_plan_pairs_device's plans and steps).  Returns the step count (steps beyond
 * step_cap are counted, not written). */
int64_t oracle_plan_pairs(const gbsa_nam* nams, const uint64_t* offsets, uint32_t n_pairs, int layout,
                          const uint8_t* types, const gbsa_nam_pair* jp, const uint32_t* jcounts, uint32_t max_tries,
                          float dropoff, gbsa_pair_plan* plans, gbsa_align_step* steps, uint64_t step_cap) {
    uint64_t total = 0;
    for (uint32_t p = 0; p < n_pairs; ++p) {
        const uint64_t e1 = layout == GBSA_PAIRS_HALVES ? p : 2ull * p;
        const uint64_t e2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)p + n_pairs : 2ull * p + 1;
        const uint64_t c1 = offsets[e1 + 1] - offsets[e1], c2 = offsets[e2 + 1] - offsets[e2];
        const gbsa_nam* n1 = nams + offsets[e1];
        const gbsa_nam* n2 = nams + offsets[e2];
        gbsa_pair_plan plan{};
        plan.type = types[p];
        plan.first_step = (uint32_t)total;
        uint64_t k = 0;
        auto push = [&](uint8_t kind, bool is_read1, uint64_t read, uint64_t nam_read, uint32_t nam) {
            if (total + k < step_cap) {
                gbsa_align_step s{};
                s.pair = p;
                s.read = (uint32_t)read;
                s.nam_read = (uint32_t)nam_read;
                s.nam = nam;
                s.kind = kind;
                s.is_read1 = is_read1 ? 1 : 0;
                steps[total + k] = s;
            }
            ++k;
        };
        /* rescue_read_part (main.cu:795-835) */
        auto rescue_read = [&](const gbsa_nam* ns, uint64_t c, uint64_t mapped, uint64_t mate, bool mapped_is_read1) {
            const int top = ns[0].n_hits;
            uint32_t tries = 0;
            for (uint64_t i = 0; i < c; ++i) {
                const float d = (float)ns[i].n_hits / (float)top;
                if (tries >= max_tries || d < dropoff) break;
                push(GBSA_STEP_EXTEND, mapped_is_read1, mapped, mapped, (uint32_t)i);
                push(GBSA_STEP_RESCUE, !mapped_is_read1, mate, mapped, (uint32_t)i);
                ++tries;
            }
        };
        if (plan.type == 1 && c1 > 0) {
            rescue_read(n1, c1, e1, e2, true);
        } else if (plan.type == 2 && c2 > 0) {
            rescue_read(n2, c2, e2, e1, false);
        } else if (plan.type == 3 && c1 > 0 && c2 > 0) {   /* align_PE_part3 */
            push(GBSA_STEP_EXTEND, true, e1, e1, 0);
            push(GBSA_STEP_EXTEND, false, e2, e2, 0);
            plan.mapq1 = pair_mapq(n1, c1);
            plan.mapq2 = pair_mapq(n2, c2);
        } else if (plan.type == 4 && c1 > 0 && c2 > 0) {   /* align_PE_part4 */
            std::vector<uint8_t> al1(c1, 0), al2(c2, 0);
            uint32_t b1 = 0, b2 = 0;
            for (uint32_t i = 0; i < c1; ++i)
                if (n1[i].score > n1[b1].score) b1 = i;
            for (uint32_t i = 0; i < c2; ++i)
                if (n2[i].score > n2[b2].score) b2 = i;
            push(GBSA_STEP_EXTEND, true, e1, e1, b1);
            al1[b1] = 1;
            push(GBSA_STEP_EXTEND, false, e2, e2, b2);
            al2[b2] = 1;
            const uint32_t nj = jcounts[p];
            const gbsa_nam_pair* J = jp + (uint64_t)p * max_tries;
            const double max_score = nj ? (double)J[0].score : 0.0;
            uint32_t high = 0;
            for (uint32_t i = 0; i < nj; ++i) {
                const float d = (float)((float)J[i].score / max_score);
                if (high >= max_tries || d < dropoff) break;
                ++plan.type4_loop_size;
                const int i1 = J[i].i1, i2 = J[i].i2;
                if (i1 >= 0) {
                    if (!al1[i1]) {
                        push(GBSA_STEP_EXTEND, true, e1, e1, (uint32_t)i1);
                        al1[i1] = 1;
                    }
                } else {
                    push(GBSA_STEP_RESCUE, true, e1, e2, (uint32_t)i2);
                }
                if (i2 >= 0) {
                    if (!al2[i2]) {
                        push(GBSA_STEP_EXTEND, false, e2, e2, (uint32_t)i2);
                        al2[i2] = 1;
                    }
                } else {
                    push(GBSA_STEP_RESCUE, false, e2, e1, (uint32_t)i1);
                }
                ++high;
            }
        }
        plan.n_steps = (uint32_t)k;
        plans[p] = plan;
        total += k;
    }
    return (int64_t)total;
}

int oracle_map_reads(const oracle_index* h, const gbsa_map_options* opt, const char* seqs, const uint64_t* offsets,
                     const uint32_t* lengths, uint32_t n_reads, gbsa_nam* nams, uint64_t nam_capacity,
                     uint64_t* nam_offsets, float* frac, uint8_t* rescued, int n_threads) {
    std::vector<ReadResult> res(n_reads);
    const int nt = n_threads <= 0 ? (int)std::max(1u, std::thread::hardware_concurrency()) : n_threads;
    std::vector<std::vector<gbsa_query_randstrobe>> qbufs((size_t)nt);
    parallel_for(n_reads, nt, [&](uint32_t i, int t) {
        map_one(h->idx, *opt, seqs + offsets[i], lengths[i], qbufs[(size_t)t], res[i]);
    });
    uint64_t total = 0;
    for (uint32_t i = 0; i < n_reads; ++i) {
        nam_offsets[i] = total;
        total += res[i].nams.size();
    }
    nam_offsets[n_reads] = total;
    if (frac)
        for (uint32_t i = 0; i < n_reads; ++i) frac[i] = res[i].frac;
    if (rescued)
        for (uint32_t i = 0; i < n_reads; ++i) rescued[i] = res[i].rescued ? 1 : 0;
    if (total > nam_capacity) return GBSA_ERR_CAPACITY;
    for (uint32_t i = 0; i < n_reads; ++i) {
        if (!res[i].nams.empty())
            std::memcpy(nams + nam_offsets[i], res[i].nams.data(), res[i].nams.size() * sizeof(gbsa_nam));
    }
    return GBSA_OK;
}

/* Roofline numerator.  Per read: ceil(L/4) bytes of 2-bit input; per query randstrobe
 * 16 B for the bucket bound pair, 16 B per table entry the in-bucket search examines
 * (entries before the first one whose hash is >= the key, plus that one, capped at
 * the bucket size), and for a found key 16 B for the filter probe plus, when not
 * filtered, 16 B per entry of the equal-hash run; 44 B per NAM written.  Work of the
 * rescue path beyond this is not counted (the figure is a lower bound). */
int oracle_algorithmic_bytes(const oracle_index* h, const gbsa_map_options* opt, const char* seqs,
                             const uint64_t* offsets, const uint32_t* lengths, uint32_t n_reads,
                             uint64_t* bytes_out, int n_threads) {
    const IndexCpu& idx = h->idx;
    const int nt = n_threads <= 0 ? (int)std::max(1u, std::thread::hardware_concurrency()) : n_threads;
    std::vector<uint64_t> per(n_reads, 0);
    std::vector<std::vector<gbsa_query_randstrobe>> qbufs((size_t)nt);
    parallel_for(n_reads, nt, [&](uint32_t i, int t) {
        auto& q = qbufs[(size_t)t];
        uint64_t b = (lengths[i] + 3) / 4;
        randstrobes_query(idx.p, seqs + offsets[i], lengths[i], q);
        for (const auto& qr : q) {
            b += 16;
            const unsigned top = (unsigned)(qr.hash >> (64 - idx.bits));
            const uint64_t a = idx.starts[top], e = idx.starts[top + 1];
            uint64_t ex = 0;
            for (uint64_t x = a; x < e; ++x) {
                ++ex;
                if (idx.rs[x].hash >= qr.hash) break;
            }
            b += 16 * ex;
            const uint64_t pos = idx.find(qr.hash);
            if (pos == UINT64_MAX) continue;
            b += 16;
            if (idx.is_filtered(pos)) continue;
            uint64_t run = 0;
            for (uint64_t x = pos; x < idx.rs.size() && idx.rs[x].hash == qr.hash; ++x) ++run;
            b += 16 * run;
        }
        ReadResult r;
        map_one(idx, *opt, seqs + offsets[i], lengths[i], q, r);
        b += 44 * (uint64_t)r.nams.size();
        per[i] = b;
    });
    uint64_t tot = 0;
    for (auto x : per) tot += x;
    *bytes_out = tot;
    return GBSA_OK;
}

}  // extern "C"

// ---- seed extension (the first step of the alignment kernels) ------------------------

// revcomp_table (step2/main.cu:1832-1849): A/C/G/T/U in either case to the upper-case
// complement, every other byte to 'N'.
static char revcomp_char(unsigned char c) {
    switch (c) {
        case 'A': case 'a': return 'T';
        case 'C': case 'c': return 'G';
        case 'G': case 'g': return 'C';
        case 'T': case 't': case 'U': case 'u': return 'A';
        default: return 'N';
    }
}

// my_hamming_align (step2/main.cu:506-580): the best-scoring segment of an ungapped
// alignment of query and ref (equal lengths n), with the end bonus at both ends; the
// CIGAR it also builds is not kept by its caller.
struct HammingAln {
    int sw_score = 0, edit_distance = 0, ref_start = 0, ref_end = 0, query_start = 0, query_end = 0;
};
static HammingAln hamming_align(const char* query, const char* ref, int n, int match, int mismatch, int end_bonus) {
    HammingAln a;
    int start = 0, score = end_bonus, best_start = 0, best_end = 0, best_score = 0;
    for (int i = 0; i < n; ++i) {
        score += query[i] == ref[i] ? match : -mismatch;
        if (score < 0) {
            start = i + 1;
            score = 0;
        }
        if (score > best_score) {
            best_start = start;
            best_score = score;
            best_end = i + 1;
        }
    }
    if (score + end_bonus > best_score) {
        best_score = score + end_bonus;
        best_end = n;
        best_start = start;
    }
    int mismatches = 0;
    for (int i = best_start; i < best_end; ++i) mismatches += query[i] == ref[i] ? 0 : 1;
    a.sw_score = best_score;
    a.edit_distance = mismatches;
    a.ref_start = a.query_start = best_start;
    a.ref_end = a.query_end = best_end;
    return a;
}

static bool same_bytes(const char* a, const char* b, int n) { return std::memcmp(a, b, (size_t)n) == 0; }

extern "C" {

int oracle_extend_seeds(const char* ref_seqs, const uint64_t* ref_offsets, const uint64_t* ref_lengths,
                        uint32_t n_refs, const char* read_seqs, const uint64_t* read_offsets,
                        const uint32_t* read_lengths, uint32_t n_reads, const gbsa_nam* nams,
                        const uint32_t* nam_reads, uint64_t n_nams, int k, const gbsa_align_params* ap,
                        gbsa_seed_alignment* out) {
    if (k < 1) return GBSA_ERR_PARAM;
    std::string rc;
    for (uint64_t i = 0; i < n_nams; ++i) {
        gbsa_nam nam = nams[i];
        const uint32_t r = nam_reads[i];
        if (r >= n_reads || nam.ref_id < 0 || (uint32_t)nam.ref_id >= n_refs) return GBSA_ERR_PARAM;
        const int L = (int)read_lengths[r];
        const int rlen = (int)ref_lengths[nam.ref_id];
        if (nam.query_start < 0 || nam.query_end > L || nam.query_end - nam.query_start < k || nam.ref_start < 0 ||
            nam.ref_end > rlen || nam.ref_end - nam.ref_start < k)
            return GBSA_ERR_PARAM;
        const char* fwd = read_seqs + read_offsets[r];
        const char* ref = ref_seqs + ref_offsets[nam.ref_id];
        rc.resize((size_t)L);
        for (int j = 0; j < L; ++j) rc[(size_t)j] = revcomp_char((unsigned char)fwd[L - 1 - j]);
        // reverse_nam_if_needed (step2/main.cu:759-793); the checks above keep every
        // k-mer inside its sequence, so each substr is k bases long
        const char* seq = nam.is_rc ? rc.data() : fwd;
        const char* seq_rc = nam.is_rc ? fwd : rc.data();
        bool consistent = same_bytes(ref + nam.ref_start, seq + nam.query_start, k) &&
                          same_bytes(ref + nam.ref_end - k, seq + nam.query_end - k, k);
        if (!consistent) {
            const int qs2 = L - nam.query_end, qe2 = L - nam.query_start;
            if (same_bytes(ref + nam.ref_start, seq_rc + qs2, k) && same_bytes(ref + nam.ref_end - k, seq_rc + qe2 - k, k)) {
                nam.is_rc = nam.is_rc ? 0 : 1;
                nam.query_start = qs2;
                nam.query_end = qe2;
                consistent = true;
            }
        }
        // extend_seed_part (step2/main.cu:582-643)
        gbsa_seed_alignment& o = out[i];
        std::memset(&o, 0, sizeof o);
        o.ref_id = nam.ref_id;
        o.query_start = nam.query_start;
        o.query_end = nam.query_end;
        o.is_rc = nam.is_rc;
        o.consistent = consistent ? 1 : 0;
        const char* query = nam.is_rc ? rc.data() : fwd;
        const int pstart = std::max(0, nam.ref_start - nam.query_start);
        const int pend = std::min(nam.ref_end + L - nam.query_end, rlen);
        if (pend - pstart == L && consistent) {
            const char* segm = ref + pstart;
            int hd = 0;
            const int limit_error = (int)(L * 0.05);
            for (int j = 0; j < L && hd <= limit_error; ++j)
                if (query[j] != segm[j]) ++hd;
            if (hd >= 0 && ((float)hd / L) < 0.05) {
                const HammingAln a = hamming_align(query, segm, L, ap->match, ap->mismatch, ap->end_bonus);
                o.done = 1;
                o.edit_distance = a.edit_distance;
                o.global_ed = a.edit_distance + a.query_start + (L - a.query_end);
                o.score = a.sw_score;
                o.ref_start = pstart + a.ref_start;
                o.length = a.ref_end - a.ref_start;
            }
        }
    }
    return GBSA_OK;
}

}  // extern "C"

// ---- mate rescue's shared-substring test ----------------------------------------------

// nt2int_mod8 (step2/main.cu:645-654): the 2-bit code of a byte from its value mod 8
// (A/a 0, C/c 1, G/g 2, T/t 3; other bytes whatever their value mod 8 selects).
static uint32_t code_mod8(unsigned char base) {
    static const uint8_t t[8] = {0, 0, 0, 1, 3, 0, 0, 2};
    return t[base % 8];
}

// has_shared_substring (step2/main.cu:657-693): a 2k/3-base substring of the read starting
// at a multiple of k/3 equals one of the reference segment's (each hashed 2 bits per base
// into 32 bits; both loops stop one substring short of the end).
static bool shared_substring(const char* read, int read_len, const char* ref, int ref_len, int k) {
    const int sub = 2 * k / 3, step = k / 3;
    std::vector<uint32_t> h0;
    for (int i = 0; i + sub < read_len; i += step) {
        uint32_t h = 0;
        for (int j = 0; j < sub; ++j) h = (h << 2) | code_mod8((unsigned char)read[i + j]);
        h0.push_back(h);
    }
    std::sort(h0.begin(), h0.end());
    for (int i = 0; i + sub < ref_len; ++i) {
        uint32_t h = 0;
        for (int j = 0; j < sub; ++j) h = (h << 2) | code_mod8((unsigned char)ref[i + j]);
        if (std::binary_search(h0.begin(), h0.end(), h)) return true;
    }
    return false;
}

extern "C" {

int oracle_rescue_mates(const char* ref_seqs, const uint64_t* ref_offsets, const uint64_t* ref_lengths,
                        uint32_t n_refs, const char* read_seqs, const uint64_t* read_offsets,
                        const uint32_t* read_lengths, uint32_t n_reads, const gbsa_nam* nams,
                        const uint32_t* mate_reads, uint64_t n_nams, int k, float mu, float sigma,
                        gbsa_mate_rescue* out) {
    if (k < 3 || k > 32) return GBSA_ERR_PARAM;
    std::string rc;
    const float spread = std::fmaf(5.0f, sigma, mu);   // mu + 5 * sigma, as one fused multiply-add
    for (uint64_t i = 0; i < n_nams; ++i) {
        const gbsa_nam& nam = nams[i];
        const uint32_t r = mate_reads[i];
        if (r >= n_reads || nam.ref_id < 0 || (uint32_t)nam.ref_id >= n_refs) return GBSA_ERR_PARAM;
        const int L = (int)read_lengths[r];
        const int sub = 2 * k / 3, step = k / 3;
        if (L > sub && (L - sub + step - 1) / step > 64) return GBSA_ERR_PARAM;
        const char* fwd = read_seqs + read_offsets[r];
        // rescue_mate_part (step2/main.cu:695-757): the mate in the orientation opposite to
        // the NAM, and its window (float arithmetic as the reference's)
        int a, b;
        const char* mate;
        if (nam.is_rc) {
            mate = fwd;
            a = (int)((float)(nam.ref_start - nam.query_start) - spread);
            b = nam.ref_start - nam.query_start + L / 2;
        } else {
            rc.resize((size_t)L);
            for (int j = 0; j < L; ++j) rc[(size_t)j] = revcomp_char((unsigned char)fwd[L - 1 - j]);
            mate = rc.data();
            a = nam.ref_end + (L - nam.query_end) - L / 2;
            b = (int)((float)(nam.ref_end + (L - nam.query_end)) + spread);
        }
        const int ref_len = (int)ref_lengths[nam.ref_id];
        const int ws = std::max(0, std::min(a, ref_len));
        const int we = std::min(ref_len, std::max(0, b));
        gbsa_mate_rescue& o = out[i];
        std::memset(&o, 0, sizeof o);
        o.ref_id = nam.ref_id;
        o.window_start = ws;
        o.window_end = we;
        o.is_rc = nam.is_rc;
        const bool unaligned = we < ws + k || !shared_substring(mate, L, ref_seqs + ref_offsets[nam.ref_id] + ws,
                                                                we - ws, k);
        if (unaligned) {
            o.done = 1;
            o.is_unaligned = 1;
            o.edit_distance = L;
        }
    }
    return GBSA_OK;
}

}  // extern "C"
