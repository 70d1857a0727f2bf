// seed.cuh — warp-cooperative canonical syncmers and randstrobes.
//
// Restates, for a warp of 32 lanes, the reference's per-base syncmer state machine
// (SyncmerIterator::next, step2/randstrobes.cu:18-79) and randstrobe selection
// (RandstrobeIterator::get, step2/randstrobes.cu:136-159; query driver
// randstrobes_query, step2/randstrobes.cu:195-241).
//
// Syncmer rule.  Window w is the k-mer starting at base w; it holds the W = k-s+1
// s-mers w .. w+W-1.  The reference keeps (min value, min position m) over a queue
// of s-mer hashes:
//   first window after a reset:  m = leftmost minimum (forward scan, strict <)
//   minimum popped (m == w-1):   m = rightmost minimum of the window (reverse scan)
//   newest s-mer strictly below: m = w+W-1
//   otherwise:                   m unchanged
// and emits a syncmer when m == w+t-1.  m is always *an* argmin of the window, so
// whenever the window's minimum is unique m is that argmin, whatever came before.
// The warp therefore decides all windows with a unique minimum in parallel (one
// lane per window) and replays the exact state machine, over 32 windows at a time
// with warp shuffles, only for chunks that contain a window with a tied minimum
// (low-complexity sequence) — the replay needs just each window's leftmost and
// rightmost argmin, computed in parallel.  A window whose values are all UINT64_MAX
// is handled like the reference (state "none").
#pragma once

#include "common.cuh"

namespace gbsa {

// Per-window facts needed by the replay, packed in a u32:
//   bit 0 valid, bit 1 first, bit 2 all-max, bits 8..15 leftmost argmin offset,
//   bits 16..23 rightmost argmin offset.
struct WinInfo {
    static __device__ __forceinline__ uint32_t pack(bool valid, bool first, bool allmax, uint32_t lo, uint32_t ro) {
        return (valid ? 1u : 0u) | (first ? 2u : 0u) | (allmax ? 4u : 0u) | (lo << 8) | (ro << 16);
    }
};

// 2-bit packing of ASCII bases into MSB-first 64-bit words plus an N bitmask
// (LSB-first 32-bit words; bases at or beyond L count as N).  Writes
// nwords = ceil(L/32) + 2 words to each array.  Each lane codes 4 consecutive bases
// per round of 128; 8 lanes then make a word with three xor-shuffles.
// Returns whether the read holds an N (any base that is not A/C/G/T/U).
//
// A lane reads its 4 bases as one 32-bit word (two aligned loads and a funnel shift
// when the read starts off a 4-byte boundary; only words that hold a base of the
// read are loaded) and codes them at once: ((b >> 1) ^ (b >> 2)) & 3 is the 2-bit
// code of A, C, G and T in either case, and a byte permute of "ACGT" by those codes
// gives back the upper-case bases, so a word holding only A/C/G/T (either case)
// is recognised with one compare.  Any other word (U, N, raw codes 0-3, other
// bytes) takes the per-base path of nt4.
__device__ __forceinline__ bool warp_pack_read(const uint8_t* seq, uint32_t L, uint64_t* packed, uint32_t* nmask) {
    const uint32_t lane = lane_id();
    const uint32_t nw = (L + 31) / 32 + 2;
    const uint32_t sub = lane & 7;   // position of the lane's 4 bases within the word
    const uintptr_t a0 = reinterpret_cast<uintptr_t>(seq);
    const uint32_t mis = (uint32_t)(a0 & 3);
    const uint32_t* words = reinterpret_cast<const uint32_t*>(a0 - mis);
    bool has_n = false;
    for (uint32_t b0 = 0; b0 < nw * 32; b0 += 128) {
        const uint32_t p0 = b0 + 4 * lane;   // the lane's first base
        uint32_t code8 = 0, nbits = 0xFu;
        if (p0 < L) {
            const uint32_t wi = (p0 + mis) >> 2;   // aligned word holding base p0
            const uint32_t lo = words[wi];
            const uint32_t hi = (mis != 0 && (wi + 1) * 4 - mis < L) ? words[wi + 1] : 0u;
            const uint32_t w = __funnelshift_r(lo, hi, 8 * mis);   // base p0 in the low byte
            const uint32_t c4 = ((w >> 1) ^ (w >> 2)) & 0x03030303u;
            const uint32_t sel = (c4 & 3u) | ((c4 >> 4) & 0x30u) | ((c4 >> 8) & 0x300u) | ((c4 >> 12) & 0x3000u);
            const uint32_t nv = min(L - p0, 4u);   // bases of the read among the 4
            const uint32_t vmask = nv == 4 ? 0xFFFFFFFFu : (1u << (8 * nv)) - 1;
            if ((((w & 0xDFDFDFDFu) ^ __byte_perm(0x54474341u, 0u, sel)) & vmask) == 0) {
                code8 = ((sel & 3u) << 6) | (((sel >> 4) & 3u) << 4) | (((sel >> 8) & 3u) << 2) | ((sel >> 12) & 3u);
                code8 &= (0xFF00u >> (2 * nv)) & 0xFFu;   // bases beyond the read pack as 0
                nbits = 0xFu & ~((1u << nv) - 1);
            } else {
                nbits = 0;
#pragma unroll
                for (uint32_t u = 0; u < 4; ++u) {
                    const uint32_t p = p0 + u;
                    const uint32_t c = p < L ? nt4(seq[p]) : 4u;
                    code8 = (code8 << 2) | (c & 3u);   // an N packs as 0
                    nbits |= (c == 4u ? 1u : 0u) << u;
                }
            }
        }
        uint64_t v = (uint64_t)code8 << (8 * (7 - sub));
        uint32_t nm = nbits << (4 * sub);
#pragma unroll
        for (int x = 1; x < 8; x <<= 1) {
            v |= __shfl_xor_sync(0xFFFFFFFFu, v, x);
            nm |= __shfl_xor_sync(0xFFFFFFFFu, nm, x);
        }
        const uint32_t wi = b0 / 32 + lane / 8;
        if (sub == 0 && wi < nw) {
            packed[wi] = v;
            nmask[wi] = nm;
            const uint32_t b = wi * 32;   // N bits of bases inside the read
            const uint32_t in = b >= L ? 0u : (L - b >= 32 ? 0xFFFFFFFFu : (1u << (L - b)) - 1);
            has_n |= (nm & in) != 0;
        }
    }
    __syncwarp();
    return __any_sync(0xFFFFFFFFu, has_n);
}

// n (<= 33) bits of an LSB-first u32 bitmask stream starting at bit p (two words
// always cover them: the shift within the first word is at most 31).
__device__ __forceinline__ uint64_t nbits33(const uint32_t* m, uint64_t p, int n) {
    const uint64_t wi = p >> 5;
    const uint32_t sh = (uint32_t)(p & 31);
    const uint64_t v = (((uint64_t)m[wi + 1] << 32) | m[wi]) >> sh;
    return v & ((1ULL << n) - 1);
}

__device__ __forceinline__ uint64_t smer_hash(const DevParams& P, const uint64_t* packed, uint64_t p) {
    if (P.s <= 16) {
        // s-mers of up to 16 bases in 32 bits: the stream seen as 32-bit groups of 16
        // bases (group g is the high half of word g/2 for even g, the low half for odd
        // g; little-endian halves sit at u32 index g ^ 1)
        const uint32_t* w32 = reinterpret_cast<const uint32_t*>(packed);
        const uint64_t g = p >> 4;
        const uint32_t sh = (uint32_t)(p & 15) * 2;
        const uint32_t hi = w32[g ^ 1], lo = w32[(g + 1) ^ 1];
        uint32_t f = __funnelshift_l(lo, hi, sh);
        f >>= 32 - 2 * P.s;   // P.s >= 1
        uint32_t r = __brev(~f);
        r = ((r >> 1) & 0x55555555u) | ((r & 0x55555555u) << 1);
        r >>= 32 - 2 * P.s;
        return xxh64((uint64_t)(f < r ? f : r));
    }
    const uint64_t f = extract_bases(packed, p, P.s);
    const uint64_t r = revcomp_bits(f, P.s);
    return xxh64(f < r ? f : r);
}

__device__ __forceinline__ uint64_t kmer_hash(const DevParams& P, const uint64_t* packed, uint64_t p) {
    const uint64_t f = extract_bases(packed, p, P.k);
    const uint64_t r = revcomp_bits(f, P.k);
    return xxh64(f < r ? f : r);
}

// Facts of window w of a sequence whose base 0 sits at stream position `base`
// (valid when w < nwin and the k-mer holds no N).  hw is a 64-entry ring holding the
// s-mer hash of position p at hw[p & 63].  The minimum is found on the high 32 bits
// of the hashes; a unique high-word minimum is the unique minimum, and only windows
// with a high-word tie (or an all-ones high word) compare the full 64-bit values.
// kW: s-mers per window when known at compile time (0: P.W).  kClean: the sequence
// holds no N, so every window below nwin is valid and only window 0 starts a run.
template <int kW = 0, bool kClean = false>
__device__ __forceinline__ uint32_t window_info(const DevParams& P, const uint32_t* nmask, uint64_t base, uint32_t w,
                                                uint32_t nwin, const uint64_t* hw) {
    if (w >= nwin) return 0;
    bool first;
    if (kClean) {
        first = w == 0;
    } else {
        // the k-mer's N bits and, for w > 0, the base before it (N before: a new run)
        const uint32_t s1 = w > 0 ? 1u : 0u;
        const uint64_t nb = nbits33(nmask, base + w - s1, P.k + (int)s1);
        if ((nb >> s1) != 0) return 0;
        first = s1 == 0 || (nb & 1u);
    }
    const int W = kW ? kW : P.W;
    const uint32_t* h32 = reinterpret_cast<const uint32_t*>(hw);
    uint32_t mh = h32[2 * (w & 63) + 1];
    uint32_t eq = 1;
#pragma unroll 8
    for (int d = 1; d < W; ++d) {
        const uint32_t v = h32[2 * ((w + d) & 63) + 1];
        eq = v < mh ? 1u << d : (v == mh ? eq | 1u << d : eq);
        mh = v < mh ? v : mh;
    }
    uint32_t lo, ro;
    bool allmax = false;
    if ((eq & (eq - 1)) == 0 && mh != 0xFFFFFFFFu) {
        lo = ro = (uint32_t)(__ffs(eq) - 1);
    } else {
        uint64_t mv = hw[w & 63];
        lo = ro = 0;
        for (int d = 1; d < W; ++d) {
            const uint64_t v = hw[(w + d) & 63];
            if (v < mv) {
                mv = v;
                lo = ro = (uint32_t)d;
            } else if (v == mv) {
                ro = (uint32_t)d;
            }
        }
        allmax = mv == ~0ULL;
    }
    return WinInfo::pack(true, first, allmax, lo, ro);
}

// A window's state is "determined" (independent of the past) when it is the first
// of a run of valid windows or its minimum is unique (and not UINT64_MAX).
__device__ __forceinline__ bool win_determined(uint32_t inf) {
    const bool first = inf & 2u, allmax = inf & 4u;
    const uint32_t lo = (inf >> 8) & 0xFF, ro = (inf >> 16) & 0xFF;
    return first || (lo == ro && !allmax);
}

// One step of the reference state machine for valid window w with facts inf,
// entering with state m (position of the current minimum, or none).
__device__ __forceinline__ uint32_t win_step(uint32_t m, uint32_t inf, uint32_t w) {
    const bool first = inf & 2u, allmax = inf & 4u;
    const uint32_t lo = (inf >> 8) & 0xFF, ro = (inf >> 16) & 0xFF;
    if (first) return allmax ? kNoneState : w + lo;       // forward scan, leftmost minimum
    if (lo == ro && !allmax) return w + lo;                // unique minimum: any path lands on it
    if (m != kNoneState && m == w - 1) return w + ro;      // popped: reverse scan, rightmost minimum
    return m;                                              // tie, not popped: the older minimum stays
}

// Processes windows [w_begin, w_end) of one sequence (base 0 at stream position
// `base` of packed/nmask, any address space; nwin windows in total) and calls
// emit(index, window) for every syncmer with window >= w_emit, in order, index
// counting from 0.  Window w_begin must be determined, invalid, or window 0, so
// that the state entering it never matters.  hbuf: 64 u64 of warp-private
// scratch.  Returns the number of syncmers emitted.
template <int kW = 0, bool kClean = false, class Emit>
__device__ uint32_t warp_syncmer_scan(const DevParams& P, const uint64_t* packed, const uint32_t* nmask, uint64_t base,
                                      uint32_t nwin, uint32_t w_begin, uint32_t w_end, uint32_t w_emit, uint64_t* hbuf,
                                      Emit&& emit) {
    const uint32_t lane = lane_id();
    uint32_t count = 0;
    uint32_t carry = kNoneState;
    const uint32_t tpos = (uint32_t)(P.t - 1);
    const uint32_t W1 = (uint32_t)(P.W - 1);
    // s-mer hashes live in a 64-entry ring (position p at hbuf[p & 63]); each chunk of
    // 32 windows needs 32 new ones beyond the W-1 it shares with the previous chunk
    if (lane < W1 && w_begin < w_end) hbuf[(w_begin + lane) & 63] = smer_hash(P, packed, base + w_begin + lane);
    for (uint32_t c = w_begin; c < w_end; c += 32) {
        const uint32_t w = c + lane;
        hbuf[(c + W1 + lane) & 63] = smer_hash(P, packed, base + c + W1 + lane);
        __syncwarp();
        const uint32_t inf = (w < w_end) ? window_info<kW, kClean>(P, nmask, base, w, nwin, hbuf) : 0u;
        const bool valid = inf & 1u;
        const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
        const uint32_t umask = __ballot_sync(0xFFFFFFFFu, valid && !win_determined(inf));
        bool sync;
        if (umask == 0) {
            const uint32_t m = valid ? win_step(kNoneState, inf, w) : kNoneState;
            sync = valid && m != kNoneState && m == w + tpos;
            if (vmask) carry = __shfl_sync(0xFFFFFFFFu, m, 31 - __clz(vmask));
        } else {
            // exact replay of the reference state machine over this chunk
            uint32_t m = carry;
            uint32_t bits = 0;
            for (int j = 0; j < 32; ++j) {
                const uint32_t ij = __shfl_sync(0xFFFFFFFFu, inf, j);
                if (ij & 1u) {
                    const uint32_t wj = c + (uint32_t)j;
                    m = win_step(m, ij, wj);
                    if (m != kNoneState && m == wj + tpos) bits |= 1u << j;
                }
            }
            sync = (bits >> lane) & 1u;
            carry = m;
        }
        const bool out = sync && w >= w_emit;
        const uint32_t smask = __ballot_sync(0xFFFFFFFFu, out);
        if (out) emit(count + __popc(smask & lanemask_lt()), w);
        count += __popc(smask);
        __syncwarp();
    }
    return count;
}

// Largest window d <= w0 from which a scan can start without knowing the past:
// window 0, an invalid window, or a determined one (for segments of long contigs).
__device__ inline uint32_t warp_find_anchor(const DevParams& P, const uint64_t* packed, const uint32_t* nmask, uint64_t base,
                                     uint32_t nwin, uint32_t w0, uint64_t* hbuf) {
    const uint32_t lane = lane_id();
    uint32_t top = w0;   // examine windows (top-31 .. top]
    for (;;) {
        const uint32_t lo_w = top >= 31 ? top - 31 : 0;
        const uint32_t w = lo_w + lane;
        hbuf[w & 63] = smer_hash(P, packed, base + w);
        if (lane < (uint32_t)(P.W - 1)) hbuf[(lo_w + 32 + lane) & 63] = smer_hash(P, packed, base + lo_w + 32 + lane);
        __syncwarp();
        bool ok = false;
        if (w <= top) {
            const uint32_t inf = window_info(P, nmask, base, w, nwin, hbuf);
            ok = !(inf & 1u) || win_determined(inf) || w == 0;
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
        __syncwarp();
        if (m) return lo_w + (31 - __clz(m));
        if (lo_w == 0) return 0;
        top = lo_w - 1;
    }
}

// Forward randstrobe with strobe 1 = syncmer j of n (RandstrobeIterator::get): the
// candidate with the smallest popcount((h1 ^ h2) & q), the first one on ties.  When
// q fits in 32 bits only the hashes' low words are compared.
__device__ __forceinline__ void randstrobe_fwd(const DevParams& P, const uint64_t* sh, const uint32_t* sp, uint32_t n,
                                               uint32_t j, uint64_t& hash, uint32_t& s1, uint32_t& s2) {
    const uint32_t w_end = min(j + P.w_max, n - 1);
    const uint64_t h1 = sh[j];
    const uint32_t p1 = sp[j];
    const uint64_t max_pos = (uint64_t)p1 + P.max_dist;
    uint32_t bi = j;
    uint32_t best = 0xFFFFFFFFu;
    if ((P.q >> 32) == 0) {
        const uint32_t* shl = reinterpret_cast<const uint32_t*>(sh);
        const uint32_t q32 = (uint32_t)P.q, h1l = (uint32_t)h1;
        for (uint32_t i = j + P.w_min; i <= w_end && sp[i] <= max_pos; ++i) {
            const uint32_t sc = __popc((h1l ^ shl[2 * i]) & q32);
            if (sc < best) {
                best = sc;
                bi = i;
            }
        }
    } else {
        for (uint32_t i = j + P.w_min; i <= w_end && sp[i] <= max_pos; ++i) {
            const uint32_t sc = __popcll((h1 ^ sh[i]) & P.q);
            if (sc < best) {
                best = sc;
                bi = i;
            }
        }
    }
    hash = h1 + sh[bi];
    s1 = p1;
    s2 = sp[bi];
}

// Reverse-complement randstrobe number jr of n: the reference reverses the syncmer
// vector and maps positions to L - pos - k (step2/randstrobes.cu:221-224), then
// runs the same selection.
__device__ __forceinline__ void randstrobe_rev(const DevParams& P, const uint64_t* sh, const uint32_t* sp, uint32_t n,
                                               uint32_t L, uint32_t jr, uint64_t& hash, uint32_t& s1, uint32_t& s2) {
    const uint32_t k = (uint32_t)P.k;
    const uint32_t w_end = min(jr + P.w_max, n - 1);
    const uint32_t i1 = n - 1 - jr;
    const uint64_t h1 = sh[i1];
    const uint32_t p1 = L - sp[i1] - k;
    const uint64_t max_pos = (uint64_t)p1 + P.max_dist;
    uint32_t bi = i1;
    uint32_t best = 0xFFFFFFFFu;
    if ((P.q >> 32) == 0) {
        const uint32_t* shl = reinterpret_cast<const uint32_t*>(sh);
        const uint32_t q32 = (uint32_t)P.q, h1l = (uint32_t)h1;
        for (uint32_t x = jr + P.w_min; x <= w_end; ++x) {
            const uint32_t ix = n - 1 - x;
            if (L - sp[ix] - k > max_pos) break;
            const uint32_t sc = __popc((h1l ^ shl[2 * ix]) & q32);
            if (sc < best) {
                best = sc;
                bi = ix;
            }
        }
    } else {
        for (uint32_t x = jr + P.w_min; x <= w_end; ++x) {
            const uint32_t ix = n - 1 - x;
            if (L - sp[ix] - k > max_pos) break;
            const uint32_t sc = __popcll((h1 ^ sh[ix]) & P.q);
            if (sc < best) {
                best = sc;
                bi = ix;
            }
        }
    }
    hash = h1 + sh[bi];
    s1 = p1;
    s2 = L - sp[bi] - k;
}

// Internal compact query randstrobe: is_reverse is implied by the index (the
// forward ones of a read come first, as in randstrobes_query).
struct Query {
    uint64_t hash;
    uint32_t start;
    uint32_t end;
};

// Seeds one read with the warp: packs it into pk/nm (capacity for L bases), finds
// its syncmers into sh/sp (capacity cap) and returns the syncmer count, or
// 0xFFFFFFFF when more than cap syncmers exist.
__device__ __forceinline__ uint32_t warp_read_syncmers(const DevParams& P, const uint8_t* seq, uint32_t L, uint64_t* pk,
                                                       uint32_t* nm, uint64_t* hbuf, uint64_t* sh, uint32_t* sp,
                                                       uint32_t cap) {
    if (L < (uint32_t)P.k) return 0;
    const bool has_n = warp_pack_read(seq, L, pk, nm);
    const uint32_t nwin = L - (uint32_t)P.k + 1;
    auto emit = [&](uint32_t idx, uint32_t w) {
        if (idx < cap) sp[idx] = w;
    };
    // reads without N (nearly all) skip the per-window N checks; the common window
    // width (5 s-mers: k - s = 4) is unrolled at compile time
    uint32_t n;
    if (has_n) n = warp_syncmer_scan(P, pk, nm, 0, nwin, 0, nwin, 0, hbuf, emit);
    else if (P.W == 5) n = warp_syncmer_scan<5, true>(P, pk, nm, 0, nwin, 0, nwin, 0, hbuf, emit);
    else n = warp_syncmer_scan<0, true>(P, pk, nm, 0, nwin, 0, nwin, 0, hbuf, emit);
    if (n > cap) return 0xFFFFFFFFu;
    __syncwarp();
    for (uint32_t i = lane_id(); i < n; i += 32) sh[i] = kmer_hash(P, pk, sp[i]);
    __syncwarp();
    return n;
}

// Number of query randstrobes per orientation for n syncmers of a read of length L
// (randstrobes_query returns none when L < w_max, step2/randstrobes.cu:197).
__device__ __forceinline__ uint32_t n_query_per_dir(const DevParams& P, uint32_t n, uint32_t L) {
    if (L < P.w_max) return 0;
    return n > P.w_min ? n - P.w_min : 0;
}

// Writes the 2*nq query randstrobes of a read (forward, then reverse complement).
// The two orientations take passes of their own: a pass that mixed them would run
// both selection loops one after the other.
__device__ __forceinline__ void warp_write_queries(const DevParams& P, const uint64_t* sh, const uint32_t* sp,
                                                   uint32_t n, uint32_t L, uint32_t nq, Query* out) {
    const uint32_t lane = lane_id();
    for (uint32_t j = lane; j < nq; j += 32) {
        uint64_t h;
        uint32_t s1, s2;
        randstrobe_fwd(P, sh, sp, n, j, h, s1, s2);
        out[j] = Query{h, s1, s2 + (uint32_t)P.k};
    }
    for (uint32_t j = lane; j < nq; j += 32) {
        uint64_t h;
        uint32_t s1, s2;
        randstrobe_rev(P, sh, sp, n, L, j, h, s1, s2);
        out[nq + j] = Query{h, s1, s2 + (uint32_t)P.k};
    }
}

}  // namespace gbsa
