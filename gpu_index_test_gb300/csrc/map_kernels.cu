// map_kernels.cu — kernels of the read → NAM path (plain form: one kernel per stage,
// a warp per read, intermediates in HBM arenas).
//
//   k_seed_smem / k_seed_long   randstrobes_query (step2/randstrobes.cu:195-241)
//   k_lookup                    the query loop of find_nams (step2/nam.cu:748-790):
//                               find, is_filtered, add_to_hits_per_ref; the rescue
//                               decision of step2/main.cu:3209-3216
//   k_nams                      merge_hits_into_nams_forward_and_reverse(sort=true)
//                               (step2/nam.cu:515-539, 347-513) + NAM sort
//   k_rescue                    find_nams_rescue (step2/nam.cu:927-985) + NAM sort
#include <algorithm>
#include <mutex>
#include <vector>

#include <cooperative_groups.h>

#include "map.cuh"
#include "runtime.h"

namespace gbsa {

namespace {

constexpr int kSeedWarps = 8;
constexpr int kWarpsPerBlock = 8;

__device__ __forceinline__ uint32_t warp_global_id() { return (blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ uint32_t warp_count() { return (gridDim.x * blockDim.x) >> 5; }

__device__ __forceinline__ uint64_t warp_bump(unsigned long long* ctr, uint64_t n) {
    uint64_t off = 0;
    if (lane_id() == 0) off = atomicAdd(ctr, (unsigned long long)n);
    return __shfl_sync(0xFFFFFFFFu, off, 0);
}

// The next read for the calling warp from a device work counter: warps pull reads one
// at a time, so reads of uneven cost (lengths, repeats) balance over a grid of resident
// warps instead of each warp owning a fixed stride of them.
__device__ __forceinline__ uint32_t warp_next(unsigned int* head) {
    uint32_t r = 0;
    if (lane_id() == 0) r = atomicAdd(head, 1u);
    return __shfl_sync(0xFFFFFFFFu, r, 0);
}

__device__ __forceinline__ void warp_fail(ReadRec& rec, Counters* ctr, uint32_t bit) {
    if (lane_id() == 0) {
        rec.flags |= kReadFailed;
        atomicOr(&ctr->status, bit);
    }
}

// Writes the query randstrobes of read r from its syncmers.
__device__ __forceinline__ void emit_read_queries(const DevParams& P, const uint64_t* sh, const uint32_t* sp,
                                                  uint32_t ns, uint32_t L, ReadRec& rec, const Arenas& A,
                                                  Counters* ctr) {
    const uint32_t nq = n_query_per_dir(P, ns, L);
    const uint64_t off = warp_bump(&ctr->q_used, 2ull * nq);
    if (off + 2ull * nq > A.q_cap) {
        warp_fail(rec, ctr, kStatusQueryOverflow);
        if (lane_id() == 0) rec.nq = rec.nq2 = 0;
        return;
    }
    warp_write_queries(P, sh, sp, ns, L, nq, A.q + off);
    if (lane_id() == 0) {
        rec.q_off = off;
        rec.nq = nq;
        rec.nq2 = 2 * nq;
    }
}

__global__ void __launch_bounds__(32 * kSeedWarps, 5) k_seed_smem(DevParams P, const uint8_t* __restrict__ seqs,
                                                                const uint64_t* __restrict__ offs,
                                                                const uint32_t* __restrict__ lens, uint32_t n,
                                                                ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    __shared__ uint64_t s_pk[kSeedWarps][kSmemMaxLen / 32 + 4];
    __shared__ uint32_t s_nm[kSeedWarps][kSmemMaxLen / 32 + 4];
    __shared__ uint64_t s_hb[kSeedWarps][64];
    __shared__ uint64_t s_sh[kSeedWarps][kSmemSyncmers];
    __shared__ uint32_t s_sp[kSeedWarps][kSmemSyncmers];
    const uint32_t w = threadIdx.x >> 5;
    for (uint32_t r = warp_next(&ctr->queue_head); r < n; r = warp_next(&ctr->queue_head)) {
        const uint32_t L = lens[r];
        ReadRec& R = rec[r];
        if (L > GBSA_MAX_READ_LEN) {
            warp_fail(R, ctr, kStatusReadTooLong);
            continue;
        }
        uint32_t ns = 0xFFFFFFFFu;
        if (L <= kSmemMaxLen)
            ns = warp_read_syncmers(P, seqs + offs[r], L, s_pk[w], s_nm[w], s_hb[w], s_sh[w], s_sp[w], kSmemSyncmers);
        if (ns == 0xFFFFFFFFu) {
            if (lane_id() == 0) {
                R.flags |= kReadLong;
                A.long_list[atomicAdd(&ctr->n_long, 1u)] = r;
            }
            continue;
        }
        emit_read_queries(P, s_sh[w], s_sp[w], ns, L, R, A, ctr);
        __syncwarp();
    }
}

// Reads that did not fit the shared-memory buffers: same code on a per-warp slot of
// global scratch memory sized for GBSA_MAX_READ_LEN.
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_seed_long(DevParams P, const uint8_t* __restrict__ seqs,
                                                                    const uint64_t* __restrict__ offs,
                                                                    const uint32_t* __restrict__ lens,
                                                                    ReadRec* __restrict__ rec, Arenas A, Counters* ctr,
                                                                    uint8_t* scratch, const BatchDesc* desc) {
    if (desc) {
        seqs = desc->seqs;
        offs = desc->offs;
        lens = desc->lens;
    }
    const uint32_t n_long = *(volatile unsigned int*)&ctr->n_long;
    uint8_t* slot = scratch + (size_t)warp_global_id() * kLongSlotBytes;
    uint64_t* pk = reinterpret_cast<uint64_t*>(slot);
    uint32_t* nm = reinterpret_cast<uint32_t*>(pk + kLongWords);
    uint64_t* hb = reinterpret_cast<uint64_t*>(nm + kLongWords);
    uint64_t* sh = hb + 64;
    uint32_t* sp = reinterpret_cast<uint32_t*>(sh + GBSA_MAX_READ_LEN);
    for (uint32_t t = warp_global_id(); t < n_long; t += warp_count()) {
        const uint32_t r = A.long_list[t];
        const uint32_t L = lens[r];
        ReadRec& R = rec[r];
        const uint32_t ns = warp_read_syncmers(P, seqs + offs[r], L, pk, nm, hb, sh, sp, GBSA_MAX_READ_LEN);
        if (ns == 0xFFFFFFFFu) {
            warp_fail(R, ctr, kStatusSyncmerOverflow);
            continue;
        }
        emit_read_queries(P, sh, sp, ns, L, R, A, ctr);
        __syncwarp();
    }
}

// Distinct 32 B sectors of [lo, hi) bytes.
__device__ __forceinline__ uint64_t sector_span(uintptr_t lo, uintptr_t hi) {
    return hi > lo ? ((hi - 1) >> 5) - (lo >> 5) + 1 : 0;
}

// Sector form of one query's gathers as the reference performs them: the bucket
// bound pair, the entries examined in the bucket, and for a found key the filter
// probe and the run walk up to the first entry of another hash (entries the search
// already touched count once).
__device__ __forceinline__ uint64_t lookup_sectors(const IndexView& I, uint64_t key, uint32_t ex, uint64_t pos,
                                                   uint32_t run) {
    const uint64_t top = key >> (64 - I.bits);
    const uintptr_t sb = I.starts32 ? reinterpret_cast<uintptr_t>(I.starts32 + top)
                                    : reinterpret_cast<uintptr_t>(I.starts + top);
    uint64_t n = sector_span(sb, sb + (I.starts32 ? 8 : 16));
    const uint64_t a = bucket_start(I, top);
    uint64_t end = a + ex;   // entries [a, end) touched
    if (pos != kNotFound) {
        const uint64_t walk_end = pos + run + 1 < I.n ? pos + run + 1 : I.n;
        end = walk_end > end ? walk_end : end;
        const uint64_t probe = pos + I.filter_cutoff;
        if (probe < I.n && (probe < a || probe >= end))
            n += sector_span(reinterpret_cast<uintptr_t>(I.rs + probe), reinterpret_cast<uintptr_t>(I.rs + probe + 1));
    }
    n += sector_span(reinterpret_cast<uintptr_t>(I.rs + a), reinterpret_cast<uintptr_t>(I.rs + end));
    return n;
}

constexpr uint32_t kRescueHeavyHits = 2000;   // estimated merge hits of a heavy rescued read

// kCount: also count the reference's algorithmic bytes and gather sectors (a
// separate instance, so that the counting code costs the mapping kernel nothing).
// find / is_filtered / walk for the queries of read r (warp): per-query index
// positions and hit counts, the nonrepetitive fraction and rescue decision, and for a
// read that is not rescued its hits (query order, then run order) in the hit arena.
// The query loop of find_nams (step2/nam.cu:748-790).
template <bool kCount>
__device__ __forceinline__ void lookup_read(const IndexView& I, const MapConfig& C, uint32_t r, ReadRec* __restrict__ rec,
                                            const Arenas& A, Counters* ctr) {
    const uint32_t lane = lane_id();
    ReadRec& R = rec[r];
    if (R.flags & kReadFailed) return;
    const uint32_t nq = R.nq, nq2 = R.nq2;
    Query* Q = A.q + R.q_off;
    uint32_t* aux = A.q_aux + R.q_off;
    uint32_t tot = 0, good = 0;
    uint64_t bytes = 0, sectors = 0;
    for (uint32_t i = lane; i < nq2; i += 32) {
        const Query q = Q[i];
        uint32_t ex = 0;
        uint64_t bend = 0;
        const uint64_t pos = index_find(I, q.hash, &ex, &bend);
        uint32_t nh = 0, run = 0;
        bytes += 16 + 16ull * ex;
        if (pos != kNotFound) {
            ++tot;
            bytes += 16;   // the reference reads hash[pos + filter_cutoff]
            if (!index_is_filtered_in(I, pos, q.hash, bend)) {
                ++good;
                nh = walk_hit_run(I, (int)q.start, (int)q.end, pos, [&](uint32_t, int, int) {}, &run);
                bytes += 16ull * run;
            }
        }
        if (kCount) sectors += lookup_sectors(I, q.hash, ex, pos, run);
        A.q_pos[R.q_off + i] = pos;
        aux[i] = nh;
    }
    tot = warp_sum(tot);
    good = warp_sum(good);
    if (kCount) {
        bytes = warp_sum(bytes);
        sectors = warp_sum(sectors);
        if (lane == 0) {
            atomicAdd(&ctr->alg_bytes, (unsigned long long)bytes);
            atomicAdd(&ctr->alg_sectors, (unsigned long long)sectors);
        }
    }
    // nonrepetitive_fraction (step2/nam.cu:892) and the rescue trigger: a double
    // comparison of the float ratio with 0.7, or no hits (step2/main.cu:3211)
    const float frac = tot > 0 ? ((float)good) / ((float)tot) : 1.0f;
    const bool rescue = C.force_rescue || (C.rescue_level > 1 && (good == 0 || (double)frac < 0.7));
    if (lane == 0) {
        R.frac = frac;
        R.n_found = tot;
    }
    if (rescue) {
        // Reads inside short tandem repeats merge thousands of hits: their seeds'
        // runs (up to the count cap) estimate the merge's hits; reads above
        // kRescueHeavyHits (C.rescue_block_hits when set) go to the heavy end of the
        // list, which the rescue kernel takes first.
        uint32_t w = 0;
        if (good < tot) {
            for (uint32_t i = lane; i < nq2; i += 32) {
                const uint64_t pos = A.q_pos[R.q_off + i];
                if (pos == kNotFound) continue;
                const uint32_t c = index_get_count(I, pos);
                w += c <= C.count_cap ? c : 0u;
            }
            w = warp_sum(w);
        }
        const bool heavy = w >= (C.rescue_block_hits ? C.rescue_block_hits : kRescueHeavyHits);
        if (lane == 0) {
            R.flags |= kReadRescue;
            if (heavy) A.rescue_list[A.rescue_cap - 1 - atomicAdd(&ctr->n_rescue_heavy, 1u)] = r;
            else A.rescue_list[atomicAdd(&ctr->n_rescue, 1u)] = r;
            R.n_hits = 0;
        }
        return;
    }
    // hit offsets in generation order (query order, then run order)
    uint64_t running = 0;
    for (uint32_t base = 0; base < nq2; base += 32) {
        const uint32_t i = base + lane;
        const uint32_t v = i < nq2 ? aux[i] : 0;
        const uint32_t inc = warp_inclusive_sum(v);
        if (i < nq2) aux[i] = (uint32_t)running + inc - v;
        running += __shfl_sync(0xFFFFFFFFu, inc, 31);
    }
    __syncwarp();
    const uint64_t H = running;
    const uint64_t hoff = warp_bump(&ctr->hit_used, H);
    if (hoff + H > A.hit_cap) {
        warp_fail(R, ctr, kStatusHitOverflow);
        return;
    }
    const uint64_t* qp = A.q_pos + R.q_off;
    for (uint32_t i = lane; i < nq2; i += 32) {
        // queries that emitted hits in the first pass (found and not filtered)
        const uint32_t next = i + 1 < nq2 ? aux[i + 1] : (uint32_t)H;
        if (next == aux[i]) continue;
        const uint64_t pos = qp[i];
        const uint32_t dir = i >= nq ? 1u : 0u;
        HitPacked* out = A.hits + hoff + aux[i];
        uint32_t k = 0;
        const int qs = (int)Q[i].start, qe = (int)Q[i].end;
        walk_hit_run(I, qs, qe, pos, [&](uint32_t ref, int rs, int re) {
            out[k++] = pack_hit((dir << 31) | ref, qs, qe, rs, re);
        });
    }
    if (lane == 0) {
        R.hit_off = hoff;
        R.n_hits = (uint32_t)H;
    }
}

template <bool kCount>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_lookup(IndexView I, MapConfig C, uint32_t n,
                                                                 ReadRec* __restrict__ rec, Arenas A, Counters* ctr,
                                                                 const BatchDesc* desc) {
    if (desc) n = min(n, desc->n_reads);   // batched form: n is the work areas' capacity
    for (uint32_t r = warp_next(&ctr->queue_head2); r < n; r = warp_next(&ctr->queue_head2))
        lookup_read<kCount>(I, C, r, rec, A, ctr);
}

// The lookup of the reads seeded by k_seed_long (the long list).
template <bool kCount>
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_lookup_long(IndexView I, MapConfig C,
                                                                      ReadRec* __restrict__ rec, Arenas A,
                                                                      Counters* ctr) {
    const uint32_t n_long = *(volatile unsigned int*)&ctr->n_long;
    for (uint32_t t = warp_global_id(); t < n_long; t += warp_count())
        lookup_read<kCount>(I, C, A.long_list[t], rec, A, ctr);
}

// Seeding and lookup of a read by one warp (the main path): randstrobes_query, then
// the query loop of find_nams on the queries just written.  Seeding is bound by
// integer issue and the lookup by the latency of random index reads, so the warps of
// an SM interleave the two: while some wait on gathers, others hash.  Reads that do
// not fit the shared-memory buffers go to the long list (k_seed_long, then
// k_lookup_long).
// 6 blocks of 8 warps per SM (48 warps: the lookup's gathers need the warps in flight;
// 40 registers) and per-warp buffers for reads up to 512 bases and 160 syncmers (21 KB
// per block, leaving the rest of the SM's unified L1 to cache index entries); longer
// reads take the long path.
constexpr int kFusedBlocksPerSm = 6;
constexpr uint32_t kFusedMaxLen = 512;
constexpr uint32_t kFusedSyncmers = 160;

template <bool kCount>
__global__ void __launch_bounds__(32 * kSeedWarps, kFusedBlocksPerSm)
    k_seed_lookup(DevParams P, IndexView I, MapConfig C, const uint8_t* __restrict__ seqs,
                  const uint64_t* __restrict__ offs, const uint32_t* __restrict__ lens, uint32_t n,
                  ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    __shared__ uint64_t s_pk[kSeedWarps][kFusedMaxLen / 32 + 4];
    __shared__ uint32_t s_nm[kSeedWarps][kFusedMaxLen / 32 + 4];
    __shared__ uint64_t s_hb[kSeedWarps][64];
    __shared__ uint64_t s_sh[kSeedWarps][kFusedSyncmers];
    __shared__ uint32_t s_sp[kSeedWarps][kFusedSyncmers];
    const uint32_t w = threadIdx.x >> 5;
    for (uint32_t r = warp_next(&ctr->queue_head); r < n; r = warp_next(&ctr->queue_head)) {
        const uint32_t L = lens[r];
        ReadRec& R = rec[r];
        if (L > GBSA_MAX_READ_LEN) {
            warp_fail(R, ctr, kStatusReadTooLong);
            continue;
        }
        uint32_t ns = 0xFFFFFFFFu;
        if (L <= kFusedMaxLen)
            ns = warp_read_syncmers(P, seqs + offs[r], L, s_pk[w], s_nm[w], s_hb[w], s_sh[w], s_sp[w], kFusedSyncmers);
        if (ns == 0xFFFFFFFFu) {
            if (lane_id() == 0) {
                R.flags |= kReadLong;
                A.long_list[atomicAdd(&ctr->n_long, 1u)] = r;
            }
            continue;
        }
        emit_read_queries(P, s_sh[w], s_sp[w], ns, L, R, A, ctr);
        __syncwarp();
        lookup_read<kCount>(I, C, r, rec, A, ctr);
        __syncwarp();
    }
}

// The batched form's seeding + lookup: the body of k_seed_lookup, but each warp pulls
// work items from a device queue (an atomic counter) until the batch's items run out,
// so reads of uneven lengths and the two mates of a pair (one item) balance over the
// persistent grid; the batch (reads, count, items) is read from desc in device memory.
// The shape (warps per block, resident blocks per SM, shared-memory read window) is a
// template of its own per variant, picked at run time.
// kLookup false: seeding alone (indexes whose entries exceed the fuse limit are looked
// up by k_lookup afterwards, as in the plain form).
template <bool kCount, bool kLookup, int kWarps, int kBlocks, uint32_t kMaxLen, uint32_t kSyncmers>
__global__ void __launch_bounds__(32 * kWarps, kBlocks)
    k_seed_lookup_q(DevParams P, IndexView I, MapConfig C, const BatchDesc* __restrict__ desc,
                    ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    __shared__ uint64_t s_pk[kWarps][kMaxLen / 32 + 4];
    __shared__ uint32_t s_nm[kWarps][kMaxLen / 32 + 4];
    __shared__ uint64_t s_hb[kWarps][64];
    __shared__ uint64_t s_sh[kWarps][kSyncmers];
    __shared__ uint32_t s_sp[kWarps][kSyncmers];
    const uint32_t w = threadIdx.x >> 5;
    const uint8_t* __restrict__ seqs = desc->seqs;
    const uint64_t* __restrict__ offs = desc->offs;
    const uint32_t* __restrict__ lens = desc->lens;
    const uint32_t* __restrict__ items = desc->items;
    const uint32_t n_items = items ? desc->n_items : desc->n_reads;
    for (;;) {
        const uint32_t it = warp_next(&ctr->queue_head);
        if (it >= n_items) break;
        // item bounds outside [0, n_reads] are clamped (reads no item covers stay empty)
        const uint32_t n_reads = desc->n_reads;
        const uint32_t r0 = min(items ? items[it] : it, n_reads);
        const uint32_t r1 = min(items ? items[it + 1] : it + 1, n_reads);
        for (uint32_t r = r0; r < r1; ++r) {
            const uint32_t L = lens[r];
            ReadRec& R = rec[r];
            if (L > GBSA_MAX_READ_LEN) {
                warp_fail(R, ctr, kStatusReadTooLong);
                continue;
            }
            uint32_t ns = 0xFFFFFFFFu;
            if (L <= kMaxLen)
                ns = warp_read_syncmers(P, seqs + offs[r], L, s_pk[w], s_nm[w], s_hb[w], s_sh[w], s_sp[w], kSyncmers);
            if (ns == 0xFFFFFFFFu) {
                if (lane_id() == 0) {
                    R.flags |= kReadLong;
                    A.long_list[atomicAdd(&ctr->n_long, 1u)] = r;
                }
                continue;
            }
            emit_read_queries(P, s_sh[w], s_sp[w], ns, L, R, A, ctr);
            __syncwarp();
            if (kLookup) {
                lookup_read<kCount>(I, C, r, rec, A, ctr);
                __syncwarp();
            }
        }
    }
}

// Scratch of `bytes` for the calling warp: its own slot from byte `slot_off` on when
// the request fits, else a bump allocation in the shared overflow arena (nullptr
// when that is full too).
__device__ __forceinline__ uint8_t* warp_scratch(const Arenas& A, Counters* ctr, uint64_t slot_off, uint64_t bytes) {
    bytes = (bytes + 255) & ~255ull;   // keep every region 256-byte aligned
    if (slot_off + bytes <= A.slot_bytes) return A.slots + (uint64_t)warp_global_id() * A.slot_bytes + slot_off;
    const uint64_t o = warp_bump(&ctr->scratch_used, bytes);
    if (o + bytes > A.ovf_cap) return nullptr;
    return A.ovf + o;
}


// Scores, sorts and writes the closed NAMs of a read to the NAM arena.  keys needs
// room for next_pow2(n_closed) entries.
// Warp bitonic sort of P (a power of two) entries that moves only the first key word
// (k1) and the NAM index (ix); the second and third words stay by NAM index and are
// read when the first words tie.
__device__ void warp_sort_idx(uint64_t* k1, uint32_t* ix, const uint64_t* k2, const uint64_t* k3, uint32_t P) {
    const uint32_t lane = lane_id();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t q = lane; q < P / 2; q += 32) {
                const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                const uint32_t ixj = i | j;
                const uint64_t xb = k1[ixj], xa = k1[i];
                bool less;
                if (xb != xa) {
                    less = xb < xa;
                } else {
                    const uint32_t ib = ix[ixj], ia = ix[i];
                    const uint64_t b2 = k2[ib], a2 = k2[ia], b3 = k3[ib], a3 = k3[ia];
                    less = b2 != a2 ? b2 < a2 : (b3 != a3 ? b3 < a3 : ib < ia);
                }
                if (less == ((i & k) == 0)) {
                    k1[i] = xb;
                    k1[ixj] = xa;
                    const uint32_t t = ix[i];
                    ix[i] = ix[ixj];
                    ix[ixj] = t;
                }
            }
            __syncwarp();
        }
    }
}

// Sorts a rescued read's NAMs (at most kWarpSortMax) with the warp in its shared
// buffers sa / sb (4 KB each, free after the merge) and writes them to the NAM arena.
__device__ void warp_finish_nams(const MapConfig& C, const NamLists& L, uint32_t* sa, uint32_t* sb, ReadRec& R,
                                 const Arenas& A, Counters* ctr) {
    const uint32_t lane = lane_id();
    const uint32_t NN = L.n_closed;
    const uint32_t P = next_pow2(NN);
    uint64_t* k1 = reinterpret_cast<uint64_t*>(sa);       // P <= 256: 2 KB
    uint32_t* ix = sa + 512;                              // 1 KB
    uint64_t* k2 = reinterpret_cast<uint64_t*>(sb);       // 2 KB
    uint64_t* k3 = k2 + 256;                              // 2 KB
    for (uint32_t t = lane; t < P; t += 32) {
        NamKey k;
        if (t < NN) {
            k = nam_key(L.closed[t], t, C.sort_mode);
        } else {   // padding sorts last (a NAM's first key word is never all ones)
            k.k1 = k.k2 = k.k3 = ~0ULL;
        }
        k1[t] = k.k1;
        ix[t] = t;
        k2[t] = k.k2;
        k3[t] = k.k3;
    }
    __syncwarp();
    warp_sort_idx(k1, ix, k2, k3, P);
    const uint64_t noff = warp_bump(&ctr->nam_used, NN);
    if (noff + NN > A.nam_cap) {
        warp_fail(R, ctr, kStatusNamOverflow);
        return;
    }
    for (uint32_t t = lane; t < NN; t += 32) A.nams[noff + t] = L.closed[ix[t]];
    if (lane == 0) {
        R.nam_off = noff;
        R.n_nams = NN;
    }
    __syncwarp();
}

constexpr uint32_t kLaneMaxHits = kLaneMaxHitsCap;   // the lane kernel's hit-count buckets cover this
constexpr uint32_t kLaneOpen = 10;   // open NAMs a lane keeps in shared memory
constexpr int kLaneWarps = 4;
// The rescue chain runs beside the two NAM kernels on another stream; the persistent
// grids are sized so that the rescue chain keeps room beside them: rescue 1 x 72 KB,
// lane kernel 3 x 40 KB, then the warp kernel 5 x 32 KB (measured against 4, and against
// 2-3 lane blocks: fewer main-stream blocks speed the rescue chain but slow the main
// stream more).
constexpr int kLaneBlocksPerSm = 3;
constexpr int kRescueBlocksPerSm = 1;

__device__ __forceinline__ bool nam_key3_less(const NamKey& a, const NamKey& b) {
    if (a.k1 != b.k1) return a.k1 < b.k1;
    if (a.k2 != b.k2) return a.k2 < b.k2;
    return a.k3 < b.k3;
}

// Open NAMs of the lanes of a block, one field per array ([slot][thread]) so that a
// warp touching slot o reads 32 consecutive words.
struct LaneOpen {
    int32_t qs[kLaneOpen][32 * kLaneWarps], qe[kLaneOpen][32 * kLaneWarps], qprev[kLaneOpen][32 * kLaneWarps];
    int32_t rs[kLaneOpen][32 * kLaneWarps], re[kLaneOpen][32 * kLaneWarps], rprev[kLaneOpen][32 * kLaneWarps];
    int32_t nh[kLaneOpen][32 * kLaneWarps];
    uint32_t ref[kLaneOpen][32 * kLaneWarps];
    __device__ NamState get(uint32_t o, uint32_t t) const {
        NamState n;
        n.qs = qs[o][t];
        n.qe = qe[o][t];
        n.qprev = qprev[o][t];
        n.rs = rs[o][t];
        n.re = re[o][t];
        n.rprev = rprev[o][t];
        n.n_hits = nh[o][t];
        n.ref_rc = ref[o][t];
        return n;
    }
    __device__ void put(uint32_t o, uint32_t t, const NamState& n) {
        qs[o][t] = n.qs;
        qe[o][t] = n.qe;
        qprev[o][t] = n.qprev;
        rs[o][t] = n.rs;
        re[o][t] = n.re;
        rprev[o][t] = n.rprev;
        nh[o][t] = n.n_hits;
        ref[o][t] = n.ref_rc;
    }
    // After its merge a lane's 8 * kLaneOpen words (every 32 * kLaneWarps-th word of
    // the struct, from its thread index on) are free: they hold the sort entries
    // (first key word, NAM index; three words each) of up to kEntries of its NAMs.
    // Only the lane touches them, and the lanes of a warp hit 32 different banks.
    static constexpr uint32_t kEntries = 8 * kLaneOpen / 3;
    static constexpr uint32_t kStride = 32 * kLaneWarps;
    __device__ uint32_t* words() { return reinterpret_cast<uint32_t*>(this); }
    __device__ uint64_t key(uint32_t e, uint32_t t) {
        const uint32_t* w = words() + 3 * e * kStride + t;
        return ((uint64_t)w[kStride] << 32) | w[0];
    }
    __device__ uint32_t index(uint32_t e, uint32_t t) { return words()[(3 * e + 2) * kStride + t]; }
    __device__ void set_entry(uint32_t e, uint32_t t, uint64_t k, uint32_t i) {
        uint32_t* w = words() + 3 * e * kStride + t;
        w[0] = (uint32_t)k;
        w[kStride] = (uint32_t)(k >> 32);
        w[2 * kStride] = i;
    }
};
static_assert(sizeof(LaneOpen) == 8 * kLaneOpen * 32 * kLaneWarps * 4, "LaneOpen is 8 word arrays");

// find_nams merge with one lane per read, for reads with at most kLaneMaxHits hits
// whose open-NAM list stays within kLaneOpen (the common case: one locus chain plus
// scattered single hits).  Same hit-major rule as nam_merge_hit_major: hits in
// (orientation, query_start, position) order, each joins the first open NAM in
// creation order of its (orientation, ref id) that accepts it.  Open NAMs live in
// shared memory; a NAM is closed (written to the read's slots in the NAM arena) when
// the open list is full and the current query start has passed it, or at the end.
// The read's NAMs are then sorted (through shared memory).  Reads that do not fit go
// to the warp-cooperative kernel.
__device__ __forceinline__ HitRec load_hit(const HitPacked* __restrict__ hits, uint32_t i, uint32_t H) {
    HitRec h;
    if (i < H) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(hits + i));
        h.ref_rc = v.x;
        h.qs = (int32_t)(v.y & 0xFFFFu);
        h.qe = (int32_t)(v.y >> 16);
        h.rs = (int32_t)v.z;
        h.re = (int32_t)v.w;
    } else {
        h.ref_rc = 0;
        h.qs = h.qe = h.rs = h.re = -1;
    }
    return h;
}

// Hit-count bucket of a read for the lane kernel: 8 wide up to 64 hits, 16 wide up
// to 128, then one bucket up to kLaneMaxHits.
__device__ __forceinline__ uint32_t lane_bucket(uint32_t H) {
    if (H <= 64) return (H - 1) >> 3;
    if (H <= 128) return 8 + ((H - 65) >> 4);
    return 12;
}

// Sorts the reads with hits for the NAM kernels: more than kLaneMaxHits hits to the
// warp kernel's list, the others into lists by hit count, so that the lanes of a
// warp of the lane kernel merge reads of similar size (a warp runs as long as its
// longest read).  Appends are aggregated per warp and bucket.
__global__ void k_bucket_reads(uint32_t n, uint32_t lane_max, const ReadRec* __restrict__ rec, Arenas A,
                               Counters* ctr, const BatchDesc* desc) {
    if (desc) n = min(n, desc->n_reads);
    const uint32_t lane = lane_id();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t r = base + threadIdx.x;
        uint32_t key = 0xFFFFFFFFu;   // no list
        if (r < n) {
            const uint32_t flags = rec[r].flags;
            const uint32_t H = rec[r].n_hits;
            if (!(flags & (kReadFailed | kReadRescue)) && H > 0) key = H > lane_max ? 16u : lane_bucket(H);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t at = 0;
        if (key != 0xFFFFFFFFu && lane == leader)
            at = atomicAdd(key == 16u ? &ctr->n_big : &ctr->lane_cnt[key], (unsigned)__popc(peers));
        at = __shfl_sync(0xFFFFFFFFu, at, leader) + __popc(peers & lanemask_lt());
        if (key == 16u) A.big_list[at] = r;
        else if (key != 0xFFFFFFFFu) A.lane_lists[(size_t)key * A.lane_cap + at] = r;
    }
}

// Sorts a lane's n_closed NAMs (out[0..n_closed), written as they closed) by the NAM
// order, stably, and returns the arena offset of the sorted list: for at most
// Sort::kEntries NAMs on (first key word, index) entries in shared memory (full keys only
// on a tie of the first word), then one pass writes the NAMs in order behind the unsorted
// ones (out + H); more NAMs are insertion-sorted in place.  keys_ready: the entries were
// written as the NAMs closed (else they are computed here from out).  The NAM loads of
// the key pass and of the ordered copy are issued four at a time (each is a round trip
// to L2: out was just written).
template <class Sort>
__device__ __forceinline__ uint64_t lane_sort_nams(const MapConfig& C, Sort& S, uint32_t t, NamState* out,
                                                   uint32_t n_closed, uint32_t H, uint64_t noff, bool keys_ready) {
    if (n_closed <= Sort::kEntries) {
        if (!keys_ready) {
            uint32_t i = 0;
            for (; i + 4 <= n_closed; i += 4) {
                const NamState a = out[i], b = out[i + 1], c = out[i + 2], d = out[i + 3];
                S.set_entry(i, t, nam_key(a, 0, C.sort_mode).k1, i);
                S.set_entry(i + 1, t, nam_key(b, 0, C.sort_mode).k1, i + 1);
                S.set_entry(i + 2, t, nam_key(c, 0, C.sort_mode).k1, i + 2);
                S.set_entry(i + 3, t, nam_key(d, 0, C.sort_mode).k1, i + 3);
            }
            for (; i < n_closed; ++i) S.set_entry(i, t, nam_key(out[i], 0, C.sort_mode).k1, i);
        }
        for (uint32_t i = 1; i < n_closed; ++i) {
            const uint64_t kx = S.key(i, t);
            if (kx > S.key(i - 1, t)) continue;   // already in place
            const uint32_t ix = S.index(i, t);
            NamKey fx;
            bool have_fx = false;
            uint32_t j = i;
            while (j > 0) {
                const uint64_t ky = S.key(j - 1, t);
                const uint32_t iy = S.index(j - 1, t);
                bool less = kx < ky;
                if (kx == ky) {
                    if (!have_fx) {
                        fx = nam_key(out[ix], 0, C.sort_mode);
                        have_fx = true;
                    }
                    less = nam_key3_less(fx, nam_key(out[iy], 0, C.sort_mode));
                }
                if (!less) break;
                S.set_entry(j, t, ky, iy);
                --j;
            }
            S.set_entry(j, t, kx, ix);
        }
        NamState* sorted = out + H;
        uint32_t i = 0;
        for (; i + 4 <= n_closed; i += 4) {
            const NamState a = out[S.index(i, t)], b = out[S.index(i + 1, t)], c = out[S.index(i + 2, t)],
                           d = out[S.index(i + 3, t)];
            sorted[i] = a;
            sorted[i + 1] = b;
            sorted[i + 2] = c;
            sorted[i + 3] = d;
        }
        for (; i < n_closed; ++i) sorted[i] = out[S.index(i, t)];
        return noff + H;
    }
    for (uint32_t i = 1; i < n_closed; ++i) {
        const NamState x = out[i];
        const NamKey kx = nam_key(x, 0, C.sort_mode);
        uint32_t j = i;
        while (j > 0) {
            const NamState y = out[j - 1];
            if (!nam_key3_less(kx, nam_key(y, 0, C.sort_mode))) break;
            out[j] = y;
            --j;
        }
        out[j] = x;
    }
    return noff;
}

// kMinBlocks: resident blocks the compiler must leave room for (0: no bound); a smaller
// register budget leaves room on the SM for the rescued reads' sorts beside it.
template <int kMinBlocks>
__global__ void __launch_bounds__(32 * kLaneWarps, kMinBlocks) k_nams_lane(MapConfig C, uint32_t n, ReadRec* __restrict__ rec,
                                                               Arenas A, Counters* ctr) {
    __shared__ LaneOpen S;
    __shared__ uint32_t s_cnt[kLaneBuckets];
    const uint32_t t = threadIdx.x;
    if (t < kLaneBuckets) s_cnt[t] = *(volatile unsigned int*)&ctr->lane_cnt[t];
    __syncthreads();
    uint32_t total = 0;
    for (uint32_t b = 0; b < kLaneBuckets; ++b) total += s_cnt[b];
    // reads by bucket, the most hits first
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        uint32_t b = kLaneBuckets - 1, j = i;
        while (j >= s_cnt[b]) j -= s_cnt[b--];
        const uint32_t r = A.lane_lists[(size_t)b * A.lane_cap + j];
        ReadRec& R = rec[r];
        const uint32_t flags = R.flags;
        const uint32_t H = R.n_hits;
        // 2H slots: the NAMs as they close, then (for the sort through shared memory)
        // the same NAMs in order
        const uint64_t noff = atomicAdd(&ctr->nam_used, 2ull * H);
        if (noff + 2ull * H > A.nam_cap) {
            R.flags = flags | kReadFailed;
            atomicOr(&ctr->status, kStatusNamOverflow);
            continue;
        }
        const HitPacked* hits = A.hits + R.hit_off;
        NamState* out = A.nams + noff;
        uint32_t n_open = 0, n_closed = 0, cur_dir = 0;
        bool overflow = false;
        // the next two hits are loaded while one merges
        HitRec nx0 = load_hit(hits, 0, H), nx1 = load_hit(hits, 1, H);
        for (uint32_t i = 0; i < H; ++i) {
            const HitRec x = nx0;
            nx0 = nx1;
            nx1 = load_hit(hits, i + 2, H);
            const uint32_t dir = x.ref_rc >> 31;
            if (dir != cur_dir) {   // the other orientation's NAMs can take no more hits
                for (uint32_t o = 0; o < n_open; ++o) out[n_closed++] = S.get(o, t);
                n_open = 0;
                cur_dir = dir;
            }
            int found = -1;
            for (uint32_t o = 0; o < n_open; ++o) {
                if (S.ref[o][t] == x.ref_rc && S.qprev[o][t] < x.qs && x.qs <= S.qe[o][t] && S.rprev[o][t] < x.rs &&
                    x.rs <= S.re[o][t]) {
                    const bool ext = x.qe > S.qe[o][t] && x.re > S.re[o][t];
                    if (ext || (x.qe <= S.qe[o][t] && x.re <= S.re[o][t])) {
                        if (ext) {
                            S.qe[o][t] = x.qe;
                            S.re[o][t] = x.re;
                        }
                        S.qprev[o][t] = x.qs;
                        S.rprev[o][t] = x.rs;
                        S.nh[o][t] += 1;
                        found = (int)o;
                        break;
                    }
                }
            }
            if (found >= 0) continue;
            if (n_open == kLaneOpen) {
                // close NAMs the current query start has passed (order kept)
                uint32_t k = 0;
                for (uint32_t o = 0; o < n_open; ++o) {
                    const NamState m = S.get(o, t);
                    if (m.qe < x.qs) out[n_closed++] = m;
                    else S.put(k++, t, m);
                }
                n_open = k;
                if (n_open == kLaneOpen) {
                    overflow = true;
                    break;
                }
            }
            S.put(n_open++, t, nam_from_hit(x));
        }
        if (overflow) {
            A.big_list[atomicAdd(&ctr->n_big, 1u)] = r;
            continue;
        }
        for (uint32_t o = 0; o < n_open; ++o) out[n_closed++] = S.get(o, t);
        // the lane's open-list words are free now: they hold the sort entries
        R.nam_off = lane_sort_nams(C, S, t, out, n_closed, H, noff, false);
        R.n_nams = n_closed;
    }
}

// The lane-per-read merge with the open NAMs in registers (lane_variant 3).  Same rule
// as k_nams_lane: each hit joins the first open NAM in creation order that accepts it,
// else opens one; when all kLaneOpen slots are in use, NAMs the current query start has
// passed are closed, and a read that still has no free slot goes to the warp kernel.
// A slot keeps its place while open: creation order is a per-slot sequence number, a
// closed NAM frees its slot (the read's NAMs are sorted by their full key at the end,
// so the order they close in does not matter).  Every slot access is unrolled over the
// kLaneOpen slots, so the lanes of a warp stay together through a hit whatever their
// open lists hold; shared memory holds only the final sort's entries.
constexpr uint32_t kLaneEntriesR = 20;   // NAMs of a read sorted in shared memory (more: in place, in HBM)

template <uint32_t kSlots>
struct LaneSlots {
    // query start | query end << 12 | creation number << 24 (query coordinates are below
    // GBSA_MAX_READ_LEN = 4096, creation numbers below kLaneMaxHitsCap + 1); creation
    // number kFree: the slot is free
    uint32_t qse[kSlots];
    uint32_t qpn[kSlots];   // previous hit's query start | n_hits << 16
    int32_t rs[kSlots], re[kSlots], rprev[kSlots];
    uint32_t ref[kSlots];
    static constexpr uint32_t kFree = 0xFFu;
    __device__ __forceinline__ uint32_t seq(uint32_t o) const { return qse[o] >> 24; }
    __device__ __forceinline__ int32_t qe(uint32_t o) const { return (int32_t)((qse[o] >> 12) & 0xFFFu); }
    __device__ __forceinline__ void free_slot(uint32_t o) { qse[o] |= kFree << 24; }
    __device__ __forceinline__ NamState get(uint32_t o) const {
        NamState n;
        n.qs = (int32_t)(qse[o] & 0xFFFu);
        n.qe = qe(o);
        n.qprev = (int32_t)(qpn[o] & 0xFFFFu);
        n.n_hits = (int32_t)(qpn[o] >> 16);
        n.rs = rs[o];
        n.re = re[o];
        n.rprev = rprev[o];
        n.ref_rc = ref[o];
        return n;
    }
};
static_assert(GBSA_MAX_READ_LEN <= 4096 && kLaneMaxHitsCap < 255, "lane slot packing");

struct LaneSortR {
    uint32_t w[3 * kLaneEntriesR][32 * kLaneWarps];
    static constexpr uint32_t kEntries = kLaneEntriesR;
    __device__ uint64_t key(uint32_t e, uint32_t t) const {
        return ((uint64_t)w[3 * e + 1][t] << 32) | w[3 * e][t];
    }
    __device__ uint32_t index(uint32_t e, uint32_t t) const { return w[3 * e + 2][t]; }
    __device__ void set_entry(uint32_t e, uint32_t t, uint64_t k, uint32_t i) {
        w[3 * e][t] = (uint32_t)k;
        w[3 * e + 1][t] = (uint32_t)(k >> 32);
        w[3 * e + 2][t] = i;
    }
};

// Writes a closing NAM to the lane's list and, while the list fits the shared-memory
// sort, its sort entry (its first key word, computed from registers).
__device__ __forceinline__ void lane_close_r(const MapConfig& C, LaneSortR& S, uint32_t t, NamState* out,
                                             uint32_t& n_closed, const NamState& m) {
    if (n_closed < LaneSortR::kEntries) S.set_entry(n_closed, t, nam_key(m, 0, C.sort_mode).k1, n_closed);
    out[n_closed++] = m;
}

// kMinBlocks: the register budget (3: 168 registers, no spills; 4: 128 registers, which
// leaves room beside two blocks per SM for the rescue kernel's block; 5 with 6 slots: 96
// registers, three blocks per SM beside the rescue kernel's block).  kSlots: open NAMs
// per lane (reads that need more go to the warp kernel).
template <int kMinBlocks, uint32_t kSlots>
__global__ void __launch_bounds__(32 * kLaneWarps, kMinBlocks)
    k_nams_lane_r(MapConfig C, uint32_t n, ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    __shared__ LaneSortR S;
    __shared__ uint32_t s_cnt[kLaneBuckets];
    const uint32_t t = threadIdx.x;
    if (t < kLaneBuckets) s_cnt[t] = *(volatile unsigned int*)&ctr->lane_cnt[t];
    __syncthreads();
    uint32_t total = 0;
    for (uint32_t b = 0; b < kLaneBuckets; ++b) total += s_cnt[b];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        uint32_t b = kLaneBuckets - 1, j = i;
        while (j >= s_cnt[b]) j -= s_cnt[b--];
        const uint32_t r = A.lane_lists[(size_t)b * A.lane_cap + j];
        ReadRec& R = rec[r];
        const uint32_t flags = R.flags;
        const uint32_t H = R.n_hits;
        const uint64_t noff = atomicAdd(&ctr->nam_used, 2ull * H);
        if (noff + 2ull * H > A.nam_cap) {
            R.flags = flags | kReadFailed;
            atomicOr(&ctr->status, kStatusNamOverflow);
            continue;
        }
        const HitPacked* hits = A.hits + R.hit_off;
        NamState* out = A.nams + noff;
        LaneSlots<kSlots> L;
#pragma unroll
        for (uint32_t o = 0; o < kSlots; ++o) L.qse[o] = LaneSlots<kSlots>::kFree << 24;
        uint32_t n_open = 0, n_closed = 0, cur_dir = 0, next_seq = 0;
        bool overflow = false;
        HitRec nx = load_hit(hits, 0, H);
        for (uint32_t i = 0; i < H; ++i) {
            const HitRec x = nx;
            nx = load_hit(hits, i + 1, H);
            const uint32_t dir = x.ref_rc >> 31;
            if (dir != cur_dir) {   // the other orientation's NAMs can take no more hits
#pragma unroll
                for (uint32_t o = 0; o < kSlots; ++o)
                    if (L.seq(o) != LaneSlots<kSlots>::kFree) {
                        lane_close_r(C, S, t, out, n_closed, L.get(o));
                        L.free_slot(o);
                    }
                n_open = 0;
                cur_dir = dir;
            }
            // the accepting NAM created first (free slots have the largest number)
            uint32_t best = kSlots, bseq = LaneSlots<kSlots>::kFree;
#pragma unroll
            for (uint32_t o = 0; o < kSlots; ++o) {
                const int32_t sqe = L.qe(o);
                const int32_t sqp = (int32_t)(L.qpn[o] & 0xFFFFu);
                bool ok = L.ref[o] == x.ref_rc && sqp < x.qs && x.qs <= sqe && L.rprev[o] < x.rs && x.rs <= L.re[o];
                ok = ok && ((x.qe > sqe && x.re > L.re[o]) || (x.qe <= sqe && x.re <= L.re[o]));
                if (ok && L.seq(o) < bseq) {
                    bseq = L.seq(o);
                    best = o;
                }
            }
            if (best < kSlots) {
#pragma unroll
                for (uint32_t o = 0; o < kSlots; ++o) {
                    if (o != best) continue;
                    if (x.qe > L.qe(o) && x.re > L.re[o]) {
                        L.qse[o] = (L.qse[o] & 0xFF000FFFu) | ((uint32_t)x.qe << 12);
                        L.re[o] = x.re;
                    }
                    L.qpn[o] = (uint32_t)x.qs | (((L.qpn[o] >> 16) + 1u) << 16);
                    L.rprev[o] = x.rs;
                }
                continue;
            }
            if (n_open == kSlots) {
                // close NAMs the current query start has passed
#pragma unroll
                for (uint32_t o = 0; o < kSlots; ++o)
                    if (L.seq(o) != LaneSlots<kSlots>::kFree && L.qe(o) < x.qs) {
                        lane_close_r(C, S, t, out, n_closed, L.get(o));
                        L.free_slot(o);
                        --n_open;
                    }
                if (n_open == kSlots) {
                    overflow = true;
                    break;
                }
            }
            bool placed = false;
#pragma unroll
            for (uint32_t o = 0; o < kSlots; ++o) {
                if (placed || L.seq(o) != LaneSlots<kSlots>::kFree) continue;
                L.qse[o] = (uint32_t)x.qs | ((uint32_t)x.qe << 12) | (next_seq << 24);
                L.qpn[o] = (uint32_t)x.qs | (1u << 16);
                L.rs[o] = x.rs;
                L.re[o] = x.re;
                L.rprev[o] = x.rs;
                L.ref[o] = x.ref_rc;
                placed = true;
            }
            ++next_seq;
            ++n_open;
        }
        if (overflow) {
            A.big_list[atomicAdd(&ctr->n_big, 1u)] = r;
            continue;
        }
#pragma unroll
        for (uint32_t o = 0; o < kSlots; ++o)
            if (L.seq(o) != LaneSlots<kSlots>::kFree) lane_close_r(C, S, t, out, n_closed, L.get(o));
        R.nam_off = lane_sort_nams(C, S, t, out, n_closed, H, noff, n_closed <= LaneSortR::kEntries);
        R.n_nams = n_closed;
    }
}

// Open NAM list of one warp in struct-of-arrays form (field f of NAM o at
// b[f * stride + o]), so that 32 lanes reading one field of 32 NAMs touch 32
// consecutive words.
struct OpenSoA {
    int32_t* b;
    uint32_t stride;
    __device__ int32_t* f(int k) const { return b + (size_t)k * stride; }
    __device__ NamState get(uint32_t o) const {
        NamState n;
        n.qs = b[o];
        n.qe = b[stride + o];
        n.qprev = b[2 * stride + o];
        n.rs = b[3 * stride + o];
        n.re = b[4 * stride + o];
        n.rprev = b[5 * stride + o];
        n.n_hits = b[6 * stride + o];
        n.ref_rc = (uint32_t)b[7 * stride + o];
        return n;
    }
    __device__ void put(uint32_t o, const NamState& n) const {
        b[o] = n.qs;
        b[stride + o] = n.qe;
        b[2 * stride + o] = n.qprev;
        b[3 * stride + o] = n.rs;
        b[4 * stride + o] = n.re;
        b[5 * stride + o] = n.rprev;
        b[6 * stride + o] = n.n_hits;
        b[7 * stride + o] = (int32_t)n.ref_rc;
    }
};

// Moves the open NAMs with query_end < qs (all of them when qs == INT_MAX) to the
// closed list, keeping the order of both lists.
__device__ __forceinline__ void soa_close_passed(const OpenSoA& O, uint32_t& n_open, NamState* closed,
                                                 uint32_t& n_closed, int qs) {
    const uint32_t lane = lane_id();
    if (qs != 0x7FFFFFFF) {
        bool any = false;
        for (uint32_t base = 0; base < n_open && !any; base += 32) {
            const uint32_t o = base + lane;
            any = __any_sync(0xFFFFFFFFu, o < n_open && O.b[O.stride + o] < qs);
        }
        if (!any) return;
    }
    uint32_t keep = 0, done = 0;
    for (uint32_t base = 0; base < n_open; base += 32) {
        const uint32_t o = base + lane;
        const bool valid = o < n_open;
        NamState n;
        if (valid) n = O.get(o);
        const bool stay = valid && n.qe >= qs;
        const uint32_t ms = __ballot_sync(0xFFFFFFFFu, stay);
        const uint32_t mc = __ballot_sync(0xFFFFFFFFu, valid && !stay);
        __syncwarp();
        if (stay) O.put(keep + __popc(ms & lanemask_lt()), n);
        else if (valid) closed[n_closed + done + __popc(mc & lanemask_lt())] = n;
        keep += __popc(ms);
        done += __popc(mc);
        __syncwarp();
    }
    n_open = keep;
    n_closed += done;
}

// Hit-major merge of nh <= 32 hits of one query randstrobe, held one per lane in
// registers (lane j holds hit j, in ref_start order), against the NAMs [0, nn) that
// were open when the query started: each hit joins the first of them in creation
// order that accepts it, else opens a new NAM.  Returns false (with the list
// unchanged from the failing hit on) when a new NAM would not fit in cap.
__device__ __forceinline__ bool soa_merge_hits(const OpenSoA& O, uint32_t nn, uint32_t& n_open, uint32_t cap,
                                               const HitRec& xl, uint32_t nh) {
    const uint32_t lane = lane_id();
    const int32_t* fqe = O.f(1);
    const int32_t* fqprev = O.f(2);
    const int32_t* fre = O.f(4);
    const int32_t* frprev = O.f(5);
    const int32_t* fref = O.f(7);
    for (uint32_t j = 0; j < nh; ++j) {
        HitRec x;
        x.ref_rc = __shfl_sync(0xFFFFFFFFu, xl.ref_rc, j);
        x.qs = __shfl_sync(0xFFFFFFFFu, xl.qs, j);
        x.qe = __shfl_sync(0xFFFFFFFFu, xl.qe, j);
        x.rs = __shfl_sync(0xFFFFFFFFu, xl.rs, j);
        x.re = __shfl_sync(0xFFFFFFFFu, xl.re, j);
        bool found = false;
        for (uint32_t base = 0; base < nn; base += 32) {
            const uint32_t o = base + lane;
            bool ok = false;
            int qe = 0, re = 0;
            if (o < nn) {
                qe = fqe[o];
                re = fre[o];
                ok = (uint32_t)fref[o] == x.ref_rc && fqprev[o] < x.qs && x.qs <= qe && frprev[o] < x.rs &&
                     x.rs <= re && ((x.qe > qe && x.re > re) || (x.qe <= qe && x.re <= re));
            }
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
            if (m) {
                if (lane == (uint32_t)(__ffs(m) - 1)) {   // the first accepting NAM takes the hit
                    if (x.qe > qe && x.re > re) {
                        O.f(1)[o] = x.qe;
                        O.f(4)[o] = x.re;
                    }
                    O.f(2)[o] = x.qs;
                    O.f(5)[o] = x.rs;
                    O.f(6)[o] += 1;
                }
                found = true;
                break;
            }
        }
        if (!found) {
            if (n_open == cap) return false;
            if (lane == 0) O.put(n_open, nam_from_hit(x));
            ++n_open;
        }
        __syncwarp();
    }
    return true;
}


// find_nams merge of one read's hits (in (orientation, query_start, position)
// order) with the open list O (capacity cap); closed NAMs are appended to closed.
// Each query randstrobe's hits are loaded 32 at a time, one per lane, and the next
// chunk is fetched while the current one merges.  Returns false when the open list
// outgrew cap.
__device__ __forceinline__ bool warp_find_nams(const HitPacked* __restrict__ hits, uint32_t H, const OpenSoA& O,
                                               uint32_t cap, NamState* closed, uint32_t& n_closed) {
    const uint32_t lane = lane_id();
    uint32_t n_open = 0, cur_dir = 0;
    n_closed = 0;
    uint32_t i = 0;
    HitRec xl = load_hit(hits, lane, H);
    while (i < H) {
        const uint32_t dir = __shfl_sync(0xFFFFFFFFu, xl.ref_rc, 0) >> 31;
        const int qs = __shfl_sync(0xFFFFFFFFu, xl.qs, 0);
        if (dir != cur_dir) {   // the other orientation's NAMs can take no more hits
            soa_close_passed(O, n_open, closed, n_closed, 0x7FFFFFFF);
            cur_dir = dir;
        }
        soa_close_passed(O, n_open, closed, n_closed, qs);
        const uint32_t nn = n_open;   // NAMs made by this query cannot take its other hits
        for (;;) {
            const bool same = i + lane < H && (xl.ref_rc >> 31) == dir && xl.qs == qs;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, same);
            const uint32_t cnt = m == 0xFFFFFFFFu ? 32u : (uint32_t)(__ffs(~m) - 1);
            const HitRec nx = load_hit(hits, i + cnt + lane, H);
            if (!soa_merge_hits(O, nn, n_open, cap, xl, cnt)) return false;
            i += cnt;
            xl = nx;
            if (cnt < 32) break;
        }
    }
    soa_close_passed(O, n_open, closed, n_closed, 0x7FFFFFFF);
    return true;
}

constexpr uint32_t kHeavyOpen = 256;   // open NAMs (and sort keys) a warp keeps in shared memory
constexpr int kHeavyWarps = 4;
constexpr int kHeavyBlocksPerSm = 5;   // register budget
constexpr int kHeavyGridPerSm = 5;     // blocks launched per SM (32 KB each)

// find_nams for the reads the lane kernel passed on (many hits, or many NAMs open
// at once): a warp per read.  The open list lives in shared memory (in global
// scratch for a read whose open list outgrows kHeavyOpen); closed NAMs go to the
// warp's global scratch, which is only written until the sort.  The read's NAMs are
// then sorted by key in shared memory (in scratch beyond kHeavyOpen NAMs) and
// gathered to the NAM arena.
// kMinBlocks: resident blocks the compiler must leave room for (its register budget);
// the grid stays kHeavyGridPerSm blocks per SM, so a larger kMinBlocks leaves registers
// free beside it for the rescued reads' sorts.
template <int kMinBlocks>
__global__ void __launch_bounds__(32 * kHeavyWarps, kMinBlocks)
    k_nams(MapConfig C, ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    __shared__ __align__(16) int32_t s_open[kHeavyWarps][8 * kHeavyOpen];
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t n_big = *(volatile unsigned int*)&ctr->n_big;
    for (uint32_t b = warp_global_id(); b < n_big; b += warp_count()) {
        const long long t0 = clock64();
        const uint32_t r = A.big_list[b];
        ReadRec& R = rec[r];
        if (R.flags & (kReadFailed | kReadRescue)) continue;
        const uint32_t H = R.n_hits;
        if (H == 0) continue;
        const HitPacked* hits = A.hits + R.hit_off;
        const uint32_t P2 = next_pow2(H);
        const bool big = H > kHeavyOpen;
        uint8_t* sc = warp_scratch(A, ctr, 0, 32ull * H + (big ? 32ull * P2 : 0) + 64);
        if (!sc) {
            warp_fail(R, ctr, kStatusScratchOverflow);
            continue;
        }
        NamState* closed = reinterpret_cast<NamState*>(sc);
        uint32_t NN = 0;
        OpenSoA O{s_open[w], kHeavyOpen};
        if (!warp_find_nams(hits, H, O, kHeavyOpen, closed, NN)) {
            // the open list outgrew shared memory: again with it in scratch
            __syncwarp();
            const OpenSoA G{reinterpret_cast<int32_t*>(closed + H), P2};
            warp_find_nams(hits, H, G, H, closed, NN);
        }
        const long long t_merge = clock64();
        __syncwarp();
        // sort: up to kHeavyOpen NAMs in the warp's shared open-list buffer (now free),
        // moving only the first key word and the NAM index; more in global scratch
        const bool small = NN <= kHeavyOpen;
        uint32_t* order = nullptr;   // sorted NAM indices
        NamKey* keys = reinterpret_cast<NamKey*>(closed + H);
        if (small) {
            static_assert(kHeavyOpen <= 256, "the sort entries fit the open-list buffer");
            int32_t* so = s_open[w];
            uint64_t* k1 = reinterpret_cast<uint64_t*>(so);         // 2 KB
            uint32_t* ix = reinterpret_cast<uint32_t*>(so + 512);   // 1 KB
            uint64_t* k2 = reinterpret_cast<uint64_t*>(so + 768);   // 2 KB
            uint64_t* k3 = k2 + 256;                                // 2 KB
            const uint32_t P = next_pow2(NN);
            for (uint32_t t = lane; t < P; t += 32) {
                NamKey k;
                if (t < NN) {
                    k = nam_key(closed[t], t, C.sort_mode);
                } else {   // padding sorts last (a NAM's first key word is never all ones)
                    k.k1 = k.k2 = k.k3 = ~0ULL;
                }
                k1[t] = k.k1;
                ix[t] = t;
                k2[t] = k.k2;
                k3[t] = k.k3;
            }
            __syncwarp();
            warp_sort_idx(k1, ix, k2, k3, P);
            order = ix;
        } else {
            for (uint32_t t = lane; t < NN; t += 32) keys[t] = nam_key(closed[t], t, C.sort_mode);
            __syncwarp();
            warp_sort_keys(keys, NN);
        }
        const uint64_t noff = warp_bump(&ctr->nam_used, NN);
        if (noff + NN > A.nam_cap) {
            warp_fail(R, ctr, kStatusNamOverflow);
            continue;
        }
        for (uint32_t t = lane; t < NN; t += 32) A.nams[noff + t] = closed[small ? order[t] : keys[t].idx];
        if (lane == 0) {
            R.nam_off = noff;
            R.n_nams = NN;
            if (A.nam_cycles) {
                uint64_t* note = A.nam_cycles + 4ull * b;   // cycles, hits, NAMs, merge cycles
                note[0] = (uint64_t)(clock64() - t0);
                note[1] = H;
                note[2] = NN;
                note[3] = (uint64_t)(t_merge - t0);
            }
        }
        __syncwarp();
    }
}

// Phase 1 of find_nams_rescue for one read (warp): RescueHit{position, count, qs,
// qe} of every found query of each orientation, sorted by (count, query_start) —
// query_start is unique per orientation, so this is the reference's
// (count, query_start, query_end) order (cmp1, step2/nam.cu:909-912); the prefix
// taken until (count > rescue_cutoff && taken >= 5) || count > cap
// (step2/nam.cu:960-969); re-sorted by query_start (cmp2).  rk/tk: 2 x Pq u64 each.
// Returns the sum and the maximum of the run lengths of the taken ones.
struct RescuePlan {
    uint32_t m[2];
    uint64_t bound;
    uint32_t maxrun;
};

// One orientation d of rescue_prepare: adds its taken prefix to plan.
__device__ void rescue_prepare_dir(const IndexView& I, const MapConfig& C, const Query* const* Qd,
                                   const uint64_t* const* Pd, const uint32_t* nqd, uint32_t Pq, uint64_t* buf, int d,
                                   RescuePlan& plan) {
    const uint32_t lane = lane_id();
    uint64_t* rk[2] = {buf, buf + Pq};
    uint64_t* tk[2] = {buf + 2 * Pq, buf + 3 * Pq};
    {
        uint32_t nd = 0;
        const uint32_t nq = nqd[d];
        for (uint32_t base = 0; base < nq; base += 32) {
            const uint32_t qi = base + lane;
            bool f = false;
            uint64_t key = 0;
            if (qi < nq) {
                const uint64_t pos = Pd[d][qi];
                if (pos != kNotFound) {
                    f = true;
                    const uint32_t cnt = index_get_count(I, pos);
                    key = ((uint64_t)cnt << 32) | ((uint64_t)Qd[d][qi].start << 16) | qi;
                }
            }
            const uint32_t bm = __ballot_sync(0xFFFFFFFFu, f);
            if (f) rk[d][nd + __popc(bm & lanemask_lt())] = key;
            nd += __popc(bm);
        }
        __syncwarp();
        warp_sort_u64(rk[d], nd);
        uint32_t stop = nd;
        for (uint32_t base = 0; base < nd; base += 32) {
            const uint32_t j = base + lane;
            bool brk = false;
            if (j < nd) {
                const uint32_t cnt = (uint32_t)(rk[d][j] >> 32);
                brk = (cnt > C.rescue_cutoff && j >= 5) || cnt > C.count_cap;
            }
            const uint32_t bm = __ballot_sync(0xFFFFFFFFu, brk);
            if (bm) {
                stop = base + (__ffs(bm) - 1);
                break;
            }
        }
        plan.m[d] = stop;
        uint64_t bsum = 0;
        uint32_t bmax = 0;
        for (uint32_t j = lane; j < stop; j += 32) {
            const uint32_t cnt = (uint32_t)(rk[d][j] >> 32);
            bsum += cnt;
            bmax = cnt > bmax ? cnt : bmax;
            tk[d][j] = ((rk[d][j] & 0xFFFFFFFFull) << 32) | cnt;   // (start, index) order, run length
        }
        plan.bound += warp_sum(bsum);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint32_t v = __shfl_xor_sync(0xFFFFFFFFu, bmax, o);
            bmax = v > bmax ? v : bmax;
        }
        plan.maxrun = bmax > plan.maxrun ? bmax : plan.maxrun;
        __syncwarp();
        warp_sort_u64(tk[d], stop);
    }
}

__device__ RescuePlan rescue_prepare(const IndexView& I, const MapConfig& C, const Query* const* Qd,
                                     const uint64_t* const* Pd, const uint32_t* nqd, uint32_t Pq, uint64_t* buf) {
    RescuePlan plan{};
    rescue_prepare_dir(I, C, Qd, Pd, nqd, Pq, buf, 0, plan);
    rescue_prepare_dir(I, C, Qd, Pd, nqd, Pq, buf, 1, plan);
    return plan;
}

// Phase 2 (warp): walk the runs of the taken rescue hits in (orientation,
// query_start) order and merge them NAM-major; all NAMs end in L.closed.  The hits
// of the current query are held in compact form in hrs/hpk/tb (room for
// plan.maxrun hits).
__device__ uint64_t rescue_merge(const IndexView& I, const Query* const* Qd, const uint64_t* const* Pd,
                                 const RescuePlan& plan, const uint64_t* tkbuf, uint32_t Pq, NamLists& L, uint32_t* hrs,
                                 uint32_t* hpk, uint8_t* tb) {
    uint64_t walk_cycles = 0;
    const uint64_t* tk[2] = {tkbuf + 2 * Pq, tkbuf + 3 * Pq};
    for (int d = 0; d < 2; ++d) {
        for (uint32_t j = 0; j < plan.m[d]; ++j) {
            const uint32_t qi = (uint32_t)(tk[d][j] >> 32) & 0xFFFF;
            const uint32_t cnt = (uint32_t)tk[d][j];
            const Query q = Qd[d][qi];
            QueryHits Q;
            Q.rs = hrs;
            Q.packed = hpk;
            Q.qs = (int)q.start;
            Q.qe = (int)q.end;
            Q.dir = (uint32_t)d;
            Q.k = I.k;
            const long long tw = clock64();
            Q.n = warp_walk_run_n(I, Q.qs, Q.qe, Pd[d][qi], cnt, hrs, hpk, plan.maxrun);
            walk_cycles += (uint64_t)(clock64() - tw);
            nam_close_merge_q(L, Q, tb);
        }
        nam_close_passed(L, 0x7FFFFFFF);
    }
    return walk_cycles;
}

constexpr uint32_t kWarpSortMax = 256;   // rescued reads with more NAMs are sorted by k_sort_jobs
constexpr uint32_t kSortTile = 2048;      // keys per shared-memory tile of the small block sort (56 KB)

// find_nams_rescue for the reads on the rescue list (a warp per read).  Reads that
// end with more than kWarpSortMax NAMs leave the sort to k_sort_jobs.
constexpr uint32_t kRescueSmemHits = 1024;   // per-warp shared buffer for one query's hits

// Hands a rescued read's NAMs to the block sort (more than kWarpSortMax) and returns
// true, or returns false (the caller's warp sorts them).
__device__ __forceinline__ bool rescue_sort_job(const Arenas& A, Counters* ctr, ReadRec& R, const NamLists& L,
                                                NamKey* keys, uint32_t r, uint32_t t) {
    if (L.n_closed <= kWarpSortMax) return false;
    // many NAMs: the block-per-read sort kernel orders them.  The count is known now
    // (the sort only orders them), so the NAM offsets of the batch can be computed
    // while the sorts run; the sort sets nam_off.
    if (lane_id() == 0) {
        R.n_nams = L.n_closed;
        const uint32_t j = L.n_closed > kSortTile ? A.jobs_cap - 1 - atomicAdd(&ctr->n_huge, 1u)
                                                  : atomicAdd(&ctr->n_heavy, 1u);
        SortJob job;
        job.closed = L.closed;
        job.keys = keys;
        job.n = L.n_closed;
        job.read = r;
        job.note = t;
        job.pad = 0;
        A.sort_jobs[j] = job;
    }
    return true;
}

// find_nams_rescue for one heavy read (entry t of the rescue list) with the whole
// block: the two orientations' plans on warps 0 and 1, each query's hit run walked by
// warp 0 and merged by block_close_merge_q.  The shared buffers of the block's warps
// serve as one: the candidates (hrs), the query's hits (hpk: positions, then packed
// words) and its taken flags (tb).
__device__ void rescue_read_block(const IndexView& I, const MapConfig& C, ReadRec* __restrict__ rec,
                                  const Arenas& A, Counters* ctr, uint32_t t, uint32_t* s_hrs, uint32_t* s_hpk,
                                  uint8_t* s_tb) {
    __shared__ uint8_t* s_sc;
    __shared__ RescuePlan s_plan[2];
    __shared__ uint32_t s_n;
    __shared__ uint32_t s_bcnt[kBlockSeg / 32];
    __shared__ uint32_t s_tot[3];
    constexpr uint32_t kBlockHits = kWarpsPerBlock * kRescueSmemHits / 2;   // hits of one query in s_hpk
    static_assert(kWarpsPerBlock * kRescueSmemHits >= kBlockSeg, "the candidates fit the shared buffers");
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const long long t0 = clock64();
    const uint32_t r = A.rescue_list[A.rescue_cap - 1 - t];
    ReadRec& R = rec[r];
    const uint32_t nqd[2] = {R.nq, R.nq2 - R.nq};
    const Query* Qd[2] = {A.q + R.q_off, A.q + R.q_off + R.nq};
    const uint64_t* Pd[2] = {A.q_pos + R.q_off, A.q_pos + R.q_off + R.nq};
    const uint32_t nqm = nqd[0] > nqd[1] ? nqd[0] : nqd[1];
    const uint32_t Pq = next_pow2(nqm > 0 ? nqm : 1);
    const uint64_t b1 = 4ull * 8 * Pq + 64;
    if (w == 0) {
        uint8_t* sc1 = warp_scratch(A, ctr, 0, b1);
        if (!sc1) warp_fail(R, ctr, kStatusScratchOverflow);
        if (lane == 0) s_sc = sc1;
    }
    __syncthreads();
    uint64_t* buf = reinterpret_cast<uint64_t*>(s_sc);
    __syncthreads();
    if (!buf) return;
    if (w < 2) {
        RescuePlan p{};
        rescue_prepare_dir(I, C, Qd, Pd, nqd, Pq, buf, (int)w, p);
        if (lane == 0) s_plan[w] = p;
    }
    __syncthreads();
    RescuePlan plan;
    plan.m[0] = s_plan[0].m[0];
    plan.m[1] = s_plan[1].m[1];
    plan.bound = s_plan[0].bound + s_plan[1].bound;
    plan.maxrun = s_plan[0].maxrun > s_plan[1].maxrun ? s_plan[0].maxrun : s_plan[1].maxrun;
    const bool notes = A.rescue_cycles && threadIdx.x == 0;
    uint64_t* note = A.rescue_cycles ? A.rescue_cycles + 8ull * t : nullptr;
    if (notes) {
        note[1] = (uint64_t)(clock64() - t0);
        note[4] = plan.bound;
        note[7] = plan.maxrun;
    }
    if (plan.bound == 0) {
        if (threadIdx.x == 0) {
            R.n_nams = 0;
            if (notes) note[0] = (uint64_t)(clock64() - t0);
        }
        __syncthreads();
        return;
    }
    const uint32_t H = (uint32_t)plan.bound;
    const uint64_t P2 = next_pow2(H);
    const bool big_run = plan.maxrun > kBlockHits;
    // open, closed and spare lists (H each) and the sort keys; big runs' hits after them
    const uint64_t b2 = 96ull * H + 32ull * P2 + (big_run ? 9ull * plan.maxrun + 64 : 0) + 256;
    if (w == 0) {
        uint8_t* sc2 = warp_scratch(A, ctr, (b1 + 255) & ~255ull, b2);
        if (!sc2) warp_fail(R, ctr, kStatusScratchOverflow);
        if (lane == 0) s_sc = sc2;
    }
    __syncthreads();
    uint8_t* sc2 = s_sc;
    __syncthreads();
    if (!sc2) return;
    NamLists L;
    L.open = reinterpret_cast<NamState*>(sc2);
    L.closed = L.open + H;
    NamKey* keys = reinterpret_cast<NamKey*>(L.closed + H);
    NamState* spare = reinterpret_cast<NamState*>(keys + P2);
    uint32_t* hrs = s_hpk;
    uint32_t* hpk = s_hpk + kBlockHits;
    uint8_t* tb = s_tb;
    if (big_run) {
        hrs = reinterpret_cast<uint32_t*>(spare + H);
        hpk = hrs + plan.maxrun;
        tb = reinterpret_cast<uint8_t*>(hpk + plan.maxrun);
    }
    L.n_open = L.n_closed = 0;
    L.cap = H;
    const long long t_merge = clock64();
    uint64_t walk_cycles = 0;
    const uint64_t* tk[2] = {buf + 2 * Pq, buf + 3 * Pq};
    for (int d = 0; d < 2; ++d) {
        for (uint32_t j = 0; j < plan.m[d]; ++j) {
            const uint32_t qi = (uint32_t)(tk[d][j] >> 32) & 0xFFFF;
            const uint32_t cnt = (uint32_t)tk[d][j];
            const Query q = Qd[d][qi];
            QueryHits Q;
            Q.rs = hrs;
            Q.packed = hpk;
            Q.qs = (int)q.start;
            Q.qe = (int)q.end;
            Q.dir = (uint32_t)d;
            Q.k = I.k;
            if (w == 0) {
                const long long tw = clock64();
                const uint32_t n = warp_walk_run_n(I, Q.qs, Q.qe, Pd[d][qi], cnt, hrs, hpk, plan.maxrun);
                walk_cycles += (uint64_t)(clock64() - tw);
                if (lane == 0) s_n = n;
            }
            __syncthreads();
            Q.n = s_n;
            block_close_merge_q(L, spare, Q, tb, s_hrs, s_bcnt, s_tot);
        }
        block_close_all(L);
    }
    if (notes) {
        note[2] = (uint64_t)(clock64() - t_merge);
        note[5] = L.n_closed;
        note[6] = walk_cycles;
    }
    if (w == 0 && !rescue_sort_job(A, ctr, R, L, keys, r, t)) {
        const long long t_fin = clock64();
        warp_finish_nams(C, L, s_hrs, s_hpk, R, A, ctr);
        if (notes) note[3] = (uint64_t)(clock64() - t_fin);
    }
    if (notes) note[0] = (uint64_t)(clock64() - t0);
    __syncthreads();
}

// find_nams_rescue for the reads on the rescue list.  With C.rescue_block_hits set and
// no more rescued reads than the grid has warps (a small batch, whose heavy reads
// would otherwise set the kernel's time while most warps idle), the heavy end of the
// list (reads whose estimated merge hits reach rescue_block_hits) is taken first, a
// block per read, then the rest a warp per read; otherwise every read a warp, heavy
// ones first.
__global__ void __launch_bounds__(32 * kWarpsPerBlock) k_rescue(IndexView I, MapConfig C, ReadRec* __restrict__ rec,
                                                                 Arenas A, Counters* ctr) {
    __shared__ __align__(16) uint32_t s_hrs[kWarpsPerBlock][kRescueSmemHits];
    __shared__ __align__(16) uint32_t s_hpk[kWarpsPerBlock][kRescueSmemHits];
    __shared__ uint8_t s_tb[kWarpsPerBlock][kRescueSmemHits];
    __shared__ uint32_t s_item;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    const uint32_t n_heavy = *(volatile unsigned int*)&ctr->n_rescue_heavy;
    const uint32_t n_rescue = n_heavy + *(volatile unsigned int*)&ctr->n_rescue;
    uint32_t first = 0;
    if (C.rescue_block_hits && n_rescue <= warp_count()) {
        for (;;) {
            if (threadIdx.x == 0) s_item = atomicAdd(&ctr->rescue_block_next, 1u);
            __syncthreads();
            const uint32_t t = s_item;
            __syncthreads();
            if (t >= n_heavy) break;
            rescue_read_block(I, C, rec, A, ctr, t, &s_hrs[0][0], &s_hpk[0][0], &s_tb[0][0]);
        }
        first = n_heavy;
    }
    // resident warps take reads in list order, heavy ones first
    for (;;) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(&ctr->rescue_next, 1u);
        t = __shfl_sync(0xFFFFFFFFu, t, 0) + first;
        if (t >= n_rescue) break;
        const long long t_start = clock64();
        const uint32_t r = t < n_heavy ? A.rescue_list[A.rescue_cap - 1 - t] : A.rescue_list[t - n_heavy];
        ReadRec& R = rec[r];
        struct CycleNote {
            const Arenas& A;
            uint32_t t;
            long long t0;
            __device__ ~CycleNote() {
                if (A.rescue_cycles && lane_id() == 0) A.rescue_cycles[8ull * t] = (uint64_t)(clock64() - t0);
            }
            __device__ void phase(int k, long long since) const {
                if (A.rescue_cycles && lane_id() == 0) A.rescue_cycles[8ull * t + k] = (uint64_t)(clock64() - since);
            }
            __device__ void set(int k, uint64_t v) const {
                if (A.rescue_cycles && lane_id() == 0) A.rescue_cycles[8ull * t + k] = v;
            }
        } note{A, t, t_start};
        const uint32_t nqd[2] = {R.nq, R.nq2 - R.nq};
        const Query* Qd[2] = {A.q + R.q_off, A.q + R.q_off + R.nq};
        const uint64_t* Pd[2] = {A.q_pos + R.q_off, A.q_pos + R.q_off + R.nq};
        const uint32_t nqm = nqd[0] > nqd[1] ? nqd[0] : nqd[1];
        const uint32_t Pq = next_pow2(nqm > 0 ? nqm : 1);
        const uint64_t b1 = 4ull * 8 * Pq + 64;
        uint8_t* sc1 = warp_scratch(A, ctr, 0, b1);
        if (!sc1) {
            warp_fail(R, ctr, kStatusScratchOverflow);
            continue;
        }
        uint64_t* buf = reinterpret_cast<uint64_t*>(sc1);
        const RescuePlan plan = rescue_prepare(I, C, Qd, Pd, nqd, Pq, buf);
        note.phase(1, t_start);
        note.set(4, plan.bound);
        note.set(7, plan.maxrun);
        if (plan.bound == 0) {
            if (lane == 0) R.n_nams = 0;
            continue;
        }
        const uint32_t H = (uint32_t)plan.bound;
        const uint64_t P2 = next_pow2(H);
        const bool big_run = plan.maxrun > kRescueSmemHits;
        const uint64_t b2 = 64ull * H + 32ull * P2 + (big_run ? 9ull * plan.maxrun + 64 : 0) + 256;
        uint8_t* sc2 = warp_scratch(A, ctr, (b1 + 255) & ~255ull, b2);
        if (!sc2) {
            warp_fail(R, ctr, kStatusScratchOverflow);
            continue;
        }
        NamLists L;
        L.open = reinterpret_cast<NamState*>(sc2);
        L.closed = L.open + H;
        NamKey* keys = reinterpret_cast<NamKey*>(L.closed + H);
        uint32_t* hrs = s_hrs[w];
        uint32_t* hpk = s_hpk[w];
        uint8_t* tb = s_tb[w];
        if (big_run) {
            hrs = reinterpret_cast<uint32_t*>(keys + P2);
            hpk = hrs + plan.maxrun;
            tb = reinterpret_cast<uint8_t*>(hpk + plan.maxrun);
        }
        L.n_open = L.n_closed = 0;
        L.cap = H;
        const long long t_merge = clock64();
        const uint64_t walk = rescue_merge(I, Qd, Pd, plan, buf, Pq, L, hrs, hpk, tb);
        note.phase(2, t_merge);
        note.set(6, walk);
        note.set(5, L.n_closed);
        if (rescue_sort_job(A, ctr, R, L, keys, r, t)) continue;
        const long long t_fin = clock64();
        static_assert(kWarpSortMax <= 256 && kRescueSmemHits >= 1024, "the sort entries fit the hit buffers");
        warp_finish_nams(C, L, s_hrs[w], s_hpk[w], R, A, ctr);
        note.phase(3, t_fin);
        __syncwarp();
    }
}

// Shared-memory tile of the block sort, one array per key field so that a warp's
// accesses are conflict-free and a compare usually reads only k1.
struct SortTile {
    uint64_t* k1;
    uint64_t* k2;
    uint64_t* k3;
    uint32_t* idx;
    __device__ NamKey get(uint32_t i) const {
        NamKey k;
        k.k1 = k1[i];
        k.k2 = k2[i];
        k.k3 = k3[i];
        k.idx = idx[i];
        k.pad = 0;
        return k;
    }
    __device__ void put(uint32_t i, const NamKey& k) {
        k1[i] = k.k1;
        k2[i] = k.k2;
        k3[i] = k.k3;
        idx[i] = k.idx;
    }
    // b < a, reading the secondary fields only when the first ones tie
    __device__ bool less_at(uint32_t b, uint32_t a) const {
        const uint64_t x = k1[b], y = k1[a];
        if (x != y) return x < y;
        const uint64_t x2 = k2[b], y2 = k2[a];
        if (x2 != y2) return x2 < y2;
        const uint64_t x3 = k3[b], y3 = k3[a];
        if (x3 != y3) return x3 < y3;
        return idx[b] < idx[a];
    }
    __device__ void swap(uint32_t i, uint32_t j) {
        const NamKey a = get(i), b = get(j);
        put(i, b);
        put(j, a);
    }
};


__device__ __forceinline__ void cmp_swap(NamKey* keys, uint32_t i, uint32_t j, uint32_t k) {
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

// Block bitonic sort of n keys (room for next_pow2(n) in global memory) by all
// threads of the block.  Every stage whose partner distance is below tcap runs on a
// shared-memory tile of tcap keys; only the stages with larger distances touch
// global memory.
__device__ void block_sort_keys(NamKey* keys, uint32_t n, SortTile tile, uint32_t tcap) {
    const uint32_t P = next_pow2(n);
    for (uint32_t i = n + threadIdx.x; i < P; i += blockDim.x) {
        NamKey k;
        k.k1 = k.k2 = k.k3 = ~0ULL;
        k.idx = 0xFFFFFFFFu;
        k.pad = 0;
        keys[i] = k;
    }
    __syncthreads();
    const uint32_t T = P < tcap ? P : tcap;
    // Runs all stages (k, j) with j < T inside each tile; k is the current merge size
    // (k <= T: the tile-local sort from scratch; k > T: finish merge level k).
    auto tile_pass = [&](uint32_t k_from, uint32_t k_to, uint32_t j_from) {
        for (uint32_t t0 = 0; t0 < P; t0 += T) {
            for (uint32_t i = threadIdx.x; i < T; i += blockDim.x) tile.put(i, keys[t0 + i]);
            __syncthreads();
            for (uint32_t k = k_from; k <= k_to; k <<= 1) {
                for (uint32_t j = (k == k_from ? j_from : k >> 1); j > 0; j >>= 1) {
                    // one compare per thread and pair: i is the lower index of the pair
                    for (uint32_t q = threadIdx.x; q < T / 2; q += blockDim.x) {
                        const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                        const uint32_t ixj = i | j;
                        const bool up = ((t0 + i) & k) == 0;   // direction uses the global index
                        if (tile.less_at(ixj, i) == up) tile.swap(i, ixj);
                    }
                    __syncthreads();
                }
            }
            for (uint32_t i = threadIdx.x; i < T; i += blockDim.x) keys[t0 + i] = tile.get(i);
            __syncthreads();
        }
    };
    tile_pass(2, T, 1);
    for (uint32_t k = 2 * T; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j >= T; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) cmp_swap(keys, i, j, k);
            __syncthreads();
        }
        tile_pass(k, k, T >> 1);
    }
}

// Shared-memory tile of the block sort that moves only the first key word and the
// NAM index: the other key words stay where they were loaded (indexed by NAM) and
// are read only when the first words tie.  A compare-exchange then moves 12 bytes
// instead of 28.
struct IdxSortTile {
    uint64_t* k1;    // first key word, moves with ix
    uint32_t* ix;    // NAM index, moves
    uint64_t* k2;    // second and third key words by NAM index (fixed)
    uint64_t* k3;
    __device__ bool less_at(uint32_t b, uint32_t a) const {
        const uint64_t x = k1[b], y = k1[a];
        if (x != y) return x < y;
        const uint32_t ib = ix[b], ia = ix[a];
        const uint64_t x2 = k2[ib], y2 = k2[ia];
        if (x2 != y2) return x2 < y2;
        const uint64_t x3 = k3[ib], y3 = k3[ia];
        if (x3 != y3) return x3 < y3;
        return ib < ia;
    }
    __device__ void swap(uint32_t i, uint32_t j) {
        const uint64_t a = k1[i];
        k1[i] = k1[j];
        k1[j] = a;
        const uint32_t b = ix[i];
        ix[i] = ix[j];
        ix[j] = b;
    }
};

// Bitonic sort of the P (a power of two) keys held in the tile.
__device__ void idx_tile_sort(IdxSortTile tile, uint32_t P) {
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t q = threadIdx.x; q < P / 2; q += blockDim.x) {
                const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                const uint32_t ixj = i | j;
                if (tile.less_at(ixj, i) == ((i & k) == 0)) tile.swap(i, ixj);
            }
            __syncthreads();
        }
    }
}

// Sorts the NAMs of the rescued reads with kWarpSortMax < NAMs <= kSortTile
// (typically reads inside short tandem repeats): one block per read, bitonic sort in
// a shared-memory tile, then the read's NAMs are written to the NAM arena in order.
// The jobs are at the front of the job list.
template <int kThreads, uint32_t kTile>
__global__ void __launch_bounds__(kThreads) k_sort_jobs(MapConfig C, ReadRec* __restrict__ rec, Arenas A,
                                                         Counters* ctr) {
    extern __shared__ __align__(16) uint8_t s_dyn[];   // kTile sort keys, one array per field
    __shared__ uint64_t s_noff;
    SortTile tile;
    tile.k1 = reinterpret_cast<uint64_t*>(s_dyn);
    tile.k2 = tile.k1 + kTile;
    tile.k3 = tile.k2 + kTile;
    tile.idx = reinterpret_cast<uint32_t*>(tile.k3 + kTile);
    IdxSortTile itile;   // the same shared memory, for jobs that fit it
    itile.k1 = tile.k1;
    itile.k2 = tile.k2;
    itile.k3 = tile.k3;
    itile.ix = tile.idx;
    const uint32_t n_jobs = *(volatile unsigned int*)&ctr->n_heavy;
    for (uint32_t h = blockIdx.x; h < n_jobs; h += gridDim.x) {
        const long long t0 = clock64();
        const SortJob job = A.sort_jobs[h];
        ReadRec& R = rec[job.read];
        const NamState* closed = job.closed;
        const uint32_t NN = job.n;
        const uint32_t P = next_pow2(NN);
        const bool in_tile = P <= kTile;
        if (in_tile) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                NamKey k;
                if (i < NN) {
                    k = nam_key(closed[i], i, C.sort_mode);
                } else {   // padding sorts last (a NAM's first key word is never all ones)
                    k.k1 = k.k2 = k.k3 = ~0ULL;
                }
                itile.k1[i] = k.k1;
                itile.ix[i] = i;
                itile.k2[i] = k.k2;
                itile.k3[i] = k.k3;
            }
            __syncthreads();
            idx_tile_sort(itile, P);
        } else {
            for (uint32_t i = threadIdx.x; i < NN; i += blockDim.x) job.keys[i] = nam_key(closed[i], i, C.sort_mode);
            __syncthreads();
            block_sort_keys(job.keys, NN, tile, kTile);
        }
        if (threadIdx.x == 0) {
            const uint64_t noff = atomicAdd(&ctr->nam_used, (unsigned long long)NN);
            if (noff + NN > A.nam_cap) {
                R.flags |= kReadFailed;
                R.n_nams = 0;   // the rescue kernel set the count ahead of the sort
                atomicOr(&ctr->status, kStatusNamOverflow);
                s_noff = ~0ULL;
            } else {
                R.nam_off = noff;
                R.n_nams = NN;
                s_noff = noff;
            }
        }
        __syncthreads();
        const uint64_t noff = s_noff;
        if (noff != ~0ULL)
            for (uint32_t i = threadIdx.x; i < NN; i += blockDim.x)
                A.nams[noff + i] = closed[in_tile ? tile.idx[i] : job.keys[i].idx];
        __syncthreads();
        if (A.rescue_cycles && threadIdx.x == 0) A.rescue_cycles[8ull * job.note + 3] = (uint64_t)(clock64() - t0);
    }
}

// ---- cluster sort of the rescued reads with more than kSortTile NAMs ------------------
//
// A cluster of kClusterCtas CTAs sorts one read's keys: each CTA holds T = P /
// kClusterCtas of the P (next power of two) keys in its shared-memory tile, so up to
// kClusterCtas * kSortTile keys are sorted without touching global memory.  Bitonic
// stages whose partner distance is below T stay within a CTA (block barrier); the
// few with larger distances compare and swap across the CTAs' tiles through
// distributed shared memory (cluster barrier).  Each CTA needs only kSortTile keys of
// shared memory, so the clusters run beside the NAM kernels of the other stream.
constexpr int kClusterCtas = 8;

// Tie break of the index-moving cluster sort: NAM indices ib and ia whose first key
// words are equal, by their second and third words (fixed, NAM e in CTA e / T at e % T)
// and then the index.
__device__ __forceinline__ bool cluster_tie_less(uint32_t ib, uint32_t ia, uint64_t* k2, uint64_t* k3, uint32_t T) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const uint64_t b2 = *cl.map_shared_rank(k2 + ib % T, ib / T), a2 = *cl.map_shared_rank(k2 + ia % T, ia / T);
    if (b2 != a2) return b2 < a2;
    const uint64_t b3 = *cl.map_shared_rank(k3 + ib % T, ib / T), a3 = *cl.map_shared_rank(k3 + ia % T, ia / T);
    if (b3 != a3) return b3 < a3;
    return ib < ia;
}

__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(256)
    k_sort_jobs_cluster(MapConfig C, ReadRec* __restrict__ rec, Arenas A, Counters* ctr) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) uint8_t s_dyn[];   // kSortTile keys, one array per field
    __shared__ uint64_t s_noff;
    cg::cluster_group cl = cg::this_cluster();
    const uint32_t rank = cl.block_rank();
    SortTile tile;
    tile.k1 = reinterpret_cast<uint64_t*>(s_dyn);
    tile.k2 = tile.k1 + kSortTile;
    tile.k3 = tile.k2 + kSortTile;
    tile.idx = reinterpret_cast<uint32_t*>(tile.k3 + kSortTile);
    const uint32_t n_jobs = *(volatile unsigned int*)&ctr->n_huge;
    const uint32_t n_clusters = gridDim.x / kClusterCtas;
    for (uint32_t h = blockIdx.x / kClusterCtas; h < n_jobs; h += n_clusters) {
        const long long t0 = clock64();
        const SortJob job = A.sort_jobs[A.jobs_cap - 1 - h];
        const NamState* closed = job.closed;
        const uint32_t NN = job.n;
        const uint32_t P = next_pow2(NN);
        const bool in_tiles = P <= kClusterCtas * kSortTile;
        if (in_tiles) {
            // Each CTA's tile moves only the first key word (k1) and the NAM index (idx) of
            // its T positions; the second and third words stay where they were loaded,
            // by NAM index, and are read (possibly from another CTA) only on ties.
            const uint32_t T = P / kClusterCtas;   // NN > kSortTile: T >= kSortTile / 4
            const uint32_t e0 = rank * T;
            for (uint32_t i = threadIdx.x; i < T; i += blockDim.x) {
                const uint32_t e = e0 + i;
                NamKey k;
                if (e < NN) {
                    k = nam_key(closed[e], e, C.sort_mode);
                } else {   // padding sorts last (a NAM's first key word is never all ones)
                    k.k1 = k.k2 = k.k3 = ~0ULL;
                }
                tile.k1[i] = k.k1;
                tile.idx[i] = e;
                tile.k2[i] = k.k2;
                tile.k3[i] = k.k3;
            }
            cl.sync();
            for (uint32_t k = 2; k <= P; k <<= 1) {
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    if (j < T) {
                        for (uint32_t q = threadIdx.x; q < T / 2; q += blockDim.x) {
                            const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                            const uint32_t ixj = i | j;
                            const uint64_t xb = tile.k1[ixj], xa = tile.k1[i];
                            const bool less =
                                xb != xa ? xb < xa : cluster_tie_less(tile.idx[ixj], tile.idx[i], tile.k2, tile.k3, T);
                            if (less == (((e0 + i) & k) == 0)) {
                                tile.k1[i] = xb;
                                tile.k1[ixj] = xa;
                                const uint32_t t = tile.idx[i];
                                tile.idx[i] = tile.idx[ixj];
                                tile.idx[ixj] = t;
                            }
                        }
                        if (j > 1) __syncthreads();
                        else cl.sync();   // the next stage may cross CTAs
                    } else {
                        // pairs (i, i | j) across CTAs; this CTA takes an equal share
                        for (uint32_t q = rank * (T / 2) + threadIdx.x; q < (rank + 1) * (T / 2); q += blockDim.x) {
                            const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                            const uint32_t ixj = i | j;
                            uint64_t* pa = cl.map_shared_rank(tile.k1 + i % T, i / T);
                            uint64_t* pb = cl.map_shared_rank(tile.k1 + ixj % T, ixj / T);
                            uint32_t* qa = cl.map_shared_rank(tile.idx + i % T, i / T);
                            uint32_t* qb = cl.map_shared_rank(tile.idx + ixj % T, ixj / T);
                            const uint64_t xa = *pa, xb = *pb;
                            const bool less = xb != xa ? xb < xa : cluster_tie_less(*qb, *qa, tile.k2, tile.k3, T);
                            if (less == ((i & k) == 0)) {
                                *pa = xb;
                                *pb = xa;
                                const uint32_t t = *qa;
                                *qa = *qb;
                                *qb = t;
                            }
                        }
                        cl.sync();
                    }
                }
            }
        }
        if (rank == 0) {
            if (!in_tiles) {
                // beyond the cluster's tiles (rare): the first CTA sorts through global memory
                for (uint32_t i = threadIdx.x; i < NN; i += blockDim.x)
                    job.keys[i] = nam_key(closed[i], i, C.sort_mode);
                __syncthreads();
                block_sort_keys(job.keys, NN, tile, kSortTile);
            }
            if (threadIdx.x == 0) {
                ReadRec& R = rec[job.read];
                const uint64_t noff = atomicAdd(&ctr->nam_used, (unsigned long long)NN);
                if (noff + NN > A.nam_cap) {
                    R.flags |= kReadFailed;
                    R.n_nams = 0;   // the rescue kernel set the count ahead of the sort
                    atomicOr(&ctr->status, kStatusNamOverflow);
                    s_noff = ~0ULL;
                } else {
                    R.nam_off = noff;
                    R.n_nams = NN;
                    s_noff = noff;
                }
            }
        }
        cl.sync();
        const uint64_t noff = *cl.map_shared_rank(&s_noff, 0u);
        if (noff != ~0ULL) {
            if (in_tiles) {
                const uint32_t T = P / kClusterCtas, e0 = rank * T;
                for (uint32_t i = threadIdx.x; i < T && e0 + i < NN; i += blockDim.x)
                    A.nams[noff + e0 + i] = closed[tile.idx[i]];
            } else if (rank == 0) {
                for (uint32_t i = threadIdx.x; i < NN; i += blockDim.x) A.nams[noff + i] = closed[job.keys[i].idx];
            }
        }
        if (A.rescue_cycles && rank == 0 && threadIdx.x == 0)
            A.rescue_cycles[8ull * job.note + 3] = (uint64_t)(clock64() - t0);
        cl.sync();   // tiles and s_noff are reused by the next job
    }
}

// Records at or beyond out_cap are not written (the caller sized out from an estimate
// and gathers again when the total turns out larger).
// mode 0: every read; 1: the reads that were not rescued (fractions and rescue flags
// of every read), while the rescued reads' sorts may still run; 2: the rescued reads
// (through the rescue list), after their sorts.
__global__ void k_gather_nams(uint32_t n, const ReadRec* __restrict__ rec, const NamState* __restrict__ arena,
                              const uint64_t* __restrict__ out_off, gbsa_nam* __restrict__ out, uint64_t out_cap,
                              float* frac, uint8_t* rescued, int mode, Arenas A, const Counters* ctr,
                              const BatchDesc* desc) {
    const uint32_t lane = lane_id();
    uint64_t* copy_off = nullptr;
    if (desc) {
        const uint32_t cap = n;
        n = min(n, desc->n_reads);
        out = desc->out;
        out_cap = desc->out_cap;
        frac = mode == 2 ? nullptr : desc->frac;
        rescued = mode == 2 ? nullptr : desc->rescued;
        if (mode != 2) {
            copy_off = desc->out_off;
            // slots past the batch hold no NAMs: out_off[cap] is the batch's total
            if (blockIdx.x == 0 && threadIdx.x == 0) copy_off[n] = out_off[cap];
        }
    }
    if (mode == 2) {
        const uint32_t n_light = ctr->n_rescue, n_heavy = ctr->n_rescue_heavy;
        for (uint32_t t = warp_global_id(); t < n_light + n_heavy; t += warp_count()) {
            const uint32_t r = t < n_light ? A.rescue_list[t] : A.rescue_list[A.rescue_cap - 1 - (t - n_light)];
            const ReadRec R = rec[r];
            const uint64_t o = out_off[r];
            for (uint32_t j = lane; j < R.n_nams; j += 32)
                if (o + j < out_cap) to_gbsa_nam(arena[R.nam_off + j], (int)j, out[o + j]);
        }
        return;
    }
    for (uint32_t r = warp_global_id(); r < n; r += warp_count()) {
        const ReadRec R = rec[r];
        const uint64_t o = out_off[r];
        const bool skip = mode == 1 && (R.flags & kReadRescue);
        for (uint32_t j = lane; j < (skip ? 0u : R.n_nams); j += 32)
            if (o + j < out_cap) to_gbsa_nam(arena[R.nam_off + j], (int)j, out[o + j]);
        if (lane == 0) {
            if (frac) frac[r] = R.frac;
            if (rescued) rescued[r] = (R.flags & kReadRescue) ? 1 : 0;
            if (copy_off) copy_off[r] = o;
        }
    }
}

__global__ void k_gather_queries(uint32_t n, const ReadRec* __restrict__ rec, const Query* __restrict__ arena,
                                 const uint64_t* __restrict__ out_off, gbsa_query_randstrobe* __restrict__ out) {
    const uint32_t lane = lane_id();
    for (uint32_t r = warp_global_id(); r < n; r += warp_count()) {
        const ReadRec R = rec[r];
        const uint64_t o = out_off[r];
        for (uint32_t j = lane; j < R.nq2; j += 32) {
            const Query q = arena[R.q_off + j];
            gbsa_query_randstrobe x;
            x.hash = q.hash;
            x.start = q.start;
            x.end = q.end;
            x.is_reverse = j >= R.nq ? 1 : 0;
            for (int b = 0; b < 7; ++b) x._pad[b] = 0;
            out[o + j] = x;
        }
    }
}

__global__ void k_read_counts(uint32_t n, const ReadRec* __restrict__ rec, int what, uint64_t* __restrict__ out,
                              const BatchDesc* desc) {
    const uint32_t live = desc ? min(n, desc->n_reads) : n;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        out[r] = r >= live ? 0 : (what == 0 ? rec[r].n_nams : (uint64_t)rec[r].nq2);
}

__global__ void k_clear_recs(uint32_t cap, ReadRec* __restrict__ rec, const BatchDesc* desc) {
    const uint32_t n = min(cap, desc->n_reads);
    unsigned long long* w = reinterpret_cast<unsigned long long*>(rec);
    static_assert(sizeof(ReadRec) % 8 == 0, "ReadRec is a whole number of 8-byte words");
    const uint64_t words = (uint64_t)n * (sizeof(ReadRec) / 8);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < words; i += (uint64_t)gridDim.x * blockDim.x)
        w[i] = 0ull;
}

__global__ void k_reset_recs(uint32_t n, ReadRec* __restrict__ rec) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        ReadRec& R = rec[r];
        R.flags = 0;
        R.hit_off = 0;
        R.n_hits = 0;
        R.frac = 0.0f;
        R.nam_off = 0;
        R.n_nams = 0;
        R.n_found = 0;
    }
}

__global__ void k_find(IndexView I, const uint64_t* __restrict__ h, uint64_t n, uint64_t* __restrict__ pos) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        pos[i] = index_find(I, h[i]);
}

__global__ void k_get_count(IndexView I, const uint64_t* __restrict__ p, uint64_t n, uint32_t* __restrict__ c) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        c[i] = p[i] < I.n ? index_get_count(I, p[i]) : 0;
}

unsigned warp_grid(uint64_t items, int warps_per_block) {
    const int sms = device_sm_count();
    const uint64_t want = (items + warps_per_block - 1) / warps_per_block;
    const uint64_t cap = (uint64_t)sms * 16;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, cap));
}

}  // namespace

uint32_t nam_kernel_warps(uint32_t n_reads) { return warp_grid(n_reads, kWarpsPerBlock) * kWarpsPerBlock; }

// Launches a kernel that probes the index, with the mapper's L2 access-policy window
// (the bucket table held persisting in L2) as a launch attribute, so that only these
// launches carry it and the caller's stream keeps its own attributes.
template <class... Exp, class... Act>
static void launch_probe(void (*kernel)(Exp...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                         const MapConfig& C, Act&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (C.l2_bytes) {
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = const_cast<void*>(C.l2_base);
        attr[0].val.accessPolicyWindow.num_bytes = C.l2_bytes;
        attr[0].val.accessPolicyWindow.hitRatio = C.l2_hit_ratio;
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    GBSA_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Act>(args)...));
}

void launch_seed(const DevParams& P, const uint8_t* seqs, const uint64_t* offs, const uint32_t* lens, uint32_t n,
                 ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st) {
    if (!n) return;
    k_seed_smem<<<warp_grid(n, kSeedWarps), 32 * kSeedWarps, 0, st>>>(P, seqs, offs, lens, n, rec, A, ctr);
    GBSA_LAUNCHED();
}

void launch_seed_long(const DevParams& P, const uint8_t* seqs, const uint64_t* offs, const uint32_t* lens,
                      ReadRec* rec, Arenas A, Counters* ctr, uint8_t* long_scratch, uint32_t long_warps,
                      cudaStream_t st, const BatchDesc* desc) {
    const unsigned blocks = std::max(1u, long_warps / kWarpsPerBlock);
    k_seed_long<<<blocks, 32 * kWarpsPerBlock, 0, st>>>(P, seqs, offs, lens, rec, A, ctr, long_scratch, desc);
    GBSA_LAUNCHED();
}

// Shapes of the batched form's seeding + lookup kernel (the autotuner's choices).
// Variant 0 is the plain form's fused kernel shape.
SeedVariant seed_variant(int v) {
    static const SeedVariant table[kSeedVariants] = {
        {8, 6, 512, 160}, {8, 5, 512, 160}, {4, 12, 512, 160}, {8, 7, 256, 96}, {16, 3, 512, 160}, {8, 6, 256, 96},
    };
    return table[v < 0 || v >= kSeedVariants ? 0 : v];
}

template <bool kCount, bool kLookup, int kWarps, int kBlocks, uint32_t kMaxLen, uint32_t kSyncmers>
static void launch_q(const DevParams& P, const IndexView& I, const MapConfig& C, const BatchDesc* desc, ReadRec* rec,
                     Arenas A, Counters* ctr, cudaStream_t st) {
    const unsigned grid = (unsigned)device_sm_count() * kBlocks;
    launch_probe(k_seed_lookup_q<kCount, kLookup, kWarps, kBlocks, kMaxLen, kSyncmers>, grid, 32 * kWarps, 0, st, C,
                 P, I, C, desc, rec, A, ctr);
}

template <bool kCount, bool kLookup>
static void launch_q_variant(int v, const DevParams& P, const IndexView& I, const MapConfig& C, const BatchDesc* desc,
                             ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st) {
    switch (v) {
        case 1: launch_q<kCount, kLookup, 8, 5, 512, 160>(P, I, C, desc, rec, A, ctr, st); break;
        case 2: launch_q<kCount, kLookup, 4, 12, 512, 160>(P, I, C, desc, rec, A, ctr, st); break;
        case 3: launch_q<kCount, kLookup, 8, 7, 256, 96>(P, I, C, desc, rec, A, ctr, st); break;
        case 4: launch_q<kCount, kLookup, 16, 3, 512, 160>(P, I, C, desc, rec, A, ctr, st); break;
        case 5: launch_q<kCount, kLookup, 8, 6, 256, 96>(P, I, C, desc, rec, A, ctr, st); break;
        default: launch_q<kCount, kLookup, 8, 6, 512, 160>(P, I, C, desc, rec, A, ctr, st); break;
    }
}

void launch_seed_lookup_queue(const DevParams& P, const IndexView& I, const MapConfig& C, const BatchDesc* desc,
                              ReadRec* rec, Arenas A, Counters* ctr, int variant, bool lookup, cudaStream_t st) {
    if (!lookup) launch_q_variant<false, false>(variant, P, I, C, desc, rec, A, ctr, st);
    else if (C.count_bytes) launch_q_variant<true, true>(variant, P, I, C, desc, rec, A, ctr, st);
    else launch_q_variant<false, true>(variant, P, I, C, desc, rec, A, ctr, st);
    GBSA_LAUNCHED();
}

void launch_seed_lookup(const DevParams& P, const IndexView& I, const MapConfig& C, const uint8_t* seqs,
                        const uint64_t* offs, const uint32_t* lens, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                        cudaStream_t st) {
    if (!n) return;
    // resident blocks only: the warps pull reads from the work counter until none is left
    const unsigned grid = std::min<unsigned>(warp_grid(n, kSeedWarps), (unsigned)device_sm_count() * kFusedBlocksPerSm);
    launch_probe(C.count_bytes ? k_seed_lookup<true> : k_seed_lookup<false>, grid, 32 * kSeedWarps, 0, st, C, P, I, C,
                 seqs, offs, lens, n, rec, A, ctr);
    GBSA_LAUNCHED();
}

void launch_lookup_long(const IndexView& I, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                        cudaStream_t st) {
    if (!n) return;
    // sized for n long reads (every read, for long-read parameter sets); warps beyond
    // the long-list count exit at once
    const unsigned blocks = warp_grid(n, kWarpsPerBlock);
    launch_probe(C.count_bytes ? k_lookup_long<true> : k_lookup_long<false>, blocks, 32 * kWarpsPerBlock, 0, st, C, I,
                 C, rec, A, ctr);
    GBSA_LAUNCHED();
}

void launch_lookup(const IndexView& I, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                   cudaStream_t st, const BatchDesc* desc) {
    if (!n) return;
    launch_probe(C.count_bytes ? k_lookup<true> : k_lookup<false>, warp_grid(n, kWarpsPerBlock), 32 * kWarpsPerBlock, 0,
                 st, C, I, C, n, rec, A, ctr, desc);
    GBSA_LAUNCHED();
}

// The NAM phase's kernels (lane and warp merges, rescue, NAM gather) run beside each
// other and need most of an SM's shared memory together (rescue 73 KB + lane merge
// 3 x 40 KB): they ask for the largest shared-memory carveout, so that the SM keeps that
// configuration through the phase instead of switching it as each kernel's blocks
// arrive (left to the driver, the lane merge took 5.0 instead of 3.3 ms on the C2 batch
// inside the batch graph).  The seeding + lookup kernels keep the default: they use the
// rest of the unified L1 to cache index entries.  Set once per device.
void nam_phase_carveout() {
    static std::mutex mu;
    static std::vector<char> done;
    int dev = 0;
    GBSA_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (done[dev]) return;
    const void* fs[] = {(const void*)k_nams_lane<0>, (const void*)k_nams_lane<6>, (const void*)k_nams_lane<8>,
                        (const void*)k_nams_lane_r<3, kLaneOpen>, (const void*)k_nams_lane_r<4, kLaneOpen>,
                        (const void*)k_nams_lane_r<5, 6>, (const void*)k_nams_lane_r<3, 6>,
                        (const void*)k_nams<kHeavyBlocksPerSm>, (const void*)k_nams<6>, (const void*)k_nams<8>,
                        (const void*)k_rescue, (const void*)k_gather_nams};
    for (const void* f : fs)
        GBSA_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
    done[dev] = 1;
}

void launch_nams(const IndexView&, const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr,
                 cudaStream_t st) {
    if (!n) return;
    nam_phase_carveout();
    if (C.lane_variant >= 3) {
        // 3: three blocks per SM at 168 registers (the SM's registers: the rescue kernel
        // starts as they retire); 4: two blocks per SM at 128 registers, beside the
        // rescue kernel's block; 5: six slots, three blocks per SM at 96 registers, beside it
        // 6: six slots at 124 registers, two blocks per SM beside the rescue kernel's block
        const unsigned per_sm = C.lane_variant == 4 || C.lane_variant == 6 ? 2u : 3u;
        const unsigned blocks = grid_for(n, 32 * kLaneWarps, (unsigned)device_sm_count() * per_sm);
        if (C.lane_variant == 4) k_nams_lane_r<4, kLaneOpen><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr);
        else if (C.lane_variant == 5) k_nams_lane_r<5, 6><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr);
        else if (C.lane_variant == 6) k_nams_lane_r<3, 6><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr);
        else k_nams_lane_r<3, kLaneOpen><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr);
        GBSA_LAUNCHED();
        return;
    }
    const unsigned blocks = grid_for(n, 32 * kLaneWarps, (unsigned)device_sm_count() * kLaneBlocksPerSm);
    switch (C.lane_variant) {
        case 1: k_nams_lane<6><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr); break;
        case 2: k_nams_lane<8><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr); break;
        default: k_nams_lane<0><<<blocks, 32 * kLaneWarps, 0, st>>>(C, n, rec, A, ctr); break;
    }
    GBSA_LAUNCHED();
}

void launch_bucket_reads(uint32_t n, uint32_t lane_max_hits, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st,
                         const BatchDesc* desc) {
    if (!n) return;
    const uint32_t lane_max = lane_max_hits == 0 ? kLaneMaxHits : std::min(lane_max_hits, kLaneMaxHits);
    k_bucket_reads<<<grid_for(n, 256, (unsigned)device_sm_count() * 8), 256, 0, st>>>(n, lane_max, rec, A, ctr,
                                                                                      desc);
    GBSA_LAUNCHED();
}

void launch_nams_warp(const MapConfig& C, uint32_t n, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st) {
    if (!n) return;
    // at most nam_kernel_warps(n) warps: one scratch slot each.  Variants 3 and 4 launch
    // 4 blocks per SM (96 / 80 registers), leaving registers for the rescued reads' sorts
    // beside them.
    const unsigned per_sm = C.warp_variant >= 3 ? 4u : (unsigned)kHeavyGridPerSm;
    const unsigned blocks = (unsigned)std::min<uint64_t>((uint64_t)device_sm_count() * per_sm,
                                                         (n + kHeavyWarps - 1) / kHeavyWarps);
    switch (C.warp_variant) {
        case 1: case 4: k_nams<6><<<blocks, 32 * kHeavyWarps, 0, st>>>(C, rec, A, ctr); break;
        case 2: k_nams<8><<<blocks, 32 * kHeavyWarps, 0, st>>>(C, rec, A, ctr); break;
        default: k_nams<kHeavyBlocksPerSm><<<blocks, 32 * kHeavyWarps, 0, st>>>(C, rec, A, ctr); break;
    }
    GBSA_LAUNCHED();
}

void launch_rescue(const IndexView& I, const MapConfig& C, uint32_t n_reads, ReadRec* rec, Arenas A, Counters* ctr,
                   cudaStream_t st) {
    if (!n_reads) return;
    nam_phase_carveout();
    // persistent, kRescueBlocksPerSm per SM (at most one scratch slot per warp)
    const unsigned blocks =
        std::min<unsigned>(warp_grid(n_reads, kWarpsPerBlock), (unsigned)device_sm_count() * kRescueBlocksPerSm);
    launch_probe(k_rescue, blocks, 32 * kWarpsPerBlock, 0, st, C, I, C, rec, A, ctr);
    GBSA_LAUNCHED();
}

void launch_sort_jobs(const MapConfig& C, ReadRec* rec, Arenas A, Counters* ctr, cudaStream_t st) {
    constexpr int kSmall = 256;
    constexpr size_t smem = kSortTile * 28;
    {
        // the kernels' dynamic shared-memory limit, set once per device (mappers may
        // launch from several threads at once)
        static std::mutex mu;
        static std::vector<char> done;
        int dev = 0;
        GBSA_CUDA(cudaGetDevice(&dev));
        std::lock_guard<std::mutex> g(mu);
        if ((int)done.size() <= dev) done.resize(dev + 1, 0);
        if (!done[dev]) {
            GBSA_CUDA(cudaFuncSetAttribute(k_sort_jobs<kSmall, kSortTile>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            GBSA_CUDA(cudaFuncSetAttribute(k_sort_jobs<2 * kSmall, kSortTile>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            GBSA_CUDA(cudaFuncSetAttribute(k_sort_jobs_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
            done[dev] = 1;
        }
    }
    const unsigned sms = (unsigned)device_sm_count();
    if (C.sort_variant == 1) k_sort_jobs<2 * kSmall, kSortTile><<<sms * 3, 2 * kSmall, smem, st>>>(C, rec, A, ctr);
    else k_sort_jobs<kSmall, kSortTile><<<sms * 4, kSmall, smem, st>>>(C, rec, A, ctr);
    GBSA_LAUNCHED();
    // sms / 2 clusters of kClusterCtas CTAs
    k_sort_jobs_cluster<<<std::max(1u, sms / 2) * kClusterCtas, 256, smem, st>>>(C, rec, A, ctr);
    GBSA_LAUNCHED();
}

void launch_gather_nams(uint32_t n, const ReadRec* rec, const NamState* arena, const uint64_t* out_off,
                        gbsa_nam* out, float* frac, uint8_t* rescued, cudaStream_t st, uint64_t out_cap, int mode,
                        const Arenas* A, const Counters* ctr, const BatchDesc* desc) {
    if (!n) return;
    const Arenas none{};
    k_gather_nams<<<warp_grid(n, kWarpsPerBlock), 32 * kWarpsPerBlock, 0, st>>>(
        n, rec, arena, out_off, out, out_cap, frac, rescued, mode, A ? *A : none, ctr, desc);
    GBSA_LAUNCHED();
}

void launch_gather_queries(uint32_t n, const ReadRec* rec, const Query* arena, const uint64_t* out_off,
                           gbsa_query_randstrobe* out, cudaStream_t st) {
    if (!n) return;
    k_gather_queries<<<warp_grid(n, kWarpsPerBlock), 32 * kWarpsPerBlock, 0, st>>>(n, rec, arena, out_off, out);
    GBSA_LAUNCHED();
}

void launch_find(const IndexView& I, const uint64_t* hashes, uint64_t n, uint64_t* pos, cudaStream_t st) {
    if (!n) return;
    k_find<<<grid_for(n, 256, 1u << 20), 256, 0, st>>>(I, hashes, n, pos);
    GBSA_LAUNCHED();
}

void launch_get_count(const IndexView& I, const uint64_t* pos, uint64_t n, uint32_t* counts, cudaStream_t st) {
    if (!n) return;
    k_get_count<<<grid_for(n, 256, 1u << 20), 256, 0, st>>>(I, pos, n, counts);
    GBSA_LAUNCHED();
}

void launch_reset_recs(uint32_t n, ReadRec* rec, cudaStream_t st) {
    if (!n) return;
    k_reset_recs<<<grid_for(n, 256, 1u << 16), 256, 0, st>>>(n, rec);
    GBSA_LAUNCHED();
}

void launch_clear_recs(uint32_t cap, ReadRec* rec, const BatchDesc* desc, cudaStream_t st) {
    if (!cap) return;
    k_clear_recs<<<(unsigned)device_sm_count() * 4, 256, 0, st>>>(cap, rec, desc);
    GBSA_LAUNCHED();
}

__global__ void k_offsets_add(const uint64_t* __restrict__ in, uint64_t* __restrict__ out, uint64_t n, uint64_t base) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i] + base;
}

void launch_offsets_add(const uint64_t* in, uint64_t* out, uint64_t n, uint64_t base, cudaStream_t st) {
    if (!n) return;
    k_offsets_add<<<grid_for(n, 256, 4096), 256, 0, st>>>(in, out, n, base);
    GBSA_LAUNCHED();
}

void launch_read_counts(uint32_t n, const ReadRec* rec, int what, uint64_t* out, cudaStream_t st,
                        const BatchDesc* desc) {
    if (!n) return;
    k_read_counts<<<grid_for(n, 256, 1u << 16), 256, 0, st>>>(n, rec, what, out, desc);
    GBSA_LAUNCHED();
}

}  // namespace gbsa
