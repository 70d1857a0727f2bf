// pairs.cu — read-pair classification and NAM-pair scoring after the NAM sort.
//
// Restates gpu_pre_cal_type (step2/main.cu:3552-3580) with top_dropoff
// (main.cu:889-898) and is_proper_nam_pair (main.cu:870-887): one thread per pair
// reads the two ends' NAM counts and their first NAMs (the first two for the
// dropoff) and writes one type byte.  The bound mu + 10 sigma is computed as one
// fused multiply-add, as nvcc contracts the reference's expression.
#include <cmath>

#include "prims.cuh"
#include "runtime.h"

namespace gbsa {
namespace {

__device__ __forceinline__ float top_dropoff(const gbsa_nam* nams, uint64_t n) {
    const int h0 = nams[0].n_hits;
    if (h0 <= 2) return 1.0f;
    if (n > 1) return __fdiv_rn((float)nams[1].n_hits, (float)h0);
    return 0.0f;
}

__device__ __forceinline__ bool is_proper_nam_pair(const gbsa_nam& n1, const gbsa_nam& n2, float limit) {
    if (n1.ref_id != n2.ref_id || n1.is_rc == n2.is_rc) return false;
    const int a = max(0, n1.ref_start - n1.query_start);
    const int b = max(0, n2.ref_start - n2.query_start);
    const bool r1_r2 = n2.is_rc && (a <= b) && ((float)(b - a) < limit);
    const bool r2_r1 = n1.is_rc && (b <= a) && ((float)(a - b) < limit);
    return r1_r2 || r2_r1;
}

__global__ void k_classify_pairs(const gbsa_nam* __restrict__ nams, const uint64_t* __restrict__ offs,
                                 uint32_t n_pairs, int layout, float threshold, float limit,
                                 uint8_t* __restrict__ types) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_pairs; i += gridDim.x * blockDim.x) {
        const uint64_t r1 = layout == GBSA_PAIRS_HALVES ? i : 2ull * i;
        const uint64_t r2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)i + n_pairs : 2ull * i + 1;
        const uint64_t o1 = offs[r1], c1 = offs[r1 + 1] - o1;
        const uint64_t o2 = offs[r2], c2 = offs[r2 + 1] - o2;
        uint8_t t;
        if (c1 == 0 && c2 == 0) t = 0;
        else if (c2 == 0) t = 1;
        else if (c1 == 0) t = 2;
        else if (top_dropoff(nams + o1, c1) < threshold && top_dropoff(nams + o2, c2) < threshold &&
                 is_proper_nam_pair(nams[o1], nams[o2], limit))
            t = 3;
        else t = 4;
        types[i] = t;
    }
}

// ---- NAM-pair scoring (get_best_scoring_nam_pairs_sort3, step2/main.cu:1475-1716) ----
//
// A thread per read pair (the work per pair is a few hundred steps; pairs with both
// ends mapped are independent).  Its top-40 heap lives in registers / local memory,
// its per-NAM "in a pair" flags, its candidate list and the explicit stack of the
// final quicksort in scratch indexed by the pair's NAM offsets.

struct NamPairHeap {
    gbsa_nam_pair h[GBSA_NAM_PAIRS_TOP_K];
    int size;
    // maintain_top_k (main.cu:1464-1473): a min-heap on score; sift-up stops at a
    // parent of score <= the child's, sift-down takes the strictly smaller child (the
    // left one on a tie)
    __device__ void add(const gbsa_nam_pair& p) {
        if (size < GBSA_NAM_PAIRS_TOP_K) {
            int i = size++;
            h[i] = p;
            while (i > 0) {
                const int up = (i - 1) / 2;
                if (h[up].score <= h[i].score) break;
                const gbsa_nam_pair t = h[up];
                h[up] = h[i];
                h[i] = t;
                i = up;
            }
        } else if (p.score > h[0].score) {
            h[0] = p;
            int i = 0;
            while (2 * i + 1 < size) {
                int sm = i;
                const int l = 2 * i + 1, r = l + 1;
                if (l < size && h[l].score < h[sm].score) sm = l;
                if (r < size && h[r].score < h[sm].score) sm = r;
                if (sm == i) break;
                const gbsa_nam_pair t = h[i];
                h[i] = h[sm];
                h[sm] = t;
                i = sm;
            }
        }
    }
};

__device__ __forceinline__ int nam_diagonal(const gbsa_nam& n) { return max(0, n.ref_start - n.query_start); }

// The final sort's comparator (main.cu:1674-1713); an absent end is an all-zero NAM
// with ref_start -1.
__device__ bool nam_pair_before(const gbsa_nam_pair& a, const gbsa_nam_pair& b, const gbsa_nam* n1,
                                const gbsa_nam* n2) {
    gbsa_nam none;
    none.nam_id = none.query_start = none.query_end = none.query_prev_hit_startpos = 0;
    none.ref_end = none.ref_prev_hit_startpos = none.n_hits = none.ref_id = 0;
    none.ref_start = -1;
    none.score = 0.0f;
    none.is_rc = 0;
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

// One strand combination of the pairing, one reference id at a time (ids below
// 3000, main.cu:1520-1570 and 1573-1623).  fwd1: mate 1 on the forward strand, mate 2's
// diagonal in [d1, d1 + span); else mate 2's diagonal in (d1 - span, d1].
__device__ void pair_pass(const gbsa_nam* n1, int b1, int e1, const gbsa_nam* n2, int b2, int e2, bool fwd1,
                          int span, NamPairHeap& heap, uint8_t* add1, uint8_t* add2, int& best) {
    int p1 = b1, p2 = b2;
    for (int ref = 0; ref < 3000; ++ref) {
        while (p1 < e1 && n1[p1].ref_id < ref) ++p1;
        while (p2 < e2 && n2[p2].ref_id < ref) ++p2;
        int q1 = p1, q2 = p2;
        while (q1 < e1 && n1[q1].ref_id == ref) ++q1;
        while (q2 < e2 && n2[q2].ref_id == ref) ++q2;
        if (p1 == e1 || p2 == e2) break;
        int best2 = -1;
        for (int j = p2; j < q2; ++j) best2 = max(best2, n2[j].n_hits);
        for (int i = p1; i < q1; ++i) {
            const int round_best = n1[i].n_hits + best2;
            if (round_best < best / 2) break;
            if (heap.size == GBSA_NAM_PAIRS_TOP_K && round_best < heap.h[0].score) break;
            const int d1 = nam_diagonal(n1[i]);
            int lo = p2, hi = q2 - 1, at = q2;   // first mate-2 NAM inside the window
            while (lo <= hi) {
                const int mid = (lo + hi) / 2;
                const bool in = fwd1 ? nam_diagonal(n2[mid]) >= d1 : nam_diagonal(n2[mid]) > d1 - span;
                if (in) {
                    at = mid;
                    hi = mid - 1;
                } else {
                    lo = mid + 1;
                }
            }
            for (int j = at; j < q2; ++j) {
                const int d2 = nam_diagonal(n2[j]);
                if (fwd1 ? d2 >= d1 + span : d2 > d1) break;
                const int joint = n1[i].n_hits + n2[j].n_hits;
                if (joint < best / 2) continue;
                gbsa_nam_pair np;
                np.score = joint;
                np.i1 = i;
                np.i2 = j;
                heap.add(np);
                add1[i] = 1;
                add2[j] = 1;
                best = max(best, joint);
            }
        }
    }
}

__global__ void k_nam_pairs(const gbsa_nam* __restrict__ nams, const uint64_t* __restrict__ offs, uint32_t n_pairs,
                            int layout, int span, uint32_t max_tries, uint8_t* flags, gbsa_nam_pair* lists,
                            int* stacks, gbsa_nam_pair* __restrict__ out, uint32_t* __restrict__ counts) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_pairs; p += gridDim.x * blockDim.x) {
        const uint64_t r1 = layout == GBSA_PAIRS_HALVES ? p : 2ull * p;
        const uint64_t r2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)p + n_pairs : 2ull * p + 1;
        const int c1 = (int)(offs[r1 + 1] - offs[r1]), c2 = (int)(offs[r2 + 1] - offs[r2]);
        if (c1 == 0 || c2 == 0) {
            counts[p] = 0;
            continue;
        }
        const gbsa_nam* n1 = nams + offs[r1];
        const gbsa_nam* n2 = nams + offs[r2];
        uint8_t* add1 = flags + offs[r1];
        uint8_t* add2 = flags + offs[r2];
        for (int i = 0; i < c1; ++i) add1[i] = 0;
        for (int i = 0; i < c2; ++i) add2[i] = 0;
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
        NamPairHeap heap;
        heap.size = 0;
        int best = 0;
        pair_pass(n1, 0, mid1, n2, mid2, c2, true, span, heap, add1, add2, best);
        pair_pass(n1, mid1, c1, n2, 0, mid2, false, span, heap, add1, add2, best);
        // the pair's list: room for its mate-1 NAMs and the heap
        const uint64_t base = offs[r1] + (uint64_t)GBSA_NAM_PAIRS_TOP_K * p;
        gbsa_nam_pair* list = lists + base;
        int len = 0;
        int best1 = best;
        if (best1 == 0)
            for (int i = 0; i < c1; ++i) best1 = max(best1, n1[i].n_hits);
        int run = 0, prev = n1[0].ref_id + 3000 * n1[0].is_rc;
        for (int i = 0; i < c1; ++i) {   // mate-1 NAMs in no pair, max_tries per (reference, strand)
            const int key = n1[i].ref_id + 3000 * n1[i].is_rc;
            if (key == prev) {
                ++run;
            } else {
                run = 1;
                prev = key;
            }
            if (run > (int)max_tries) continue;
            if (n1[i].n_hits < best1 / 2 || add1[i]) continue;
            gbsa_nam_pair np;
            np.score = n1[i].n_hits;
            np.i1 = i;
            np.i2 = -1;
            list[len++] = np;
        }
        int best2 = best;
        if (best2 == 0)
            for (int i = 0; i < c2; ++i) best2 = max(best2, n2[i].n_hits);
        for (int i = 0; i < c2; ++i) {   // mate-2 NAMs in no pair, through the heap
            if (n2[i].n_hits < best2 / 2 || add2[i]) continue;
            gbsa_nam_pair np;
            np.score = n2[i].n_hits;
            np.i1 = -1;
            np.i2 = i;
            heap.add(np);
        }
        for (int i = 0; i < heap.size; ++i) list[len++] = heap.h[i];
        // quick_sort_iterative (main.cu:317-358): Lomuto partition around the last
        // element, ranges on an explicit stack (left part pushed first)
        if (len > 1) {
            int* st = stacks + 2 * base;
            int top = -1;
            st[++top] = 0;
            st[++top] = len - 1;
            while (top >= 0) {
                const int hi = st[top--];
                const int lo = st[top--];
                const gbsa_nam_pair pivot = list[hi];
                int i = lo - 1;
                for (int j = lo; j < hi; ++j)
                    if (nam_pair_before(list[j], pivot, n1, n2)) {
                        ++i;
                        const gbsa_nam_pair t = list[i];
                        list[i] = list[j];
                        list[j] = t;
                    }
                const gbsa_nam_pair t = list[i + 1];
                list[i + 1] = list[hi];
                list[hi] = t;
                const int pv = i + 1;
                if (pv - 1 > lo) {
                    st[++top] = lo;
                    st[++top] = pv - 1;
                }
                if (pv + 1 < hi) {
                    st[++top] = pv + 1;
                    st[++top] = hi;
                }
            }
        }
        const uint32_t k = min((uint32_t)len, max_tries);
        for (uint32_t i = 0; i < k; ++i) out[(uint64_t)p * max_tries + i] = list[i];
        counts[p] = k;
    }
}

}  // namespace
}  // namespace gbsa

using namespace gbsa;

extern "C" int gbsa_nam_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs,
                                     int layout, float mu, float sigma, uint32_t max_tries, gbsa_nam_pair* d_pairs,
                                     uint32_t* d_counts, void* stream) {
    try {
        if (layout != GBSA_PAIRS_INTERLEAVED && layout != GBSA_PAIRS_HALVES)
            throw Error(GBSA_ERR_PARAM, "layout must be GBSA_PAIRS_INTERLEAVED or GBSA_PAIRS_HALVES");
        if (max_tries == 0) throw Error(GBSA_ERR_PARAM, "max_tries must be at least 1");
        if (n_pairs == 0) return GBSA_OK;
        cudaStream_t st = (cudaStream_t)stream;
        // scratch: a flag per NAM, and per pair a list and a quicksort stack with room
        // for its mate-1 NAMs plus the heap
        uint64_t total = 0;
        GBSA_CUDA(cudaMemcpyAsync(&total, d_nam_offsets + 2ull * n_pairs, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        const uint64_t slots = total + (uint64_t)GBSA_NAM_PAIRS_TOP_K * n_pairs + 1;
        // scratch in stream order (cudaMalloc / cudaFree would wait for the whole device,
        // other callers' work included)
        const size_t b_flags = (total + 1 + 255) & ~size_t(255);
        const size_t b_lists = (sizeof(gbsa_nam_pair) * slots + 255) & ~size_t(255);
        uint8_t* scratch = nullptr;
        GBSA_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), b_flags + b_lists + 8 * slots, st));
        const int span = (int)mu + 10 * (int)sigma;
        k_nam_pairs<<<grid_for(n_pairs, 128, (unsigned)device_sm_count() * 16), 128, 0, st>>>(
            d_nams, d_nam_offsets, n_pairs, layout, span, max_tries, scratch,
            reinterpret_cast<gbsa_nam_pair*>(scratch + b_flags), reinterpret_cast<int*>(scratch + b_flags + b_lists),
            d_pairs, d_counts);
        const cudaError_t launch = cudaGetLastError();
        GBSA_CUDA(cudaFreeAsync(scratch, st));
        GBSA_CUDA(launch);
        GBSA_LAUNCHED();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

extern "C" int gbsa_classify_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs,
                                          int layout, float dropoff_threshold, float mu, float sigma,
                                          uint8_t* d_types, void* stream) {
    try {
        if (layout != GBSA_PAIRS_INTERLEAVED && layout != GBSA_PAIRS_HALVES)
            throw Error(GBSA_ERR_PARAM, "layout must be GBSA_PAIRS_INTERLEAVED or GBSA_PAIRS_HALVES");
        if (n_pairs == 0) return GBSA_OK;
        const float limit = std::fma(10.0f, sigma, mu);
        k_classify_pairs<<<grid_for(n_pairs, 256, (unsigned)device_sm_count() * 8), 256, 0, (cudaStream_t)stream>>>(
            d_nams, d_nam_offsets, n_pairs, layout, dropoff_threshold, limit, d_types);
        GBSA_LAUNCHED();
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

// ---- alignment orchestration (align_PE_part0..4, step2/main.cu:1857-2165) ---------------
//
// A thread per read pair lists, in the order the reference's align_PE_part<type> runs
// them, the seed extensions (extend_seed_part after reverse_nam_if_needed) and mate
// rescues (rescue_mate_part of a NAM after reverse_nam_if_needed) of the pair, and
// computes the pair's mapq for type 3 (get_mapq, main.cu:900-910).  Two passes: the
// first counts each pair's steps, an exclusive scan places them, the second writes them.

namespace gbsa {
namespace {

__device__ __forceinline__ void plan_push(gbsa_align_step* out, uint32_t& k, bool write, uint32_t pair, uint8_t kind,
                                          bool is_read1, uint64_t read, uint64_t nam_read, uint32_t nam) {
    if (write) {
        gbsa_align_step s;
        s.pair = pair;
        s.read = (uint32_t)read;
        s.nam_read = (uint32_t)nam_read;
        s.nam = nam;
        s.kind = kind;
        s.is_read1 = is_read1 ? 1 : 0;
        s._pad[0] = s._pad[1] = 0;
        out[k] = s;
    }
    ++k;
}

// get_mapq (main.cu:900-910): the reference's float expression — min_matches is a float
// rounded from the double n_hits / 10.0 (capped at 1), the log is logf of the float
// score, the products are float in the reference's order — truncated to int, capped at
// 60 and returned as uint8 (a negative value wraps, as the reference's return type makes
// it).
__device__ __forceinline__ uint8_t pair_mapq(const gbsa_nam* nams, uint64_t n) {
    if (n <= 1) return 60;
    const float s1 = nams[0].score, s2 = nams[1].score;
    const double mm = nams[0].n_hits / 10.0;
    const float min_matches = (float)(mm < 1.0 ? mm : 1.0);
    const float f = __fmul_rn(__fmul_rn(__fmul_rn(40.0f, __fsub_rn(1.0f, __fdiv_rn(s2, s1))), min_matches), logf(s1));
    const int uncapped = (int)f;
    return (uint8_t)(uncapped < 60 ? uncapped : 60);
}

// rescue_read_part (main.cu:795-835): the NAMs of the mapped end in order while fewer than
// max_tries were tried and n_hits / the first NAM's n_hits >= dropoff; each is extended on
// its read, then its mate is rescued from it.
__device__ void plan_rescue_read(gbsa_align_step* out, uint32_t& k, bool write, uint32_t p, const gbsa_nam* nams,
                                 uint64_t n, uint64_t mapped, uint64_t mate, bool mapped_is_read1, uint32_t max_tries,
                                 float dropoff) {
    const int top = nams[0].n_hits;
    uint32_t tries = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const float d = (float)nams[i].n_hits / (float)top;
        if (tries >= max_tries || d < dropoff) break;
        plan_push(out, k, write, p, GBSA_STEP_EXTEND, mapped_is_read1, mapped, mapped, (uint32_t)i);
        plan_push(out, k, write, p, GBSA_STEP_RESCUE, !mapped_is_read1, mate, mapped, (uint32_t)i);
        ++tries;
    }
}

template <bool kWrite>
__global__ void k_plan_pairs(const gbsa_nam* __restrict__ nams, const uint64_t* __restrict__ offs, uint32_t n_pairs,
                             int layout, const uint8_t* __restrict__ types, const gbsa_nam_pair* __restrict__ jp,
                             const uint32_t* __restrict__ jcounts, uint32_t max_tries, float dropoff,
                             uint64_t* __restrict__ counts, gbsa_pair_plan* __restrict__ plans,
                             gbsa_align_step* __restrict__ steps, uint64_t step_cap, uint8_t* scratch,
                             unsigned int* bad) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_pairs; p += gridDim.x * blockDim.x) {
        const uint64_t e1 = layout == GBSA_PAIRS_HALVES ? p : 2ull * p;
        const uint64_t e2 = layout == GBSA_PAIRS_HALVES ? (uint64_t)p + n_pairs : 2ull * p + 1;
        const uint64_t o1 = offs[e1], c1 = offs[e1 + 1] - o1;
        const uint64_t o2 = offs[e2], c2 = offs[e2 + 1] - o2;
        const gbsa_nam* n1 = nams + o1;
        const gbsa_nam* n2 = nams + o2;
        const uint8_t type = types[p];
        uint64_t first = 0;
        gbsa_align_step* out = steps;
        bool write = false;
        if (kWrite) {
            first = counts[p];
            write = first + (counts[p + 1] - first) <= step_cap;
            out = steps + first;
        }
        uint32_t k = 0;
        gbsa_pair_plan plan;
        plan.type = type;
        plan.mapq1 = plan.mapq2 = 0;
        plan._pad = 0;
        plan.type4_loop_size = 0;
        if (type == 1 && c1 > 0) {
            plan_rescue_read(out, k, write, p, n1, c1, e1, e2, true, max_tries, dropoff);
        } else if (type == 2 && c2 > 0) {
            plan_rescue_read(out, k, write, p, n2, c2, e2, e1, false, max_tries, dropoff);
        } else if (type == 3 && c1 > 0 && c2 > 0) {
            plan_push(out, k, write, p, GBSA_STEP_EXTEND, true, e1, e1, 0);
            plan_push(out, k, write, p, GBSA_STEP_EXTEND, false, e2, e2, 0);
            plan.mapq1 = pair_mapq(n1, c1);
            plan.mapq2 = pair_mapq(n2, c2);
        } else if (type == 4 && c1 > 0 && c2 > 0) {
            // per-NAM "aligned" flags in scratch indexed by the NAM's position in the batch
            uint8_t* al1 = scratch + o1;
            uint8_t* al2 = scratch + o2;
            for (uint64_t i = 0; i < c1; ++i) al1[i] = 0;
            for (uint64_t i = 0; i < c2; ++i) al2[i] = 0;
            // the best-scoring NAM of each end first (the first of equal maxima)
            uint32_t b1 = 0, b2 = 0;
            for (uint32_t i = 0; i < c1; ++i)
                if (n1[i].score > n1[b1].score) b1 = i;
            for (uint32_t i = 0; i < c2; ++i)
                if (n2[i].score > n2[b2].score) b2 = i;
            plan_push(out, k, write, p, GBSA_STEP_EXTEND, true, e1, e1, b1);
            al1[b1] = 1;
            plan_push(out, k, write, p, GBSA_STEP_EXTEND, false, e2, e2, b2);
            al2[b2] = 1;
            const uint32_t nj = jcounts[p];
            const gbsa_nam_pair* J = jp + (uint64_t)p * max_tries;
            const double max_score = nj ? (double)J[0].score : 0.0;
            uint32_t high = 0;
            int loop = 0;
            for (uint32_t i = 0; i < nj; ++i) {
                const float d = (float)((double)J[i].score / max_score);
                if (high >= max_tries || d < dropoff) break;
                ++loop;
                const int i1 = J[i].i1, i2 = J[i].i2;
                if (i1 >= 0 && (uint64_t)i1 < c1) {
                    if (!al1[i1]) {
                        plan_push(out, k, write, p, GBSA_STEP_EXTEND, true, e1, e1, (uint32_t)i1);
                        al1[i1] = 1;
                    }
                } else if (i2 >= 0 && (uint64_t)i2 < c2) {
                    plan_push(out, k, write, p, GBSA_STEP_RESCUE, true, e1, e2, (uint32_t)i2);
                } else if (bad) {
                    atomicAdd(bad, 1u);   // a pair entry with neither NAM: not produced by the pair scoring
                }
                if (i2 >= 0 && (uint64_t)i2 < c2) {
                    if (!al2[i2]) {
                        plan_push(out, k, write, p, GBSA_STEP_EXTEND, false, e2, e2, (uint32_t)i2);
                        al2[i2] = 1;
                    }
                } else if (i1 >= 0 && (uint64_t)i1 < c1) {
                    plan_push(out, k, write, p, GBSA_STEP_RESCUE, false, e2, e1, (uint32_t)i1);
                }
                ++high;
            }
            plan.type4_loop_size = loop;
        }
        if (!kWrite) {
            counts[p] = k;
        } else {
            plan.first_step = (uint32_t)first;
            plan.n_steps = k;
            plans[p] = plan;
        }
    }
}

}  // namespace
}  // namespace gbsa

using namespace gbsa;

extern "C" int gbsa_plan_pairs_device(const gbsa_nam* d_nams, const uint64_t* d_nam_offsets, uint32_t n_pairs,
                                      int layout, const uint8_t* d_types, const gbsa_nam_pair* d_pairs,
                                      const uint32_t* d_pair_counts, uint32_t max_tries, float dropoff,
                                      gbsa_pair_plan* d_plans, gbsa_align_step* d_steps, uint64_t step_capacity,
                                      uint64_t* n_steps, void* stream) {
    try {
        if (layout != GBSA_PAIRS_INTERLEAVED && layout != GBSA_PAIRS_HALVES)
            throw Error(GBSA_ERR_PARAM, "layout must be GBSA_PAIRS_INTERLEAVED or GBSA_PAIRS_HALVES");
        if (max_tries == 0) throw Error(GBSA_ERR_PARAM, "max_tries must be at least 1");
        if (n_steps) *n_steps = 0;
        if (n_pairs == 0) return GBSA_OK;
        cudaStream_t st = (cudaStream_t)stream;
        uint64_t total_nams = 0;
        GBSA_CUDA(cudaMemcpyAsync(&total_nams, d_nam_offsets + 2ull * n_pairs, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        // scratch in stream order: step counts (then offsets) per pair, an "aligned" flag
        // per NAM, the status word, the scan's partials
        const size_t b_cnt = (8ull * (n_pairs + 1) + 255) & ~size_t(255);
        const size_t b_flags = (total_nams + 1 + 255) & ~size_t(255);
        uint8_t* scratch = nullptr;
        GBSA_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), b_cnt + b_flags + 256, st));
        uint64_t* counts = reinterpret_cast<uint64_t*>(scratch);
        uint8_t* flags = scratch + b_cnt;
        unsigned int* bad = reinterpret_cast<unsigned int*>(scratch + b_cnt + b_flags);
        struct Free {
            uint8_t* p;
            cudaStream_t s;
            ~Free() { cudaFreeAsync(p, s); }
        } release{scratch, st};
        GBSA_CUDA(cudaMemsetAsync(bad, 0, 4, st));
        const unsigned grid = grid_for(n_pairs, 128, (unsigned)device_sm_count() * 16);
        k_plan_pairs<false><<<grid, 128, 0, st>>>(d_nams, d_nam_offsets, n_pairs, layout, d_types, d_pairs, d_pair_counts,
                                                   max_tries, dropoff, counts, nullptr, nullptr, 0, flags, nullptr);
        GBSA_LAUNCHED();
        Workspace ws;
        scan_exclusive_u64(counts, counts, n_pairs, counts + n_pairs, ws, st);
        k_plan_pairs<true><<<grid, 128, 0, st>>>(d_nams, d_nam_offsets, n_pairs, layout, d_types, d_pairs, d_pair_counts,
                                                  max_tries, dropoff, counts, d_plans, d_steps, step_capacity, flags,
                                                  bad);
        GBSA_LAUNCHED();
        uint64_t total = 0;
        unsigned int h_bad = 0;
        GBSA_CUDA(cudaMemcpyAsync(&total, counts + n_pairs, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaMemcpyAsync(&h_bad, bad, 4, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));   // the scan's workspace is freed on return
        if (n_steps) *n_steps = total;
        if (h_bad) throw Error(GBSA_ERR_PARAM, "a NAM pair with neither NAM");
        if (total > step_capacity) throw Error(GBSA_ERR_CAPACITY, "step capacity too small");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}
