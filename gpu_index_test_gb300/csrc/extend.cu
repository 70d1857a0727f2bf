// extend.cu — seed extension of NAMs, the first step of the reference's alignment
// kernels (align_PE_part1..4, step2/main.cu:1876-2165): reverse_nam_if_needed
// (main.cu:759-793), then extend_seed_part (main.cu:582-643) with my_hamming_align
// (main.cu:506-580).
//
// A thread per NAM; the kernel is bound by the latency of its byte loads (random
// reference windows, and reads walked a byte at a time), so the loads are issued in
// independent groups: the k-mer checks have no early exit, and the scan loads 8 bases of
// both sequences before it scans them (8 measured faster than 4 or 16: more loads in
// flight against more registers, fewer warps; 1.65 ms for 2M NAMs against 1.94 ms for
// one base at a time; staging the warp's sequences in shared memory was slower), and the
// grid is one wave of resident blocks (1.55 ms).  The
// NAM's two k-mer checks come first.  Then one pass over the read and its projected
// reference window counts the Hamming distance and runs the best-segment scan together;
// the reference runs the scan only when the distance admits the ungapped path, and its
// result is kept only then.  The reference's distance loop stops once the count exceeds
// the limit, so its count is min(mismatches, limit + 1).  The mismatches inside the best
// segment come from the running mismatch count at the segment's two ends, so the read is
// walked once.
#include "runtime.h"

namespace gbsa {
namespace {

// revcomp_table (step2/main.cu:1832-1849): A/C/G/T/U in either case to the upper-case
// complement, every other byte to 'N'.  c & 0xDF equals one of these letters only for
// that letter in either case.  (The reference indexes its table with a signed char, so
// bytes of 128 and above read outside it; here they give 'N'.)
__device__ __forceinline__ uint8_t revcomp_base(uint8_t c) {
    switch (c & 0xDF) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T':
        case 'U': return 'A';
        default: return 'N';
    }
}

// The read in one orientation: the reverse complement is read backwards through the
// table, as the reference's rc copy (main.cu:1893-1900).
struct ReadView {
    const uint8_t* fwd;
    int L;
    bool rc;
    __device__ __forceinline__ uint8_t at(int j) const {
        return rc ? revcomp_base(__ldg(fwd + (L - 1 - j))) : __ldg(fwd + j);
    }
};

// No early exit, so that the k loads are independent and in flight together.
__device__ __forceinline__ bool kmer_equal(const uint8_t* ref, const ReadView& q, int qpos, int k) {
    bool eq = true;
#pragma unroll 8
    for (int t = 0; t < k; ++t) eq &= __ldg(ref + t) == q.at(qpos + t);
    return eq;
}

constexpr int kScanBlock = 8;   // bases of the read and the window loaded before they are scanned

__global__ void __launch_bounds__(128)
    k_extend_seeds(const uint8_t* __restrict__ ref_seqs, const uint64_t* __restrict__ ref_offs,
                   const uint64_t* __restrict__ ref_lens, uint32_t n_refs, const uint8_t* __restrict__ read_seqs,
                   const uint64_t* __restrict__ read_offs, const uint32_t* __restrict__ read_lens, uint32_t n_reads,
                   const gbsa_nam* __restrict__ nams, const uint32_t* __restrict__ nam_reads, uint64_t n, int k,
                   gbsa_align_params ap, gbsa_seed_alignment* __restrict__ out, unsigned int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        gbsa_nam nam = nams[i];
        gbsa_seed_alignment o;
        o.ref_id = o.ref_start = o.edit_distance = o.global_ed = o.score = o.length = 0;
        o.query_start = o.query_end = 0;
        o.is_rc = o.done = o.consistent = o._pad = 0;
        const uint32_t r = nam_reads[i];
        bool ok = r < n_reads && nam.ref_id >= 0 && (uint32_t)nam.ref_id < n_refs;
        int L = 0, rlen = 0;
        if (ok) {
            L = (int)read_lens[r];
            rlen = (int)ref_lens[nam.ref_id];
            // every k-mer the checks compare then lies inside its sequence
            ok = nam.query_start >= 0 && nam.query_end <= L && nam.query_end - nam.query_start >= k &&
                 nam.ref_start >= 0 && nam.ref_end <= rlen && nam.ref_end - nam.ref_start >= k;
        }
        if (!ok) {
            atomicAdd(bad, 1u);
            out[i] = o;
            continue;
        }
        const uint8_t* fwd = read_seqs + read_offs[r];
        const uint8_t* ref = ref_seqs + ref_offs[nam.ref_id];
        // reverse_nam_if_needed (step2/main.cu:759-793)
        bool consistent = kmer_equal(ref + nam.ref_start, ReadView{fwd, L, nam.is_rc != 0}, nam.query_start, k) &&
                          kmer_equal(ref + nam.ref_end - k, ReadView{fwd, L, nam.is_rc != 0}, nam.query_end - k, k);
        if (!consistent) {
            const int qs2 = L - nam.query_end, qe2 = L - nam.query_start;
            const ReadView other{fwd, L, nam.is_rc == 0};
            if (kmer_equal(ref + nam.ref_start, other, qs2, k) && kmer_equal(ref + nam.ref_end - k, other, qe2 - k, k)) {
                nam.is_rc = nam.is_rc ? 0 : 1;
                nam.query_start = qs2;
                nam.query_end = qe2;
                consistent = true;
            }
        }
        o.ref_id = nam.ref_id;
        o.query_start = nam.query_start;
        o.query_end = nam.query_end;
        o.is_rc = nam.is_rc;
        o.consistent = consistent ? 1 : 0;
        // extend_seed_part (step2/main.cu:582-643)
        const int pstart = max(0, nam.ref_start - nam.query_start);
        const int pend = min(nam.ref_end + L - nam.query_end, rlen);
        if (pend - pstart == L && consistent) {
            const ReadView q{fwd, L, nam.is_rc != 0};
            const uint8_t* segm = ref + pstart;
            const int limit_error = (int)(L * 0.05);
            int total_mm = 0;
            // my_hamming_align's scan (main.cu:518-538), with the mismatch count at the
            // current segment start (cm_start) and at the best segment's ends
            int start = 0, score = ap.end_bonus, best_start = 0, best_end = 0, best_score = 0;
            int cm_start = 0, best_cm_start = 0, best_cm_end = 0;
            // kScanBlock bases of both sequences are loaded at once (independent loads in
            // flight together), then scanned
            for (int j0 = 0; j0 < L; j0 += kScanBlock) {
                uint8_t qb[kScanBlock], sb[kScanBlock];
#pragma unroll
                for (int t = 0; t < kScanBlock; ++t) {
                    const bool in = j0 + t < L;
                    qb[t] = in ? q.at(j0 + t) : 0;
                    sb[t] = in ? __ldg(segm + j0 + t) : 0;
                }
#pragma unroll
                for (int t = 0; t < kScanBlock; ++t) {
                    const int j = j0 + t;
                    if (j >= L) break;
                    const bool mm = qb[t] != sb[t];
                    total_mm += mm ? 1 : 0;
                    score += mm ? -ap.mismatch : ap.match;
                    if (score < 0) {
                        start = j + 1;
                        score = 0;
                        cm_start = total_mm;
                    }
                    if (score > best_score) {
                        best_start = start;
                        best_score = score;
                        best_end = j + 1;
                        best_cm_start = cm_start;
                        best_cm_end = total_mm;
                    }
                }
            }
            if (score + ap.end_bonus > best_score) {
                best_score = score + ap.end_bonus;
                best_end = L;
                best_start = start;
                best_cm_start = cm_start;
                best_cm_end = total_mm;
            }
            const int hamming_dist = min(total_mm, limit_error + 1);
            if (hamming_dist >= 0 && ((float)hamming_dist / L) < 0.05) {
                o.done = 1;
                o.edit_distance = best_cm_end - best_cm_start;
                o.global_ed = o.edit_distance + best_start + (L - best_end);
                o.score = best_score;
                o.ref_start = pstart + best_start;
                o.length = best_end - best_start;
            }
        }
        out[i] = o;
    }
}

// ---- mate rescue (rescue_mate_part with has_shared_substring) --------------------------

// nt2int_mod8 (step2/main.cu:645-654) as nibbles of one word: the 2-bit code of a byte
// from its value mod 8.
__device__ __forceinline__ uint32_t code_mod8(uint8_t base) { return (0x20031000u >> ((base & 7) * 4)) & 0xFu; }

constexpr int kMaxMateSubstrings = 64;   // sampled substrings of a mate (the reference keeps 50)
constexpr int kRescueWarps = 8;

// Hash of the sub bases at s (2 bits per base into 32 bits, as the reference's loop: a
// substring of more than 16 bases keeps its last 16); rc: s is the end of a read walked
// backwards through the complement table.
__device__ __forceinline__ uint32_t substring_hash(const uint8_t* s, int sub, bool rc) {
    uint32_t h = 0;
    for (int j = 0; j < sub; ++j) h = (h << 2) | code_mod8(rc ? revcomp_base(__ldg(s - j)) : __ldg(s + j));
    return h;
}

// A warp per NAM: the window where the mate lies (float arithmetic as the reference's:
// the int offset converted to float, mu + 5 sigma as one fused multiply-add, truncation
// back to int), then has_shared_substring (step2/main.cu:657-693).  The lanes hash the
// mate's 2k/3-base substrings at multiples of k/3 into the warp's shared list, then take
// the window's substring positions 32 at a time (consecutive positions, so the loads
// coalesce) and compare each one's hash with the whole list (every lane reads the same
// entry: a broadcast); the scan ends at the first group with a match, which gives the
// reference's answer (a match at any position).  Both position sets stop one substring
// short of the end, as the reference's loops.  Bound by the latency of the window's
// loads and the list compares: 2M NAMs in about 8.5 ms (a thread per NAM with the list in
// a per-thread array took 7.9 ms, its local arrays missing L1 on nearly every access;
// with the list in shared memory 11 ms; unrolled hash and compare loops 9.4 ms).
__global__ void __launch_bounds__(32 * kRescueWarps)
    k_rescue_mates(const uint8_t* __restrict__ ref_seqs, const uint64_t* __restrict__ ref_offs,
                   const uint64_t* __restrict__ ref_lens, uint32_t n_refs, const uint8_t* __restrict__ read_seqs,
                   const uint64_t* __restrict__ read_offs, const uint32_t* __restrict__ read_lens, uint32_t n_reads,
                   const gbsa_nam* __restrict__ nams, const uint32_t* __restrict__ mate_reads, uint64_t n, int k,
                   float mu, float sigma, gbsa_mate_rescue* __restrict__ out, unsigned int* bad) {
    __shared__ uint32_t s_list[kRescueWarps][kMaxMateSubstrings];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t* list = s_list[w];
    const int sub = 2 * k / 3, step = k / 3;
    const float spread = __fmaf_rn(5.0f, sigma, mu);
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t i = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const gbsa_nam nam = nams[i];
        const uint32_t r = mate_reads[i];
        gbsa_mate_rescue o;
        o.ref_id = o.window_start = o.window_end = o.edit_distance = 0;
        o.is_rc = o.done = o.is_unaligned = o._pad = 0;
        bool ok = r < n_reads && nam.ref_id >= 0 && (uint32_t)nam.ref_id < n_refs;
        const int L = ok ? (int)read_lens[r] : 0;
        const int n_sub = L > sub ? (L - sub + step - 1) / step : 0;   // p = 0, step, ... with p + sub < L
        if (n_sub > kMaxMateSubstrings) ok = false;
        if (!ok) {
            if (lane == 0) {
                atomicAdd(bad, 1u);
                out[i] = o;
            }
            continue;
        }
        const uint8_t* fwd = read_seqs + read_offs[r];
        // rescue_mate_part (step2/main.cu:695-757)
        const bool mate_fwd = nam.is_rc != 0;   // the mate in the orientation opposite to the NAM
        int a, b;
        if (mate_fwd) {
            a = __float2int_rz(__fsub_rn(__int2float_rn(nam.ref_start - nam.query_start), spread));
            b = nam.ref_start - nam.query_start + L / 2;
        } else {
            a = nam.ref_end + (L - nam.query_end) - L / 2;
            b = __float2int_rz(__fadd_rn(__int2float_rn(nam.ref_end + (L - nam.query_end)), spread));
        }
        const int ref_len = (int)ref_lens[nam.ref_id];
        const int ws = max(0, min(a, ref_len));
        const int we = min(ref_len, max(0, b));
        bool shared = false;
        if (we >= ws + k) {
            for (int t = (int)lane; t < n_sub; t += 32) {
                const int q = t * step;   // the mate's substring [q, q + sub) in its orientation
                list[t] = mate_fwd ? substring_hash(fwd + q, sub, false) : substring_hash(fwd + (L - 1 - q), sub, true);
            }
            __syncwarp();
            const uint8_t* win = ref_seqs + ref_offs[nam.ref_id] + ws;
            const int n_pos = we - ws - sub;   // positions p with p + sub < window length
            for (int base = 0; base < n_pos && !shared; base += 32) {
                const int p = base + (int)lane;
                bool hit = false;
                if (p < n_pos) {
                    const uint32_t h = substring_hash(win + p, sub, false);
                    for (int e = 0; e < n_sub; ++e) hit |= list[e] == h;
                }
                shared = __any_sync(0xFFFFFFFFu, hit);
            }
            __syncwarp();   // the next NAM rewrites the list
        }
        if (lane == 0) {
            o.ref_id = nam.ref_id;
            o.window_start = ws;
            o.window_end = we;
            o.is_rc = nam.is_rc;
            if (!shared) {
                o.done = 1;
                o.is_unaligned = 1;
                o.edit_distance = L;
            }
            out[i] = o;
        }
    }
}

}  // namespace
}  // namespace gbsa

using namespace gbsa;

extern "C" int gbsa_extend_seeds_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                                        const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                                        const uint64_t* d_read_offsets, const uint32_t* d_read_lengths,
                                        uint32_t n_reads, const gbsa_nam* d_nams, const uint32_t* d_nam_reads,
                                        uint64_t n_nams, int k, const gbsa_align_params* params,
                                        gbsa_seed_alignment* d_out, void* stream) {
    try {
        if (!params) throw Error(GBSA_ERR_PARAM, "params must not be null");
        if (k < 1) throw Error(GBSA_ERR_PARAM, "k must be at least 1");
        if (n_nams == 0) return GBSA_OK;
        cudaStream_t st = (cudaStream_t)stream;
        // the status word is allocated in stream order: a cudaFree would wait for the
        // whole device
        unsigned int* bad = nullptr;
        GBSA_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&bad), sizeof(unsigned int), st));
        unsigned int h_bad = 0;
        const cudaError_t e = [&] {
            // one wave of resident blocks (the loop strides over the NAMs)
            int per_sm = 0;
            cudaError_t r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_extend_seeds, 128, 0);
            if (r != cudaSuccess) return r;
            const unsigned max_blocks = (unsigned)device_sm_count() * (unsigned)(per_sm > 0 ? per_sm : 1);
            r = cudaMemsetAsync(bad, 0, sizeof(unsigned int), st);
            if (r != cudaSuccess) return r;
            k_extend_seeds<<<grid_for(n_nams, 128, max_blocks), 128, 0, st>>>(
                d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets, d_read_lengths,
                n_reads, d_nams, d_nam_reads, n_nams, k, *params, d_out, bad);
            g_launches.fetch_add(1, std::memory_order_relaxed);   // counted as GBSA_LAUNCHED, without a throw
            r = cudaGetLastError();
            if (r != cudaSuccess) return r;
            return cudaMemcpyAsync(&h_bad, bad, sizeof h_bad, cudaMemcpyDeviceToHost, st);
        }();
        GBSA_CUDA(cudaFreeAsync(bad, st));
        GBSA_CUDA(e);
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (h_bad)
            throw Error(GBSA_ERR_PARAM, std::to_string(h_bad) +
                                            " NAM(s) name a read or contig out of range or leave their read or contig");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

extern "C" int gbsa_rescue_mates_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                                        const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                                        const uint64_t* d_read_offsets, const uint32_t* d_read_lengths,
                                        uint32_t n_reads, const gbsa_nam* d_nams, const uint32_t* d_mate_reads,
                                        uint64_t n_nams, int k, float mu, float sigma, gbsa_mate_rescue* d_out,
                                        void* stream) {
    try {
        if (k < 3 || k > 32) throw Error(GBSA_ERR_PARAM, "k must be in [3, 32]");
        if (n_nams == 0) return GBSA_OK;
        cudaStream_t st = (cudaStream_t)stream;
        unsigned int* bad = nullptr;
        GBSA_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&bad), sizeof(unsigned int), st));
        unsigned int h_bad = 0;
        const cudaError_t e = [&] {
            int per_sm = 0;
            cudaError_t r =
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rescue_mates, 32 * kRescueWarps, 0);
            if (r != cudaSuccess) return r;
            const uint64_t want = (n_nams + kRescueWarps - 1) / kRescueWarps;   // a warp per NAM
            const unsigned blocks = (unsigned)std::min<uint64_t>(
                want, (uint64_t)device_sm_count() * (uint64_t)(per_sm > 0 ? per_sm : 1));
            r = cudaMemsetAsync(bad, 0, sizeof(unsigned int), st);
            if (r != cudaSuccess) return r;
            k_rescue_mates<<<blocks, 32 * kRescueWarps, 0, st>>>(
                d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets, d_read_lengths,
                n_reads, d_nams, d_mate_reads, n_nams, k, mu, sigma, d_out, bad);
            g_launches.fetch_add(1, std::memory_order_relaxed);   // counted as GBSA_LAUNCHED, without a throw
            r = cudaGetLastError();
            if (r != cudaSuccess) return r;
            return cudaMemcpyAsync(&h_bad, bad, sizeof h_bad, cudaMemcpyDeviceToHost, st);
        }();
        GBSA_CUDA(cudaFreeAsync(bad, st));
        GBSA_CUDA(e);
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (h_bad)
            throw Error(GBSA_ERR_PARAM, std::to_string(h_bad) +
                                            " NAM(s) name a contig or mate out of range or a mate with more than 64 "
                                            "sampled substrings");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

// ---- the steps of the alignment orchestration ------------------------------------------
//
// Runs the step lists of gbsa_plan_pairs_device: every step's NAM goes through the seed
// extension kernel on its own read (an extension step keeps the record; a rescue step
// keeps only reverse_nam_if_needed's answer — orientation, query interval, consistency —
// since the reference runs only that check before rescue_mate_part), then the rescue
// steps' NAMs, in the orientation that check left them, through the mate rescue kernel.

namespace gbsa {
namespace {

__global__ void k_gather_step_nams(const gbsa_nam* __restrict__ nams, const uint64_t* __restrict__ offs,
                                   const gbsa_align_step* __restrict__ steps, uint64_t n, gbsa_nam* __restrict__ out,
                                   uint32_t* __restrict__ out_reads) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        const gbsa_align_step st = steps[s];
        out[s] = nams[offs[st.nam_read] + st.nam];
        out_reads[s] = st.nam_read;
    }
}

__global__ void k_rescue_list(const gbsa_align_step* __restrict__ steps, uint64_t n, const gbsa_nam* __restrict__ step_nams,
                              gbsa_seed_alignment* __restrict__ ext, gbsa_nam* __restrict__ rnams,
                              uint32_t* __restrict__ rmates, uint64_t* __restrict__ ridx, unsigned long long* count,
                              gbsa_mate_rescue* __restrict__ resc) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x) {
        gbsa_mate_rescue none;
        none.ref_id = none.window_start = none.window_end = none.edit_distance = 0;
        none.is_rc = none.done = none.is_unaligned = none._pad = 0;
        resc[s] = none;
        const gbsa_align_step st = steps[s];
        if (st.kind != GBSA_STEP_RESCUE) continue;
        gbsa_seed_alignment e = ext[s];
        gbsa_nam nm = step_nams[s];
        nm.is_rc = e.is_rc;
        nm.query_start = e.query_start;
        nm.query_end = e.query_end;
        // the reference only checks the orientation before the rescue: no alignment record
        e.ref_start = e.edit_distance = e.global_ed = e.score = e.length = 0;
        e.done = 0;
        ext[s] = e;
        const unsigned long long j = atomicAdd(count, 1ull);
        rnams[j] = nm;
        rmates[j] = st.read;
        ridx[j] = s;
    }
}

__global__ void k_scatter_rescues(const gbsa_mate_rescue* __restrict__ in, const uint64_t* __restrict__ idx, uint64_t n,
                                  gbsa_mate_rescue* __restrict__ out) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
        out[idx[j]] = in[j];
}

}  // namespace
}  // namespace gbsa

extern "C" int gbsa_run_align_steps_device(const uint8_t* d_ref_seqs, const uint64_t* d_ref_offsets,
                                           const uint64_t* d_ref_lengths, uint32_t n_refs, const uint8_t* d_read_seqs,
                                           const uint64_t* d_read_offsets, const uint32_t* d_read_lengths,
                                           uint32_t n_reads, const gbsa_nam* d_nams, const uint64_t* d_nam_offsets,
                                           const gbsa_align_step* d_steps, uint64_t n_steps, int k,
                                           const gbsa_align_params* params, float mu, float sigma,
                                           gbsa_seed_alignment* d_ext, gbsa_mate_rescue* d_resc, void* stream) {
    try {
        if (n_steps == 0) return GBSA_OK;
        cudaStream_t st = (cudaStream_t)stream;
        // scratch in stream order: the steps' NAMs and reads, the rescue list (NAMs, mates,
        // step indices), its count and the rescue records
        const size_t b_nams = (sizeof(gbsa_nam) * n_steps + 255) & ~size_t(255);
        const size_t b_u32 = (4ull * n_steps + 255) & ~size_t(255);
        const size_t b_u64 = (8ull * n_steps + 255) & ~size_t(255);
        const size_t b_res = (sizeof(gbsa_mate_rescue) * n_steps + 255) & ~size_t(255);
        uint8_t* sc = nullptr;
        GBSA_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&sc), 2 * b_nams + 2 * b_u32 + b_u64 + b_res + 256, st));
        struct Free {
            uint8_t* p;
            cudaStream_t s;
            ~Free() { cudaFreeAsync(p, s); }
        } release{sc, st};
        gbsa_nam* step_nams = reinterpret_cast<gbsa_nam*>(sc);
        uint32_t* step_reads = reinterpret_cast<uint32_t*>(sc + b_nams);
        gbsa_nam* rnams = reinterpret_cast<gbsa_nam*>(sc + b_nams + b_u32);
        uint32_t* rmates = reinterpret_cast<uint32_t*>(sc + 2 * b_nams + b_u32);
        uint64_t* ridx = reinterpret_cast<uint64_t*>(sc + 2 * b_nams + 2 * b_u32);
        gbsa_mate_rescue* rout = reinterpret_cast<gbsa_mate_rescue*>(sc + 2 * b_nams + 2 * b_u32 + b_u64);
        unsigned long long* count = reinterpret_cast<unsigned long long*>(sc + 2 * b_nams + 2 * b_u32 + b_u64 + b_res);
        GBSA_CUDA(cudaMemsetAsync(count, 0, 8, st));
        const unsigned grid = grid_for(n_steps, 256, (unsigned)device_sm_count() * 8);
        k_gather_step_nams<<<grid, 256, 0, st>>>(d_nams, d_nam_offsets, d_steps, n_steps, step_nams, step_reads);
        GBSA_LAUNCHED();
        int rc = gbsa_extend_seeds_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets,
                                          d_read_lengths, n_reads, step_nams, step_reads, n_steps, k, params, d_ext,
                                          stream);
        if (rc != GBSA_OK) throw Error(rc, gbsa_last_error());
        k_rescue_list<<<grid, 256, 0, st>>>(d_steps, n_steps, step_nams, d_ext, rnams, rmates, ridx, count, d_resc);
        GBSA_LAUNCHED();
        unsigned long long n_resc = 0;
        GBSA_CUDA(cudaMemcpyAsync(&n_resc, count, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (n_resc) {
            rc = gbsa_rescue_mates_device(d_ref_seqs, d_ref_offsets, d_ref_lengths, n_refs, d_read_seqs, d_read_offsets,
                                          d_read_lengths, n_reads, rnams, rmates, n_resc, k, mu, sigma, rout, stream);
            if (rc != GBSA_OK) throw Error(rc, gbsa_last_error());
            k_scatter_rescues<<<grid_for(n_resc, 256, (unsigned)device_sm_count() * 8), 256, 0, st>>>(rout, ridx, n_resc,
                                                                                                    d_resc);
            GBSA_LAUNCHED();
        }
        GBSA_CUDA(cudaStreamSynchronize(st));
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}
