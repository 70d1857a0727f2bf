// index_build.cu — StrobemerIndex::populate on the GPU.
//
// Restates step2/index.cu:143-311 (populate, count_randstrobes, assign_randstrobes;
// commented out in the reference) with the RandstrobeGenerator of
// step2/randstrobes.cu:161-190:
//   1. pack the contigs into a 2-bit stream + N bitmask (one pass over the bases);
//   2. canonical syncmers of every contig, a warp per 2048-window segment (count
//      pass, exclusive scan, write pass); a segment starts at an "anchor" window
//      whose syncmer state does not depend on earlier windows;
//   3. one forward randstrobe per syncmer with at least w_min successors in its
//      contig, packed = (ref_index << 8) + (strobe2 - strobe1); contigs shorter than
//      w_max keep zeroed entries (counted, never assigned, as in the reference);
//   4. stable LSD radix sort by (hash, position) — ties keep generation order, which
//      is (ref_index, position), i.e. the table ends up sorted by (hash, position,
//      packed);
//   5. bucket start table with the reference's first-bucket rule, and the run-length
//      statistics that give filter_cutoff (float product unique_mers * f).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "index.h"
#include "prims.cuh"
#include "seed.cuh"

namespace gbsa {

namespace {

constexpr uint32_t kSegWindows = 2048;
constexpr int kSegWarps = 8;

// one thread per 32 bases; g is padded with 'N' to a multiple of 32 plus 64 bytes
__global__ void k_pack_genome(const uint8_t* __restrict__ g, uint64_t nwords, uint64_t* __restrict__ packed,
                              uint32_t* __restrict__ nmask) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nwords; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4* src = reinterpret_cast<const uint4*>(g + 32 * i);
        const uint4 a = src[0], b = src[1];
        const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint64_t word = 0;
        uint32_t nm = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const uint32_t c = nt4((uint8_t)(w[j >> 2] >> (8 * (j & 3))));
            nm |= (c == 4u ? 1u : 0u) << j;
            word = (word << 2) | (c & 3u);
        }
        packed[i] = word;
        nmask[i] = nm;
    }
}

struct SegTables {
    const uint32_t* seg_contig;
    const uint32_t* seg_w0;
    const uint32_t* seg_w1;
    const uint64_t* contig_base;
    const uint32_t* contig_nwin;
};

template <bool kWrite>
__global__ void __launch_bounds__(32 * kSegWarps) k_contig_syncmers(DevParams P, const uint64_t* __restrict__ packed,
                                                                    const uint32_t* __restrict__ nmask, SegTables T,
                                                                    uint32_t n_seg, uint64_t* __restrict__ seg_count,
                                                                    const uint64_t* __restrict__ seg_off,
                                                                    uint64_t* __restrict__ sh, uint32_t* __restrict__ sp) {
    __shared__ uint64_t s_h[kSegWarps][64];
    const uint32_t wid = threadIdx.x >> 5;
    uint64_t* hbuf = s_h[wid];
    for (uint32_t s = blockIdx.x * kSegWarps + wid; s < n_seg; s += gridDim.x * kSegWarps) {
        const uint32_t c = T.seg_contig[s];
        const uint32_t w0 = T.seg_w0[s], w1 = T.seg_w1[s];
        const uint64_t base = T.contig_base[c];
        const uint32_t nwin = T.contig_nwin[c];
        const uint32_t anchor = warp_find_anchor(P, packed, nmask, base, nwin, w0, hbuf);
        if (kWrite) {
            const uint64_t o = seg_off[s];
            const uint32_t n = warp_syncmer_scan(P, packed, nmask, base, nwin, anchor, w1, w0, hbuf,
                                                 [&](uint32_t idx, uint32_t w) { sp[o + idx] = w; });
            __syncwarp();
            for (uint32_t i = lane_id(); i < n; i += 32) sh[o + i] = kmer_hash(P, packed, base + sp[o + i]);
        } else {
            const uint32_t n = warp_syncmer_scan(P, packed, nmask, base, nwin, anchor, w1, w0, hbuf,
                                                 [](uint32_t, uint32_t) {});
            if (lane_id() == 0) seg_count[s] = n;
        }
    }
}

__global__ void k_ref_randstrobes(DevParams P, const uint64_t* __restrict__ sh, const uint32_t* __restrict__ sp,
                                  uint64_t n_sm, const uint64_t* __restrict__ contig_sm, uint32_t n_contigs,
                                  const uint64_t* __restrict__ contig_ref_off, const uint64_t* __restrict__ contig_len,
                                  gbsa_ref_randstrobe* __restrict__ out) {
    for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n_sm; g += (uint64_t)gridDim.x * blockDim.x) {
        // contig of syncmer g: last c with contig_sm[c] <= g
        uint32_t lo = 0, hi = n_contigs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (contig_sm[mid] <= g) lo = mid;
            else hi = mid;
        }
        const uint32_t c = lo;
        if (contig_len[c] < P.w_max) continue;   // step2/index.cu:282-284
        const uint64_t b = contig_sm[c];
        const uint32_t nc = (uint32_t)(contig_sm[c + 1] - b);
        const uint32_t j = (uint32_t)(g - b);
        if (j + P.w_min >= nc) continue;
        uint64_t h;
        uint32_t s1, s2;
        randstrobe_fwd(P, sh + b, sp + b, nc, j, h, s1, s2);
        gbsa_ref_randstrobe r;
        r.hash = h;
        r.position = s1;
        r.packed = (uint32_t)((uint64_t)c << 8) + (s2 - s1);
        out[contig_ref_off[c] + j] = r;
    }
}

__global__ void k_first_distinct(const gbsa_ref_randstrobe* __restrict__ rs, uint64_t n,
                                 unsigned long long* __restrict__ p1) {
    const uint64_t h0 = rs[0].hash;
    for (uint64_t i = 1 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (rs[i].hash != h0) {
            atomicMin(p1, (unsigned long long)i);
            return;
        }
    }
}

__global__ void k_bucket_starts(const gbsa_ref_randstrobe* __restrict__ rs, uint64_t n, int bits,
                                const unsigned long long* __restrict__ p1, uint64_t* __restrict__ starts) {
    const uint64_t nb = 1ULL << bits;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t t = rs[i].hash >> (64 - bits);
        if (i == 0) {
            const uint64_t v = *p1;
            for (uint64_t b = 0; b <= t; ++b) starts[b] = v;
        } else {
            const uint64_t tp = rs[i - 1].hash >> (64 - bits);
            for (uint64_t b = tp + 1; b <= t; ++b) starts[b] = i;
        }
        if (i == n - 1) {
            for (uint64_t b = t + 1; b <= nb; ++b) starts[b] = n;
        }
    }
}

__global__ void k_run_flags(const gbsa_ref_randstrobe* __restrict__ rs, uint64_t n, uint64_t* __restrict__ flags) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        flags[i] = (i == 0 || rs[i].hash != rs[i - 1].hash) ? 1 : 0;
}

__global__ void k_run_starts(const gbsa_ref_randstrobe* __restrict__ rs, uint64_t n, const uint64_t* __restrict__ idx,
                             uint64_t* __restrict__ run_start) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (i == 0 || rs[i].hash != rs[i - 1].hash) run_start[idx[i]] = i;
}

// histogram of run lengths: bins 1..100 exact, bin 101 = longer
__global__ void k_run_hist(const uint64_t* __restrict__ run_start, uint64_t n_runs, uint64_t n,
                           unsigned long long* __restrict__ hist) {
    __shared__ unsigned int h[102];
    for (int i = threadIdx.x; i < 102; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n_runs; j += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t e = (j + 1 < n_runs) ? run_start[j + 1] : n;
        const uint64_t len = e - run_start[j];
        atomicAdd(&h[len > 101 ? 101 : len], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 102; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], (unsigned long long)h[i]);
}

}  // namespace

// filter_cutoff and the creation statistics from the run-length histogram, with the
// reference's arithmetic (step2/index.cu:213-243).
static void finish_stats(gbsa_index& ix, const std::vector<unsigned long long>& H, uint64_t unique, float f) {
    uint64_t once = 0, high = 0, mid = 0, size = 0;
    uint32_t fc = 30;
    const uint64_t index_cutoff = (uint64_t)((float)unique * f);
    if (ix.n == 0) {
        mid = 1;   // the reference closes an empty "run" of count 0 (index.cu:214-223)
    } else {
        once = H[1];
        high = H[101];
        for (int v = 2; v <= 100; ++v) mid += H[v];
        size = high + mid;
        if (size > 0) {
            uint32_t value = 0;
            if (index_cutoff < size) {
                uint64_t cum = 0;
                for (int v = 101; v >= 2; --v) {
                    if (index_cutoff < cum + H[v]) {
                        value = (uint32_t)v;   // v == 101 stands for any count > 100
                        break;
                    }
                    cum += H[v];
                }
            } else {
                for (int v = 2; v <= 101; ++v)
                    if (H[v]) {
                        value = (uint32_t)v;
                        break;
                    }
            }
            fc = std::min(100u, std::max(30u, value));
        }
    }
    ix.filter_cutoff = fc;
    ix.info.tot_occur_once = once;
    ix.info.tot_high_ab = high;
    ix.info.tot_mid_ab = mid;
    ix.info.index_cutoff = index_cutoff;
    ix.info.distinct_strobemers = unique;
    ix.info.filter_cutoff = fc;
}

void build_index(gbsa_index& ix, const char* seqs, const uint64_t* offsets, const uint64_t* lengths,
                 uint32_t n_contigs, float f) {
    const DevParams P = ix.dp;
    Workspace ws;
    cudaStream_t st;
    GBSA_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};

    // ---- genome upload + packing -------------------------------------------
    std::vector<uint64_t> cbase(n_contigs + 1, 0);
    for (uint32_t c = 0; c < n_contigs; ++c) cbase[c + 1] = cbase[c] + lengths[c];
    const uint64_t total = cbase[n_contigs];
    const uint64_t nwords = (total + 31) / 32 + 4;
    DeviceBuffer d_g(nwords * 32 + 64);
    GBSA_CUDA(cudaMemsetAsync(d_g.as<uint8_t>(), 'N', nwords * 32 + 64, st));
    {
        // contiguous input → one copy; otherwise one copy per contig
        bool contiguous = true;
        for (uint32_t c = 0; c < n_contigs; ++c) contiguous &= (offsets[c] == offsets[0] + cbase[c]);
        if (contiguous && total) {
            GBSA_CUDA(cudaMemcpyAsync(d_g.as<uint8_t>(), seqs + offsets[0], total, cudaMemcpyHostToDevice, st));
        } else {
            for (uint32_t c = 0; c < n_contigs; ++c)
                if (lengths[c])
                    GBSA_CUDA(cudaMemcpyAsync(d_g.as<uint8_t>() + cbase[c], seqs + offsets[c], lengths[c],
                                              cudaMemcpyHostToDevice, st));
        }
    }
    DeviceBuffer d_packed(nwords * 8 + 64), d_nmask(nwords * 4 + 64);
    k_pack_genome<<<grid_for(nwords, 256, 65535), 256, 0, st>>>(d_g.as<uint8_t>(), nwords, d_packed.as<uint64_t>(),
                                                                d_nmask.as<uint32_t>());
    GBSA_LAUNCHED();

    // ---- segments -------------------------------------------------------------
    std::vector<uint32_t> seg_c, seg_w0, seg_w1, cnwin(n_contigs);
    std::vector<uint64_t> cfirst_seg(n_contigs + 1, 0);
    for (uint32_t c = 0; c < n_contigs; ++c) {
        cfirst_seg[c] = seg_c.size();
        const uint64_t L = lengths[c];
        if (L >= 1ULL << 32) throw Error(GBSA_ERR_PARAM, "contig longer than 2^32 - 1 bases");
        const uint32_t nwin = L >= (uint64_t)P.k ? (uint32_t)(L - P.k + 1) : 0;
        cnwin[c] = nwin;
        for (uint32_t w = 0; w < nwin; w += kSegWindows) {
            seg_c.push_back(c);
            seg_w0.push_back(w);
            seg_w1.push_back(std::min(nwin, w + kSegWindows));
        }
    }
    cfirst_seg[n_contigs] = seg_c.size();
    const uint32_t n_seg = (uint32_t)seg_c.size();
    DeviceBuffer d_segc(4 * (n_seg + 1)), d_segw0(4 * (n_seg + 1)), d_segw1(4 * (n_seg + 1));
    DeviceBuffer d_cbase(8 * (n_contigs + 1)), d_cnwin(4 * (n_contigs + 1));
    if (n_seg) {
        GBSA_CUDA(cudaMemcpyAsync(d_segc.as<void>(), seg_c.data(), 4 * n_seg, cudaMemcpyHostToDevice, st));
        GBSA_CUDA(cudaMemcpyAsync(d_segw0.as<void>(), seg_w0.data(), 4 * n_seg, cudaMemcpyHostToDevice, st));
        GBSA_CUDA(cudaMemcpyAsync(d_segw1.as<void>(), seg_w1.data(), 4 * n_seg, cudaMemcpyHostToDevice, st));
    }
    GBSA_CUDA(cudaMemcpyAsync(d_cbase.as<void>(), cbase.data(), 8 * (n_contigs + 1), cudaMemcpyHostToDevice, st));
    if (n_contigs)
        GBSA_CUDA(cudaMemcpyAsync(d_cnwin.as<void>(), cnwin.data(), 4 * n_contigs, cudaMemcpyHostToDevice, st));
    SegTables T{d_segc.as<uint32_t>(), d_segw0.as<uint32_t>(), d_segw1.as<uint32_t>(), d_cbase.as<uint64_t>(),
                d_cnwin.as<uint32_t>()};

    DeviceBuffer d_segcnt(8 * (n_seg + 1)), d_segoff(8 * (n_seg + 1));
    uint64_t n_sm = 0;
    const unsigned seg_blocks = grid_for(n_seg, kSegWarps, 1u << 20);
    if (n_seg) {
        k_contig_syncmers<false><<<seg_blocks, 32 * kSegWarps, 0, st>>>(P, d_packed.as<uint64_t>(),
                                                                        d_nmask.as<uint32_t>(), T, n_seg,
                                                                        d_segcnt.as<uint64_t>(), nullptr, nullptr,
                                                                        nullptr);
        GBSA_LAUNCHED();
        uint64_t* d_tot = ws.get<uint64_t>(1);
        scan_exclusive_u64(d_segcnt.as<uint64_t>(), d_segoff.as<uint64_t>(), n_seg, d_tot, ws, st);
        GBSA_CUDA(cudaMemcpyAsync(&n_sm, d_tot, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
    }
    DeviceBuffer d_sh(8 * (n_sm + 1)), d_sp(4 * (n_sm + 1));
    if (n_seg) {
        k_contig_syncmers<true><<<seg_blocks, 32 * kSegWarps, 0, st>>>(P, d_packed.as<uint64_t>(),
                                                                       d_nmask.as<uint32_t>(), T, n_seg, nullptr,
                                                                       d_segoff.as<uint64_t>(), d_sh.as<uint64_t>(),
                                                                       d_sp.as<uint32_t>());
        GBSA_LAUNCHED();
    }
    d_g.release();

    // ---- per-contig syncmer ranges and randstrobe offsets (count_randstrobes) ---
    std::vector<uint64_t> segoff(n_seg + 1, 0);
    if (n_seg) GBSA_CUDA(cudaMemcpyAsync(segoff.data(), d_segoff.as<uint64_t>(), 8 * n_seg, cudaMemcpyDeviceToHost, st));
    GBSA_CUDA(cudaStreamSynchronize(st));
    segoff[n_seg] = n_sm;
    std::vector<uint64_t> csm(n_contigs + 1), cref(n_contigs + 1, 0), clen(n_contigs + 1, 0);
    for (uint32_t c = 0; c <= n_contigs; ++c) csm[c] = segoff[cfirst_seg[c]];
    uint64_t n_rs = 0;
    for (uint32_t c = 0; c < n_contigs; ++c) {
        const uint64_t nc = csm[c + 1] - csm[c];
        cref[c] = n_rs;
        n_rs += nc < P.w_min ? 0 : nc - P.w_min;
        clen[c] = lengths[c];
    }
    cref[n_contigs] = n_rs;
    ix.n = n_rs;
    ix.info.tot_strobemer_count = n_rs;
    DeviceBuffer d_csm(8 * (n_contigs + 1)), d_cref(8 * (n_contigs + 1)), d_clen(8 * (n_contigs + 1));
    GBSA_CUDA(cudaMemcpyAsync(d_csm.as<void>(), csm.data(), 8 * (n_contigs + 1), cudaMemcpyHostToDevice, st));
    GBSA_CUDA(cudaMemcpyAsync(d_cref.as<void>(), cref.data(), 8 * (n_contigs + 1), cudaMemcpyHostToDevice, st));
    GBSA_CUDA(cudaMemcpyAsync(d_clen.as<void>(), clen.data(), 8 * (n_contigs + 1), cudaMemcpyHostToDevice, st));

    DeviceBuffer d_a(16 * (n_rs + 1)), d_b(16 * (n_rs + 1));
    GBSA_CUDA(cudaMemsetAsync(d_a.as<void>(), 0, 16 * (n_rs + 1), st));
    if (n_sm) {
        k_ref_randstrobes<<<grid_for(n_sm, 256, 1u << 20), 256, 0, st>>>(
            P, d_sh.as<uint64_t>(), d_sp.as<uint32_t>(), n_sm, d_csm.as<uint64_t>(), n_contigs, d_cref.as<uint64_t>(),
            d_clen.as<uint64_t>(), d_a.as<gbsa_ref_randstrobe>());
        GBSA_LAUNCHED();
    }
    d_sh.release();
    d_sp.release();
    d_packed.release();
    d_nmask.release();

    // ---- sort --------------------------------------------------------------------
    gbsa_ref_randstrobe* sorted =
        radix_sort_ref_randstrobes(d_a.as<gbsa_ref_randstrobe>(), d_b.as<gbsa_ref_randstrobe>(), n_rs, ws, st);
    if (sorted == d_a.as<gbsa_ref_randstrobe>()) {
        ix.rs = std::move(d_a);
    } else {
        ix.rs = std::move(d_b);
    }

    // ---- bucket table ------------------------------------------------------------
    const uint64_t nb = (1ULL << ix.bits) + 1;
    ix.starts.resize(8 * nb);
    const gbsa_ref_randstrobe* rs = ix.rs.as<gbsa_ref_randstrobe>();
    if (n_rs == 0) {
        GBSA_CUDA(cudaMemsetAsync(ix.starts.as<void>(), 0, 8 * nb, st));
    } else {
        unsigned long long* d_p1 = ws.get<unsigned long long>(1);
        GBSA_CUDA(cudaMemcpyAsync(d_p1, &n_rs, 8, cudaMemcpyHostToDevice, st));
        k_first_distinct<<<grid_for(n_rs, 256, 1u << 16), 256, 0, st>>>(rs, n_rs, d_p1);
        GBSA_LAUNCHED();
        k_bucket_starts<<<grid_for(n_rs, 256, 1u << 20), 256, 0, st>>>(rs, n_rs, ix.bits, d_p1,
                                                                       ix.starts.as<uint64_t>());
        GBSA_LAUNCHED();
    }

    // ---- run-length statistics → filter_cutoff ---------------------------------------
    std::vector<unsigned long long> H(102, 0);
    uint64_t unique = 0;
    if (n_rs) {
        uint64_t* flags = ws.get<uint64_t>(n_rs);
        uint64_t* idx = ws.get<uint64_t>(n_rs);
        uint64_t* d_runs = ws.get<uint64_t>(1);
        k_run_flags<<<grid_for(n_rs, 256, 1u << 20), 256, 0, st>>>(rs, n_rs, flags);
        GBSA_LAUNCHED();
        scan_exclusive_u64(flags, idx, n_rs, d_runs, ws, st);
        GBSA_CUDA(cudaMemcpyAsync(&unique, d_runs, 8, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        uint64_t* run_start = flags;   // reuse
        k_run_starts<<<grid_for(n_rs, 256, 1u << 20), 256, 0, st>>>(rs, n_rs, idx, run_start);
        GBSA_LAUNCHED();
        unsigned long long* d_h = ws.get<unsigned long long>(102);
        GBSA_CUDA(cudaMemsetAsync(d_h, 0, 102 * 8, st));
        k_run_hist<<<grid_for(unique, 256, 4096), 256, 0, st>>>(run_start, unique, n_rs, d_h);
        GBSA_LAUNCHED();
        GBSA_CUDA(cudaMemcpyAsync(H.data(), d_h, 102 * 8, cudaMemcpyDeviceToHost, st));
    }
    GBSA_CUDA(cudaStreamSynchronize(st));
    finish_stats(ix, H, unique, f);
    ix.info.size = ix.n;
    ix.info.bits = ix.bits;
    make_compact_starts(ix, st);
}

__global__ void k_narrow_starts(const uint64_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (uint32_t)in[i];
}

void make_compact_starts(gbsa_index& ix, cudaStream_t st) {
    if (ix.n >= (1ull << 32)) return;
    const uint64_t nb = (1ULL << ix.bits) + 1;
    ix.starts32.resize(4 * nb);
    k_narrow_starts<<<grid_for(nb, 256, 1u << 16), 256, 0, st>>>(ix.starts.as<uint64_t>(), ix.starts32.as<uint32_t>(),
                                                                 nb);
    GBSA_LAUNCHED();
    GBSA_CUDA(cudaStreamSynchronize(st));
}

}  // namespace gbsa
