// prims.cu — exclusive scan and stable LSD radix sort (see prims.cuh).
#include "prims.cuh"

namespace gbsa {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr size_t kScanTile = (size_t)kScanThreads * kScanItems;

template <int NT>
__device__ uint64_t block_exclusive_sum(uint64_t v, uint64_t* s_warp, uint64_t& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint64_t inc = warp_inclusive_sum(v);
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        uint64_t x = lane < NT / 32 ? s_warp[lane] : 0;
        uint64_t xi = warp_inclusive_sum(x);
        if (lane < NT / 32) s_warp[lane] = xi - x;
        if (lane == NT / 32 - 1) s_warp[32] = xi;
    }
    __syncthreads();
    total = s_warp[32];
    const uint64_t r = s_warp[wid] + inc - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_partials(const uint64_t* in, size_t n, uint64_t* partials) {
    __shared__ uint64_t s_warp[33];
    const size_t base = (size_t)blockIdx.x * kScanTile;
    uint64_t v = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const size_t idx = base + (size_t)i * kScanThreads + threadIdx.x;
        if (idx < n) v += in[idx];
    }
    uint64_t total;
    block_exclusive_sum<kScanThreads>(v, s_warp, total);
    if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint64_t* in, uint64_t* out, size_t n,
                                                             const uint64_t* offsets, uint64_t* d_total) {
    __shared__ uint64_t s_warp[33];
    const size_t base = (size_t)blockIdx.x * kScanTile;
    // each thread owns kScanItems consecutive elements
    uint64_t v[kScanItems];
    uint64_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const size_t idx = base + (size_t)threadIdx.x * kScanItems + i;
        v[i] = idx < n ? in[idx] : 0;
        sum += v[i];
    }
    uint64_t total;
    uint64_t run = block_exclusive_sum<kScanThreads>(sum, s_warp, total) + (offsets ? offsets[blockIdx.x] : 0);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const size_t idx = base + (size_t)threadIdx.x * kScanItems + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
    if (d_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanThreads - 1) *d_total = run;
}

// ---- radix sort --------------------------------------------------------------
constexpr int kSortThreads = 256;
constexpr int kSortRounds = 16;
constexpr size_t kSortTile = (size_t)kSortThreads * kSortRounds;

__device__ __forceinline__ uint32_t digit_of(const gbsa_ref_randstrobe& r, int pass) {
    // passes 0..3: position bytes (least significant key), 4..11: hash bytes
    if (pass < 4) return (r.position >> (8 * pass)) & 0xFF;
    return (uint32_t)(r.hash >> (8 * (pass - 4))) & 0xFF;
}

__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const gbsa_ref_randstrobe* in, size_t n, int pass,
                                                              uint64_t* block_hist, size_t nblocks,
                                                              unsigned long long* global_hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const size_t idx = base + (size_t)r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[digit_of(in[idx], pass)], 1u);
    }
    __syncthreads();
    const uint32_t c = h[threadIdx.x];
    block_hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = c;
    if (c) atomicAdd(&global_hist[threadIdx.x], (unsigned long long)c);
}

__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const gbsa_ref_randstrobe* in,
                                                                 gbsa_ref_randstrobe* out, size_t n, int pass,
                                                                 const uint64_t* block_off, size_t nblocks) {
    __shared__ uint64_t s_base[256];
    __shared__ uint32_t s_run[256];
    __shared__ uint32_t s_wcnt[kSortThreads / 32][256];
    __shared__ uint32_t s_woff[kSortThreads / 32][256];
    const uint32_t t = threadIdx.x, lane = t & 31, wid = t >> 5;
    s_base[t] = block_off[(size_t)t * nblocks + blockIdx.x];
    s_run[t] = 0;
    for (int w = 0; w < kSortThreads / 32; ++w) s_wcnt[w][t] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const size_t idx = base + (size_t)r * kSortThreads + t;
        const bool valid = idx < n;
        gbsa_ref_randstrobe rec;
        uint32_t d = 256;
        if (valid) {
            rec = in[idx];
            d = digit_of(rec, pass);
        }
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & lanemask_lt());
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) s_wcnt[wid][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = s_run[t];
            for (int w = 0; w < kSortThreads / 32; ++w) {
                const uint32_t c = s_wcnt[w][t];
                s_woff[w][t] = run;
                run += c;
                s_wcnt[w][t] = 0;
            }
            s_run[t] = run;
        }
        __syncthreads();
        if (valid) out[s_base[d] + s_woff[wid][d] + rank] = rec;
    }
}

}  // namespace

void scan_exclusive_u64(const uint64_t* in, uint64_t* out, size_t n, uint64_t* d_total, Workspace& ws,
                        cudaStream_t st) {
    if (n == 0) {
        if (d_total) GBSA_CUDA(cudaMemsetAsync(d_total, 0, sizeof(uint64_t), st));
        return;
    }
    const size_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        k_scan_apply<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr, d_total);
        GBSA_LAUNCHED();
        return;
    }
    uint64_t* partials = ws.get<uint64_t>(nb);
    k_scan_partials<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, partials);
    GBSA_LAUNCHED();
    scan_exclusive_u64(partials, partials, nb, nullptr, ws, st);
    k_scan_apply<<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, n, partials, d_total);
    GBSA_LAUNCHED();
}

gbsa_ref_randstrobe* radix_sort_ref_randstrobes(gbsa_ref_randstrobe* a, gbsa_ref_randstrobe* b, size_t n,
                                                Workspace& ws, cudaStream_t st) {
    if (n <= 1) return a;
    const size_t nb = (n + kSortTile - 1) / kSortTile;
    uint64_t* bh = ws.get<uint64_t>(256 * nb);
    unsigned long long* gh = ws.get<unsigned long long>(256);
    std::vector<unsigned long long> hgh(256);
    gbsa_ref_randstrobe* src = a;
    gbsa_ref_randstrobe* dst = b;
    for (int pass = 0; pass < 12; ++pass) {
        GBSA_CUDA(cudaMemsetAsync(gh, 0, 256 * sizeof(unsigned long long), st));
        k_radix_hist<<<(unsigned)nb, kSortThreads, 0, st>>>(src, n, pass, bh, nb, gh);
        GBSA_LAUNCHED();
        GBSA_CUDA(cudaMemcpyAsync(hgh.data(), gh, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        bool trivial = false;
        for (int d = 0; d < 256; ++d) trivial |= (hgh[d] == n);
        if (trivial) continue;
        scan_exclusive_u64(bh, bh, 256 * nb, nullptr, ws, st);
        k_radix_scatter<<<(unsigned)nb, kSortThreads, 0, st>>>(src, dst, n, pass, bh, nb);
        GBSA_LAUNCHED();
        std::swap(src, dst);
    }
    return src;
}

}  // namespace gbsa
