// noalloc.cu — randstrobes_query for callers that cannot allocate device memory.
//
// Who needs this: callers whose device memory is owned by a host framework (a
// caching allocator or a fixed pool handed out by the application) and callers in
// latency-critical serving loops.  Neither can call cudaMalloc / cudaFree in the
// middle of their work: the framework forbids it, and cudaFree waits for the whole
// device.  The regular entry points allocate their work areas on first use and
// grow them on demand, so these callers need a variant that allocates nothing.
//
// gbsa_randstrobes_query_noalloc seeds reads that are already in device memory and
// writes the query randstrobes to caller-provided device buffers.  The only scratch
// it needs is the per-warp working area of the seeding kernel (2-bit read, N mask,
// s-mer hash window and the syncmer list of one read of up to GBSA_MAX_READ_LEN
// bases), which lives in the file-scope array below: kNoallocWarps slots, about
// 3.3 MB, held by every GPU that loads the library until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it.  All calls share
// the array and it keeps the last
// call's contents: the status words are cleared at the start of every call, and
// calls that overlap on the GPU (different streams or threads running at the same
// time) race on it.  Every call waits for its stream twice (it reads the total and
// the status words back to the host before returning).
#include <mutex>

#include "map.cuh"
#include "runtime.h"

namespace gbsa {

namespace {

constexpr uint32_t kNoallocWarps = 64;
constexpr uint32_t kNoallocWarpsPerBlock = 4;
constexpr size_t kNoallocStatusBytes = 256;
constexpr size_t kNoallocBytes = kNoallocStatusBytes + (size_t)kNoallocWarps * kLongSlotBytes;

__device__ __align__(256) uint8_t g_noalloc_scratch[kNoallocBytes];

// Status block at the start of the array.
struct NoallocStatus {
    unsigned long long total;   // query randstrobes of all reads
    unsigned int flags;         // kStatus* bits
};

struct Slot {
    uint64_t* pk;
    uint32_t* nm;
    uint64_t* hb;
    uint64_t* sh;
    uint32_t* sp;
};

__device__ __forceinline__ Slot slot_of(uint8_t* base, uint32_t warp) {
    uint8_t* s = base + kNoallocStatusBytes + (size_t)warp * kLongSlotBytes;
    Slot r;
    r.pk = reinterpret_cast<uint64_t*>(s);
    r.nm = reinterpret_cast<uint32_t*>(r.pk + kLongWords);
    r.hb = reinterpret_cast<uint64_t*>(r.nm + kLongWords);
    r.sh = r.hb + 64;
    r.sp = reinterpret_cast<uint32_t*>(r.sh + GBSA_MAX_READ_LEN);
    return r;
}

// Pass 1 (kWrite = false): counts[r] = query randstrobes of read r.
// Pass 2 (kWrite = true): writes them at offsets[r] (reference order: forward ones by
// start, then the reverse-complement ones).
template <bool kWrite>
__global__ void __launch_bounds__(32 * kNoallocWarpsPerBlock)
    k_noalloc_seed(DevParams P, const uint8_t* __restrict__ seqs, const uint64_t* __restrict__ offs,
                   const uint32_t* __restrict__ lens, uint32_t n, uint64_t* __restrict__ offsets,
                   gbsa_query_randstrobe* __restrict__ out, uint64_t cap, uint8_t* scratch) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    NoallocStatus* st = reinterpret_cast<NoallocStatus*>(scratch);
    const Slot S = slot_of(scratch, warp);
    const uint32_t lane = lane_id();
    for (uint32_t r = warp; r < n; r += nwarps) {
        const uint32_t L = lens[r];
        if (L > GBSA_MAX_READ_LEN) {
            if (lane == 0) {
                atomicOr(&st->flags, kStatusReadTooLong);
                if (!kWrite) offsets[r] = 0;
            }
            continue;
        }
        const uint32_t ns = warp_read_syncmers(P, seqs + offs[r], L, S.pk, S.nm, S.hb, S.sh, S.sp, GBSA_MAX_READ_LEN);
        const uint32_t nq = ns == 0xFFFFFFFFu ? 0 : n_query_per_dir(P, ns, L);
        if (!kWrite) {
            if (lane == 0) offsets[r] = 2ull * nq;
            __syncwarp();
            continue;
        }
        const uint64_t o = offsets[r];
        if (o + 2ull * nq > cap) {
            if (lane == 0) atomicOr(&st->flags, kStatusQueryOverflow);
            continue;
        }
        for (uint32_t j = lane; j < 2 * nq; j += 32) {
            uint64_t h;
            uint32_t s1, s2;
            if (j < nq) randstrobe_fwd(P, S.sh, S.sp, ns, j, h, s1, s2);
            else randstrobe_rev(P, S.sh, S.sp, ns, L, j - nq, h, s1, s2);
            gbsa_query_randstrobe x;
            x.hash = h;
            x.start = s1;
            x.end = s2 + (uint32_t)P.k;
            x.is_reverse = j >= nq ? 1 : 0;
            for (int b = 0; b < 7; ++b) x._pad[b] = 0;
            out[o + j] = x;
        }
        __syncwarp();
    }
}

// Exclusive scan of offsets[0..n) in place with one block; offsets[n] = total.
__global__ void __launch_bounds__(1024) k_noalloc_scan(uint64_t* offsets, uint32_t n, uint8_t* scratch) {
    __shared__ uint64_t s_warp[32];
    __shared__ uint64_t s_carry;
    const uint32_t t = threadIdx.x, lane = t & 31, wid = t >> 5;
    if (t == 0) s_carry = 0;
    __syncthreads();
    // 64-bit indices: with 32-bit ones a count near 2^32 would wrap and never end
    for (uint64_t base = 0; base < n; base += 1024) {
        const uint64_t i = base + t;
        const uint64_t v = i < n ? offsets[i] : 0;
        const uint64_t inc = warp_inclusive_sum(v);
        if (lane == 31) s_warp[wid] = inc;
        __syncthreads();
        if (wid == 0) {
            const uint64_t x = s_warp[lane];
            s_warp[lane] = warp_inclusive_sum(x) - x;
        }
        __syncthreads();
        const uint64_t excl = s_carry + s_warp[wid] + inc - v;
        if (i < n) offsets[i] = excl;
        __syncthreads();
        if (t == 1023) s_carry = excl + v;
        __syncthreads();
    }
    if (t == 0) {
        offsets[n] = s_carry;
        reinterpret_cast<NoallocStatus*>(scratch)->total = s_carry;
    }
}

std::mutex g_noalloc_mu;
uint8_t* g_noalloc_ptr[64] = {};

// Device address of the array on the current device (looked up once per device).
uint8_t* noalloc_scratch() {
    int dev = 0;
    GBSA_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error(GBSA_ERR_CUDA, "device ordinal out of range");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw Error(GBSA_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch) failed: ") +
                                           cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<uint8_t*>(p);
    }
    return g_noalloc_ptr[dev];
}

}  // namespace

}  // namespace gbsa

using namespace gbsa;

extern "C" int gbsa_randstrobes_query_noalloc(const gbsa_params* p, const char* d_seqs, const uint64_t* d_offsets,
                                              const uint32_t* d_lengths, uint32_t n_reads,
                                              gbsa_query_randstrobe* d_out, uint64_t out_capacity,
                                              uint64_t* d_out_offsets, uint64_t* out_total, void* stream) {
    try {
        if (!params_valid(*p)) throw Error(GBSA_ERR_PARAM, "invalid index parameters");
        cudaStream_t st = (cudaStream_t)stream;
        uint8_t* scratch = noalloc_scratch();
        const DevParams P = make_dev_params(*p);
        const uint8_t* seqs = reinterpret_cast<const uint8_t*>(d_seqs);
        GBSA_CUDA(cudaMemsetAsync(scratch, 0, kNoallocStatusBytes, st));
        const unsigned blocks = kNoallocWarps / kNoallocWarpsPerBlock;
        if (n_reads) {
            k_noalloc_seed<false><<<blocks, 32 * kNoallocWarpsPerBlock, 0, st>>>(P, seqs, d_offsets, d_lengths, n_reads,
                                                                               d_out_offsets, d_out, out_capacity,
                                                                               scratch);
            GBSA_LAUNCHED();
        }
        k_noalloc_scan<<<1, 1024, 0, st>>>(d_out_offsets, n_reads, scratch);
        GBSA_LAUNCHED();
        NoallocStatus h{};
        GBSA_CUDA(cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (out_total) *out_total = h.total;
        if (h.flags & kStatusReadTooLong)
            throw Error(GBSA_ERR_READ_TOO_LONG, "a read is longer than GBSA_MAX_READ_LEN (4096) bases");
        if (h.total > out_capacity)
            throw Error(GBSA_ERR_CAPACITY, "output capacity too small: " + std::to_string(h.total) +
                                               " query randstrobes needed");
        if (n_reads) {
            k_noalloc_seed<true><<<blocks, 32 * kNoallocWarpsPerBlock, 0, st>>>(P, seqs, d_offsets, d_lengths, n_reads,
                                                                              d_out_offsets, d_out, out_capacity,
                                                                              scratch);
            GBSA_LAUNCHED();
        }
        GBSA_CUDA(cudaMemcpyAsync(&h, scratch, sizeof h, cudaMemcpyDeviceToHost, st));
        GBSA_CUDA(cudaStreamSynchronize(st));
        if (h.flags & kStatusQueryOverflow) throw Error(GBSA_ERR_CAPACITY, "output capacity too small");
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}
