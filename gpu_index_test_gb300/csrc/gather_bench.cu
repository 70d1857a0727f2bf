// gather_bench.cu — achievable bandwidth of random 32-byte gathers on this GPU.
//
// The lookup reads the index at random: each probe brings one or two 32 B sectors
// from the bucket table or the entry array.  A streaming copy (the HBM peak of the
// roofline) is not reachable by such a pattern, so the lookup is also compared with
// this measurement: every thread reads sectors at independent pseudo-random
// addresses of a buffer (8 loads in flight per thread, cached in L2 only), over a
// buffer much larger than L2 (HBM gathers) or one that fits it (L2 gathers).
#include <algorithm>

#include "lookup.cuh"
#include "runtime.h"

namespace gbsa {
namespace {

__global__ void k_fill(uint4* buf, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        buf[i] = make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0x9E3779B9u, 0x7F4A7C15u);
}

__global__ void __launch_bounds__(256) k_gather(const uint4* __restrict__ buf, uint64_t n_sectors, uint32_t rounds,
                                                uint32_t* __restrict__ out) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t x = 0x9E3779B97F4A7C15ULL ^ (tid * 0xD1B54A32D192ED03ULL);
    uint32_t acc = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint4 v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            const uint64_t s = __umul64hi(x, n_sectors);   // uniform in [0, n_sectors)
            v[j] = __ldcg(buf + 2 * s);                   // the first 16 B of the sector
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) acc ^= v[j].x ^ v[j].w;
    }
    out[tid] = acc;
}

// The lookup's own access pattern on the lookup's own buffers: for a uniform random
// key, the bucket bound pair from the index's bucket table (the 32-bit copy when it
// has one), then the first entry of the bucket, a load that depends on the first.
// 8 probes in flight per thread.  Sectors: the bucket pair's, plus the entry's for a
// non-empty bucket.
__global__ void __launch_bounds__(256) k_gather_index(IndexView I, uint32_t rounds, uint32_t* __restrict__ out,
                                                      unsigned long long* __restrict__ sectors) {
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t x = 0x9E3779B97F4A7C15ULL ^ (tid * 0xD1B54A32D192ED03ULL);
    uint32_t acc = 0, n_sec = 0;
    const int sh = 64 - I.bits;
    for (uint32_t r = 0; r < rounds; ++r) {
        uint64_t a[8], b[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            const uint64_t top = (x * 0x2545F4914F6CDD1DULL) >> sh;
            a[j] = bucket_start(I, top);
            b[j] = bucket_start(I, top + 1);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            n_sec += 1;
            if (a[j] < b[j]) {
                acc ^= (uint32_t)__ldcg(&I.rs[a[j]].hash);
                n_sec += 1;
            }
        }
    }
    out[tid] = acc;
    n_sec += __shfl_xor_sync(0xFFFFFFFFu, n_sec, 16);
    n_sec += __shfl_xor_sync(0xFFFFFFFFu, n_sec, 8);
    n_sec += __shfl_xor_sync(0xFFFFFFFFu, n_sec, 4);
    n_sec += __shfl_xor_sync(0xFFFFFFFFu, n_sec, 2);
    n_sec += __shfl_xor_sync(0xFFFFFFFFu, n_sec, 1);
    if ((threadIdx.x & 31) == 0) atomicAdd(sectors, (unsigned long long)n_sec);
}

}  // namespace
}  // namespace gbsa

using namespace gbsa;

extern "C" int gbsa_bench_gather_index(const gbsa_index* idx, double* probes_per_s, double* sectors_per_s,
                                       double* gb_per_s) {
    try {
        if (!idx) throw Error(GBSA_ERR_PARAM, "null index");
        GBSA_CUDA(cudaSetDevice(idx->device));
        const IndexView I = view_of(*idx);
        if (I.n == 0) throw Error(GBSA_ERR_PARAM, "empty index");
        const int sms = device_sm_count();
        const unsigned blocks = (unsigned)sms * 8, threads = 256;
        const uint32_t rounds = 32;
        DeviceBuffer out(4ull * blocks * threads), sec(8);
        cudaEvent_t e0, e1;
        GBSA_CUDA(cudaEventCreate(&e0));
        GBSA_CUDA(cudaEventCreate(&e1));
        GBSA_CUDA(cudaMemset(sec.as<void>(), 0, 8));
        k_gather_index<<<blocks, threads>>>(I, rounds, out.as<uint32_t>(), sec.as<unsigned long long>());   // warm-up
        GBSA_LAUNCHED();
        float best = 1e30f;
        for (int rep = 0; rep < 5; ++rep) {
            GBSA_CUDA(cudaMemset(sec.as<void>(), 0, 8));
            GBSA_CUDA(cudaEventRecord(e0));
            k_gather_index<<<blocks, threads>>>(I, rounds, out.as<uint32_t>(), sec.as<unsigned long long>());
            GBSA_LAUNCHED();
            GBSA_CUDA(cudaEventRecord(e1));
            GBSA_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            GBSA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        unsigned long long n_sec = 0;
        GBSA_CUDA(cudaMemcpy(&n_sec, sec.as<void>(), 8, cudaMemcpyDeviceToHost));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double probes = (double)blocks * threads * rounds * 8;
        if (probes_per_s) *probes_per_s = probes / (best / 1e3);
        if (sectors_per_s) *sectors_per_s = (double)n_sec / (best / 1e3);
        if (gb_per_s) *gb_per_s = (double)n_sec * 32.0 / (best / 1e3) / 1e9;
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}

extern "C" int gbsa_bench_gather(uint64_t buffer_bytes, double* sectors_per_s, double* gb_per_s) {
    try {
        if (buffer_bytes < 4096) throw Error(GBSA_ERR_PARAM, "buffer must hold at least 4096 bytes");
        const uint64_t n_sectors = buffer_bytes / 32;
        const int sms = device_sm_count();
        const unsigned blocks = (unsigned)sms * 8, threads = 256;
        const uint32_t rounds = 64;
        DeviceBuffer buf(n_sectors * 32), out(4ull * blocks * threads);
        k_fill<<<(unsigned)sms * 16, 256>>>(buf.as<uint4>(), n_sectors * 2);
        GBSA_LAUNCHED();
        cudaEvent_t e0, e1;
        GBSA_CUDA(cudaEventCreate(&e0));
        GBSA_CUDA(cudaEventCreate(&e1));
        k_gather<<<blocks, threads>>>(buf.as<uint4>(), n_sectors, rounds, out.as<uint32_t>());   // warm-up
        GBSA_LAUNCHED();
        float best = 1e30f;
        for (int rep = 0; rep < 5; ++rep) {
            GBSA_CUDA(cudaEventRecord(e0));
            k_gather<<<blocks, threads>>>(buf.as<uint4>(), n_sectors, rounds, out.as<uint32_t>());
            GBSA_LAUNCHED();
            GBSA_CUDA(cudaEventRecord(e1));
            GBSA_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            GBSA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double sectors = (double)blocks * threads * rounds * 8;
        if (sectors_per_s) *sectors_per_s = sectors / (best / 1e3);
        if (gb_per_s) *gb_per_s = sectors * 32.0 / (best / 1e3) / 1e9;
        return GBSA_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GBSA_ERR_CUDA;
    }
}
