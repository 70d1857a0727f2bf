// pairs.cu — read-pair classification after the NAM sort.
//
// Restates gpu_pre_cal_type (step2/main.cu:3552-3580) with top_dropoff
// (main.cu:889-898) and is_proper_nam_pair (main.cu:870-887): one thread per pair
// reads the two ends' NAM counts and their first NAMs (the first two for the
// dropoff) and writes one type byte.  The bound mu + 10 sigma is computed as one
// fused multiply-add, as nvcc contracts the reference's expression.
#include <cmath>

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

}  // namespace
}  // namespace gbsa

using namespace gbsa;

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
