// common.cuh — shared device helpers of the GB300 strobealign path.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gbsa.h"

namespace gbsa {

constexpr int kWarp = 32;
constexpr uint64_t kNotFound = ~0ULL;
constexpr uint32_t kNoneState = 0xFFFFFFFFu;

// ---- xxh64 reduced to a single u64 (step2/hash.hpp:97-119) ------------------
constexpr uint64_t kP1 = 0x9E3779B185EBCA87ULL;
constexpr uint64_t kP2 = 0xC2B2AE3D27D4EB4FULL;
constexpr uint64_t kP3 = 0x165667B19E3779F9ULL;
constexpr uint64_t kP4 = 0x85EBCA77C2B2AE63ULL;
constexpr uint64_t kP5 = 0x27D4EB2F165667C5ULL;

__host__ __device__ __forceinline__ uint64_t rotl64(uint64_t x, int r) {
    return (x << r) | (x >> (64 - r));
}

__host__ __device__ __forceinline__ uint64_t xxh64(uint64_t v) {
    uint64_t acc = kP5 + 8;
    acc ^= rotl64(v * kP2, 31) * kP1;
    acc = rotl64(acc, 27) * kP1 + kP4;
    acc = (acc ^ (acc >> 33)) * kP2;
    acc = (acc ^ (acc >> 29)) * kP3;
    return acc ^ (acc >> 32);
}

// Nucleotide → 2-bit code, 4 for anything else (step2/randstrobes.hpp:26-43:
// A/a→0, C/c→1, G/g→2, T/t/U/u→3, and raw byte values 0..3 map to themselves).
__host__ __device__ __forceinline__ uint32_t nt4(uint8_t c) {
    if (c < 4) return c;
    const uint8_t u = c & 0xDF;  // upper-case for letters
    if (c >= 'A' && c <= 'z') {
        switch (u) {
            case 'A': return 0;
            case 'C': return 1;
            case 'G': return 2;
            case 'T': return 3;
            case 'U': return 3;
            default: break;
        }
    }
    return 4;
}

// Device copy of the index parameters actually used by the kernels.
struct DevParams {
    int k, s, t;        // t = t_syncmer (1-based offset of the s-mer minimum)
    int W;              // k - s + 1, s-mers per k-mer
    uint32_t w_min, w_max;
    uint64_t q;
    uint32_t max_dist;
    uint64_t kmask, smask;
};

inline DevParams make_dev_params(const gbsa_params& p) {
    DevParams d;
    d.k = p.k;
    d.s = p.s;
    d.t = p.t_syncmer;
    d.W = p.k - p.s + 1;
    d.w_min = p.w_min;
    d.w_max = p.w_max;
    d.q = p.q;
    d.max_dist = (uint32_t)p.max_dist;
    d.kmask = p.k >= 32 ? ~0ULL : ((1ULL << (2 * p.k)) - 1);
    d.smask = p.s >= 32 ? ~0ULL : ((1ULL << (2 * p.s)) - 1);
    return d;
}

// Reverse complement of a 2-bit packed word holding n bases in its low 2n bits
// (first base in the highest pair).  Equals the reference's rolling reverse
// strand word xk[1] / xs[1] (step2/randstrobes.cu:24-26).
__device__ __forceinline__ uint64_t revcomp_bits(uint64_t x, int n) {
    // a bit reversal puts the 2-bit groups in reverse order with the two bits of
    // each group swapped; swapping them back and complementing gives the reverse
    // complement of the 32 bases, of which the last n are kept
    x = __brevll(~x);
    x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
    return n >= 32 ? x : (x >> (64 - 2 * n));
}

// n (<= 32) bases starting at position p of a 2-bit stream packed MSB-first in
// 64-bit words (base i sits in bits 63-2*(i%32) .. 62-2*(i%32) of word i/32).
__device__ __forceinline__ uint64_t extract_bases(const uint64_t* words, uint64_t p, int n) {
    const uint64_t wi = p >> 5;
    const uint32_t sh = (uint32_t)(p & 31) * 2;
    // (lo >> 1) >> (63 - sh) is lo >> (64 - sh) for sh > 0 and 0 for sh == 0
    const uint64_t v = (words[wi] << sh) | ((words[wi + 1] >> 1) >> (63 - sh));
    return n >= 32 ? v : (v >> (64 - 2 * n));
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <class T>
__device__ __forceinline__ T warp_inclusive_sum(T v) {
    const uint32_t l = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (l >= (uint32_t)o) v += n;
    }
    return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Device status word bits (set by kernels, read by the host after a launch).
constexpr uint32_t kStatusQueryOverflow = 1u << 0;
constexpr uint32_t kStatusHitOverflow = 1u << 1;
constexpr uint32_t kStatusNamOverflow = 1u << 2;
constexpr uint32_t kStatusScratchOverflow = 1u << 3;
constexpr uint32_t kStatusSyncmerOverflow = 1u << 4;
constexpr uint32_t kStatusReadTooLong = 1u << 5;

}  // namespace gbsa
