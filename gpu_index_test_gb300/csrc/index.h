// index.h — the device-resident StrobemerIndex behind the opaque gbsa_index handle.
//
// Layout in HBM (step2/index.hpp:180-182 kept as is, so export is a plain copy):
//   rs      RefRandstrobe[n], 16 B each, sorted by (hash, position, packed)
//   starts  u64[2^bits + 1]  bucket start table; starts[top bits of hash] .. starts[+1]
//           bounds the bucket, with the reference's first-bucket rule
//           (step2/index.cu:207-210: buckets up to the first hash's own start at the
//           second distinct hash)
#pragma once

#include <cstdint>

#include "common.cuh"
#include "runtime.h"

struct gbsa_index {
    gbsa_params params{};
    gbsa::DevParams dp{};
    int bits = 0;
    uint32_t filter_cutoff = 0;
    uint64_t n = 0;
    gbsa_index_info info{};
    int device = 0;
    gbsa::DeviceBuffer rs;       // gbsa_ref_randstrobe[n]
    gbsa::DeviceBuffer starts;   // uint64_t[2^bits + 1]
    gbsa::DeviceBuffer starts32; // uint32_t[2^bits + 1] copy read by the kernels when n < 2^32
};

namespace gbsa {

// Read-only view of the index used by device code.
struct IndexView {
    const gbsa_ref_randstrobe* rs;
    const uint64_t* starts;
    const uint32_t* starts32;   // half-size table (half the L2 footprint), or null
    uint64_t n;
    int bits;
    uint32_t filter_cutoff;
    int k;
};

inline IndexView view_of(const gbsa_index& ix) {
    return IndexView{ix.rs.as<gbsa_ref_randstrobe>(), ix.starts.as<uint64_t>(),
                     ix.starts32.size() ? ix.starts32.as<uint32_t>() : nullptr, ix.n, ix.bits, ix.filter_cutoff,
                     ix.params.k};
}

// Builds the 32-bit copy of the bucket table when every start fits (n < 2^32).
void make_compact_starts(gbsa_index& ix, cudaStream_t st);

// Validates parameters like the reference constructors (step2/indexparameters.hpp:24-68).
bool params_valid(const gbsa_params& p);
int pick_bits_host(const gbsa_params& p, uint64_t total_length);

}  // namespace gbsa
