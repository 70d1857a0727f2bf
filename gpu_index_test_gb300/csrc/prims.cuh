// prims.cuh — device-wide primitives: exclusive scan and a stable LSD radix sort of
// 16-byte RefRandstrobe records.  Hand-written; no library sort or scan is used.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "runtime.h"

namespace gbsa {

// Exclusive prefix sum of n u64 values (in may equal out).  If total is non-null it
// receives the sum (device pointer).  Uses ws for block partials.
void scan_exclusive_u64(const uint64_t* in, uint64_t* out, size_t n, uint64_t* d_total, Workspace& ws,
                        cudaStream_t st);

// Sorts n RefRandstrobe records by (hash, position), stably: records that tie on both
// keep their input order.  a and b are two device buffers of n records; returns the
// one holding the result.  Skips digit passes whose digit is constant over the input.
gbsa_ref_randstrobe* radix_sort_ref_randstrobes(gbsa_ref_randstrobe* a, gbsa_ref_randstrobe* b, size_t n,
                                                Workspace& ws, cudaStream_t st);

}  // namespace gbsa
