/* Forced-include shim for compiling the reference's CPU sources with the host C++
 * compiler (oracle/build_ref.sh).  Compiled by nvcc, the reference's
 * `__device__ static unsigned char seq_nt4_table[256]` (step2/randstrobes.hpp:26) is a
 * device variable, and host code reads an uninitialised host shadow of it, so the
 * host SyncmerIterator sees every base as 'A'.  Built as plain C++ the table is an
 * ordinary initialised host array.  The CUDA qualifiers come from cuda_runtime.h;
 * the one device intrinsic used in header-defined device functions gets a host
 * definition here. */
#pragma once
#include <cuda_runtime.h>
#define __popcll(x) __builtin_popcountll(x)
