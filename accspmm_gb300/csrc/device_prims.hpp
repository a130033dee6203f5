// device_prims.hpp -- device-wide scan and radix sort (device_prims.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace accspmm {

// out[0..n] = exclusive prefix sums of in[0..n) (mod 2^32), out[n] = total.
// `out` may alias `in`.  Temporary memory is stream-ordered.
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs by key bits [0, nbits); the
// sorted pairs land in keys_out / vals_out, which must not alias the inputs.
int radix_sort_pairs(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                     uint32_t* vals_out, size_t n, int nbits, cudaStream_t s);

}  // namespace accspmm
