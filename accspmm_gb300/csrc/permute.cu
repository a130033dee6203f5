// permute.cu -- row permutation of a dense row-major matrix on the device,
// the B-side and C-side companions of a reordered matrix (reorder.cpp):
// gather dst[i] = src[idx[i]] or scatter dst[idx[i]] = src[i], K floats a
// row moved as float4s, one warp per row.
#include "common.hpp"
#include "device_util.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

__global__ void permute_rows_kernel(const float4* __restrict__ src, float4* __restrict__ dst,
                                    const uint32_t* __restrict__ idx, uint32_t rows, uint32_t k4,
                                    uint32_t scatter) {
    const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (warp >= rows) return;
    const uint32_t i = uint32_t(warp), j = idx[i];
    if (j >= rows) return;  // rejected on the host side; never reads or writes out of range
    const float4* s = src + uint64_t(scatter ? i : j) * k4;
    float4* d = dst + uint64_t(scatter ? j : i) * k4;
    for (uint32_t c = lane; c < k4; c += 32) d[c] = s[c];
}

}  // namespace

int permute_rows_impl(const float* src, float* dst, const uint32_t* idx, uint32_t rows, uint32_t K,
                      int scatter, void* stream) {
    if (!src || !dst || !idx) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null pointer");
    if (src == dst) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "src and dst must not be the same buffer");
    if (K == 0 || K % 4 || ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K must be a multiple of 4 and the matrices 16-byte aligned");
    if (rows == 0) return ACCSPMM_SUCCESS;
    const uint64_t threads = uint64_t(rows) * 32;
    const uint64_t blocks = (threads + 255) / 256;
    if (blocks > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "too many rows");
    permute_rows_kernel<<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(src), reinterpret_cast<float4*>(dst), idx, rows, K / 4,
        scatter ? 1u : 0u);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
