// permute.cu -- row permutation of a dense row-major matrix on the device,
// the B-side and C-side companions of a reordered matrix (reorder.cpp):
// gather dst[i] = src[idx[i]] or scatter dst[idx[i]] = src[i], K floats a
// row moved as float4s, eight rows per warp.
#include "common.hpp"
#include "device_util.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

// Each warp moves kRows consecutive rows as one flat run of kRows * k4
// float4s (lane e of a pass takes element e: row e / k4, column e % k4), so
// rows shorter than a warp's 32 float4s still use every lane, and each pass
// issues kBatch loads per lane before their stores.  One row per warp, one
// load in flight, moved 4.3 TB/s at K = 128.
constexpr uint32_t kRows = 8;
constexpr uint32_t kBatch = 4;

__global__ void permute_rows_kernel(const float4* __restrict__ src, float4* __restrict__ dst,
                                    const uint32_t* __restrict__ idx, uint32_t rows, uint32_t k4,
                                    uint32_t scatter) {
    const uint64_t warp = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t r0 = warp * kRows;
    if (r0 >= rows) return;
    // lane q < kRows holds the index of row r0 + q (rows if past the end)
    const uint32_t jl = (lane < kRows && r0 + lane < rows) ? __ldg(idx + r0 + lane) : rows;
    const uint32_t n_el = kRows * k4;
    for (uint32_t e0 = 0; e0 < n_el; e0 += 32 * kBatch) {
        float4 v[kBatch];
        uint64_t dpos[kBatch];
        bool ok[kBatch];
#pragma unroll
        for (uint32_t u = 0; u < kBatch; ++u) {
            const uint32_t e = e0 + 32 * u + lane;
            const uint32_t q = e / k4, c = e - q * k4;
            const uint32_t j = __shfl_sync(0xffffffffu, jl, q < kRows ? q : 0);
            const uint64_t i = r0 + q;
            // past the run, past the last row, or an index outside [0, rows):
            // nothing is read or written
            ok[u] = e < n_el && i < rows && j < rows;
            const uint64_t so = (scatter ? i : uint64_t(j)) * k4 + c;
            dpos[u] = (scatter ? uint64_t(j) : i) * k4 + c;
            if (ok[u]) v[u] = __ldg(src + so);
        }
#pragma unroll
        for (uint32_t u = 0; u < kBatch; ++u)
            if (ok[u]) dst[dpos[u]] = v[u];
    }
}

}  // namespace

int permute_rows_impl(const float* src, float* dst, const uint32_t* idx, uint32_t rows, uint32_t K,
                      int scatter, void* stream) {
    if (!src || !dst || !idx) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null pointer");
    if (src == dst) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "src and dst must not be the same buffer");
    if (K == 0 || K % 4 || ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K must be a multiple of 4 and the matrices 16-byte aligned");
    if (K > (1u << 28)) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "K=%u too large", K);
    if (rows == 0) return ACCSPMM_SUCCESS;
    const uint64_t threads = (uint64_t(rows) + kRows - 1) / kRows * 32;
    const uint64_t blocks = (threads + 255) / 256;
    if (blocks > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "too many rows");
    permute_rows_kernel<<<unsigned(blocks), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(src), reinterpret_cast<float4*>(dst), idx, rows, K / 4,
        scatter ? 1u : 0u);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
