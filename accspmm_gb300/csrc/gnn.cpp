// gnn.cpp -- the callers the SpMM path exists for: one graph-convolution
// layer out = act(A (H W) + bias), the dense product by the tcgen05 GEMM of
// dense_gemm.cu, the sparse one by the METCF kernel with bias and activation
// applied as C is stored (no extra pass over C); and multi-hop propagation A^h B on the device with
// pool-allocated intermediates.  No counterpart in the reference, whose driver
// (src/mma_tf32.cu:185-243) multiplies A by a constant B only.
#include <cuda_runtime.h>

#include "accspmm.h"
#include "common.hpp"
#include "spmm_internal.hpp"

namespace accspmm {

int gcn_layer_impl(const accspmm_metcf_t* adj, const float* H, uint32_t k_in, const float* W,
                   uint32_t k_out, const float* bias, int act, float* out, int precision,
                   void* stream) {
    if (!adj || adj->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    if (!H || !W || !out) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "H, W and out must be device pointers");
    if (k_in == 0 || k_out == 0 || k_out % 4)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "k_in > 0 and k_out a positive multiple of 4 required");
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaMemPool_t pool = nullptr;
    int r = library_pool(&pool);
    if (r) return r;
    const uint32_t n = adj->cols;  // rows of H
    float* xw = nullptr;
    cudaError_t ce = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&xw), size_t(n) * k_out * 4 + 16, pool, s);
    if (ce != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_ALLOC, "pool allocation failed: %s", cudaGetErrorString(ce));
    // XW = H W on the tensor cores (dense_gemm.cu), TF32 or 3xTF32 as the SpMM
    r = dense_gemm_impl(H, n, k_in, W, k_out, xw, precision, s);
    if (r) {
        cudaFreeAsync(xw, s);
        return r;
    }
    r = spmm_bias_act_impl(adj, xw, out, k_out, precision, bias, act, stream);
    cudaFreeAsync(xw, s);
    return r;
}

int spmm_chain_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, uint32_t hops,
                    int precision, void* stream) {
    if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    if (m->rows != m->cols) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "a chain needs a square matrix");
    if (hops == 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "hops must be at least 1");
    if (hops == 1) return spmm_tf32_impl(m, B, C, K, precision, stream);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaMemPool_t pool = nullptr;
    int r = library_pool(&pool);
    if (r) return r;
    // hops - 1 intermediates ping-pong between two pool buffers of 8W x K
    const size_t bytes = size_t(m->num_windows) * 8 * K * 4 + 16;
    float* t[2] = {nullptr, nullptr};
    for (int i = 0; i < (hops > 2 ? 2 : 1) && !r; ++i) {
        cudaError_t ce = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&t[i]), bytes, pool, s);
        if (ce != cudaSuccess) {
            r = ACCSPMM_ERROR_ALLOC;
            set_error("pool allocation failed: %s", cudaGetErrorString(ce));
        }
    }
    const float* in = B;
    for (uint32_t h = 0; h < hops && !r; ++h) {
        float* out = h + 1 == hops ? C : t[h & 1];
        r = spmm_tf32_impl(m, in, out, K, precision, stream);
        in = out;
    }
    for (float* p : t)
        if (p) cudaFreeAsync(p, s);
    return r;
}

}  // namespace accspmm
