// gnn.cpp -- the caller the SpMM path exists for: one graph-convolution layer
// out = act(A (H W) + bias), the dense product by cuBLAS, the sparse one by
// the METCF kernel with bias and activation applied as C is stored (no extra
// pass over C).  No counterpart in the reference, whose driver
// (src/mma_tf32.cu:185-243) multiplies A by a constant B only.
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <mutex>

#include "accspmm.h"
#include "common.hpp"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

// One cuBLAS handle per device; calls through it are serialised by `mu`
// (a handle's stream binding is per handle).
struct Blas {
    std::mutex mu;
    cublasHandle_t h = nullptr;
};

int blas_for_device(Blas** out) {
    static std::mutex mu;
    static Blas blas[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        ACC_FAIL(ACCSPMM_ERROR_CUDA, "no current device");
    std::lock_guard<std::mutex> lock(mu);
    if (!blas[dev].h) {
        const cublasStatus_t st = cublasCreate(&blas[dev].h);
        if (st != CUBLAS_STATUS_SUCCESS) ACC_FAIL(ACCSPMM_ERROR_CUDA, "cublasCreate failed (%d)", int(st));
    }
    *out = &blas[dev];
    return ACCSPMM_SUCCESS;
}

}  // namespace

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
    if (n > 0) {
        Blas* b = nullptr;
        r = blas_for_device(&b);
        if (r) {
            cudaFreeAsync(xw, s);
            return r;
        }
        std::lock_guard<std::mutex> lock(b->mu);
        // row-major XW (n x k_out) = H (n x k_in) W (k_in x k_out) is the
        // column-major product W^T-as-stored times H^T-as-stored
        const float one = 1.f, zero = 0.f;
        const cublasComputeType_t ct =
            precision == ACCSPMM_PREC_TF32 ? CUBLAS_COMPUTE_32F_FAST_TF32 : CUBLAS_COMPUTE_32F;
        cublasStatus_t st = cublasSetStream(b->h, s);
        if (st == CUBLAS_STATUS_SUCCESS)
            st = cublasGemmEx(b->h, CUBLAS_OP_N, CUBLAS_OP_N, int(k_out), int(n), int(k_in), &one, W,
                              CUDA_R_32F, int(k_out), H, CUDA_R_32F, int(k_in), &zero, xw, CUDA_R_32F,
                              int(k_out), ct, CUBLAS_GEMM_DEFAULT);
        if (st != CUBLAS_STATUS_SUCCESS) {
            cudaFreeAsync(xw, s);
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "cublasGemmEx failed (%d)", int(st));
        }
    }
    r = spmm_bias_act_impl(adj, xw, out, k_out, precision, bias, act, stream);
    cudaFreeAsync(xw, s);
    return r;
}

}  // namespace accspmm
