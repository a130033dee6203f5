// capi.cpp -- the extern "C" entry points of include/accspmm.h: argument
// checks, host/device dispatch, copies between memory spaces, destruction.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "accspmm.h"
#include "common.hpp"
#include "host_formats.hpp"
#include "options.hpp"
#include "spmm_internal.hpp"

using namespace accspmm;

namespace {

#define CAPI_CUDA(call)                                                      \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess)                                               \
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "%s failed: %s", #call,             \
                     cudaGetErrorString(e_));                                \
    } while (0)

cudaStream_t st(void* s) { return static_cast<cudaStream_t>(s); }

// Allocates n elements in `space` (stream-ordered on the device).
template <class T>
int alloc_in(int32_t space, size_t n, T** p, cudaStream_t s) {
    *p = nullptr;
    if (space == ACCSPMM_HOST) {
        *p = static_cast<T*>(std::malloc(sizeof(T) * (n ? n : 1)));
        if (!*p) ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation of %zu bytes failed", sizeof(T) * n);
        return ACCSPMM_SUCCESS;
    }
    CAPI_CUDA(cudaMallocAsync(reinterpret_cast<void**>(p), sizeof(T) * (n ? n : 1), s));
    return ACCSPMM_SUCCESS;
}

template <class T>
void free_in(int32_t space, T* p) {
    if (!p) return;
    if (space == ACCSPMM_HOST) std::free(p);
    else cudaFree(p);
}

template <class T>
int copy_arr(T* dst, int32_t dspace, const T* src, int32_t sspace, size_t n, cudaStream_t s) {
    if (n == 0) return ACCSPMM_SUCCESS;
    if (dspace == ACCSPMM_HOST && sspace == ACCSPMM_HOST) {
        std::memcpy(dst, src, sizeof(T) * n);
        return ACCSPMM_SUCCESS;
    }
    CAPI_CUDA(cudaMemcpyAsync(dst, src, sizeof(T) * n, cudaMemcpyDefault, s));
    return ACCSPMM_SUCCESS;
}

bool valid_space(int32_t s) { return s == ACCSPMM_HOST || s == ACCSPMM_DEVICE; }

// A host CSR the host builders may index through: arrays present, row_ptr
// from 0 to nnz without decreasing, columns below cols.
int check_host_csr(const accspmm_csr_t* csr) {
    if (csr->space != ACCSPMM_HOST) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "the CSR must be in host memory");
    if (!csr->row_ptr || (csr->nnz && (!csr->col_idx || !csr->data)))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "CSR arrays missing");
    if (csr->row_ptr[0] != 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr[0] != 0");
    if (csr->row_ptr[csr->rows] != csr->nnz) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr[rows] != nnz");
    for (uint32_t r = 0; r < csr->rows; ++r)
        if (csr->row_ptr[r] > csr->row_ptr[r + 1])
            ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr decreases at row %u", r);
    for (uint32_t i = 0; i < csr->nnz; ++i)
        if (csr->col_idx[i] >= csr->cols) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "column %u >= cols", csr->col_idx[i]);
    return ACCSPMM_SUCCESS;
}

}  // namespace

extern "C" {

const char* accspmm_version(void) { return "accspmm-gb300 0.1.0 (sm_103a)"; }

const char* accspmm_last_error(void) { return last_error(); }

int accspmm_read_mtx(const char* path, accspmm_coo_t* coo) {
    clear_error();
    if (!path || !coo) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    return read_mtx_host(path, coo);
}

int accspmm_csr_from_coo(const accspmm_coo_t* coo, accspmm_csr_t* csr, void* stream) {
    clear_error();
    if (!coo || !csr) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (coo->nnz && (!coo->row || !coo->col || !coo->data))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "COO arrays missing");
    if (coo->space == ACCSPMM_HOST) return csr_from_coo_host(coo, csr);
    if (coo->space == ACCSPMM_DEVICE) return csr_from_coo_device(coo, csr, stream);
    ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad memory space %d", coo->space);
}

int accspmm_metcf_from_csr(const accspmm_csr_t* csr, accspmm_metcf_t* metcf, void* stream) {
    clear_error();
    if (!csr || !metcf) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (!csr->row_ptr || (csr->nnz && (!csr->col_idx || !csr->data)))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "CSR arrays missing");
    if (csr->space == ACCSPMM_HOST) {
        if (int r = check_host_csr(csr)) return r;
        return metcf_from_csr_host(csr, metcf);
    }
    if (csr->space == ACCSPMM_DEVICE) return metcf_from_csr_device(csr, metcf, stream);
    ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad memory space %d", csr->space);
}

int accspmm_adpbme_from_metcf(const accspmm_metcf_t* metcf, uint32_t t_load, uint32_t t_comp,
                              uint32_t t_write, uint32_t target_num, accspmm_adpbme_t* adp,
                              void* stream) {
    clear_error();
    if (!metcf || !adp) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (metcf->space == ACCSPMM_HOST)
        return adpbme_from_metcf_host(metcf, t_load, t_comp, t_write, target_num, adp);
    if (metcf->space == ACCSPMM_DEVICE)
        return adpbme_from_metcf_device(metcf, t_load, t_comp, t_write, target_num, adp, stream);
    ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad memory space %d", metcf->space);
}

int accspmm_balance_strategy(const accspmm_metcf_t* metcf, int* adaptive, void* stream) {
    clear_error();
    if (!metcf || !adaptive) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (metcf->space == ACCSPMM_HOST) {
        *adaptive = balance_strategy_host(metcf->row_window_offset, metcf->num_windows,
                                          metcf->num_tiles);
        return ACCSPMM_SUCCESS;
    }
    if (metcf->space == ACCSPMM_DEVICE) return balance_strategy_device(metcf, adaptive, stream);
    ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad memory space %d", metcf->space);
}

int accspmm_adaptive_c_rows(const accspmm_adpbme_t* adp, uint32_t* c_rows, void* stream) {
    clear_error();
    if (!adp || !c_rows) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    uint64_t by_groups = uint64_t(adp->num_groups) * kWin;
    uint64_t by_rows = 0;
    if (adp->num_tiles) {
        uint32_t last = 0;
        if (adp->space == ACCSPMM_HOST) {
            last = adp->row_indices[adp->num_tiles - 1];
        } else {
            CAPI_CUDA(cudaMemcpyAsync(&last, adp->row_indices + adp->num_tiles - 1, 4,
                                      cudaMemcpyDeviceToHost, st(stream)));
            CAPI_CUDA(cudaStreamSynchronize(st(stream)));
        }
        by_rows = uint64_t(last) + kWin;
    }
    uint64_t r = by_groups > by_rows ? by_groups : by_rows;
    if (r > 0xFFFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "C rows overflow");
    *c_rows = uint32_t(r);
    return ACCSPMM_SUCCESS;
}

int accspmm_coo_copy(const accspmm_coo_t* src, int32_t dst_space, accspmm_coo_t* dst, void* stream) {
    clear_error();
    if (!src || !dst || !valid_space(dst_space) || !valid_space(src->space))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    cudaStream_t s = st(stream);
    accspmm_coo_t d = *src;
    d.space = dst_space;
    d.owned = 1;
    d.row = d.col = nullptr;
    d.data = nullptr;
    int r = alloc_in(dst_space, src->nnz, &d.row, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.col, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.data, s);
    if (!r) r = copy_arr(d.row, dst_space, src->row, src->space, src->nnz, s);
    if (!r) r = copy_arr(d.col, dst_space, src->col, src->space, src->nnz, s);
    if (!r) r = copy_arr(d.data, dst_space, src->data, src->space, src->nnz, s);
    if (!r && (dst_space == ACCSPMM_HOST || src->space == ACCSPMM_HOST))
        CAPI_CUDA(cudaStreamSynchronize(s));
    if (r) {
        accspmm_coo_destroy(&d);
        return r;
    }
    *dst = d;
    return ACCSPMM_SUCCESS;
}

int accspmm_csr_copy(const accspmm_csr_t* src, int32_t dst_space, accspmm_csr_t* dst, void* stream) {
    clear_error();
    if (!src || !dst || !valid_space(dst_space) || !valid_space(src->space))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    cudaStream_t s = st(stream);
    accspmm_csr_t d = *src;
    d.space = dst_space;
    d.owned = 1;
    d.row_ptr = d.col_idx = nullptr;
    d.data = nullptr;
    int r = alloc_in(dst_space, size_t(src->rows) + 1, &d.row_ptr, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.col_idx, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.data, s);
    if (!r) r = copy_arr(d.row_ptr, dst_space, src->row_ptr, src->space, size_t(src->rows) + 1, s);
    if (!r) r = copy_arr(d.col_idx, dst_space, src->col_idx, src->space, src->nnz, s);
    if (!r) r = copy_arr(d.data, dst_space, src->data, src->space, src->nnz, s);
    if (!r && (dst_space == ACCSPMM_HOST || src->space == ACCSPMM_HOST))
        CAPI_CUDA(cudaStreamSynchronize(s));
    if (r) {
        accspmm_csr_destroy(&d);
        return r;
    }
    *dst = d;
    return ACCSPMM_SUCCESS;
}

int accspmm_metcf_copy(const accspmm_metcf_t* src, int32_t dst_space, accspmm_metcf_t* dst,
                       void* stream) {
    clear_error();
    if (!src || !dst || !valid_space(dst_space) || !valid_space(src->space))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    cudaStream_t s = st(stream);
    const size_t W = src->num_windows, T = src->num_tiles;
    accspmm_metcf_t d = *src;
    d.space = dst_space;
    d.owned = 1;
    d.row_window_offset = d.tc_offset = d.sparse_a2b = nullptr;
    d.tc_local_bit = nullptr;
    d.data = nullptr;
    int r = alloc_in(dst_space, W + 1, &d.row_window_offset, s);
    if (!r) r = alloc_in(dst_space, T + 1, &d.tc_offset, s);
    if (!r) r = alloc_in(dst_space, T, &d.tc_local_bit, s);
    if (!r) r = alloc_in(dst_space, T * kWin, &d.sparse_a2b, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.data, s);
    if (!r) r = copy_arr(d.row_window_offset, dst_space, src->row_window_offset, src->space, W + 1, s);
    if (!r) r = copy_arr(d.tc_offset, dst_space, src->tc_offset, src->space, T + 1, s);
    if (!r) r = copy_arr(d.tc_local_bit, dst_space, src->tc_local_bit, src->space, T, s);
    if (!r) r = copy_arr(d.sparse_a2b, dst_space, src->sparse_a2b, src->space, T * kWin, s);
    if (!r) r = copy_arr(d.data, dst_space, src->data, src->space, src->nnz, s);
    if (!r && (dst_space == ACCSPMM_HOST || src->space == ACCSPMM_HOST))
        CAPI_CUDA(cudaStreamSynchronize(s));
    if (r) {
        accspmm_metcf_destroy(&d);
        return r;
    }
    *dst = d;
    return ACCSPMM_SUCCESS;
}

int accspmm_adpbme_copy(const accspmm_adpbme_t* src, int32_t dst_space, accspmm_adpbme_t* dst,
                        void* stream) {
    clear_error();
    if (!src || !dst || !valid_space(dst_space) || !valid_space(src->space))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    cudaStream_t s = st(stream);
    const size_t G = src->num_groups, T = src->num_tiles;
    accspmm_adpbme_t d = *src;
    d.space = dst_space;
    d.owned = 1;
    d.group_offset = d.tc_offset = d.row_indices = d.sparse_a2b = nullptr;
    d.tc_local_bit = nullptr;
    d.data = nullptr;
    int r = alloc_in(dst_space, G + 1, &d.group_offset, s);
    if (!r) r = alloc_in(dst_space, T + 1, &d.tc_offset, s);
    if (!r) r = alloc_in(dst_space, T, &d.row_indices, s);
    if (!r) r = alloc_in(dst_space, T, &d.tc_local_bit, s);
    if (!r) r = alloc_in(dst_space, T * kWin, &d.sparse_a2b, s);
    if (!r) r = alloc_in(dst_space, src->nnz, &d.data, s);
    if (!r) r = copy_arr(d.group_offset, dst_space, src->group_offset, src->space, G + 1, s);
    if (!r) r = copy_arr(d.tc_offset, dst_space, src->tc_offset, src->space, T + 1, s);
    if (!r) r = copy_arr(d.row_indices, dst_space, src->row_indices, src->space, T, s);
    if (!r) r = copy_arr(d.tc_local_bit, dst_space, src->tc_local_bit, src->space, T, s);
    if (!r) r = copy_arr(d.sparse_a2b, dst_space, src->sparse_a2b, src->space, T * kWin, s);
    if (!r) r = copy_arr(d.data, dst_space, src->data, src->space, src->nnz, s);
    if (!r && (dst_space == ACCSPMM_HOST || src->space == ACCSPMM_HOST))
        CAPI_CUDA(cudaStreamSynchronize(s));
    if (r) {
        accspmm_adpbme_destroy(&d);
        return r;
    }
    *dst = d;
    return ACCSPMM_SUCCESS;
}

int accspmm_reorder_rcm(const accspmm_csr_t* csr, uint32_t* perm, uint64_t* bandwidth_before,
                        uint64_t* bandwidth_after) {
    clear_error();
    if (!csr || !perm) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (int r = check_host_csr(csr)) return r;
    return reorder_rcm_host(csr, perm, bandwidth_before, bandwidth_after);
}

int accspmm_csr_permute(const accspmm_csr_t* csr, const uint32_t* perm, accspmm_csr_t* out) {
    clear_error();
    if (!csr || !perm || !out) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (int r = check_host_csr(csr)) return r;
    return csr_permute_host(csr, perm, out);
}

int accspmm_dense_permute_rows(const float* src, float* dst, const uint32_t* idx, uint32_t rows,
                               uint32_t K, int32_t scatter, void* stream) {
    clear_error();
    return permute_rows_impl(src, dst, idx, rows, K, scatter, stream);
}

int accspmm_metcf_save(const accspmm_metcf_t* metcf, const char* path, void* stream) {
    clear_error();
    if (!metcf || !path || !valid_space(metcf->space)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    return metcf_save(metcf, path, stream);
}

int accspmm_metcf_load(const char* path, int32_t space, accspmm_metcf_t* metcf, void* stream) {
    clear_error();
    if (!path || !metcf || !valid_space(space)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    return metcf_load(path, space, metcf, stream);
}

int accspmm_adpbme_save(const accspmm_adpbme_t* adp, const char* path, void* stream) {
    clear_error();
    if (!adp || !path || !valid_space(adp->space)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    return adpbme_save(adp, path, stream);
}

int accspmm_adpbme_load(const char* path, int32_t space, accspmm_adpbme_t* adp, void* stream) {
    clear_error();
    if (!path || !adp || !valid_space(space)) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad argument");
    return adpbme_load(path, space, adp, stream);
}

void accspmm_coo_destroy(accspmm_coo_t* c) {
    if (!c || !c->owned) return;
    free_in(c->space, c->row);
    free_in(c->space, c->col);
    free_in(c->space, c->data);
    std::memset(c, 0, sizeof *c);
}

void accspmm_csr_destroy(accspmm_csr_t* c) {
    if (!c || !c->owned) return;
    free_in(c->space, c->row_ptr);
    free_in(c->space, c->col_idx);
    free_in(c->space, c->data);
    std::memset(c, 0, sizeof *c);
}

void accspmm_metcf_destroy(accspmm_metcf_t* m) {
    if (!m || !m->owned) return;
    if (m->space == ACCSPMM_DEVICE) schedule_cache_forget(m->row_window_offset);
    free_in(m->space, m->row_window_offset);
    free_in(m->space, m->tc_offset);
    free_in(m->space, m->tc_local_bit);
    free_in(m->space, m->sparse_a2b);
    free_in(m->space, m->data);
    std::memset(m, 0, sizeof *m);
}

void accspmm_adpbme_destroy(accspmm_adpbme_t* a) {
    if (!a || !a->owned) return;
    if (a->space == ACCSPMM_DEVICE) adaptive_cache_forget(a);
    free_in(a->space, a->group_offset);
    free_in(a->space, a->tc_offset);
    free_in(a->space, a->row_indices);
    free_in(a->space, a->tc_local_bit);
    free_in(a->space, a->sparse_a2b);
    free_in(a->space, a->data);
    std::memset(a, 0, sizeof *a);
}

int accspmm_spmm_tf32(const accspmm_metcf_t* metcf, const float* B, float* C, uint32_t K,
                      int32_t precision, void* stream) {
    clear_error();
    return spmm_tf32_impl(metcf, B, C, K, precision, stream);
}

int accspmm_spmm_adaptive(const accspmm_adpbme_t* adp, const float* B, float* C, uint32_t c_rows,
                          uint32_t K, int32_t precision, void* stream) {
    clear_error();
    return spmm_adaptive_impl(adp, B, C, c_rows, K, precision, stream);
}

int accspmm_spmm_bias_act(const accspmm_metcf_t* metcf, const float* B, float* C, uint32_t K,
                          int32_t precision, const float* bias, int32_t activation, void* stream) {
    clear_error();
    return spmm_bias_act_impl(metcf, B, C, K, precision, bias, activation, stream);
}

int accspmm_gcn_layer(const accspmm_metcf_t* adj, const float* H, uint32_t k_in, const float* W,
                      uint32_t k_out, const float* bias, int32_t activation, float* out,
                      int32_t precision, void* stream) {
    clear_error();
    return gcn_layer_impl(adj, H, k_in, W, k_out, bias, activation, out, precision, stream);
}

int accspmm_dense_matmul(const float* H, uint32_t n, uint32_t k_in, const float* W, uint32_t k_out,
                         float* XW, int32_t precision, void* stream) {
    clear_error();
    return dense_gemm_impl(H, n, k_in, W, k_out, XW, precision, static_cast<cudaStream_t>(stream));
}

int accspmm_spmm_chain(const accspmm_metcf_t* metcf, const float* B, float* C, uint32_t K,
                       uint32_t hops, int32_t precision, void* stream) {
    clear_error();
    return spmm_chain_impl(metcf, B, C, K, hops, precision, stream);
}

int accspmm_gather_floor(const accspmm_metcf_t* metcf, const float* B, uint32_t K,
                         uint32_t slice_width, int32_t repeats, float* avg_ms, void* stream) {
    clear_error();
#ifdef ACCSPMM_LAB
    return gather_floor_impl(metcf, B, K, slice_width, repeats, avg_ms, stream);
#else
    (void)metcf, (void)B, (void)K, (void)slice_width, (void)repeats, (void)avg_ms, (void)stream;
    ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED,
             "accspmm_gather_floor is a measurement entry point of libaccspmm_lab.so");
#endif
}

int accspmm_set_option(int32_t option, int32_t value) {
    clear_error();
    return set_option(option, value);
}

int accspmm_get_option(int32_t option_id, int32_t* value) {
    clear_error();
    if (!value) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "null argument");
    if (option_id < 0 || option_id > ACCSPMM_OPT_KERNEL)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown option %d", option_id);
    *value = option(option_id);
    return ACCSPMM_SUCCESS;
}

int accspmm_spmm_host(const accspmm_metcf_t* metcf, const accspmm_adpbme_t* adp,
                      const float* B_host, float* C_host, uint32_t K, int32_t precision,
                      void* stream) {
    clear_error();
    return spmm_host_impl(metcf, adp, B_host, C_host, K, precision, stream, nullptr);
}

int accspmm_spmm_adaptive_noalloc(const accspmm_adpbme_t* adp, const float* B, float* C,
                                  uint32_t c_rows, uint32_t K, int32_t precision, void* stream) {
    clear_error();
    return spmm_adaptive_noalloc_impl(adp, B, C, c_rows, K, precision, stream);
}

uint32_t accspmm_noalloc_max_c_rows(void) { return noalloc_max_c_rows(); }

int accspmm_autotune_metcf(const accspmm_metcf_t* metcf, const float* B, float* C, uint32_t K,
                           int32_t precision, void* stream, accspmm_tune_result_t* result) {
    clear_error();
    return autotune_impl(metcf, B, C, K, precision, stream, result);
}

void accspmm_autotune_clear(void) { autotune_clear(); }

int accspmm_device_status(void* stream) {
    clear_error();
    // the SpMM kernels' word (the stream is synchronised first), then the
    // dense GEMM's; both are cleared by reading them
    const int r = device_status_impl(stream);
    unsigned int g = 0;
    const int rg = dense_gemm_status_take(&g);
    if (r) return r;
    if (rg) return rg;
    if (g) ACC_FAIL(ACCSPMM_ERROR_TIMEOUT, "a bounded wait in the dense GEMM kernel expired");
    return ACCSPMM_SUCCESS;
}

int accspmm_selftest_bounded_wait(uint32_t limit_ms, void* stream) {
    clear_error();
    return bounded_wait_selftest(limit_ms, static_cast<cudaStream_t>(stream));
}

int accspmm_time_spmm(const accspmm_metcf_t* metcf, const accspmm_adpbme_t* adp, const float* B,
                      float* C, uint32_t c_rows, uint32_t K, int32_t precision, int32_t warmup,
                      int32_t exe, float* avg_ms, void* stream) {
    clear_error();
    if (!adp && !metcf) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "no matrix");
    return time_spmm_impl(metcf, adp, B, C, c_rows, K, precision, warmup, exe, avg_ms, stream);
}

}  // extern "C"
