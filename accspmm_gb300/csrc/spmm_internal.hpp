// spmm_internal.hpp -- SpMM entry points shared between translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "accspmm.h"

namespace accspmm {

int sm_count();

// Windows per CTA the launch-shape chooser picks for a matrix signature.
uint32_t window_block_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision);

// One launch of the window-block kernel over W windows described by rwo;
// the launch shape is chosen from (w_cfg, T, K, precision).
// stable_rwo: rwo belongs to a library-owned matrix and stays unchanged
// until schedule_cache_forget(rwo), so a heaviest-first block schedule may be
// computed once and kept for it.  allow_pack: the launch may pack B into TF32
// planes in a buffer from the library's pool first (TF32 shapes with the
// rolling ring).
int spmm_window_launch(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                       const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                       uint32_t T, uint32_t cols, const float* B, float* C, uint32_t K,
                       int precision, cudaStream_t s, bool stable_rwo = false,
                       bool allow_pack = false);
// Drops the block schedules kept for these window offsets (before they are freed).
void schedule_cache_forget(const uint32_t* rwo);
// Epilogue applied when C is stored: C = act(A B + bias[col]).
struct Epilogue {
    const float* bias = nullptr;  // K floats on the device, 16-byte aligned, or nullptr
    uint32_t act = 0;             // ACCSPMM_ACT_NONE / ACCSPMM_ACT_RELU
};

// The same launch restricted to feature slices [slice_begin, slice_begin +
// slice_count) of the chosen slice width (or of slice_fs columns when
// slice_fs is nonzero): identical arithmetic for the columns it covers.
int spmm_window_launch_slices(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                              const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                              uint32_t T, uint32_t cols, const float* B, float* C, uint32_t K,
                              int precision, uint32_t slice_begin, uint32_t slice_count,
                              const Epilogue& epi, cudaStream_t s, int slice_fs,
                              bool stable_rwo = false, bool allow_pack = false);
// Slice width, CTAs per SM (register-direct kernel) and windows per CTA the
// launch-shape chooser picks.
void launch_shape_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision, int* fs, int* occ,
                      uint32_t* wb);
int gather_floor_impl(const accspmm_metcf_t* m, const float* B, uint32_t K, uint32_t slice_width,
                      int repeats, float* avg_ms, void* stream);
// Feature columns per slice the launch-shape chooser picks.
uint32_t slice_width_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision);
// rowWindowOffset of W windows derived from an AdpBME's rowIndices, with the
// rowIndices checked on the way: bits raised when tiles lie past the W windows
// (2) or rowIndices are not non-decreasing multiples of 8 (4) go to *err when
// err is non-null (a zeroed device word) and, when `sticky`, to the device
// status word that accspmm_device_status reports.
int rwo_from_row_indices(const uint32_t* ri, uint32_t T, uint32_t W, uint32_t* rwo, uint32_t* err,
                         bool sticky, cudaStream_t s);
int spmm_host_impl(const accspmm_metcf_t* m, const accspmm_adpbme_t* ad, const float* B_host,
                   float* C_host, uint32_t K, int precision, void* stream, int* direct_c);
int spmm_bias_act_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K,
                       int precision, const float* bias, int act, void* stream);
int gcn_layer_impl(const accspmm_metcf_t* adj, const float* H, uint32_t k_in, const float* W,
                   uint32_t k_out, const float* bias, int act, float* out, int precision,
                   void* stream);
// XW = H W (n x k_in times k_in x k_out, row-major fp32) on the tcgen05
// tensor cores, TF32 or 3xTF32 (dense_gemm.cu).
int dense_gemm_impl(const float* H, uint32_t n, uint32_t k_in, const float* W, uint32_t k_out, float* XW,
                    int precision, cudaStream_t s);
// Reads and clears the dense GEMM's status word (1: a bounded wait expired).
int dense_gemm_status_take(unsigned int* v);
int permute_rows_impl(const float* src, float* dst, const uint32_t* idx, uint32_t rows, uint32_t K,
                      int scatter, void* stream);
int spmm_chain_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, uint32_t hops,
                    int precision, void* stream);
// Per-device memory pool of the library (keeps freed memory for later calls).
int library_pool(cudaMemPool_t* pool);
int autotune_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                  void* stream, accspmm_tune_result_t* out);
void autotune_clear();

int spmm_tf32_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                   void* stream);
// Drops the window offsets cached for an owned AdpBME (before its arrays are freed).
void adaptive_cache_forget(const accspmm_adpbme_t* ad);
// Window offsets of W windows derived from an owned AdpBME's rowIndices, kept
// with the object until accspmm_adpbme_destroy.
int adaptive_rwo(const accspmm_adpbme_t* ad, uint32_t W, cudaStream_t s, const uint32_t** out);
int spmm_adaptive_impl(const accspmm_adpbme_t* ad, const float* B, float* C, uint32_t c_rows,
                       uint32_t K, int precision, void* stream);
int device_status_impl(void* stream);
// Launches one warp whose bounded wait expires on purpose (spmm_bulk.cu).
int bounded_wait_selftest(uint32_t limit_ms, cudaStream_t s);
int spmm_adaptive_noalloc_impl(const accspmm_adpbme_t* ad, const float* B, float* C,
                               uint32_t c_rows, uint32_t K, int precision, void* stream);
uint32_t noalloc_max_c_rows();
int time_spmm_impl(const accspmm_metcf_t* m, const accspmm_adpbme_t* ad, const float* B, float* C,
                   uint32_t c_rows, uint32_t K, int precision, int warmup, int exe, float* avg_ms,
                   void* stream);

}  // namespace accspmm
