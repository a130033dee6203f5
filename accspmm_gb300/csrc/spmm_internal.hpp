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
int spmm_window_launch(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                       const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                       uint32_t T, uint32_t cols, const float* B, float* C, uint32_t K,
                       int precision, cudaStream_t s);
int autotune_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                  void* stream, accspmm_tune_result_t* out);
void autotune_clear();

int spmm_tf32_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                   void* stream);
int spmm_adaptive_impl(const accspmm_adpbme_t* ad, const float* B, float* C, uint32_t c_rows,
                       uint32_t K, int precision, void* stream);
int device_status_impl(void* stream);
int spmm_adaptive_noalloc_impl(const accspmm_adpbme_t* ad, const float* B, float* C,
                               uint32_t c_rows, uint32_t K, int precision, void* stream);
uint32_t noalloc_max_c_rows();
int time_spmm_impl(const accspmm_metcf_t* m, const accspmm_adpbme_t* ad, const float* B, float* C,
                   uint32_t c_rows, uint32_t K, int precision, int warmup, int exe, float* avg_ms,
                   void* stream);

}  // namespace accspmm
