// spmm_batch.hpp -- batched SpMM: per-matrix descriptors and the launcher
// shared by batch plans and the request server.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "accspmm.h"

namespace accspmm {

// One matrix of a batched launch (device memory, read by the kernel).
struct BatchDesc {
    const uint32_t* rwo;
    const uint32_t* tc_offset;
    const uint64_t* bits;
    const uint32_t* a2b;
    const float* vals;
    const float* B;
    float* C;
    uint32_t W, cols, K;
    uint32_t wb, n_slices, n_wblocks;  // launch shape of this matrix
    uint32_t item0;                    // first work item of this matrix
    uint32_t index;                    // position in the caller's list
    const uint8_t* bp;                 // B packed to TF32 (pack_tf32_put layout), or nullptr
    uint32_t bpitch;                   // bytes per packed row
};

// Host description of one matrix of a batch.
struct BatchInput {
    const uint32_t* rwo;
    const uint32_t* tc_offset;
    const uint64_t* bits;
    const uint32_t* a2b;
    const float* vals;
    const float* B;
    float* C;
    uint32_t W;      // windows computed (C has 8 W rows)
    uint32_t w_cfg;  // windows the launch shape is chosen from
    uint32_t T;
    uint32_t cols;
    uint32_t K;
};

// Slice width of a narrow-group launch whose widest matrix has max_k columns.
int batch_fs_for(uint32_t max_k);
// Whether a batch item runs in the wide group (128-column slices, tile ring).
bool batch_item_is_wide(uint32_t K, int precision);

// Descriptors in launch order (largest first), with item numbering.
int make_batch_descs(const BatchInput* in, uint32_t n, int fs, int precision,
                     std::vector<BatchDesc>* out, uint32_t* total_items, uint32_t* max_wb);

// Resets the work counter and launches the persistent batched kernel.
// packed: every descriptor has a packed B (wide TF32 group only).
int launch_batch(const BatchDesc* d_desc, uint32_t n_desc, uint32_t total_items, uint32_t max_wb,
                 uint32_t* d_counter, int fs, int precision, cudaStream_t s, bool packed = false);

}  // namespace accspmm
