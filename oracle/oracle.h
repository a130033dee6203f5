/*
 * oracle.h -- CPU restatement of the AccSpMM METCF SpMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this code; it is the checker that the tests, the smoke check and the CPU
 * baseline leg of bench.py compare the CUDA path against.  Every function
 * cites the reference file:line whose behaviour it restates (paths are
 * relative to the AccSpMM source tree).
 *
 * Parity pin: the format functions (reader, CSR, METCF, AdpBME, balance) are
 * checked in the tests against golden fixtures produced by the reference's own
 * host code (include/mmio.hpp + include/format.hpp compiled from source by
 * oracle/Makefile, target `ref`).  The SpMM functions restate the intended
 * math of include/mma_tf32.cuh (bitmap decode, TF32 rounding with cvt.rna,
 * FP32 accumulation); the reference ships no SpMM golden output, so the SpMM
 * values are checked against an FP64 evaluation of the same METCF decode.
 */
#ifndef ACCSPMM_ORACLE_H
#define ACCSPMM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/mmio.hpp:171-210 (read_from_mtx) with :24-72 (banner),
 * :74-93 (size line) and :106-168 (handle_coo).  Returns the reference's codes
 * (0, -1, -2, 3).  On success *row/*col/*data are malloc'd (free with
 * oracle_free).  Integer-valued files are parsed as integers (the reference
 * scans "%d" into a double, which is undefined behaviour). */
int oracle_read_mtx(const char* path, uint32_t* rows, uint32_t* cols,
                    uint32_t* nnz, uint32_t** row, uint32_t** col,
                    float** data);
void oracle_free(void* p);

/* include/format.hpp:110-142: stable counting sort of COO by row. */
void oracle_csr_from_coo(uint32_t rows, uint32_t nnz, const uint32_t* row,
                         const uint32_t* col, const float* data,
                         uint32_t* row_ptr, uint32_t* col_idx, float* vals);

/* include/format.hpp:215-274 (METCFBit::convertFromCSR), sizes first:
 * number of 8x8 tiles T for the CSR. */
uint64_t oracle_metcf_num_tiles(uint32_t rows, const uint32_t* row_ptr,
                                const uint32_t* col_idx);
/* Fills rwo[W+1], tc_offset[T+1], bits[T], a2b[8T], out_data[nnz]. */
void oracle_metcf_fill(uint32_t rows, const uint32_t* row_ptr,
                       const uint32_t* col_idx, const float* vals,
                       uint32_t* rwo, uint32_t* tc_offset, uint64_t* bits,
                       uint32_t* a2b, float* out_data);

/* include/format.hpp:340-429 (AdpBME::CSR2AdpBME): the greedy group packing
 * over the tile sequence given by rwo.  Returns G; writes group_offset[G+1]
 * when non-NULL. */
uint32_t oracle_adpbme_groups(uint32_t num_windows, const uint32_t* rwo,
                              uint32_t t_load, uint32_t t_comp,
                              uint32_t t_write, uint32_t target_num,
                              uint32_t* group_offset);
/* include/format.hpp:364: rowIndices[t] = first row of tile t's window. */
void oracle_adpbme_row_indices(uint32_t num_windows, const uint32_t* rwo,
                               uint32_t* row_indices);

/* include/utils.hpp:75-85 (balanceStrategy). */
int oracle_balance_strategy(const uint32_t* rwo, uint32_t num_windows,
                            uint32_t num_tiles);

/* TF32 rounding of include/ptx_tf32.hpp:19-24 (cvt.rna.tf32.f32), restated
 * from the PTX ISA definition: round the FP32 significand to 10 bits, to
 * nearest, ties away from zero; NaN/Inf pass through. */
float oracle_tf32_rna(float x);

/* C = decode(METCF) * B in FP64 (no rounding of operands).  B is cols x K
 * row-major, C is (8W) x K row-major.  Tile values are indexed by popcount
 * of the bitmap exactly as include/mma_tf32.cuh:71-79 reads them. */
void oracle_spmm_metcf_f64(uint32_t num_windows, uint32_t cols,
                           const uint32_t* rwo, const uint32_t* tc_offset,
                           const uint64_t* bits, const uint32_t* a2b,
                           const float* vals, const float* B, uint32_t K,
                           double* C);
/* Same decode with both operands rounded to TF32 (rna) and FP32
 * accumulation, tile by tile in tile order, k = 0..7 inside a tile. */
void oracle_spmm_metcf_tf32(uint32_t num_windows, uint32_t cols,
                            const uint32_t* rwo, const uint32_t* tc_offset,
                            const uint64_t* bits, const uint32_t* a2b,
                            const float* vals, const float* B, uint32_t K,
                            float* C);

/* CSR SpMM over the layout of include/format.hpp:96-142.  FP64 variant is an
 * oracle; the FP32 OpenMP variant is the CPU baseline (rows [row_begin,
 * row_end) only, so a bounded sample can be timed).  C has rows x K. */
void oracle_spmm_csr_f64(uint32_t rows, const uint32_t* row_ptr,
                         const uint32_t* col_idx, const float* vals,
                         const float* B, uint32_t K, double* C);
void oracle_spmm_csr_f32_omp(uint32_t row_begin, uint32_t row_end,
                             const uint32_t* row_ptr, const uint32_t* col_idx,
                             const float* vals, const float* B, uint32_t K,
                             float* C, int threads);
int oracle_omp_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
