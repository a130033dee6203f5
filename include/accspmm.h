/*
 * accspmm.h -- C ABI of the GB300 METCF SpMM library (libaccspmm.so).
 *
 * Drop-in boundary for the AccSpMM path: Matrix Market load -> CSR -> METCF
 * (8x8 row-window tiles with 64-bit occupancy bitmaps) -> load-balance choice
 * -> AdpBME grouping -> TF32 tensor-core SpMM C = A * B.  Each entry point
 * names the reference interface it replaces (paths relative to the AccSpMM
 * source tree).  The reference has no library ABI; its interface is the set of
 * header-only C++ calls made by src/mma_tf32.cu, and this header restates each
 * of them with plain pointers and sizes.
 *
 * Conventions
 *  - Every function returns an int status (ACCSPMM_SUCCESS == 0).  Codes that
 *    exist in include/common.hpp:71-95 keep their numeric values.  Errors are
 *    returned, never printed and ignored (the reference prints CUDA errors
 *    and continues, include/utils.hpp:6-22); accspmm_last_error() gives the
 *    message of the calling thread's last failure.
 *  - Index and offset arrays are uint32 like the reference's `vint`;
 *    products with the feature width are computed in 64-bit.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Device work is enqueued on it; functions that must return a
 *    host value (sizes, flags) synchronise that stream, and the builders
 *    (CSR, METCF, AdpBME) return only when their inputs are no longer read.
 *    Inputs of the SpMM calls must stay allocated until the stream's work is
 *    done; *_destroy frees immediately (cudaFree) and must not race with
 *    queued work that reads the object.
 *  - Objects whose `space` is ACCSPMM_DEVICE hold device pointers.  Objects
 *    filled by the library own their arrays; release them with the matching
 *    *_destroy call.  Objects a caller fills by hand are never freed by the
 *    library.
 *  - Dense matrices are row-major float32: B has `cols` rows and K columns,
 *    C has 8 * num_windows rows (plain path) or `c_rows` rows (adaptive path)
 *    and K columns; K must be a positive multiple of 4 and B, C 16-byte
 *    aligned.
 */
#ifndef ACCSPMM_H
#define ACCSPMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    ACCSPMM_SUCCESS = 0,              /* SUCCESS            common.hpp:83 */
    ACCSPMM_ERROR_NOT_MATCH = 1,      /* ERROR_NOT_MATCH    common.hpp:72 */
    ACCSPMM_ERROR_OPEN_FILE = 2,      /* ERROR_OPEN_FILE    common.hpp:73 */
    ACCSPMM_ERROR_READ_MTX = 3,       /* ERROR_READ_MTX     common.hpp:74 */
    ACCSPMM_ERROR_ARGS = 4,           /* ERROR_ARGS         common.hpp:75 */
    ACCSPMM_MM_LOADING_FILE_ERROR = -1, /* common.hpp:84 */
    ACCSPMM_MM_READ_BANNER_ERROR = -2,  /* common.hpp:85 */
    ACCSPMM_RET_ERROR = -4,             /* common.hpp:86 */
    ACCSPMM_MM_PREMATURE_EOF = 12,      /* common.hpp:90 */
    ACCSPMM_MM_UNSUPPORTED_TYPE = 15,   /* common.hpp:93 */
    /* no counterpart in the reference */
    ACCSPMM_ERROR_INVALID_VALUE = 30,
    ACCSPMM_ERROR_ALLOC = 31,
    ACCSPMM_ERROR_CUDA = 32,
    ACCSPMM_ERROR_UNSUPPORTED = 33,
    ACCSPMM_ERROR_OVERFLOW = 34,
    ACCSPMM_ERROR_TIMEOUT = 35,
    ACCSPMM_ERROR_ADMISSION = 36,
    ACCSPMM_ERROR_CANCELLED = 37,
    ACCSPMM_ERROR_FORMAT = 38  /* a binary METCF / AdpBME file is invalid */
};

/* arithmetic of the SpMM */
enum {
    ACCSPMM_PREC_TF32 = 0,   /* both operands rounded to TF32 (cvt.rna), FP32 accumulate */
    ACCSPMM_PREC_3XTF32 = 1  /* hi/lo TF32 splits of A and B, three MMAs, FP32 accumulate */
};

/* activation of the SpMM epilogue */
enum { ACCSPMM_ACT_NONE = 0, ACCSPMM_ACT_RELU = 1 };

/* memory space of an object's arrays */
enum { ACCSPMM_HOST = 0, ACCSPMM_DEVICE = 1 };

/* ---- formats ----------------------------------------------------------- */
/* COO<T>, include/format.hpp:33-94 (0-based indices). */
typedef struct accspmm_coo {
    uint32_t rows, cols, nnz;
    uint32_t* row;
    uint32_t* col;
    float* data;
    int32_t space;
    int32_t owned;
} accspmm_coo_t;

/* CSR<T>, include/format.hpp:96-169. */
typedef struct accspmm_csr {
    uint32_t rows, cols, nnz;
    uint32_t* row_ptr;   /* [rows + 1] */
    uint32_t* col_idx;   /* [nnz] */
    float* data;         /* [nnz] */
    int32_t space;
    int32_t owned;
} accspmm_csr_t;

/* METCFBit<T>, include/format.hpp:202-274.  W = ceil(rows / 8) row windows,
 * T tiles of 8 rows x 8 distinct columns. */
typedef struct accspmm_metcf {
    uint32_t rows, cols, nnz;
    uint32_t num_windows;          /* W */
    uint32_t num_tiles;            /* T */
    uint32_t* row_window_offset;   /* [W + 1] rowWindowOffset */
    uint32_t* tc_offset;           /* [T + 1] tcOffset */
    uint64_t* tc_local_bit;        /* [T]     tcLocalBit, bit (r%8)*8 + c%8 */
    uint32_t* sparse_a2b;          /* [8T]    sparseA2B, UINT32_MAX = padding */
    float* data;                   /* [nnz]   values, tile by tile */
    int32_t space;
    int32_t owned;
} accspmm_metcf_t;

/* AdpBME<T>, include/format.hpp:327-429. */
typedef struct accspmm_adpbme {
    uint32_t rows, cols, nnz;
    uint32_t num_tiles;            /* T */
    uint32_t num_groups;           /* G */
    uint32_t* group_offset;        /* [G + 1] groupOffset */
    uint32_t* tc_offset;           /* [T + 1] */
    uint32_t* row_indices;         /* [T]     first row of each tile's window */
    uint64_t* tc_local_bit;        /* [T] */
    uint32_t* sparse_a2b;          /* [8T] */
    float* data;                   /* [nnz] */
    int32_t space;
    int32_t owned;
} accspmm_adpbme_t;

/* ---- library ----------------------------------------------------------- */
const char* accspmm_version(void);
/* Message of the calling thread's most recent failing call ("" if none). */
const char* accspmm_last_error(void);

/* ---- loading and conversion (host) -------------------------------------- */
/* read_from_mtx<float>, include/mmio.hpp:171-210 (with mm_read_banner :24,
 * mm_read_mtx_crd_size :74, handle_coo :106).  Same return codes: 0,
 * MM_LOADING_FILE_ERROR, MM_READ_BANNER_ERROR, ERROR_READ_MTX.  Symmetric and
 * Hermitian files are expanded (nnz' = 2 nnz - diag) in the reference's
 * order; pattern -> 1.0; complex keeps the real part.  Unlike the reference,
 * integer values are parsed as integers, and a truncated or out-of-range
 * entry list returns ERROR_READ_MTX instead of undefined data.  The body is
 * parsed on all host threads. */
int accspmm_read_mtx(const char* path, accspmm_coo_t* coo);

/* CSR<T>::CSR(const COO<T>*), include/format.hpp:110-142: stable counting
 * sort by row.  Host -> host, or device -> device when coo->space is
 * ACCSPMM_DEVICE (stream-ordered). */
int accspmm_csr_from_coo(const accspmm_coo_t* coo, accspmm_csr_t* csr,
                         void* stream);

/* METCFBit<T>::convertFromCSR, include/format.hpp:215-274.  Bit-exact with
 * the reference layout.  Host CSR -> host METCF on all host threads; device
 * CSR -> device METCF built by CUDA kernels on `stream`.  The device
 * builders' temporaries (about 24 bytes a nonzero at their peak) come from
 * the library's memory pool per device, which keeps freed memory for later
 * calls instead of returning it at each synchronize. */
int accspmm_metcf_from_csr(const accspmm_csr_t* csr, accspmm_metcf_t* metcf,
                           void* stream);

/* AdpBME<T>::CSR2AdpBME(csr, t_load, t_comp, t_write, target_num),
 * include/format.hpp:340-429, computed from an existing METCF (the per-tile
 * arrays are identical; the reference recomputes them).  Host or device, by
 * metcf->space.  The reference's driver uses (3, 1, 2, 16),
 * src/mma_tf32.cu:222. */
int accspmm_adpbme_from_metcf(const accspmm_metcf_t* metcf, uint32_t t_load,
                              uint32_t t_comp, uint32_t t_write,
                              uint32_t target_num, accspmm_adpbme_t* adp,
                              void* stream);

/* balanceStrategy, include/utils.hpp:75-85: *adaptive = 1 when the window
 * imbalance degree exceeds IMBALANCE_THRESHOLD (8).  Host or device. */
int accspmm_balance_strategy(const accspmm_metcf_t* metcf, int* adaptive,
                             void* stream);

/* Number of C rows the adaptive path writes: max(8 G, rowIndices.back() + 8),
 * src/mma_tf32.cu:112. */
int accspmm_adaptive_c_rows(const accspmm_adpbme_t* adp, uint32_t* c_rows,
                            void* stream);

/* Copies between host and device (the H2D/D2H of src/mma_tf32.cu:53-68,
 * :139-156).  The destination is library-owned.  A copy from or to host
 * memory has completed when the call returns. */
int accspmm_metcf_copy(const accspmm_metcf_t* src, int32_t dst_space,
                       accspmm_metcf_t* dst, void* stream);
int accspmm_csr_copy(const accspmm_csr_t* src, int32_t dst_space,
                     accspmm_csr_t* dst, void* stream);
int accspmm_coo_copy(const accspmm_coo_t* src, int32_t dst_space,
                     accspmm_coo_t* dst, void* stream);
int accspmm_adpbme_copy(const accspmm_adpbme_t* src, int32_t dst_space,
                        accspmm_adpbme_t* dst, void* stream);

/* Locality reordering.  No counterpart in the reference, whose benchmark
 * matrix was reordered offline.  accspmm_reorder_rcm computes a reverse
 * Cuthill-McKee numbering of a square host CSR (on the pattern of A + A^T,
 * pseudo-peripheral start vertex per connected component):
 * perm[new] = old, `rows` entries.  The bandwidth max |row - col| before and
 * after is reported if the pointers are non-NULL.  accspmm_csr_permute forms
 * P A P^T on the host (A'[i, j] = A[perm[i], perm[j]], each row's columns
 * sorted); the result is library-owned.  With it, A B = P^T (A' (P B)):
 * accspmm_dense_permute_rows gathers (scatter = 0: dst[i] = src[idx[i]]) or
 * scatters (scatter = 1: dst[idx[i]] = src[i]) the K-float rows of a device
 * matrix by a device index array of `rows` entries, which must be a
 * permutation of 0..rows-1 (entries >= rows are skipped). */
int accspmm_reorder_rcm(const accspmm_csr_t* csr, uint32_t* perm,
                        uint64_t* bandwidth_before, uint64_t* bandwidth_after);
int accspmm_csr_permute(const accspmm_csr_t* csr, const uint32_t* perm,
                        accspmm_csr_t* out);
int accspmm_dense_permute_rows(const float* src, float* dst, const uint32_t* idx,
                               uint32_t rows, uint32_t K, int32_t scatter,
                               void* stream);

/* Binary METCF / AdpBME files.  No counterpart in the reference, which
 * re-parses the .mtx text and rebuilds METCF on every run
 * (src/mma_tf32.cu:196-222).  A file holds the struct's sizes and arrays, each
 * with a 64-bit checksum; little-endian hosts only.  *_save accepts a host or
 * device object (a device one is copied to the host first).  *_load reads
 * into `space` (a library-owned object; release it with *_destroy) and
 * validates the arrays -- offsets monotone and matching the sizes, bitmap
 * popcounts no larger than the per-tile value counts, columns in range or padding
 * -- so that a damaged file returns ACCSPMM_ERROR_FORMAT (truncation, wrong
 * magic or version, checksum or consistency failure) instead of reaching a
 * kernel.  ACCSPMM_ERROR_OPEN_FILE if the file cannot be opened or written. */
int accspmm_metcf_save(const accspmm_metcf_t* metcf, const char* path, void* stream);
int accspmm_metcf_load(const char* path, int32_t space, accspmm_metcf_t* metcf,
                       void* stream);
int accspmm_adpbme_save(const accspmm_adpbme_t* adp, const char* path, void* stream);
int accspmm_adpbme_load(const char* path, int32_t space, accspmm_adpbme_t* adp,
                        void* stream);

void accspmm_coo_destroy(accspmm_coo_t* coo);
void accspmm_csr_destroy(accspmm_csr_t* csr);
void accspmm_metcf_destroy(accspmm_metcf_t* metcf);
void accspmm_adpbme_destroy(accspmm_adpbme_t* adp);

/* ---- SpMM ---------------------------------------------------------------- */
/* TF32Compute::compute, include/tf32_comp.hpp:52-80 (kernels
 * tf32_mma_kernel / tf32_mma_g512_kernel, include/mma_tf32.cuh:13-550), one
 * launch, no timing loop.  C = decode(METCF) * B over all 8W rows; C is
 * fully written (rows of empty windows become 0).  Device METCF, B, C.
 * Launches of a few waves of a library-owned METCF run their window blocks
 * heaviest first: the first such call per (matrix, window block size) sorts
 * the blocks on the GPU, waits for that on the host once, and keeps the
 * schedule until accspmm_metcf_destroy (results do not depend on it).
 * Calls may be captured into a CUDA graph; a call captured before the
 * schedule exists runs the blocks in window order.  In TF32 with K <= 32 or
 * K > 48 and a B of at least 4 MiB (or as a tuned shape says) a call first
 * rounds B to TF32 and packs each row to 2.5 bytes a value in a buffer of
 * 320 cols ceil(K / 128) bytes (160 cols at K <= 64, 80 cols at K <= 32)
 * from the library's memory pool (released in stream order): the SpMM then
 * gathers 10 instead of 16 sectors of each 128-column row slice (5 of 8 of
 * a 64-column one, 3 of 4 of a 32-column one),
 * with bit-identical results, and at 128- and 64-column slices prefetches
 * into L2 the rows of the tile group two ahead of the one it loads (when K
 * spans an odd number of slices).
 * ACCSPMM_OPT_PACK and ACCSPMM_OPT_PREFETCH (accspmm_set_option) turn them
 * off or on. */
int accspmm_spmm_tf32(const accspmm_metcf_t* metcf, const float* B, float* C,
                      uint32_t K, int32_t precision, void* stream);

/* TF32Compute::adpBalanceCompute, include/tf32_comp.hpp:82-113 (kernels
 * tf32_mma_balance_kernel / _g128_kernel, include/mma_tf32.cuh:552-1042),
 * one launch.  Load balance follows the AdpBME tile order; partial row
 * windows are summed in a fixed order (no float atomics), so the result is
 * deterministic.  C has c_rows rows (accspmm_adaptive_c_rows) and is
 * overwritten, where the reference accumulated into a pre-zeroed C.  The
 * window offsets derived from rowIndices (4 (c_rows/8 + 2) bytes) are kept
 * with a library-owned AdpBME after its first call, until
 * accspmm_adpbme_destroy: that first call per (object, c_rows) derives them
 * and waits for them on the host once, and must not be captured into a CUDA
 * graph (it returns ACCSPMM_ERROR_UNSUPPORTED inside a capture); later calls
 * may be captured.  For an AdpBME the caller filled they are derived into
 * stream-ordered scratch on every call.  B is packed as in accspmm_spmm_tf32.
 * The derivation checks rowIndices: tiles whose window lies at or past
 * c_rows / 8 (a c_rows below rowIndices.back() + 8, the reference's sizing
 * rule, src/mma_tf32.cu:112) and rowIndices that are not non-decreasing
 * multiples of 8 (include/format.hpp:364 writes each tile's window start).
 * For a library-owned AdpBME the call returns ACCSPMM_ERROR_INVALID_VALUE
 * (every call with that c_rows); for a caller-filled one the call is enqueued
 * and accspmm_device_status reports ACCSPMM_ERROR_INVALID_VALUE afterwards
 * (tiles past c_rows are then missing from C, misordered ones may be summed
 * into the wrong windows; no read leaves the arrays). */
int accspmm_spmm_adaptive(const accspmm_adpbme_t* adp, const float* B,
                          float* C, uint32_t c_rows, uint32_t K,
                          int32_t precision, void* stream);

/* accspmm_spmm_tf32 with an epilogue applied as C is stored:
 * C = act(A B + bias), bias[j] added to column j (bias: K floats on the
 * device, 16-byte aligned, or NULL), act ACCSPMM_ACT_NONE or _RELU.  Rows of
 * C past the matrix's rows (padding of the last window) hold act(bias).
 * Bit-identical to accspmm_spmm_tf32 followed by a separate FP32 bias add and
 * activation.  No counterpart in the reference. */
int accspmm_spmm_bias_act(const accspmm_metcf_t* metcf, const float* B, float* C,
                          uint32_t K, int32_t precision, const float* bias,
                          int32_t activation, void* stream);

/* One graph-convolution layer, out = act(A (H W) + bias): H is cols x k_in,
 * W is k_in x k_out (row-major, device), out is 8 num_windows x k_out.  H W
 * is computed by accspmm_dense_matmul (tcgen05 tensor cores, TF32 or 3xTF32
 * as `precision` says) into a buffer from the library's memory pool, then
 * multiplied by A with the bias/activation epilogue of accspmm_spmm_bias_act.
 * k_out must be a multiple of 4.  No counterpart in the reference. */
int accspmm_gcn_layer(const accspmm_metcf_t* adj, const float* H, uint32_t k_in,
                      const float* W, uint32_t k_out, const float* bias,
                      int32_t activation, float* out, int32_t precision,
                      void* stream);

/* Dense product XW = H W on the device: H is n x k_in, W is k_in x k_out and
 * XW is n x k_out, all row-major fp32 (XW 16-byte aligned, k_out a positive
 * multiple of 4).  The dense half of accspmm_gcn_layer, run on the tcgen05
 * tensor cores with the accumulator in tensor memory: TF32 (both operands
 * rounded with cvt.rna, FP32 accumulation) or 3xTF32 (hi/lo splits, near-FP32
 * accuracy).  Temporary buffers (W transposed; H repacked when k_in is not a
 * multiple of 4 or H is not 16-byte aligned) come from the library's memory
 * pool; n = 0 is a no-op.  Enqueued on `stream`; a bounded wait that expires inside the kernel
 * is reported by accspmm_device_status.  No counterpart in the reference
 * (its driver multiplies A by a constant B only, src/mma_tf32.cu:185-243). */
int accspmm_dense_matmul(const float* H, uint32_t n, uint32_t k_in, const float* W,
                         uint32_t k_out, float* XW, int32_t precision, void* stream);

/* Multi-hop propagation C = A^hops B of a square matrix, all on the device:
 * hops launches of accspmm_spmm_tf32, each product feeding the next through
 * intermediates (8 num_windows x K) from the library's memory pool, no host
 * round trip.  The two-hop case is the A (A B) chain of the request server.
 * No counterpart in the reference. */
int accspmm_spmm_chain(const accspmm_metcf_t* metcf, const float* B, float* C,
                       uint32_t K, uint32_t hops, int32_t precision, void* stream);

/* SpMM with B and C in host memory: the host wrappers tf32_spmm and
 * adp_tf32_spmm, src/mma_tf32.cu:12-183 (device buffers, B copied in, one
 * kernel, C copied out), as one pipelined call.  Pass exactly one of `metcf`
 * (plain path) and `adp` (adaptive path), on the device.  B_host has `cols`
 * rows and K columns; C_host receives A * B as 8 * ceil(rows / 8) rows of K
 * columns (both paths; the adaptive path's extra zero rows are not written).
 * The work is cut into feature slices of about a quarter of K (32 to 64
 * columns), and the host-to-device copy of slice i + 1 overlaps the kernel
 * of slice i.  For a library-owned AdpBME the first call derives and keeps
 * its window offsets (one host wait), as accspmm_spmm_adaptive does.
 * When C_host is page-locked (cudaHostAlloc / cudaHostRegister) and 16-byte
 * aligned the kernel writes C straight into it over the host link;
 * otherwise C is staged on the device and copied back slice by slice.
 * Page-locked B_host lets its copies run asynchronously.  Results are
 * bit-identical to accspmm_spmm_tf32 / accspmm_spmm_adaptive on the same
 * inputs.  Device buffers come from a library memory pool per device that
 * keeps its memory for later calls.  Enqueued on `stream`: C_host is
 * complete once the stream's work up to this call is done; B_host and
 * C_host must stay valid until then. */
int accspmm_spmm_host(const accspmm_metcf_t* metcf, const accspmm_adpbme_t* adp,
                      const float* B_host, float* C_host, uint32_t K,
                      int32_t precision, void* stream);

/* Allocation-free variant of accspmm_spmm_adaptive, for callers that cannot
 * allocate device memory at call time: plugins inside a host application
 * that owns all device memory through its own pool (a cudaMalloc outside
 * that pool can fail once the pool holds the memory, and escapes the host's
 * accounting), latency-critical loops (cudaFree synchronises the device and
 * stalls every other stream), and processes whose device memory is budgeted
 * once at start-up.  No counterpart in the reference.  It calls no cudaMalloc, cudaFree or other
 * allocating routine: its scratch (the row-window offsets derived from
 * rowIndices, 4 (c_rows / 8 + 2) bytes) lives in a 4 MiB array compiled into
 * the library, which every GPU that loads the library holds until the
 * process exits.  c_rows may be at most accspmm_noalloc_max_c_rows()
 * (8,388,592); larger sizes return ACCSPMM_ERROR_INVALID_VALUE.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress)
 * and caches it for the life of the process; make that first call before any
 * stream capture, and do not call this entry point after a cudaDeviceReset
 * (the cached address belongs to the context the reset destroyed).  Every call
 * shares the one array and leaves the last call's contents in it, so calls
 * that overlap on the GPU (unordered streams) race; order them on one stream
 * or with events.  Same inputs and outputs as accspmm_spmm_adaptive and the
 * same bits; rowIndices are checked in stream order and inconsistencies are
 * reported by accspmm_device_status, as for a caller-filled AdpBME there.
 * Unlike accspmm_spmm_adaptive it never packs B (the packed copy would need
 * 320 cols ceil(K / 128) bytes of scratch): on a B of 4 MiB or more at
 * K <= 32 or K > 48 it runs the kernel that reads fp32 B, 2.29 against 1.64 ms per call
 * on the 1M-row power-law matrix at K = 128 (GB300). */
int accspmm_spmm_adaptive_noalloc(const accspmm_adpbme_t* adp, const float* B,
                                  float* C, uint32_t c_rows, uint32_t K,
                                  int32_t precision, void* stream);
uint32_t accspmm_noalloc_max_c_rows(void);

/* The timing loop of TF32Compute::executeKernel, include/tf32_comp.hpp:33-46:
 * `warmup` untimed launches, then `exe` launches between two CUDA events on
 * `stream`; *avg_ms = elapsed / exe.  `adp` may be NULL (plain path). */
int accspmm_time_spmm(const accspmm_metcf_t* metcf, const accspmm_adpbme_t* adp,
                      const float* B, float* C, uint32_t c_rows, uint32_t K,
                      int32_t precision, int32_t warmup, int32_t exe,
                      float* avg_ms, void* stream);

/* Measurement build only (libaccspmm_lab.so; the product library returns
 * ACCSPMM_ERROR_UNSUPPORTED): the gather floor of accspmm_spmm_tf32 on this matrix and B --
 * the average time (one warm-up, then `repeats` launches timed with CUDA
 * events on `stream`) of a kernel that moves exactly the B rows the SpMM
 * kernel gathers, with the SpMM's launch shape, lane pattern and batching
 * (slice_width 0), or with the register-direct shape of another slice width
 * (32, 64 or 128 columns), and does nothing else (no sparse values, MMAs or
 * C stores).  The SpMM's time over the fastest floor is how much its
 * arithmetic and bookkeeping cost on top of its unavoidable row gathers.  No
 * counterpart in the reference. */
int accspmm_gather_floor(const accspmm_metcf_t* metcf, const float* B, uint32_t K,
                         uint32_t slice_width, int32_t repeats, float* avg_ms,
                         void* stream);

/* ---- autotuning ----------------------------------------------------------- */
/* No counterpart in the reference (its launch shape is fixed: warps = K/32 or
 * K/64 per CTA, one CTA per window or group).  Times the candidate launch
 * shapes -- kernel variant (register-direct at 3 or 2 CTAs per SM, with or
 * without the rolling tile ring that keeps gathers in flight through the
 * MMAs; double-buffered), feature-slice width (32/64/128 columns) and windows
 * per CTA (4/8/16/32, the load-balance granularity), and for TF32 at
 * 128-column slices with the ring B read directly or packed -- on this matrix
 * with this B, and keeps the fastest for the
 * matrix's signature (windows, tiles, K, precision) for the rest of the
 * process: later plain, adaptive and batched calls on a matrix with that
 * signature use it.  C is overwritten.  Results of different shapes agree
 * within the TF32 tolerance but not bit for bit (partial windows are summed
 * at different boundaries). */
typedef struct accspmm_tune_result {
    int32_t kernel;            /* 0 register-direct, 4 double-buffered */
    uint32_t slice_width;      /* feature columns per CTA */
    uint32_t windows_per_cta;
    float best_ms;             /* time of the chosen shape */
    float default_ms;          /* time of the default shape */
    uint32_t candidates;
    uint32_t ctas_per_sm;      /* resident CTAs per SM of the chosen kernel */
    int32_t tile_ring;         /* rolling tile ring: 1 on, 0 off, -1 the default rule */
    int32_t packed_b;          /* gathers from a packed TF32 copy of B: 1 on, 0 off, -1 the default rule */
} accspmm_tune_result_t;

int accspmm_autotune_metcf(const accspmm_metcf_t* metcf, const float* B, float* C,
                           uint32_t K, int32_t precision, void* stream,
                           accspmm_tune_result_t* result);
/* Forgets every tuned shape. */
void accspmm_autotune_clear(void);

/* ---- options ------------------------------------------------------------- */
/* Process-wide launch options.  No counterpart in the reference, whose launch
 * shape is compiled in (include/tf32_comp.hpp:19-31, src/mma_tf32.cu:223).
 * Each option starts from the environment variable named beside it, read
 * once, at the first call that needs an option; afterwards only
 * accspmm_set_option changes it, for every thread, from the next call on (a
 * call already enqueued keeps the shape it was launched with).  Options change
 * speed, not arithmetic: results are the same bits whatever they are set to,
 * except ACCSPMM_OPT_WINDOWS_PER_CTA, which moves the boundaries at which
 * partial row windows are summed (results then agree within the TF32
 * tolerance).  accspmm_set_option returns ACCSPMM_ERROR_INVALID_VALUE for a
 * value outside the listed ones, ACCSPMM_ERROR_UNSUPPORTED for a measurement
 * kernel in a library built without them. */
enum {
    ACCSPMM_OPT_PACK = 0,             /* ACCSPMM_PACK (0 -> 0, 2 -> 1): -1 (default) TF32
                                         launches at 128-column slices (K > 64), at
                                         64-column slices with 48 < K <= 64 and at 32-column
                                         slices (K <= 32) pack a B of at least 4 MiB to
                                         2.5-byte TF32 rows first; 0 never; 1
                                         whenever the launch shape allows */
    ACCSPMM_OPT_PREFETCH = 1,         /* ACCSPMM_PREFETCH (0 -> 0, 1 -> 1): -1 (default)
                                         the packed kernel prefetches into L2 the rows of
                                         the tile group two ahead when K spans an odd
                                         number of its 128- or 64-column slices (where it
                                         measured faster; never at 32-column slices, where
                                         it measured slower); 0 never; 1 always */
    ACCSPMM_OPT_SCHEDULE = 2,         /* ACCSPMM_SCHEDULE: 1 (default) launches of a few
                                         waves run their window blocks heaviest first; 0 in
                                         window order */
    ACCSPMM_OPT_SLICE_WIDTH = 3,      /* ACCSPMM_FS: 0 (default, the chooser's), 32, 64 or
                                         128 feature columns per CTA */
    ACCSPMM_OPT_CTAS_PER_SM = 4,      /* ACCSPMM_OCC: 0 (default), 2 or 3 */
    ACCSPMM_OPT_TILE_RING = 5,        /* ACCSPMM_ROLL: -1 (default rule), 0 off, 1 on */
    ACCSPMM_OPT_WINDOWS_PER_CTA = 6,  /* ACCSPMM_WB: 0 (default) or 1 .. 1024 */
    ACCSPMM_OPT_HOST_SLICE_WIDTH = 7, /* ACCSPMM_HOST_FS: 0 (default), 32, 64 or 128
                                         columns per accspmm_spmm_host slice */
    ACCSPMM_OPT_HOST_DIRECT_C = 8,    /* ACCSPMM_HOST_DIRECT: 1 (default) the kernels store a
                                         page-locked C_host straight over the host link; 0
                                         stage it on the device */
    ACCSPMM_OPT_KERNEL = 9            /* ACCSPMM_KERNEL (direct, pipe, bulk, lean, db, tma,
                                         staged): 0 (default) the register-direct kernels;
                                         the measurement variants 1 .. 6 exist only in the
                                         measurement build, libaccspmm_lab.so */
};
/* values of ACCSPMM_OPT_KERNEL */
enum {
    ACCSPMM_KERNEL_DIRECT = 0,
    ACCSPMM_KERNEL_PIPE = 1,   /* per-warp cp.async ring */
    ACCSPMM_KERNEL_BULK = 2,   /* per-warp cp.async.bulk ring, one row per copy */
    ACCSPMM_KERNEL_LEAN = 3,   /* register-direct at 64-80 registers a thread */
    ACCSPMM_KERNEL_DB = 4,     /* double-buffered register-direct */
    ACCSPMM_KERNEL_TMA = 5,    /* per-warp ring fed by tensor-map gather4 copies */
    ACCSPMM_KERNEL_STAGED = 6  /* slice-major over B staged in 32-column TF32 slices */
};
int accspmm_set_option(int32_t option, int32_t value);
int accspmm_get_option(int32_t option, int32_t* value);

/* ---- batches ------------------------------------------------------------- */
/* No counterpart in the reference (one matrix per process there).  A batch
 * plan runs many device METCF matrices of different sizes and feature widths
 * in one persistent launch: work items (window block x feature slice) of all
 * matrices are numbered largest matrix first and taken by resident CTAs from
 * an atomic counter.  Each item is computed exactly as in the matrix's own
 * accspmm_spmm_tf32 launch, so results are bit-identical to one launch per
 * matrix.  The plan keeps the pointers it was given: B and C contents may
 * change between runs, the buffers may not move or be freed. */
typedef struct accspmm_batch_item {
    const accspmm_metcf_t* metcf;  /* device METCF */
    const float* B;                /* cols x K */
    float* C;                      /* 8 num_windows x K */
    uint32_t K;
} accspmm_batch_item_t;

typedef struct accspmm_batch accspmm_batch_t;

int accspmm_batch_create(const accspmm_batch_item_t* items, uint32_t n,
                         int32_t precision, accspmm_batch_t** batch);
/* One persistent launch on `stream` (counter reset + kernel). */
int accspmm_batch_run(accspmm_batch_t* batch, void* stream);
/* Captures accspmm_batch_run into a CUDA graph on `stream` (not the legacy
 * default stream) and instantiates it; accspmm_batch_launch_graph replays it. */
int accspmm_batch_capture(accspmm_batch_t* batch, void* stream);
int accspmm_batch_launch_graph(accspmm_batch_t* batch, void* stream);
int accspmm_batch_info(const accspmm_batch_t* batch, uint32_t* n_items,
                       uint32_t* work_items, uint32_t* slice_width);
void accspmm_batch_destroy(accspmm_batch_t* batch);

/* ---- serving ------------------------------------------------------------- */
/* No counterpart in the reference.  A continuous-batching request server over
 * resident device METCF matrices.  Any thread submits requests (matrix index,
 * host B of cols x K floats, host C of 8 num_windows x K floats, precision,
 * chain 1 for C = A B or 2 for C = A (A B) on a square matrix); a worker
 * thread admits pending requests in arrival order while their device memory
 * (B, C, chain temporary) fits in hbm_budget_bytes and one of `streams`
 * launch slots is free, runs up to max_batch of them in one batched launch
 * (copies in, kernel, copies out on the slot's stream) and marks them done
 * from a stream callback.  Batches on different slots overlap on the device.
 * A request's result is the same bits alone or in any mix.  Host buffers
 * should be pinned (cudaHostAlloc) for the copies to overlap; they must stay
 * valid until accspmm_server_wait returns. */
typedef struct accspmm_server accspmm_server_t;

typedef struct accspmm_server_config {
    size_t hbm_budget_bytes;  /* device memory for request buffers */
    uint32_t max_batch;       /* requests per launch (0: 64) */
    uint32_t streams;         /* launch slots in flight (0: 4) */
} accspmm_server_config_t;

typedef struct accspmm_server_stats {
    uint64_t submitted, completed, rejected, cancelled, launches;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> completion */
    double throughput_rps;                   /* completed / (last completion - first submit) */
    double mean_batch;                       /* requests per launch */
    size_t peak_bytes;                       /* peak admitted device memory */
} accspmm_server_stats_t;

/* The graphs must stay resident and unchanged for the server's lifetime. */
int accspmm_server_create(const accspmm_metcf_t* graphs, uint32_t n_graphs,
                          const accspmm_server_config_t* config,
                          accspmm_server_t** server);
/* Returns ACCSPMM_ERROR_ADMISSION if one request alone exceeds the budget. */
int accspmm_server_submit(accspmm_server_t* server, uint32_t graph,
                          const float* B_host, float* C_host, uint32_t K,
                          int32_t precision, uint32_t chain,
                          uint64_t* request_id);
/* Blocks until the request is done (timeout_ms < 0: no limit); returns its
 * status, ACCSPMM_ERROR_TIMEOUT if the limit passed first. */
int accspmm_server_wait(accspmm_server_t* server, uint64_t request_id,
                        int32_t timeout_ms);
/* Cancels a request that has not been admitted yet. */
int accspmm_server_cancel(accspmm_server_t* server, uint64_t request_id);
int accspmm_server_stats(accspmm_server_t* server, accspmm_server_stats_t* stats);
int accspmm_server_reset_stats(accspmm_server_t* server);
/* Finishes the admitted and pending requests, then stops the worker. */
void accspmm_server_destroy(accspmm_server_t* server);

/* Synchronises `stream`, then reports (and clears) the sticky status of the
 * SpMM calls on the current device since the last report:
 * ACCSPMM_ERROR_INVALID_VALUE if an adaptive call on a caller-filled AdpBME
 * (accspmm_spmm_adaptive, _noalloc, accspmm_spmm_host) found rowIndices past
 * its c_rows / 8 windows or not non-decreasing multiples of 8 (the message
 * says which); ACCSPMM_ERROR_TIMEOUT if a bounded wait on an asynchronous copy
 * expired (the affected output rows are then undefined); else
 * ACCSPMM_SUCCESS.  No counterpart in the reference, which checks neither. */
int accspmm_device_status(void* stream);

/* Self-test of that failure path: launches one warp on `stream` that waits on
 * an mbarrier nothing arrives on.  Its wait gives up after limit_ms (1 to
 * 2000) and records ACCSPMM_ERROR_TIMEOUT in the status word, which the next
 * accspmm_device_status reports and clears; nothing traps and the GPU context
 * stays usable.  No counterpart in the reference. */
int accspmm_selftest_bounded_wait(uint32_t limit_ms, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ACCSPMM_H */
