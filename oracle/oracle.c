/*
 * oracle.c -- CPU restatement of the AccSpMM METCF SpMM path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path, never linked into
 * the product library.  See oracle.h for the reference citations and the
 * parity pin.  Plain C, single-threaded except the timed CSR baseline.
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Reference return codes, include/common.hpp:71-95. */
#define O_SUCCESS 0
#define O_MM_LOADING_FILE_ERROR (-1)
#define O_MM_READ_BANNER_ERROR (-2)
#define O_ERROR_READ_MTX 3
#define O_MM_PREMATURE_EOF 12
#define O_MM_NO_HEADER 14
#define O_MM_UNSUPPORTED_TYPE 15

void oracle_free(void* p) { free(p); }

/* ---------------------------------------------------------------------- */
/* Matrix Market reader: include/mmio.hpp:24-210                           */
/* ---------------------------------------------------------------------- */

/* Typecode characters as in include/common.hpp:111-140:
 * [0] 'M', [1] 'C' coordinate / 'A' array, [2] R/C/P/I, [3] G/S/H/K. */
static int o_read_banner(FILE* f, char tc[4]) {
    char line[1025], banner[64], mtx[64], crd[64], dtype[64], storage[64];
    tc[0] = tc[1] = tc[2] = ' ';
    tc[3] = 'G';
    if (!fgets(line, sizeof line, f)) return O_MM_PREMATURE_EOF;
    if (sscanf(line, "%63s %63s %63s %63s %63s", banner, mtx, crd, dtype,
               storage) != 5)
        return O_MM_PREMATURE_EOF;
    if (strcmp(banner, "%%MatrixMarket") != 0) return O_MM_NO_HEADER;
    /* case-sensitive, as the reference (lower-casing is commented out) */
    if (strcmp(mtx, "matrix") != 0) return O_MM_UNSUPPORTED_TYPE;
    tc[0] = 'M';
    if (strcmp(crd, "coordinate") == 0) tc[1] = 'C';
    else if (strcmp(crd, "array") == 0) tc[1] = 'A';
    if (strcmp(dtype, "real") == 0) tc[2] = 'R';
    else if (strcmp(dtype, "complex") == 0) tc[2] = 'C';
    else if (strcmp(dtype, "pattern") == 0) tc[2] = 'P';
    else if (strcmp(dtype, "integer") == 0) tc[2] = 'I';
    else return O_MM_UNSUPPORTED_TYPE;
    if (strcmp(storage, "general") == 0) tc[3] = 'G';
    else if (strcmp(storage, "symmetric") == 0) tc[3] = 'S';
    else if (strcmp(storage, "Hermitian") == 0) tc[3] = 'H';
    else if (strcmp(storage, "skew-symmetric") == 0) tc[3] = 'K';
    else return O_MM_UNSUPPORTED_TYPE;
    return O_SUCCESS;
}

/* include/mmio.hpp:74-93: skip '%' lines, then "M N nnz". */
static int o_read_size(FILE* f, uint32_t* m, uint32_t* n, uint32_t* nz) {
    char line[1025];
    *m = *n = *nz = 0;
    do {
        if (!fgets(line, sizeof line, f)) return O_MM_PREMATURE_EOF;
    } while (line[0] == '%');
    if (sscanf(line, "%u %u %u", m, n, nz) == 3) return O_SUCCESS;
    for (;;) {
        int k = fscanf(f, "%u %u %u", m, n, nz);
        if (k == 3) return O_SUCCESS;
        /* The reference loops forever on a matching failure; stop instead. */
        if (k == EOF || k >= 0) return O_MM_PREMATURE_EOF;
    }
}

int oracle_read_mtx(const char* path, uint32_t* rows, uint32_t* cols,
                    uint32_t* nnz, uint32_t** row, uint32_t** col,
                    float** data) {
    char tc[4];
    uint32_t m, n, nz, i, diag = 0;
    int is_pattern, is_real, is_complex, is_integer, symmetric;
    uint32_t *tr, *tcl;
    double* td;
    FILE* f = fopen(path, "r");
    *row = *col = NULL;
    *data = NULL;
    if (!f) return O_MM_LOADING_FILE_ERROR;
    if (o_read_banner(f, tc) != O_SUCCESS) {
        fclose(f);
        return O_MM_READ_BANNER_ERROR;
    }
    is_pattern = tc[2] == 'P';
    is_real = !is_pattern && tc[2] == 'R';
    is_complex = !is_pattern && !is_real && tc[2] == 'C';
    is_integer = !is_pattern && !is_real && !is_complex && tc[2] == 'I';
    if (o_read_size(f, &m, &n, &nz) != O_SUCCESS) {
        fclose(f);
        return O_ERROR_READ_MTX;
    }
    symmetric = tc[3] == 'S' || tc[3] == 'H';
    tr = (uint32_t*)malloc(sizeof(uint32_t) * (nz ? nz : 1));
    tcl = (uint32_t*)malloc(sizeof(uint32_t) * (nz ? nz : 1));
    td = (double*)malloc(sizeof(double) * (nz ? nz : 1));
    for (i = 0; i < nz; ++i) {
        unsigned r = 0, c = 0;
        double v = 0.0, im = 0.0;
        int iv = 0, k = 0;
        if (is_real) k = fscanf(f, "%u %u %lg", &r, &c, &v), k = (k == 3);
        else if (is_complex) k = fscanf(f, "%u %u %lg %lg", &r, &c, &v, &im), k = (k == 4);
        else if (is_integer) k = fscanf(f, "%u %u %d", &r, &c, &iv), v = iv, k = (k == 3);
        else if (is_pattern) k = fscanf(f, "%u %u", &r, &c), v = 1.0, k = (k == 2);
        /* The reference keeps going with stale values; report instead. */
        if (!k || r < 1 || c < 1 || r > m || c > n) {
            free(tr); free(tcl); free(td); fclose(f);
            return O_ERROR_READ_MTX;
        }
        tr[i] = r - 1;
        tcl[i] = c - 1;
        td[i] = v;
        if (r == c) ++diag;
    }
    fclose(f);
    *rows = m;
    *cols = n;
    if (symmetric) {
        /* include/mmio.hpp:133-158: nnz' = 2 nnz - diag, mirror after each */
        uint32_t total = nz * 2 - diag, k = 0;
        *row = (uint32_t*)malloc(sizeof(uint32_t) * (total ? total : 1));
        *col = (uint32_t*)malloc(sizeof(uint32_t) * (total ? total : 1));
        *data = (float*)malloc(sizeof(float) * (total ? total : 1));
        for (i = 0; i < nz; ++i) {
            (*row)[k] = tr[i]; (*col)[k] = tcl[i]; (*data)[k] = (float)td[i]; ++k;
            if (tr[i] != tcl[i]) {
                (*row)[k] = tcl[i]; (*col)[k] = tr[i]; (*data)[k] = (float)td[i]; ++k;
            }
        }
        *nnz = total;
    } else {
        *row = (uint32_t*)malloc(sizeof(uint32_t) * (nz ? nz : 1));
        *col = (uint32_t*)malloc(sizeof(uint32_t) * (nz ? nz : 1));
        *data = (float*)malloc(sizeof(float) * (nz ? nz : 1));
        for (i = 0; i < nz; ++i) {
            (*row)[i] = tr[i]; (*col)[i] = tcl[i]; (*data)[i] = (float)td[i];
        }
        *nnz = nz;
    }
    free(tr); free(tcl); free(td);
    return O_SUCCESS;
}

/* ---------------------------------------------------------------------- */
/* CSR: include/format.hpp:110-142                                         */
/* ---------------------------------------------------------------------- */
void oracle_csr_from_coo(uint32_t rows, uint32_t nnz, const uint32_t* row,
                         const uint32_t* col, const float* data,
                         uint32_t* row_ptr, uint32_t* col_idx, float* vals) {
    uint32_t i;
    memset(row_ptr, 0, sizeof(uint32_t) * ((size_t)rows + 1));
    for (i = 0; i < nnz; ++i) row_ptr[row[i] + 1]++;
    for (i = 0; i < rows; ++i) row_ptr[i + 1] += row_ptr[i];
    for (i = 0; i < nnz; ++i) {
        uint32_t dst = row_ptr[row[i]]++;
        vals[dst] = data[i];
        col_idx[dst] = col[i];
    }
    for (i = rows; i > 0; --i) row_ptr[i] = row_ptr[i - 1];
    row_ptr[0] = 0;
}

/* ---------------------------------------------------------------------- */
/* METCF: include/format.hpp:179-199 (unique columns), :23-30 (padding),   */
/* :215-274 (tiles, bitmaps, data order)                                   */
/* ---------------------------------------------------------------------- */
static int o_cmp_u32(const void* a, const void* b) {
    uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : x > y;
}

/* Sorted unique columns of window rows [r0, r1).  Returns count; *out is
 * malloc'd. */
static uint32_t o_window_unique(const uint32_t* row_ptr, const uint32_t* col_idx,
                                uint32_t r0, uint32_t r1, uint32_t** out) {
    uint32_t b = row_ptr[r0], e = row_ptr[r1], n = e - b, u = 0, i;
    uint32_t* v = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    memcpy(v, col_idx + b, sizeof(uint32_t) * n);
    qsort(v, n, sizeof(uint32_t), o_cmp_u32);
    for (i = 0; i < n; ++i)
        if (i == 0 || v[i] != v[i - 1]) v[u++] = v[i];
    *out = v;
    return u;
}

static uint32_t o_rank(const uint32_t* uniq, uint32_t u, uint32_t c) {
    uint32_t lo = 0, hi = u;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (uniq[mid] < c) lo = mid + 1; else hi = mid;
    }
    return lo;
}

uint64_t oracle_metcf_num_tiles(uint32_t rows, const uint32_t* row_ptr,
                                const uint32_t* col_idx) {
    uint64_t t = 0;
    uint32_t r;
    for (r = 0; r < rows; r += 8) {
        uint32_t r1 = r + 8 < rows ? r + 8 : rows, *u;
        uint32_t nu = o_window_unique(row_ptr, col_idx, r, r1, &u);
        t += (nu + 7) / 8;
        free(u);
    }
    return t;
}

void oracle_metcf_fill(uint32_t rows, const uint32_t* row_ptr,
                       const uint32_t* col_idx, const float* vals,
                       uint32_t* rwo, uint32_t* tc_offset, uint64_t* bits,
                       uint32_t* a2b, float* out_data) {
    uint32_t r, w = 0, tile_base = 0, data_pos = 0;
    rwo[0] = 0;
    tc_offset[0] = 0;
    for (r = 0; r < rows; r += 8, ++w) {
        uint32_t r1 = r + 8 < rows ? r + 8 : rows, *u, i, rr, e;
        uint32_t nu = o_window_unique(row_ptr, col_idx, r, r1, &u);
        uint32_t nt = (nu + 7) / 8, t;
        uint32_t* cnt = (uint32_t*)calloc(nt ? nt : 1, sizeof(uint32_t));
        uint32_t* fill = (uint32_t*)calloc(nt ? nt : 1, sizeof(uint32_t));
        for (i = 0; i < nt * 8; ++i) a2b[(size_t)tile_base * 8 + i] = i < nu ? u[i] : 0xFFFFFFFFu;
        for (t = 0; t < nt; ++t) bits[tile_base + t] = 0;
        /* counts and bitmaps, rows ascending, CSR order within a row */
        for (rr = r; rr < r1; ++rr)
            for (e = row_ptr[rr]; e < row_ptr[rr + 1]; ++e) {
                uint32_t k = o_rank(u, nu, col_idx[e]);
                cnt[k / 8]++;
                bits[tile_base + k / 8] |= 1ull << ((rr % 8) * 8 + k % 8);
            }
        for (t = 0; t < nt; ++t) {
            tc_offset[tile_base + t + 1] = tc_offset[tile_base + t] + cnt[t];
        }
        /* data appended tile by tile in (row, CSR position) order */
        for (rr = r; rr < r1; ++rr)
            for (e = row_ptr[rr]; e < row_ptr[rr + 1]; ++e) {
                uint32_t k = o_rank(u, nu, col_idx[e]);
                uint32_t tt = k / 8;
                out_data[tc_offset[tile_base + tt] + fill[tt]++] = vals[e];
            }
        (void)data_pos;
        tile_base += nt;
        rwo[w + 1] = tile_base;
        free(cnt); free(fill); free(u);
    }
}

/* ---------------------------------------------------------------------- */
/* AdpBME grouping: include/format.hpp:340-382, :418-423                   */
/* ---------------------------------------------------------------------- */
uint32_t oracle_adpbme_groups(uint32_t num_windows, const uint32_t* rwo,
                              uint32_t t_load, uint32_t t_comp,
                              uint32_t t_write, uint32_t target_num,
                              uint32_t* group_offset) {
    uint32_t target = target_num * (t_load + t_comp) + t_write;
    uint32_t cur_time = 0, cur_size = 0, g = 0, w, i;
    uint32_t pos = 0; /* running tile count = prefix of group sizes */
    if (group_offset) group_offset[0] = 0;
    for (w = 0; w < num_windows; ++w) {
        uint32_t nt = rwo[w + 1] - rwo[w];
        for (i = 0; i < nt; ++i) {
            uint32_t add = i == 0 ? t_load + t_comp + t_write : t_load + t_comp;
            if (cur_size > 0 && cur_time + add > target) {
                pos += cur_size;
                ++g;
                if (group_offset) group_offset[g] = pos;
                cur_time = 0;
                cur_size = 0;
            }
            cur_time += add;
            cur_size++;
        }
    }
    if (cur_size != 0) {
        pos += cur_size;
        ++g;
        if (group_offset) group_offset[g] = pos;
    }
    return g;
}

void oracle_adpbme_row_indices(uint32_t num_windows, const uint32_t* rwo,
                               uint32_t* row_indices) {
    uint32_t w, t;
    for (w = 0; w < num_windows; ++w)
        for (t = rwo[w]; t < rwo[w + 1]; ++t) row_indices[t] = w * 8;
}

/* include/utils.hpp:75-85: windows 0..W-2 only, unsigned difference cast to
 * int before abs, integer averages. */
int oracle_balance_strategy(const uint32_t* rwo, uint32_t num_windows,
                            uint32_t num_tiles) {
    uint32_t avg, sum = 0, i;
    if (num_windows == 0) return 0;
    avg = num_tiles / num_windows;
    for (i = 1; i + 1 < num_windows + 1; ++i) {
        uint32_t cur = rwo[i] - rwo[i - 1];
        int d = (int)(cur - avg);
        sum += (uint32_t)(d < 0 ? -d : d);
    }
    return (sum / num_windows) > 8;
}

/* ---------------------------------------------------------------------- */
/* SpMM                                                                    */
/* ---------------------------------------------------------------------- */
float oracle_tf32_rna(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return x; /* Inf / NaN */
    /* add half an ulp of the 10-bit significand to the magnitude, then
     * truncate: ties go away from zero because the sign bit is untouched */
    u = (u + 0x00001000u) & 0xFFFFE000u;
    memcpy(&x, &u, 4);
    return x;
}

/* Value of tile element (r, c) under the popcount indexing of
 * include/mma_tf32.cuh:71-79; 0 if the bit is clear. */
static int o_tile_value(uint64_t bits, uint32_t base, const float* vals,
                        uint32_t bit, float* v) {
    uint64_t below;
    if (!((bits >> bit) & 1ull)) return 0;
    below = bit == 63 ? bits : (bits & ((2ull << bit) - 1ull));
    *v = vals[base + (uint32_t)__builtin_popcountll(below) - 1];
    return 1;
}

void oracle_spmm_metcf_f64(uint32_t num_windows, uint32_t cols,
                           const uint32_t* rwo, const uint32_t* tc_offset,
                           const uint64_t* bits, const uint32_t* a2b,
                           const float* vals, const float* B, uint32_t K,
                           double* C) {
    uint32_t w, t, r, c, f;
    memset(C, 0, sizeof(double) * (size_t)num_windows * 8 * K);
    for (w = 0; w < num_windows; ++w)
        for (t = rwo[w]; t < rwo[w + 1]; ++t)
            for (r = 0; r < 8; ++r)
                for (c = 0; c < 8; ++c) {
                    float a;
                    uint32_t brow = a2b[(size_t)t * 8 + c];
                    if (!o_tile_value(bits[t], tc_offset[t], vals, r * 8 + c, &a)) continue;
                    if (brow >= cols) continue;
                    for (f = 0; f < K; ++f)
                        C[((size_t)w * 8 + r) * K + f] +=
                            (double)a * (double)B[(size_t)brow * K + f];
                }
}

void oracle_spmm_metcf_tf32(uint32_t num_windows, uint32_t cols,
                            const uint32_t* rwo, const uint32_t* tc_offset,
                            const uint64_t* bits, const uint32_t* a2b,
                            const float* vals, const float* B, uint32_t K,
                            float* C) {
    uint32_t w, t, r, c, f;
    memset(C, 0, sizeof(float) * (size_t)num_windows * 8 * K);
    for (w = 0; w < num_windows; ++w)
        for (t = rwo[w]; t < rwo[w + 1]; ++t)
            for (r = 0; r < 8; ++r)
                for (c = 0; c < 8; ++c) {
                    float a;
                    uint32_t brow = a2b[(size_t)t * 8 + c];
                    if (!o_tile_value(bits[t], tc_offset[t], vals, r * 8 + c, &a)) continue;
                    if (brow >= cols) continue;
                    a = oracle_tf32_rna(a);
                    for (f = 0; f < K; ++f)
                        C[((size_t)w * 8 + r) * K + f] +=
                            a * oracle_tf32_rna(B[(size_t)brow * K + f]);
                }
}

void oracle_spmm_csr_f64(uint32_t rows, const uint32_t* row_ptr,
                         const uint32_t* col_idx, const float* vals,
                         const float* B, uint32_t K, double* C) {
    uint32_t r, e, f;
    memset(C, 0, sizeof(double) * (size_t)rows * K);
    for (r = 0; r < rows; ++r)
        for (e = row_ptr[r]; e < row_ptr[r + 1]; ++e)
            for (f = 0; f < K; ++f)
                C[(size_t)r * K + f] += (double)vals[e] * (double)B[(size_t)col_idx[e] * K + f];
}

void oracle_spmm_csr_f32_omp(uint32_t row_begin, uint32_t row_end,
                             const uint32_t* row_ptr, const uint32_t* col_idx,
                             const float* vals, const float* B, uint32_t K,
                             float* C, int threads) {
    long r;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (r = (long)row_begin; r < (long)row_end; ++r) {
        float* out = C + (size_t)r * K;
        uint32_t e, f;
        for (f = 0; f < K; ++f) out[f] = 0.0f;
        for (e = row_ptr[r]; e < row_ptr[r + 1]; ++e) {
            const float a = vals[e];
            const float* brow = B + (size_t)col_idx[e] * K;
            for (f = 0; f < K; ++f) out[f] += a * brow[f];
        }
    }
}

int oracle_omp_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
