// metcf_io.cpp -- binary METCF / AdpBME files: save once, load in place of
// re-reading the Matrix Market text and rebuilding the format.
//
// The reference has no such format: every run of src/mma_tf32.cu parses the
// .mtx text (include/mmio.hpp:171-210) and rebuilds METCF
// (include/format.hpp:215-274) and AdpBME (:340-429).  A file here is
//
//   magic (8 bytes: "ACSPMTCF" METCF, "ACSPADPB" AdpBME)
//   u32 version (1), u32 field count F, u32 fields[F]
//     METCF:  rows, cols, nnz, num_windows, num_tiles
//     AdpBME: rows, cols, nnz, num_tiles, num_groups
//   then per array, in struct order: u64 byte length, payload, u64 checksum
//
// all little-endian.  The checksum is a 64-bit FNV-1a over the payload's
// 4 MiB chunks (chunk hashes computed in parallel, then folded in order), so
// it does not depend on the thread count.  A loaded object is validated
// before it is returned -- offsets monotone and consistent with the sizes,
// per-tile popcounts no larger than the tile's value count, column indices in range
// or padding -- because the SpMM kernels index values and B rows through
// these arrays: a corrupted file must fail with ACCSPMM_ERROR_FORMAT, never
// reach a kernel.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>

#include "accspmm.h"
#include "common.hpp"
#include "host_formats.hpp"

namespace accspmm {

namespace {

constexpr char kMagicMetcf[8] = {'A', 'C', 'S', 'P', 'M', 'T', 'C', 'F'};
constexpr char kMagicAdp[8] = {'A', 'C', 'S', 'P', 'A', 'D', 'P', 'B'};
constexpr uint32_t kVersion = 1;
constexpr size_t kChunk = size_t(4) << 20;
constexpr uint64_t kFnvBasis = 0xcbf29ce484222325ull, kFnvPrime = 0x100000001b3ull;

uint64_t fnv_bytes(const unsigned char* p, size_t n, uint64_t h) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= kFnvPrime;
    }
    return h;
}

uint64_t checksum(const void* data, size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    const size_t nch = (bytes + kChunk - 1) / kChunk;
    std::vector<uint64_t> part(nch);
    parallel_chunks(nch, [&](size_t b, size_t e, unsigned) {
        for (size_t c = b; c < e; ++c) {
            const size_t off = c * kChunk;
            part[c] = fnv_bytes(p + off, std::min(kChunk, bytes - off), kFnvBasis);
        }
    }, 1);
    uint64_t h = fnv_bytes(reinterpret_cast<const unsigned char*>(&bytes), sizeof bytes, kFnvBasis);
    for (uint64_t x : part) h = fnv_bytes(reinterpret_cast<const unsigned char*>(&x), sizeof x, h);
    return h;
}

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

bool little_endian() {
    const uint32_t x = 1;
    unsigned char b;
    std::memcpy(&b, &x, 1);
    return b == 1;
}

int write_all(std::FILE* f, const void* p, size_t n, const char* path) {
    if (n && std::fwrite(p, 1, n, f) != n) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "write to %s failed", path);
    return ACCSPMM_SUCCESS;
}

int write_header(std::FILE* f, const char* magic, const uint32_t* fields, uint32_t nf,
                 const char* path) {
    int r = write_all(f, magic, 8, path);
    if (!r) r = write_all(f, &kVersion, 4, path);
    if (!r) r = write_all(f, &nf, 4, path);
    if (!r) r = write_all(f, fields, 4 * size_t(nf), path);
    return r;
}

int write_array(std::FILE* f, const void* p, size_t bytes, const char* path) {
    const uint64_t len = bytes, sum = checksum(p, bytes);
    int r = write_all(f, &len, 8, path);
    if (!r) r = write_all(f, p, bytes, path);
    if (!r) r = write_all(f, &sum, 8, path);
    return r;
}

int read_all(std::FILE* f, void* p, size_t n, const char* path) {
    if (n && std::fread(p, 1, n, f) != n) ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s is truncated", path);
    return ACCSPMM_SUCCESS;
}

int read_header(std::FILE* f, const char* magic, uint32_t* fields, uint32_t nf, const char* path) {
    char m[8];
    uint32_t ver = 0, n = 0;
    int r = read_all(f, m, 8, path);
    if (r) return r;
    if (std::memcmp(m, magic, 8) != 0) ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: wrong magic", path);
    if ((r = read_all(f, &ver, 4, path)) || (r = read_all(f, &n, 4, path))) return r;
    if (ver != kVersion) ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: unsupported version %u", path, ver);
    if (n != nf) ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: %u header fields, expected %u", path, n, nf);
    return read_all(f, fields, 4 * size_t(nf), path);
}

// Reads one array of exactly `count` elements of T into a new malloc'd buffer.
template <class T>
int read_array(std::FILE* f, size_t count, T** out, const char* what, const char* path) {
    *out = nullptr;
    uint64_t len = 0, sum = 0;
    int r = read_all(f, &len, 8, path);
    if (r) return r;
    if (len != sizeof(T) * count)
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: %s has %llu bytes, expected %zu", path, what,
                 (unsigned long long)len, sizeof(T) * count);
    T* p = static_cast<T*>(std::malloc(sizeof(T) * (count ? count : 1)));
    if (!p) ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation of %zu bytes failed", sizeof(T) * count);
    if ((r = read_all(f, p, sizeof(T) * count, path)) || (r = read_all(f, &sum, 8, path))) {
        std::free(p);
        return r;
    }
    if (sum != checksum(p, sizeof(T) * count)) {
        std::free(p);
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: checksum of %s does not match", path, what);
    }
    *out = p;
    return ACCSPMM_SUCCESS;
}

// Offsets off[0..n] start at 0, never decrease and end at `last`.
bool offsets_ok(const uint32_t* off, size_t n, uint64_t last) {
    if (off[0] != 0 || off[n] != last) return false;
    std::atomic<bool> ok{true};
    parallel_chunks(n, [&](size_t b, size_t e, unsigned) {
        for (size_t i = b; i < e; ++i)
            if (off[i + 1] < off[i]) {
                ok = false;
                return;
            }
    });
    return ok;
}

// Per tile: the bitmap has at most as many set bits as the tile has values
// (fewer when the input held duplicate entries, which share a bit but keep
// their values); every sparseA2B entry is a column index or padding.  The
// kernels read value tcOffset[t] + popc(bits below and at a bit) - 1, which
// these two conditions keep inside the tile's values.
bool tiles_ok(const uint32_t* tc_offset, const uint64_t* bits, const uint32_t* a2b, size_t T,
              uint32_t cols) {
    std::atomic<bool> ok{true};
    parallel_chunks(T, [&](size_t b, size_t e, unsigned) {
        for (size_t t = b; t < e && ok; ++t) {
            if (uint32_t(__builtin_popcountll(bits[t])) > tc_offset[t + 1] - tc_offset[t]) ok = false;
            for (size_t j = 0; j < kWin; ++j) {
                const uint32_t c = a2b[t * kWin + j];
                if (c != kPad && c >= cols) ok = false;
            }
        }
    });
    return ok;
}

int validate_metcf(const accspmm_metcf_t& m, const char* path) {
    if (m.num_windows != (uint64_t(m.rows) + kWin - 1) / kWin)
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: %u windows for %u rows", path, m.num_windows, m.rows);
    if (!offsets_ok(m.row_window_offset, m.num_windows, m.num_tiles))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: rowWindowOffset is not a valid offset array", path);
    if (!offsets_ok(m.tc_offset, m.num_tiles, m.nnz))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: tcOffset is not a valid offset array", path);
    if (!tiles_ok(m.tc_offset, m.tc_local_bit, m.sparse_a2b, m.num_tiles, m.cols))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: tile bitmaps, value counts or columns are inconsistent", path);
    return ACCSPMM_SUCCESS;
}

int validate_adp(const accspmm_adpbme_t& a, const char* path) {
    const uint64_t wrows = (uint64_t(a.rows) + kWin - 1) / kWin * kWin;
    if (!offsets_ok(a.group_offset, a.num_groups, a.num_tiles))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: groupOffset is not a valid offset array", path);
    if (!offsets_ok(a.tc_offset, a.num_tiles, a.nnz))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: tcOffset is not a valid offset array", path);
    std::atomic<bool> ok{true};
    parallel_chunks(a.num_tiles, [&](size_t b, size_t e, unsigned) {
        for (size_t t = b; t < e; ++t) {
            const uint32_t r = a.row_indices[t];
            if (r % kWin || r >= wrows || (t > 0 && r < a.row_indices[t - 1])) {
                ok = false;
                return;
            }
        }
    });
    if (!ok) ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: rowIndices are not sorted window starts", path);
    if (!tiles_ok(a.tc_offset, a.tc_local_bit, a.sparse_a2b, a.num_tiles, a.cols))
        ACC_FAIL(ACCSPMM_ERROR_FORMAT, "%s: tile bitmaps, value counts or columns are inconsistent", path);
    return ACCSPMM_SUCCESS;
}

// Host copy of a possibly-device object, owned by `holder` when copied.
template <class Obj, class CopyFn, class DestroyFn>
int host_view(const Obj* src, Obj* holder, const Obj** view, CopyFn copy, DestroyFn, void* stream) {
    if (src->space == ACCSPMM_HOST) {
        *view = src;
        return ACCSPMM_SUCCESS;
    }
    int r = copy(src, ACCSPMM_HOST, holder, stream);
    if (r) return r;
    *view = holder;
    return ACCSPMM_SUCCESS;
}

}  // namespace

int metcf_save(const accspmm_metcf_t* src, const char* path, void* stream) {
    if (!little_endian()) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "binary files need a little-endian host");
    accspmm_metcf_t tmp;
    std::memset(&tmp, 0, sizeof tmp);
    const accspmm_metcf_t* m = nullptr;
    int r = host_view(src, &tmp, &m, accspmm_metcf_copy, accspmm_metcf_destroy, stream);
    if (r) return r;
    std::unique_ptr<accspmm_metcf_t, void (*)(accspmm_metcf_t*)> guard(&tmp, accspmm_metcf_destroy);
    File f;
    f.f = std::fopen(path, "wb");
    if (!f.f) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "cannot open %s for writing", path);
    const size_t W = m->num_windows, T = m->num_tiles;
    const uint32_t fields[5] = {m->rows, m->cols, m->nnz, m->num_windows, m->num_tiles};
    r = write_header(f.f, kMagicMetcf, fields, 5, path);
    if (!r) r = write_array(f.f, m->row_window_offset, 4 * (W + 1), path);
    if (!r) r = write_array(f.f, m->tc_offset, 4 * (T + 1), path);
    if (!r) r = write_array(f.f, m->tc_local_bit, 8 * T, path);
    if (!r) r = write_array(f.f, m->sparse_a2b, 4 * kWin * T, path);
    if (!r) r = write_array(f.f, m->data, 4 * size_t(m->nnz), path);
    if (!r && std::fflush(f.f) != 0) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "write to %s failed", path);
    return r;
}

int metcf_load(const char* path, int32_t space, accspmm_metcf_t* out, void* stream) {
    if (!little_endian()) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "binary files need a little-endian host");
    File f;
    f.f = std::fopen(path, "rb");
    if (!f.f) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "cannot open %s", path);
    uint32_t h[5];
    int r = read_header(f.f, kMagicMetcf, h, 5, path);
    if (r) return r;
    accspmm_metcf_t m;
    std::memset(&m, 0, sizeof m);
    m.rows = h[0];
    m.cols = h[1];
    m.nnz = h[2];
    m.num_windows = h[3];
    m.num_tiles = h[4];
    m.space = ACCSPMM_HOST;
    m.owned = 1;
    std::unique_ptr<accspmm_metcf_t, void (*)(accspmm_metcf_t*)> guard(&m, accspmm_metcf_destroy);
    const size_t W = m.num_windows, T = m.num_tiles;
    r = read_array(f.f, W + 1, &m.row_window_offset, "rowWindowOffset", path);
    if (!r) r = read_array(f.f, T + 1, &m.tc_offset, "tcOffset", path);
    if (!r) r = read_array(f.f, T, &m.tc_local_bit, "tcLocalBit", path);
    if (!r) r = read_array(f.f, kWin * T, &m.sparse_a2b, "sparseA2B", path);
    if (!r) r = read_array(f.f, size_t(m.nnz), &m.data, "data", path);
    if (!r) r = validate_metcf(m, path);
    if (r) return r;
    if (space == ACCSPMM_DEVICE) return accspmm_metcf_copy(&m, ACCSPMM_DEVICE, out, stream);
    *out = m;
    guard.release();
    return ACCSPMM_SUCCESS;
}

int adpbme_save(const accspmm_adpbme_t* src, const char* path, void* stream) {
    if (!little_endian()) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "binary files need a little-endian host");
    accspmm_adpbme_t tmp;
    std::memset(&tmp, 0, sizeof tmp);
    const accspmm_adpbme_t* a = nullptr;
    int r = host_view(src, &tmp, &a, accspmm_adpbme_copy, accspmm_adpbme_destroy, stream);
    if (r) return r;
    std::unique_ptr<accspmm_adpbme_t, void (*)(accspmm_adpbme_t*)> guard(&tmp, accspmm_adpbme_destroy);
    File f;
    f.f = std::fopen(path, "wb");
    if (!f.f) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "cannot open %s for writing", path);
    const size_t G = a->num_groups, T = a->num_tiles;
    const uint32_t fields[5] = {a->rows, a->cols, a->nnz, a->num_tiles, a->num_groups};
    r = write_header(f.f, kMagicAdp, fields, 5, path);
    if (!r) r = write_array(f.f, a->group_offset, 4 * (G + 1), path);
    if (!r) r = write_array(f.f, a->tc_offset, 4 * (T + 1), path);
    if (!r) r = write_array(f.f, a->row_indices, 4 * T, path);
    if (!r) r = write_array(f.f, a->tc_local_bit, 8 * T, path);
    if (!r) r = write_array(f.f, a->sparse_a2b, 4 * kWin * T, path);
    if (!r) r = write_array(f.f, a->data, 4 * size_t(a->nnz), path);
    if (!r && std::fflush(f.f) != 0) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "write to %s failed", path);
    return r;
}

int adpbme_load(const char* path, int32_t space, accspmm_adpbme_t* out, void* stream) {
    if (!little_endian()) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "binary files need a little-endian host");
    File f;
    f.f = std::fopen(path, "rb");
    if (!f.f) ACC_FAIL(ACCSPMM_ERROR_OPEN_FILE, "cannot open %s", path);
    uint32_t h[5];
    int r = read_header(f.f, kMagicAdp, h, 5, path);
    if (r) return r;
    accspmm_adpbme_t a;
    std::memset(&a, 0, sizeof a);
    a.rows = h[0];
    a.cols = h[1];
    a.nnz = h[2];
    a.num_tiles = h[3];
    a.num_groups = h[4];
    a.space = ACCSPMM_HOST;
    a.owned = 1;
    std::unique_ptr<accspmm_adpbme_t, void (*)(accspmm_adpbme_t*)> guard(&a, accspmm_adpbme_destroy);
    const size_t G = a.num_groups, T = a.num_tiles;
    r = read_array(f.f, G + 1, &a.group_offset, "groupOffset", path);
    if (!r) r = read_array(f.f, T + 1, &a.tc_offset, "tcOffset", path);
    if (!r) r = read_array(f.f, T, &a.row_indices, "rowIndices", path);
    if (!r) r = read_array(f.f, T, &a.tc_local_bit, "tcLocalBit", path);
    if (!r) r = read_array(f.f, kWin * T, &a.sparse_a2b, "sparseA2B", path);
    if (!r) r = read_array(f.f, size_t(a.nnz), &a.data, "data", path);
    if (!r) r = validate_adp(a, path);
    if (r) return r;
    if (space == ACCSPMM_DEVICE) return accspmm_adpbme_copy(&a, ACCSPMM_DEVICE, out, stream);
    *out = a;
    guard.release();
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
