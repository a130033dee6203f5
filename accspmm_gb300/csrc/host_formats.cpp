// host_formats.cpp -- host side of the path: Matrix Market reader, COO -> CSR,
// CSR -> METCF, METCF -> AdpBME, balance strategy.  All multi-threaded over
// the host cores; results are independent of the thread count.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cstdlib>
#include <charconv>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>

#include "common.hpp"
#include "host_formats.hpp"

namespace accspmm {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

const char* last_error() { return g_last_error.c_str(); }

unsigned host_threads() {
    static unsigned n = [] {
        const char* e = std::getenv("ACCSPMM_HOST_THREADS");
        if (e && std::atoi(e) > 0) return unsigned(std::atoi(e));
        unsigned h = std::thread::hardware_concurrency();
        return h ? h : 1u;
    }();
    return n;
}

template <class T>
T* host_alloc(size_t n) {
    return static_cast<T*>(std::malloc(sizeof(T) * (n ? n : 1)));
}

// ---------------------------------------------------------------------------
// Matrix Market reader.  Behaviour of include/mmio.hpp:24-210.
// ---------------------------------------------------------------------------
namespace {

inline bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f';
}

// Splits a line into whitespace-separated tokens (sscanf "%s" semantics).
std::vector<std::string> tokens_of(const char* b, const char* e) {
    std::vector<std::string> out;
    while (b < e) {
        while (b < e && is_space(*b)) ++b;
        const char* s = b;
        while (b < e && !is_space(*b)) ++b;
        if (b > s) out.emplace_back(s, b);
    }
    return out;
}

// "%u" on one token: optional sign then decimal digits (the reference's
// fscanf accepts a sign; negative values wrap).  Returns false if the token
// does not start with a number.
bool parse_u32(const char*& p, const char* e, uint32_t* out) {
    while (p < e && is_space(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) { neg = *p == '-'; ++p; }
    if (p >= e || *p < '0' || *p > '9') return false;
    uint64_t v = 0;
    while (p < e && *p >= '0' && *p <= '9') { v = v * 10 + uint64_t(*p - '0'); ++p; }
    uint32_t r = uint32_t(v);
    *out = neg ? uint32_t(0u - r) : r;
    return true;
}

struct Banner {
    char kind = ' ';     // 'C' coordinate, 'A' array
    char field = ' ';    // R C P I
    char storage = 'G';  // G S H K
};

int read_banner(const char* line_b, const char* line_e, Banner* bn) {
    auto t = tokens_of(line_b, line_e);
    if (t.size() < 5) return 12;  // MM_PREMATURE_EOF
    if (t[0] != "%%MatrixMarket") return 14;  // MM_NO_HEADER
    if (t[1] != "matrix") return 15;
    if (t[2] == "coordinate") bn->kind = 'C';
    else if (t[2] == "array") bn->kind = 'A';
    if (t[3] == "real") bn->field = 'R';
    else if (t[3] == "complex") bn->field = 'C';
    else if (t[3] == "pattern") bn->field = 'P';
    else if (t[3] == "integer") bn->field = 'I';
    else return 15;
    if (t[4] == "general") bn->storage = 'G';
    else if (t[4] == "symmetric") bn->storage = 'S';
    else if (t[4] == "Hermitian") bn->storage = 'H';  // case-sensitive, mmio.hpp:66
    else if (t[4] == "skew-symmetric") bn->storage = 'K';
    else return 15;
    return 0;
}

const char* line_end(const char* p, const char* e) {
    const char* q = static_cast<const char*>(std::memchr(p, '\n', size_t(e - p)));
    return q ? q : e;
}

}  // namespace

// The file's bytes, mapped read-only (the parsing threads fault its pages in
// in parallel; no copy).  Every parse below is bounded by explicit ends, so
// no terminating NUL is needed.
struct MappedFile {
    const char* p = nullptr;
    size_t n = 0;
    ~MappedFile() {
        if (p && n) munmap(const_cast<char*>(p), n);
    }
};

int read_mtx_host(const char* path, accspmm_coo_t* coo) {
    std::memset(coo, 0, sizeof *coo);
    MappedFile mf;
    {
        const int fd = open(path, O_RDONLY);
        if (fd < 0) ACC_FAIL(ACCSPMM_MM_LOADING_FILE_ERROR, "cannot open %s: %s", path, std::strerror(errno));
        struct stat sb;
        if (fstat(fd, &sb) != 0) {
            close(fd);
            ACC_FAIL(ACCSPMM_MM_LOADING_FILE_ERROR, "cannot stat %s: %s", path, std::strerror(errno));
        }
        mf.n = size_t(sb.st_size);
        if (mf.n) {
            void* m = mmap(nullptr, mf.n, PROT_READ, MAP_PRIVATE, fd, 0);
            if (m == MAP_FAILED) {
                close(fd);
                mf.n = 0;
                ACC_FAIL(ACCSPMM_MM_LOADING_FILE_ERROR, "cannot map %s: %s", path, std::strerror(errno));
            }
            mf.p = static_cast<const char*>(m);
        }
        close(fd);
    }
    static const char kEmpty[1] = {0};
    const char* p = mf.n ? mf.p : kEmpty;
    const char* e = p + mf.n;

    // banner: first line (fgets of at most 1024 chars, mmio.hpp:35)
    const char* le = line_end(p, e);
    Banner bn;
    if (read_banner(p, std::min(le, p + 1024), &bn) != 0)
        ACC_FAIL(ACCSPMM_MM_READ_BANNER_ERROR, "%s: Matrix Market banner not recognised", path);
    p = le < e ? le + 1 : e;

    // size line, mmio.hpp:74-93: skip lines starting with '%'
    uint32_t m = 0, n = 0, nz = 0;
    for (;;) {
        if (p >= e) ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: missing size line", path);
        le = line_end(p, e);
        if (*p != '%') break;
        p = le < e ? le + 1 : e;
    }
    {
        const char* q = p;
        uint32_t v[3];
        int k = 0;
        while (k < 3 && parse_u32(q, le, &v[k])) ++k;
        if (k == 3) {
            m = v[0]; n = v[1]; nz = v[2];
            p = le < e ? le + 1 : e;
        } else {
            // sscanf failed on that line: the reference falls back to fscanf
            // from the next line on; only whitespace-separated numbers work.
            q = le < e ? le + 1 : e;
            k = 0;
            while (k < 3 && parse_u32(q, e, &v[k])) ++k;
            if (k != 3) ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: unreadable size line", path);
            m = v[0]; n = v[1]; nz = v[2];
            p = q;
        }
    }
    if (bn.kind == 'A')
        ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: dense 'array' files are not supported", path);

    const int tpe = bn.field == 'C' ? 4 : bn.field == 'P' ? 2 : 3;  // tokens per entry
    const bool symmetric = bn.storage == 'S' || bn.storage == 'H';

    // body: split into chunks that start at token boundaries
    const char* body = p;
    size_t blen = size_t(e - body);
    size_t nch = num_chunks_for(blen, 1 << 20);
    std::vector<const char*> cb(nch + 1);
    cb[0] = body;
    cb[nch] = e;
    for (size_t c = 1; c < nch; ++c) {
        const char* q = body + blen * c / nch;
        if (q < cb[c - 1]) q = cb[c - 1];
        while (q < e && !is_space(*q)) ++q;  // move to the end of the token
        cb[c] = q;
    }
    std::vector<uint64_t> ntok(nch, 0);
    parallel_chunks(nch, [&](size_t b, size_t en, unsigned) {
        for (size_t c = b; c < en; ++c) {
            const char* q = cb[c];
            uint64_t t = 0;
            while (q < cb[c + 1]) {
                while (q < cb[c + 1] && is_space(*q)) ++q;
                if (q >= cb[c + 1]) break;
                ++t;
                while (q < cb[c + 1] && !is_space(*q)) ++q;
            }
            ntok[c] = t;
        }
    }, 1);
    std::vector<uint64_t> tstart(nch + 1, 0);
    for (size_t c = 0; c < nch; ++c) tstart[c + 1] = tstart[c] + ntok[c];
    const uint64_t need = uint64_t(nz) * uint64_t(tpe);
    if (tstart[nch] < need)
        ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: %u entries announced, file ends early", path, nz);

    // raw 1-based indices and values; an entry may straddle two chunks, so
    // each token is stored where it belongs and validated in a second pass.
    // Without a symmetric expansion they are parsed straight into the COO.
    struct Free {
        void operator()(void* q) const { std::free(q); }
    };
    std::unique_ptr<uint32_t, Free> ur(host_alloc<uint32_t>(nz)), uc(host_alloc<uint32_t>(nz));
    std::unique_ptr<float, Free> uv(host_alloc<float>(nz));
    if (!ur || !uc || !uv) ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation failed");
    uint32_t* tr = ur.get();
    uint32_t* tc = uc.get();
    float* tv = uv.get();
    if (tpe == 2)  // pattern entries are 1.0, mmio.hpp:127
        parallel_chunks(nz, [&](size_t b, size_t en, unsigned) { std::fill(tv + b, tv + en, 1.0f); });
    std::vector<int> bad(nch, 0);
    parallel_chunks(nch, [&](size_t b, size_t en, unsigned) {
        for (size_t c = b; c < en; ++c) {
            const char* q = cb[c];
            uint64_t g = tstart[c];
            while (q < cb[c + 1] && g < need) {
                while (q < cb[c + 1] && is_space(*q)) ++q;
                if (q >= cb[c + 1]) break;
                const char* tokb = q;
                while (q < cb[c + 1] && !is_space(*q)) ++q;
                uint64_t entry = g / uint64_t(tpe);
                int field = int(g % uint64_t(tpe));
                ++g;
                if (field < 2) {
                    const char* z = tokb;
                    uint32_t v;
                    if (!parse_u32(z, q, &v) || z != q) { bad[c] = 1; break; }
                    (field == 0 ? tr : tc)[entry] = v;
                } else if (field == 2) {
                    // std::from_chars: correctly rounded like strtod, without
                    // the locale; it takes no '+', which fscanf("%lf") does
                    const char* tb = tokb;
                    if (*tb == '+' && q - tb > 1 && tb[1] != '+' && tb[1] != '-') ++tb;
                    double v = 0.0;
                    const auto fc = std::from_chars(tb, q, v);
                    if (fc.ec != std::errc() || fc.ptr != q) {
                        // hexadecimal floats and out-of-range values: the C
                        // library's parse, on a NUL-terminated copy
                        std::string tok(tokb, q);
                        char* z = nullptr;
                        v = std::strtod(tok.c_str(), &z);
                        if (z != tok.c_str() + tok.size()) { bad[c] = 1; break; }
                    }
                    tv[entry] = float(v);
                }
                // field 3 is the imaginary part, dropped (mmio.hpp:123)
            }
        }
    }, 1);
    for (size_t c = 0; c < nch; ++c)
        if (bad[c]) ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: malformed entry", path);
    size_t nchk = num_chunks_for(nz);
    std::vector<uint64_t> diag(nchk, 0);
    std::vector<int> oob(nchk, 0);
    parallel_chunks(nz, [&](size_t b, size_t en, unsigned c) {
        for (size_t i = b; i < en; ++i) {
            uint32_t r = tr[i], col = tc[i];
            if (r < 1 || col < 1 || r > m || col > n) { oob[c] = 1; return; }
            diag[c] += r == col;
            tr[i] = r - 1;
            tc[i] = col - 1;
        }
    });
    for (size_t c = 0; c < nchk; ++c)
        if (oob[c]) ACC_FAIL(ACCSPMM_ERROR_READ_MTX, "%s: entry index out of range", path);
    uint64_t ndiag = 0;
    for (auto d : diag) ndiag += d;

    coo->rows = m;
    coo->cols = n;
    coo->space = ACCSPMM_HOST;
    coo->owned = 1;
    if (symmetric) {
        // mmio.hpp:133-158: each entry followed by its mirror when off-diagonal
        uint64_t total = 2ull * nz - ndiag;
        if (total > 0xFFFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "%s: expanded nnz exceeds 2^32", path);
        coo->nnz = uint32_t(total);
        coo->row = host_alloc<uint32_t>(total);
        coo->col = host_alloc<uint32_t>(total);
        coo->data = host_alloc<float>(total);
        size_t nc2 = num_chunks_for(nz);
        std::vector<uint64_t> off(nc2 + 1, 0);
        parallel_chunks(nz, [&](size_t b, size_t en, unsigned c) {
            uint64_t k = 0;
            for (size_t i = b; i < en; ++i) k += tr[i] != tc[i];
            off[c + 1] = k;
        });
        for (size_t c = 0; c < nc2; ++c) off[c + 1] += off[c];
        parallel_chunks(nz, [&](size_t b, size_t en, unsigned c) {
            uint64_t k = b + off[c];
            for (size_t i = b; i < en; ++i) {
                coo->row[k] = tr[i]; coo->col[k] = tc[i]; coo->data[k] = tv[i]; ++k;
                if (tr[i] != tc[i]) {
                    coo->row[k] = tc[i]; coo->col[k] = tr[i]; coo->data[k] = tv[i]; ++k;
                }
            }
        });
    } else {
        coo->nnz = nz;
        coo->row = ur.release();
        coo->col = uc.release();
        coo->data = uv.release();
    }
    return ACCSPMM_SUCCESS;
}

// ---------------------------------------------------------------------------
// COO -> CSR, include/format.hpp:110-142 (stable by row).
// ---------------------------------------------------------------------------
int csr_from_coo_host(const accspmm_coo_t* coo, accspmm_csr_t* csr) {
    const uint32_t rows = coo->rows, nnz = coo->nnz;
    std::memset(csr, 0, sizeof *csr);
    csr->rows = rows;
    csr->cols = coo->cols;
    csr->nnz = nnz;
    csr->space = ACCSPMM_HOST;
    csr->owned = 1;
    csr->row_ptr = host_alloc<uint32_t>(size_t(rows) + 1);
    csr->col_idx = host_alloc<uint32_t>(nnz);
    csr->data = host_alloc<float>(nnz);
    if (!csr->row_ptr || !csr->col_idx || !csr->data) {
        accspmm_csr_destroy(csr);
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation failed");
    }
    for (uint32_t i = 0; i < nnz; ++i)
        if (coo->row[i] >= rows) {
            accspmm_csr_destroy(csr);
            ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "COO row %u out of range", coo->row[i]);
        }
    size_t nch = num_chunks_for(nnz, 1 << 16);
    if (uint64_t(nch) * rows > (uint64_t(1) << 28)) nch = 1;
    std::vector<uint32_t> cnt(nch * size_t(rows), 0);
    auto body_count = [&](size_t b, size_t e, unsigned c) {
        uint32_t* my = cnt.data() + size_t(c) * rows;
        for (size_t i = b; i < e; ++i) my[coo->row[i]]++;
    };
    if (nch == 1) body_count(0, nnz, 0);
    else parallel_chunks(nnz, body_count, 1 << 16);
    // offsets in (row, chunk) order keep the scatter stable
    uint32_t run = 0;
    for (uint32_t r = 0; r < rows; ++r) {
        csr->row_ptr[r] = run;
        for (size_t c = 0; c < nch; ++c) {
            uint32_t k = cnt[c * rows + r];
            cnt[c * rows + r] = run;
            run += k;
        }
    }
    csr->row_ptr[rows] = run;
    auto body_scatter = [&](size_t b, size_t e, unsigned c) {
        uint32_t* my = cnt.data() + size_t(c) * rows;
        for (size_t i = b; i < e; ++i) {
            uint32_t d = my[coo->row[i]]++;
            csr->col_idx[d] = coo->col[i];
            csr->data[d] = coo->data[i];
        }
    };
    if (nch == 1) body_scatter(0, nnz, 0);
    else parallel_chunks(nnz, body_scatter, 1 << 16);
    return ACCSPMM_SUCCESS;
}

// ---------------------------------------------------------------------------
// CSR -> METCF, include/format.hpp:215-274, parallel over row windows.  A
// window's values occupy exactly its CSR range [row_ptr[8w], row_ptr[8w+8])
// in the output, and its first tile index is the prefix of tile counts, so
// every window is built independently once the tile prefix is known.
// ---------------------------------------------------------------------------
int metcf_from_csr_host(const accspmm_csr_t* csr, accspmm_metcf_t* out) {
    const uint32_t rows = csr->rows;
    const uint32_t W = (rows + kWin - 1) / kWin;
    const uint32_t* rp = csr->row_ptr;
    const uint32_t* ci = csr->col_idx;
    std::memset(out, 0, sizeof *out);
    // pass 1: sorted unique columns per window, kept in a scratch copy laid out
    // like col_idx (a window's unique list fits in its own CSR range)
    std::vector<uint32_t> uniq(csr->nnz ? csr->nnz : 1);
    std::vector<uint32_t> nuniq(W);
    parallel_chunks(W, [&](size_t b, size_t e, unsigned) {
        for (size_t w = b; w < e; ++w) {
            uint32_t r0 = uint32_t(w) * kWin, r1 = std::min(r0 + kWin, rows);
            uint32_t s = rp[r0], t = rp[r1];
            uint32_t* u = uniq.data() + s;
            std::copy(ci + s, ci + t, u);
            std::sort(u, u + (t - s));
            nuniq[w] = uint32_t(std::unique(u, u + (t - s)) - u);
        }
    }, 256);
    std::vector<uint32_t> rwo(size_t(W) + 1, 0);
    uint64_t T = 0;
    for (uint32_t w = 0; w < W; ++w) {
        rwo[w] = uint32_t(T);
        T += (nuniq[w] + kWin - 1) / kWin;
    }
    if (T > 0xFFFFFFFFull / kWin) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "tile count %llu too large", (unsigned long long)T);
    rwo[W] = uint32_t(T);

    out->rows = rows;
    out->cols = csr->cols;
    out->nnz = csr->nnz;
    out->num_windows = W;
    out->num_tiles = uint32_t(T);
    out->space = ACCSPMM_HOST;
    out->owned = 1;
    out->row_window_offset = host_alloc<uint32_t>(size_t(W) + 1);
    out->tc_offset = host_alloc<uint32_t>(size_t(T) + 1);
    out->tc_local_bit = host_alloc<uint64_t>(size_t(T));
    out->sparse_a2b = host_alloc<uint32_t>(size_t(T) * kWin);
    out->data = host_alloc<float>(csr->nnz);
    if (!out->row_window_offset || !out->tc_offset || !out->tc_local_bit || !out->sparse_a2b || !out->data) {
        accspmm_metcf_destroy(out);
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation failed");
    }
    std::copy(rwo.begin(), rwo.end(), out->row_window_offset);
    out->tc_offset[0] = 0;

    parallel_chunks(W, [&](size_t b, size_t e, unsigned) {
        std::vector<uint32_t> rank, cnt, fill;
        for (size_t w = b; w < e; ++w) {
            uint32_t r0 = uint32_t(w) * kWin, r1 = std::min(r0 + kWin, rows);
            uint32_t s = rp[r0], t = rp[r1];
            const uint32_t* u = uniq.data() + s;
            uint32_t nu = nuniq[w], nt = (nu + kWin - 1) / kWin, t0 = rwo[w];
            uint32_t* a2b = out->sparse_a2b + size_t(t0) * kWin;
            for (uint32_t i = 0; i < nt * kWin; ++i) a2b[i] = i < nu ? u[i] : kPad;
            uint64_t* bits = out->tc_local_bit + t0;
            std::fill(bits, bits + nt, uint64_t(0));
            rank.resize(t - s);
            cnt.assign(nt, 0);
            for (uint32_t r = r0; r < r1; ++r)
                for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) {
                    uint32_t c = uint32_t(std::lower_bound(u, u + nu, ci[k]) - u);
                    rank[k - s] = c;
                    cnt[c / kWin]++;
                    bits[c / kWin] |= uint64_t(1) << ((r % kWin) * kWin + c % kWin);
                }
            // tcOffset continues from the window's first value position
            fill.assign(nt, 0);
            uint32_t run = s;
            for (uint32_t j = 0; j < nt; ++j) {
                fill[j] = run;
                run += cnt[j];
                out->tc_offset[t0 + j + 1] = run;
            }
            // values tile by tile, (row, CSR position) order within a tile
            for (uint32_t k = s; k < t; ++k) {
                uint32_t j = rank[k - s] / kWin;
                out->data[fill[j]++] = csr->data[k];
            }
        }
    }, 256);
    return ACCSPMM_SUCCESS;
}

// ---------------------------------------------------------------------------
// AdpBME grouping, include/format.hpp:346-382, :418-423.
// ---------------------------------------------------------------------------
std::vector<uint32_t> adp_groups_host(uint32_t W, const uint32_t* rwo, uint32_t t_load,
                                      uint32_t t_comp, uint32_t t_write, uint32_t target_num) {
    const uint32_t target = target_num * (t_load + t_comp) + t_write;
    uint32_t cur_time = 0, cur_size = 0, pos = 0;
    std::vector<uint32_t> g{0};
    for (uint32_t w = 0; w < W; ++w) {
        uint32_t nt = rwo[w + 1] - rwo[w];
        for (uint32_t i = 0; i < nt; ++i) {
            uint32_t add = i == 0 ? t_load + t_comp + t_write : t_load + t_comp;
            if (cur_size > 0 && cur_time + add > target) {
                pos += cur_size;
                g.push_back(pos);
                cur_time = 0;
                cur_size = 0;
            }
            cur_time += add;
            cur_size++;
        }
    }
    if (cur_size != 0) g.push_back(pos + cur_size);
    return g;
}

int adpbme_from_metcf_host(const accspmm_metcf_t* m, uint32_t t_load, uint32_t t_comp,
                           uint32_t t_write, uint32_t target_num, accspmm_adpbme_t* a) {
    std::memset(a, 0, sizeof *a);
    const uint32_t T = m->num_tiles, W = m->num_windows;
    std::vector<uint32_t> g = adp_groups_host(W, m->row_window_offset, t_load, t_comp,
                                              t_write, target_num);
    a->rows = m->rows;
    a->cols = m->cols;
    a->nnz = m->nnz;
    a->num_tiles = T;
    a->num_groups = uint32_t(g.size() - 1);
    a->space = ACCSPMM_HOST;
    a->owned = 1;
    a->group_offset = host_alloc<uint32_t>(g.size());
    a->tc_offset = host_alloc<uint32_t>(size_t(T) + 1);
    a->row_indices = host_alloc<uint32_t>(T);
    a->tc_local_bit = host_alloc<uint64_t>(T);
    a->sparse_a2b = host_alloc<uint32_t>(size_t(T) * kWin);
    a->data = host_alloc<float>(m->nnz);
    if (!a->group_offset || !a->tc_offset || !a->row_indices || !a->tc_local_bit ||
        !a->sparse_a2b || !a->data) {
        accspmm_adpbme_destroy(a);
        ACC_FAIL(ACCSPMM_ERROR_ALLOC, "host allocation failed");
    }
    std::copy(g.begin(), g.end(), a->group_offset);
    std::memcpy(a->tc_offset, m->tc_offset, sizeof(uint32_t) * (size_t(T) + 1));
    std::memcpy(a->tc_local_bit, m->tc_local_bit, sizeof(uint64_t) * T);
    std::memcpy(a->sparse_a2b, m->sparse_a2b, sizeof(uint32_t) * kWin * size_t(T));
    std::memcpy(a->data, m->data, sizeof(float) * m->nnz);
    const uint32_t* rwo = m->row_window_offset;
    parallel_chunks(W, [&](size_t b, size_t e, unsigned) {
        for (size_t w = b; w < e; ++w)
            for (uint32_t t = rwo[w]; t < rwo[w + 1]; ++t) a->row_indices[t] = uint32_t(w) * kWin;
    }, 1024);
    return ACCSPMM_SUCCESS;
}

// include/utils.hpp:75-85.
int balance_strategy_host(const uint32_t* rwo, uint32_t W, uint32_t T) {
    if (W == 0) return 0;
    uint32_t avg = T / W, sum = 0;
    for (uint32_t i = 1; i < W; ++i) {
        int d = int(rwo[i] - rwo[i - 1] - avg);
        sum += uint32_t(d < 0 ? -d : d);
    }
    return (sum / W) > 8 ? 1 : 0;
}

}  // namespace accspmm
