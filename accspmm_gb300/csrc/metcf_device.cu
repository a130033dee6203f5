// metcf_device.cu -- CSR -> METCF, METCF -> AdpBME, balance strategy and
// COO -> CSR, all on the GPU and bit-exact with the reference's host builders
// (include/format.hpp:110-142, :215-274, :340-429; include/utils.hpp:75-85).
//
// METCF on the device:
//  1. every window's entries (contiguous in CSR order) are ordered by
//     (column, CSR position) in place: a bitonic sort in shared memory per
//     window of up to 2,048 entries; the entries of larger windows are
//     gathered and ordered by one stable radix sort of the keys
//     (window << colbits) | col.  Either way the result is the entries
//     ordered by (window, column, position) with key = (window << colbits) |
//     col and value = CSR position.
//  2. unique-key flags, scanned, give each entry the rank of its column among
//     the window's sorted distinct columns (include/format.hpp:179-199).
//  3. tiles per window = ceil(distinct / 8), scanned -> rowWindowOffset.
//  4. per entry: sparseA2B slot (first of its key), bitmap bit via atomicOr,
//     per-tile count via atomicAdd (both order-independent).
//  5. counts scanned -> tcOffset.
//  6. a tile's entries are contiguous in sorted order; an entry's place among
//     them in CSR order (include/format.hpp:241-263 appends row by row, CSR
//     order within a row) is the number of tile entries with a smaller CSR
//     position.
#include <algorithm>

#include "common.hpp"
#include "device_prims.hpp"
#include "device_util.cuh"
#include "host_formats.hpp"

namespace accspmm {

namespace {

int bits_for(uint64_t x) {
    int b = 0;
    while (x) {
        ++b;
        x >>= 1;
    }
    return b;
}

// Error flags a kernel raises for malformed input (read back by the host).
enum : uint32_t { kErrColRange = 1u, kErrRowPtr = 2u };

// Entries of window w: [row_ptr[8w], row_ptr[min(8w + 8, rows)]), or none
// when row_ptr is malformed there (flagged).
__device__ __forceinline__ bool window_range(const uint32_t* __restrict__ row_ptr, uint32_t rows,
                                             uint32_t nnz, uint32_t w, uint32_t* s, uint32_t* e,
                                             uint32_t* __restrict__ err, bool report) {
    const uint32_t r0 = w * kWin, r1 = min(r0 + kWin, rows);
    *s = row_ptr[r0];
    *e = row_ptr[r1];
    if (*s > *e || *e > nnz) {
        if (report) atomicOr(err, kErrRowPtr);
        return false;
    }
    return true;
}

constexpr uint32_t kSortSmall = 256;    // entries a window sorted by the small class may hold
constexpr uint32_t kSortLarge = 2048;   // the largest window sorted in shared memory
constexpr int kSortThreads = 128;

// One block per window with lo < entries <= CAP: its (column, position)
// pairs sorted ascending by a bitonic network in shared memory (the pairs
// are distinct, so the order is the stable one), written as sorted keys and
// CSR positions in the window's own range.  Windows of the class lo = 0
// also check the row offsets and column indices.  Key: the column above
// the position in the window, 32 bits when colbits + log2(CAP) <= 32,
// else 64.
template <uint32_t CAP, typename Key>
__global__ void __launch_bounds__(kSortThreads)
    window_sort_kernel(const uint32_t* __restrict__ row_ptr, const uint32_t* __restrict__ col_idx,
                       uint32_t rows, uint32_t cols, uint32_t nnz, int colbits, uint32_t lo,
                       uint64_t* __restrict__ skeys, uint32_t* __restrict__ svals,
                       uint32_t* __restrict__ err) {
    static_assert((CAP & (CAP - 1)) == 0, "power-of-two window class");
    constexpr int RB = sizeof(Key) == 8 ? 32 : (CAP == 256 ? 8 : 11);  // position bits
    static_assert(sizeof(Key) == 8 || (1u << RB) == CAP, "position field holds 0 .. CAP - 1");
    __shared__ Key sk[CAP];
    const uint32_t w = blockIdx.x;
    uint32_t s, e;
    if (!window_range(row_ptr, rows, nnz, w, &s, &e, err, lo == 0 && threadIdx.x == 0)) return;
    const uint32_t n = e - s;
    if (n <= lo || n > CAP) return;
    uint32_t P = 1;
    while (P < n) P <<= 1;
    bool bad = false;
    for (uint32_t j = threadIdx.x; j < P; j += kSortThreads) {
        // padding sorts last: a real key is below all ones, as j < n - 1
        // < P - 1 wherever padding exists
        Key v = ~Key(0);
        if (j < n) {
            const uint32_t c = col_idx[s + j];
            bad |= c >= cols;
            v = (Key(c) << RB) | Key(j);
        }
        sk[j] = v;
    }
    if (bad) atomicOr(err, kErrColRange);
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            // pair q compares i (bit j clear: q with a zero inserted at
            // bit j) with i + j
            for (uint32_t q = threadIdx.x; q < P / 2; q += kSortThreads) {
                const uint32_t i = ((q & ~(j - 1)) << 1) | (q & (j - 1)), x = i + j;
                const Key a = sk[i], b = sk[x];
                if ((a > b) == ((i & k) == 0)) {
                    sk[i] = b;
                    sk[x] = a;
                }
            }
            __syncthreads();
        }
    }
    const uint64_t wk = uint64_t(w) << colbits;
    for (uint32_t j = threadIdx.x; j < n; j += kSortThreads) {
        const Key v = sk[j];
        skeys[s + j] = wk | uint64_t(v >> RB);
        svals[s + j] = s + uint32_t(v & ((Key(1) << RB) - 1));
    }
}

// Entries of windows above kSortLarge (valid ones), 0 for the others.
__global__ void large_window_sizes_kernel(const uint32_t* __restrict__ row_ptr, uint32_t rows,
                                          uint32_t nnz, uint32_t W, uint32_t* __restrict__ sizes) {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    uint32_t s, e;
    const bool ok = window_range(row_ptr, rows, nnz, w, &s, &e, nullptr, false);
    sizes[w] = ok && e - s > kSortLarge ? e - s : 0u;
}

// One thread per entry of the large windows (compact index j; offs is the
// exclusive scan of their sizes): the entry's key and CSR position gathered
// to the compact arrays (dir 0), or the sorted compact pair j written back to
// its window's range (dir 1).
__global__ void large_window_move_kernel(const uint32_t* __restrict__ row_ptr,
                                         const uint32_t* __restrict__ col_idx, uint32_t cols,
                                         uint32_t W, int colbits, const uint32_t* __restrict__ offs,
                                         uint32_t L, int dir, uint64_t* __restrict__ ckeys,
                                         uint32_t* __restrict__ cvals, uint64_t* __restrict__ skeys,
                                         uint32_t* __restrict__ svals, uint32_t* __restrict__ err) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= L) return;
    // the window holding j: the last w with offs[w] <= j (windows of size
    // zero share their successor's offset)
    uint32_t lo = 0, hi = W;  // offs[lo] <= j < offs[hi + 1]
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo + 1) / 2;
        if (offs[mid] <= j) lo = mid;
        else hi = mid - 1;
    }
    const uint32_t w = lo, k = j - offs[w], s = row_ptr[w * kWin];
    if (dir == 0) {
        const uint32_t c = col_idx[s + k];
        if (c >= cols) atomicOr(err, kErrColRange);
        ckeys[j] = (uint64_t(w) << colbits) | c;
        cvals[j] = s + k;
    } else {
        skeys[s + k] = ckeys[j];
        svals[s + k] = cvals[j];
    }
}

__global__ void uniq_flags_kernel(const uint64_t* __restrict__ skeys, uint32_t n,
                                  uint32_t* __restrict__ flags) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (i == 0 || skeys[i] != skeys[i - 1]) ? 1u : 0u;
}

// E = exclusive scan of the unique flags.  Window w's sorted entries occupy
// [row_ptr[8w], row_ptr[8w+8]) because the sort key starts with the window.
__global__ void window_tiles_kernel(const uint32_t* __restrict__ row_ptr, uint32_t rows,
                                    uint32_t nnz, uint32_t W, const uint32_t* __restrict__ E,
                                    uint32_t* __restrict__ tiles) {
    uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    // malformed offsets (reported by the sort) count no entries here
    uint32_t e = min(row_ptr[min(w * kWin + kWin, rows)], nnz), s = min(row_ptr[w * kWin], e);
    uint32_t u = E[e] - E[s];
    tiles[w] = (u + kWin - 1) / kWin;
}

__device__ __forceinline__ uint32_t row_of_entry(const uint32_t* __restrict__ row_ptr,
                                                 uint32_t rows, uint32_t w, uint32_t e) {
    uint32_t r = w * kWin, r1 = min(r + kWin, rows);
    while (r + 1 < r1 && row_ptr[r + 1] <= e) ++r;
    return r;
}

__global__ void metcf_tiles_kernel(const uint64_t* __restrict__ skeys,
                                   const uint32_t* __restrict__ svals, uint32_t n, int colbits,
                                   const uint32_t* __restrict__ row_ptr, uint32_t rows,
                                   const uint32_t* __restrict__ E,
                                   const uint32_t* __restrict__ rwo,
                                   uint32_t* __restrict__ a2b, uint64_t* __restrict__ bits,
                                   uint32_t* __restrict__ counts,
                                   uint32_t* __restrict__ seg_start) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t key = skeys[i];
    const uint32_t w = uint32_t(key >> colbits);
    const uint32_t col = uint32_t(key & ((uint64_t(1) << colbits) - 1));
    const uint32_t e = svals[i];
    const uint32_t ws = row_ptr[w * kWin];
    const uint32_t base = E[ws + 1];
    const uint32_t rank = E[i + 1] - base;
    const uint32_t t0 = rwo[w];
    const uint32_t tile = t0 + rank / kWin;
    if (E[i + 1] != E[i]) a2b[size_t(t0) * kWin + rank] = col;
    const uint32_t r = row_of_entry(row_ptr, rows, w, e);
    atomicOr(reinterpret_cast<unsigned long long*>(bits + tile),
             1ull << ((r % kWin) * kWin + rank % kWin));
    atomicAdd(counts + tile, 1u);
    bool first = i == ws || ((E[i] - base) / kWin) != rank / kWin;
    if (first) seg_start[tile] = i;
}

__global__ void metcf_data_kernel(const uint64_t* __restrict__ skeys,
                                  const uint32_t* __restrict__ svals, uint32_t n, int colbits,
                                  const uint32_t* __restrict__ row_ptr,
                                  const uint32_t* __restrict__ E,
                                  const uint32_t* __restrict__ rwo,
                                  const uint32_t* __restrict__ tc_offset,
                                  const uint32_t* __restrict__ seg_start,
                                  const float* __restrict__ csr_data, float* __restrict__ data) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t w = uint32_t(skeys[i] >> colbits);
    const uint32_t ws = row_ptr[w * kWin];
    const uint32_t rank = E[i + 1] - E[ws + 1];
    const uint32_t tile = rwo[w] + rank / kWin;
    const uint32_t s0 = seg_start[tile];
    const uint32_t cnt = tc_offset[tile + 1] - tc_offset[tile];
    const uint32_t e = svals[i];
    uint32_t pos = 0;
    for (uint32_t j = s0; j < s0 + cnt; ++j) pos += svals[j] < e;
    data[tc_offset[tile] + pos] = csr_data[e];
}

// ---- AdpBME ----------------------------------------------------------------

__global__ void row_indices_kernel(const uint32_t* __restrict__ rwo, uint32_t W,
                                   uint32_t* __restrict__ row_indices) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (warp >= W) return;
    for (uint32_t t = rwo[warp] + lane; t < rwo[warp + 1]; t += 32) row_indices[t] = warp * kWin;
}

// Greedy packing state (include/format.hpp:366-382): 0 = empty group,
// tau + 1 = non-empty group whose time is tau.  One step for a tile of cost a.
__device__ __forceinline__ uint32_t adp_step(uint32_t st, uint32_t a, uint32_t target,
                                             bool* split) {
    if (st == 0) {
        *split = false;
        return a + 1;
    }
    uint32_t tau = st - 1;
    *split = tau + a > target;
    return *split ? a + 1 : tau + a + 1;
}

// The greedy packing is a finite-state machine over the tiles: its input per
// tile is whether the tile starts a window (cost a_first) or not (a_other).
// Tiles are cut into chunks of kAdpChunk; each chunk tabulates the state it
// ends in for every state it may start in, the tables are composed level by
// level (kAdpGroup chunks into one table, then a walk over those), and every
// chunk replays its tiles from its true start state to mark the splits.
// Each step is exact integer arithmetic, so the marks equal a sequential walk.
constexpr uint32_t kAdpChunk = 256;   // tiles per chunk (one warp replays one chunk)
constexpr uint32_t kAdpPiece = 16384; // u16 table entries staged in shared memory at a time

__device__ __forceinline__ bool is_first_tile(const uint32_t* row_indices, uint32_t t) {
    return t == 0 || row_indices[t] != row_indices[t - 1];
}

// table[c][s] = state after chunk c when entered in state s (one block per
// chunk, one thread per state).
__global__ void adp_chunk_table_kernel(const uint32_t* __restrict__ row_indices, uint32_t T,
                                       uint32_t a_first, uint32_t a_other, uint32_t target,
                                       uint32_t nstates, uint16_t* __restrict__ table) {
    __shared__ uint8_t first[kAdpChunk];
    const uint32_t c = blockIdx.x, t0 = c * kAdpChunk;
    const uint32_t len = min(kAdpChunk, T - t0);
    for (uint32_t j = threadIdx.x; j < len; j += blockDim.x)
        first[j] = is_first_tile(row_indices, t0 + j) ? 1 : 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < nstates; s += blockDim.x) {
        uint32_t st = s;
        bool sp;
        for (uint32_t j = 0; j < len; ++j) st = adp_step(st, first[j] ? a_first : a_other, target, &sp);
        table[size_t(c) * nstates + s] = uint16_t(st);
    }
}

// out[b][s] = the composition of tables b*group .. min(n, (b+1)*group) - 1
// applied to s (one block per group, one thread per state; the group's
// tables are staged in shared memory, group * nstates <= kAdpPiece).
__global__ void adp_compose_kernel(const uint16_t* __restrict__ table, uint32_t n, uint32_t nstates,
                                   uint32_t group, uint16_t* __restrict__ out) {
    __shared__ uint16_t tab[kAdpPiece];
    const uint32_t c0 = blockIdx.x * group, cnt = min(group, n - c0);
    const uint16_t* src = table + size_t(c0) * nstates;
    for (uint32_t j = threadIdx.x; j < cnt * nstates; j += blockDim.x) tab[j] = src[j];
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < nstates; s += blockDim.x) {
        uint32_t st = s;
        for (uint32_t j = 0; j < cnt; ++j) st = tab[j * nstates + st];
        out[size_t(blockIdx.x) * nstates + s] = uint16_t(st);
    }
}

// Block b walks tables b*group .. min(n, (b+1)*group) - 1 from the state
// start[b] (0 when start is null) and writes the state each table is
// entered in: in_state[c].  The tables pass through shared memory in
// pieces; one thread walks each piece.
__global__ void adp_walk_kernel(const uint16_t* __restrict__ table, uint32_t n, uint32_t nstates,
                                uint32_t group, const uint32_t* __restrict__ start,
                                uint32_t* __restrict__ in_state) {
    __shared__ uint16_t tab[kAdpPiece];
    __shared__ uint32_t st_sh;
    const uint32_t c0 = blockIdx.x * group, c1 = min(n, c0 + group);
    const uint32_t per_piece = kAdpPiece / nstates;
    if (threadIdx.x == 0) st_sh = start ? start[blockIdx.x] : 0u;
    for (uint32_t p0 = c0; p0 < c1; p0 += per_piece) {
        const uint32_t cnt = min(per_piece, c1 - p0);
        const uint16_t* src = table + size_t(p0) * nstates;
        __syncthreads();  // the previous piece is walked
        for (uint32_t j = threadIdx.x; j < cnt * nstates; j += blockDim.x) tab[j] = src[j];
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t st = st_sh;
            for (uint32_t j = 0; j < cnt; ++j) {
                in_state[p0 + j] = st;
                st = tab[j * nstates + st];
            }
            st_sh = st;
        }
    }
}

// One warp per chunk: the chunk's window-start flags become eight ballot
// words, one lane walks the 256 steps from the chunk's start state
// collecting the split marks as bits, and the warp stores them as flags.
__global__ void adp_replay_kernel(const uint32_t* __restrict__ row_indices, uint32_t T,
                                  uint32_t a_first, uint32_t a_other, uint32_t target,
                                  const uint32_t* __restrict__ in_state, uint32_t nchunks,
                                  uint32_t* __restrict__ split_flag) {
    static_assert(kAdpChunk == 8 * 32, "eight ballot words per chunk");
    const uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (c >= nchunks) return;
    const uint32_t t0 = c * kAdpChunk, len = min(kAdpChunk, T - t0);
    uint32_t firsts[8], splits[8];
    uint32_t prev = (lane == 0 && t0 > 0) ? row_indices[t0 - 1] : 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t i = j * 32 + lane;
        const uint32_t r = i < len ? row_indices[t0 + i] : 0u;
        const uint32_t up = __shfl_up_sync(0xffffffffu, r, 1);
        const uint32_t before = lane == 0 ? prev : up;
        const bool f = i < len && (t0 + i == 0 || r != before);
        firsts[j] = __ballot_sync(0xffffffffu, f);
        prev = __shfl_sync(0xffffffffu, r, 31);
    }
    uint32_t st = in_state[c];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        uint32_t bits = 0;
        const uint32_t n_here = len > uint32_t(j) * 32 ? min(32u, len - uint32_t(j) * 32) : 0u;
        for (uint32_t b = 0; b < n_here; ++b) {
            bool sp;
            st = adp_step(st, ((firsts[j] >> b) & 1u) ? a_first : a_other, target, &sp);
            bits |= uint32_t(sp) << b;
        }
        splits[j] = bits;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint32_t i = j * 32 + lane;
        if (i < len) split_flag[t0 + i] = (splits[j] >> lane) & 1u;
    }
}

// Sequential fallback for parameter sets whose state space is too large.
__global__ void adp_sequential_kernel(const uint32_t* __restrict__ row_indices, uint32_t T,
                                      uint32_t a_first, uint32_t a_other, uint32_t target,
                                      uint32_t* __restrict__ split_flag) {
    uint32_t st = 0;
    for (uint32_t t = 0; t < T; ++t) {
        bool sp;
        st = adp_step(st, is_first_tile(row_indices, t) ? a_first : a_other, target, &sp);
        split_flag[t] = sp ? 1u : 0u;
    }
}

__global__ void adp_offsets_kernel(const uint32_t* __restrict__ split_flag,
                                   const uint32_t* __restrict__ split_pos, uint32_t T,
                                   uint32_t* __restrict__ group_offset) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) group_offset[0] = 0;
    if (t < T && split_flag[t]) group_offset[split_pos[t] + 1] = t;
    if (t == T) group_offset[split_pos[T] + 1] = T;  // end of the last group
}

// ---- balance strategy --------------------------------------------------------

__global__ void balance_kernel(const uint32_t* __restrict__ rwo, uint32_t W,
                               uint32_t* __restrict__ sum) {
    __shared__ uint32_t part[32];
    const uint32_t avg = rwo[W] / W;
    uint32_t acc = 0;
    for (uint32_t i = 1 + blockIdx.x * blockDim.x + threadIdx.x; i < W; i += gridDim.x * blockDim.x) {
        int d = int(rwo[i] - rwo[i - 1] - avg);
        acc += uint32_t(d < 0 ? -d : d);
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : 0;
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) atomicAdd(sum, acc);
    }
}

// ---- COO -> CSR ------------------------------------------------------------------

__global__ void coo_keys_kernel(const uint32_t* __restrict__ row, uint32_t nnz, uint32_t rows,
                                uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                uint32_t* __restrict__ counts, uint32_t* __restrict__ err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    uint32_t r = row[i];
    if (r >= rows) {
        atomicOr(err, 1u);
        r = 0;
    }
    keys[i] = r;
    vals[i] = i;
    atomicAdd(counts + r, 1u);
}

__global__ void coo_gather_kernel(const uint32_t* __restrict__ perm, uint32_t nnz,
                                  const uint32_t* __restrict__ col, const float* __restrict__ data,
                                  uint32_t* __restrict__ col_out, float* __restrict__ data_out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    uint32_t p = perm[i];
    col_out[i] = col[p];
    data_out[i] = data[p];
}

inline unsigned blocks_for(size_t n, unsigned threads) { return unsigned((n + threads - 1) / threads); }

// Orders every window's entries by (column, CSR position) into skeys /
// svals (keys (window << colbits) | col, values CSR positions): windows of
// up to 256 and up to 2,048 entries sorted in shared memory, larger windows
// gathered into compact arrays, radix-sorted together and written back.
int sort_window_entries(const accspmm_csr_t* csr, uint32_t W, int colbits, int wbits, uint64_t* skeys,
                        uint32_t* svals, uint32_t* err, cudaStream_t s) {
    if (W == 0) return ACCSPMM_SUCCESS;
    const uint32_t rows = csr->rows, cols = csr->cols, nnz = csr->nnz;
    // 32-bit keys while a column and an 11-bit position fit (cols <= 2^21)
    if (colbits + 11 <= 32) {
        window_sort_kernel<kSortSmall, uint32_t><<<W, kSortThreads, 0, s>>>(
            csr->row_ptr, csr->col_idx, rows, cols, nnz, colbits, 0, skeys, svals, err);
        ACC_LAUNCH_CHECK();
        window_sort_kernel<kSortLarge, uint32_t><<<W, kSortThreads, 0, s>>>(
            csr->row_ptr, csr->col_idx, rows, cols, nnz, colbits, kSortSmall, skeys, svals, err);
    } else {
        window_sort_kernel<kSortSmall, uint64_t><<<W, kSortThreads, 0, s>>>(
            csr->row_ptr, csr->col_idx, rows, cols, nnz, colbits, 0, skeys, svals, err);
        ACC_LAUNCH_CHECK();
        window_sort_kernel<kSortLarge, uint64_t><<<W, kSortThreads, 0, s>>>(
            csr->row_ptr, csr->col_idx, rows, cols, nnz, colbits, kSortSmall, skeys, svals, err);
    }
    ACC_LAUNCH_CHECK();
    DevBuf<uint32_t> sizes, offs;
    ACC_CUDA(sizes.alloc(W, s));
    ACC_CUDA(offs.alloc(size_t(W) + 1, s));
    large_window_sizes_kernel<<<blocks_for(W, 256), 256, 0, s>>>(csr->row_ptr, rows, nnz, W, sizes.p);
    ACC_LAUNCH_CHECK();
    int st = scan_exclusive_u32(sizes.p, offs.p, W, s);
    if (st) return st;
    uint32_t L = 0;
    ACC_CUDA(cudaMemcpyAsync(&L, offs.p + W, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaStreamSynchronize(s));
    if (L == 0) return ACCSPMM_SUCCESS;
    DevBuf<uint64_t> ck, cks;
    DevBuf<uint32_t> cv, cvs;
    ACC_CUDA(ck.alloc(L, s));
    ACC_CUDA(cv.alloc(L, s));
    ACC_CUDA(cks.alloc(L, s));
    ACC_CUDA(cvs.alloc(L, s));
    const unsigned grid = blocks_for(L, 256);
    large_window_move_kernel<<<grid, 256, 0, s>>>(csr->row_ptr, csr->col_idx, cols, W, colbits, offs.p, L, 0,
                                                  ck.p, cv.p, nullptr, nullptr, err);
    ACC_LAUNCH_CHECK();
    st = radix_sort_pairs(ck.p, cv.p, cks.p, cvs.p, L, colbits + wbits, s);
    if (st) return st;
    large_window_move_kernel<<<grid, 256, 0, s>>>(csr->row_ptr, csr->col_idx, cols, W, colbits, offs.p, L, 1,
                                                  cks.p, cvs.p, skeys, svals, err);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

}  // namespace

int metcf_from_csr_device(const accspmm_csr_t* csr, accspmm_metcf_t* out, void* stream) {
    cudaStream_t s = as_stream(stream);
    std::memset(out, 0, sizeof *out);
    const uint32_t rows = csr->rows, cols = csr->cols, nnz = csr->nnz;
    const uint32_t W = (rows + kWin - 1) / kWin;
    const int colbits = std::max(1, bits_for(cols ? cols - 1 : 0));
    const int wbits = bits_for(W ? W - 1 : 0);
    if (colbits + wbits > 64) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "matrix too large for 64-bit keys");

    DevBuf<uint64_t> skeys;
    DevBuf<uint32_t> svals, flags, E, tiles, err;
    DevBuf<uint32_t> rwo, tc_offset, a2b, counts, seg;
    DevBuf<uint64_t> bits;
    DevBuf<float> data;
    ACC_CUDA(err.alloc(1, s));
    ACC_CUDA(cudaMemsetAsync(err.p, 0, 4, s));
    ACC_CUDA(skeys.alloc(nnz, s));
    ACC_CUDA(svals.alloc(nnz, s));
    int st = sort_window_entries(csr, W, colbits, wbits, skeys.p, svals.p, err.p, s);
    if (st) return st;
    ACC_CUDA(flags.alloc(nnz, s));
    ACC_CUDA(E.alloc(size_t(nnz) + 1, s));
    if (nnz) {
        uniq_flags_kernel<<<blocks_for(nnz, 256), 256, 0, s>>>(skeys.p, nnz, flags.p);
        ACC_LAUNCH_CHECK();
    }
    st = scan_exclusive_u32(flags.p, E.p, nnz, s);
    if (st) return st;
    flags.reset();
    ACC_CUDA(tiles.alloc(W, s));
    ACC_CUDA(rwo.alloc(size_t(W) + 1, s));
    if (W) {
        window_tiles_kernel<<<blocks_for(W, 256), 256, 0, s>>>(csr->row_ptr, rows, nnz, W, E.p, tiles.p);
        ACC_LAUNCH_CHECK();
    }
    st = scan_exclusive_u32(tiles.p, rwo.p, W, s);
    if (st) return st;
    uint32_t host_T = 0, host_err = 0, host_nnz_end = 0, host_first = 0;
    ACC_CUDA(cudaMemcpyAsync(&host_T, rwo.p + W, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaMemcpyAsync(&host_err, err.p, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaMemcpyAsync(&host_nnz_end, csr->row_ptr + rows, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaMemcpyAsync(&host_first, csr->row_ptr, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaStreamSynchronize(s));
    // entries outside every window (before row_ptr[0]) would have no sorted
    // key: refused before any kernel reads the sorted entries by position
    if (host_first != 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr[0]=%u, not 0", host_first);
    if (host_nnz_end != nnz) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr[rows]=%u but nnz=%u", host_nnz_end, nnz);
    if (host_err & kErrRowPtr) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "row_ptr is not non-decreasing");
    if (host_err & kErrColRange) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "column index >= cols");
    const uint32_t T = host_T;
    if (uint64_t(T) * kWin > 0xFFFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "tile count too large");

    ACC_CUDA(tc_offset.alloc(size_t(T) + 1, s));
    ACC_CUDA(bits.alloc(T, s));
    ACC_CUDA(a2b.alloc(size_t(T) * kWin, s));
    ACC_CUDA(counts.alloc(T, s));
    ACC_CUDA(seg.alloc(T, s));
    ACC_CUDA(data.alloc(nnz, s));
    ACC_CUDA(cudaMemsetAsync(a2b.p, 0xFF, size_t(T) * kWin * 4, s));
    ACC_CUDA(cudaMemsetAsync(bits.p, 0, size_t(T) * 8, s));
    ACC_CUDA(cudaMemsetAsync(counts.p, 0, size_t(T) * 4, s));
    if (nnz) {
        metcf_tiles_kernel<<<blocks_for(nnz, 256), 256, 0, s>>>(
            skeys.p, svals.p, nnz, colbits, csr->row_ptr, rows, E.p, rwo.p, a2b.p, bits.p,
            counts.p, seg.p);
        ACC_LAUNCH_CHECK();
    }
    st = scan_exclusive_u32(counts.p, tc_offset.p, T, s);
    if (st) return st;
    if (nnz) {
        metcf_data_kernel<<<blocks_for(nnz, 256), 256, 0, s>>>(
            skeys.p, svals.p, nnz, colbits, csr->row_ptr, E.p, rwo.p, tc_offset.p, seg.p,
            csr->data, data.p);
        ACC_LAUNCH_CHECK();
    }
    // the input CSR is read until here: finish before returning so that the
    // caller may free it as soon as the call returns
    ACC_CUDA(cudaStreamSynchronize(s));
    out->rows = rows;
    out->cols = cols;
    out->nnz = nnz;
    out->num_windows = W;
    out->num_tiles = T;
    out->space = ACCSPMM_DEVICE;
    out->owned = 1;
    out->row_window_offset = rwo.release();
    out->tc_offset = tc_offset.release();
    out->tc_local_bit = bits.release();
    out->sparse_a2b = a2b.release();
    out->data = data.release();
    return ACCSPMM_SUCCESS;
}

int adpbme_from_metcf_device(const accspmm_metcf_t* m, uint32_t t_load, uint32_t t_comp,
                             uint32_t t_write, uint32_t target_num, accspmm_adpbme_t* a,
                             void* stream) {
    cudaStream_t s = as_stream(stream);
    std::memset(a, 0, sizeof *a);
    const uint32_t T = m->num_tiles, W = m->num_windows;
    const uint64_t target64 = uint64_t(target_num) * (uint64_t(t_load) + t_comp) + t_write;
    const uint64_t af64 = uint64_t(t_load) + t_comp + t_write, ao64 = uint64_t(t_load) + t_comp;
    if (target64 > 0xFFFFFFFFull || af64 > 0xFFFFFFFFull)
        ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "AdpBME cost parameters overflow");
    const uint32_t target = uint32_t(target64), af = uint32_t(af64), ao = uint32_t(ao64);

    DevBuf<uint32_t> go, tco, ri, a2b, flag, pos, in_state;
    DevBuf<uint64_t> bits;
    DevBuf<float> data;
    DevBuf<uint16_t> table;
    ACC_CUDA(ri.alloc(T, s));
    if (W) {
        row_indices_kernel<<<blocks_for(size_t(W) * 32, 256), 256, 0, s>>>(m->row_window_offset, W, ri.p);
        ACC_LAUNCH_CHECK();
    }
    ACC_CUDA(flag.alloc(T, s));
    const uint64_t smax = std::max<uint64_t>(target, std::max(af, ao));
    const uint64_t nstates = smax + 2;
    if (T) {
        if (nstates <= 1024 && smax + 1 < 65535) {
            const uint32_t ns = uint32_t(nstates);
            const uint32_t nch = (T + kAdpChunk - 1) / kAdpChunk;
            // chunks per composed table: as many as fit one shared-memory piece
            const uint32_t group = std::max<uint32_t>(1, std::min<uint32_t>(64, kAdpPiece / ns));
            const uint32_t nsup = (nch + group - 1) / group;
            DevBuf<uint16_t> sup;
            DevBuf<uint32_t> sup_in;
            ACC_CUDA(table.alloc(size_t(nch) * ns, s));
            ACC_CUDA(in_state.alloc(nch, s));
            ACC_CUDA(sup.alloc(size_t(nsup) * ns, s));
            ACC_CUDA(sup_in.alloc(nsup, s));
            const unsigned thr = unsigned(std::min<uint64_t>(1024, (nstates + 31) / 32 * 32));
            adp_chunk_table_kernel<<<nch, thr, 0, s>>>(ri.p, T, af, ao, target, ns, table.p);
            ACC_LAUNCH_CHECK();
            adp_compose_kernel<<<nsup, thr, 0, s>>>(table.p, nch, ns, group, sup.p);
            ACC_LAUNCH_CHECK();
            // the composed tables in order from state 0, then each group's
            // chunks from its composed start state
            adp_walk_kernel<<<1, 256, 0, s>>>(sup.p, nsup, ns, nsup, nullptr, sup_in.p);
            ACC_LAUNCH_CHECK();
            adp_walk_kernel<<<nsup, 256, 0, s>>>(table.p, nch, ns, group, sup_in.p, in_state.p);
            ACC_LAUNCH_CHECK();
            adp_replay_kernel<<<blocks_for(size_t(nch) * 32, 256), 256, 0, s>>>(ri.p, T, af, ao, target,
                                                                               in_state.p, nch, flag.p);
            ACC_LAUNCH_CHECK();
        } else {
            adp_sequential_kernel<<<1, 1, 0, s>>>(ri.p, T, af, ao, target, flag.p);
            ACC_LAUNCH_CHECK();
        }
    }
    ACC_CUDA(pos.alloc(size_t(T) + 1, s));
    int st = scan_exclusive_u32(flag.p, pos.p, T, s);
    if (st) return st;
    uint32_t nsplit = 0;
    ACC_CUDA(cudaMemcpyAsync(&nsplit, pos.p + T, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaStreamSynchronize(s));
    const uint32_t G = T ? nsplit + 1 : 0;
    ACC_CUDA(go.alloc(size_t(G) + 1, s));
    if (T) {
        adp_offsets_kernel<<<blocks_for(size_t(T) + 1, 256), 256, 0, s>>>(flag.p, pos.p, T, go.p);
        ACC_LAUNCH_CHECK();
    } else {
        ACC_CUDA(cudaMemsetAsync(go.p, 0, 4, s));
    }
    ACC_CUDA(tco.alloc(size_t(T) + 1, s));
    ACC_CUDA(bits.alloc(T, s));
    ACC_CUDA(a2b.alloc(size_t(T) * kWin, s));
    ACC_CUDA(data.alloc(m->nnz, s));
    ACC_CUDA(cudaMemcpyAsync(tco.p, m->tc_offset, (size_t(T) + 1) * 4, cudaMemcpyDeviceToDevice, s));
    if (T) {
        ACC_CUDA(cudaMemcpyAsync(bits.p, m->tc_local_bit, size_t(T) * 8, cudaMemcpyDeviceToDevice, s));
        ACC_CUDA(cudaMemcpyAsync(a2b.p, m->sparse_a2b, size_t(T) * kWin * 4, cudaMemcpyDeviceToDevice, s));
    }
    if (m->nnz)
        ACC_CUDA(cudaMemcpyAsync(data.p, m->data, size_t(m->nnz) * 4, cudaMemcpyDeviceToDevice, s));
    ACC_CUDA(cudaStreamSynchronize(s));  // the input METCF may be freed after return
    a->rows = m->rows;
    a->cols = m->cols;
    a->nnz = m->nnz;
    a->num_tiles = T;
    a->num_groups = G;
    a->space = ACCSPMM_DEVICE;
    a->owned = 1;
    a->group_offset = go.release();
    a->tc_offset = tco.release();
    a->row_indices = ri.release();
    a->tc_local_bit = bits.release();
    a->sparse_a2b = a2b.release();
    a->data = data.release();
    return ACCSPMM_SUCCESS;
}

int balance_strategy_device(const accspmm_metcf_t* m, int* adaptive, void* stream) {
    cudaStream_t s = as_stream(stream);
    const uint32_t W = m->num_windows;
    if (W == 0) {
        *adaptive = 0;
        return ACCSPMM_SUCCESS;
    }
    DevBuf<uint32_t> sum;
    ACC_CUDA(sum.alloc(1, s));
    ACC_CUDA(cudaMemsetAsync(sum.p, 0, 4, s));
    unsigned blocks = std::min<unsigned>(1024, blocks_for(W, 256));
    balance_kernel<<<blocks, 256, 0, s>>>(m->row_window_offset, W, sum.p);
    ACC_LAUNCH_CHECK();
    uint32_t h = 0;
    ACC_CUDA(cudaMemcpyAsync(&h, sum.p, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaStreamSynchronize(s));
    *adaptive = (h / W) > 8 ? 1 : 0;
    return ACCSPMM_SUCCESS;
}

int csr_from_coo_device(const accspmm_coo_t* coo, accspmm_csr_t* csr, void* stream) {
    cudaStream_t s = as_stream(stream);
    std::memset(csr, 0, sizeof *csr);
    const uint32_t rows = coo->rows, nnz = coo->nnz;
    DevBuf<uint64_t> keys, skeys;
    DevBuf<uint32_t> vals, svals, counts, rp, ci, err;
    DevBuf<float> d;
    ACC_CUDA(err.alloc(1, s));
    ACC_CUDA(cudaMemsetAsync(err.p, 0, 4, s));
    ACC_CUDA(keys.alloc(nnz, s));
    ACC_CUDA(vals.alloc(nnz, s));
    ACC_CUDA(counts.alloc(rows, s));
    ACC_CUDA(cudaMemsetAsync(counts.p, 0, size_t(rows) * 4, s));
    if (nnz) {
        coo_keys_kernel<<<blocks_for(nnz, 256), 256, 0, s>>>(coo->row, nnz, rows, keys.p, vals.p,
                                                             counts.p, err.p);
        ACC_LAUNCH_CHECK();
    }
    ACC_CUDA(rp.alloc(size_t(rows) + 1, s));
    int st = scan_exclusive_u32(counts.p, rp.p, rows, s);
    if (st) return st;
    ACC_CUDA(skeys.alloc(nnz, s));
    ACC_CUDA(svals.alloc(nnz, s));
    st = radix_sort_pairs(keys.p, vals.p, skeys.p, svals.p, nnz,
                          std::max(1, bits_for(rows ? rows - 1 : 0)), s);
    if (st) return st;
    ACC_CUDA(ci.alloc(nnz, s));
    ACC_CUDA(d.alloc(nnz, s));
    if (nnz) {
        coo_gather_kernel<<<blocks_for(nnz, 256), 256, 0, s>>>(svals.p, nnz, coo->col, coo->data,
                                                               ci.p, d.p);
        ACC_LAUNCH_CHECK();
    }
    uint32_t host_err = 0;
    ACC_CUDA(cudaMemcpyAsync(&host_err, err.p, 4, cudaMemcpyDeviceToHost, s));
    ACC_CUDA(cudaStreamSynchronize(s));
    if (host_err) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "COO row index >= rows");
    csr->rows = rows;
    csr->cols = coo->cols;
    csr->nnz = nnz;
    csr->space = ACCSPMM_DEVICE;
    csr->owned = 1;
    csr->row_ptr = rp.release();
    csr->col_idx = ci.release();
    csr->data = d.release();
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
