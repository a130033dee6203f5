// spmm.cu -- METCF SpMM C = A * B on tensor cores (TF32 and 3xTF32), the
// plain and adaptive entry points, and the reference's timing loop.
//
// Work decomposition (replaces the one-CTA-per-window kernels of
// include/mma_tf32.cuh:13-550 and the group kernels of :552-1042):
//  - a CTA owns `wb` consecutive row windows and one feature slice of FS
//    columns; its tile range [rwo[w0], rwo[w0+wb]) is cut into 8 equal
//    contiguous pieces, one per warp, so a long window is shared by several
//    warps and every warp gets the same number of tiles;
//  - a warp walks its tiles and keeps 8 x FS accumulators in registers;
//    windows that lie inside its piece are stored straight to C, the (at
//    most two) windows cut by a piece boundary go to shared-memory slots and
//    are summed in warp order after a barrier -- no float atomics, so the
//    result does not depend on scheduling;
//  - rows of empty windows are written as zeros, so C is fully overwritten.
// Per tile a lane loads its two B rows (tile columns tq and tq+4) as FS/32
// float4 each -- eight lanes cover 128 contiguous bytes of a row -- which is
// exactly the m16n8k8 A-operand fragment when the feature order inside a
// 32-column group is permuted (row g of the MMA holds features 4g..4g+3 of
// one float4, row g+8 the same lanes of the next group).  The tile's sparse
// values become the k8 x n8 operand: value (row g, col tq) is
// data[tcOffset + popc(bitmap & ((2 << bit) - 1)) - 1] (include/mma_tf32.cuh:
// 71-79).  Tile metadata is fetched a batch ahead with one coalesced load.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.hpp"
#include "device_util.cuh"
#include "mbarrier.cuh"
#include "spmm_common.cuh"
#include "spmm_direct.cuh"
#include "options.hpp"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

constexpr int kNW = kDirectNW;  // warps per CTA of the register-direct kernels



// One-matrix launch of the register-direct kernel: one CTA per work item.
// U tiles per batch; MINB resident CTAs per SM (the register budget); EPI:
// the bias / activation epilogue is applied as C is stored.
template <int FS, int PREC, int U, int MINB, bool EPI, int NW = kNW, bool ROLL = false>
__global__ void __launch_bounds__(NW * 32, MINB) spmm_window_kernel(const SpmmArgs a) {
    extern __shared__ __align__(16) float smem[];
    float* part = smem;  // [2 * NW] slots
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * NW * 8 * FS);
    Block<FS, NW> blk;
    blk.init(a, s_rwo, part);
    direct_item<FS, PREC, U, EPI, NW, ROLL>(a, blk);
}

// The register-direct kernel with the rolling ring reading B from its packed
// TF32 rows (a.bp): bit-identical to spmm_window_kernel<FS, TF32, U,
// MINB, false, NW, true>, with a quarter fewer gathered sectors.
template <int FS, int U, int MINB, int NW = kNW, bool PF = false, int PFK = 2, bool EPI = false>
__global__ void __launch_bounds__(NW * 32, MINB) spmm_window_packed_kernel(const SpmmArgs a) {
    extern __shared__ __align__(16) float smem[];
    float* part = smem;  // [2 * NW] slots
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * NW * 8 * FS);
    Block<FS, NW> blk;
    blk.init(a, s_rwo, part);
    // launched as a programmatic dependent of the packing launch: the block
    // set-up above overlaps its tail; the packed rows are read only after it
    // has finished and its writes are visible
    asm volatile("griddepcontrol.wait;" ::: "memory");
    direct_item_packed<FS, U, NW, PF, PFK, EPI>(a, blk);
}

// B rounded to TF32 (cvt.rna, as the SpMM's operands are) and packed row by
// row, 320 bytes per 128-column slice (`pitch` = 320 x slices, the last
// slice padded): every bit the tensor core reads (31..13) in 2.5 bytes a
// value, a gathered row one contiguous run in one DRAM page.  In a slice the
// SpMM lane of column group g takes values 32h + 4g + 0..3 (h = 0..3): their
// halfwords of bits 31..16 for h = 2hp, 2hp + 1 are 16 adjacent bytes at
// 128 hp + 16 g (one 16-byte load each), and bits 15..12 of all 16 values
// are 8 adjacent nibble bytes at 256 + 8 g (one 8-byte load), byte 2h + j / 2
// holding value j's bits in its high nibble for even j, low nibble for odd.
// One float4 of B per thread and step, read once with a streaming load.  (FS
// = 64: the same layout in 160-byte slices of 64 columns, pack_tf32_put.)
template <int FS = 128>
__global__ void pack_tf32_kernel(const float4* __restrict__ B, uint8_t* __restrict__ P, uint32_t K,
                                 uint32_t pitch, size_t n4, uint8_t* __restrict__ zero_row) {
    // the SpMM launched after this one may start its set-up once every block
    // of this grid has started
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t k4 = K / 4;
    // the zero row read for padding columns (pitch is a multiple of 8)
    if (blockIdx.x == 0)
        for (uint32_t j = threadIdx.x; j < pitch / 8; j += blockDim.x)
            reinterpret_cast<uint2*>(zero_row)[j] = make_uint2(0u, 0u);
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n4;
         i += size_t(gridDim.x) * blockDim.x) {
        const size_t row = i / k4;
        const uint32_t c = uint32_t(i - row * k4) * 4;
        pack_tf32_put<FS>(P + row * pitch, c, __ldcs(B + i));
    }
}

#ifdef ACCSPMM_LAB
// Zero source for the padding rows of a tile (FS <= 128 floats).
__device__ __align__(16) float g_zero_row_direct[128] = {0.f};

// Double-buffered register-direct kernel: the gathers of batch q + 1 are
// issued before the MMAs of batch q, so every warp keeps a batch of B rows
// in flight while it computes instead of alternating load and compute phases.
template <int FS, int PREC, int U, int MINB = 2>
__global__ void __launch_bounds__(kNW * 32, MINB) spmm_db_kernel(const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    constexpr int MA = (8 * U + 31) / 32;

    extern __shared__ __align__(16) float smem[];
    float* part = smem;
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * kNW * 8 * FS);
    Block<FS, kNW> blk;
    blk.init(a, s_rwo, part);
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    if (tb < te) {
        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        uint32_t ma[MA];
        uint64_t mb;
        uint32_t mo;
        auto load_meta = [&](uint32_t t) {
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                uint32_t e = 32 * j + lane;
                ma[j] = (e < 8 * U && t + e / 8 < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            uint32_t tl = t + uint32_t(lane);
            bool ok = lane < U && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };

        BitDecode dec;
        dec.init(g, tq);
        // lane offsets inside a row slice, clamped to the row; padding reads
        // a zero row
        const uint32_t kr = a.K - blk.f0;
        uint32_t off[H];
#pragma unroll
        for (int h = 0; h < H; ++h) off[h] = min(uint32_t(32 * h + 4 * g), kr - 4);
        const float* Bs = a.B + blk.f0;

        struct Batch {
            float4 r0[U][H], r1[U][H];
            float av0[U], av1[U];
        };
        auto gather = [&](Batch& bt) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
                const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
                const float* p0 = i0 < a.cols ? Bs + size_t(i0) * a.K : g_zero_row_direct;
                const float* p1 = i1 < a.cols ? Bs + size_t(i1) * a.K : g_zero_row_direct;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    bt.r0[u][h] = ldg_f4_ordered(p0 + off[h]);
                    bt.r1[u][h] = ldg_f4_ordered(p1 + off[h]);
                }
                const uint64_t bm = shfl_u64(mb, u);
                const uint32_t to = __shfl_sync(0xffffffffu, mo, u);
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm, x0, x1, q0, q1);
                bt.av0[u] = q0 ? ldg_f32_ordered(a.vals + to + x0) : 0.f;
                bt.av1[u] = q1 ? ldg_f32_ordered(a.vals + to + x1) : 0.f;
            }
        };
        auto compute = [&](uint32_t t, const Batch& bt) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t tt = t + u;
                if (tt >= te) break;
                if (tt >= next_bound) {
                    blk.flush(a, acc, wl, tb, te, first_win);
                    first_win = false;
#pragma unroll
                    for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                    while (blk.s_rwo[wl + 1] <= tt) ++wl;
                    next_bound = blk.s_rwo[wl + 1];
                }
                tile_mma<H, PREC>(acc, bt.r0[u], bt.r1[u], bt.av0[u], bt.av1[u]);
            }
        };

        Batch b0, b1;
        load_meta(tb);
        gather(b0);
        if (tb + U < te) load_meta(tb + U);
        for (uint32_t t = tb; t < te; t += 2 * U) {
            // b0 holds batch t, the metadata registers batch t + U
            if (t + U < te) {
                gather(b1);
                if (t + 2 * U < te) load_meta(t + 2 * U);
            }
            compute(t, b0);
            if (t + U >= te) break;
            // b1 holds batch t + U, the metadata registers batch t + 2U
            if (t + 2 * U < te) {
                gather(b0);
                if (t + 3 * U < te) load_meta(t + 3 * U);
            }
            compute(t + U, b1);
        }
        blk.flush(a, acc, wl, tb, te, first_win);
    }
    __syncthreads();
    blk.finish(a);
}

template <int FS, int PREC, int U, int MINB = 2>
int launch_db(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = size_t(2 * kNW * 8 * FS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_db_kernel<FS, PREC, U, MINB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_db_kernel<FS, PREC, U, MINB><<<unsigned(grid), kNW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

#endif  // ACCSPMM_LAB

// Sticky status of the SpMM calls on this device, reported and cleared by
// accspmm_device_status: kStatusTimeout -- a bounded wait on an asynchronous
// copy expired; kStatusRowsPastC -- an adaptive call's rowIndices named windows
// at or past c_rows / 8, whose tiles were left out of C; kStatusUnsorted -- an
// adaptive call's rowIndices were not non-decreasing multiples of 8 (tiles may
// have been summed into the wrong windows).
constexpr unsigned kStatusTimeout = 1u, kStatusRowsPastC = 2u, kStatusUnsorted = 4u;
__device__ unsigned int g_spmm_status = 0;

// The adaptive path's window offsets from an AdpBME's rowIndices, plus the
// checks of rowIndices that the derivation relies on, in one pass of
// max(T, Weff + 1) threads:
//  - thread w <= Weff: rwo[w] = first tile whose window start row is >= 8w (a
//    binary search; for any rowIndices the result is monotone in w and within
//    [0, T], so the SpMM reads only valid tiles whatever the input), and
//    w == Weff raises kStatusRowsPastC if tiles remain past the last window;
//  - thread t < T: rowIndices[t] must be a multiple of 8 not below
//    rowIndices[t - 1] (CSR2AdpBME writes the first row of each tile's window,
//    window by window, include/format.hpp:364), else kStatusUnsorted.
// Raised bits go to *err (when non-null) and, when `sticky`, to the device
// status word as well.
__global__ void rwo_from_row_indices_kernel(const uint32_t* __restrict__ ri, uint32_t T,
                                            uint32_t Weff, uint32_t* __restrict__ rwo,
                                            uint32_t* __restrict__ err, int sticky) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned bits = 0;
    if (i <= Weff) {
        const uint64_t row = uint64_t(i) * kWin;
        uint32_t lo = 0, hi = T;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (uint64_t(ri[mid]) < row) lo = mid + 1;
            else hi = mid;
        }
        rwo[i] = lo;
        if (i == Weff && lo < T) bits |= kStatusRowsPastC;
    }
    if (i < T) {
        const uint32_t r = ri[i];
        if ((r % kWin) != 0 || (i > 0 && ri[i - 1] > r)) bits |= kStatusUnsorted;
    }
    // one atomic per warp at most
    const unsigned any = __reduce_or_sync(0xffffffffu, bits);
    if (any && (threadIdx.x & 31) == 0) {
        if (err) atomicOr(err, any);
        if (sticky) atomicOr(&g_spmm_status, any);
    }
}

// The failure path of the bounded waits, exercised on purpose: one warp
// waits on an mbarrier that nothing arrives on.  The wait gives up after
// limit_ns, the kernel records kStatusTimeout and returns; nothing traps and
// the context stays usable.
__global__ void bounded_wait_selftest_kernel(uint64_t limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = smem_addr(&bar);
    if (threadIdx.x == 0) {
        mbar_init(b, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool landed = mbar_wait(b, 0u, limit_ns);  // phase 0 never completes
    if (!__all_sync(0xffffffffu, landed) && threadIdx.x == 0) atomicOr(&g_spmm_status, kStatusTimeout);
}

// Heaviest-first schedule of nb window blocks of wb windows: order[i] = the
// block with the i-th largest tile count (ties by block index).  One CTA
// sorts (~tiles, block) keys with a bitonic network in shared memory;
// P = nb rounded up to a power of two, at most kOrderMaxBlocks.
constexpr uint32_t kOrderMaxBlocks = 4096;
constexpr uint32_t kOrderMaxWaves = 6;  // launches of at most this many waves of CTAs

__global__ void __launch_bounds__(1024) block_order_kernel(const uint32_t* __restrict__ rwo, uint32_t W,
                                                           uint32_t wb, uint32_t nb, uint32_t P,
                                                           uint32_t* __restrict__ order) {
    extern __shared__ unsigned long long s_keys[];
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        unsigned long long k = ~0ull;
        if (i < nb) {
            const uint32_t w0 = i * wb, w1 = min(w0 + wb, W);
            const uint32_t tiles = rwo[w1] - rwo[w0];
            k = (static_cast<unsigned long long>(~tiles) << 32) | i;
        }
        s_keys[i] = k;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long x = s_keys[i], y = s_keys[ixj];
                    if ((x > y) == ((i & k) == 0)) {
                        s_keys[i] = y;
                        s_keys[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) order[i] = uint32_t(s_keys[i]);
}

// Heaviest-first schedules of library-owned matrices, per (window offsets,
// windows, windows per block, device).  The first call computes one on its
// stream and waits for it on the host, so every kept schedule is complete:
// later calls on any stream, including calls captured into a CUDA graph, use
// it without an event wait (a capturing stream may not wait on an event
// recorded outside the capture).
struct OrderKey {
    const uint32_t* rwo;
    uint32_t W, wb;
    int dev;
    bool operator<(const OrderKey& o) const {
        return std::tie(rwo, W, wb, dev) < std::tie(o.rwo, o.W, o.wb, o.dev);
    }
};
struct OrderEntry {
    uint32_t* order = nullptr;
};
std::mutex g_order_mu;
std::map<OrderKey, OrderEntry> g_order_cache;

int cached_order(const uint32_t* rwo, uint32_t W, uint32_t wb, uint32_t nb, cudaStream_t s,
                 const uint32_t** out) {
    int dev = 0;
    ACC_CUDA(cudaGetDevice(&dev));
    const OrderKey key{rwo, W, wb, dev};
    std::lock_guard<std::mutex> lock(g_order_mu);
    auto it = g_order_cache.find(key);
    if (it != g_order_cache.end()) {
        *out = it->second.order;
        return ACCSPMM_SUCCESS;
    }
    // a stream being captured into a graph may not allocate: keep the
    // launch order there (same results) until a call outside a capture
    // has built the schedule
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ACC_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
        *out = nullptr;
        return ACCSPMM_SUCCESS;
    }
    uint32_t P = 1;
    while (P < nb) P <<= 1;
    OrderEntry e;
    ACC_CUDA(cudaMalloc(&e.order, size_t(nb) * 4));
    block_order_kernel<<<1, 1024, size_t(P) * 8, s>>>(rwo, W, wb, nb, P, e.order);
    cudaError_t ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
        cudaStreamSynchronize(s);
        cudaFree(e.order);
        ACC_FAIL(ACCSPMM_ERROR_CUDA, "block schedule: %s", cudaGetErrorString(ce));
    }
    g_order_cache.emplace(key, e);
    *out = e.order;
    return ACCSPMM_SUCCESS;
}

}  // namespace

void schedule_cache_forget(const uint32_t* rwo) {
    std::lock_guard<std::mutex> lock(g_order_mu);
    for (auto it = g_order_cache.begin(); it != g_order_cache.end();) {
        if (it->first.rwo == rwo) {
            cudaFree(it->second.order);  // waits for queued work that reads it
            it = g_order_cache.erase(it);
        } else {
            ++it;
        }
    }
}

int rwo_from_row_indices(const uint32_t* ri, uint32_t T, uint32_t W, uint32_t* rwo, uint32_t* err,
                         bool sticky, cudaStream_t s) {
    const uint64_t n = std::max<uint64_t>(uint64_t(W) + 1, T);
    rwo_from_row_indices_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(ri, T, W, rwo, err, sticky ? 1 : 0);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

int bounded_wait_selftest(uint32_t limit_ms, cudaStream_t s) {
    if (limit_ms == 0 || limit_ms > 2000)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "limit_ms must be in [1, 2000]");
    bounded_wait_selftest_kernel<<<1, 32, 0, s>>>(uint64_t(limit_ms) * 1000000ull);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

int device_status_impl(void* stream) {
    ACC_CUDA(cudaStreamSynchronize(as_stream(stream)));
    unsigned int v = 0;
    ACC_CUDA(cudaMemcpyFromSymbol(&v, g_spmm_status, sizeof v));
    if (v) {
        const unsigned int z = 0;
        ACC_CUDA(cudaMemcpyToSymbol(g_spmm_status, &z, sizeof z));
    }
#ifdef ACCSPMM_LAB
    unsigned int vb = 0;
    if (int st = bulk_status_take(&vb)) return st;
    if (vb) v |= kStatusTimeout;
#endif
    if (v & (kStatusRowsPastC | kStatusUnsorted))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "an adaptive SpMM call since the last check had inconsistent rowIndices:%s%s%s",
                 (v & kStatusRowsPastC) ? " tiles of windows at or past c_rows / 8 were left out of C (c_rows too small);" : "",
                 (v & kStatusUnsorted) ? " rowIndices are not non-decreasing multiples of 8;" : "",
                 (v & kStatusTimeout) ? " a bounded wait also expired" : "");
    if (v & kStatusTimeout) ACC_FAIL(ACCSPMM_ERROR_TIMEOUT, "a bounded wait in the SpMM kernels expired");
    return ACCSPMM_SUCCESS;
}

namespace {

// Kernel kinds, the values of ACCSPMM_OPT_KERNEL.  The product library
// builds only kDirect (the register-direct kernels, with or without packed
// B); the others are measurement variants built into libaccspmm_lab.so.
enum KernelKind {
    kDirect = ACCSPMM_KERNEL_DIRECT,
    kPipe = ACCSPMM_KERNEL_PIPE,
    kBulk = ACCSPMM_KERNEL_BULK,
    kLean = ACCSPMM_KERNEL_LEAN,
    kDb = ACCSPMM_KERNEL_DB,
    kTma = ACCSPMM_KERNEL_TMA,
    kStaged = ACCSPMM_KERNEL_STAGED
};

struct Config {
    int kernel;
    int fs;
    int occ;   // register-direct kernel: resident CTAs per SM (2 or 3)
    int ring;  // register-direct kernel: rolling tile ring (-1 by the default rule, 0 off, 1 on)
    int nw;
    int hints;
    uint32_t wb;
    uint32_t slice_major;
    int pack;  // TF32 ring at 128-column slices: gather from a packed copy of B (-1 by the default rule, 0 off, 1 on)
};

// Tuned launch shapes, by matrix signature (autotune below).
struct TuneKey {
    uint32_t w, t, k;
    int prec;
    bool operator<(const TuneKey& o) const {
        return std::tie(w, t, k, prec) < std::tie(o.w, o.t, o.k, o.prec);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, Config> g_tuned;
// configuration forced by the autotuner while it times a candidate
thread_local const Config* g_forced = nullptr;

// Launch shape from (W, T, K, precision).  Defaults measured on GB300 with
// the 1M-row power-law workload (K = 32 ... 256), all register-direct with up
// to 32 windows per CTA (fewer for small matrices so that every SM gets work):
//  - TF32, K > 64: 128-column slices at 2 CTAs per SM with the rolling
//    two-tile ring (one slice decodes each tile once);
//  - TF32, 32 < K <= 64: 64-column slices at 3 CTAs per SM with the ring;
//  - 3xTF32 (K > 32): 64-column slices at 3 CTAs per SM, batch then compute
//    (the ring spills there);
//  - K <= 32: 32-column slices at 3 CTAs per SM, batch then compute.
// A shape found by accspmm_autotune_metcf for the same signature replaces
// the default; the launch options (accspmm_set_option: slice width, CTAs
// per SM, tile ring, windows per CTA, packing) override both.
Config choose_config(uint32_t W, uint32_t T, uint32_t K, int precision) {
    if (g_forced) return *g_forced;
    Config c;
    c.kernel = kDirect;
    c.fs = K <= 32 ? 32 : (K <= 64 || precision == ACCSPMM_PREC_3XTF32) ? 64 : 128;
    c.occ = c.fs == 128 ? 2 : 3;
    c.ring = -1;
    c.nw = c.fs == 32 ? 8 : 4;
    c.hints = 1;
    c.slice_major = 0;
    c.pack = -1;
    {
        uint64_t slices = (K + c.fs - 1) / c.fs;
        uint64_t want = uint64_t(sm_count()) * 4;
        uint64_t wb = std::max<uint64_t>(1, (uint64_t(W) * slices) / want);
        c.wb = uint32_t(std::min<uint64_t>(32, std::max<uint64_t>(2, wb)));
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(TuneKey{W, T, K, precision});
        if (it != g_tuned.end()) c = it->second;
    }
    c.kernel = option(ACCSPMM_OPT_KERNEL) != kDirect ? option(ACCSPMM_OPT_KERNEL) : c.kernel;
    if (const int fs = option(ACCSPMM_OPT_SLICE_WIDTH)) c.fs = fs;
    if (const int occ = option(ACCSPMM_OPT_CTAS_PER_SM)) c.occ = occ;
    if (const int ring = option(ACCSPMM_OPT_TILE_RING); ring >= 0) c.ring = ring;
    if (const int wb = option(ACCSPMM_OPT_WINDOWS_PER_CTA)) c.wb = uint32_t(wb);
    if (const int pk = option(ACCSPMM_OPT_PACK); pk >= 0) c.pack = pk;
#ifdef ACCSPMM_LAB
    // shape details of the measurement variants
    const int nw = lab_env("ACCSPMM_NW", 0);
    if (nw == 2 || nw == 4 || nw == 8) c.nw = nw;
    if (c.kernel == kPipe && c.fs >= 64) c.nw = 4;  // stage ring must fit in shared memory
    if ((c.kernel == kBulk || c.kernel == kTma) && c.nw == 8) c.nw = 4;
    c.hints = lab_env("ACCSPMM_HINTS", c.hints) ? 1 : 0;
    c.slice_major = lab_env("ACCSPMM_ORDER_SLICE", 0) ? 1u : 0u;
#endif
    return c;
}

template <int FS, int PREC, int U, int MINB, bool EPI, int NW = kNW, bool ROLL = false>
int launch_direct_t(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = size_t(2 * NW * 8 * FS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_window_kernel<FS, PREC, U, MINB, EPI, NW, ROLL>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_window_kernel<FS, PREC, U, MINB, EPI, NW, ROLL><<<unsigned(grid), NW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

// Whether the register-direct kernel uses the rolling tile ring by default
// (measured on GB300, 1M-row workload: 8-9 % faster for TF32 at 64 columns
// and 3 CTAs per SM, 3-4 % faster again at 128 columns and 2 CTAs per SM;
// slower where the ring spills: 32 columns, 3xTF32).
template <int FS, int PREC, int MINB>
constexpr bool kRollDefault = PREC == ACCSPMM_PREC_TF32 && ((FS == 64 && MINB == 3) || (FS == 128 && MINB == 2));

// occ = 2: the batch of DirectBatch (64 floats of B per lane in flight) at 2
// CTAs per SM; occ = 3: half that batch at 3 CTAs per SM (80 registers a
// thread), which keeps more warps' gathers in flight per SM.
template <int FS, int PREC>
int launch_direct(const SpmmArgs& a, int occ, int ring, cudaStream_t s) {
    const bool epi = a.bias != nullptr || a.act != 0;
    if (occ == 3) {
        constexpr int U = (DirectBatch<FS>::U + 1) / 2;
        const bool use_roll = ring < 0 ? kRollDefault<FS, PREC, 3> : ring != 0;
        if (use_roll) {
            if (epi) return launch_direct_t<FS, PREC, U, 3, true, kNW, true>(a, s);
            return launch_direct_t<FS, PREC, U, 3, false, kNW, true>(a, s);
        }
        if (epi) return launch_direct_t<FS, PREC, U, 3, true>(a, s);
        return launch_direct_t<FS, PREC, U, 3, false>(a, s);
    }
    constexpr int U = DirectBatch<FS>::U;
    if (ring < 0 ? kRollDefault<FS, PREC, 2> : ring != 0) {
        if (epi) return launch_direct_t<FS, PREC, U, 2, true, kNW, true>(a, s);
        return launch_direct_t<FS, PREC, U, 2, false, kNW, true>(a, s);
    }
    return epi ? launch_direct_t<FS, PREC, U, 2, true>(a, s) : launch_direct_t<FS, PREC, U, 2, false>(a, s);
}

template <int FS, int U, int MINB, bool PF = false, int PFK = 2, bool EPI = false>
int launch_packed_t(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = size_t(2 * kNW * 8 * FS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_window_packed_kernel<FS, U, MINB, kNW, PF, PFK, EPI>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    // a programmatic dependent launch of the packing kernel before it (the
    // kernel waits for it with griddepcontrol.wait before reading B)
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(unsigned(grid));
    lc.blockDim = dim3(kNW * 32);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    ACC_CUDA(cudaLaunchKernelEx(&lc, spmm_window_packed_kernel<FS, U, MINB, kNW, PF, PFK, EPI>, a));
    return ACCSPMM_SUCCESS;
}

}  // namespace

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!cached[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 148;
    }
    return cached[dev];
}

uint32_t window_block_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision) {
    return choose_config(w_cfg, T, K, precision).wb;
}

void launch_shape_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision, int* fs, int* occ,
                      uint32_t* wb) {
    const Config c = choose_config(w_cfg, T, K, precision);
    *fs = c.fs;
    *occ = c.kernel == kDirect ? c.occ : 2;
    *wb = c.wb;
}

uint32_t slice_width_for(uint32_t w_cfg, uint32_t T, uint32_t K, int precision) {
    return uint32_t(choose_config(w_cfg, T, K, precision).fs);
}

int spmm_window_launch(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                       const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                       uint32_t T, uint32_t cols, const float* B, float* C, uint32_t K,
                       int precision, cudaStream_t s, bool stable_rwo, bool allow_pack) {
    return spmm_window_launch_slices(rwo, tc_offset, bits, a2b, vals, W, w_cfg, T, cols, B, C, K,
                                     precision, 0, 0xFFFFFFFFu, Epilogue{}, s, 0, stable_rwo,
                                     allow_pack);
}

int spmm_window_launch_slices(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                              const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                              uint32_t T, uint32_t cols, const float* B, float* C, uint32_t K,
                              int precision, uint32_t slice_begin, uint32_t slice_count,
                              const Epilogue& epi, cudaStream_t s, int slice_fs, bool stable_rwo,
                              bool allow_pack) {
    if (W == 0) return ACCSPMM_SUCCESS;
    // the launch shape depends only on (w_cfg, T, K, precision), so every
    // entry point cuts a matrix into the same pieces and sums partial windows
    // in the same order
    Config cfg = choose_config(w_cfg, T, K, precision);
    // The bias/activation epilogue lengthens the store path inside the tile
    // loop; at 128-column slices that made the register-direct kernel reading
    // fp32 B spill (2.76 ms against 2.31 ms without the epilogue on the
    // 1M-row matrix at K = 128), so epilogue launches that do not pack B use
    // 64-column slices at 3 CTAs per SM, which keep the ring without spilling
    // (2.56 ms, against 2.78 ms for the SpMM followed by a separate bias +
    // ReLU pass).  The packed-B kernel keeps its 128 registers without spills
    // with the epilogue, so launches that pack B keep 128-column slices.
    // Same blocks, same arithmetic.
    const bool packs_at_128 = allow_pack && precision == ACCSPMM_PREC_TF32 && cfg.fs == 128 && cfg.occ == 2 &&
                              cfg.ring != 0 &&
                              (cfg.pack > 0 || (cfg.pack < 0 && uint64_t(cols) * K * 4 >= (uint64_t(4) << 20)));
    if ((epi.bias || epi.act) && !slice_fs && cfg.fs == 128 && !packs_at_128) slice_fs = 64;
    if (slice_fs && slice_fs != cfg.fs) {
        // another slice width (the feature columns a CTA covers do not change
        // any element's arithmetic; the window blocks stay the chooser's)
        cfg.fs = slice_fs;
        cfg.kernel = kDirect;
        cfg.occ = slice_fs == 128 ? 2 : 3;
    }
    const uint32_t slices = (K + uint32_t(cfg.fs) - 1) / uint32_t(cfg.fs);
    if (slice_begin >= slices) return ACCSPMM_SUCCESS;
    slice_count = std::min(slice_count, slices - slice_begin);
    SpmmArgs a{rwo, tc_offset, bits, a2b, vals, B, C, W, cols, K, cfg.wb, slice_count,
               (W + cfg.wb - 1) / cfg.wb, cfg.slice_major, slice_begin, epi.bias, epi.act, nullptr,
               nullptr, 0};
    // A launch of a few waves ends with its heaviest window blocks: run them
    // first (longest-processing-time order).  Larger launches keep window
    // order, which keeps neighbouring windows' B rows in L2 together.  On the
    // 16,384-row symmetric power-law matrix at K = 128 (683 blocks of 3
    // windows, the heaviest 260 tiles against a mean of 95) the adaptive
    // SpMM took 53.0 us instead of 62.0 us.
    if (stable_rwo && !cfg.slice_major && a.n_wblocks <= kOrderMaxBlocks &&
        uint64_t(a.n_wblocks) * a.n_slices <= uint64_t(kOrderMaxWaves) * sm_count() * uint32_t(cfg.occ) &&
        option(ACCSPMM_OPT_SCHEDULE) != 0) {
        int st = cached_order(rwo, W, cfg.wb, a.n_wblocks, s, &a.order);
        if (st) return st;
    }
    // only the register-direct kernel has the epilogue; it cuts the matrix
    // into the same pieces as the other variants
    if (epi.bias || epi.act) cfg.kernel = kDirect;
    const bool x3 = precision == ACCSPMM_PREC_3XTF32;
#ifdef ACCSPMM_LAB
    if (cfg.kernel == kPipe) return launch_pipe(a, cfg.fs, precision, cfg.nw, cfg.hints, s);
    if (cfg.kernel == kBulk) return launch_bulk(a, cfg.fs, precision, cfg.nw, cfg.hints, s);
    if (cfg.kernel == kTma) return launch_tma(a, cfg.fs, precision, cfg.nw, s);
    if (cfg.kernel == kLean) return launch_lean(a, cfg.fs, precision, lab_env("ACCSPMM_MINB", 4), s);
    if (cfg.kernel == kDb) {
        const int u = lab_env("ACCSPMM_U", 0);
        switch (cfg.fs) {
            case 32: return x3 ? launch_db<32, ACCSPMM_PREC_3XTF32, 4>(a, s) : launch_db<32, ACCSPMM_PREC_TF32, 4>(a, s);
            case 64:
                if (u == 1) return x3 ? launch_db<64, ACCSPMM_PREC_3XTF32, 1>(a, s) : launch_db<64, ACCSPMM_PREC_TF32, 1>(a, s);
                return x3 ? launch_db<64, ACCSPMM_PREC_3XTF32, 2>(a, s) : launch_db<64, ACCSPMM_PREC_TF32, 2>(a, s);
            default: return x3 ? launch_db<128, ACCSPMM_PREC_3XTF32, 1>(a, s) : launch_db<128, ACCSPMM_PREC_TF32, 1>(a, s);
        }
    }
    if (cfg.kernel == kStaged) {
        // the slice-major staged kernel covers whole launches in TF32 only
        const bool whole = slice_begin == 0 && uint64_t(slice_count) * uint32_t(cfg.fs) >= K;
        if (!x3 && whole) {
            cudaMemPool_t pool;
            int st = library_pool(&pool);
            if (st) return st;
            void* S = nullptr;
            ACC_CUDA(cudaMallocFromPoolAsync(&S, staged_bytes(cols, K), pool, s));
            st = spmm_staged_launch(a, B, static_cast<float*>(S), uint32_t(lab_env("ACCSPMM_STAGE_V", 0)), s);
            cudaFreeAsync(S, s);
            if (st) ACC_FAIL(st, "staged SpMM launch failed");
            return ACCSPMM_SUCCESS;
        }
    }
#endif
    const int occ = cfg.occ;
    // TF32 at 128-column slices with the ring: B is first rounded to TF32 and
    // packed to 2.5 bytes a value (pack_tf32_kernel), so the SpMM gathers 10
    // of every 16 sectors of a row in 3 instead of 4 loads; the MMAs see the
    // same operand bits, so the results are bit-identical.  The default rule
    // packs a B of at least 4 MiB; per adaptive call, packing included,
    // against the same launch reading fp32 B: 1M-row power-law matrix 1.64
    // against 2.29 ms at K = 128; 524,288 rows 0.85 against 1.23 ms (K = 128)
    // and 1.68 against 2.30 ms (K = 256); 65,536 rows 111 against 164 us; the
    // 16,384-row symmetric matrix (an 8 MiB B that fits the L2) 43.7 against
    // 52.4 us.  (At 64-column slices, K = 64, a 3-byte packing cost what the
    // gathers saved.)  The autotuner times both ways.
    const bool ring_on = cfg.ring != 0;
    const uint64_t b_bytes = uint64_t(cols) * K * 4;
    const bool pack_rule = cfg.pack > 0 || (cfg.pack < 0 && b_bytes >= (uint64_t(4) << 20));
    const bool wide_pack = cfg.fs == 128 && occ == 2 && pack_rule;
    // 64-column slices at 3 CTAs per SM (the default for 32 < K <= 64):
    // 160-byte packed slices of 64 columns, by default for 48 < K <= 64 with a
    // B of at least 4 MiB: adaptive step, packing included, at K = 64 1.07
    // against 1.27 ms on the 1M-row power-law matrix, 255 against 326 us on
    // 262,144 rows, 78 against 102 us on 65,536, 30.9 against 33.1 us on the
    // 16,384-row matrix; at K = 48 (a packed slice still holds 64 columns)
    // 1.07 against 1.08 ms on 1M rows but 30.2 against 28.0 us on 16K rows
    const bool narrow_pack = cfg.fs == 64 && occ == 3 &&
                             (cfg.pack > 0 || (cfg.pack < 0 && K > 48 && K <= 64 && b_bytes >= (uint64_t(4) << 20)));
    // 32-column slices at 3 CTAs per SM (the default for K <= 32): 80-byte
    // packed slices, by default with a B of at least 4 MiB: adaptive step,
    // packing included, 1M-row power-law matrix 0.63 against 0.84 ms at
    // K = 32 and 0.61 against 0.73 ms at K = 16; 262,144 rows 165 against
    // 196 us (K = 32); 65,536 rows 54 against 62 us (K = 32) and 53.5
    // against 55.7 us (K = 16, a 4 MiB B); a 2 MiB B (the 16,384-row matrix
    // at K = 32) lost, 24.8 against 20.8 us
    const bool tiny_pack = cfg.fs == 32 && occ == 3 &&
                           (cfg.pack > 0 || (cfg.pack < 0 && b_bytes >= (uint64_t(4) << 20)));
    const bool epi_on = epi.bias || epi.act;
    if (allow_pack && !x3 && ring_on && (wide_pack || narrow_pack || tiny_pack)) {
        cudaMemPool_t pool;
        int st = library_pool(&pool);
        if (st) return st;
        const uint32_t fs = uint32_t(cfg.fs);
        const uint32_t pitch = (fs * 5 / 2) * ((K + fs - 1) / fs);
        void* packed = nullptr;
        ACC_CUDA(cudaMallocFromPoolAsync(&packed, (size_t(cols) + 1) * pitch + 64, pool, s));
        a.bp = static_cast<const uint8_t*>(packed);
        a.bpitch = pitch;
        const size_t n4 = size_t(cols) * (K / 4);
        const unsigned blocks = unsigned(std::min<size_t>((n4 + 255) / 256 + 1, size_t(sm_count()) * 16));
        // the packed rows, then the zero row at index cols that padding reads
        if (fs == 32)
            pack_tf32_kernel<32><<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(B), static_cast<uint8_t*>(packed),
                                                        K, pitch, n4, static_cast<uint8_t*>(packed) + size_t(cols) * pitch);
        else if (fs == 64)
            pack_tf32_kernel<64><<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(B), static_cast<uint8_t*>(packed),
                                                        K, pitch, n4, static_cast<uint8_t*>(packed) + size_t(cols) * pitch);
        else
            pack_tf32_kernel<128><<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(B), static_cast<uint8_t*>(packed),
                                                         K, pitch, n4, static_cast<uint8_t*>(packed) + size_t(cols) * pitch);
        st = cudaGetLastError() == cudaSuccess ? ACCSPMM_SUCCESS : ACCSPMM_ERROR_CUDA;
        // the B rows of the tile group two ahead are prefetched into L2,
        // bit-identical; by default only when K spans an odd number of
        // 128-column slices: on the 1M-row power-law matrix (adaptive step)
        // the prefetch measured 1.643 against 1.667 ms at K = 128 and 4.64
        // against 4.80 ms at K = 384, but 3.41 against 3.34 ms at K = 256,
        // 3.31 against 3.24 at K = 192 and 6.71 against 6.57 at K = 512
        const int pf_opt = option(ACCSPMM_OPT_PREFETCH);
        const bool pf = pf_opt == 1 || (pf_opt < 0 && (a.n_slices & 1u));
        // the same rule for 160-byte slices: K = 64 (one slice) 1.040
        // against 1.064 ms per adaptive step on the 1M-row matrix
        const bool pf64 = pf;
        const bool pf32 = pf_opt == 1;
        if (st == ACCSPMM_SUCCESS && fs == 32) {
            if (epi_on)
                st = launch_packed_t<32, 4, 3, false, 2, true>(a, s);
            else
                st = pf32 ? launch_packed_t<32, 4, 3, true>(a, s) : launch_packed_t<32, 4, 3>(a, s);
        } else if (st == ACCSPMM_SUCCESS && fs == 64) {
            // two tiles in flight per warp at 3 CTAs per SM, the unpacked
            // 64-column default's shape
            if (epi_on)
                st = launch_packed_t<64, 2, 3, false, 2, true>(a, s);
            else
                st = pf64 ? launch_packed_t<64, 2, 3, true>(a, s) : launch_packed_t<64, 2, 3>(a, s);
        } else if (st == ACCSPMM_SUCCESS && epi_on) {
            st = pf ? launch_packed_t<128, DirectBatch<128>::U, 2, true, 2, true>(a, s)
                    : launch_packed_t<128, DirectBatch<128>::U, 2, false, 2, true>(a, s);
        } else if (st == ACCSPMM_SUCCESS) {
#ifdef ACCSPMM_LAB
            if (pf && lab_env("ACCSPMM_PFK", 2) == 1)
                st = launch_packed_t<128, DirectBatch<128>::U, 2, true, 1>(a, s);
            else
#endif
            st = pf ? launch_packed_t<128, DirectBatch<128>::U, 2, true>(a, s)
                    : launch_packed_t<128, DirectBatch<128>::U, 2>(a, s);
        }
        cudaFreeAsync(packed, s);
        if (st) ACC_FAIL(st, "packed SpMM launch failed");
        return ACCSPMM_SUCCESS;
    }
    switch (cfg.fs) {
        case 32: return x3 ? launch_direct<32, ACCSPMM_PREC_3XTF32>(a, occ, cfg.ring, s) : launch_direct<32, ACCSPMM_PREC_TF32>(a, occ, cfg.ring, s);
        case 64: return x3 ? launch_direct<64, ACCSPMM_PREC_3XTF32>(a, occ, cfg.ring, s) : launch_direct<64, ACCSPMM_PREC_TF32>(a, occ, cfg.ring, s);
        default: return x3 ? launch_direct<128, ACCSPMM_PREC_3XTF32>(a, occ, cfg.ring, s) : launch_direct<128, ACCSPMM_PREC_TF32>(a, occ, cfg.ring, s);
    }
}

static int check_dense(const float* B, const float* C, uint32_t K, int precision) {
    if (K == 0 || (K % 4) != 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K=%u must be a positive multiple of 4", K);
    if (!B || !C) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "B and C must be device pointers");
    if ((reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(C)) & 15u)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "B and C must be 16-byte aligned");
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    return ACCSPMM_SUCCESS;
}

int spmm_tf32_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                   void* stream) {
    if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    int st = check_dense(B, C, K, precision);
    if (st) return st;
    return spmm_window_launch(m->row_window_offset, m->tc_offset, m->tc_local_bit, m->sparse_a2b,
                              m->data, m->num_windows, m->num_windows, m->num_tiles, m->cols, B, C,
                              K, precision, as_stream(stream), m->owned != 0, true);
}

int spmm_bias_act_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K,
                       int precision, const float* bias, int act, void* stream) {
    if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    int st = check_dense(B, C, K, precision);
    if (st) return st;
    if (reinterpret_cast<uintptr_t>(bias) & 15u)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bias must be 16-byte aligned");
    if (act != ACCSPMM_ACT_NONE && act != ACCSPMM_ACT_RELU)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown activation %d", act);
    Epilogue epi;
    epi.bias = bias;
    epi.act = uint32_t(act);
    return spmm_window_launch_slices(m->row_window_offset, m->tc_offset, m->tc_local_bit,
                                     m->sparse_a2b, m->data, m->num_windows, m->num_windows,
                                     m->num_tiles, m->cols, B, C, K, precision, 0, 0xFFFFFFFFu, epi,
                                     as_stream(stream), 0, m->owned != 0, true);
}

namespace {

// Window offsets derived from the rowIndices of library-owned AdpBME objects,
// kept per (rowIndices array, window count, device) so that repeated adaptive
// calls on one object derive them once.  Library-owned arrays are not changed
// after they are built; accspmm_adpbme_destroy forgets the object's entries.
// The first call derives them on its stream and waits for that on the host,
// so kept offsets are complete and later calls on any stream, or captured
// into a CUDA graph, use them without an event wait.
struct RwoKey {
    const uint32_t* ri;
    uint32_t weff;
    int dev;
    bool operator<(const RwoKey& o) const { return std::tie(ri, weff, dev) < std::tie(o.ri, o.weff, o.dev); }
};
struct RwoEntry {
    uint32_t* rwo = nullptr;  // [weff + 2]: offsets, then an error word
    uint32_t err = 0;         // that error word, read once when the offsets were derived
};
std::mutex g_rwo_mu;
std::map<RwoKey, RwoEntry> g_rwo_cache;

// Cached offsets of an owned AdpBME (computed on `s`, and waited for, the
// first time).
int cached_rwo(const accspmm_adpbme_t* ad, uint32_t Weff, cudaStream_t s, const uint32_t** out) {
    int dev = 0;
    ACC_CUDA(cudaGetDevice(&dev));
    const RwoKey key{ad->row_indices, Weff, dev};
    std::lock_guard<std::mutex> lock(g_rwo_mu);
    auto it = g_rwo_cache.find(key);
    if (it == g_rwo_cache.end()) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        ACC_CUDA(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED,
                     "the first adaptive call on an AdpBME derives its window offsets and must not be "
                     "captured into a graph: call it once outside the capture");
        RwoEntry e;
        ACC_CUDA(cudaMalloc(&e.rwo, (size_t(Weff) + 2) * 4));
        cudaError_t ce = cudaMemsetAsync(e.rwo + Weff + 1, 0, 4, s);
        if (ce == cudaSuccess) {
            const uint64_t n = std::max<uint64_t>(uint64_t(Weff) + 1, ad->num_tiles);
            rwo_from_row_indices_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(
                ad->row_indices, ad->num_tiles, Weff, e.rwo, e.rwo + Weff + 1, 0);
            ce = cudaGetLastError();
        }
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
        if (ce == cudaSuccess) ce = cudaMemcpy(&e.err, e.rwo + Weff + 1, 4, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) {
            cudaStreamSynchronize(s);
            cudaFree(e.rwo);
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "window-offset cache: %s", cudaGetErrorString(ce));
        }
        it = g_rwo_cache.emplace(key, e).first;
    }
    // a library-built AdpBME always passes; the check matters for one loaded
    // from a file or copied from a caller's arrays
    if (it->second.err & kStatusUnsorted)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "AdpBME rowIndices are not non-decreasing multiples of 8");
    if (it->second.err & kStatusRowsPastC)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE,
                 "c_rows=%u leaves tiles of later windows out of C: it must be at least the last rowIndices "
                 "entry + 8 (accspmm_adaptive_c_rows)", Weff * kWin);
    *out = it->second.rwo;
    return ACCSPMM_SUCCESS;
}

}  // namespace

int adaptive_rwo(const accspmm_adpbme_t* ad, uint32_t W, cudaStream_t s, const uint32_t** out) {
    if (!ad->owned) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "only library-owned AdpBME objects are cached");
    return cached_rwo(ad, W, s, out);
}

void adaptive_cache_forget(const accspmm_adpbme_t* ad) {
    std::lock_guard<std::mutex> lock(g_rwo_mu);
    for (auto it = g_rwo_cache.begin(); it != g_rwo_cache.end();) {
        if (it->first.ri == ad->row_indices) {
            schedule_cache_forget(it->second.rwo);
            cudaFree(it->second.rwo);  // waits for queued work that reads it
            it = g_rwo_cache.erase(it);
        } else {
            ++it;
        }
    }
}

int spmm_adaptive_impl(const accspmm_adpbme_t* ad, const float* B, float* C, uint32_t c_rows,
                       uint32_t K, int precision, void* stream) {
    if (!ad || ad->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "AdpBME must be on the device");
    int st = check_dense(B, C, K, precision);
    if (st) return st;
    if (c_rows % kWin) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "c_rows=%u must be a multiple of 8", c_rows);
    cudaStream_t s = as_stream(stream);
    const uint32_t Weff = c_rows / kWin, T = ad->num_tiles;
    if (Weff == 0) return ACCSPMM_SUCCESS;
    if (ad->owned) {
        const uint32_t* rwo = nullptr;
        st = cached_rwo(ad, Weff, s, &rwo);
        if (st) return st;
        return spmm_window_launch(rwo, ad->tc_offset, ad->tc_local_bit, ad->sparse_a2b, ad->data, Weff,
                                  (ad->rows + kWin - 1) / kWin, T, ad->cols, B, C, K, precision, s, true,
                                  true);
    }
    // a caller-filled object may change between calls: derive every time,
    // in stream order (inconsistent rowIndices raise the device status word
    // that accspmm_device_status reports; no host wait here)
    DevBuf<uint32_t> scratch;  // rwo[Weff + 1]
    ACC_CUDA(scratch.alloc(size_t(Weff) + 1, s));
    uint32_t* rwo = scratch.p;
    st = rwo_from_row_indices(ad->row_indices, T, Weff, rwo, nullptr, true, s);
    if (st) return st;
    return spmm_window_launch(rwo, ad->tc_offset, ad->tc_local_bit, ad->sparse_a2b, ad->data, Weff,
                              (ad->rows + kWin - 1) / kWin, T, ad->cols, B, C, K, precision, s, false,
                              true);
}

// ---------------------------------------------------------------------------
// Allocation-free adaptive SpMM.  Callers that may not allocate device memory
// -- plugins inside a host application that owns all device memory through
// its own pool, latency-critical loops in which cudaFree's device-wide
// synchronisation would stall other streams, processes whose memory budget
// is fixed at start-up -- use this variant: its only scratch (the
// rowWindowOffset derived from rowIndices plus a status word) lives in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits.  All calls share the array, so calls that overlap on the
// GPU (different streams, no ordering between them) race on it.  It never
// packs B (that copy would need a scratch the size of B), so on a B of
// 4 MiB or more at K <= 32 or K > 48 it runs the kernel that reads fp32 B: the same
// bits, 2.29 against 1.64 ms on the 1M-row power-law matrix at K = 128.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoAllocWords = 1u << 20;  // 4 MiB: windows + 2 words
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (the host-side symbol is not a device address) and kept for the
// life of the process: it belongs to the device's primary context, so it does
// not survive a cudaDeviceReset of that device.
static int noalloc_scratch(uint32_t** out) {
    static std::mutex mu;
    static uint32_t* ptr[64] = {nullptr};
    int dev = 0;
    ACC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            ACC_FAIL(ACCSPMM_ERROR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                     cudaGetErrorString(e));
        ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = ptr[dev];
    return ACCSPMM_SUCCESS;
}

uint32_t noalloc_max_c_rows() { return (kNoAllocWords - 2) * kWin; }

int spmm_adaptive_noalloc_impl(const accspmm_adpbme_t* ad, const float* B, float* C,
                               uint32_t c_rows, uint32_t K, int precision, void* stream) {
    if (!ad || ad->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "AdpBME must be on the device");
    int st = check_dense(B, C, K, precision);
    if (st) return st;
    if (c_rows % kWin) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "c_rows=%u must be a multiple of 8", c_rows);
    if (c_rows > noalloc_max_c_rows())
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE,
                 "c_rows=%u exceeds the allocation-free maximum of %u rows; use accspmm_spmm_adaptive",
                 c_rows, noalloc_max_c_rows());
    cudaStream_t s = as_stream(stream);
    const uint32_t Weff = c_rows / kWin, T = ad->num_tiles;
    if (Weff == 0) return ACCSPMM_SUCCESS;
    uint32_t* scratch = nullptr;
    st = noalloc_scratch(&scratch);
    if (st) return st;
    uint32_t* rwo = scratch;  // [Weff + 1], fully rewritten below
    // inconsistent rowIndices raise the device status word that
    // accspmm_device_status reports (no host wait, nothing else to clear)
    st = rwo_from_row_indices(ad->row_indices, T, Weff, rwo, nullptr, true, s);
    if (st) return st;
    return spmm_window_launch(rwo, ad->tc_offset, ad->tc_local_bit, ad->sparse_a2b, ad->data, Weff,
                              (ad->rows + kWin - 1) / kWin, T, ad->cols, B, C, K, precision, s);
}

// Times the candidate launch shapes on (m, B, C) and keeps the fastest for
// m's signature.  C is overwritten.
int autotune_impl(const accspmm_metcf_t* m, const float* B, float* C, uint32_t K, int precision,
                  void* stream, accspmm_tune_result_t* out) {
    if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    int st = check_dense(B, C, K, precision);
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    const TuneKey key{m->num_windows, m->num_tiles, K, precision};
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tuned.erase(key);
    }
    const Config dflt = choose_config(m->num_windows, m->num_tiles, K, precision);
    std::vector<Config> cand;
    // (kernel, CTAs per SM, tile ring): register-direct at 3 and 2 CTAs per
    // SM with and without the rolling ring, double-buffered at 2
#ifdef ACCSPMM_LAB
    const int shapes[][3] = {{kDirect, 3, 1}, {kDirect, 3, 0}, {kDirect, 2, 1}, {kDirect, 2, 0}, {kDb, 2, 0}};
#else
    const int shapes[][3] = {{kDirect, 3, 1}, {kDirect, 3, 0}, {kDirect, 2, 1}, {kDirect, 2, 0}};
#endif
    for (const auto& ko : shapes)
        for (int fs : {32, 64, 128}) {
            if (fs > 32 && uint32_t(fs / 2) >= K) continue;  // slices far wider than K
            for (uint32_t wb : {1u, 2u, 4u, 8u, 16u, 32u}) {
                // 1 and 2 windows per CTA only where the chooser itself goes
                // below 4 (matrices of a few thousand windows)
                if (wb < 4 && dflt.wb >= 4) continue;
                Config c = dflt;
                c.kernel = ko[0];
                c.occ = ko[1];
                c.ring = ko[2];
                c.fs = fs;
                c.wb = wb;
                c.slice_major = 0;
                c.pack = 0;
                cand.push_back(c);
                // TF32 with the ring at 128-column slices (2 CTAs per SM), 64
                // or 32 (3): also gathering from a packed B
                if (precision == ACCSPMM_PREC_TF32 && c.kernel == kDirect && c.ring == 1 &&
                    ((fs == 128 && c.occ == 2) || (fs <= 64 && c.occ == 3))) {
                    c.pack = 1;
                    cand.push_back(c);
                }
            }
        }
    cudaEvent_t e0, e1;
    ACC_CUDA(cudaEventCreate(&e0));
    ACC_CUDA(cudaEventCreate(&e1));
    auto time_cfg = [&](const Config& c, float* ms) -> int {
        g_forced = &c;
        int r = 0;
        for (int i = 0; i < 1 && !r; ++i) r = spmm_tf32_impl(m, B, C, K, precision, stream);
        cudaEventRecord(e0, s);
        for (int i = 0; i < 3 && !r; ++i) r = spmm_tf32_impl(m, B, C, K, precision, stream);
        cudaEventRecord(e1, s);
        g_forced = nullptr;
        if (r) return r;
        ACC_CUDA(cudaEventSynchronize(e1));
        ACC_CUDA(cudaEventElapsedTime(ms, e0, e1));
        *ms /= 3.f;
        return ACCSPMM_SUCCESS;
    };
    float best_ms = 1e30f, dflt_ms = 0.f;
    Config best = dflt;
    st = time_cfg(dflt, &dflt_ms);
    if (!st) {
        best_ms = dflt_ms;
        for (const Config& c : cand) {
            float ms = 0.f;
            st = time_cfg(c, &ms);
            if (st) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = c;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tuned[key] = best;
    }
    if (out) {
        out->kernel = best.kernel;
        out->ctas_per_sm = best.kernel == kDirect ? uint32_t(best.occ) : 2u;
        out->tile_ring = best.kernel == kDirect ? (best.ring < 0 ? -1 : best.ring) : 0;
        out->slice_width = uint32_t(best.fs);
        out->windows_per_cta = best.wb;
        out->best_ms = best_ms;
        out->default_ms = dflt_ms;
        out->candidates = uint32_t(cand.size()) + 1;
        out->packed_b = best.pack;
    }
    return ACCSPMM_SUCCESS;
}

void autotune_clear() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned.clear();
}


int time_spmm_impl(const accspmm_metcf_t* m, const accspmm_adpbme_t* ad, const float* B, float* C,
                   uint32_t c_rows, uint32_t K, int precision, int warmup, int exe, float* avg_ms,
                   void* stream) {
    if (!avg_ms || exe <= 0 || warmup < 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad timing arguments");
    cudaStream_t s = as_stream(stream);
    auto run = [&]() -> int {
        return ad ? spmm_adaptive_impl(ad, B, C, c_rows, K, precision, stream)
                  : spmm_tf32_impl(m, B, C, K, precision, stream);
    };
    for (int i = 0; i < warmup; ++i) {
        int st = run();
        if (st) return st;
    }
    ACC_CUDA(cudaStreamSynchronize(s));
    cudaEvent_t e0, e1;
    ACC_CUDA(cudaEventCreate(&e0));
    ACC_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, s);
    int st = 0;
    for (int i = 0; i < exe && !st; ++i) st = run();
    cudaEventRecord(e1, s);
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    if (ce != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_CUDA, "timing failed: %s", cudaGetErrorString(ce));
    *avg_ms = ms / float(exe);
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
