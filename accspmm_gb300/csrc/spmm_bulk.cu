// spmm_bulk.cu -- the SpMM kernel fed by bulk asynchronous copies (TMA).
//
// Same decomposition and arithmetic as the other SpMM kernels (a CTA per
// window block and feature slice, equal per-warp tile pieces, partial windows
// summed in warp order).  Each warp owns a ring of D shared-memory stages of U
// tiles (B rows [U][8][FS] floats plus the tiles' bitmaps and value offsets)
// with one mbarrier per stage.  For batch q + D - 1 the warp's lane 8u + k
// issues one cp.async.bulk of row k of tile u -- min(FS, K - f0) floats of B
// row sparseA2B[8t + 8u + k], or of a static zero row for padding -- and lane 0
// posts the expected byte count; the warp then waits for batch q's barrier
// and runs the MMAs from shared memory.  Gathers of 8U rows per instruction
// keep up to (D - 1) U tiles of B in flight per warp without holding them in
// registers.  Every wait is bounded: if a barrier does not complete within
// the limit the kernel records ACCSPMM_ERROR_TIMEOUT in a device status word
// (read by accspmm_device_status), stops consuming, waits (bounded) for its
// own copies in flight and finishes normally.
//
// The tensor-map variant (spmm_tma_kernel, ACCSPMM_KERNEL=tma) issues the same
// gathers four rows at a time with cp.async.bulk.tensor.2d ... tile::gather4:
// B is described by a 2D tensor map (K x cols floats, box FS x 1), each
// instruction copies the FS-float slices of four B rows named by sparseA2B
// into the stage, and a padding entry (UINT32_MAX, row -1) or a column past
// cols lies outside the tensor and is filled with zeros by the copy engine,
// so no zero-row source is needed.
#include <cuda.h>

#include <mutex>

#include "common.hpp"
#include "device_util.cuh"
#include "mbarrier.cuh"
#include "spmm_common.cuh"

namespace accspmm {

// Zero source for the padding rows of a tile (FS <= 128 floats).
static __device__ __align__(16) float g_zero_row[128] = {0.f};
// Sticky status of this file's bounded waits that expired (0 = none), folded
// into accspmm_device_status by bulk_status_take.
static __device__ unsigned int g_bulk_status = 0;

namespace {

template <int FS>
struct BulkCfg {
    static constexpr int kU = FS >= 128 ? 2 : (FS == 64 ? 4 : 8);  // tiles per batch
    static constexpr int kD = 4;                                    // stages per warp
    static constexpr int kB = kU * 8 * FS;                          // floats of B per stage
    static constexpr int kMeta = kU * 4;                            // (bits lo, hi, off, -) per tile
    static constexpr int kStage = kB + kMeta;                       // floats per stage
};

template <bool HINTS>
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar,
                                          uint64_t pol) {
    if constexpr (HINTS) {
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint "
            "[%0], [%1], %2, [%3], %4;" ::"r"(dst),
            "l"(src), "r"(bytes), "r"(bar), "l"(pol)
            : "memory");
    } else {
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
            "l"(src), "r"(bytes), "r"(bar)
            : "memory");
    }
}

template <int FS, int PREC, int NW, bool HINTS>
__global__ void __launch_bounds__(NW * 32) spmm_bulk_kernel(const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    using Cf = BulkCfg<FS>;
    constexpr int kU = Cf::kU, kD = Cf::kD;
    constexpr int MA = (8 * kU + 31) / 32;
    static_assert(8 * kU <= 64, "at most two a2b registers per lane");

    extern __shared__ __align__(128) float smem[];
    float* ring = smem;                                      // [NW][kD][kStage]
    float* part = ring + size_t(NW) * kD * Cf::kStage;       // [2 NW][8][FS]
    uint64_t* bars = reinterpret_cast<uint64_t*>(part + 2 * NW * 8 * FS);  // [NW][kD]
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(bars + NW * kD);

    Block<FS, NW> blk;
    blk.init(a, s_rwo, part);
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    uint64_t pol_keep = 0;
    if constexpr (HINTS) asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));

    if (tb < te) {
        float* my_ring = ring + size_t(blk.warp) * kD * Cf::kStage;
        const uint32_t bar0 = smem_addr(bars + blk.warp * kD);
        if (lane == 0) {
            for (int d = 0; d < kD; ++d) mbar_init(bar0 + 8u * d, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();

        const uint32_t nb = (te - tb + kU - 1) / kU;
        const uint32_t rowf = min(uint32_t(FS), a.K - blk.f0);  // floats copied per row
        const uint32_t rowb = rowf * 4u;

        // metadata of batch b: lane L holds a2b[8t + L] (+32), bits / offset of tile `lane`
        uint32_t ma[MA];
        uint64_t mb;
        uint32_t mo;
        auto load_meta = [&](uint32_t b) {
            const uint32_t t = tb + b * kU;
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                const uint32_t e = 32 * j + lane;
                ma[j] = (b < nb && e < 8 * kU && t + e / 8 < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            const uint32_t tl = t + uint32_t(lane);
            const bool ok = b < nb && lane < kU && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };

        auto issue = [&](uint32_t b) {
            if (b >= nb) return;
            const uint32_t s = b % kD;
            float* st = my_ring + size_t(s) * Cf::kStage;
            const uint32_t t = tb + b * kU;
            const uint32_t ntiles = min(uint32_t(kU), te - t);
            const uint32_t bar = bar0 + 8u * s;
            // the stage was last read by this warp's generic loads
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (lane == 0) mbar_expect_tx(bar, ntiles * 8u * rowb);
            __syncwarp();
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                const uint32_t e = 32 * j + lane;  // (tile, row) = (e / 8, e % 8)
                if (e < 8 * kU && e / 8 < ntiles) {
                    const uint32_t idx = ma[j];
                    const float* src = idx < a.cols ? a.B + size_t(idx) * a.K + blk.f0 : g_zero_row;
                    bulk_copy<HINTS>(smem_addr(st + e * FS), src, rowb, bar, pol_keep);
                }
            }
            if (lane < kU) {
                uint32_t* sm = reinterpret_cast<uint32_t*>(st + Cf::kB) + 4 * lane;
                sm[0] = uint32_t(mb);
                sm[1] = uint32_t(mb >> 32);
                sm[2] = mo;
                if (uint32_t(lane) < ntiles) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.vals + mo));
            }
        };

        BitDecode dec;
        dec.init(g, tq);
        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        bool failed = false;
        uint32_t fail_q = 0;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        // prologue: batches 0 .. kD-2 in flight
        for (int d = 0; d < kD - 1; ++d) {
            load_meta(uint32_t(d));
            issue(uint32_t(d));
        }
        load_meta(kD - 1);
        for (uint32_t q = 0; q < nb && !failed; ++q) {
            issue(q + kD - 1);
            load_meta(q + kD);
            const uint32_t s = q % kD;
            const bool landed = mbar_wait(bar0 + 8u * s, (q / kD) & 1u);
            if (!__all_sync(0xffffffffu, landed)) {  // warp-uniform outcome
                failed = true;
                fail_q = q;
                break;
            }
            __syncwarp();
            const float* st = my_ring + size_t(s) * Cf::kStage;
            const uint32_t* sm = reinterpret_cast<const uint32_t*>(st + Cf::kB);
            const uint32_t t = tb + q * kU;
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const uint32_t tt = t + u;
                if (tt >= te) break;
                if (tt >= next_bound) {
                    blk.flush(a, acc, wl, tb, te, first_win);
                    first_win = false;
#pragma unroll
                    for (int mm = 0; mm < NM; ++mm) acc[mm][0] = acc[mm][1] = acc[mm][2] = acc[mm][3] = 0.f;
                    while (blk.s_rwo[wl + 1] <= tt) ++wl;
                    next_bound = blk.s_rwo[wl + 1];
                }
                const uint64_t bm = uint64_t(sm[4 * u]) | (uint64_t(sm[4 * u + 1]) << 32);
                const uint32_t to = sm[4 * u + 2];
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm, x0, x1, q0, q1);
                const float av0 = q0 ? __ldg(a.vals + to + x0) : 0.f;
                const float av1 = q1 ? __ldg(a.vals + to + x1) : 0.f;
                float4 r0[H], r1[H];
                const float* sb = st + u * 8 * FS + 4 * g;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    r0[h] = *reinterpret_cast<const float4*>(sb + tq * FS + 32 * h);
                    r1[h] = *reinterpret_cast<const float4*>(sb + (tq + 4) * FS + 32 * h);
                }
                tile_mma<H, PREC>(acc, r0, r1, av0, av1);
            }
            __syncwarp();
        }
        if (failed) {
            if (lane == 0) atomicOr(&g_bulk_status, 1u);
            // batches fail_q .. fail_q + kD - 1 may still have copies in
            // flight into this warp's ring: let them land (bounded) first
            for (uint32_t b = fail_q; b < nb && b < fail_q + kD; ++b)
                mbar_wait(bar0 + 8u * (b % kD), (b / kD) & 1u);
        } else {
            blk.flush(a, acc, wl, tb, te, first_win);
        }
    }
    __syncthreads();
    blk.finish(a);
}

// A stage of the TMA kernel: the bulk kernel's stage rounded up to 128 bytes.
template <int FS>
struct TmaStage {
    static constexpr int kFloats = (BulkCfg<FS>::kStage + 31) / 32 * 32;
};

template <int FS, int NW>
size_t tma_smem(uint32_t wb) {
    using Cf = BulkCfg<FS>;
    return 128 + (size_t(NW) * Cf::kD * TmaStage<FS>::kFloats + size_t(2 * NW * 8 * FS)) * 4 +
           size_t(NW) * Cf::kD * 8 + size_t(wb + 1) * 4;
}

// Four rows of the tensor-mapped B, columns [x, x + FS), into consecutive
// FS-float rows at dst; completion counted on the mbarrier at bar.
__device__ __forceinline__ void tma_gather4(uint32_t dst, const CUtensorMap* tm, int x, int r0, int r1,
                                            int r2, int r3, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(bar)
        : "memory");
}

template <int FS, int PREC, int NW>
__global__ void __launch_bounds__(NW * 32) spmm_tma_kernel(const __grid_constant__ CUtensorMap tmB,
                                                           const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    using Cf = BulkCfg<FS>;
    constexpr int kU = Cf::kU, kD = Cf::kD;
    constexpr int MA = (8 * kU + 31) / 32;
    static_assert(8 * kU <= 64, "at most two a2b registers per lane");

    extern __shared__ __align__(128) float smem[];
    // stages start on 128-byte boundaries (the base is rounded up at run time;
    // the launch adds 128 bytes of slack)
    float* ring = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem) + 127) & ~uintptr_t(127));
    float* part = ring + size_t(NW) * kD * TmaStage<FS>::kFloats;  // [2 NW][8][FS]
    uint64_t* bars = reinterpret_cast<uint64_t*>(part + 2 * NW * 8 * FS);  // [NW][kD]
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(bars + NW * kD);

    Block<FS, NW> blk;
    blk.init(a, s_rwo, part);
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    if (tb < te) {
        float* my_ring = ring + size_t(blk.warp) * kD * TmaStage<FS>::kFloats;
        const uint32_t bar0 = smem_addr(bars + blk.warp * kD);
        if (lane == 0) {
            for (int d = 0; d < kD; ++d) mbar_init(bar0 + 8u * d, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();

        const uint32_t nb = (te - tb + kU - 1) / kU;
        const uint32_t stage_bytes_per_tile = 8u * FS * 4u;  // full boxes, padding rows included

        uint32_t ma[MA];
        uint64_t mb;
        uint32_t mo;
        auto load_meta = [&](uint32_t b) {
            const uint32_t t = tb + b * kU;
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                const uint32_t e = 32 * j + lane;
                ma[j] = (b < nb && e < 8 * kU && t + e / 8 < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            const uint32_t tl = t + uint32_t(lane);
            const bool ok = b < nb && lane < kU && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };

        // lane 2u + h (h = 0, 1) issues rows 4h .. 4h + 3 of tile u of batch b
        auto issue = [&](uint32_t b) {
            if (b >= nb) return;
            const uint32_t s = b % kD;
            float* st = my_ring + size_t(s) * TmaStage<FS>::kFloats;
            const uint32_t t = tb + b * kU;
            const uint32_t ntiles = min(uint32_t(kU), te - t);
            const uint32_t bar = bar0 + 8u * s;
            // the stage was last read by this warp's generic loads
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            if (lane == 0) mbar_expect_tx(bar, ntiles * stage_bytes_per_tile);
            __syncwarp();
            // lane 2u + h needs entries 8u + 4h + k of the batch (register
            // e / 32 of lane e % 32); every shuffle reads the same register
            // index in all lanes, the reader keeps the one it needs
            const int e0 = (lane & ~1) * 4 + (lane & 1) * 4;  // 8u + 4h
            int rows[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int e = e0 + k;
                uint32_t v = kPad;
#pragma unroll
                for (int j = 0; j < MA; ++j) {
                    const uint32_t vj = __shfl_sync(0xffffffffu, ma[j], e & 31);
                    if (e / 32 == j) v = vj;
                }
                rows[k] = v < a.cols ? int(v) : -1;  // outside the tensor: zero fill
            }
            const uint32_t u = uint32_t(lane) >> 1, h = uint32_t(lane) & 1u;
            if (u < ntiles)
                tma_gather4(smem_addr(st + (u * 8 + 4 * h) * FS), &tmB, int(blk.f0), rows[0], rows[1],
                            rows[2], rows[3], bar);
            if (lane < kU) {
                uint32_t* sm = reinterpret_cast<uint32_t*>(st + Cf::kB) + 4 * lane;
                sm[0] = uint32_t(mb);
                sm[1] = uint32_t(mb >> 32);
                sm[2] = mo;
            }
        };

        BitDecode dec;
        dec.init(g, tq);
        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        bool failed = false;
        uint32_t fail_q = 0;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        for (int d = 0; d < kD - 1; ++d) {
            load_meta(uint32_t(d));
            issue(uint32_t(d));
        }
        load_meta(kD - 1);
        for (uint32_t q = 0; q < nb && !failed; ++q) {
            issue(q + kD - 1);
            load_meta(q + kD);
            const uint32_t s = q % kD;
            const bool landed = mbar_wait(bar0 + 8u * s, (q / kD) & 1u);
            if (!__all_sync(0xffffffffu, landed)) {
                failed = true;
                fail_q = q;
                break;
            }
            __syncwarp();
            const float* st = my_ring + size_t(s) * TmaStage<FS>::kFloats;
            const uint32_t* sm = reinterpret_cast<const uint32_t*>(st + Cf::kB);
            const uint32_t t = tb + q * kU;
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const uint32_t tt = t + u;
                if (tt >= te) break;
                if (tt >= next_bound) {
                    blk.flush(a, acc, wl, tb, te, first_win);
                    first_win = false;
#pragma unroll
                    for (int mm = 0; mm < NM; ++mm) acc[mm][0] = acc[mm][1] = acc[mm][2] = acc[mm][3] = 0.f;
                    while (blk.s_rwo[wl + 1] <= tt) ++wl;
                    next_bound = blk.s_rwo[wl + 1];
                }
                const uint64_t bm = uint64_t(sm[4 * u]) | (uint64_t(sm[4 * u + 1]) << 32);
                const uint32_t to = sm[4 * u + 2];
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm, x0, x1, q0, q1);
                const float av0 = q0 ? __ldg(a.vals + to + x0) : 0.f;
                const float av1 = q1 ? __ldg(a.vals + to + x1) : 0.f;
                float4 r0[H], r1[H];
                const float* sb = st + u * 8 * FS + 4 * g;
#pragma unroll
                for (int hh = 0; hh < H; ++hh) {
                    r0[hh] = *reinterpret_cast<const float4*>(sb + tq * FS + 32 * hh);
                    r1[hh] = *reinterpret_cast<const float4*>(sb + (tq + 4) * FS + 32 * hh);
                }
                tile_mma<H, PREC>(acc, r0, r1, av0, av1);
            }
            __syncwarp();
        }
        if (failed) {
            if (lane == 0) atomicOr(&g_bulk_status, 1u);
            for (uint32_t b = fail_q; b < nb && b < fail_q + kD; ++b)
                mbar_wait(bar0 + 8u * (b % kD), (b / kD) & 1u);
        } else {
            blk.flush(a, acc, wl, tb, te, first_win);
        }
    }
    __syncthreads();
    blk.finish(a);
}

template <int FS, int NW>
size_t bulk_smem(uint32_t wb) {
    using Cf = BulkCfg<FS>;
    return (size_t(NW) * Cf::kD * Cf::kStage + size_t(2 * NW * 8 * FS)) * 4 + size_t(NW) * Cf::kD * 8 +
           size_t(wb + 1) * 4;
}

template <int FS, int PREC, int NW, bool HINTS>
int launch_one(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = bulk_smem<FS, NW>(a.wb);
    if (smem > 227 * 1024) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "shared memory %zu too large", smem);
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_bulk_kernel<FS, PREC, NW, HINTS>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_bulk_kernel<FS, PREC, NW, HINTS><<<unsigned(grid), NW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

template <int FS, int PREC>
int launch_nw(const SpmmArgs& a, int nw, int hints, cudaStream_t s) {
    if (nw == 4) return hints ? launch_one<FS, PREC, 4, true>(a, s) : launch_one<FS, PREC, 4, false>(a, s);
    return hints ? launch_one<FS, PREC, 2, true>(a, s) : launch_one<FS, PREC, 2, false>(a, s);
}

template <int PREC>
int launch_prec(const SpmmArgs& a, int fs, int nw, int hints, cudaStream_t s) {
    switch (fs) {
        case 32: return launch_nw<32, PREC>(a, nw, hints, s);
        case 64: return launch_nw<64, PREC>(a, nw, hints, s);
        default: return launch_nw<128, PREC>(a, nw, hints, s);
    }
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (the library links the runtime statically and not libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiledFn* out) {
    static std::mutex mu;
    static EncodeTiledFn fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                         cudaEnableDefault, &q);
        if (e != cudaSuccess || !p || q != cudaDriverEntryPointSuccess)
            ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    *out = fn;
    return ACCSPMM_SUCCESS;
}

template <int FS, int PREC, int NW>
int launch_tma_one(const SpmmArgs& a, cudaStream_t s) {
    EncodeTiledFn enc = nullptr;
    int r = encode_fn(&enc);
    if (r) return r;
    // B: K x cols floats, row stride K * 4 bytes (a multiple of 16 since K % 4
    // == 0), base 16-byte aligned (checked by the entry points); box FS x 1
    // (FS * 4 bytes, a multiple of 16); x coordinates are slice starts, FS-
    // float multiples, so every copy starts on a 16-byte boundary
    CUtensorMap tm;
    const cuuint64_t dims[2] = {a.K, a.cols};
    const cuuint64_t strides[1] = {cuuint64_t(a.K) * 4};
    const cuuint32_t box[2] = {FS, 1};
    const cuuint32_t es[2] = {1, 1};
    const CUresult cr = enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(a.B), dims, strides, box,
                            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (cr != CUDA_SUCCESS) ACC_FAIL(ACCSPMM_ERROR_CUDA, "cuTensorMapEncodeTiled failed (%d)", int(cr));
    const size_t smem = tma_smem<FS, NW>(a.wb);
    if (smem > 227 * 1024) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "shared memory %zu too large", smem);
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_tma_kernel<FS, PREC, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      227 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_tma_kernel<FS, PREC, NW><<<unsigned(grid), NW * 32, smem, s>>>(tm, a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

template <int PREC>
int launch_tma_prec(const SpmmArgs& a, int fs, int nw, cudaStream_t s) {
    switch (fs) {
        case 32: return nw == 4 ? launch_tma_one<32, PREC, 4>(a, s) : launch_tma_one<32, PREC, 2>(a, s);
        case 64: return nw == 4 ? launch_tma_one<64, PREC, 4>(a, s) : launch_tma_one<64, PREC, 2>(a, s);
        default: return nw == 4 ? launch_tma_one<128, PREC, 4>(a, s) : launch_tma_one<128, PREC, 2>(a, s);
    }
}

}  // namespace

int launch_tma(const SpmmArgs& a, int fs, int precision, int nw, cudaStream_t s) {
    if (a.K % 4) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K must be a multiple of 4");
    if (reinterpret_cast<uintptr_t>(a.B) & 15u) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "B must be 16-byte aligned");
    return precision == ACCSPMM_PREC_3XTF32 ? launch_tma_prec<ACCSPMM_PREC_3XTF32>(a, fs, nw, s)
                                            : launch_tma_prec<ACCSPMM_PREC_TF32>(a, fs, nw, s);
}

int launch_bulk(const SpmmArgs& a, int fs, int precision, int nw, int hints, cudaStream_t s) {
    if (a.K % 4) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K must be a multiple of 4");
    return precision == ACCSPMM_PREC_3XTF32 ? launch_prec<ACCSPMM_PREC_3XTF32>(a, fs, nw, hints, s)
                                            : launch_prec<ACCSPMM_PREC_TF32>(a, fs, nw, hints, s);
}

int bulk_status_take(unsigned int* v) {
    ACC_CUDA(cudaMemcpyFromSymbol(v, g_bulk_status, sizeof *v));
    if (*v) {
        const unsigned int z = 0;
        ACC_CUDA(cudaMemcpyToSymbol(g_bulk_status, &z, sizeof z));
    }
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
