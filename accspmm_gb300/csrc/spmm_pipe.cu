// spmm_pipe.cu -- the SpMM kernel with a per-warp cp.async pipeline.
//
// Same decomposition and arithmetic as the register-direct kernel (a CTA per
// window block and feature slice, equal per-warp tile pieces, partial windows
// summed in warp order), but each warp streams its tiles through a private
// ring of D shared-memory stages of U tiles:
//   stage = B rows [U][8][FS] | tile values [U][64] | bitmaps [U]
// The warp issues the 16-byte cp.async copies of batch q + D - 1 (rows of B
// gathered through sparseA2B; padding and rows past K are zero-filled with a
// source size of 0), then waits for batch q and runs its MMAs from shared
// memory.  A warp only ever waits on its own copies (cp.async.wait_group), so
// there is no cross-warp handshake.  Tile metadata (sparseA2B, bitmaps,
// tcOffset) is loaded into registers two batches ahead.  With `HINTS`, B is
// fetched with an L2 evict_last policy and the streamed METCF arrays with
// evict_first, so the gathered rows of B stay in L2 longer.
#include "common.hpp"
#include "device_util.cuh"
#include "spmm_common.cuh"

namespace accspmm {

namespace {

constexpr int kD = 4;  // stages in flight per warp

// tiles per batch: 4, or 2 for 128-column slices so that a stage stays small
template <int FS>
struct Stage {
    static constexpr int kU = FS >= 128 ? 2 : 4;
    static constexpr int kB = kU * 8 * FS;   // floats of B rows
    static constexpr int kV = kU * 64;       // tile values
    static constexpr int kM = kU * 2;        // bitmaps (as float pairs)
    static constexpr int kFloats = kB + kV + kM;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

template <bool HINTS>
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_size,
                                           uint64_t pol) {
    if constexpr (HINTS) {
        asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2, %3;\n" ::"r"(dst),
                     "l"(src), "r"(src_size), "l"(pol));
    } else {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                     "r"(src_size));
    }
}

template <bool HINTS>
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, uint64_t pol) {
    if constexpr (HINTS) {
        asm volatile("cp.async.ca.shared.global.L2::cache_hint [%0], [%1], 4, %2;\n" ::"r"(dst),
                     "l"(src), "l"(pol));
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src));
    }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

template <bool HINTS>
__device__ __forceinline__ uint32_t ld_meta_u32(const uint32_t* p, uint64_t pol) {
    uint32_t v;
    if constexpr (HINTS)
        asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
    else
        v = __ldg(p);
    return v;
}

template <bool HINTS>
__device__ __forceinline__ uint64_t ld_meta_u64(const uint64_t* p, uint64_t pol) {
    unsigned long long v;
    if constexpr (HINTS)
        asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
    else
        v = __ldg(reinterpret_cast<const unsigned long long*>(p));
    return v;
}

// Tile metadata of one batch, distributed over the lanes:
//   ma[j]: sparseA2B entry 32 j + lane of the batch (8 per tile), PAD past te
//   mb:    bitmap of tile `lane` (lanes < U), 0 past te
//   mo:    tcOffset[min(t + lane, te)] (lanes <= U)
template <int MA>
struct Meta {
    uint32_t ma[MA];
    uint64_t mb;
    uint32_t mo;
};

template <int FS, int PREC, int NW, bool HINTS>
__global__ void __launch_bounds__(NW * 32) spmm_pipe_kernel(const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    using S = Stage<FS>;
    constexpr int kU = S::kU;
    constexpr int MA = (8 * kU + 31) / 32;
    constexpr int CH = FS / 4;             // 16-byte chunks per row segment
    constexpr int IPT = (8 * CH) / 32;     // 16-byte copies per lane per tile
    static_assert((8 * CH) % 32 == 0, "FS must be a multiple of 16");

    extern __shared__ __align__(16) float smem[];
    float* ring = smem;                                       // [NW][kD][S::kFloats]
    float* part = ring + size_t(NW) * kD * S::kFloats;        // [2 NW][8][FS]
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(part + 2 * NW * 8 * FS);

    Block<FS, NW> blk;
    blk.init(a, s_rwo, part);
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    uint64_t pol_keep = 0, pol_stream = 0;
    if constexpr (HINTS) {
        asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));
        asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_stream));
    }

    if (tb < te) {
        float* my_ring = ring + size_t(blk.warp) * kD * S::kFloats;
        const uint32_t nb = (te - tb + kU - 1) / kU;

        auto load_meta = [&](uint32_t b, Meta<MA>& m) {
            const uint32_t t = tb + b * kU;
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                const uint32_t e = 32 * j + lane;
                const uint32_t tile = t + e / 8;
                m.ma[j] = (b < nb && e < 8 * kU && tile < te)
                              ? ld_meta_u32<HINTS>(a.a2b + size_t(t) * 8 + e, pol_stream)
                              : kPad;
            }
            const uint32_t tl = t + uint32_t(lane);
            m.mb = (b < nb && lane < kU && tl < te) ? ld_meta_u64<HINTS>(a.bits + tl, pol_stream) : 0ull;
            m.mo = (b < nb && lane <= kU) ? ld_meta_u32<HINTS>(a.tc_offset + min(tl, te), pol_stream) : 0u;
        };

        // copies of batch b into its stage
        auto issue = [&](uint32_t b, const Meta<MA>& m) {
            float* st = my_ring + size_t(b % kD) * S::kFloats;
            if (b < nb) {
                const uint32_t sB = smem_u32(st);
#pragma unroll
                for (int u = 0; u < kU; ++u) {
#pragma unroll
                    for (int i = 0; i < IPT; ++i) {
                        const int c = 32 * i + lane;      // chunk of this tile
                        const int k = c / CH, q = c % CH;  // row, 16-byte chunk
                        const int src_lane = (8 * u + k) & 31;
                        const uint32_t idx = __shfl_sync(0xffffffffu, m.ma[(8 * u + k) / 32], src_lane);
                        const uint32_t f = blk.f0 + 4 * uint32_t(q);
                        const bool ok = idx < a.cols && f < a.K;
                        const float* src = ok ? a.B + size_t(idx) * a.K + f : a.B;
                        cp_async16<HINTS>(sB + uint32_t(((u * 8 + k) * FS + 4 * q) * 4), src,
                                          ok ? 16u : 0u, pol_keep);
                    }
                    const uint32_t o0 = __shfl_sync(0xffffffffu, m.mo, u);
                    const uint32_t o1 = __shfl_sync(0xffffffffu, m.mo, u + 1);
                    const uint32_t cnt = min(o1 - o0, 64u);
                    const uint32_t sV = smem_u32(st + S::kB + u * 64);
                    if (uint32_t(lane) < cnt) cp_async4<HINTS>(sV + 4u * lane, a.vals + o0 + lane, pol_stream);
                    if (uint32_t(lane) + 32 < cnt)
                        cp_async4<HINTS>(sV + 4u * (lane + 32), a.vals + o0 + lane + 32, pol_stream);
                }
                if (lane < kU) reinterpret_cast<uint64_t*>(st + S::kB + S::kV)[lane] = m.mb;
            }
            cp_async_commit();
        };

        BitDecode dec;
        dec.init(g, tq);

        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        Meta<MA> m0, m1;
        load_meta(0, m0);
        load_meta(1, m1);
        // prologue: batches 0 .. kD-2 in flight
#pragma unroll
        for (int d = 0; d < kD - 1; ++d) {
            issue(uint32_t(d), m0);
            m0 = m1;
            load_meta(uint32_t(d) + 2, m1);
        }
        for (uint32_t q = 0; q < nb; ++q) {
            issue(q + kD - 1, m0);
            m0 = m1;
            load_meta(q + kD + 1, m1);
            cp_async_wait<kD - 1>();
            __syncwarp();
            const float* st = my_ring + size_t(q % kD) * S::kFloats;
            const uint64_t* sm = reinterpret_cast<const uint64_t*>(st + S::kB + S::kV);
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
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(sm[u], x0, x1, q0, q1);
                const float* sv = st + S::kB + u * 64;
                const float av0 = q0 ? sv[x0] : 0.f;
                const float av1 = q1 ? sv[x1] : 0.f;
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
        cp_async_wait<0>();
        blk.flush(a, acc, wl, tb, te, first_win);
    }
    __syncthreads();
    blk.finish(a);
}

template <int NW>
size_t smem_bytes_for(int fs, uint32_t wb) {
    size_t stage = fs == 32 ? Stage<32>::kFloats : fs == 64 ? Stage<64>::kFloats : Stage<128>::kFloats;
    return (size_t(NW) * kD * stage + size_t(2 * NW * 8 * fs)) * 4 + size_t(wb + 1) * 4;
}

template <int FS, int PREC, int NW, bool HINTS>
int launch_one(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = smem_bytes_for<NW>(FS, a.wb);
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_pipe_kernel<FS, PREC, NW, HINTS>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set |= 1u << dev;
    }
    if (smem > 227 * 1024) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "shared memory %zu too large", smem);
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_pipe_kernel<FS, PREC, NW, HINTS><<<unsigned(grid), NW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

template <int FS, int PREC>
int launch_nw(const SpmmArgs& a, int nw, int hints, cudaStream_t s) {
    if (nw == 4) return hints ? launch_one<FS, PREC, 4, true>(a, s) : launch_one<FS, PREC, 4, false>(a, s);
    return hints ? launch_one<FS, PREC, 8, true>(a, s) : launch_one<FS, PREC, 8, false>(a, s);
}

template <int PREC>
int launch_prec(const SpmmArgs& a, int fs, int nw, int hints, cudaStream_t s) {
    switch (fs) {
        case 32: return launch_nw<32, PREC>(a, nw, hints, s);
        case 64: return launch_nw<64, PREC>(a, nw, hints, s);
        default: return launch_nw<128, PREC>(a, nw, hints, s);
    }
}

}  // namespace

size_t pipe_smem_bytes(int fs, int nw, uint32_t wb) {
    return nw == 4 ? smem_bytes_for<4>(fs, wb) : smem_bytes_for<8>(fs, wb);
}

int launch_pipe(const SpmmArgs& a, int fs, int precision, int nw, int hints, cudaStream_t s) {
    return precision == ACCSPMM_PREC_3XTF32 ? launch_prec<ACCSPMM_PREC_3XTF32>(a, fs, nw, hints, s)
                                            : launch_prec<ACCSPMM_PREC_TF32>(a, fs, nw, hints, s);
}

}  // namespace accspmm
