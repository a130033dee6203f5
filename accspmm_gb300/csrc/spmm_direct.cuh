// spmm_direct.cuh -- the register-direct SpMM of one work item, shared by the
// one-matrix kernel (spmm.cu) and the batched kernel (spmm_batch.cu).
#pragma once

#include "spmm_common.cuh"

namespace accspmm {

constexpr int kDirectNW = 8;  // warps per CTA

__device__ __forceinline__ uint64_t shfl_u64(uint64_t v, int src) {
    uint32_t lo = __shfl_sync(0xffffffffu, uint32_t(v), src);
    uint32_t hi = __shfl_sync(0xffffffffu, uint32_t(v >> 32), src);
    return (uint64_t(hi) << 32) | lo;
}

// Register-direct SpMM of one work item (window block, feature slice) by one
// CTA: each lane loads its B fragments straight from global memory, a batch
// of U tiles at a time.  `blk` must be initialised for the item.
// Default batch: 64 floats of B fragments per lane in flight.
template <int FS>
struct DirectBatch {
    static constexpr int U = FS >= 128 ? 2 : (FS == 64 ? 4 : 8);
};

// ROLL: a register ring of U tile slots, each reloaded with the tile U ahead
// as soon as its MMAs have consumed it, instead of a whole batch of loads
// followed by a whole batch of MMAs.
template <int FS, int PREC, int U = DirectBatch<FS>::U, bool EPI = false, int NW = kDirectNW,
          bool ROLL = false>
__device__ __forceinline__ void direct_item(const SpmmArgs& a, const Block<FS, NW>& blk) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    constexpr int MA = (8 * U + 31) / 32;             // a2b registers per lane

    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    bool fok[H];
#pragma unroll
    for (int h = 0; h < H; ++h) fok[h] = blk.f0 + 32 * h + 4 * g < a.K;

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
                uint32_t tile = t + e / 8;
                ma[j] = (e < 8 * U && tile < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            uint32_t tl = t + uint32_t(lane);
            bool ok = lane < U && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };
        load_meta(tb);

        BitDecode dec;
        dec.init(g, tq);
        const float* Bl = a.B + blk.f0 + 4 * g;
        if constexpr (ROLL) {
            float av0[U], av1[U];
            float4 r0[U][H], r1[U][H];
            // loads tile (batch of ma/mb/mo) + u into slot u; tiles past te
            // carry padding metadata and load nothing
            auto issue = [&](int u) {
                const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
                const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
                const uint64_t bm = shfl_u64(mb, u);
                const uint32_t to = __shfl_sync(0xffffffffu, mo, u);
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm, x0, x1, q0, q1);
                av0[u] = q0 ? ldg_f32_ordered(a.vals + to + x0) : 0.f;
                av1[u] = q1 ? ldg_f32_ordered(a.vals + to + x1) : 0.f;
                const bool v0 = i0 < a.cols, v1 = i1 < a.cols;
                const float* p0 = Bl + size_t(v0 ? i0 : 0) * a.K;
                const float* p1 = Bl + size_t(v1 ? i1 : 0) * a.K;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    r0[u][h] = (v0 && fok[h]) ? ldg_f4_ordered(p0 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                    r1[u][h] = (v1 && fok[h]) ? ldg_f4_ordered(p1 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            };
#pragma unroll
            for (int u = 0; u < U; ++u) issue(u);
            load_meta(tb + U);  // padding when past te
            for (uint32_t t = tb; t < te; t += U) {
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const uint32_t tt = t + u;
                    if (tt < te) {
                        if (tt >= next_bound) {
                            blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
                            first_win = false;
#pragma unroll
                            for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                            while (blk.s_rwo[wl + 1] <= tt) ++wl;
                            next_bound = blk.s_rwo[wl + 1];
                        }
                        tile_mma<H, PREC>(acc, r0[u], r1[u], av0[u], av1[u]);
                    }
                    issue(u);  // tile t + U + u
                }
                load_meta(t + 2 * U);
            }
            blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
        } else {
        for (uint32_t t = tb; t < te; t += U) {
            float av0[U], av1[U];
            float4 r0[U][H], r1[U][H];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
                const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
                const uint64_t bm = shfl_u64(mb, u);
                const uint32_t to = __shfl_sync(0xffffffffu, mo, u);
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm, x0, x1, q0, q1);
                av0[u] = q0 ? ldg_f32_ordered(a.vals + to + x0) : 0.f;
                av1[u] = q1 ? ldg_f32_ordered(a.vals + to + x1) : 0.f;
                const bool v0 = i0 < a.cols, v1 = i1 < a.cols;
                const float* p0 = Bl + size_t(v0 ? i0 : 0) * a.K;
                const float* p1 = Bl + size_t(v1 ? i1 : 0) * a.K;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    r0[u][h] = (v0 && fok[h]) ? ldg_f4_ordered(p0 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                    r1[u][h] = (v1 && fok[h]) ? ldg_f4_ordered(p1 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            if (t + U < te) load_meta(t + U);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t tt = t + u;
                if (tt >= te) break;
                if (tt >= next_bound) {
                    blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
                    first_win = false;
#pragma unroll
                    for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                    while (blk.s_rwo[wl + 1] <= tt) ++wl;
                    next_bound = blk.s_rwo[wl + 1];
                }
                tile_mma<H, PREC>(acc, r0[u], r1[u], av0[u], av1[u]);
            }
        }
        blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
        }
    }
    __syncthreads();
    blk.template finish<EPI>(a);
}


// direct_item with the rolling tile ring for TF32 with B packed (a.bp, rows
// of a.bpitch bytes: 2.5 bytes a value instead of four, so 10 of every 16
// sectors of a gathered row).  Same pieces, same MMAs on the same operand bits, same
// order: bit-identical to direct_item<FS, TF32, U, false, NW, true>.
// PF: the B rows of the tile group two ahead of the one being loaded are
// prefetched into L2 (one bulk prefetch of the row's 320-byte slice per
// sparseA2B entry), so that the ring's loads of them find L2 instead of DRAM;
// a hint only, it changes no value.
// The packed buffer holds a zero row at index cols and every row is
// a.bpitch bytes long, so a padding entry (or any index >= cols) reads the zero
// row and no load is predicated (columns past K read the row's padding bytes,
// whose products land only in columns that are not stored): 8 % fewer
// instructions and 5 % less time than predicated loads on the 1M-row
// power-law matrix at K = 128 and 256.
// One float4 of B (columns c .. c + 3 of a row, c % 4 == 0) rounded to TF32
// and stored into the row's packed form at `row`, the layout
// direct_item_packed reads.  A row is cut into FS-column slices of
// FS * 5 / 2 bytes (320 at FS = 128, 160 at FS = 64, 80 at FS = 32): the
// halfwords of bits 31..16 of the slice's values (2 FS bytes), ordered so
// that each lane's values come in runs of 16 bytes (8 at FS = 32), then the
// nibbles of bits 15..12 (FS / 2 bytes, FS / 16 per lane).
template <int FS = 128>
__device__ __forceinline__ void pack_tf32_put(uint8_t* row, uint32_t c, float4 v) {
    static_assert(FS == 128 || FS == 64 || FS == 32, "packed slices are 128, 64 or 32 columns");
    constexpr uint32_t H = FS / 32;
    const uint32_t r0 = f2tf32(v.x), r1 = f2tf32(v.y), r2 = f2tf32(v.z), r3 = f2tf32(v.w);
    // slice c / FS of the row: column group g = (c / 4) % 8, h = (c / 32) % H
    uint8_t* base = row + (FS * 5 / 2) * (c / FS);
    const uint32_t g = (c >> 2) & 7, h = (c >> 5) & (H - 1);
    // 32-column slices: one group per lane, halfwords in 8-byte runs
    const uint32_t hw_off = FS == 32 ? 8 * g : 128 * (h >> 1) + 16 * g + 8 * (h & 1);
    *reinterpret_cast<uint2*>(base + hw_off) =
        make_uint2((r0 >> 16) | (r1 & 0xFFFF0000u), (r2 >> 16) | (r3 & 0xFFFF0000u));
    *reinterpret_cast<uint16_t*>(base + 2 * FS + 2 * H * g + 2 * h) =
        uint16_t(((r0 >> 8) & 0xF0u) | ((r1 >> 12) & 0x0Fu) | (((r2 >> 8) & 0xF0u) << 8) |
                 (((r3 >> 12) & 0x0Fu) << 8));
}

// PFK: how rows are prefetched -- 1 one cp.async.bulk.prefetch.L2 of the
// 320-byte slice per row (its address operand is uniform, so the lanes'
// prefetches issue one after another), 2 three prefetch.global.L2 of the
// slice's 128-byte lines per row, issued by the lanes together.
template <int FS, int U, int NW = kDirectNW, bool PF = false, int PFK = 2, bool EPI = false>
__device__ __forceinline__ void direct_item_packed(const SpmmArgs& a, const Block<FS, NW>& blk) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    // a2b registers per lane: the group's 8U entries, and with PF the 8U of
    // the group after (lanes 8U .. 16U - 1, or a register of their own at U = 4)
    constexpr int MA = ((PF ? 16 : 8) * U + 31) / 32;

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
                uint32_t tile = t + e / 8;
                // PF: entries 8U .. 16U - 1 are those of the group after
                ma[j] = (e < (PF ? 16 * U : 8 * U) && tile < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            uint32_t tl = t + uint32_t(lane);
            bool ok = lane < U && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };
        load_meta(tb);

        BitDecode dec;
        dec.init(g, tq);
        // a row's slice f0 / FS is SB = 5 FS / 2 bytes at SB (f0 / FS): this
        // lane's halfwords of column groups h = 2hp, 2hp + 1 at 128 hp + 16 g,
        // its FS / 16 nibble bytes at 2 FS + (FS / 16) g
        constexpr int SB = FS * 5 / 2;
        constexpr int HW_LANE = FS == 32 ? 8 : 16;  // bytes between lanes' halfword runs
        const uint8_t* Pl = a.bp + SB * (blk.f0 / FS) + HW_LANE * g;
        const int nb_off = 2 * FS + (FS / 16) * g - HW_LANE * g;
        float av0[U], av1[U];
        // nibble bytes per row: 8 at 128-column slices, 4 at 64, 2 at 32
        using Nib = std::conditional_t<H == 4, uint2, uint32_t>;
        uint2 h0[U][H], h1[U][H];
        Nib n0[U], n1[U];
        auto issue = [&](int u) {
            const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
            const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
            const uint64_t bm = shfl_u64(mb, u);
            const uint32_t to = __shfl_sync(0xffffffffu, mo, u);
            uint32_t x0, x1;
            bool q0, q1;
            dec.decode(bm, x0, x1, q0, q1);
            av0[u] = q0 ? ldg_f32_ordered(a.vals + to + x0) : 0.f;
            av1[u] = q1 ? ldg_f32_ordered(a.vals + to + x1) : 0.f;
            const uint8_t* w0 = Pl + size_t(min(i0, a.cols)) * a.bpitch;
            const uint8_t* w1 = Pl + size_t(min(i1, a.cols)) * a.bpitch;
#pragma unroll
            for (int hp = 0; hp < H / 2; ++hp) {
                // halfwords of values 32h + 4g + 0..3, h = 2hp and 2hp + 1, at w + 128 hp
                const uint4 p0 = ldg_u4_ordered(w0 + 128 * hp);
                const uint4 p1 = ldg_u4_ordered(w1 + 128 * hp);
                h0[u][2 * hp] = make_uint2(p0.x, p0.y);
                h1[u][2 * hp] = make_uint2(p1.x, p1.y);
                h0[u][2 * hp + 1] = make_uint2(p0.z, p0.w);
                h1[u][2 * hp + 1] = make_uint2(p1.z, p1.w);
            }
            if constexpr (H == 1) {
                // the 4 values' halfwords, 8 bytes
                h0[u][0] = ldg_u2_ordered(w0);
                h1[u][0] = ldg_u2_ordered(w1);
            }
            // nibbles of all 4H values in one load
            if constexpr (H == 4) {
                n0[u] = ldg_u2_ordered(w0 + nb_off);
                n1[u] = ldg_u2_ordered(w1 + nb_off);
            } else if constexpr (H == 1) {
                n0[u] = ldg_u16_ordered(w0 + nb_off);
                n1[u] = ldg_u16_ordered(w1 + nb_off);
            } else {
                n0[u] = ldg_u32_ordered(w0 + nb_off);
                n1[u] = ldg_u32_ordered(w1 + nb_off);
            }
        };
        // PF: entry e of the group after the one that load_meta fetched for
        // issue (two groups ahead of the loads) sits in lane 8U + e of ma[0]
        // when 16U <= 32, else in lane e of ma[1]; each such lane prefetches
        // that row's slice
        static_assert(!PF || 16 * U == 32 || 8 * U == 32, "one prefetched row per lane");
        constexpr int kPfReg = 8 * U >= 32 ? 1 : 0;
        auto prefetch_rows = [&]() {
            const uint32_t e = ma[PF ? kPfReg : 0];
            if (PF && (kPfReg == 1 || lane >= 8 * U) && e < a.cols) {
                const uint8_t* r = a.bp + size_t(e) * a.bpitch + SB * (blk.f0 / FS);
                if (PFK == 1) {
                    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(r), "n"(SB) : "memory");
                } else if constexpr (FS == 32) {
                    // an 80-byte slice starts on a 16-byte boundary: the
                    // lines of its first and last bytes
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(r));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(r + SB - 1));
                } else {
                    // the 128-byte lines that hold the slice: three for a
                    // 320-byte slice (rows start on 64-byte boundaries), two
                    // for a 160-byte one (32-byte boundaries)
#pragma unroll
                    for (int off = 0; off < SB; off += 128)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(r + off));
                }
            }
        };
#pragma unroll
        for (int u = 0; u < U; ++u) issue(u);
        load_meta(tb + U);  // padding when past te
        for (uint32_t t = tb; t < te; t += U) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t tt = t + u;
                if (tt < te) {
                    if (tt >= next_bound) {
                        blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
                        first_win = false;
#pragma unroll
                        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                        while (blk.s_rwo[wl + 1] <= tt) ++wl;
                        next_bound = blk.s_rwo[wl + 1];
                    }
                    if constexpr (H == 4)
                        tile_mma_packed<H>(acc, h0[u], n0[u], h1[u], n1[u], av0[u], av1[u]);
                    else
                        tile_mma_packed<H>(acc, h0[u], make_uint2(n0[u], 0u), h1[u], make_uint2(n1[u], 0u),
                                           av0[u], av1[u]);
                }
                issue(u);  // tile t + U + u
                if (u == 0) prefetch_rows();  // tiles t + 2U .. t + 3U - 1
            }
            load_meta(t + 2 * U);
        }
        blk.template flush<EPI>(a, acc, wl, tb, te, first_win);
    }
    __syncthreads();
    blk.template finish<EPI>(a);
}

}  // namespace accspmm
