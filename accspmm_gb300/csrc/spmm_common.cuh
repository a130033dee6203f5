// spmm_common.cuh -- pieces shared by the SpMM kernels: arguments, the MMA
// of one tile, the accumulator layout, and the CTA framework that cuts a block
// of row windows into equal per-warp tile pieces and sums the windows cut by
// piece boundaries in a fixed order.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.hpp"

namespace accspmm {

struct SpmmArgs {
    const uint32_t* rwo;
    const uint32_t* tc_offset;
    const uint64_t* bits;
    const uint32_t* a2b;
    const float* vals;
    const float* B;
    float* C;
    uint32_t W;            // windows covered (C has 8W rows)
    uint32_t cols;         // rows of B
    uint32_t K;            // columns of B and C
    uint32_t wb;           // windows per CTA
    uint32_t n_slices;     // feature slices of FS columns in this launch
    uint32_t n_wblocks;    // window blocks
    uint32_t slice_major;  // CTA order: every window block of slice 0 first
    uint32_t slice0;       // first feature slice of this launch
    const float* bias;     // epilogue: C = act(A B + bias[col]); nullptr: no bias
    uint32_t act;          // epilogue activation: 0 none, 1 ReLU
    // CTA i runs window block order[i] (nullptr: block i).  Only the
    // schedule changes: a block's arithmetic does not depend on its CTA.
    // (No default member initializer: the batched kernel keeps a SpmmArgs in
    // shared memory; brace initialisation without it leaves it null.)
    const uint32_t* order;
    // B rounded to TF32 and packed to 2.5 bytes a value (pack_tf32_put): row
    // i at bp + i * bpitch bytes, 320 bytes per 128-column slice (halfwords of
    // bits 31..16, then nibbles of bits 15..12), and a zero row at index cols
    // that padding entries read.  nullptr: the kernels read B.
    const uint8_t* bp;
    uint32_t bpitch;
};

// TF32 operand rounded to nearest, ties away from zero: the reference's
// cvt.rna.tf32.f32 (include/ptx_tf32.hpp:19-24).  (Adding half a TF32 ulp to
// the bit pattern and letting the MMA drop the low 13 bits gives the same
// values for finite inputs, but measured twice as slow on GB300 in this
// kernel: the cvt keeps the gathers of a batch in flight together.)
__device__ __forceinline__ uint32_t f2tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// The same rounding as a float (13 low bits zero): the high part of a 3xTF32
// split.
__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(f2tf32(x)); }

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Loads issued as volatile asm keep their program order relative to the
// (volatile) MMAs, so a whole batch of gathers is in flight before the first
// MMA of the batch waits on it.
__device__ __forceinline__ float4 ldg_f4_ordered(const float* p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ float ldg_f32_ordered(const float* p) {
    float v;
    asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ float comp(const float4& v, int j) {
    return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
}

// Packed TF32 B at 128- or 64-column slices (pack_tf32_put).  For one
// gathered row a lane of column group g holds hw[h] = bits 31..16 of values
// 32h + 4g + 0..3 (two to a word, h < FS / 32) and nb = FS / 16 nibble
// bytes: byte 2h + (j >> 1) holds bits 15..12 of value 32h + 4g + j, even j
// in the high nibble.  Word hp of nb covers h = 2hp and 2hp + 1.
__device__ __forceinline__ uint4 ldg_u4_ordered(const uint8_t* p) {
    uint4 v;
    asm volatile("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

__device__ __forceinline__ uint2 ldg_u2_ordered(const uint8_t* p) {
    uint2 v;
    asm volatile("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t ldg_u16_ordered(const uint8_t* p) {
    unsigned short v;
    asm volatile("ld.global.nc.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t ldg_u32_ordered(const uint8_t* p) {
    uint32_t v;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// The 32-bit TF32 operand of value j of column group h (HB = h & 1): one
// byte permute puts its halfword in bits 31..16 and the nibble byte that
// holds its bits 15..12 in bits 15..8, its nibble on top (for odd j from the
// nibble word shifted up by four bits).  Bits 11..0 take whatever comes along,
// and the tensor core reads only bits 31..13, which equal the value's cvt.rna
// rounding (the packing stored them).
template <int J, int HB>
__device__ __forceinline__ uint32_t unpack_tf32(uint2 hw, uint32_t nbw, uint32_t nbw_shl4) {
    constexpr uint32_t lo_b = 4 + 2 * HB + (J >> 1);  // byte of the second source
    constexpr uint32_t hi_b0 = 2 * (J & 1), hi_b1 = hi_b0 + 1;
    constexpr uint32_t sel = 0u | (lo_b << 4) | (hi_b0 << 8) | (hi_b1 << 12);
    const uint32_t w = J < 2 ? hw.x : hw.y;
    const uint32_t nb = (J & 1) ? nbw_shl4 : nbw;
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(w), "r"(nb), "n"(sel));
    return r;
}

// Accumulators of one warp: 8 window rows x FS features.  H = FS / 32 float4
// per B row per lane, NM MMAs per tile.  acc[m][0..3] follow the m16n8 D
// fragment: [0] (g, 2tq), [1] (g, 2tq+1), [2] (g+8, 2tq), [3] (g+8, 2tq+1).
// For H >= 2, MMA m = 4 hp + j has row g = feature 32 (2hp) + 4g + j and
// row g+8 = feature 32 (2hp+1) + 4g + j; for H == 1, MMA j (0, 1) has row g =
// feature 4g + j and row g+8 = feature 4g + j + 2.
template <int H>
struct Layout {
    static constexpr int NM = H >= 2 ? 2 * H : 2;
    // float4 of output row n = 2tq + p, feature group h (features 32h + 4g + 0..3)
    __device__ static __forceinline__ float4 get(const float (&acc)[NM][4], int p, int h) {
        if constexpr (H >= 2) {
            const int hp = h >> 1, q = h & 1;
            return make_float4(acc[hp * 4 + 0][p + 2 * q], acc[hp * 4 + 1][p + 2 * q],
                               acc[hp * 4 + 2][p + 2 * q], acc[hp * 4 + 3][p + 2 * q]);
        } else {
            return make_float4(acc[0][p], acc[1][p], acc[0][p + 2], acc[1][p + 2]);
        }
    }
};

// The MMAs of one tile.  r0 / r1: this lane's float4s of B rows a2b[tq] and
// a2b[tq + 4]; av0 / av1: sparse values (row g, col tq) and (row g, col tq + 4).
template <int H, int PREC>
__device__ __forceinline__ void tile_mma(float (&acc)[Layout<H>::NM][4], const float4 (&r0)[H],
                                         const float4 (&r1)[H], float av0, float av1) {
    constexpr int NM = Layout<H>::NM;
    if constexpr (PREC == ACCSPMM_PREC_TF32) {
        const uint32_t b0 = f2tf32(av0), b1 = f2tf32(av1);
#pragma unroll
        for (int m = 0; m < NM; ++m) {
            float x0, x1, x2, x3;
            if constexpr (H >= 2) {
                const int hp = m >> 2, j = m & 3;
                x0 = comp(r0[2 * hp], j); x1 = comp(r0[2 * hp + 1], j);
                x2 = comp(r1[2 * hp], j); x3 = comp(r1[2 * hp + 1], j);
            } else {
                x0 = comp(r0[0], m); x1 = comp(r0[0], m + 2);
                x2 = comp(r1[0], m); x3 = comp(r1[0], m + 2);
            }
            mma_tf32(acc[m], f2tf32(x0), f2tf32(x1), f2tf32(x2), f2tf32(x3), b0, b1);
        }
    } else {
        // 3xTF32 (Ootomo & Yokota 2022): x = hi + lo with hi, lo TF32;
        // d = B_lo*A_hi + B_hi*A_lo + B_hi*A_hi per tile (small terms first),
        // then added to the FP32 accumulators outside the tensor core.
        const float ah0 = tf32_hi(av0), ah1 = tf32_hi(av1);
        const uint32_t bh0 = __float_as_uint(ah0), bh1 = __float_as_uint(ah1);
        const uint32_t bl0 = f2tf32(av0 - ah0), bl1 = f2tf32(av1 - ah1);
#pragma unroll
        for (int m = 0; m < NM; ++m) {
            float x[4];
            if constexpr (H >= 2) {
                const int hp = m >> 2, j = m & 3;
                x[0] = comp(r0[2 * hp], j); x[1] = comp(r0[2 * hp + 1], j);
                x[2] = comp(r1[2 * hp], j); x[3] = comp(r1[2 * hp + 1], j);
            } else {
                x[0] = comp(r0[0], m); x[1] = comp(r0[0], m + 2);
                x[2] = comp(r1[0], m); x[3] = comp(r1[0], m + 2);
            }
            uint32_t hi[4], lo[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float h = tf32_hi(x[q]);
                hi[q] = __float_as_uint(h);
                lo[q] = f2tf32(x[q] - h);
            }
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            mma_tf32(d, lo[0], lo[1], lo[2], lo[3], bh0, bh1);
            mma_tf32(d, hi[0], hi[1], hi[2], hi[3], bl0, bl1);
            mma_tf32(d, hi[0], hi[1], hi[2], hi[3], bh0, bh1);
            acc[m][0] += d[0]; acc[m][1] += d[1]; acc[m][2] += d[2]; acc[m][3] += d[3];
        }
    }
}

// tile_mma for TF32 with B already rounded and packed: the same MMAs on the
// same operand bits (element j of float4 h of a row is value j of column
// group h of the packed row).
template <int H>
__device__ __forceinline__ void tile_mma_packed(float (&acc)[Layout<H>::NM][4], const uint2 (&h0)[H], uint2 n0,
                                                const uint2 (&h1)[H], uint2 n1, float av0, float av1) {
    static_assert(H == 4 || H == 2 || H == 1, "packed B is gathered at 128-, 64- or 32-column slices");
    constexpr int NM = Layout<H>::NM;
    const uint32_t b0 = f2tf32(av0), b1 = f2tf32(av1);
    const uint32_t n0s[2] = {n0.x << 4, n0.y << 4}, n1s[2] = {n1.x << 4, n1.y << 4};
    const uint32_t n0w[2] = {n0.x, n0.y}, n1w[2] = {n1.x, n1.y};
    if constexpr (H == 1) {
        // Layout<1>: MMA m takes values m and m + 2 of the lane's group
        mma_tf32(acc[0], unpack_tf32<0, 0>(h0[0], n0w[0], n0s[0]), unpack_tf32<2, 0>(h0[0], n0w[0], n0s[0]),
                 unpack_tf32<0, 0>(h1[0], n1w[0], n1s[0]), unpack_tf32<2, 0>(h1[0], n1w[0], n1s[0]), b0, b1);
        mma_tf32(acc[1], unpack_tf32<1, 0>(h0[0], n0w[0], n0s[0]), unpack_tf32<3, 0>(h0[0], n0w[0], n0s[0]),
                 unpack_tf32<1, 0>(h1[0], n1w[0], n1s[0]), unpack_tf32<3, 0>(h1[0], n1w[0], n1s[0]), b0, b1);
    } else {
#pragma unroll
    for (int m = 0; m < NM; ++m) {
        const int hp = m >> 2, j = m & 3;
        uint32_t x0, x1, x2, x3;
#define ACC_PK(J)                                                                                \
    if (j == J) {                                                                                \
        x0 = unpack_tf32<J, 0>(h0[2 * hp], n0w[hp], n0s[hp]);                                    \
        x1 = unpack_tf32<J, 1>(h0[2 * hp + 1], n0w[hp], n0s[hp]);                                \
        x2 = unpack_tf32<J, 0>(h1[2 * hp], n1w[hp], n1s[hp]);                                    \
        x3 = unpack_tf32<J, 1>(h1[2 * hp + 1], n1w[hp], n1s[hp]);                                \
    }
        ACC_PK(0) ACC_PK(1) ACC_PK(2) ACC_PK(3)
#undef ACC_PK
        mma_tf32(acc[m], x0, x1, x2, x3, b0, b1);
    }
    }
}

// Per-lane decode of the two sparse values a lane feeds to the MMA, tile
// elements (row g, col tq) and (row g, col tq + 4): bits 8g + tq and
// 8g + tq + 4 of the bitmap, which lie in the same 32-bit word.  A value's
// index in the tile's data is the number of set bits at or below its bit,
// minus one (include/mma_tf32.cuh:71-79).
struct BitDecode {
    uint32_t pm0, pm1, mlo, mhi, between;
    bool hiw;
    __device__ __forceinline__ void init(int g, int tq) {
        const uint32_t bit0 = uint32_t(g) * 8 + uint32_t(tq);
        hiw = g >= 4;
        const uint32_t sh0 = bit0 & 31;  // at most 27
        pm0 = 1u << sh0;
        pm1 = 1u << (sh0 + 4);
        mlo = hiw ? 0xffffffffu : (2u << sh0) - 1u;
        mhi = hiw ? (2u << sh0) - 1u : 0u;
        between = (pm1 | (pm1 - 1u)) & ~(pm0 | (pm0 - 1u));  // bits (bit0, bit0 + 4]
    }
    // indices (count - 1) and presence of the two elements
    __device__ __forceinline__ void decode(uint64_t bm, uint32_t& i0, uint32_t& i1, bool& p0,
                                           bool& p1) const {
        const uint32_t lo = uint32_t(bm), hi = uint32_t(bm >> 32);
        const uint32_t w = hiw ? hi : lo;
        const uint32_t c0 = __popc(lo & mlo) + __popc(hi & mhi);
        i0 = c0 - 1;
        i1 = c0 + __popc(w & between) - 1;
        p0 = (w & pm0) != 0;
        p1 = (w & pm1) != 0;
    }
};

template <int FS>
__device__ __forceinline__ void store_rows(float* __restrict__ C, uint32_t K, uint32_t row0,
                                           uint32_t f0, int g, int tq,
                                           const float4 (&out)[2][FS / 32]) {
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        float* rowp = C + size_t(row0 + 2 * tq + p) * K;
#pragma unroll
        for (int h = 0; h < FS / 32; ++h) {
            uint32_t f = f0 + 32 * h + 4 * g;
            if (f < K) __stcs(reinterpret_cast<float4*>(rowp + f), out[p][h]);
        }
    }
}

// store_rows with the epilogue applied first: + bias[feature], then the
// activation.  Every element of C is stored exactly once, so the epilogue is
// applied once.  A separate function (and a compile-time switch in the
// callers) so that kernels without an epilogue keep their code unchanged.
template <int FS>
__device__ __forceinline__ void store_rows_epilogue(const SpmmArgs& a, uint32_t row0, uint32_t f0,
                                                    int g, int tq, float4 (&out)[2][FS / 32]) {
#pragma unroll
    for (int h = 0; h < FS / 32; ++h) {
        const uint32_t f = f0 + 32 * h + 4 * g;
        float4 b = make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.bias && f < a.K) b = *reinterpret_cast<const float4*>(a.bias + f);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            float4& v = out[p][h];
            v.x += b.x; v.y += b.y; v.z += b.z; v.w += b.w;
            if (a.act == ACCSPMM_ACT_RELU) {
                v.x = fmaxf(v.x, 0.f); v.y = fmaxf(v.y, 0.f);
                v.z = fmaxf(v.z, 0.f); v.w = fmaxf(v.w, 0.f);
            }
        }
    }
    store_rows<FS>(a.C, a.K, row0, f0, g, tq, out);
}

// CTA geometry: window block, feature slice, and the warp pieces of the
// block's tile range.  `part` holds 2 NW partial slots of 8 x FS floats,
// s_rwo the block's wb + 1 window offsets.
template <int FS, int NW>
struct Block {
    static constexpr int H = FS / 32;
    uint32_t w0, nwin, f0, t_begin, t_total;
    const uint32_t* s_rwo;
    float* part;
    int lane, warp, g, tq;

    // work item of a CTA of a one-matrix launch
    __device__ __forceinline__ void init(const SpmmArgs& a, uint32_t* s_rwo_mem, float* part_mem) {
        uint32_t wbk, slice;
        if (a.slice_major) {
            slice = blockIdx.x / a.n_wblocks;
            wbk = blockIdx.x - slice * a.n_wblocks;
        } else {
            wbk = blockIdx.x / a.n_slices;
            slice = blockIdx.x - wbk * a.n_slices;
        }
        if (a.order) wbk = __ldg(a.order + wbk);
        init_item(a, wbk, slice, s_rwo_mem, part_mem);
    }

    // explicit work item (window block wbk, feature slice `slice`)
    __device__ __forceinline__ void init_item(const SpmmArgs& a, uint32_t wbk, uint32_t slice,
                                              uint32_t* s_rwo_mem, float* part_mem) {
        w0 = wbk * a.wb;
        const uint32_t w1 = min(w0 + a.wb, a.W);
        nwin = w1 - w0;
        f0 = (a.slice0 + slice) * FS;
        for (uint32_t i = threadIdx.x; i <= nwin; i += blockDim.x) s_rwo_mem[i] = a.rwo[w0 + i];
        __syncthreads();
        s_rwo = s_rwo_mem;
        part = part_mem;
        lane = threadIdx.x & 31;
        warp = threadIdx.x >> 5;
        g = lane >> 2;
        tq = lane & 3;
        t_begin = s_rwo[0];
        t_total = s_rwo[nwin] - t_begin;
    }

    __device__ __forceinline__ uint32_t bound(int i) const {
        return t_begin + uint32_t((uint64_t(t_total) * uint32_t(i)) / NW);
    }

    // local index of the window containing tile t (t inside the block)
    __device__ __forceinline__ uint32_t window_of(uint32_t t) const {
        uint32_t wl = 0;
        for (uint32_t jb = 0; jb < nwin; jb += 32) {
            const uint32_t j = jb + uint32_t(lane);
            const bool in = j < nwin && s_rwo[j] <= t && t < s_rwo[j + 1];
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (bal) wl = jb + uint32_t(__ffs(bal) - 1);
        }
        return wl;
    }

    __device__ __forceinline__ float* slot(int s) const { return part + size_t(s) * 8 * FS; }

    // Store a finished window: straight to C if it lies inside [tb, te),
    // else into this warp's first (is_first) or last partial slot.  EPI:
    // apply the bias / activation epilogue when storing to C.
    template <bool EPI = false>
    __device__ __forceinline__ void flush(const SpmmArgs& a, const float (&acc)[Layout<H>::NM][4],
                                          uint32_t wloc, uint32_t tb, uint32_t te,
                                          bool is_first) const {
        const uint32_t rb = s_rwo[wloc], re = s_rwo[wloc + 1];
        float4 out[2][H];
#pragma unroll
        for (int p = 0; p < 2; ++p)
#pragma unroll
            for (int h = 0; h < H; ++h) out[p][h] = Layout<H>::get(acc, p, h);
        if (rb >= tb && re <= te) {
            if constexpr (EPI) store_rows_epilogue<FS>(a, (w0 + wloc) * kWin, f0, g, tq, out);
            else store_rows<FS>(a.C, a.K, (w0 + wloc) * kWin, f0, g, tq, out);
        } else {
            float* sp = slot(2 * warp + (is_first ? 0 : 1));
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int h = 0; h < H; ++h)
                    *reinterpret_cast<float4*>(sp + (2 * tq + p) * FS + 32 * h + 4 * g) = out[p][h];
        }
    }

    // After a CTA barrier: windows cut by piece boundaries are summed from
    // the slots in warp order, empty windows are written as zeros.
    template <bool EPI = false>
    __device__ __forceinline__ void finish(const SpmmArgs& a) const {
        auto warp_of = [&](uint32_t t) -> int {
            int i = NW - 1;
            while (i > 0 && bound(i) > t) --i;
            return i;
        };
        for (uint32_t wloc = warp; wloc < nwin; wloc += NW) {
            const uint32_t rb = s_rwo[wloc], re = s_rwo[wloc + 1];
            float4 out[2][H];
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int h = 0; h < H; ++h) out[p][h] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (rb != re) {
                const int ia = warp_of(rb), ib = warp_of(re - 1);
                if (ia == ib) continue;  // stored by its warp
                for (int i = ia; i <= ib; ++i) {
                    const uint32_t bi = bound(i);
                    if (bi == bound(i + 1)) continue;  // empty piece
                    const float* sp = slot(2 * i + (rb <= bi ? 0 : 1));
#pragma unroll
                    for (int p = 0; p < 2; ++p)
#pragma unroll
                        for (int h = 0; h < H; ++h) {
                            float4 v = *reinterpret_cast<const float4*>(sp + (2 * tq + p) * FS + 32 * h + 4 * g);
                            out[p][h].x += v.x; out[p][h].y += v.y;
                            out[p][h].z += v.z; out[p][h].w += v.w;
                        }
                }
            }
            if constexpr (EPI) store_rows_epilogue<FS>(a, (w0 + wloc) * kWin, f0, g, tq, out);
            else store_rows<FS>(a.C, a.K, (w0 + wloc) * kWin, f0, g, tq, out);
        }
    }
};

// Launch of the cp.async-pipelined kernel (spmm_pipe.cu).
int launch_pipe(const SpmmArgs& a, int fs, int precision, int nw, int hints, cudaStream_t s);
size_t pipe_smem_bytes(int fs, int nw, uint32_t wb);
// Launch of the bulk-copy (TMA) kernel and its status word (spmm_bulk.cu).
int launch_bulk(const SpmmArgs& a, int fs, int precision, int nw, int hints, cudaStream_t s);
// Reads and clears the bulk kernels' sticky wait status (after a stream sync).
int bulk_status_take(unsigned int* v);
// Launch of the tensor-map gather4 (TMA) kernel (spmm_bulk.cu).
int launch_tma(const SpmmArgs& a, int fs, int precision, int nw, cudaStream_t s);
// Launch of the occupancy-sized register-direct kernel (spmm_lean.cu).
int launch_lean(const SpmmArgs& a, int fs, int precision, int minb, cudaStream_t s);
// Slice-major SpMM over B staged in 32-column TF32 slices (spmm_slice.cu):
// bytes of the staging buffer, and the staging pass + SpMM launch (all of
// a's windows and K columns; S holds staged_bytes(a.cols, a.K) bytes).
size_t staged_bytes(uint32_t cols, uint32_t K);
int spmm_staged_launch(const SpmmArgs& a, const float* B, float* S, uint32_t variant, cudaStream_t s);

}  // namespace accspmm
