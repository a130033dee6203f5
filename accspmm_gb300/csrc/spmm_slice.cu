// spmm_slice.cu -- the slice-major SpMM over B staged in 32-column slices.
//
// A B of a few hundred MB gathered row by row in window order misses the L2
// for every uniformly random neighbour: each gathered row is the whole K-wide
// row, and all of B is live at once.  This path cuts B into 32-column slices,
// each rounded to TF32 once (cvt.rna, the rounding the MMA operands get on
// every other path) and stored contiguously as 128-byte rows with a zero row
// at the end:
//
//   S[s][r][c] = tf32(B[r][32 s + c])  (c < K - 32 s, else 0),  S[s][cols][:] = 0
//
// and runs the work items (window block, slice) slice by slice: CTA i takes
// slice i / n_wblocks, window block i % n_wblocks, so the CTAs in flight
// gather from one 128-byte-row slice at a time (128 MB for a million rows),
// which the L2 can hold while the next slice's rows stay out.  Measured with
// random 128-byte row gathers on GB300: 15.5 TB/s from a 128 MB buffer,
// 17.5 TB/s from 64 MB, 8.3 TB/s from 320 MB.
//
// The per-tile work of a slice is kept small because each tile is visited
// once per slice: a lane loads one float4 of each of its two B rows (the
// m16n8k8 A-operand fragment of 32 features, already TF32: no conversion),
// a padding column (sparseA2B = UINT32_MAX, or any index >= cols) reads the
// zero row instead of being predicated, and the tile's bitmap word and value
// offset for the lane's half of the tile come with one shuffle each.
//
// Each CTA cuts its window block into the same per-warp tile pieces as every
// other SpMM kernel of the library (Block<FS, NW>), walks them in the same
// order, feeds the MMAs the same operand bits and sums windows cut by piece
// boundaries in the same order, so the result is bit-identical to
// accspmm_spmm_tf32's other launch shapes and to the batched kernel.
#include <algorithm>

#include "device_util.cuh"
#include "spmm_common.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

constexpr int kSliceFS = 32;  // columns per staged slice (128-byte rows)
constexpr int kSliceNW = 8;   // warps per CTA (the pieces of Block<FS, 8>)

// B (cols x K, row-major) -> S (slices x (cols + 1) x 32), rounded to TF32.
// One float4 of S per thread and step; B is read row-major (each row once,
// streaming), S written 128 bytes at a time.  The zero rows and the columns
// past K of the last slice are written too, so the SpMM loads them freely.
__global__ void stage_tf32_kernel(const float4* __restrict__ B, float4* __restrict__ S, uint32_t cols,
                                  uint32_t K, uint32_t slices) {
    const uint32_t per_row = slices * (kSliceFS / 4);  // float4 of one row across all slices
    const size_t total = size_t(cols + 1) * per_row;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += size_t(gridDim.x) * blockDim.x) {
        const uint32_t r = uint32_t(i / per_row);
        const uint32_t c4 = uint32_t(i - size_t(r) * per_row);
        const uint32_t c = 4 * c4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (r < cols && c < K) {
            const float4 x = __ldcs(B + (size_t(r) * K + c) / 4);  // K % 4 == 0: the whole float4 lies in the row
            v = make_float4(__uint_as_float(f2tf32(x.x)), __uint_as_float(f2tf32(x.y)),
                            __uint_as_float(f2tf32(x.z)), __uint_as_float(f2tf32(x.w)));
        }
        const uint32_t s = c4 / (kSliceFS / 4), q = c4 % (kSliceFS / 4);
        S[(size_t(s) * (cols + 1) + r) * (kSliceFS / 4) + q] = v;
    }
}

// One work item (window block, slice) of the staged SpMM by one CTA.  U
// tiles per warp in flight as a rolling ring: as soon as a slot's MMAs have
// consumed it, it is reloaded with the tile U ahead.
//
// Metadata of U tiles is fetched per warp with one coalesced load of their
// 8U sparseA2B entries (lane e holds entry e) and, in lanes 0 .. 2U - 1, the
// bitmap word (lane & 1) of tile lane / 2 and that half-tile's first value
// offset (tcOffset, plus the popcount of the low word for the high half).  A
// lane of column group g (tile row g) reads word g / 4 only, so its two
// values are data[base + popc(word & bits <= b) - 1] with b = 8g + tq and
// 8g + tq + 4 taken in that word.
template <int U, bool CO>
__device__ __forceinline__ void staged_item(const SpmmArgs& a, const Block<kSliceFS, kSliceNW>& blk,
                                            const float* __restrict__ S) {
    static_assert(2 * U <= 32 && 8 * U <= 64, "one metadata load per U tiles");
    constexpr int MA = (8 * U + 31) / 32;  // sparseA2B registers per lane
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    if (tb < te) {
        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        float acc[2][4];
#pragma unroll
        for (int m = 0; m < 2; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        uint32_t ma[MA], mw, mo;
        auto load_meta = [&](uint32_t t) {
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                const uint32_t e = 32 * j + lane;
                ma[j] = (e < 8 * U && t + e / 8 < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            const uint32_t tl = t + uint32_t(lane >> 1);
            const bool ok = lane < 2 * U && tl < te;
            const uint2 bm = ok ? __ldg(reinterpret_cast<const uint2*>(a.bits) + tl) : make_uint2(0u, 0u);
            const uint32_t off = ok ? __ldg(a.tc_offset + tl) : 0u;
            mw = (lane & 1) ? bm.y : bm.x;
            mo = off + ((lane & 1) ? uint32_t(__popc(bm.x)) : 0u);
        };
        load_meta(tb);

        // this lane's bits in its word: b = (8g + tq) & 31 and b + 4
        const int hw = g >> 2;
        const uint32_t b0 = (uint32_t(g) * 8 + uint32_t(tq)) & 31u;
        const uint32_t upto0 = (2u << b0) - 1u;                   // bits <= b0 (b0 <= 27)
        const uint32_t between = ((2u << (b0 + 4)) - 1u) & ~upto0;  // bits (b0, b0 + 4]
        const uint32_t pm0 = 1u << b0, pm1 = 1u << (b0 + 4);
        // this lane's 16 bytes of a staged row of the CTA's slice: chunk g of
        // rows tq and tq + 4 (fragment order), or (CO) chunk lane & 7 of
        // rows lane / 8 and 4 + lane / 8, one 128-byte line per 8 lanes, moved
        // into fragment order by shuffles from lane 8 tq + g
        const float* Sl = S + size_t(blk.f0 / kSliceFS) * (size_t(a.cols) + 1) * kSliceFS +
                          4 * (CO ? (lane & 7) : g);
        const int rsel = CO ? (lane >> 3) : tq;
        const int src = 8 * tq + g;

        float4 r0[U], r1[U];
        float av0[U], av1[U];
        auto issue = [&](int u) {
            const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + rsel) & 31);
            const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + rsel + 4) & 31);
            const uint32_t w = __shfl_sync(0xffffffffu, mw, 2 * u + hw);
            const uint32_t ob = __shfl_sync(0xffffffffu, mo, 2 * u + hw);
            const uint32_t c0 = __popc(w & upto0);
            const uint32_t c1 = c0 + __popc(w & between);
            av0[u] = (w & pm0) ? ldg_f32_ordered(a.vals + ob + c0 - 1) : 0.f;
            av1[u] = (w & pm1) ? ldg_f32_ordered(a.vals + ob + c1 - 1) : 0.f;
            r0[u] = ldg_f4_ordered(Sl + size_t(min(i0, a.cols)) * kSliceFS);
            r1[u] = ldg_f4_ordered(Sl + size_t(min(i1, a.cols)) * kSliceFS);
        };
        // the m16n8k8 MMAs of one tile: MMA j has row g = feature 4g + j,
        // row g + 8 = feature 4g + j + 2 (Layout<1>)
        auto compute = [&](int u) {
            const uint32_t bb0 = f2tf32(av0[u]), bb1 = f2tf32(av1[u]);
            float4 x0 = r0[u], x1 = r1[u];
            if constexpr (CO) {
                x0.x = __shfl_sync(0xffffffffu, x0.x, src); x0.y = __shfl_sync(0xffffffffu, x0.y, src);
                x0.z = __shfl_sync(0xffffffffu, x0.z, src); x0.w = __shfl_sync(0xffffffffu, x0.w, src);
                x1.x = __shfl_sync(0xffffffffu, x1.x, src); x1.y = __shfl_sync(0xffffffffu, x1.y, src);
                x1.z = __shfl_sync(0xffffffffu, x1.z, src); x1.w = __shfl_sync(0xffffffffu, x1.w, src);
            }
            mma_tf32(acc[0], __float_as_uint(x0.x), __float_as_uint(x0.z), __float_as_uint(x1.x),
                     __float_as_uint(x1.z), bb0, bb1);
            mma_tf32(acc[1], __float_as_uint(x0.y), __float_as_uint(x0.w), __float_as_uint(x1.y),
                     __float_as_uint(x1.w), bb0, bb1);
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
                        blk.template flush<false>(a, acc, wl, tb, te, first_win);
                        first_win = false;
#pragma unroll
                        for (int m = 0; m < 2; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                        while (blk.s_rwo[wl + 1] <= tt) ++wl;
                        next_bound = blk.s_rwo[wl + 1];
                    }
                    compute(u);
                }
                issue(u);  // tile t + U + u
            }
            load_meta(t + 2 * U);
        }
        blk.template flush<false>(a, acc, wl, tb, te, first_win);
    }
    __syncthreads();
    blk.template finish<false>(a);
}

template <int U, int MINB, bool CO>
__global__ void __launch_bounds__(kSliceNW * 32, MINB) spmm_staged_kernel(const SpmmArgs a,
                                                                          const float* __restrict__ S) {
    extern __shared__ __align__(16) float smem[];
    float* part = smem;  // [2 * NW] slots of 8 x 32 floats
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * kSliceNW * 8 * kSliceFS);
    Block<kSliceFS, kSliceNW> blk;
    blk.init(a, s_rwo, part);
    staged_item<U, CO>(a, blk, S);
}

template <int U, int MINB, bool CO>
int launch_staged_t(const SpmmArgs& a, const float* S, cudaStream_t s) {
    const size_t smem = size_t(2 * kSliceNW * 8 * kSliceFS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_staged_kernel<U, MINB, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_staged_kernel<U, MINB, CO><<<unsigned(grid), kSliceNW * 32, smem, s>>>(a, S);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

}  // namespace

size_t staged_bytes(uint32_t cols, uint32_t K) {
    const uint32_t slices = (K + kSliceFS - 1) / kSliceFS;
    return size_t(slices) * (size_t(cols) + 1) * kSliceFS * 4;
}

int spmm_staged_launch(const SpmmArgs& a_in, const float* B, float* S, uint32_t variant, cudaStream_t s) {
    SpmmArgs a = a_in;
    const uint32_t slices = (a.K + kSliceFS - 1) / kSliceFS;
    a.n_slices = slices;
    a.slice0 = 0;
    a.slice_major = 1;
    a.order = nullptr;
    const size_t n4 = staged_bytes(a.cols, a.K) / 16;
    const unsigned blocks = unsigned(std::min<size_t>((n4 + 255) / 256, size_t(sm_count()) * 16));
    stage_tf32_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(B), reinterpret_cast<float4*>(S),
                                             a.cols, a.K, slices);
    ACC_LAUNCH_CHECK();
    switch (variant) {
        case 1: return launch_staged_t<4, 2, false>(a, S, s);
        case 2: return launch_staged_t<4, 3, true>(a, S, s);
        case 3: return launch_staged_t<4, 2, true>(a, S, s);
        case 4: return launch_staged_t<2, 4, true>(a, S, s);
        case 5: return launch_staged_t<8, 2, true>(a, S, s);
        default: return launch_staged_t<4, 3, false>(a, S, s);
    }
}

}  // namespace accspmm
