// spmm_lean.cu -- the register-direct SpMM kernel sized for occupancy.
//
// Random 256-512 byte row gathers from a B larger than L2 reach their
// bandwidth only with many warps in flight per SM (about 32), so this kernel
// keeps a lane's state small: a batch of U tiles of B fragments, the next
// batch's sparseA2B entries, and 8 x FS accumulators per warp.  A lane loads
// its own metadata (no shuffles); padding entries of sparseA2B read a static
// zero row instead of being predicated, and in a partial last feature slice
// the lanes past K read a clamped in-row offset whose outputs are never
// stored, so the gather loop has no per-load predicates.  Decomposition,
// arithmetic and the partial-window order are those of the other SpMM
// kernels (spmm_common.cuh), so all variants give identical results.
#include "common.hpp"
#include "device_util.cuh"
#include "spmm_common.cuh"

namespace accspmm {

// Zero source for the padding rows of a tile (FS <= 128 floats).
static __device__ __align__(16) float g_lean_zero[128] = {0.f};

namespace {

constexpr int kNW = 8;  // warps per CTA

template <int FS, int PREC, int U, int MINB>
__global__ void __launch_bounds__(kNW * 32, MINB) spmm_lean_kernel(const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;

    extern __shared__ __align__(16) float smem[];
    float* part = smem;  // [2 kNW][8][FS]
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * kNW * 8 * FS);
    Block<FS, kNW> blk;
    blk.init(a, s_rwo, part);
    const int g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);

    if (tb < te) {
        BitDecode dec;
        dec.init(g, tq);
        // this lane's float4 offsets inside a row slice, clamped to the row
        const uint32_t kr = a.K - blk.f0;  // features left in this slice (>= 4)
        uint32_t off[H];
#pragma unroll
        for (int h = 0; h < H; ++h) off[h] = min(uint32_t(32 * h + 4 * g), kr - 4);
        const float* Bs = a.B + blk.f0;
        const uint32_t* a2b_l = a.a2b + tq;  // lane's two entries: [8t + tq], [8t + tq + 4]

        uint32_t wl = blk.window_of(tb);
        uint32_t next_bound = blk.s_rwo[wl + 1];
        bool first_win = true;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        // sparseA2B entries of the next batch
        uint32_t n0[U], n1[U];
        auto load_idx = [&](uint32_t t) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const bool ok = t + u < te;
                n0[u] = ok ? __ldg(a2b_l + size_t(t + u) * 8) : kPad;
                n1[u] = ok ? __ldg(a2b_l + size_t(t + u) * 8 + 4) : kPad;
            }
        };
        load_idx(tb);

        for (uint32_t t = tb; t < te; t += U) {
            float4 r0[U][H], r1[U][H];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const float* p0 = n0[u] < a.cols ? Bs + size_t(n0[u]) * a.K : g_lean_zero;
                const float* p1 = n1[u] < a.cols ? Bs + size_t(n1[u]) * a.K : g_lean_zero;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    r0[u][h] = ldg_f4_ordered(p0 + off[h]);
                    r1[u][h] = ldg_f4_ordered(p1 + off[h]);
                }
            }
            uint64_t bm[U];
            uint32_t to[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t tt = min(t + u, te - 1);
                bm[u] = __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tt);
                to[u] = __ldg(a.tc_offset + tt);
            }
            if (t + U < te) load_idx(t + U);
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
                uint32_t x0, x1;
                bool q0, q1;
                dec.decode(bm[u], x0, x1, q0, q1);
                const float av0 = q0 ? __ldg(a.vals + to[u] + x0) : 0.f;
                const float av1 = q1 ? __ldg(a.vals + to[u] + x1) : 0.f;
                tile_mma<H, PREC>(acc, r0[u], r1[u], av0, av1);
            }
        }
        blk.flush(a, acc, wl, tb, te, first_win);
    }
    __syncthreads();
    blk.finish(a);
}

template <int FS, int PREC, int U, int MINB>
int launch_one(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = size_t(2 * kNW * 8 * FS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_lean_kernel<FS, PREC, U, MINB>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_lean_kernel<FS, PREC, U, MINB><<<unsigned(grid), kNW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

template <int PREC>
int launch_prec(const SpmmArgs& a, int fs, int minb, cudaStream_t s) {
    switch (fs) {
        case 32: return minb >= 4 ? launch_one<32, PREC, 4, 4>(a, s) : launch_one<32, PREC, 4, 3>(a, s);
        case 64: return minb >= 4 ? launch_one<64, PREC, 2, 4>(a, s) : launch_one<64, PREC, 2, 3>(a, s);
        default: return minb >= 3 ? launch_one<128, PREC, 1, 3>(a, s) : launch_one<128, PREC, 2, 2>(a, s);
    }
}

}  // namespace

int launch_lean(const SpmmArgs& a, int fs, int precision, int minb, cudaStream_t s) {
    return precision == ACCSPMM_PREC_3XTF32 ? launch_prec<ACCSPMM_PREC_3XTF32>(a, fs, minb, s)
                                            : launch_prec<ACCSPMM_PREC_TF32>(a, fs, minb, s);
}

}  // namespace accspmm
