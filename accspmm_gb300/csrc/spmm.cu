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

#include "common.hpp"
#include "device_util.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

constexpr int kNW = 8;  // warps per CTA

struct SpmmArgs {
    const uint32_t* rwo;
    const uint32_t* tc_offset;
    const uint64_t* bits;
    const uint32_t* a2b;
    const float* vals;
    const float* B;
    float* C;
    uint32_t W;         // windows covered (C has 8W rows)
    uint32_t cols;      // rows of B
    uint32_t K;         // columns of B and C
    uint32_t wb;        // windows per CTA
    uint32_t n_slices;  // feature slices
};

__device__ __forceinline__ uint32_t f2tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float4 ldg_f4(const float* p) {
    return __ldg(reinterpret_cast<const float4*>(p));
}

__device__ __forceinline__ float comp(const float4& v, int j) {
    return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w;
}

__device__ __forceinline__ uint64_t shfl_u64(uint64_t v, int src) {
    uint32_t lo = __shfl_sync(0xffffffffu, uint32_t(v), src);
    uint32_t hi = __shfl_sync(0xffffffffu, uint32_t(v >> 32), src);
    return (uint64_t(hi) << 32) | lo;
}

// Sparse value of tile element `bit` (row-major 8x8), 0 if absent.
__device__ __forceinline__ float tile_value(uint64_t bm, uint32_t off, const float* __restrict__ vals,
                                            uint32_t bit) {
    if (!((bm >> bit) & 1ull)) return 0.0f;
    uint64_t below = bm & ((2ull << bit) - 1ull);  // 2 << 63 wraps to 0: all bits
    return __ldg(vals + off + __popcll(below) - 1);
}

// Accumulator layout helpers.  H = FS / 32 float4 per B row per lane;
// NM = MMAs per tile.  acc[m][0..3] follow the m16n8 D fragment: [0] (g, 2tq),
// [1] (g, 2tq+1), [2] (g+8, 2tq), [3] (g+8, 2tq+1); m-row -> feature below.
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

template <int FS>
__device__ __forceinline__ void store_rows(float* __restrict__ C, uint32_t K, uint32_t row0,
                                           uint32_t f0, int g, int tq, const float4 (&out)[2][FS / 32]) {
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

// Shared-memory partial slot: [8 rows][FS] floats.
template <int FS>
__device__ __forceinline__ float* slot_ptr(float* part, int slot) {
    return part + size_t(slot) * 8 * FS;
}

template <int FS, int PREC>
__global__ void __launch_bounds__(kNW * 32, 2) spmm_window_kernel(const SpmmArgs a) {
    constexpr int H = FS / 32;
    using L = Layout<H>;
    constexpr int NM = L::NM;
    constexpr int U = H >= 4 ? 2 : (H == 2 ? 4 : 8);  // tiles per batch
    constexpr int MA = (8 * U + 31) / 32;             // a2b registers per lane

    extern __shared__ float smem[];
    float* part = smem;  // [2 * kNW] slots
    uint32_t* s_rwo = reinterpret_cast<uint32_t*>(smem + 2 * kNW * 8 * FS);

    const uint32_t wbk = blockIdx.x / a.n_slices;
    const uint32_t slice = blockIdx.x - wbk * a.n_slices;
    const uint32_t w0 = wbk * a.wb;
    const uint32_t w1 = min(w0 + a.wb, a.W);
    const uint32_t nwin = w1 - w0;
    const uint32_t f0 = slice * FS;
    for (uint32_t i = threadIdx.x; i <= nwin; i += blockDim.x) s_rwo[i] = a.rwo[w0 + i];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tq = lane & 3;
    const uint32_t t_begin = s_rwo[0];
    const uint32_t t_total = s_rwo[nwin] - t_begin;
    auto bound = [&](int i) -> uint32_t {
        return t_begin + uint32_t((uint64_t(t_total) * uint32_t(i)) / kNW);
    };
    const uint32_t tb = bound(warp), te = bound(warp + 1);

    // feature offsets of this lane's float4s and whether they are inside K
    bool fok[H];
#pragma unroll
    for (int h = 0; h < H; ++h) fok[h] = f0 + 32 * h + 4 * g < a.K;

    if (tb < te) {
        // window (local index) containing tb
        uint32_t wl = 0;
        for (uint32_t jb = 0; jb < nwin; jb += 32) {
            const uint32_t j = jb + uint32_t(lane);
            const bool in = j < nwin && s_rwo[j] <= tb && tb < s_rwo[j + 1];
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            if (bal) wl = jb + uint32_t(__ffs(bal) - 1);
        }
        uint32_t next_bound = s_rwo[wl + 1];
        bool first_win = true;
        float acc[NM][4];
#pragma unroll
        for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;

        auto flush = [&](uint32_t wloc) {
            const uint32_t rb = s_rwo[wloc], re = s_rwo[wloc + 1];
            float4 out[2][H];
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int h = 0; h < H; ++h) out[p][h] = L::get(acc, p, h);
            if (rb >= tb && re <= te) {
                store_rows<FS>(a.C, a.K, (w0 + wloc) * kWin, f0, g, tq, out);
            } else {
                float* sp = slot_ptr<FS>(part, 2 * warp + (first_win ? 0 : 1));
#pragma unroll
                for (int p = 0; p < 2; ++p)
#pragma unroll
                    for (int h = 0; h < H; ++h)
                        *reinterpret_cast<float4*>(sp + (2 * tq + p) * FS + 32 * h + 4 * g) = out[p][h];
            }
        };

        // metadata of a batch of U tiles starting at t
        uint32_t ma[MA];
        uint64_t mb;
        uint32_t mo;
        auto load_meta = [&](uint32_t t) {
#pragma unroll
            for (int j = 0; j < MA; ++j) {
                uint32_t e = 32 * j + lane;            // entry within the batch
                uint32_t tile = t + e / 8;
                ma[j] = (e < 8 * U && tile < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
            }
            uint32_t tl = t + uint32_t(lane);
            bool ok = lane < U && tl < te;
            mb = ok ? __ldg(reinterpret_cast<const unsigned long long*>(a.bits) + tl) : 0ull;
            mo = ok ? __ldg(a.tc_offset + tl) : 0u;
        };
        load_meta(tb);

        const uint32_t bit0 = uint32_t(g) * 8 + uint32_t(tq), bit1 = bit0 + 4;
        for (uint32_t t = tb; t < te; t += U) {
            // gather: A values and B rows of the whole batch
            float av0[U], av1[U];
            float4 r0[U][H], r1[U][H];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
                const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
                const uint64_t bm = shfl_u64(mb, u);
                const uint32_t to = __shfl_sync(0xffffffffu, mo, u);
                av0[u] = tile_value(bm, to, a.vals, bit0);
                av1[u] = tile_value(bm, to, a.vals, bit1);
                const bool v0 = i0 < a.cols, v1 = i1 < a.cols;
                const float* p0 = a.B + size_t(v0 ? i0 : 0) * a.K + f0 + 4 * g;
                const float* p1 = a.B + size_t(v1 ? i1 : 0) * a.K + f0 + 4 * g;
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    r0[u][h] = (v0 && fok[h]) ? ldg_f4(p0 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                    r1[u][h] = (v1 && fok[h]) ? ldg_f4(p1 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            if (t + U < te) load_meta(t + U);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t tt = t + u;
                if (tt >= te) break;
                if (tt >= next_bound) {
                    flush(wl);
                    first_win = false;
#pragma unroll
                    for (int m = 0; m < NM; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.f;
                    while (s_rwo[wl + 1] <= tt) ++wl;
                    next_bound = s_rwo[wl + 1];
                }
                if constexpr (PREC == ACCSPMM_PREC_TF32) {
                    const uint32_t b0 = f2tf32(av0[u]), b1 = f2tf32(av1[u]);
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const int j = m & 3;
                        float x0, x1, x2, x3;
                        if constexpr (H >= 2) {
                            const int hp = m >> 2;
                            x0 = comp(r0[u][2 * hp], j); x1 = comp(r0[u][2 * hp + 1], j);
                            x2 = comp(r1[u][2 * hp], j); x3 = comp(r1[u][2 * hp + 1], j);
                        } else {
                            x0 = comp(r0[u][0], m); x1 = comp(r0[u][0], m + 2);
                            x2 = comp(r1[u][0], m); x3 = comp(r1[u][0], m + 2);
                        }
                        mma_tf32(acc[m], f2tf32(x0), f2tf32(x1), f2tf32(x2), f2tf32(x3), b0, b1);
                    }
                } else {
                    // 3xTF32 (Ootomo & Yokota 2022): x = hi + lo with hi, lo TF32;
                    // d = B_lo*A_hi + B_hi*A_lo + B_hi*A_hi per tile, then added to
                    // the FP32 accumulators outside the tensor core.
                    const uint32_t bh0 = f2tf32(av0[u]), bh1 = f2tf32(av1[u]);
                    const uint32_t bl0 = f2tf32(av0[u] - __uint_as_float(bh0));
                    const uint32_t bl1 = f2tf32(av1[u] - __uint_as_float(bh1));
#pragma unroll
                    for (int m = 0; m < NM; ++m) {
                        const int j = m & 3;
                        float x[4];
                        if constexpr (H >= 2) {
                            const int hp = m >> 2;
                            x[0] = comp(r0[u][2 * hp], j); x[1] = comp(r0[u][2 * hp + 1], j);
                            x[2] = comp(r1[u][2 * hp], j); x[3] = comp(r1[u][2 * hp + 1], j);
                        } else {
                            x[0] = comp(r0[u][0], m); x[1] = comp(r0[u][0], m + 2);
                            x[2] = comp(r1[u][0], m); x[3] = comp(r1[u][0], m + 2);
                        }
                        uint32_t hi[4], lo[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            hi[q] = f2tf32(x[q]);
                            lo[q] = f2tf32(x[q] - __uint_as_float(hi[q]));
                        }
                        float d[4] = {0.f, 0.f, 0.f, 0.f};
                        mma_tf32(d, lo[0], lo[1], lo[2], lo[3], bh0, bh1);
                        mma_tf32(d, hi[0], hi[1], hi[2], hi[3], bl0, bl1);
                        mma_tf32(d, hi[0], hi[1], hi[2], hi[3], bh0, bh1);
                        acc[m][0] += d[0]; acc[m][1] += d[1]; acc[m][2] += d[2]; acc[m][3] += d[3];
                    }
                }
            }
        }
        flush(wl);
    }
    __syncthreads();

    // windows cut by piece boundaries: sum the slots in warp order; empty
    // windows: zeros
    auto warp_of = [&](uint32_t t) -> int {
        int i = kNW - 1;
        while (i > 0 && bound(i) > t) --i;
        return i;
    };
    for (uint32_t wloc = warp; wloc < nwin; wloc += kNW) {
        const uint32_t rb = s_rwo[wloc], re = s_rwo[wloc + 1];
        float4 out[2][H];
        if (rb == re) {
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int h = 0; h < H; ++h) out[p][h] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const int ia = warp_of(rb), ib = warp_of(re - 1);
            if (ia == ib) continue;  // stored by its warp
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int h = 0; h < H; ++h) out[p][h] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int i = ia; i <= ib; ++i) {
                const uint32_t bi = bound(i);
                if (bi == bound(i + 1)) continue;  // empty piece
                const float* sp = slot_ptr<FS>(part, 2 * i + (rb <= bi ? 0 : 1));
#pragma unroll
                for (int p = 0; p < 2; ++p)
#pragma unroll
                    for (int h = 0; h < H; ++h) {
                        float4 v = *reinterpret_cast<const float4*>(sp + (2 * tq + p) * FS + 32 * h + 4 * g);
                        out[p][h].x += v.x; out[p][h].y += v.y; out[p][h].z += v.z; out[p][h].w += v.w;
                    }
            }
        }
        store_rows<FS>(a.C, a.K, (w0 + wloc) * kWin, f0, g, tq, out);
    }
}

// rwo[w] = first tile whose window (row_indices / 8) is >= w, for w in
// [0, Weff]; tiles claiming windows >= Weff raise *err.
__global__ void rwo_from_row_indices_kernel(const uint32_t* __restrict__ ri, uint32_t T,
                                            uint32_t Weff, uint32_t* __restrict__ rwo,
                                            uint32_t* __restrict__ err) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > T) return;
    uint32_t lo = t == 0 ? 0u : ri[t - 1] / kWin + 1;
    uint32_t hi = t == T ? Weff : ri[t] / kWin;
    if (t < T && hi >= Weff) {
        atomicOr(err, 1u);
        hi = Weff;
    }
    if (t > 0 && t < T && ri[t] < ri[t - 1]) atomicOr(err, 2u);
    for (uint32_t w = lo; w <= hi && w <= Weff; ++w) rwo[w] = t;
}

struct Config {
    int fs;
    uint32_t wb;
};

Config choose_config(uint32_t W, uint32_t K) {
    Config c;
    c.fs = K <= 32 ? 32 : 64;
    if (const char* e = std::getenv("ACCSPMM_FS")) {
        int v = std::atoi(e);
        if (v == 32 || v == 64 || v == 128) c.fs = v;
    }
    uint32_t slices = (K + c.fs - 1) / c.fs;
    // enough CTAs to fill every SM several times over, 4..32 windows each
    uint64_t want = uint64_t(sm_count()) * 16;
    uint64_t wb = (uint64_t(W) * slices + want - 1) / want;
    c.wb = uint32_t(std::min<uint64_t>(32, std::max<uint64_t>(4, wb)));
    if (const char* e = std::getenv("ACCSPMM_WB")) {
        int v = std::atoi(e);
        if (v >= 1 && v <= 256) c.wb = uint32_t(v);
    }
    return c;
}

template <int FS, int PREC>
int launch_fs(const SpmmArgs& a, cudaStream_t s) {
    const size_t smem = size_t(2 * kNW * 8 * FS) * 4 + size_t(a.wb + 1) * 4;
    static unsigned attr_set = 0;  // one bit per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 32 && !(attr_set & (1u << dev))) {
        ACC_CUDA(cudaFuncSetAttribute(spmm_window_kernel<FS, PREC>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_set |= 1u << dev;
    }
    const uint64_t grid = uint64_t((a.W + a.wb - 1) / a.wb) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    spmm_window_kernel<FS, PREC><<<unsigned(grid), kNW * 32, smem, s>>>(a);
    ACC_LAUNCH_CHECK();
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

int spmm_window_launch(const uint32_t* rwo, const uint32_t* tc_offset, const uint64_t* bits,
                       const uint32_t* a2b, const float* vals, uint32_t W, uint32_t w_cfg,
                       uint32_t cols, const float* B, float* C, uint32_t K, int precision,
                       cudaStream_t s) {
    if (W == 0) return ACCSPMM_SUCCESS;
    // the launch shape depends only on (w_cfg, K), so both entry points cut a
    // matrix into the same pieces and sum partial windows in the same order
    Config cfg = choose_config(w_cfg, K);
    SpmmArgs a{rwo, tc_offset, bits, a2b, vals, B, C, W, cols, K, cfg.wb,
               (K + uint32_t(cfg.fs) - 1) / uint32_t(cfg.fs)};
    const bool x3 = precision == ACCSPMM_PREC_3XTF32;
    switch (cfg.fs) {
        case 32: return x3 ? launch_fs<32, ACCSPMM_PREC_3XTF32>(a, s) : launch_fs<32, ACCSPMM_PREC_TF32>(a, s);
        case 64: return x3 ? launch_fs<64, ACCSPMM_PREC_3XTF32>(a, s) : launch_fs<64, ACCSPMM_PREC_TF32>(a, s);
        default: return x3 ? launch_fs<128, ACCSPMM_PREC_3XTF32>(a, s) : launch_fs<128, ACCSPMM_PREC_TF32>(a, s);
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
                              m->data, m->num_windows, m->num_windows, m->cols, B, C, K, precision,
                              as_stream(stream));
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
    DevBuf<uint32_t> scratch;  // rwo[Weff + 1] then an error word
    ACC_CUDA(scratch.alloc(size_t(Weff) + 2, s));
    uint32_t* rwo = scratch.p;
    uint32_t* err = scratch.p + Weff + 1;
    ACC_CUDA(cudaMemsetAsync(err, 0, 4, s));
    rwo_from_row_indices_kernel<<<(T + 1 + 255) / 256, 256, 0, s>>>(ad->row_indices, T, Weff, rwo, err);
    ACC_LAUNCH_CHECK();
    return spmm_window_launch(rwo, ad->tc_offset, ad->tc_local_bit, ad->sparse_a2b, ad->data, Weff,
                              (ad->rows + kWin - 1) / kWin, ad->cols, B, C, K, precision, s);
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
