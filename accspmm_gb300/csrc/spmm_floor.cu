// spmm_floor.cu -- the gather floor of a METCF SpMM: the time to move exactly
// the B rows the SpMM kernel gathers, in the kernel's own order, and nothing
// else.
//
// The kernel is the one-matrix register-direct kernel with everything but its
// B-row gathers taken out: the same work items (window block x feature slice,
// from the same launch-shape chooser or at another slice width), the same
// equal per-warp tile pieces, the same lane pattern (eight lanes per 128
// contiguous bytes of a row, tile columns tq and tq + 4), the same batch of
// tiles in flight and the same CTAs per SM -- but no sparse values, no MMAs
// and no C stores.  The
// gathered rows are summed into one register so that the loads are not
// removed.  Its time is what the SpMM would take if its arithmetic, value
// loads and stores were free: the denominator of the "fraction of the gather
// floor" that bench.py reports beside the HBM roofline, for a kernel whose
// traffic is set by the matrix's column pattern rather than by its
// compulsory bytes.  No counterpart in the reference.
#include "common.hpp"
#include "device_util.cuh"
#include "spmm_common.cuh"
#include "spmm_direct.cuh"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

template <int FS, int U, int MINB>
__global__ void __launch_bounds__(kDirectNW * 32, MINB) gather_floor_kernel(const SpmmArgs a, float* sink) {
    constexpr int H = FS / 32;
    constexpr int MA = (8 * U + 31) / 32;
    extern __shared__ __align__(16) uint32_t s_rwo_floor[];
    Block<FS, kDirectNW> blk;
    blk.init(a, s_rwo_floor, nullptr);
    const int lane = blk.lane, g = blk.g, tq = blk.tq;
    const uint32_t tb = blk.bound(blk.warp), te = blk.bound(blk.warp + 1);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    bool fok[H];
#pragma unroll
    for (int h = 0; h < H; ++h) fok[h] = blk.f0 + 32 * h + 4 * g < a.K;
    const float* Bl = a.B + blk.f0 + 4 * g;
    for (uint32_t t = tb; t < te; t += U) {
        uint32_t ma[MA];
#pragma unroll
        for (int j = 0; j < MA; ++j) {
            const uint32_t e = 32 * j + lane;
            ma[j] = (e < 8 * U && t + e / 8 < te) ? __ldg(a.a2b + size_t(t) * 8 + e) : kPad;
        }
        float4 r[U][2][H];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t i0 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq) & 31);
            const uint32_t i1 = __shfl_sync(0xffffffffu, ma[(8 * u) / 32], (8 * u + tq + 4) & 31);
            const bool v0 = i0 < a.cols, v1 = i1 < a.cols;
            const float* p0 = Bl + size_t(v0 ? i0 : 0) * a.K;
            const float* p1 = Bl + size_t(v1 ? i1 : 0) * a.K;
#pragma unroll
            for (int h = 0; h < H; ++h) {
                r[u][0][h] = (v0 && fok[h]) ? ldg_f4_ordered(p0 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
                r[u][1][h] = (v1 && fok[h]) ? ldg_f4_ordered(p1 + 32 * h) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < 2; ++q)
#pragma unroll
                for (int h = 0; h < H; ++h) {
                    acc.x += r[u][q][h].x; acc.y += r[u][q][h].y;
                    acc.z += r[u][q][h].z; acc.w += r[u][q][h].w;
                }
    }
    // never true for finite B: keeps the loads without a store per thread
    if (acc.x == 1.5e38f && acc.y == -1.5e38f) sink[0] = acc.z + acc.w;
}

template <int FS, int U, int MINB>
int launch_floor(const SpmmArgs& a, float* sink, cudaStream_t s) {
    const size_t smem = size_t(a.wb + 1) * 4;
    const uint64_t grid = uint64_t(a.n_wblocks) * a.n_slices;
    if (grid == 0) return ACCSPMM_SUCCESS;
    if (grid > 0x7FFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "grid too large");
    gather_floor_kernel<FS, U, MINB><<<unsigned(grid), kDirectNW * 32, smem, s>>>(a, sink);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

// the register-direct kernel's (FS, batch, CTAs per SM) for occ = 2 or 3
int launch_floor_shape(const SpmmArgs& a, int fs, int occ, float* sink, cudaStream_t s) {
    if (occ == 3) {
        switch (fs) {
            case 32: return launch_floor<32, (DirectBatch<32>::U + 1) / 2, 3>(a, sink, s);
            case 64: return launch_floor<64, (DirectBatch<64>::U + 1) / 2, 3>(a, sink, s);
            default: return launch_floor<128, (DirectBatch<128>::U + 1) / 2, 3>(a, sink, s);
        }
    }
    switch (fs) {
        case 32: return launch_floor<32, DirectBatch<32>::U, 2>(a, sink, s);
        case 64: return launch_floor<64, DirectBatch<64>::U, 2>(a, sink, s);
        default: return launch_floor<128, DirectBatch<128>::U, 2>(a, sink, s);
    }
}

}  // namespace

int gather_floor_impl(const accspmm_metcf_t* m, const float* B, uint32_t K, uint32_t slice_width,
                      int repeats, float* avg_ms, void* stream) {
    if (!m || m->space != ACCSPMM_DEVICE) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "METCF must be on the device");
    if (!B || K == 0 || K % 4 || (reinterpret_cast<uintptr_t>(B) & 15u))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "B must be a 16-byte aligned device pointer, K a multiple of 4");
    if (!avg_ms || repeats <= 0) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "bad timing arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int fs = 0, occ = 0;
    uint32_t wb = 0;
    launch_shape_for(m->num_windows, m->num_tiles, K, ACCSPMM_PREC_TF32, &fs, &occ, &wb);
    if (slice_width) {
        if (slice_width != 32 && slice_width != 64 && slice_width != 128)
            ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "slice_width must be 0, 32, 64 or 128");
        fs = int(slice_width);
        occ = fs == 128 ? 2 : 3;  // the register-direct kernel's CTAs per SM at that width
    }
    const uint32_t W = m->num_windows;
    SpmmArgs a{m->row_window_offset, m->tc_offset, m->tc_local_bit, m->sparse_a2b, m->data, B,
               nullptr, W, m->cols, K, wb, (K + uint32_t(fs) - 1) / uint32_t(fs), (W + wb - 1) / wb,
               0, 0, nullptr, 0, nullptr, nullptr, 0};
    DevBuf<float> sink;
    ACC_CUDA(sink.alloc(1, s));
    int r = launch_floor_shape(a, fs, occ, sink.p, s);  // warm-up
    if (r) return r;
    cudaEvent_t e0, e1;
    ACC_CUDA(cudaEventCreate(&e0));
    ACC_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, s);
    for (int i = 0; i < repeats && !r; ++i) r = launch_floor_shape(a, fs, occ, sink.p, s);
    cudaEventRecord(e1, s);
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r) return r;
    if (ce != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_CUDA, "timing failed: %s", cudaGetErrorString(ce));
    *avg_ms = ms / float(repeats);
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
