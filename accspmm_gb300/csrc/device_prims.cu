// device_prims.cu -- device-wide exclusive scan and stable LSD radix sort,
// the building blocks of the GPU METCF builder.
#include "device_prims.hpp"
#include "device_util.cuh"

namespace accspmm {

// ---------------------------------------------------------------------------
// Exclusive scan of uint32 (mod 2^32), out[0..n] with out[n] = total.
// Tiles of 2048 items (256 threads x 8 consecutive items); tile sums are
// scanned recursively and added back.
// ---------------------------------------------------------------------------
namespace {
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads)
scan_tiles_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, size_t n,
                  uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        size_t idx = base + i;
        v[i] = idx < n ? in[idx] : 0u;
        sum += v[i];
    }
    // inclusive warp scan of per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    uint32_t warp_off = 0, block_tot = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        uint32_t t = warp_tot[w];
        if (w < warp) warp_off += t;
        block_tot += t;
    }
    uint32_t run = warp_off + incl - sum;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        size_t idx = base + i;
        if (idx < n) out[idx] = run;
        if (idx == n) out[n] = run;  // the total, relative to this tile
        run += v[i];
    }
    if (threadIdx.x == 0 && tile_sums) tile_sums[blockIdx.x] = block_tot;
}

__global__ void scan_add_kernel(uint32_t* __restrict__ out, size_t n_plus_1,
                                const uint32_t* __restrict__ tile_off) {
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n_plus_1) out[i] += tile_off[i / kScanTile];
}
}  // namespace

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s) {
    size_t tiles = (n + 1 + kScanTile - 1) / kScanTile;  // out has n + 1 entries
    if (tiles <= 1) {
        scan_tiles_kernel<<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
        ACC_LAUNCH_CHECK();
        return ACCSPMM_SUCCESS;
    }
    DevBuf<uint32_t> sums, sums_scan;
    ACC_CUDA(sums.alloc(tiles, s));
    ACC_CUDA(sums_scan.alloc(tiles + 1, s));
    scan_tiles_kernel<<<unsigned(tiles), kScanThreads, 0, s>>>(in, out, n, sums.p);
    ACC_LAUNCH_CHECK();
    int st = scan_exclusive_u32(sums.p, sums_scan.p, tiles, s);
    if (st) return st;
    size_t m = n + 1;
    scan_add_kernel<<<unsigned((m + 255) / 256), 256, 0, s>>>(out, m, sums_scan.p);
    ACC_LAUNCH_CHECK();
    return ACCSPMM_SUCCESS;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (uint64 key, uint32 value) pairs, 8-bit digits.
// A tile of 4096 items is split into 8 warp segments of 512 items processed
// in 16 rounds of 32, so (warp, round, lane) is input order; each element's
// place among equal digits comes from __match_any_sync + popc, which keeps
// the scatter stable.
// ---------------------------------------------------------------------------
namespace {
constexpr int kRsThreads = 256;
constexpr int kRsWarps = kRsThreads / 32;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;

__global__ void __launch_bounds__(kRsThreads)
radix_hist_kernel(const uint64_t* __restrict__ keys, size_t n, int shift,
                  uint32_t* __restrict__ hist, uint32_t ntiles) {
    __shared__ uint32_t h[256];
    for (int i = threadIdx.x; i < 256; i += kRsThreads) h[i] = 0;
    __syncthreads();
    const size_t base = size_t(blockIdx.x) * kRsTile;
#pragma unroll 4
    for (int r = 0; r < kRsRounds; ++r) {
        size_t idx = base + size_t(r) * kRsThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kRsThreads) hist[size_t(d) * ntiles + blockIdx.x] = h[d];
}

__global__ void __launch_bounds__(kRsThreads)
radix_scatter_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                     uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, size_t n,
                     int shift, const uint32_t* __restrict__ offs, uint32_t ntiles) {
    __shared__ uint32_t wh[kRsWarps][256];
    for (int i = threadIdx.x; i < kRsWarps * 256; i += kRsThreads) (&wh[0][0])[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const size_t seg = size_t(blockIdx.x) * kRsTile + size_t(warp) * 32 * kRsRounds;
    uint64_t k[kRsRounds];
    uint32_t v[kRsRounds];
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
        size_t idx = seg + size_t(r) * 32 + lane;
        bool valid = idx < n;
        k[r] = valid ? kin[idx] : 0ull;
        v[r] = valid ? vin[idx] : 0u;
        unsigned d = valid ? unsigned((k[r] >> shift) & 255u) : 256u;
        unsigned m = __match_any_sync(0xffffffffu, d);
        if (valid && lane == __ffs(m) - 1) wh[warp][d] += __popc(m);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kRsThreads) {
        uint32_t run = offs[size_t(d) * ntiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kRsWarps; ++w) {
            uint32_t c = wh[w][d];
            wh[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kRsRounds; ++r) {
        size_t idx = seg + size_t(r) * 32 + lane;
        bool valid = idx < n;
        unsigned d = valid ? unsigned((k[r] >> shift) & 255u) : 256u;
        unsigned m = __match_any_sync(0xffffffffu, d);
        if (valid) {
            uint32_t pos = wh[warp][d] + __popc(m & lt_mask);
            kout[pos] = k[r];
            vout[pos] = v[r];
        }
        __syncwarp();
        if (valid && lane == __ffs(m) - 1) wh[warp][d] += __popc(m);
        __syncwarp();
    }
}
}  // namespace

int radix_sort_pairs(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                     uint32_t* vals_out, size_t n, int nbits, cudaStream_t s) {
    if (n == 0) return ACCSPMM_SUCCESS;
    if (n > 0xFFFFFFFFull) ACC_FAIL(ACCSPMM_ERROR_OVERFLOW, "radix sort of %zu items", n);
    const int npass = (nbits + 7) / 8;
    if (npass == 0) {
        ACC_CUDA(cudaMemcpyAsync(keys_out, keys_in, n * 8, cudaMemcpyDeviceToDevice, s));
        ACC_CUDA(cudaMemcpyAsync(vals_out, vals_in, n * 4, cudaMemcpyDeviceToDevice, s));
        return ACCSPMM_SUCCESS;
    }
    const uint32_t ntiles = uint32_t((n + kRsTile - 1) / kRsTile);
    DevBuf<uint64_t> ktmp;
    DevBuf<uint32_t> vtmp, hist, offs;
    ACC_CUDA(ktmp.alloc(n, s));
    ACC_CUDA(vtmp.alloc(n, s));
    ACC_CUDA(hist.alloc(size_t(256) * ntiles, s));
    ACC_CUDA(offs.alloc(size_t(256) * ntiles + 1, s));
    const uint64_t* ksrc = keys_in;
    const uint32_t* vsrc = vals_in;
    for (int p = 0; p < npass; ++p) {
        bool to_out = ((npass - 1 - p) % 2) == 0;
        uint64_t* kdst = to_out ? keys_out : ktmp.p;
        uint32_t* vdst = to_out ? vals_out : vtmp.p;
        radix_hist_kernel<<<ntiles, kRsThreads, 0, s>>>(ksrc, n, 8 * p, hist.p, ntiles);
        ACC_LAUNCH_CHECK();
        int st = scan_exclusive_u32(hist.p, offs.p, size_t(256) * ntiles, s);
        if (st) return st;
        radix_scatter_kernel<<<ntiles, kRsThreads, 0, s>>>(ksrc, vsrc, kdst, vdst, n, 8 * p,
                                                            offs.p, ntiles);
        ACC_LAUNCH_CHECK();
        ksrc = kdst;
        vsrc = vdst;
    }
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
