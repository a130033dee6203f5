// spmm_host.cpp -- SpMM with B and C in host memory: the host wrappers
// tf32_spmm / adp_tf32_spmm of src/mma_tf32.cu:12-183 (cudaMalloc, copy B in,
// launch, copy C out), rebuilt as one pipelined call.
//
// The product is cut into feature slices of the launch-shape chooser's width
// cut to about a quarter of K, 32 to 64 columns (four slices at K = 128 and
// K = 256), each launched with the chooser's window blocks, so every element's arithmetic is that of the
// one-launch entry point and the result is bit-identical to it.  Per slice, on the
// library's copy streams:
//   copy stream 1: B[:, slice] host -> device (a 2D copy of the slice's
//                  columns), then an event;
//   caller stream: waits for that event, launches the slice;
//   C output:      if C_host is pinned (page-locked, device-mapped) the
//                  kernel stores the slice straight into it across the
//                  host link, so no D2H pass exists; otherwise copy stream 2
//                  copies C[:, slice] device -> host after the launch.
// The H2D copy of slice i + 1 overlaps the launch of slice i, and with a
// pinned C the host-link writes of slice i overlap both.  Device buffers come
// from a per-device memory pool that keeps its memory between calls, so
// repeated calls do not map and unmap device memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "accspmm.h"
#include "common.hpp"
#include "options.hpp"
#include "spmm_internal.hpp"

namespace accspmm {

namespace {

#define HOST_CUDA(call)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) ACC_FAIL(ACCSPMM_ERROR_CUDA, "%s failed: %s", #call,        \
                                        cudaGetErrorString(e_));                           \
    } while (0)

struct DeviceCtx {
    cudaMemPool_t pool = nullptr;
    cudaStream_t h2d = nullptr, d2h = nullptr;
};

// Per-device pool and copy streams, created on first use.
int device_ctx(DeviceCtx** out) {
    static std::mutex mu;
    static DeviceCtx ctx[64];
    static bool made[64] = {false};
    int dev = 0;
    HOST_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) ACC_FAIL(ACCSPMM_ERROR_UNSUPPORTED, "device %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!made[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        HOST_CUDA(cudaMemPoolCreate(&ctx[dev].pool, &props));
        uint64_t keep = ~uint64_t(0);  // keep freed memory in the pool
        HOST_CUDA(cudaMemPoolSetAttribute(ctx[dev].pool, cudaMemPoolAttrReleaseThreshold, &keep));
        HOST_CUDA(cudaStreamCreateWithFlags(&ctx[dev].h2d, cudaStreamNonBlocking));
        HOST_CUDA(cudaStreamCreateWithFlags(&ctx[dev].d2h, cudaStreamNonBlocking));
        made[dev] = true;
    }
    *out = &ctx[dev];
    return ACCSPMM_SUCCESS;
}

// Pool allocation released (stream-ordered on `s`) when the holder goes out
// of scope.
struct PoolBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    ~PoolBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

// Events of one call, destroyed on return (destroying an event whose work is
// still queued is allowed: its resources are released when it completes).
struct Events {
    std::vector<cudaEvent_t> ev;
    ~Events() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    int make(cudaEvent_t* e) {
        HOST_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        ev.push_back(*e);
        return ACCSPMM_SUCCESS;
    }
};

// On scope exit, orders the caller's stream after everything enqueued on the
// copy streams, so that the stream-ordered frees of the call's buffers (and
// the caller's later work) follow every copy, on success and on error.
struct JoinCopies {
    DeviceCtx* ctx;
    cudaStream_t s;
    ~JoinCopies() {
        for (cudaStream_t c : {ctx->h2d, ctx->d2h}) {
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) continue;
            if (cudaEventRecord(e, c) == cudaSuccess) cudaStreamWaitEvent(s, e, 0);
            cudaEventDestroy(e);
        }
    }
};

// Device address through which a kernel may write `p`, or nullptr when `p`
// is not page-locked host memory.
float* mapped_host(float* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return static_cast<float*>(at.devicePointer);
}

}  // namespace

int library_pool(cudaMemPool_t* pool) {
    DeviceCtx* ctx = nullptr;
    int r = device_ctx(&ctx);
    if (r) return r;
    *pool = ctx->pool;
    return ACCSPMM_SUCCESS;
}

int spmm_host_impl(const accspmm_metcf_t* m, const accspmm_adpbme_t* ad, const float* B_host,
                   float* C_host, uint32_t K, int precision, void* stream, int* direct_c) {
    if ((m == nullptr) == (ad == nullptr))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "pass exactly one of a METCF and an AdpBME");
    if ((m && m->space != ACCSPMM_DEVICE) || (ad && ad->space != ACCSPMM_DEVICE))
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "the matrix must be on the device");
    if (!B_host || !C_host) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "B and C must be host pointers");
    if (K == 0 || K % 4) ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "K=%u must be a positive multiple of 4", K);
    if (precision != ACCSPMM_PREC_TF32 && precision != ACCSPMM_PREC_3XTF32)
        ACC_FAIL(ACCSPMM_ERROR_INVALID_VALUE, "unknown precision %d", precision);
    const uint32_t rows = m ? m->rows : ad->rows, cols = m ? m->cols : ad->cols;
    const uint32_t T = m ? m->num_tiles : ad->num_tiles;
    const uint32_t W = (rows + kWin - 1) / kWin;
    const size_t crows = size_t(W) * kWin;
    if (direct_c) *direct_c = 0;
    if (W == 0) return ACCSPMM_SUCCESS;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    DeviceCtx* ctx = nullptr;
    int r = device_ctx(&ctx);
    if (r) return r;

    // C written by the kernel straight into host memory when it is pinned and
    // 16-byte aligned (the kernel stores float4s), else staged on the device
    float* c_dev = (reinterpret_cast<uintptr_t>(C_host) & 15u) || option(ACCSPMM_OPT_HOST_DIRECT_C) == 0
                       ? nullptr
                       : mapped_host(C_host);
    const bool direct = c_dev != nullptr;
    if (direct_c) *direct_c = direct ? 1 : 0;

    PoolBuf dB, dC, dR;
    dB.s = dC.s = dR.s = s;
    HOST_CUDA(cudaMallocFromPoolAsync(&dB.p, size_t(cols) * K * 4 + 16, ctx->pool, s));
    if (!direct) {
        HOST_CUDA(cudaMallocFromPoolAsync(&dC.p, crows * K * 4 + 16, ctx->pool, s));
        c_dev = static_cast<float*>(dC.p);
    }
    const uint32_t* rwo = m ? m->row_window_offset : nullptr;
    if (ad && ad->owned) {
        // derived once per library-owned object and kept with it
        r = adaptive_rwo(ad, W, s, &rwo);
        if (r) return r;
    } else if (ad) {
        // window offsets of the W real windows from rowIndices (windows past
        // W hold no tiles), the same derivation as accspmm_spmm_adaptive
        HOST_CUDA(cudaMallocFromPoolAsync(&dR.p, (size_t(W) + 1) * 4, ctx->pool, s));
        uint32_t* rw = static_cast<uint32_t*>(dR.p);
        r = rwo_from_row_indices(ad->row_indices, T, W, rw, nullptr, true, s);
        if (r) return r;
        rwo = rw;
    }
    const uint32_t w_cfg = W;  // the chooser's key: the matrix's own windows
    // the chooser's slice width, cut to about a quarter of K (at least 32,
    // at most 64 columns): on the 1M-row power-law matrix four slices
    // pipelined the link transfers better than two (K = 128: 4.40 against
    // 4.67 ms; K = 64, two slices of 32: 2.37 against 2.77 ms for one), and
    // slices narrower than 64 columns at K = 256 repeated too much of the
    // per-tile work (8 slices of 32: 11.4 ms, 4 of 64: 8.2 ms)
    uint32_t fs = slice_width_for(w_cfg, T, K, precision);
    fs = std::min(fs, std::max<uint32_t>(32u, (K / 4u) / 32u * 32u));
    if (fs > 64) fs = 64;
    if (const int fs_opt = option(ACCSPMM_OPT_HOST_SLICE_WIDTH)) fs = uint32_t(fs_opt);
    const uint32_t nsl = (K + fs - 1) / fs;
    float* dBf = static_cast<float*>(dB.p);

    JoinCopies join{ctx, s};  // runs before the buffers' frees
    Events evs;
    cudaEvent_t start;
    if ((r = evs.make(&start))) return r;
    HOST_CUDA(cudaEventRecord(start, s));  // allocations above are ordered before it
    HOST_CUDA(cudaStreamWaitEvent(ctx->h2d, start, 0));
    if (!direct) HOST_CUDA(cudaStreamWaitEvent(ctx->d2h, start, 0));
    for (uint32_t i = 0; i < nsl; ++i) {
        const uint32_t f0 = i * fs, w = std::min(fs, K - f0);
        HOST_CUDA(cudaMemcpy2DAsync(dBf + f0, size_t(K) * 4, B_host + f0, size_t(K) * 4,
                                    size_t(w) * 4, cols, cudaMemcpyHostToDevice, ctx->h2d));
        cudaEvent_t in;
        if ((r = evs.make(&in))) return r;
        HOST_CUDA(cudaEventRecord(in, ctx->h2d));
        HOST_CUDA(cudaStreamWaitEvent(s, in, 0));
        r = m ? spmm_window_launch_slices(rwo, m->tc_offset, m->tc_local_bit, m->sparse_a2b, m->data,
                                          W, w_cfg, T, cols, dBf, c_dev, K, precision, i, 1,
                                          Epilogue{}, s, int(fs), m->owned != 0)
              : spmm_window_launch_slices(rwo, ad->tc_offset, ad->tc_local_bit, ad->sparse_a2b,
                                          ad->data, W, w_cfg, T, cols, dBf, c_dev, K, precision, i,
                                          1, Epilogue{}, s, int(fs), ad->owned != 0);
        if (r) return r;
        if (!direct) {
            cudaEvent_t done;
            if ((r = evs.make(&done))) return r;
            HOST_CUDA(cudaEventRecord(done, s));
            HOST_CUDA(cudaStreamWaitEvent(ctx->d2h, done, 0));
            HOST_CUDA(cudaMemcpy2DAsync(C_host + f0, size_t(K) * 4, c_dev + f0, size_t(K) * 4,
                                        size_t(w) * 4, crows, cudaMemcpyDeviceToHost, ctx->d2h));
        }
    }
    // `join` makes the caller's stream complete only after C is in host
    // memory; the pool buffers are released in its order after that
    return ACCSPMM_SUCCESS;
}

}  // namespace accspmm
